// Size-specialised 2-D real transforms of the lenslet-grid channel images
// (the hot-path forward transform with its channel gather, and the inverse
// transform with its plane / Richardson-Lucy epilogues).
//
// Each kernel is compiled for one transform size F (an even 7-smooth number
// <= 160), so every index and loop bound is a compile-time constant.  A 1-D
// length-F transform is a two-pass Cooley-Tukey split F = P1 * P2 (both
// <= 16): pass 1 runs P2 DFTs of length P1 on the stride-P2 subsequences and
// applies the inter-pass twiddles w_F^(t*k1); pass 2 runs P1 DFTs of length P2.
// Both passes work in place in shared memory (each thread writes exactly the
// locations it read), so the result of frequency K = k1 + P1*k2 ends up at
// position pi(K) = k1*P2 + k2.  The small DFTs run in registers with
// compile-time twiddles.  One CTA transforms one channel image.
//
// Forward (rfft2, real gathered image -> F x (F/2+1) spectrum):
//   R1  rows 2q, 2q+1 packed as one complex row, row pass 1      global -> B
//   R2  row pass 2 and the split of the two real rows' spectra   B -> A
//   R3  column pass 1 (rows beyond the image read as zero)      A -> A
//   R4  column pass 2, natural-order store                      A -> global
// Inverse (irfft2, spectrum -> real Ly x Lx channel image):
//   A1  column pass 1 on the (summed) input spectra              global -> A
//   A2  column pass 2                                            A -> A
//   B1  Hermitian expansion of rows 2q, 2q+1 packed as one complex
//       row, row pass 1                                          A -> B
//   B2  row pass 2 and the pixel epilogue                        B -> global
#pragma once

#include "flf_internal.cuh"

#include <type_traits>

namespace flf {
namespace sfft {

// ----------------------------------------------------------------------------
// Compile-time helpers
// ----------------------------------------------------------------------------

// cos / sin of 2*pi*num/den by their Taylor series after reducing the angle to
// [-pi, pi] (about 1e-15 absolute error, evaluated only at compile time).
__host__ __device__ constexpr double taylor_cos(double x) {
  double term = 1.0, sum = 1.0;
  for (int n = 1; n < 40; n++) {
    term *= -x * x / ((2.0 * n - 1.0) * (2.0 * n));
    sum += term;
  }
  return sum;
}
__host__ __device__ constexpr double taylor_sin(double x) {
  double term = x, sum = x;
  for (int n = 1; n < 40; n++) {
    term *= -x * x / ((2.0 * n) * (2.0 * n + 1.0));
    sum += term;
  }
  return sum;
}
__host__ __device__ constexpr double angle(int num, int den) {
  int r = ((num % den) + den) % den;        // [0, den)
  if (2 * r > den) r -= den;                // (-den/2, den/2]
  return 2.0 * 3.14159265358979323846264338327950288 * (double)r / (double)den;
}
__host__ __device__ constexpr double cos2pi(int num, int den) { return taylor_cos(angle(num, den)); }
__host__ __device__ constexpr double sin2pi(int num, int den) { return taylor_sin(angle(num, den)); }

// Register split F = P1 * P2 with P2 <= P1 <= 16 and P1 - P2 smallest.
__host__ __device__ constexpr int split_p1(int F) {
  int best = -1, gap = 1 << 30;
  for (int p1 = 1; p1 <= 16; p1++) {
    if (F % p1) continue;
    const int p2 = F / p1;
    if (p2 > 16 || p1 < p2) continue;
    if (p1 - p2 < gap) { gap = p1 - p2; best = p1; }
  }
  return best;
}

__host__ __device__ constexpr bool smooth_even(int F) {
  if (F < 2 || (F & 1)) return false;
  int n = F;
  while (n % 2 == 0) n /= 2;
  while (n % 3 == 0) n /= 3;
  while (n % 5 == 0) n /= 5;
  while (n % 7 == 0) n /= 7;
  return n == 1;
}

template <int F> struct Shape {
  static_assert(smooth_even(F) && F <= 160, "transform size must be even, 7-smooth and <= 160");
  static constexpr int P1 = split_p1(F);
  static constexpr int P2 = F / P1;
  static constexpr int FH = F / 2 + 1;
  static constexpr int PA = FH;       // row pitch (complex) of the F x FH buffer A
  static constexpr int PB = F + 1;    // row pitch of the packed-row buffer B (odd: no bank conflicts across rows)
  static constexpr int NT = F <= 48 ? 128 : 256;
  // CTAs per SM that shared memory allows at the largest row-pair count
  // (nq = F/2), capped so that a thread keeps at least 80 registers; passed
  // to __launch_bounds__ so the register budget follows occupancy.
  static constexpr int SMEM_MAX = (F + F * PA + (F / 2) * PB) * 8;
  static constexpr int MINB_SMEM = 233472 / SMEM_MAX < 1 ? 1 : 233472 / SMEM_MAX;
  static constexpr int MINB_REGS = 65536 / (80 * NT);
  static constexpr int MINB = MINB_SMEM < MINB_REGS ? MINB_SMEM : MINB_REGS;
  static_assert(P1 >= 1 && P2 >= 1 && P1 * P2 == F && P1 <= 16 && P2 <= 16, "no register split");
};

// Compile-time loop: fn(std::integral_constant<int, I>) for I in [B, E).
template <int B, int E> struct SFor {
  template <class Fn> __device__ __forceinline__ static void run(Fn &&fn) {
    if constexpr (B < E) {
      fn(std::integral_constant<int, B>());
      SFor<B + 1, E>::run(fn);
    }
  }
};

__device__ __forceinline__ float2 add2(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 sub2(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float2 conj2(float2 a) { return make_float2(a.x, -a.y); }
// a * w with w = (c, s)
__device__ __forceinline__ float2 mulw(float2 a, float2 w) {
  return make_float2(fmaf(a.x, w.x, -a.y * w.y), fmaf(a.x, w.y, a.y * w.x));
}
// a * i * S  (S = +1 or -1)
template <int S> __device__ __forceinline__ float2 mul_iS(float2 a) {
  return S > 0 ? make_float2(-a.y, a.x) : make_float2(a.y, -a.x);
}

// a * exp(S * 2 pi i * NUM / DEN), trivial factors folded away.
template <int NUM, int DEN, int S> __device__ __forceinline__ float2 twc(float2 a) {
  constexpr int r = ((NUM % DEN) + DEN) % DEN;
  if constexpr (r == 0) {
    return a;
  } else if constexpr (2 * r == DEN) {
    return make_float2(-a.x, -a.y);
  } else if constexpr (4 * r == DEN) {
    return mul_iS<S>(a);
  } else if constexpr (4 * r == 3 * DEN) {
    return mul_iS<-S>(a);
  } else {
    constexpr float c = (float)cos2pi(r, DEN);
    constexpr float s = (float)(S * sin2pi(r, DEN));
    return make_float2(fmaf(a.x, c, -a.y * s), fmaf(a.x, s, a.y * c));
  }
}

// ----------------------------------------------------------------------------
// Register DFTs: x <- DFT_P(x) with kernel exp(S * 2 pi i n k / P), natural
// order in and out.
// ----------------------------------------------------------------------------
template <int P> struct FirstFactor {
  static constexpr int v = (P % 4 == 0 && P != 4) ? 4 : (P % 2 == 0 && P != 2) ? 2 : (P % 3 == 0 && P != 3) ? 3
                         : (P % 5 == 0 && P != 5) ? 5 : (P % 7 == 0 && P != 7) ? 7 : 1;
};

template <int P, int S> struct Dft;

template <int S> struct Dft<1, S> {
  __device__ __forceinline__ static void run(float2 (&)[1]) {}
};

template <int S> struct Dft<2, S> {
  __device__ __forceinline__ static void run(float2 (&x)[2]) {
    const float2 a = x[0], b = x[1];
    x[0] = add2(a, b);
    x[1] = sub2(a, b);
  }
};

template <int S> struct Dft<4, S> {
  __device__ __forceinline__ static void run(float2 (&x)[4]) {
    const float2 a = add2(x[0], x[2]), b = sub2(x[0], x[2]);
    const float2 c = add2(x[1], x[3]), d = mul_iS<S>(sub2(x[1], x[3]));
    x[0] = add2(a, c);
    x[2] = sub2(a, c);
    x[1] = add2(b, d);
    x[3] = sub2(b, d);
  }
};

// Odd prime P: X_k = x0 + sum_j (x_j + x_{P-j}) cos(2 pi jk/P)
//                      + i S sum_j (x_j - x_{P-j}) sin(2 pi jk/P),  X_{P-k} likewise with -i S.
template <int P, int S> struct DftOddPrime {
  __device__ __forceinline__ static void run(float2 (&x)[P]) {
    constexpr int H = (P - 1) / 2;
    float2 sp[H], sm[H];
    SFor<1, H + 1>::run([&](auto J) {
      constexpr int j = decltype(J)::value;
      sp[j - 1] = add2(x[j], x[P - j]);
      sm[j - 1] = sub2(x[j], x[P - j]);
    });
    const float2 x0 = x[0];
    float2 s0 = x0;
    SFor<0, H>::run([&](auto J) { s0 = add2(s0, sp[decltype(J)::value]); });
    float2 out[P];
    out[0] = s0;
    SFor<1, H + 1>::run([&](auto K) {
      constexpr int k = decltype(K)::value;
      float2 re = x0, im = make_float2(0.f, 0.f);
      SFor<1, H + 1>::run([&](auto J) {
        constexpr int j = decltype(J)::value;
        constexpr float c = (float)cos2pi(j * k, P);
        constexpr float s = (float)sin2pi(j * k, P);
        re.x = fmaf(sp[j - 1].x, c, re.x);
        re.y = fmaf(sp[j - 1].y, c, re.y);
        im.x = fmaf(sm[j - 1].x, s, im.x);
        im.y = fmaf(sm[j - 1].y, s, im.y);
      });
      const float2 t = mul_iS<S>(im);
      out[k] = add2(re, t);
      out[P - k] = sub2(re, t);
    });
    SFor<0, P>::run([&](auto K) { x[decltype(K)::value] = out[decltype(K)::value]; });
  }
};
template <int S> struct Dft<3, S> : DftOddPrime<3, S> {};
template <int S> struct Dft<5, S> : DftOddPrime<5, S> {};
template <int S> struct Dft<7, S> : DftOddPrime<7, S> {};

// Composite P = A * B: n = b + B a, K = k1 + A k2,
// X[k1 + A k2] = sum_b w_P^(b k1) w_B^(b k2) sum_a x[b + B a] w_A^(a k1).
template <int P, int S> struct Dft {
  static constexpr int A = FirstFactor<P>::v;
  static constexpr int B = P / A;
  static_assert(A > 1 && B > 1, "unsupported register DFT length");
  __device__ __forceinline__ static void run(float2 (&x)[P]) {
    float2 y[B][A];
    SFor<0, B>::run([&](auto Bi) {
      constexpr int b = decltype(Bi)::value;
      float2 t[A];
      SFor<0, A>::run([&](auto Ai) { t[decltype(Ai)::value] = x[b + B * decltype(Ai)::value]; });
      Dft<A, S>::run(t);
      SFor<0, A>::run([&](auto Ki) {
        constexpr int k1 = decltype(Ki)::value;
        y[b][k1] = twc<b * k1, P, S>(t[k1]);
      });
    });
    SFor<0, A>::run([&](auto Ki) {
      constexpr int k1 = decltype(Ki)::value;
      float2 u[B];
      SFor<0, B>::run([&](auto Bi) { u[decltype(Bi)::value] = y[decltype(Bi)::value][k1]; });
      Dft<B, S>::run(u);
      SFor<0, B>::run([&](auto K2) { x[k1 + A * decltype(K2)::value] = u[decltype(K2)::value]; });
    });
  }
};

// Per-launch constants of the specialised kernels (built by the launcher).
struct SizedArgs {
  int nq;      // packed row pairs (Ly + 1) / 2
  Div16 dnq;   // division by nq
  int a_len;   // complex elements of region A: max(F * PA, channel image Ly * Lxp floats)
  Div16 dlx4;  // division by Lxp / 4 (16-byte groups per channel-image row)
};

// ----------------------------------------------------------------------------
// Pass helpers on one length-F transform whose element e sits at base + e*es
// in shared memory.  Pass 1 (thread t < P2) reads x[t + P2 k] from `in`,
// pass 2 (thread k1 < P1) reads positions k1*P2 + t.
// ----------------------------------------------------------------------------
template <int F, int S>
__device__ __forceinline__ void twiddle_pass1(float2 (&x)[Shape<F>::P1], const float2 *__restrict__ TW, int t) {
  constexpr int P1 = Shape<F>::P1, P2 = Shape<F>::P2;
  SFor<1, P1>::run([&](auto K) {
    constexpr int k1 = decltype(K)::value;
    const float2 w = TW[k1 * P2 + t];            // exp(-2 pi i t k1 / F)
    x[k1] = mulw(x[k1], S < 0 ? w : conj2(w));
  });
}

template <int F, int S>
__device__ __forceinline__ void pass2(float *__restrict__ base_f, int es) {
  constexpr int P2 = Shape<F>::P2;
  float2 *base = reinterpret_cast<float2 *>(base_f);
  float2 u[P2];
  SFor<0, P2>::run([&](auto T) { u[decltype(T)::value] = base[decltype(T)::value * es]; });
  Dft<P2, S>::run(u);
  SFor<0, P2>::run([&](auto T) { base[decltype(T)::value * es] = u[decltype(T)::value]; });
}

// Shared-memory layout of both kernels: TW[P1*P2] | A[F][PA] | B[nq][PB].
// Shared-memory layout of both kernels: TW[F] | A[a_len] | B[nq][PB] (complex).
// Region A holds the F x FH spectrum and, before R1 or after B1, the real
// channel image (Ly x Lxp floats).
template <int F> int region_a(int Ly, int Lxp) {
  const int img = (Ly * Lxp + 1) / 2;
  return F * Shape<F>::PA > img ? F * Shape<F>::PA : img;
}
template <int F> size_t smem_bytes(int nq, int a_len) {
  return sizeof(float2) * ((size_t)F + a_len + (size_t)nq * Shape<F>::PB);
}

template <int F>
__device__ __forceinline__ void load_twiddles(float2 *TW, const float2 *__restrict__ W) {
  constexpr int P2 = Shape<F>::P2, NT = Shape<F>::NT;
  for (int i = threadIdx.x; i < F; i += NT) {   // i = k1 * P2 + t
    const int k1 = i / P2, t = i - k1 * P2;
    TW[i] = W[t * k1];                             // t * k1 < F
  }
}

// ----------------------------------------------------------------------------
// Forward transform of channel-major images (Rfft2Params mode 0): image g is
// channel ch = g % NN = b*N + a, Ly x Lx samples of pixels (r*N + b, c*N + a);
// samples outside the Y x X image read as zero.  Output spectrum
// dst[g][ky][kx], ky < F, kx <= F/2, natural order.
// ----------------------------------------------------------------------------
template <int F>
__global__ void __launch_bounds__(Shape<F>::NT, Shape<F>::MINB) k_rfft2_sized(Rfft2Params p, SizedArgs sa) {
  using Sh = Shape<F>;
  constexpr int P1 = Sh::P1, P2 = Sh::P2, FH = Sh::FH, PA = Sh::PA, PB = Sh::PB, NT = Sh::NT;
  extern __shared__ __align__(16) float smf[];
  float2 *TW = reinterpret_cast<float2 *>(smf);
  float2 *A = TW + F;
  float2 *Bq = A + sa.a_len;
  load_twiddles<F>(TW, reinterpret_cast<const float2 *>(p.twiddle));

  const int g = blockIdx.x;
  const int N = p.N, NN = N * N;
  const int ch = g % NN;
  const int b = ch / N, a = ch - b * N;
  const int nq = sa.nq, Ly = p.Ly, Lx = p.Lx, X = p.X, Y = p.Y, Lxp = p.Lxp;

  // R0: the channel image into region A with 16-byte loads.
  {
    const float4 *src = reinterpret_cast<const float4 *>(p.chan + (long long)g * Ly * Lxp);
    float4 *st = reinterpret_cast<float4 *>(A);
    const int n4 = Ly * Lxp / 4;
    for (int i = threadIdx.x; i < n4; i += NT) st[i] = __ldg(src + i);
  }
  __syncthreads();

  // R1: row pairs (2q, 2q+1) as one complex row; row pass 1 into B.
  const float *img = reinterpret_cast<const float *>(A);
  for (int task = threadIdx.x; task < nq * P2; task += NT) {
    const int t = (int)sa.dnq.div(task);
    const int q = task - t * nq;
    const int r0 = 2 * q, r1 = r0 + 1;
    const bool ok0 = r0 * N + b < Y, ok1 = r1 < Ly && r1 * N + b < Y;
    const float *s0 = img + r0 * Lxp, *s1 = s0 + Lxp;
    float2 x[P1];
    SFor<0, P1>::run([&](auto K) {
      constexpr int k = decltype(K)::value;
      const int c = t + P2 * k;
      const bool okc = c < Lx && c * N + a < X;
      x[k] = make_float2(okc && ok0 ? s0[c] : 0.f, okc && ok1 ? s1[c] : 0.f);
    });
    Dft<P1, -1>::run(x);
    twiddle_pass1<F, -1>(x, TW, t);
    float2 *row = Bq + q * PB + t;
    SFor<0, P1>::run([&](auto K) { row[P2 * decltype(K)::value] = x[decltype(K)::value]; });
  }
  __syncthreads();

  // R2: row pass 2 for the frequency pair (k1, P1 - k1) and the split of the
  // packed spectrum Z into the two real rows' half spectra:
  // Y0[K] = (Z[K] + conj Z[F-K]) / 2, Y1[K] = (Z[K] - conj Z[F-K]) / 2i, K <= F/2.
  constexpr int NPAIR = P1 / 2 + 1;
  for (int task = threadIdx.x; task < nq * NPAIR; task += NT) {
    const int kp = (int)sa.dnq.div(task);
    const int q = task - kp * nq;
    const int k1a = kp, k1b = (P1 - kp) % P1;
    const float2 *row = Bq + q * PB;
    float2 za[P2], zb[P2];
    SFor<0, P2>::run([&](auto T) { za[decltype(T)::value] = row[k1a * P2 + decltype(T)::value]; });
    Dft<P2, -1>::run(za);
    if (k1b != k1a) {
      SFor<0, P2>::run([&](auto T) { zb[decltype(T)::value] = row[k1b * P2 + decltype(T)::value]; });
      Dft<P2, -1>::run(zb);
    }
    float2 *y0 = A + (2 * q) * PA, *y1 = y0 + PA;
    auto emit = [&](int K, float2 z, float2 zp) {   // zp = Z[F - K]
      const float2 m = conj2(zp);
      const float2 d = sub2(z, m);
      y0[K] = make_float2((z.x + m.x) * 0.5f, (z.y + m.y) * 0.5f);
      y1[K] = make_float2(d.y * 0.5f, -d.x * 0.5f);
    };
    if (k1a == 0) {
      SFor<0, P2>::run([&](auto T) {
        constexpr int k2 = decltype(T)::value;
        if (P1 * k2 <= F / 2) emit(P1 * k2, za[k2], za[(P2 - k2) % P2]);
      });
    } else if (k1b == k1a) {   // k1 = P1/2 (P1 even)
      SFor<0, P2>::run([&](auto T) {
        constexpr int k2 = decltype(T)::value;
        const int K = k1a + P1 * k2;
        if (K <= F / 2) emit(K, za[k2], za[P2 - 1 - k2]);
      });
    } else {
      SFor<0, P2>::run([&](auto T) {
        constexpr int k2 = decltype(T)::value;
        const int Ka = k1a + P1 * k2, Kb = k1b + P1 * k2;
        if (Ka <= F / 2) emit(Ka, za[k2], zb[P2 - 1 - k2]);
        if (Kb <= F / 2) emit(Kb, zb[k2], za[P2 - 1 - k2]);
      });
    }
  }
  __syncthreads();

  // R3: column pass 1 over the FH columns; rows >= 2 nq are zero.
  const int nrows = 2 * nq;
  for (int task = threadIdx.x; task < FH * P2; task += NT) {
    const int t = task / FH, c = task - t * FH;
    float2 x[P1];
    SFor<0, P1>::run([&](auto K) {
      constexpr int k = decltype(K)::value;
      const int r = t + P2 * k;
      x[k] = r < nrows ? A[r * PA + c] : make_float2(0.f, 0.f);
    });
    Dft<P1, -1>::run(x);
    twiddle_pass1<F, -1>(x, TW, t);
    SFor<0, P1>::run([&](auto K) { A[(t + P2 * decltype(K)::value) * PA + c] = x[decltype(K)::value]; });
  }
  __syncthreads();

  // R4: column pass 2; frequency ky = k1 + P1 k2 stored in natural order.
  float2 *dst = reinterpret_cast<float2 *>(p.dst) + (long long)g * (F * FH);
  for (int task = threadIdx.x; task < FH * P1; task += NT) {
    const int k1 = task / FH, c = task - k1 * FH;
    float2 u[P2];
    SFor<0, P2>::run([&](auto T) { u[decltype(T)::value] = A[(k1 * P2 + decltype(T)::value) * PA + c]; });
    Dft<P2, -1>::run(u);
    SFor<0, P2>::run([&](auto T) { dst[(k1 + P1 * decltype(T)::value) * FH + c] = u[decltype(T)::value]; });
  }
}

// ----------------------------------------------------------------------------
// Inverse transform (unscaled) of image g, channel j = g % NN = beta*N + alpha,
// summed over nsum partial spectra, cropped to Ly x Lx and written as a
// channel-major image (stored, or added to what is there).  The final pass
// zeroes the samples outside the Y x X image and the row padding, and can
// store num / value instead of the value.
// ----------------------------------------------------------------------------
template <int F>
__global__ void __launch_bounds__(Shape<F>::NT, Shape<F>::MINB) k_irfft2_sized(Irfft2Params p, SizedArgs sa) {
  using Sh = Shape<F>;
  constexpr int P1 = Sh::P1, P2 = Sh::P2, FH = Sh::FH, PA = Sh::PA, PB = Sh::PB, NT = Sh::NT;
  extern __shared__ __align__(16) float smf[];
  float2 *TW = reinterpret_cast<float2 *>(smf);
  float2 *A = TW + F;
  float2 *Bq = A + sa.a_len;
  load_twiddles<F>(TW, p.twiddle);

  const int g = blockIdx.x;
  const float2 *src = p.src + (long long)g * (F * FH);
  const int nsum = p.nsum;
  __syncthreads();

  // A1: column pass 1 straight from the input spectra.
  for (int task = threadIdx.x; task < FH * P2; task += NT) {
    const int t = task / FH, c = task - t * FH;
    float2 x[P1];
    SFor<0, P1>::run([&](auto K) {
      constexpr int k = decltype(K)::value;
      x[k] = src[(t + P2 * k) * FH + c];
    });
    for (int s = 1; s < nsum; s++) {
      const float2 *ps = src + s * p.sum_stride;
      SFor<0, P1>::run([&](auto K) {
        constexpr int k = decltype(K)::value;
        x[k] = add2(x[k], ps[(t + P2 * k) * FH + c]);
      });
    }
    Dft<P1, 1>::run(x);
    twiddle_pass1<F, 1>(x, TW, t);
    SFor<0, P1>::run([&](auto K) { A[(t + P2 * decltype(K)::value) * PA + c] = x[decltype(K)::value]; });
  }
  __syncthreads();

  // A2: column pass 2; spatial row y ends up at row (y % P1) * P2 + y / P1.
  for (int task = threadIdx.x; task < FH * P1; task += NT) {
    const int k1 = task / FH, c = task - k1 * FH;
    pass2<F, 1>(reinterpret_cast<float *>(A + (k1 * P2) * PA + c), PA);
  }
  __syncthreads();

  // B1: rows (2q, 2q+1) expanded to full Hermitian rows a, b and packed as
  // z = a + i b; row pass 1 into B.  The imaginary parts of the DC and
  // Nyquist columns are dropped (a real inverse transform).
  const int nq = sa.nq;
  for (int task = threadIdx.x; task < nq * P2; task += NT) {
    const int q = task / P2, t = task - q * P2;
    const int y0 = 2 * q, y1 = y0 + 1;
    const float2 *ra = A + ((y0 % P1) * P2 + y0 / P1) * PA;
    const float2 *rb = A + ((y1 % P1) * P2 + y1 / P1) * PA;
    float2 x[P1];
    SFor<0, P1>::run([&](auto K) {
      constexpr int k = decltype(K)::value;
      const int n = t + P2 * k;
      float2 va, vb;
      if (n <= F / 2) {
        va = ra[n];
        vb = rb[n];
        if (n == 0 || n == F / 2) { va.y = 0.f; vb.y = 0.f; }
      } else {
        va = conj2(ra[F - n]);
        vb = conj2(rb[F - n]);
      }
      x[k] = make_float2(va.x - vb.y, va.y + vb.x);
    });
    Dft<P1, 1>::run(x);
    twiddle_pass1<F, 1>(x, TW, t);
    float2 *row = Bq + q * PB + t;
    SFor<0, P1>::run([&](auto K) { row[P2 * decltype(K)::value] = x[decltype(K)::value]; });
  }
  __syncthreads();

  // B2: row pass 2; x = k1 + P1 k2 of the packed row q holds sample (2q, x)
  // in .x and (2q+1, x) in .y, staged as a real Ly x Lxp image in region A
  // (free since B1).
  const int Ly = p.Ly, Lx = p.Lx, Lxp = p.Lxp;
  float *img = reinterpret_cast<float *>(A);
  for (int task = threadIdx.x; task < nq * P1; task += NT) {
    const int k1 = (int)sa.dnq.div(task);
    const int q = task - k1 * nq;
    float2 u[P2];
    const float2 *row = Bq + q * PB + k1 * P2;
    SFor<0, P2>::run([&](auto T) { u[decltype(T)::value] = row[decltype(T)::value]; });
    Dft<P2, 1>::run(u);
    float *s0 = img + 2 * q * Lxp;
    const bool has1 = 2 * q + 1 < Ly;
    SFor<0, P2>::run([&](auto T) {
      constexpr int k2 = decltype(T)::value;
      const int c = k1 + P1 * k2;
      if (c < Lx) {
        s0[c] = u[k2].x;
        if (has1) s0[Lxp + c] = u[k2].y;
      }
    });
  }
  __syncthreads();

  // Copy-out with 16-byte accesses.
  const int N = p.N, NN = N * N;
  const int j = g % NN;
  const int beta = j / N, alpha = j - beta * N;
  const int X = p.X, Y = p.Y;
  const int n4 = Ly * Lxp / 4, lx4 = Lxp / 4;
  float4 *dst = reinterpret_cast<float4 *>(p.chan + (long long)g * Ly * Lxp);
  const float4 *num = p.num ? reinterpret_cast<const float4 *>(p.num + (long long)g * Ly * Lxp) : nullptr;
  const float4 *st = reinterpret_cast<const float4 *>(img);
  for (int i = threadIdx.x; i < n4; i += NT) {
    float4 v = st[i];
    if (p.add) {
      const float4 o = dst[i];
      v.x += o.x; v.y += o.y; v.z += o.z; v.w += o.w;
    }
    if (p.final_pass) {
      const int r = (int)sa.dlx4.div(i);
      const int c0 = (i - r * lx4) * 4;
      const bool rowok = r * N + beta < Y;
      float4 nv = make_float4(0.f, 0.f, 0.f, 0.f);
      if (num) nv = __ldg(num + i);
      float e[4] = {v.x, v.y, v.z, v.w};
      const float n[4] = {nv.x, nv.y, nv.z, nv.w};
#pragma unroll
      for (int k = 0; k < 4; k++) {
        const int c = c0 + k;
        const bool ok = rowok && c < Lx && c * N + alpha < X;
        // the standard RL error image num / Hx (lfdeconv.py:192)
        e[k] = ok ? (num ? __fdiv_rn(n[k], e[k]) : e[k]) : 0.f;
      }
      v = make_float4(e[0], e[1], e[2], e[3]);
    }
    dst[i] = v;
  }
}

template <int F> cudaError_t rfft2_sized(const Rfft2Params &p, cudaStream_t s);
template <int F> cudaError_t irfft2_sized(const Irfft2Params &p, cudaStream_t s);

// Every even 7-smooth size up to kMaxF; each is instantiated in one of the
// flf_fft_part*.cu translation units.
#define FLF_SFFT_SIZES(X)                                                                      \
  X(2) X(4) X(6) X(8) X(10) X(12) X(14) X(16) X(18) X(20) X(24) X(28) X(30) X(32) X(36) X(40) \
  X(42) X(48) X(50) X(54) X(56) X(60) X(64) X(70) X(72) X(80) X(84) X(90) X(96) X(98) X(100)  \
  X(108) X(112) X(120) X(126) X(128) X(140) X(144) X(150) X(160)

#define FLF_SFFT_DEFINE_LAUNCHERS                                                                     \
  template <int F> static SizedArgs sized_args(int Ly, int Lxp) {                                    \
    SizedArgs sa;                                                                                     \
    sa.nq = (Ly + 1) / 2;                                                                             \
    sa.dnq = Div16::make((unsigned)sa.nq);                                                            \
    sa.a_len = region_a<F>(Ly, Lxp);                                                                  \
    sa.dlx4 = Div16::make((unsigned)(Lxp / 4));                                                       \
    return sa;                                                                                        \
  }                                                                                                   \
  template <int F> cudaError_t rfft2_sized(const Rfft2Params &p, cudaStream_t s) {                    \
    const SizedArgs sa = sized_args<F>(p.Ly, p.Lxp);                                                  \
    const size_t sm = smem_bytes<F>(sa.nq, sa.a_len);                                                 \
    cudaError_t e = cudaFuncSetAttribute((const void *)k_rfft2_sized<F>,                              \
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);       \
    if (e != cudaSuccess) return e;                                                                   \
    k_rfft2_sized<F><<<p.nimg, Shape<F>::NT, sm, s>>>(p, sa);                                         \
    return cudaGetLastError();                                                                        \
  }                                                                                                   \
  template <int F> cudaError_t irfft2_sized(const Irfft2Params &p, cudaStream_t s) {                  \
    const SizedArgs sa = sized_args<F>(p.Ly, p.Lxp);                                                  \
    const size_t sm = smem_bytes<F>(sa.nq, sa.a_len);                                                 \
    cudaError_t e = cudaFuncSetAttribute((const void *)k_irfft2_sized<F>,                             \
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);       \
    if (e != cudaSuccess) return e;                                                                   \
    k_irfft2_sized<F><<<p.nimg, Shape<F>::NT, sm, s>>>(p, sa);                                        \
    return cudaGetLastError();                                                                        \
  }

}  // namespace sfft
}  // namespace flf
