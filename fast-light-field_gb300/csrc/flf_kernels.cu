// CUDA kernels of libflf.so (sm_103a): lenslet-grid FFTs, the fused spectral
// multiply-accumulate over planes and lenslet offsets, inverse transform with
// crop / plane reduction / Richardson-Lucy epilogues, and the PSF transfer
// matrix precompute.  Host code that sequences them is flf_api.cu.
#include "flf_internal.cuh"

#include <cstdio>

namespace flf {

// ----------------------------------------------------------------------------
// Complex helpers, templated on the real type (float runtime, double precompute)
// ----------------------------------------------------------------------------
template <typename R> struct CT;
template <> struct CT<float> { typedef float2 T; };
template <> struct CT<double> { typedef double2 T; };

template <typename C> __device__ __forceinline__ C cmk(decltype(C::x) a, decltype(C::x) b) {
  C r; r.x = a; r.y = b; return r;
}
template <typename C> __device__ __forceinline__ C cadd(C a, C b) { return cmk<C>(a.x + b.x, a.y + b.y); }
template <typename C> __device__ __forceinline__ C csub(C a, C b) { return cmk<C>(a.x - b.x, a.y - b.y); }
template <typename C> __device__ __forceinline__ C cmul(C a, C b) {
  return cmk<C>(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
template <typename C> __device__ __forceinline__ C cconj(C a) { return cmk<C>(a.x, -a.y); }

// acc += a * b  (complex multiply-accumulate, 4 FMAs)
__device__ __forceinline__ void cmac(float2 &acc, float2 a, float2 b) {
  acc.x = fmaf(a.x, b.x, acc.x);
  acc.x = fmaf(-a.y, b.y, acc.x);
  acc.y = fmaf(a.x, b.y, acc.y);
  acc.y = fmaf(a.y, b.x, acc.y);
}
// acc += conj(a) * b
__device__ __forceinline__ void cmacc(float2 &acc, float2 a, float2 b) {
  acc.x = fmaf(a.x, b.x, acc.x);
  acc.x = fmaf(a.y, b.y, acc.x);
  acc.y = fmaf(a.x, b.y, acc.y);
  acc.y = fmaf(-a.y, b.x, acc.y);
}

// ----------------------------------------------------------------------------
// Shared-memory Stockham FFT (mixed radix 2/3/4/5/7), batched over the images
// a CTA holds.  Stage with radix p and span m: butterfly i of a transform
// reads x[i + j*n/p], applies w^(j*(i mod m)) with w = exp(-2 pi i/(p m)),
// does a p-point DFT and writes y[(i - i mod m)*p + i mod m + j*m].
// The output is in natural order after the last stage.
// ----------------------------------------------------------------------------
template <typename C>
__device__ __forceinline__ C twid(const C *W, int idx, bool inv) {
  C w = W[idx];
  return inv ? cconj(w) : w;
}

template <typename C, int P>
__device__ __forceinline__ void dft_small(C (&u)[P], const C *W, int n, bool inv) {
  if (P == 2) {
    C a = u[0], b = u[1];
    u[0] = cadd(a, b);
    u[1] = csub(a, b);
  } else if (P == 4) {
    C a = cadd(u[0], u[2]), b = csub(u[0], u[2]);
    C c = cadd(u[1], u[3]), d = csub(u[1], u[3]);
    // -i*d (forward) or +i*d (inverse)
    C id = inv ? cmk<C>(-d.y, d.x) : cmk<C>(d.y, -d.x);
    u[0] = cadd(a, c);
    u[2] = csub(a, c);
    u[1] = cadd(b, id);
    u[3] = csub(b, id);
  } else {
    C v[P];
    const int st = n / P;
#pragma unroll
    for (int l = 0; l < P; l++) {
      C s = u[0];
#pragma unroll
      for (int j = 1; j < P; j++) s = cadd(s, cmul(u[j], twid(W, ((j * l) % P) * st, inv)));
      v[l] = s;
    }
#pragma unroll
    for (int l = 0; l < P; l++) u[l] = v[l];
  }
}

template <typename C, int P>
__device__ void fft_stage(const C *__restrict__ src, C *__restrict__ dst, int imgStride, int nimg,
                          int ntrans, int es, int ts, int n, int m, const C *W, bool inv) {
  const int nb = n / P;
  const int step = n / (P * m);
  const int total = nimg * ntrans * nb;
  for (int idx = threadIdx.x; idx < total; idx += blockDim.x) {
    const int i = idx % nb;
    const int tr = idx / nb;
    const int img = tr / ntrans;
    const int tl = tr - img * ntrans;
    const int base = img * imgStride + tl * ts;
    const int k = i % m;
    C u[P];
#pragma unroll
    for (int j = 0; j < P; j++) u[j] = src[base + (i + j * nb) * es];
#pragma unroll
    for (int j = 1; j < P; j++) u[j] = cmul(u[j], twid(W, j * k * step, inv));
    dft_small<C, P>(u, W, n, inv);
    const int ob = (i - k) * P + k;
#pragma unroll
    for (int j = 0; j < P; j++) dst[base + (ob + j * m) * es] = u[j];
  }
}

// Runs all stages of plan `pl` on a batch of transforms; returns the buffer
// holding the result (A or B).
template <typename C>
__device__ C *fft_pass(C *A, C *B, int imgStride, int nimg, int ntrans, int es, int ts,
                       const FftPlan &pl, const C *W, bool inv) {
  C *src = A, *dst = B;
  int m = 1;
  for (int s = 0; s < pl.nst; s++) {
    const int p = pl.rad[s];
    switch (p) {
      case 2: fft_stage<C, 2>(src, dst, imgStride, nimg, ntrans, es, ts, pl.n, m, W, inv); break;
      case 3: fft_stage<C, 3>(src, dst, imgStride, nimg, ntrans, es, ts, pl.n, m, W, inv); break;
      case 4: fft_stage<C, 4>(src, dst, imgStride, nimg, ntrans, es, ts, pl.n, m, W, inv); break;
      case 5: fft_stage<C, 5>(src, dst, imgStride, nimg, ntrans, es, ts, pl.n, m, W, inv); break;
      default: fft_stage<C, 7>(src, dst, imgStride, nimg, ntrans, es, ts, pl.n, m, W, inv); break;
    }
    __syncthreads();
    C *t = src; src = dst; dst = t;
    m *= p;
  }
  return src;
}

// ----------------------------------------------------------------------------
// Forward real 2-D transform f x f -> f x (f/2+1), with the lenslet-channel
// gather of the input (the reference's strided sub-image FFT,
// special_fftconvolve.py:85-105 / py_light_field.cpp:1001-1027, done for all
// offsets at once).  Two real rows are packed into one complex row for the
// row pass and split afterwards.
// ----------------------------------------------------------------------------
template <typename R>
__global__ void __launch_bounds__(256) k_rfft2(Rfft2Params p) {
  typedef typename CT<R>::T C;
  extern __shared__ __align__(16) unsigned char smraw[];
  const int f = p.plan.n, fh = f / 2 + 1, isz = f * fh;
  C *W = reinterpret_cast<C *>(smraw);
  C *A = W + f;
  C *Bf = A + p.imgs_per_cta * isz;
  const C *tw = reinterpret_cast<const C *>(p.twiddle);
  for (int i = threadIdx.x; i < f; i += blockDim.x) W[i] = tw[i];

  const int g0 = blockIdx.x * p.imgs_per_cta;
  const int nb = min(p.imgs_per_cta, p.nimg - g0);
  const int nq = p.nq_rows;
  const int N = p.N, NN = N * N;

  for (int idx = threadIdx.x; idx < nb * nq * f; idx += blockDim.x) {
    const int c = idx % f;
    const int q = (idx / f) % nq;
    const int img = idx / (f * nq);
    const int g = g0 + img;
    const int r0 = 2 * q, r1 = 2 * q + 1;
    R v0 = 0, v1 = 0;
    if (p.mode == 0) {
      const int ch = g % NN;
      const int tz = g / NN;
      const int zi = tz % p.nz;
      const int t = tz / p.nz;
      const int b = ch / N, a = ch % N;
      const int plane = p.planes ? p.planes[zi] : zi;
      const float *base = p.src + plane * p.src_sz + t * p.src_st;
      const int x = c * N + a;
      if (c < p.Lx && x < p.X) {
        const int y0 = r0 * N + b, y1 = r1 * N + b;
        if (r0 < p.Ly && y0 < p.Y) v0 = (R)base[(long long)y0 * p.X + x];
        if (r1 < p.Ly && y1 < p.Y) v1 = (R)base[(long long)y1 * p.X + x];
      }
    } else {
      const R *im = reinterpret_cast<const R *>(p.src_img) + (long long)g * f * f;
      v0 = im[r0 * f + c];
      v1 = im[r1 * f + c];
    }
    A[img * isz + q * f + c] = cmk<C>(v0, v1);
  }
  __syncthreads();

  C *Rr = fft_pass<C>(A, Bf, isz, nb, nq, 1, f, p.plan, W, false);
  C *Yb = (Rr == A) ? Bf : A;

  const int half = f / 2;
  for (int idx = threadIdx.x; idx < nb * half * fh; idx += blockDim.x) {
    const int k = idx % fh;
    const int q = (idx / fh) % half;
    const int img = idx / (half * fh);
    C y0 = cmk<C>(0, 0), y1 = cmk<C>(0, 0);
    if (q < nq) {
      const C Z = Rr[img * isz + q * f + k];
      const C Zc = cconj(Rr[img * isz + q * f + ((f - k) % f)]);
      y0 = cmk<C>((Z.x + Zc.x) * (R)0.5, (Z.y + Zc.y) * (R)0.5);
      const C d = csub(Z, Zc);
      y1 = cmk<C>(d.y * (R)0.5, -d.x * (R)0.5);
    }
    Yb[img * isz + (2 * q) * fh + k] = y0;
    Yb[img * isz + (2 * q + 1) * fh + k] = y1;
  }
  __syncthreads();

  C *Out = fft_pass<C>(Yb, Rr, isz, nb, fh, fh, 1, p.plan, W, false);
  C *dst = reinterpret_cast<C *>(p.dst) + (long long)g0 * isz;
  for (int idx = threadIdx.x; idx < nb * isz; idx += blockDim.x) dst[idx] = Out[idx];
}

// ----------------------------------------------------------------------------
// Inverse real 2-D transform f x (f/2+1) -> f x f (unscaled: 1/f^2 is folded
// into the transfer matrices), summed over partial spectra, cropped to the
// Ly x Lx lenslet grid and scattered back to pixels (p*N + beta, q*N + alpha).
// This is the reference's InverseRFFTList + CropAfterFFT
// (py_light_field.cpp:925-950, projector.py:792-796) with the RL update of
// lfdeconv.py:112-183 fused into the store.
// ----------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_irfft2(Irfft2Params p) {
  extern __shared__ __align__(16) unsigned char smraw[];
  const int f = p.plan.n, fh = f / 2 + 1, isz = f * fh;
  float2 *W = reinterpret_cast<float2 *>(smraw);
  float2 *A = W + f;
  float2 *Bf = A + p.imgs_per_cta * isz;
  for (int i = threadIdx.x; i < f; i += blockDim.x) W[i] = p.twiddle[i];

  const int g0 = blockIdx.x * p.imgs_per_cta;
  const int nb = min(p.imgs_per_cta, p.nimg - g0);
  const float2 *src = p.src + (long long)g0 * isz;
  for (int idx = threadIdx.x; idx < nb * isz; idx += blockDim.x) {
    float2 v = src[idx];
    for (int s = 1; s < p.nsum; s++) {
      const float2 w = src[s * p.sum_stride + idx];
      v.x += w.x;
      v.y += w.y;
    }
    A[idx] = v;
  }
  __syncthreads();

  float2 *Rr = fft_pass<float2>(A, Bf, isz, nb, fh, fh, 1, p.plan, W, true);
  float2 *Zb = (Rr == A) ? Bf : A;

  const int nq = (p.Ly + 1) / 2;
  const int half = f / 2;
  for (int idx = threadIdx.x; idx < nb * nq * f; idx += blockDim.x) {
    const int c = idx % f;
    const int q = (idx / f) % nq;
    const int img = idx / (f * nq);
    const float2 *r0 = Rr + img * isz + (2 * q) * fh;
    const float2 *r1 = r0 + fh;
    float2 a, b;
    if (c <= half) {
      a = r0[c];
      b = r1[c];
      if (c == 0 || c == half) { a.y = 0.f; b.y = 0.f; }
    } else {
      a = cconj(r0[f - c]);
      b = cconj(r1[f - c]);
    }
    Zb[img * isz + q * f + c] = make_float2(a.x - b.y, a.y + b.x);
  }
  __syncthreads();

  float2 *Out = fft_pass<float2>(Zb, Rr, isz, nb, nq, 1, f, p.plan, W, true);

  const int N = p.N, NN = N * N;
  for (int idx = threadIdx.x; idx < nb * p.Ly * p.Lx; idx += blockDim.x) {
    const int c = idx % p.Lx;
    const int r = (idx / p.Lx) % p.Ly;
    const int img = idx / (p.Lx * p.Ly);
    const int g = g0 + img;
    const int j = g % NN;
    const int tz = g / NN;
    const int zo = tz % p.nzo;
    const int t = tz / p.nzo;
    const int y = r * N + j / N, x = c * N + j % N;
    if (y >= p.Y || x >= p.X) continue;
    const float2 zv = Out[img * isz + (r >> 1) * f + c];
    const float val = (r & 1) ? zv.y : zv.x;
    const int plane = p.planes ? p.planes[zo] : zo;
    const long long pix = (long long)y * p.X + x;
    float *o = p.out.p + plane * p.out.sz + t * p.out.st + pix;
    switch (p.epi) {
      case EPI_STORE: *o = val; break;
      case EPI_DIVIDE: {
        const float yv = p.aux.p[plane * p.aux.sz + t * p.aux.st + pix];
        *o = __fdiv_rn(yv, val);
        break;
      }
      case EPI_RL_PREVEDEL: {
        const float htf = p.aux.p[plane * p.aux.sz + t * p.aux.st + pix];
        float r2 = __fmul_rn(*o, __fdiv_rn(htf, val));
        if (r2 != r2) r2 = 0.f;
        *o = r2;
        break;
      }
      default: {
        float r2 = __fmul_rn(*o, val);
        if (p.norm.p) r2 = __fdiv_rn(r2, p.norm.p[plane * p.norm.sz + t * p.norm.st + pix]);
        if (r2 != r2) r2 = 0.f;
        *o = r2;
        break;
      }
    }
  }
}

// ----------------------------------------------------------------------------
// Fused spectral multiply-accumulate (the hot kernel).
//
// One CTA owns one frequency pair (u, u*) and, for forward projection, a group
// of planes (accumulated in registers: the reference's plane sum moved into
// Fourier space) or, for back projection, one plane.  Each thread owns one
// mirror orbit of output channels (4, 2 or 1 channels) for both frequencies;
// row groups split the stored rows and are reduced through shared memory at
// the end.  Every stored matrix element is read once from HBM and feeds
// 4 complex multiply-adds per frame.  This replaces the reference's
// expandX + calculateRows{,Mirrored} launches (projector.py:395-459) and
// CalculateRow/CalculateRowBoth (py_light_field.cpp:303-341), which read and
// wrote the accumulator once per lenslet offset.
// ----------------------------------------------------------------------------
template <int K> struct Orb;
template <> struct Orb<0> {  // generic orbit [q, My q, Mx q, Mxy q]
  static constexpr int NS = 4;
  __device__ static constexpr int sy(int k) { return k ^ 1; }
  __device__ static constexpr int sx(int k) { return k ^ 2; }
  __device__ static constexpr int sxy(int k) { return 3 - k; }
};
template <> struct Orb<1> {  // alpha = c: [q, My q]
  static constexpr int NS = 2;
  __device__ static constexpr int sy(int k) { return k ^ 1; }
  __device__ static constexpr int sx(int k) { return k; }
  __device__ static constexpr int sxy(int k) { return k ^ 1; }
};
template <> struct Orb<2> {  // beta = c: [q, Mx q]
  static constexpr int NS = 2;
  __device__ static constexpr int sy(int k) { return k; }
  __device__ static constexpr int sx(int k) { return k ^ 1; }
  __device__ static constexpr int sxy(int k) { return k ^ 1; }
};
template <> struct Orb<3> {  // centre
  static constexpr int NS = 1;
  __device__ static constexpr int sy(int) { return 0; }
  __device__ static constexpr int sx(int) { return 0; }
  __device__ static constexpr int sxy(int) { return 0; }
};

template <int NS>
__device__ __forceinline__ void load_slots(const float2 *__restrict__ ptr, float2 (&t)[4]) {
  if (NS == 4) {
    const float4 a = __ldcs(reinterpret_cast<const float4 *>(ptr));
    const float4 b = __ldcs(reinterpret_cast<const float4 *>(ptr) + 1);
    t[0] = make_float2(a.x, a.y); t[1] = make_float2(a.z, a.w);
    t[2] = make_float2(b.x, b.y); t[3] = make_float2(b.z, b.w);
  } else if (NS == 2) {
    const float4 a = __ldcs(reinterpret_cast<const float4 *>(ptr));
    t[0] = make_float2(a.x, a.y); t[1] = make_float2(a.z, a.w);
  } else {
    t[0] = __ldcs(ptr);
  }
}

template <int TF, int K>
__device__ __forceinline__ void mac_rows(const float2 *__restrict__ Pk, const float2 *comb,
                                         const short4 *rowS, const Layout &L, int g, int G,
                                         float2 (&U)[TF][4], float2 (&V)[TF][4]) {
  typedef Orb<K> O;
  constexpr int NS = O::NS;
  const int RS = L.RS, NN2 = 2 * L.NN;
  // generic rows: each stored element t feeds channel i at u, Mxy i at u,
  // My i at u*, Mx i at u*.
  constexpr int UNR = 4;
  int r = g;
  for (; r + (UNR - 1) * G < L.nrowG; r += UNR * G) {
    float2 t[UNR][4];
#pragma unroll
    for (int w = 0; w < UNR; w++) load_slots<NS>(Pk + (long long)(r + w * G) * RS, t[w]);
#pragma unroll
    for (int w = 0; w < UNR; w++) {
      const short4 si = rowS[r + w * G];
#pragma unroll
      for (int tf = 0; tf < TF; tf++) {
        const float2 *cb = comb + tf * NN2;
        const float2 s0 = cb[si.x], s1 = cb[si.y], s2 = cb[si.z], s3 = cb[si.w];
#pragma unroll
        for (int k = 0; k < NS; k++) {
          cmac(U[tf][k], t[w][k], s0);
          cmacc(U[tf][k], t[w][O::sxy(k)], s1);
          cmac(V[tf][O::sy(k)], t[w][k], s2);
          cmacc(V[tf][O::sx(k)], t[w][k], s3);
        }
      }
    }
  }
  for (; r < L.nrowG; r += G) {
    float2 t[4];
    load_slots<NS>(Pk + (long long)r * RS, t);
    const short4 si = rowS[r];
#pragma unroll
    for (int tf = 0; tf < TF; tf++) {
      const float2 *cb = comb + tf * NN2;
      const float2 s0 = cb[si.x], s1 = cb[si.y], s2 = cb[si.z], s3 = cb[si.w];
#pragma unroll
      for (int k = 0; k < NS; k++) {
        cmac(U[tf][k], t[k], s0);
        cmacc(U[tf][k], t[O::sxy(k)], s1);
        cmac(V[tf][O::sy(k)], t[k], s2);
        cmacc(V[tf][O::sx(k)], t[k], s3);
      }
    }
  }
  // centre-cross representatives: rows (u, u*) pairs
  for (int k2 = g; k2 < L.nrep; k2 += G) {
    const int rr = L.nrowG + 2 * k2;
    float2 t[4], s[4];
    load_slots<NS>(Pk + (long long)rr * RS, t);
    load_slots<NS>(Pk + (long long)(rr + 1) * RS, s);
    const short4 si = rowS[L.nrowG + k2];
    const int rk = (k2 < L.c) ? 1 : ((k2 < 2 * L.c) ? 2 : 3);
#pragma unroll
    for (int tf = 0; tf < TF; tf++) {
      const float2 *cb = comb + tf * NN2;
      const float2 s0 = cb[si.x], s1 = cb[si.y], s2 = cb[si.z], s3 = cb[si.w];
#pragma unroll
      for (int k = 0; k < NS; k++) {
        cmac(U[tf][k], t[k], s0);
        cmac(V[tf][k], s[k], s1);
      }
      if (rk == 1) {
#pragma unroll
        for (int k = 0; k < NS; k++) {
          cmac(V[tf][O::sy(k)], t[k], s2);
          cmac(U[tf][O::sy(k)], s[k], s3);
        }
      } else if (rk == 2) {
#pragma unroll
        for (int k = 0; k < NS; k++) {
          cmacc(V[tf][O::sx(k)], t[k], s2);
          cmacc(U[tf][O::sx(k)], s[k], s3);
        }
      }
    }
  }
}

template <int TF, bool FWD>
__global__ void __launch_bounds__(512) k_mac(MacParams p) {
  extern __shared__ __align__(16) unsigned char smraw[];
  const Layout &L = p.L;
  const int NN = L.NN, NT = L.nthr, c = L.c, c2 = c * c;
  float2 *comb = reinterpret_cast<float2 *>(smraw);                 // [TF][2 NN]
  short4 *rowS = reinterpret_cast<short4 *>(comb + TF * 2 * NN);   // [nrowG + nrep]
  float *red = reinterpret_cast<float *>(rowS + (L.nrowG + L.nrep));  // [G][NT][16]
  for (int i = threadIdx.x; i < L.nrowG + L.nrep; i += blockDim.x) rowS[i] = p.rowS[i];

  const int kp = blockIdx.x;
  const int uy = kp / p.fq, ux = kp % p.fq;
  const int us = uy ? p.f - uy : 0;
  const bool selfp = (us == uy);
  const int ffh = p.f * p.fh;
  const int tid = threadIdx.x;
  const int g = tid / NT, o = tid % NT;
  const bool active = g < p.G;
  const int kind = (o < c2) ? 0 : ((o < c2 + c) ? 1 : ((o < c2 + 2 * c) ? 2 : 3));
  const int slotbase = (kind == 0) ? 4 * o
                      : (kind == 1) ? 4 * c2 + 2 * (o - c2)
                      : (kind == 2) ? 4 * c2 + 2 * c + 2 * (o - c2 - c)
                                    : NN - 1;

  float2 U[TF][4], V[TF][4];
#pragma unroll
  for (int tf = 0; tf < TF; tf++)
#pragma unroll
    for (int k = 0; k < 4; k++) { U[tf][k] = make_float2(0.f, 0.f); V[tf][k] = make_float2(0.f, 0.f); }

  int z0, z1;
  if (FWD) { z0 = blockIdx.y * p.zgroup; z1 = min(z0 + p.zgroup, p.nz); }
  else { z0 = blockIdx.y; z1 = z0 + 1; }

  for (int zi = z0; zi < z1; zi++) {
    __syncthreads();
    const int zs = FWD ? zi : 0;
    for (int idx = tid; idx < TF * NN; idx += blockDim.x) {
      const int t = idx / NN, i = idx % NN;
      float2 a = make_float2(0.f, 0.f), b = make_float2(0.f, 0.f);
      if (t < p.T) {
        const float2 *sb = p.S + ((long long)(t * p.nzS + zs) * NN + i) * ffh;
        a = sb[uy * p.fh + ux];
        b = sb[us * p.fh + ux];
      }
      comb[t * 2 * NN + i] = a;
      comb[t * 2 * NN + NN + i] = b;
    }
    __syncthreads();
    if (active) {
      const int plane = p.planes[zi];
      const float2 *Pk = p.P + ((long long)plane * p.nkp + kp) * (long long)L.nrow * L.RS + slotbase;
      switch (kind) {
        case 0: mac_rows<TF, 0>(Pk, comb, rowS, L, g, p.G, U, V); break;
        case 1: mac_rows<TF, 1>(Pk, comb, rowS, L, g, p.G, U, V); break;
        case 2: mac_rows<TF, 2>(Pk, comb, rowS, L, g, p.G, U, V); break;
        default: mac_rows<TF, 3>(Pk, comb, rowS, L, g, p.G, U, V); break;
      }
    }
  }

  const int ns = (kind == 0) ? 4 : ((kind == 3) ? 1 : 2);
  const int zo = FWD ? blockIdx.y : z0;
#pragma unroll
  for (int tf = 0; tf < TF; tf++) {
    __syncthreads();
    if (active) {
      float *rp = red + (g * NT + o) * 16;
#pragma unroll
      for (int k = 0; k < 4; k++) {
        rp[2 * k] = U[tf][k].x; rp[2 * k + 1] = U[tf][k].y;
        rp[8 + 2 * k] = V[tf][k].x; rp[8 + 2 * k + 1] = V[tf][k].y;
      }
    }
    __syncthreads();
    if (g == 0 && tf < p.T) {
      float s[16];
#pragma unroll
      for (int e = 0; e < 16; e++) s[e] = 0.f;
      for (int gg = 0; gg < p.G; gg++) {
        const float *rp = red + (gg * NT + o) * 16;
#pragma unroll
        for (int e = 0; e < 16; e++) s[e] += rp[e];
      }
      long long obase;
      if (FWD) obase = ((long long)(zo * p.T + tf) * NN) * ffh;
      else obase = ((long long)(tf * p.nzo + zo) * NN) * ffh;
      for (int k = 0; k < ns; k++) {
        const int q = p.slotcol[slotbase + k];
        float2 *op = p.O + obase + (long long)q * ffh;
        if (selfp) {
          op[uy * p.fh + ux] = make_float2(s[2 * k] + s[8 + 2 * k], s[2 * k + 1] + s[8 + 2 * k + 1]);
        } else {
          op[uy * p.fh + ux] = make_float2(s[2 * k], s[2 * k + 1]);
          op[us * p.fh + ux] = make_float2(s[8 + 2 * k], s[8 + 2 * k + 1]);
        }
      }
    }
  }
}

// ----------------------------------------------------------------------------
// Precompute: lenslet-grid kernels K_iq (real f x f images, circular) built
// from the stored PSF quadrant through the reference's symmetry map
// (projector.py:159-189): offset (b, a) uses H[bb][aa] (aa >= bb) or the
// transpose of H[aa][bb], flipped along rows when b > c and columns when a > c.
// ----------------------------------------------------------------------------
template <typename R>
__global__ void k_build_k(BuildKParams p) {
  const int N = p.N, NN = N * N, c = N / 2, nh = c + 1, h = p.h, f = p.f, Rr = p.R;
  const int img = blockIdx.x;             // rl * NN + q
  const int rl = img / NN, q = img % NN;
  const int i = p.rep_ch[p.rep0 + rl];
  const int b = i / N, a = i % N, be = q / N, al = q % N;
  const int bb = min(b, N - 1 - b), aa = min(a, N - 1 - a);
  R *dst = reinterpret_cast<R *>(p.dst) + (long long)img * f * f;
  for (int e = threadIdx.x; e < f * f; e += blockDim.x) {
    const int mm = e / f, nn = e % f;
    const int m = (mm <= Rr) ? mm : ((mm >= f - Rr) ? mm - f : 1 << 20);
    const int n = (nn <= Rr) ? nn : ((nn >= f - Rr) ? nn - f : 1 << 20);
    R v = 0;
    if (m < (1 << 19) && n < (1 << 19)) {
      const int y = m * N + be - b + p.ch;
      const int x = n * N + al - a + p.ch;
      if (y >= 0 && y < h && x >= 0 && x < h) {
        const int yy = (b > c) ? h - 1 - y : y;
        const int xx = (a > c) ? h - 1 - x : x;
        float hv;
        if (aa >= bb) hv = p.H[((long long)(bb * nh + aa) * h + yy) * h + xx];
        else hv = p.H[((long long)(aa * nh + bb) * h + xx) * h + yy];
        v = (R)hv;
      }
    }
    dst[e] = v;
  }
}

template <typename R>
__global__ void k_pack(PackParams p) {
  typedef typename CT<R>::T C;
  const Layout &L = p.L;
  const int NN = L.NN, ffh = p.f * p.fh;
  const long long total = (long long)p.nrep_chunk * NN * p.nkp;
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < total;
       idx += (long long)gridDim.x * blockDim.x) {
    const int q = (int)(idx % NN);
    const long long r2 = idx / NN;
    const int rl = (int)(r2 % p.nrep_chunk);
    const int kp = (int)(r2 / p.nrep_chunk);
    const int uy = kp / p.fq, ux = kp % p.fq;
    const int us = uy ? p.f - uy : 0;
    const bool selfp = (us == uy);
    const int rep = p.rep0 + rl;
    const int kind = p.rep_kind[rep];
    const int row = p.rep_row[rep];
    const int ch = p.rep_ch[rep];
    const C *sp = reinterpret_cast<const C *>(p.spec) + ((long long)rl * NN + q) * ffh;
    const int slot = p.col_slot[q];
    float2 *dst = p.P + ((long long)kp * L.nrow + row) * L.RS + slot;
    const R sc = (R)p.scale;
    const C a = sp[uy * p.fh + ux];
    if (kind == 0) {
      const bool zero = selfp && ((ch % L.N) > L.c);
      dst[0] = zero ? make_float2(0.f, 0.f) : make_float2((float)(a.x * sc), (float)(a.y * sc));
    } else {
      dst[0] = make_float2((float)(a.x * sc), (float)(a.y * sc));
      const C b = sp[us * p.fh + ux];
      dst[L.RS] = selfp ? make_float2(0.f, 0.f) : make_float2((float)(b.x * sc), (float)(b.y * sc));
    }
  }
}

// ----------------------------------------------------------------------------
// Launchers
// ----------------------------------------------------------------------------
size_t rfft2_smem_bytes(int f, int imgs, int fp64) {
  const size_t cs = fp64 ? sizeof(double2) : sizeof(float2);
  const size_t isz = (size_t)f * (f / 2 + 1);
  return cs * ((size_t)f + 2 * (size_t)imgs * isz);
}
size_t irfft2_smem_bytes(int f, int imgs) { return rfft2_smem_bytes(f, imgs, 0); }

static cudaError_t set_smem(const void *fn, size_t bytes) {
  return cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

cudaError_t launch_rfft2(const Rfft2Params &p, int fp64, cudaStream_t s) {
  const size_t sm = rfft2_smem_bytes(p.plan.n, p.imgs_per_cta, fp64);
  const int grid = (p.nimg + p.imgs_per_cta - 1) / p.imgs_per_cta;
  if (grid == 0) return cudaSuccess;
  cudaError_t e;
  if (fp64) {
    if ((e = set_smem((const void *)k_rfft2<double>, sm)) != cudaSuccess) return e;
    k_rfft2<double><<<grid, 256, sm, s>>>(p);
  } else {
    if ((e = set_smem((const void *)k_rfft2<float>, sm)) != cudaSuccess) return e;
    k_rfft2<float><<<grid, 256, sm, s>>>(p);
  }
  return cudaGetLastError();
}

cudaError_t launch_irfft2(const Irfft2Params &p, cudaStream_t s) {
  const size_t sm = irfft2_smem_bytes(p.plan.n, p.imgs_per_cta);
  const int grid = (p.nimg + p.imgs_per_cta - 1) / p.imgs_per_cta;
  if (grid == 0) return cudaSuccess;
  cudaError_t e = set_smem((const void *)k_irfft2, sm);
  if (e != cudaSuccess) return e;
  k_irfft2<<<grid, 256, sm, s>>>(p);
  return cudaGetLastError();
}

int mac_max_frames() { return 4; }

template <int TF>
static cudaError_t launch_mac_tf(const MacParams &p, bool fwd, cudaStream_t s) {
  const Layout &L = p.L;
  const size_t sm = sizeof(float2) * TF * 2 * L.NN + sizeof(short4) * (L.nrowG + L.nrep) +
                    sizeof(float) * (size_t)p.G * L.nthr * 16;
  dim3 grid(p.nkp, p.nzo);
  const int block = p.G * L.nthr;
  cudaError_t e;
  if (fwd) {
    if ((e = set_smem((const void *)k_mac<TF, true>, sm)) != cudaSuccess) return e;
    k_mac<TF, true><<<grid, block, sm, s>>>(p);
  } else {
    if ((e = set_smem((const void *)k_mac<TF, false>, sm)) != cudaSuccess) return e;
    k_mac<TF, false><<<grid, block, sm, s>>>(p);
  }
  return cudaGetLastError();
}

cudaError_t launch_mac(const MacParams &p, bool forward, cudaStream_t s) {
  if (p.T <= 1) return launch_mac_tf<1>(p, forward, s);
  if (p.T <= 2) return launch_mac_tf<2>(p, forward, s);
  return launch_mac_tf<4>(p, forward, s);
}

cudaError_t launch_build_k(const BuildKParams &p, int nimg, cudaStream_t s) {
  if (nimg == 0) return cudaSuccess;
  if (p.fp64) k_build_k<double><<<nimg, 256, 0, s>>>(p);
  else k_build_k<float><<<nimg, 256, 0, s>>>(p);
  return cudaGetLastError();
}

cudaError_t launch_pack(const PackParams &p, cudaStream_t s) {
  const long long total = (long long)p.nrep_chunk * p.L.NN * p.nkp;
  if (total == 0) return cudaSuccess;
  long long blocks = (total + 255) / 256;
  if (blocks > 65535LL * 16) blocks = 65535LL * 16;
  if (p.fp64) k_pack<double><<<(unsigned)blocks, 256, 0, s>>>(p);
  else k_pack<float><<<(unsigned)blocks, 256, 0, s>>>(p);
  return cudaGetLastError();
}

}  // namespace flf
