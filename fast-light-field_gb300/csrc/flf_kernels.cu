// CUDA kernels of libflf.so (sm_103a): lenslet-grid FFTs, the fused spectral
// multiply-accumulate over planes and lenslet offsets, inverse transform with
// crop / plane reduction / Richardson-Lucy epilogues, and the PSF transfer
// matrix precompute.  Host code that sequences them is flf_api.cu.
#include "flf_internal.cuh"
#include "flf_fft.cuh"

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
// Forward real 2-D transform f x f -> f x (f/2+1) of contiguous images, in
// float or double (the transfer-matrix precompute; the hot-path transforms are
// the size-specialised kernels of flf_fft.cuh).  Two real rows are packed into
// one complex row for the row pass and split afterwards.
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

  for (int idx = threadIdx.x; idx < nb * nq * f; idx += blockDim.x) {
    const int c = idx % f;
    const int q = (idx / f) % nq;
    const int img = idx / (f * nq);
    const R *im = reinterpret_cast<const R *>(p.src_img) + (long long)(g0 + img) * f * f;
    A[img * isz + q * f + c] = cmk<C>(im[(2 * q) * f + c], im[(2 * q + 1) * f + c]);
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
// ---------------------------------------------------------------------------
// Bulk-copy pipeline primitives (sm_90+ PTX: mbarrier, cp.async.bulk).
// Every wait is bounded by a wall-clock limit read from %globaltimer.
// ---------------------------------------------------------------------------
__device__ __forceinline__ unsigned smem_u32(const void *ptr) {
  return (unsigned)__cvta_generic_to_shared(ptr);
}
__device__ __forceinline__ void mbar_init(unsigned long long *bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(unsigned long long *bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void mbar_arrive(unsigned long long *bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];\n" ::"r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(unsigned long long *bar, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;\n" : "=l"(t));
  return t;
}
// Wait for phase `parity` of `bar`; false after `limit_ns` nanoseconds.
__device__ __forceinline__ bool mbar_wait(unsigned long long *bar, unsigned parity,
                                          unsigned long long limit_ns) {
  if (mbar_try_wait(bar, parity)) return true;
  const unsigned long long t0 = global_ns();
  while (!mbar_try_wait(bar, parity))
    if (global_ns() - t0 > limit_ns) return false;
  return true;
}
// Global -> shared bulk copy completing `bytes` of transaction count on `bar`.
__device__ __forceinline__ void bulk_g2s(void *sdst, const void *gsrc, unsigned bytes,
                                         unsigned long long *bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::"r"(
          smem_u32(sdst)),
      "l"(gsrc), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}

// Orders this thread's earlier generic-proxy shared-memory accesses (as seen
// through a CTA fence) before its later async-proxy (bulk copy) accesses.
__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
}

constexpr unsigned long long kWaitLimitNs = 1000000000ull;   // 1 s per wait

// Loads the four virtual slots [q, My q, Mx q, Mxy q] of this thread's orbit
// from one staged row at the thread's slot offsets.  Degenerate orbits repeat
// their stored entries (alpha = c: [q, My q, q, My q]; beta = c:
// [q, q, Mx q, Mx q]; centre: [q] x 4), so every thread runs the same 4-slot
// update with no branch (the padded slots compute duplicates that are never
// written).
__device__ __forceinline__ void load_slots(const float2 *row, const int (&off)[4], float2 (&t)[4]) {
#pragma unroll
  for (int k = 0; k < 4; k++) t[k] = row[off[k]];
}

// Slot permutations of the orbit [q, My q, Mx q, Mxy q].
__device__ __forceinline__ constexpr int sy(int k) { return k ^ 1; }
__device__ __forceinline__ constexpr int sx(int k) { return k ^ 2; }
__device__ __forceinline__ constexpr int sxy(int k) { return 3 - k; }

// Packed two-lane FP32 arithmetic (sm_100+): __ffma2_rn performs two
// independent IEEE fused multiply-adds in one instruction, halving the issue
// slots of the complex multiply-accumulate.  f2x is the two-lane value.
typedef float2 f2x;
__device__ __forceinline__ f2x pk(float lo, float hi) { return make_float2(lo, hi); }
__device__ __forceinline__ float2 unpk(f2x v) { return v; }
__device__ __forceinline__ void ffma2(f2x &acc, f2x a, f2x b) { acc = __ffma2_rn(a, b, acc); }

// Per row group, the input spectra enter as four packed operand pairs
// (A_j, B_j), j = 0..3.  Each complex accumulator is kept as two lane pairs
// P and Q with value (P.x - Q.y, P.y + Q.x), so that with t = (t.x, t.y)
//   acc += t * s        is  P = fma2(t, (s.x, s.x)), Q = fma2(t, (s.y, s.y))
//   acc += conj(t) * s  is  P = fma2(t, (s.x,-s.x)), Q = fma2(t, (s.y,-s.y))
// and no lane swap of t is needed.  sv[tf][side][use][group][j] = float4(A_j, B_j)
// for the threads of frequency pair `side` reading a group of their own half
// block (use 0) or of the other half block through the transpose (use 1);
// built from comb once per plane.  An operand is zero where its flags say so,
// or where the receiving pair is self-paired (u = u*) and the term would be
// counted twice.
__device__ void build_sv(float4 *sv, const float2 *comb, const short4 *rowS, const short *rowF, const Layout &L,
                         int TF, bool selfp0, bool selfp1) {
  const int G = L.ngrp, NN2 = 2 * L.NN;
  for (int idx = threadIdx.x; idx < TF * 4 * G * 4; idx += blockDim.x) {
    const int j = idx & 3;
    const int g = (idx >> 2) % G;
    const int su = ((idx >> 2) / G) & 3;          // side * 2 + use
    const int tf = (idx >> 2) / (4 * G);
    const int side = su >> 1, use = su & 1;
    const short4 si = rowS[use * G + g];
    const int fl = rowF[use * G + g];
    const int ci = (j == 0) ? si.x : (j == 1) ? si.y : (j == 2) ? si.z : si.w;
    const bool conj = (fl >> j) & 1;
    const bool zero = ((fl >> (8 + j)) & 1) || ((side ? selfp1 : selfp0) && ((fl >> (4 + j)) & 1));
    const float2 sc = zero ? make_float2(0.f, 0.f) : comb[(tf * 2 + side) * NN2 + ci];
    sv[idx] = conj ? make_float4(sc.x, -sc.x, sc.y, -sc.y) : make_float4(sc.x, sc.x, sc.y, sc.y);
  }
}

// Split accumulators of one thread: U (frequency u) and V (u*) for the four
// virtual slots of its orbit and each frame, as P / Q lane pairs.
template <int TF> struct MacAcc {
  f2x UP[TF][4], UQ[TF][4], VP[TF][4], VQ[TF][4];
  __device__ __forceinline__ void zero() {
#pragma unroll
    for (int tf = 0; tf < TF; tf++)
#pragma unroll
      for (int k = 0; k < 4; k++) {
        UP[tf][k] = make_float2(0.f, 0.f); UQ[tf][k] = make_float2(0.f, 0.f);
        VP[tf][k] = make_float2(0.f, 0.f); VQ[tf][k] = make_float2(0.f, 0.f);
      }
  }
};
__device__ __forceinline__ float2 pq_value(f2x P, f2x Q) { return make_float2(P.x - Q.y, P.y + Q.x); }

// One generic stored row t (input channel i at u): feeds channel i at u,
// Mxy i at u, My i at u*, Mx i at u*.
// SW: the thread's virtual slots are those of a transposed orbit, [r, Mx r,
// My r, Mxy r], so the My and Mx slot permutations trade places.
template <int TF, bool SW>
__device__ __forceinline__ void mac_generic_row(const float2 (&t)[4], const float4 *svr, int svstride,
                                                MacAcc<TF> &a) {
#pragma unroll
  for (int tf = 0; tf < TF; tf++) {
    const float4 q0 = svr[tf * svstride + 0], q1 = svr[tf * svstride + 1];
    const float4 q2 = svr[tf * svstride + 2], q3 = svr[tf * svstride + 3];
    const f2x A0 = pk(q0.x, q0.y), B0 = pk(q0.z, q0.w), A1 = pk(q1.x, q1.y), B1 = pk(q1.z, q1.w);
    const f2x A2 = pk(q2.x, q2.y), B2 = pk(q2.z, q2.w), A3 = pk(q3.x, q3.y), B3 = pk(q3.z, q3.w);
#pragma unroll
    for (int k = 0; k < 4; k++) {
      ffma2(a.UP[tf][k], t[k], A0);
      ffma2(a.UQ[tf][k], t[k], B0);
      ffma2(a.UP[tf][k], t[sxy(k)], A1);
      ffma2(a.UQ[tf][k], t[sxy(k)], B1);
      ffma2(a.VP[tf][SW ? sx(k) : sy(k)], t[k], A2);
      ffma2(a.VQ[tf][SW ? sx(k) : sy(k)], t[k], B2);
      ffma2(a.VP[tf][SW ? sy(k) : sx(k)], t[k], A3);
      ffma2(a.VQ[tf][SW ? sy(k) : sx(k)], t[k], B3);
    }
  }
}

// A centre-cross row pair (t at u, s at u*) of representative kind rk.
template <int TF, bool SW>
__device__ __forceinline__ void mac_pair_rows(const float2 (&t)[4], const float2 (&s)[4], int rk,
                                              const float4 *svr, int svstride, MacAcc<TF> &a) {
#pragma unroll
  for (int tf = 0; tf < TF; tf++) {
    const float4 q0 = svr[tf * svstride + 0], q1 = svr[tf * svstride + 1];
    const f2x A0 = pk(q0.x, q0.y), B0 = pk(q0.z, q0.w), A1 = pk(q1.x, q1.y), B1 = pk(q1.z, q1.w);
#pragma unroll
    for (int k = 0; k < 4; k++) {
      ffma2(a.UP[tf][k], t[k], A0);
      ffma2(a.UQ[tf][k], t[k], B0);
      ffma2(a.VP[tf][k], s[k], A1);
      ffma2(a.VQ[tf][k], s[k], B1);
    }
    if (rk != 3) {
      const float4 q2 = svr[tf * svstride + 2], q3 = svr[tf * svstride + 3];
      const f2x A2 = pk(q2.x, q2.y), B2 = pk(q2.z, q2.w), A3 = pk(q3.x, q3.y), B3 = pk(q3.z, q3.w);
      if ((rk == 1) != SW) {   // My partner (rk 1) or Mx partner (rk 2), in this thread's slot order
#pragma unroll
        for (int k = 0; k < 4; k++) {
          ffma2(a.VP[tf][sy(k)], t[k], A2);
          ffma2(a.VQ[tf][sy(k)], t[k], B2);
          ffma2(a.UP[tf][sy(k)], s[k], A3);
          ffma2(a.UQ[tf][sy(k)], s[k], B3);
        }
      } else {
#pragma unroll
        for (int k = 0; k < 4; k++) {
          ffma2(a.VP[tf][sx(k)], t[k], A2);
          ffma2(a.VQ[tf][sx(k)], t[k], B2);
          ffma2(a.UP[tf][sx(k)], s[k], A3);
          ffma2(a.UQ[tf][sx(k)], s[k], B3);
        }
      }
    }
  }
}

// Asynchronous 8-byte global -> shared copy (completes at cp.async.wait_all).
__device__ __forceinline__ void cp_async8(void *smem, const void *gmem) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(smem_u32(smem)), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

// Stage the input spectra of plane slot `zs` at the four frequencies of the
// quad into shared memory: comb[t][side][i] = S_i[u_side], comb[t][side][NN + i]
// = S_i[u_side*], with u_0 = (uy, ux), u_1 = (ux, uy) (rows py, ps; column px).
__device__ __forceinline__ void stage_comb(float2 *comb, const MacParams &p, int TF, int zs, int uy, int ux) {
  const int us = uy ? p.f - uy : 0, vs = ux ? p.f - ux : 0;
  const int NN = p.L.NN, ffh = p.f * p.fh;
  for (int idx = threadIdx.x; idx < TF * 2 * NN; idx += blockDim.x) {
    const int i = idx % NN;
    const int side = (idx / NN) & 1;
    const int t = idx / (2 * NN);
    float2 *dst = comb + (t * 2 + side) * 2 * NN;
    if (t < p.T) {
      const float2 *sb = p.S + ((long long)(t * p.nzS + zs) * NN + i) * ffh;
      const int fy = side ? ux : uy, fys = side ? vs : us, fx = side ? uy : ux;
      cp_async8(dst + i, sb + fy * p.fh + fx);
      cp_async8(dst + NN + i, sb + fys * p.fh + fx);
    } else {
      dst[i] = make_float2(0.f, 0.f);
      dst[NN + i] = make_float2(0.f, 0.f);
    }
  }
  cp_async_commit();
}

// Shared memory of k_mac: ring | sv | scratch (comb staging, later the
// share and side reduction) | rowS | rowF | mbarriers.
__host__ __device__ inline size_t mac_scratch_elems(const Layout &L, int TF, int split, bool fwd) {
  const size_t comb = (size_t)(fwd ? 2 : 1) * TF * 2 * 2 * L.NN;                    // float2
  const size_t red = (size_t)(2 * split - 1) * ((L.nthr + 31) / 32 * 32) * 8 * TF;   // f2x = 8 B
  return comb > red ? comb : red;
}

size_t mac_smem_bytes(const Layout &L, int TF, int stages, int chunk_rows, int split, bool fwd) {
  return sizeof(float2) * ((size_t)stages * chunk_rows * L.RS + mac_scratch_elems(L, TF, split, fwd)) +
         sizeof(float4) * (size_t)TF * 4 * L.ngrp * 4 + sizeof(short4) * 2 * L.ngrp + sizeof(short) * 2 * L.ngrp +
         2 * sizeof(unsigned long long) * stages + 16;
}

// Launch bounds: blocks of at most 128 threads (orbit groups of Nnum <= 15
// with a row split of 2) or of at most 256, and the CTAs per SM the register
// budget is sized for.
template <int TF, bool WIDE> struct MacOcc {
  static constexpr int threads = WIDE ? 256 : 128;
  static constexpr int v = WIDE ? (TF == 1 ? 2 : 1) : (TF == 1 ? 4 : (TF == 2 ? 3 : 2));
};

// One CTA = one frequency quad {(uy, ux), (ux, uy)} and a group of planes.
// The threads form two sides, one per frequency pair of the quad; thread
// (side, h, o) owns the mirror orbit o of output channels at its pair's
// frequencies u and u* for the rows of its share h (rows are dealt round-robin
// to the `split` threads of an orbit).  Every stored row of the quad's half
// blocks streams through shared memory once and feeds both sides: the side it
// belongs to through the thread's own orbit slots, and (for transposable
// groups) the other side through the slots of the transposed orbit, since
// T_{Tr i, Tr j}[(uy, ux)] = T_ij[(ux, uy)].  Shares (and, for a diagonal quad,
// whose two sides are the same pair, the sides) are added through shared
// memory when a plane's output is due, so there is no atomic and every output
// is written by exactly one thread.
// The stored rows stream through a ring of shared-memory stages filled by
// bulk copies (crossing plane boundaries).  Forward projection accumulates the
// planes of the group (the group sums are added by the inverse transform);
// back projection writes each plane's spectra when the plane is done.  The
// spectra of the next plane are staged with cp.async while the current plane
// streams.
template <int TF, bool FWD, bool WIDE>
__global__ void __launch_bounds__(MacOcc<TF, WIDE>::threads, MacOcc<TF, WIDE>::v) k_mac(MacParams p) {
  extern __shared__ __align__(16) unsigned char smraw[];
  __shared__ int s_abort;
  __shared__ int s_issued;                      // chunks handed to the bulk-copy engine
  __shared__ int s_plane[kMacMaxZgroup];        // plane slots of this CTA's z range
  volatile int *abortf = &s_abort;
  const Layout &L = p.L;
  const int NN = L.NN, NT = L.nthr, RS = L.RS, NN2 = 2 * L.NN, G = L.ngrp, c = L.c;
  const int CH = p.chunk_rows, NST = p.stages, H = p.split;
  const int NTP = (NT + 31) / 32 * 32;
  float2 *ring = reinterpret_cast<float2 *>(smraw);                          // [NST][CH*RS]
  float4 *sv = reinterpret_cast<float4 *>(ring + (size_t)NST * CH * RS);     // [TF][2][2][G][4]
  float2 *scratch = reinterpret_cast<float2 *>(sv + TF * 4 * G * 4);        // comb [1|2][TF][2][2NN] / red
  f2x *red = reinterpret_cast<f2x *>(scratch);                              // [2H-1][NTP][TF][8]
  short4 *rowS = reinterpret_cast<short4 *>(scratch + mac_scratch_elems(L, TF, H, FWD));
  short *rowF = reinterpret_cast<short *>(rowS + 2 * G);
  unsigned long long *full = reinterpret_cast<unsigned long long *>(
      (reinterpret_cast<uintptr_t>(rowF + 2 * G) + 7) & ~(uintptr_t)7);
  int *released = reinterpret_cast<int *>(full + NST);   // [NST] warps done with each slot, ever

  const int tid = threadIdx.x;
  const int nwarps = (blockDim.x + 31) >> 5;
  if (tid == 0) {
    for (int i = 0; i < NST; i++) {
      mbar_init(full + i, 1);
      released[i] = 0;
    }
    *abortf = 0;
    s_issued = 0;
    fence_mbar_init();
  }
  for (int i = tid; i < 2 * G; i += blockDim.x) {
    rowS[i] = p.rowS[i];
    rowF[i] = p.rowF[i];
  }
  {
    const int zb = blockIdx.y * p.zgroup, nzl = min(p.zgroup, p.nz - zb);
    for (int i = tid; i < nzl; i += blockDim.x) s_plane[i] = p.planes[zb + i];
  }

  // quad k = ux (ux + 1) / 2 + uy, uy <= ux
  const int kq = blockIdx.x;
  int ux = (int)((sqrtf(8.f * (float)kq + 1.f) - 1.f) * 0.5f);
  while ((ux + 1) * (ux + 2) / 2 <= kq) ux++;
  while (ux * (ux + 1) / 2 > kq) ux--;
  const int uy = kq - ux * (ux + 1) / 2;
  const bool diag = (uy == ux);
  const int hb0 = 2 * kq - ux;                   // first half block of the quad
  const int nhalf = diag ? 1 : 2;
  const bool selfp0 = (uy == 0) || (2 * uy == p.f), selfp1 = (ux == 0) || (2 * ux == p.f);
  const int ffh = p.f * p.fh;
  const int HS = H * NTP;                        // threads per side
  const int ts = tid / HS;                       // side of this thread
  const int h = (tid - ts * HS) / NTP, o = tid - ts * HS - h * NTP;
  const bool active = o < NT;
  const int kind = (o < c * c) ? 0 : ((o < c * c + c) ? 1 : ((o < c * c + 2 * c) ? 2 : 3));
  // virtual slots of orbit o: every half block is read at these (side 1 owns
  // the transposed orbit, its half block is stored in transposed column order)
  int off[4];
  {
    const short4 a = p.oslots[active ? o : 0];
    off[0] = a.x; off[1] = a.y; off[2] = a.z; off[3] = a.w;
  }
  const int ns = (kind == 0) ? 4 : ((kind == 3) ? 1 : 2);
  const int z0 = blockIdx.y * p.zgroup;
  const int z1 = min(z0 + p.zgroup, p.nz);
  const int nrq = nhalf * L.nrow;                // stored rows of the quad per plane
  const int cpb = (nrq + CH - 1) / CH;           // chunks per (quad, plane)
  const int total = (z1 - z0) * cpb;
  const size_t halfElems = (size_t)L.nrow * RS;
  const int combStride = TF * 2 * NN2;           // one plane's staged spectra (float2)
  const int svs = 4 * G * 4;                     // sv stride between frames (float4)

  MacAcc<TF> acc;
  acc.zero();

  stage_comb(scratch, p, TF, FWD ? z0 : 0, uy, ux);
  cp_async_wait_all();
  __syncthreads();   // barriers initialised, row tables and first spectra staged
  build_sv(sv, scratch, rowS, rowF, L, TF, selfp0, selfp1);
  __syncthreads();   // (back projection: the staging area is free for the reduction)

  // Chunk g goes to ring slot g % NST.  Thread 0 fills the whole ring; after
  // that, the warp that releases a slot last (each warp counts itself out
  // once it has finished its rows of the chunk) refills it at once with chunk
  // g + NST, so no thread ever waits for a slot to drain.
  // p.drop_chunk >= 0 (a test of the bounded waits only): the first CTA never
  // issues that chunk, so the waits on its slot run out after p.wait_ns
  const int drop = blockIdx.x == 0 && blockIdx.y == 0 ? p.drop_chunk : -1;
  auto issue = [&](int gn) {
    if (gn == drop) return;
    const int zl_n = gn / cpb, ch_n = gn - zl_n * cpb, sl = gn % NST;
    const int r0 = ch_n * CH;
    const int nr = min(CH, nrq - r0);
    const float2 *src = p.P + ((long long)s_plane[zl_n] * p.nkp + hb0) * (long long)halfElems + (long long)r0 * RS;
    const unsigned bytes = (unsigned)(nr * RS * sizeof(float2));
    mbar_arrive_expect_tx(full + sl, bytes);
    bulk_g2s(ring + (size_t)sl * CH * RS, src, bytes, full + sl);
  };
  if (tid == 0) {
    const int pre = min(NST, total);
    for (int g = 0; g < pre; g++) issue(g);
    s_issued = pre;
  }

  bool dead = false;
  int zl = 0, ch = 0, slot = 0;
  int round = 0;
  for (int g = 0; g < total; g++) {
    const int zi = z0 + zl;
    if (FWD && ch == 0) {
      if (zl > 0) {
        cp_async_wait_all();
        __syncthreads();   // spectra of plane zi staged; all threads done with plane zi-1
        build_sv(sv, scratch + (zl & 1) * combStride, rowS, rowF, L, TF, selfp0, selfp1);
        __syncthreads();
      }
      if (zi + 1 < z1) stage_comb(scratch + ((zl + 1) & 1) * combStride, p, TF, zi + 1, uy, ux);
    }
    if (*abortf) dead = true;
    if (!dead && !mbar_wait(full + slot, round & 1, p.wait_ns)) {
      dead = true;
      *abortf = 1;
      atomicExch(p.err, 2);
    }
    if (!dead && active) {
      const int r0 = ch * CH;
      const int r1 = min(nrq, r0 + CH);
      const float2 *stage = ring + (size_t)slot * CH * RS;
      // the chunk's rows, one half block at a time
      for (int bs = r0 / L.nrow; bs * L.nrow < r1; bs++) {
        const int base = bs * L.nrow;
        const int lo = max(r0, base) - base, hi = min(r1, base + L.nrow) - base;   // half-block rows
        const int use = (bs == ts) ? 0 : 1;       // warp-uniform: a side is whole warps
        const float4 *svb = sv + (ts * 2 + use) * G * 4;
        const float2 *srow = stage + (base - r0) * RS;
        // generic rows (through the transpose only the first nrowGT), then row pairs
        const int rg = min(hi, use ? L.nrowGT : L.nrowG);
        const int pr1 = min(hi, use ? L.nrowG + 2 * c : L.nrow);
        const int pr0 = max(lo, L.nrowG);
        if (ts == 0) {
#pragma unroll 2
          for (int r = lo + h; r < rg; r += H) {
            float2 t[4];
            load_slots(srow + (size_t)r * RS, off, t);
            mac_generic_row<TF, false>(t, svb + r * 4, svs, acc);
          }
          for (int r = pr0 + 2 * h; r < pr1; r += 2 * H) {
            const int k2 = (r - L.nrowG) >> 1;
            float2 t[4], s2[4];
            load_slots(srow + (size_t)r * RS, off, t);
            load_slots(srow + (size_t)(r + 1) * RS, off, s2);
            mac_pair_rows<TF, false>(t, s2, use ? 2 : ((k2 < c) ? 1 : 3), svb + (L.nrowG + k2) * 4, svs, acc);
          }
        } else {
#pragma unroll 2
          for (int r = lo + h; r < rg; r += H) {
            float2 t[4];
            load_slots(srow + (size_t)r * RS, off, t);
            mac_generic_row<TF, true>(t, svb + r * 4, svs, acc);
          }
          for (int r = pr0 + 2 * h; r < pr1; r += 2 * H) {
            const int k2 = (r - L.nrowG) >> 1;
            float2 t[4], s2[4];
            load_slots(srow + (size_t)r * RS, off, t);
            load_slots(srow + (size_t)(r + 1) * RS, off, s2);
            mac_pair_rows<TF, true>(t, s2, use ? 2 : ((k2 < c) ? 1 : 3), svb + (L.nrowG + k2) * 4, svs, acc);
          }
        }
      }
    }
    __syncwarp();
    if ((tid & 31) == 0 && !dead) {
      __threadfence_block();                       // this warp's reads of the slot come first
      const int before = atomicAdd(released + slot, 1);
      if (before == round * nwarps + nwarps - 1 && g + NST < total && !*abortf) {
        __threadfence_block();
        fence_proxy_async_smem();                  // ... before the bulk copy that overwrites it
        issue(g + NST);
        atomicAdd(&s_issued, 1);
      }
    }

    const bool out_due = (ch == cpb - 1) && (!FWD || zi + 1 == z1);
    if (out_due) {
      f2x U[TF][4], V[TF][4];
#pragma unroll
      for (int tf = 0; tf < TF; tf++)
#pragma unroll
        for (int k = 0; k < 4; k++) {
          U[tf][k] = pq_value(acc.UP[tf][k], acc.UQ[tf][k]);
          V[tf][k] = pq_value(acc.VP[tf][k], acc.VQ[tf][k]);
        }
      // writers: share 0 of each side, or of side 0 only for a diagonal quad
      // (its two sides are the same frequency pair); the others add into them
      const bool writer = (h == 0) && (!diag || ts == 0);
      if (H > 1 || diag) {
        if (FWD) cp_async_wait_all();   // the staging area doubles as reduction buffer
        __syncthreads();
        if (!writer && active) {
          const int idx = diag ? ts * H + h - 1 : ts * (H - 1) + h - 1;
          // in a diagonal quad, side 1's orbit is the transposed orbit T(o) of side 0,
          // with its My and Mx slots swapped
          int ot = o;
          if (diag && ts) {
            const int c2 = c * c;
            ot = (o < c2) ? (o % c) * c + o / c : ((o < c2 + c) ? o + c : ((o < c2 + 2 * c) ? o - c : o));
          }
          f2x *rp = red + ((size_t)idx * NTP + ot) * TF * 8;
#pragma unroll
          for (int tf = 0; tf < TF; tf++)
#pragma unroll
            for (int k = 0; k < 4; k++) {
              const int kk = (diag && ts) ? ((k == 1) ? 2 : ((k == 2) ? 1 : k)) : k;
              rp[tf * 8 + kk] = U[tf][k];
              rp[tf * 8 + 4 + kk] = V[tf][k];
            }
        }
        __syncthreads();
        if (writer && active) {
          const int n0 = diag ? 0 : ts * (H - 1), n1 = diag ? 2 * H - 1 : n0 + H - 1;
          for (int idx = n0; idx < n1; idx++) {
            const f2x *rp = red + ((size_t)idx * NTP + o) * TF * 8;
#pragma unroll
            for (int tf = 0; tf < TF; tf++)
#pragma unroll
              for (int k = 0; k < 4; k++) {
                const float2 a = unpk(U[tf][k]), b = unpk(rp[tf * 8 + k]);
                const float2 cc2 = unpk(V[tf][k]), d = unpk(rp[tf * 8 + 4 + k]);
                U[tf][k] = pk(a.x + b.x, a.y + b.y);
                V[tf][k] = pk(cc2.x + d.x, cc2.y + d.y);
              }
          }
        }
      }
      if (writer && active && !dead) {
        const int oy = ts ? ux : uy, ox = ts ? uy : ux;
        const int osy = oy ? p.f - oy : 0;
        const bool sp = ts ? selfp1 : selfp0;
#pragma unroll
        for (int tf = 0; tf < TF; tf++) {
          if (tf >= p.T) break;
          const long long obase = FWD ? ((long long)(blockIdx.y * p.T + tf) * NN) * ffh
                                      : ((long long)(tf * p.nzo + zi) * NN) * ffh;
#pragma unroll
          for (int k = 0; k < 4; k++) {
            const int vk = (kind == 2) ? ((k & 1) ? 2 : 0) : k;   // stored slot k -> virtual slot
            if (k < ns) {
              int sl = off[0];
#pragma unroll
              for (int m = 1; m < 4; m++)
                if (m == vk) sl = off[m];
              int q = p.slotcol[sl];
              if (ts) q = (q % L.N) * L.N + q / L.N;   // side 1: the transposed channel
              float2 *op = p.O + obase + (long long)q * ffh;
              float2 u = unpk(U[tf][0]), v = unpk(V[tf][0]);
#pragma unroll
              for (int m = 1; m < 4; m++)
                if (m == vk) { u = unpk(U[tf][m]); v = unpk(V[tf][m]); }
              if (sp) {
                op[oy * p.fh + ox] = make_float2(u.x + v.x, u.y + v.y);
              } else {
                op[oy * p.fh + ox] = u;
                op[osy * p.fh + ox] = v;
              }
            }
          }
        }
      }
      acc.zero();
      if (H > 1 || diag) __syncthreads();   // the reduction buffer is free again
    }
    if (++ch == cpb) { ch = 0; zl++; }
    if (++slot == NST) { slot = 0; round++; }
  }
  // Never leave a bulk copy in flight into this CTA's shared memory.
  __syncthreads();
  if (tid == 0 && *abortf) {
    const int issued = s_issued;
    for (int g = max(0, issued - NST); g < issued; g++)
      if (g != drop) mbar_wait(full + (g % NST), (g / NST) & 1, kWaitLimitNs / 10);
  }
  cp_async_wait_all();
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

// Packed matrices of a chunk of representatives: the value of frequency pair
// (py, px) goes to its half block (quad (py, px) side 0 when py <= px, quad
// (px, py) side 1 otherwise); a row pair also stores the row at (f - py, px).
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
    const int fy = kp / p.fq, fx = kp % p.fq;       // frequency pair (fy, fx)
    const int lo = min(fy, fx), hi = max(fy, fx);
    const int hb = 2 * (hi * (hi + 1) / 2 + lo) - hi + (fy > fx ? 1 : 0);
    const int fs = fy ? p.f - fy : 0;
    const int rep = p.rep0 + rl;
    const int kind = p.rep_kind[rep];
    const int row = p.rep_row[rep];
    const C *sp = reinterpret_cast<const C *>(p.spec) + ((long long)rl * NN + q) * ffh;
    // the second half block of a quad holds channel Tr q at the slot of q
    const int slot = p.col_slot[fy > fx ? (q % L.N) * L.N + q / L.N : q];
    float2 *dst = p.P + ((long long)hb * L.nrow + row) * L.RS + slot;
    const R sc = (R)p.scale;
    const C a = sp[fy * p.fh + fx];
    dst[0] = make_float2((float)(a.x * sc), (float)(a.y * sc));
    if (kind != 0) {
      const C b = sp[fs * p.fh + fx];
      dst[L.RS] = make_float2((float)(b.x * sc), (float)(b.y * sc));
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
static cudaError_t set_smem(const void *fn, size_t bytes) {
  return cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

// ----------------------------------------------------------------------------
// Lenslet interleave.  A pixel row y = r*N + b holds row r of the N channel
// images (b, a), a = 0..N-1, interleaved with stride N.  Both kernels work
// on one pixel row per CTA so that every global access is coalesced: the
// pixel row is read or written contiguously and each channel row is a
// contiguous run of Lxp floats.  This is the reference's strided sub-image
// access (special_fftconvolve.py:85-105, py_light_field.cpp:1001-1027 on
// input; projector.py:792-796 and the RL update of lfdeconv.py:112-183 on
// output) moved out of the transforms.
// ----------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_split(SplitParams p) {
  extern __shared__ float row[];                 // X floats
  const int y = blockIdx.x, s = blockIdx.y;
  const int N = p.N, NN = N * N, X = p.X, Lx = p.Lx, Lxp = p.Lxp, Ly = p.Ly;
  const int t = s / p.nz, zi = s - t * p.nz;
  const int r = y / N, b = y - r * N;
  const bool inside = y < p.Y;                   // rows of the last lenslet row beyond Y are zeros
  if (inside) {
    const int plane = p.planes ? p.planes[zi] : zi;
    const float *src = p.src + plane * p.src_sz + t * p.src_st + (long long)y * X;
    for (int x = threadIdx.x; x < X; x += blockDim.x) row[x] = __ldg(src + x);
  }
  __syncthreads();
  float *dst = p.dst + ((long long)s * NN + b * N) * Ly * Lxp + (long long)r * Lxp;
  const long long cstride = (long long)Ly * Lxp;
  for (int i = threadIdx.x; i < N * Lxp; i += blockDim.x) {
    const int a = (int)p.dlxp.div(i);
    const int c = i - a * Lxp;
    const int x = c * N + a;
    dst[a * cstride + c] = (inside && c < Lx && x < X) ? row[x] : 0.f;
  }
}

__global__ void __launch_bounds__(256) k_merge(MergeParams p) {
  extern __shared__ float sm[];                  // N rows of pitch Lx | 1
  const int y = blockIdx.x, s = blockIdx.y;
  const int N = p.N, NN = N * N, X = p.X, Lx = p.Lx, Lxp = p.Lxp, Ly = p.Ly;
  const int pitch = Lx | 1;
  const int t = s / p.nzo, zo = s - t * p.nzo;
  const int r = y / N, beta = y - r * N;
  const float *src = p.src + ((long long)s * NN + beta * N) * Ly * Lxp + (long long)r * Lxp;
  const long long cstride = (long long)Ly * Lxp;
  for (int i = threadIdx.x; i < N * Lx; i += blockDim.x) {
    const int a = (int)p.dlx.div(i);
    const int c = i - a * Lx;
    sm[a * pitch + c] = __ldg(src + a * cstride + c);
  }
  __syncthreads();
  const int plane = p.planes ? p.planes[zo] : zo;
  const long long row = (long long)y * X;
  float *out = p.out.p + plane * p.out.sz + t * p.out.st + row;
  const float *aux = p.aux.p ? p.aux.p + plane * p.aux.sz + t * p.aux.st + row : nullptr;
  const float *nrm = p.norm.p ? p.norm.p + plane * p.norm.sz + t * p.norm.st + row : nullptr;
  const int epi = p.epi;
  const bool need_o = epi == EPI_ADD || epi == EPI_RL_PREVEDEL || epi == EPI_RL_STANDARD;
  const bool need_a = epi == EPI_DIVIDE || epi == EPI_RL_PREVEDEL;
  const bool need_n = epi == EPI_RL_STANDARD && nrm != nullptr;
  constexpr int U = 4;                           // pixels per thread per round, loads first
  for (int x0 = threadIdx.x; x0 < X; x0 += U * blockDim.x) {
    float v[U], ov[U], av[U], nv[U];
#pragma unroll
    for (int k = 0; k < U; k++) {
      const int x = x0 + k * blockDim.x;
      const bool ok = x < X;
      const int c = ok ? (int)p.dn.div(x) : 0;
      v[k] = ok ? sm[(x - c * N) * pitch + c] : 0.f;
      ov[k] = (ok && need_o) ? out[x] : 0.f;
      av[k] = (ok && need_a) ? __ldg(aux + x) : 0.f;
      nv[k] = (ok && need_n) ? __ldg(nrm + x) : 1.f;
    }
#pragma unroll
    for (int k = 0; k < U; k++) {
      const int x = x0 + k * blockDim.x;
      if (x >= X) break;
      float res;
      switch (epi) {
        case EPI_STORE: res = v[k]; break;
        case EPI_ADD: res = ov[k] + v[k]; break;
        case EPI_DIVIDE: res = __fdiv_rn(av[k], v[k]); break;
        case EPI_RL_PREVEDEL:          // x * (Htf / Ht(H x)), lfdeconv.py:112-145
          res = __fmul_rn(ov[k], __fdiv_rn(av[k], v[k]));
          if (res != res) res = 0.f;
          break;
        default:                       // x * Ht(y / H x) [/ norm], lfdeconv.py:147-183
          res = __fmul_rn(ov[k], v[k]);
          if (need_n) res = __fdiv_rn(res, nv[k]);
          if (res != res) res = 0.f;
          break;
      }
      out[x] = res;
    }
  }
}

cudaError_t launch_split(const SplitParams &p0, cudaStream_t s) {
  if (p0.nsets == 0) return cudaSuccess;
  SplitParams p = p0;
  p.dlxp = Div16::make((unsigned)p.Lxp);
  const dim3 grid(p.Ly * p.N, p.nsets);
  k_split<<<grid, 256, p.X * sizeof(float), s>>>(p);
  return cudaGetLastError();
}

cudaError_t launch_merge(const MergeParams &p0, cudaStream_t s) {
  if (p0.nsets == 0) return cudaSuccess;
  MergeParams p = p0;
  p.dlx = Div16::make((unsigned)p.Lx);
  p.dn = Div16::make((unsigned)p.N);
  const dim3 grid(p.Y, p.nsets);
  k_merge<<<grid, 256, p.N * (p.Lx | 1) * sizeof(float), s>>>(p);
  return cudaGetLastError();
}

// ----------------------------------------------------------------------------
// Rectification resample: bilinear interpolation of a float image at a
// separable grid of query coordinates, in double precision.  This is the
// reference's RectBivariateSpline(kx = ky = 1) evaluation (rectify.py:8-81):
// a degree-1 B-spline through the pixel values is the bilinear interpolant.
// Queries outside [0, H-1] x [0, W-1] are clamped to the edge.
// ----------------------------------------------------------------------------
__device__ __forceinline__ void bilinear_cell(double q, int n, int &i0, double &t) {
  if (n < 2) { i0 = 0; t = 0.0; return; }
  const double qc = fmin(fmax(q, 0.0), (double)(n - 1));
  i0 = min((int)floor(qc), n - 2);
  t = qc - (double)i0;
}

__global__ void __launch_bounds__(256) k_resample_bilinear(ResampleParams p) {
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (long long)p.ny * p.nx) return;
  const int r = (int)(idx / p.nx), c = (int)(idx - (long long)r * p.nx);
  int y0, x0;
  double fy, fx;
  bilinear_cell(p.yq[r], p.H, y0, fy);
  bilinear_cell(p.xq[c], p.W, x0, fx);
  const int y1 = min(y0 + 1, p.H - 1), x1 = min(x0 + 1, p.W - 1);
  const float *row0 = p.img + (long long)y0 * p.W, *row1 = p.img + (long long)y1 * p.W;
  const double top = (1.0 - fx) * (double)row0[x0] + fx * (double)row0[x1];
  const double bot = (1.0 - fx) * (double)row1[x0] + fx * (double)row1[x1];
  p.out[idx] = (1.0 - fy) * top + fy * bot;
}

cudaError_t launch_resample_bilinear(const ResampleParams &p, cudaStream_t s) {
  const long long n = (long long)p.ny * p.nx;
  if (n == 0) return cudaSuccess;
  k_resample_bilinear<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(p);
  return cudaGetLastError();
}

// Transforms: the hot path runs the size-specialised kernels (flf_fft.cuh),
// one per even 7-smooth size up to kMaxF; the precompute (contiguous float or
// double images) runs the runtime-plan kernel above.
cudaError_t launch_rfft2(const Rfft2Params &p, int fp64, cudaStream_t s) {
  if (p.nimg == 0) return cudaSuccess;
  if (p.mode == 0) {
    if (fp64) return cudaErrorInvalidValue;
    switch (p.plan.n) {
#define FLF_CASE(F) \
      case F: return sfft::rfft2_sized<F>(p, s);
      FLF_SFFT_SIZES(FLF_CASE)
#undef FLF_CASE
      default: return cudaErrorInvalidValue;
    }
  }
  const size_t sm = rfft2_smem_bytes(p.plan.n, p.imgs_per_cta, fp64);
  const int grid = (p.nimg + p.imgs_per_cta - 1) / p.imgs_per_cta;
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
  if (p.nimg == 0) return cudaSuccess;
  switch (p.plan.n) {
#define FLF_CASE(F) \
    case F: return sfft::irfft2_sized<F>(p, s);
    FLF_SFFT_SIZES(FLF_CASE)
#undef FLF_CASE
    default: return cudaErrorInvalidValue;
  }
}

int mac_max_frames() { return 4; }

template <int TF>
static cudaError_t launch_mac_tf(const MacParams &p, bool fwd, cudaStream_t s) {
  const size_t sm = mac_smem_bytes(p.L, TF, p.stages, p.chunk_rows, p.split, fwd);
  dim3 grid(p.nquads, p.nzo_grid);
  const int block = 2 * p.split * (((p.L.nthr + 31) / 32) * 32);
  const void *fn = block <= 128 ? (fwd ? (const void *)k_mac<TF, true, false> : (const void *)k_mac<TF, false, false>)
                                : (fwd ? (const void *)k_mac<TF, true, true> : (const void *)k_mac<TF, false, true>);
  cudaError_t e = set_smem(fn, sm);
  if (e != cudaSuccess) return e;
  if (block <= 128) {
    if (fwd) k_mac<TF, true, false><<<grid, block, sm, s>>>(p);
    else k_mac<TF, false, false><<<grid, block, sm, s>>>(p);
  } else {
    if (fwd) k_mac<TF, true, true><<<grid, block, sm, s>>>(p);
    else k_mac<TF, false, true><<<grid, block, sm, s>>>(p);
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
