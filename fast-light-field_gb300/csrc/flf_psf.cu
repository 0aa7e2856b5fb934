// Light-field PSF generation on the GPU: the GB300 counterpart of the
// reference's generate_psf.py (GeneratePSF, generate_psf.py:63-737).
//
//   k_psf_debye      Debye integral of the objective's field at image-side
//                    points (generate_psf.py:96-144, 263-315), by composite
//                    Gauss-Legendre quadrature over theta in [0, alpha]
//                    instead of adaptive quad.  The phase factor and the
//                    smooth part of the integrand depend on the depth only,
//                    so the host folds them with the weights into one complex
//                    weight per node; a point costs one FP64 J0 per node.
//   k_psf_lf_input   the field of one depth, expanded from its octant
//                    (:317-348), shifted to a lenslet offset and multiplied by
//                    the microlens array (:168-205, 527-528): the input of
//                    the Fresnel propagation (an FFT pair, cuFFT).
//   k_psf_lf_bin     shift back, aperture window, |f|^2, OSR x OSR binning
//                    and the lenslet-grid crop (:456-513, 529-546).
//   k_psf_ht         Ht from H (:624-690) as a gather: the reference stamps
//                    the rotated H of every offset into a scratch image, cuts
//                    and shifts it; that composition is a closed-form index
//                    map onto H.
#include "flf_internal.cuh"

namespace flf {

namespace {

__device__ __forceinline__ void octant_point(long long t, int &m1, int &m2) {
  // t = m1 (m1 + 1) / 2 + m2, 0 <= m2 <= m1
  int m = (int)floor((sqrt(8.0 * (double)t + 1.0) - 1.0) * 0.5);
  while ((long long)(m + 1) * (m + 2) / 2 <= t) m++;
  while ((long long)m * (m + 1) / 2 > t) m--;
  m1 = m;
  m2 = (int)(t - (long long)m * (m + 1) / 2);
}

}  // namespace

// One warp per point.  mode 0: the octant m2 <= m1 <= count-1 (offsets from
// the centre in grid steps); mode 1: the line m1 = t, m2 = 0, t < count.
__global__ void __launch_bounds__(256) k_psf_debye(PsfDebyeParams p) {
  const long long warp = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (warp >= p.npoints) return;
  int m1, m2;
  if (p.mode == 0) {
    octant_point(warp, m1, m2);
  } else {
    m1 = (int)warp;
    m2 = 0;
  }
  // the reference's operation order: x = dx * (offset), r = |x| / M,
  // v = k r sin(alpha), vFactor = v / sin(alpha)
  const double x1 = p.dx * (double)m1, x2 = p.dx * (double)m2;
  const double r = sqrt(x1 * x1 + x2 * x2) / p.M;
  const double v = p.k * r * p.sin_alpha;
  const double vf = v / p.sin_alpha;
  double re = 0.0, im = 0.0;
  for (int q = lane; q < p.nodes; q += 32) {
    const double j = j0(p.s[q] * vf);
    const double2 w = p.cw[q];
    re = fma(w.x, j, re);
    im = fma(w.y, j, im);
  }
  for (int o = 16; o > 0; o >>= 1) {
    re += __shfl_down_sync(0xffffffffu, re, o);
    im += __shfl_down_sync(0xffffffffu, im, o);
  }
  if (lane == 0) p.out[warp] = make_double2(p.koi_re * re - p.koi_im * im, p.koi_re * im + p.koi_im * re);
}

// F[q][i][j] = wave(i - sx_q, j - sy_q) * ML(i, j) for the lenslet offsets
// q = q0 .. q0+nq-1 (a = q / nh, b = q % nh; sx = OSR (a + 1 - nh)).
// wave(i', j') is the octant value at (max, min) of the centre offsets inside
// the square of half-width `support`, 0 outside and off the grid; with
// `max_bug` the reference's maximum over rotations at z = 0 keeps only
// values that compare above 0 (positive real part, or zero real part and
// positive imaginary part).  ML is the lens phase of the nearest lens centre
// (centres every m = 2 h + 1 samples from the grid centre).
__global__ void __launch_bounds__(256) k_psf_lf_input(PsfInputParams p) {
  const long long n = (long long)p.L * p.L;
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int qi = blockIdx.y;
  if (e >= n) return;
  const int i = (int)(e / p.L), j = (int)(e - (long long)i * p.L);
  const int q = p.q0 + qi;
  const int a = q / p.nh, b = q - a * p.nh;
  const int sx = p.osr * (a + 1 - p.nh), sy = p.osr * (b + 1 - p.nh);
  const int c = (p.L - 1) / 2;
  double2 v = make_double2(0.0, 0.0);
  const int si = i - sx, sj = j - sy;
  if (si >= 0 && si < p.L && sj >= 0 && sj < p.L) {
    const int di = abs(si - c), dj = abs(sj - c);
    const int m1 = max(di, dj), m2 = min(di, dj);
    if (m1 <= p.support) {
      double2 w = p.wave[(long long)m1 * (m1 + 1) / 2 + m2];
      if (p.max_bug && !(w.x > 0.0 || (w.x == 0.0 && w.y > 0.0))) w = make_double2(0.0, 0.0);
      const int m = 2 * p.lens_h + 1;
      int ri = (i - c) % m, rj = (j - c) % m;
      if (ri > p.lens_h) ri -= m;
      if (ri < -p.lens_h) ri += m;
      if (rj > p.lens_h) rj -= m;
      if (rj < -p.lens_h) rj += m;
      const double2 l = p.lens[(ri + p.lens_h) * m + (rj + p.lens_h)];
      v = make_double2(w.x * l.x - w.y * l.y, w.x * l.y + w.y * l.x);
    }
  }
  p.out[(long long)qi * n + e] = v;
}

// H[q][I][J] = sum over an OSR x OSR block of |f1_AP|^2, f1_AP[i][j] =
// F[q][i + sx][j + sy] inside the aperture window [lo, hi]^2 (and on the
// grid), the block of (I, J) starting at (first + I OSR, first + J OSR).
__global__ void __launch_bounds__(256) k_psf_lf_bin(PsfBinParams p) {
  const long long n = (long long)p.S * p.S;
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int qi = blockIdx.y;
  if (e >= n) return;
  const int I = (int)(e / p.S), J = (int)(e - (long long)I * p.S);
  const int q = p.q0 + qi;
  const int a = q / p.nh, b = q - a * p.nh;
  const int sx = p.osr * (a + 1 - p.nh), sy = p.osr * (b + 1 - p.nh);
  const double2 *F = p.field + (long long)qi * p.L * p.L;
  double acc = 0.0;
  for (int di = 0; di < p.osr; di++) {
    const int i = p.first + I * p.osr + di;
    const int fi = i + sx;
    if (i < p.lo || i > p.hi || fi < 0 || fi >= p.L) continue;
    for (int dj = 0; dj < p.osr; dj++) {
      const int j = p.first + J * p.osr + dj;
      const int fj = j + sy;
      if (j < p.lo || j > p.hi || fj < 0 || fj >= p.L) continue;
      const double2 f = F[(long long)fi * p.L + fj];
      acc += f.x * f.x + f.y * f.y;
    }
  }
  p.out[(long long)qi * n + e] = (float)acc;
}

// Ht[z][a][b][i][j] from H[z][A][B][X][Y] (both [Z][nh][nh][S][S]):
// aa = (i mod N + a) mod N, A = aa <= N/2 ? aa : N-1-aa, X = aa <= N/2 ? S-1-i : i
// (likewise bb, B, Y from j and b); zero where the shift by ceil(N/2)-1-a
// (rows) or ceil(N/2)-1-b (columns) leaves the S x S window.
__global__ void __launch_bounds__(256) k_psf_ht(PsfHtParams p) {
  const long long n = (long long)p.S * p.S;
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int zab = blockIdx.y;
  if (e >= n) return;
  const int i = (int)(e / p.S), j = (int)(e - (long long)i * p.S);
  const int z = zab / (p.nh * p.nh), ab = zab - z * p.nh * p.nh;
  const int a = ab / p.nh, b = ab - a * p.nh;
  const int N = p.N, half = N / 2, ch = (N + 1) / 2;
  const int pi = i - (ch - a - 1), pj = j - (ch - b - 1);
  float v = 0.f;
  if (pi >= 0 && pi < p.S && pj >= 0 && pj < p.S) {
    const int aa = (i % N + a) % N, bb = (j % N + b) % N;
    const int A = aa <= half ? aa : N - 1 - aa, X = aa <= half ? p.S - 1 - i : i;
    const int B = bb <= half ? bb : N - 1 - bb, Y = bb <= half ? p.S - 1 - j : j;
    v = p.H[(((long long)z * p.nh + A) * p.nh + B) * n + (long long)X * p.S + Y];
  }
  p.Ht[(long long)zab * n + e] = v;
}

cudaError_t launch_psf_debye(const PsfDebyeParams &p, cudaStream_t s) {
  if (p.npoints <= 0) return cudaSuccess;
  const long long threads = p.npoints * 32;
  k_psf_debye<<<(unsigned)((threads + 255) / 256), 256, 0, s>>>(p);
  return cudaGetLastError();
}

cudaError_t launch_psf_lf_input(const PsfInputParams &p, cudaStream_t s) {
  const long long n = (long long)p.L * p.L;
  if (p.nq <= 0 || n == 0) return cudaSuccess;
  k_psf_lf_input<<<dim3((unsigned)((n + 255) / 256), (unsigned)p.nq), 256, 0, s>>>(p);
  return cudaGetLastError();
}

cudaError_t launch_psf_lf_bin(const PsfBinParams &p, cudaStream_t s) {
  const long long n = (long long)p.S * p.S;
  if (p.nq <= 0 || n == 0) return cudaSuccess;
  k_psf_lf_bin<<<dim3((unsigned)((n + 255) / 256), (unsigned)p.nq), 256, 0, s>>>(p);
  return cudaGetLastError();
}

cudaError_t launch_psf_ht(const PsfHtParams &p, cudaStream_t s) {
  const long long n = (long long)p.S * p.S;
  if (p.Z <= 0 || n == 0) return cudaSuccess;
  k_psf_ht<<<dim3((unsigned)((n + 255) / 256), (unsigned)(p.Z * p.nh * p.nh)), 256, 0, s>>>(p);
  return cudaGetLastError();
}

}  // namespace flf
