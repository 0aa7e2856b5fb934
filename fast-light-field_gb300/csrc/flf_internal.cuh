// Internal declarations shared by the CUDA translation units of libflf.so.
//
// Data model (lenslet-grid / polyphase form of the reference's projection):
//  * An image of Y x X pixels is split into N*N "channels", one per pixel
//    offset (b, a) inside a lenslet: s_{ba}(p, q) = img(p*N + b, q*N + a),
//    each an Ly x Lx image (Ly = ceil(Y/N)).  Channel index i = b*N + a.
//  * One z plane of the reference's projection (sum over offsets of masked
//    'same' convolutions, projector.py:1084-1126) is, per output channel
//    j = (beta, alpha), out_j = sum_i K_ij (*) s_i with the lenslet-grid
//    kernel K_ij(m, n) = Hfull_i(m*N + beta - b + ch, n*N + alpha - a + ch),
//    |m|,|n| <= R = floor((ch + N - 1)/N), ch = (h-1)/2.
//  * With an f x f circular transform (f >= max(Ly, Lx) + R) this is, for
//    every frequency u, a complex matrix-vector product
//    out_j[u] = sum_i T_ij[u] S_i[u], T = rfft2(K) / f^2.
//  * The PSF symmetries of the reference (projector.py:159-189) give
//    T_{My i, My j}[u] = T_ij[u*]           (b != c), u* = (-uy, ux)
//    T_{Mx i, Mx j}[u] = conj T_ij[u*]      (a != c)
//    T_{Mxy i, Mxy j}[u] = conj T_ij[u]     (b != c and a != c)
//    and the transpose of the PSF set gives T_{Tr i, Tr j}[(uy, ux)] =
//    T_ij[(ux, uy)], so the stored matrices cover a quarter of the
//    frequencies and about a quarter of the rows; see the packed layout below.
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace flf {

constexpr int kMaxStages = 12;
constexpr int kMaxF = 160;          // largest lenslet-grid FFT size (float)
constexpr int kMaxF64 = 112;        // largest size for the fp64 precompute
constexpr int kMacMaxZgroup = 64;   // planes per multiply-accumulate CTA

struct FftPlan {
  int n;                 // transform length (f)
  int nst;               // number of radix stages
  int rad[kMaxStages];   // radices, each in {2,3,4,5,7}
};

// Packed transfer-matrix layout for one (plane, direction), using the mirror
// symmetries above and the transpose symmetry of the reference's PSF set
// (offset (a, b) uses the transpose of offset (b, a)'s PSF when their folded
// indices differ, projector.py:176-179), which on the lenslet grid reads
//   T_{Tr i, Tr j}[(uy, ux)] = T_ij[(ux, uy)],   Tr(b, a) = (a, b).
// Frequency pairs (uy, ux), uy, ux in [0, f/2], come in quads {(uy, ux), (ux,
// uy)}, uy <= ux, ordered ux-major: quad k = ux(ux+1)/2 + uy.  Each quad holds
// one half block per frequency pair (one for a diagonal quad uy = ux): half
// blocks 2k - ux and 2k - ux + 1, so a plane has fq^2 half blocks in all.
//   P[half block][row][slot], rows = (c+1)(c+2) per half block, slot stride RS.
// Rows of a half block: the generic input orbits (b, a'), a' <= b < c, as their
// rows i = (b, a') and Mx i = (b, N-1-a') at u (c(c+1) rows, the c(c-1) rows
// of the orbits with a' < b first); then row pairs (u, u*) of the centre-cross
// representatives (b, c), b < c, and of the centre.  Orbits with a' < b and the
// (b, c) pairs also stand for their transposes (a', b) and (c, b), which have
// no rows.  Slots: output channels of the mirror orbits, slot-major: the c^2
// generic orbits [q, My q, Mx q, Mxy q] as four blocks of c^2, the c orbits
// [q, My q] (alpha = c) and the c orbits [q, Mx q] (beta = c) as two blocks of
// c each, then the centre.  The second half block of a quad keeps its columns
// in transposed order (the slot of channel j holds channel Tr j); thread t of
// the second frequency pair owns the transposed orbit of t, so both sides read
// both half blocks at the slots of orbit t: consecutive for a warp.
struct Layout {
  int N, NN, c, nh;
  int nrowG;      // c(c+1) generic rows per half block
  int nrowGT;     // c(c-1) of them (stored first) stand for their transposes too
  int nrep;       // c+1 row pairs per half block
  int nrow;       // (c+1)(c+2) rows per half block
  int ngrp;       // (c+1)^2 row groups (generic rows and row pairs) per half block
  int RS;         // row stride in complex elements
  int nthr;       // nh^2: output orbits (threads per row share)
};

inline Layout make_layout(int N) {
  Layout L;
  L.N = N; L.NN = N * N; L.c = N / 2; L.nh = L.c + 1;
  L.nrowG = L.c * (L.c + 1);
  L.nrowGT = L.c * (L.c - 1);
  L.nrep = L.c + 1;
  L.nrow = L.nrowG + 2 * L.nrep;
  L.ngrp = L.nrowG + L.nrep;
  L.RS = (L.NN + 1) & ~1;
  L.nthr = L.nh * L.nh;
  return L;
}

// Row-group flags (MacParams::rowF): bits 0-3 conjugate operand j, bits 4-7
// zero operand j when the receiving frequency pair is self-paired (u = u*),
// bits 8-11 operand j always zero, bit 12 the group also feeds the other
// frequency pair of its quad through the transpose.
constexpr int kRowTransposable = 1 << 12;

// ----------------------------------------------------------------------------
// Runtime division by an invariant divisor d (1 <= d < 2^16) for n < 2^16:
// n / d = (n * m) >> 32 with m = ceil(2^32 / d) (Granlund & Montgomery,
// "Division by invariant integers using multiplication", PLDI 1994; exact
// because n * (m * d - 2^32) < 2^32 for these ranges).  m is kept in 64 bits
// (m = 2^32 for d = 1) and the product is one wide multiply.
// ----------------------------------------------------------------------------
struct Div16 {
  unsigned long long m;
  __host__ static Div16 make(unsigned d) {
    Div16 r;
    r.m = ((1ull << 32) + d - 1) / d;
    return r;
  }
  __device__ __forceinline__ unsigned div(unsigned n) const { return (unsigned)(((unsigned long long)n * m) >> 32); }
};

// Epilogue modes of the pixel merge kernel.
enum Epilogue : int {
  EPI_STORE = 0,         // out = value
  EPI_DIVIDE = 1,        // out = aux / value           (y / Hx)
  EPI_RL_PREVEDEL = 2,   // x = x * (aux / value), NaN -> 0
  EPI_RL_STANDARD = 3,   // x = x * value [/ norm], NaN -> 0
  EPI_ADD = 4,           // out += value                 (sum over transform groups)
};

struct Strided {         // base + plane*sz + frame*st + y*X + x
  float *p;
  long long sz, st;
};

// ----------------------------------------------------------------------------
// Kernel parameter blocks
// ----------------------------------------------------------------------------

// Channel-major images: image g is Ly rows of Lxp floats (Lxp = Lx rounded up
// to a multiple of 4, so every row and image starts on a 16-byte boundary);
// element (r, c) of channel ch = b*N + a is pixel (r*N + b, c*N + a).  The
// columns c in [Lx, Lxp) are padding.
inline int channel_pitch(int Lx) { return (Lx + 3) & ~3; }

struct Rfft2Params {
  FftPlan plan;
  int N, Y, X, Ly, Lx;
  int nimg;                 // total images
  int mode;                 // 0: channel-major float images (chan); 1: contiguous f*f images
  const float *chan;        // mode 0: [nimg][Ly][Lxp], image g = set * NN + ch
  int Lxp;
  const void *src_img;      // mode 1: Real images [nimg][f][f]
  void *dst;                // Complex<Real> [nimg][f][fh]
  const void *twiddle;      // Complex<Real> [f]
  int imgs_per_cta;         // mode 1
  int nq_rows;              // mode 1: row pairs carrying data (<= f/2)
};

struct Irfft2Params {
  FftPlan plan;
  int N, Y, X, Ly, Lx;
  int nimg;                 // images g = set * NN + j
  const float2 *src;        // spectra [nsum][nimg][f][fh]
  long long sum_stride;     // elements between partial sums
  int nsum;
  float *chan;              // output: channel-major [nimg][Ly][Lxp]
  int Lxp;
  int add;                  // add to chan instead of overwriting it
  int final_pass;           // zero the positions outside the Y x X image (and the padding)
  const float *num;         // final pass, optional: store num / value (channel-major, like chan)
  const float2 *twiddle;
};

// Pixel images <-> channel-major images (the lenslet interleave).
struct SplitParams {        // src + plane*src_sz + t*src_st: Y x X pixels
  const float *src;
  long long src_sz, src_st;
  const int *planes;        // plane id per z index (device); NULL -> z index
  int nz, nsets;            // set s = t * nz + zi
  int N, Y, X, Ly, Lx, Lxp;
  float *dst;               // [nsets][NN][Ly][Lxp]
  Div16 dlxp;               // set by the launcher
};

struct MergeParams {
  const float *src;         // [nsets][NN][Ly][Lxp], set s = t * nzo + zo
  int nzo, nsets;
  const int *planes;        // plane id per zo (device); NULL -> zo
  int N, Y, X, Ly, Lx, Lxp;
  int epi;
  Strided out;              // destination (or x for RL updates)
  Strided aux;              // y (EPI_DIVIDE) or Htf (EPI_RL_PREVEDEL)
  Strided norm;             // EPI_RL_STANDARD normaliser (p may be NULL)
  Div16 dlx, dn;            // set by the launcher
};

struct ResampleParams {     // bilinear resample of img [H][W] at yq [ny] x xq [nx] -> out [ny][nx]
  const float *img;
  int H, W;
  const double *yq, *xq;
  int ny, nx;
  double *out;
};

struct MacParams {
  Layout L;
  int f, fh, fq, nkp;       // transform size, f/2+1, f/2+1, fq*fq half blocks per plane
  int nquads;               // fq(fq+1)/2 frequency quads (grid.x)
  int T;                    // frames in this launch (<= template TF)
  const float2 *P;          // packed matrices [plane][half block][nrow][RS]
  const int *planes;        // plane id per z index
  int nz;                   // planes in the list
  int zgroup;               // forward: planes per CTA group
  const float2 *S;          // input spectra [T][nzS][NN][f][fh]
  int nzS;                  // planes in S (forward nz, backward 1)
  float2 *O;                // output spectra
  int nzo;                  // forward: number of z groups (output sets); backward: nz
  int nzo_grid;             // grid.y: number of z groups of this launch
  const short4 *rowS;       // [2][ngrp]: operand channels of each row group for its own frequency
                            // pair (use 0) and through the transpose (use 1); + NN: at u*
  const short *rowF;        // [2][ngrp]: operand flags (kRowTransposable, conj / zero bits)
  const short4 *oslots;     // [2][nthr]: an orbit's four virtual slots, own and transposed
  const short *slotcol;     // slot -> output channel
  int stages;               // shared-memory ring stages of the bulk-copy pipeline
  int chunk_rows;           // stored rows per stage (even)
  int split;                // threads sharing one orbit's rows (1..4)
  int *err;                 // set nonzero when a bounded wait gives up
  unsigned long long wait_ns;   // limit of each wait for a ring slot (1 s)
  int drop_chunk;           // test of the bounded waits: chunk the first CTA never issues (-1: none)
};

struct BuildKParams {       // lenslet-grid kernels K_iq for the precompute
  int N, h, ch, R, f;
  const float *H;           // reduced PSF [nh][nh][h][h] (device)
  const int *rep_ch;        // input channel of each row representative
  int rep0, nrep_chunk;     // representatives in this chunk
  void *dst;                // Real [nrep_chunk][NN][f][f]
  int fp64;
};

struct PackParams {
  Layout L;
  int f, fh, fq, nkp;       // nkp = fq * fq frequency pairs (half blocks)
  const void *spec;         // Complex<Real> [nrep_chunk][NN][f][fh]
  int rep0, nrep_chunk;
  const int *rep_row;       // packed row of representative (first row)
  const int *rep_kind;      // 0 generic row, otherwise a row pair (u, u*)
  const int *rep_ch;
  const short *col_slot;    // channel -> slot
  float2 *P;                // this plane's packed blocks [fq * fq][nrow][RS]
  double scale;             // 1/f^2
  int fp64;
};

// Launchers (flf_kernels.cu)
cudaError_t launch_rfft2(const Rfft2Params &p, int fp64, cudaStream_t s);
cudaError_t launch_irfft2(const Irfft2Params &p, cudaStream_t s);
cudaError_t launch_split(const SplitParams &p, cudaStream_t s);
cudaError_t launch_resample_bilinear(const ResampleParams &p, cudaStream_t s);

// PSF generation (flf_psf.cu)
struct PsfDebyeParams {      // Koi * sum_q cw[q] J0(s[q] vFactor) per point
  double2 *out;
  int mode;                  // 0: octant points m2 <= m1 (npoints = (n+1)(n+2)/2); 1: line m1 = t, m2 = 0
  long long npoints;
  double dx, M, k, sin_alpha;
  const double *s;           // sin(theta) at the nodes
  const double2 *cw;         // node weight x smooth integrand x depth phase
  int nodes;
  double koi_re, koi_im;
};
struct PsfInputParams {      // shifted field x microlens array for nq lenslet offsets
  double2 *out;              // [nq][L][L]
  const double2 *wave;       // octant values, (support+1)(support+2)/2
  int support, max_bug;
  const double2 *lens;       // [2h+1][2h+1]
  int lens_h, L, nh, osr, q0, nq;
};
struct PsfBinParams {        // |f|^2 binned onto the lenslet-grid crop
  float *out;                // [nq][S][S]
  const double2 *field;      // [nq][L][L]
  int L, S, nh, osr, q0, nq, lo, hi, first;
};
struct PsfHtParams {         // Ht gathered from H, both [Z][nh][nh][S][S]
  float *Ht;
  const float *H;
  int Z, nh, S, N;
};
cudaError_t launch_psf_debye(const PsfDebyeParams &p, cudaStream_t s);
cudaError_t launch_psf_lf_input(const PsfInputParams &p, cudaStream_t s);
cudaError_t launch_psf_lf_bin(const PsfBinParams &p, cudaStream_t s);
cudaError_t launch_psf_ht(const PsfHtParams &p, cudaStream_t s);

// Learned warm start (flf_net.cu): channels-last BF16 volumes [B][Z][Y][X][C]
struct ConvParams {          // y = act(conv3x3x3(x, w) + bias) (* (mask > 0))
  const __nv_bfloat16 *x;    // [M][Ci]
  const __nv_bfloat16 *w;    // [27][Ci][Co], tap = (dz+1)*9 + (dy+1)*3 + (dx+1)
  const float *bias;         // [Co] or null
  const __nv_bfloat16 *mask; // [M][Co] or null
  __nv_bfloat16 *y;          // [M][Co]
  int B, Z, Y, X, Ci, Co, relu;
  float *ws;                 // [splits][M][Co] FP32 partial sums when the K loop is split (splits > 1)
  int splits;
  const __nv_bfloat16 *wp;   // or null: the same weights packed by k_conv3d_pack_weights (per tap
                             // and 16 input channels one [2][Co][8] block), what the tcgen05
                             // kernel of the wide layers reads
  __nv_bfloat16 *pool = nullptr;   // or [B][Z/2][Y/2][X/2][Co]: y's 2x2x2 average pooling as well
                                   // (launch_conv3d_pool)
};
struct WgradParams {         // dw[tap][ci][co] += sum_v x[v + tap][ci] dy[v][co]
  const __nv_bfloat16 *x;
  const __nv_bfloat16 *dy;
  float *dw;
  int B, Z, Y, X, Ci, Co;
  long long chunk;           // voxels per CTA (set by the launcher)
  float *part;               // [chunks][27][Ci][Co] partial gradients, reduced in chunk order (or null)
};
cudaError_t launch_conv3d(ConvParams p, long long ws_elems, cudaStream_t s);
cudaError_t launch_conv3d_pool(const ConvParams &p, cudaStream_t s);
cudaError_t launch_conv3d_x1(const ConvParams &p, cudaStream_t s);
long long net_launches();
int net_set_conv_wide_tcgen05(int mode);
cudaError_t launch_conv3d_pack(const void *w, void *wp, int Ci, int Co, cudaStream_t s);
cudaError_t launch_conv3d_wgrad(WgradParams p, long long ws_elems, cudaStream_t s, int num_sms);
cudaError_t launch_conv3d_tc16(const ConvParams &p, cudaStream_t s);
cudaError_t launch_conv3d_tma16(const ConvParams &p, cudaStream_t s, bool sw32);
int net_set_conv16_tcgen05(int mode);
int net_status_read_and_clear();
cudaError_t launch_conv3d_flip(const void *w, void *w2, int Ci, int Co, cudaStream_t s);
cudaError_t launch_bias_grad(const void *g, float *db, float *ws, long long ws_elems, long long M, int C,
                             cudaStream_t s);
cudaError_t launch_pool2(const void *in, void *out, int B, int Z, int Y, int X, int C, cudaStream_t s);
cudaError_t launch_pool2_bwd(const void *gpool, const void *gskip, const void *act, void *gin, int B, int Z, int Y,
                             int X, int C, cudaStream_t s);
cudaError_t launch_up2_add(const void *low, const void *skip, void *out, int B, int Z, int Y, int X, int C,
                           cudaStream_t s);
cudaError_t launch_up2_bwd(const void *g, const void *act, void *glow, int B, int Z, int Y, int X, int C,
                           cudaStream_t s);
cudaError_t launch_mse_grad(const void *y, const float *target, void *g, float *loss, long long M, int C,
                            cudaStream_t s);
cudaError_t launch_adam(float *w, const float *g, float *m, float *v, void *wb, long long n, float lr, float b1,
                        float b2, float eps, float c1, float c2, float wd, cudaStream_t s);
cudaError_t launch_render_blobs(float *vol, void *acc, int Z, int Y, int X, const float *pts, int npts, float sigma,
                                cudaStream_t s);
struct WsInputParams {        // warm-start network input from Htf
  const float *htf;           // [Z][T][Y][X]
  const float *hth1, *ht1;    // [Z][Y][X]
  float *sum_x1;              // [T] scratch: frame sums of Htf / HtH1
  __nv_bfloat16 *out;         // [T][Zp][Yp][Xp][16]
  int T, Z, Y, X, Zp, Yp, Xp;
  float count;                // Z * Y * X (frame sums -> means)
  float c2, c3;               // 1 / mean(HtH1), 1 / mean(Ht1)
};
struct HeadOut {              // warm-start head output (k_conv3d_t16<true>)
  float *x0;                  // [Zr][T][Yr][Xr] start volume
  const float *sum_x1;        // [T] frame sums of Htf / HtH1
  float count;                // Zr * Yr * Xr
  float bias, floor;
  int T, Zr, Yr, Xr;
};
cudaError_t launch_ws_input(const WsInputParams &p, cudaStream_t s);
cudaError_t launch_ws_head(const void *d, const void *w, float bias, float floor_, const float *sum_x1, float *x0,
                           int T, int Z, int Y, int X, int Zp, int Yp, int Xp, cudaStream_t s);
cudaError_t launch_merge(const MergeParams &p, cudaStream_t s);
cudaError_t launch_mac(const MacParams &p, bool forward, cudaStream_t s);
cudaError_t launch_build_k(const BuildKParams &p, int nimg, cudaStream_t s);
cudaError_t launch_pack(const PackParams &p, cudaStream_t s);
size_t rfft2_smem_bytes(int f, int imgs, int fp64);
int mac_max_frames();
// Shared memory one CTA may opt in to (sm_100 family).
constexpr size_t kMacSmemMax = 227 * 1024;
size_t mac_smem_bytes(const Layout &L, int TF, int stages, int chunk_rows, int split, bool fwd);

}  // namespace flf
