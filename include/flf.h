/*
 * flf.h - C ABI of the GB300 light-field projection library (libflf.so).
 *
 * This is the native boundary that replaces the reference's CPython extension
 * `py_light_field` for the Richardson-Lucy hot path of jmtayloruk/fast-light-field.
 * The reference binds that extension from Python (method table
 * py_light_field/py_light_field.cpp:1956-1973); a Python host binds this file
 * with ctypes (fast-light-field_gb300/_flf.py).
 *
 * Conventions
 *  - Every call returns an int status: FLF_OK (0) or a negative FLF_E_* code.
 *    The message of the last failure on a context is read with
 *    flf_last_error(); failures of flf_ctx_create() are read with
 *    flf_last_error(NULL, ...).
 *  - Array arguments named *_dev are CUDA device pointers owned by the caller
 *    (float32, C-contiguous).  Host arrays are plain float pointers.
 *  - Volumes are laid out [Z][T][Y][X] (plane, frame, row, column), images
 *    [T][Y][X], exactly as the reference's numpy arrays
 *    (lfdeconv.py:27-70).  `planes` lists the plane ids taking part, as the
 *    reference's `planes` argument (projector.py:806, 851).
 *  - `stream` is a cudaStream_t (NULL = legacy default stream).  Calls are
 *    stream-ordered and not thread-safe for one context.
 *  - The context owns the PSFs, the precomputed transfer matrices (the GB300
 *    form of the reference's FH cache) and all workspaces.
 */
#ifndef FLF_H
#define FLF_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define FLF_OK 0
#define FLF_E_ARG (-1)      /* bad argument: shape, range, null pointer   */
#define FLF_E_CUDA (-2)     /* a CUDA runtime call failed                  */
#define FLF_E_NOMEM (-3)    /* device or host allocation failed            */
#define FLF_E_STATE (-4)    /* call out of order (e.g. PSF not uploaded)   */
#define FLF_E_TIMEOUT (-5)  /* a bounded device wait gave up               */

/* Projection direction / PSF set selector. */
#define FLF_DIR_FORWARD 0   /* H:  volume -> image  (reference useHt=False) */
#define FLF_DIR_BACKWARD 1  /* Ht: image  -> volume (reference useHt=True)  */

/* Richardson-Lucy update variants (lfdeconv.py:112-183). */
#define FLF_RL_PREVEDEL 0   /* x <- x * Htf / Ht(H x); NaN -> 0             */
#define FLF_RL_STANDARD 1   /* x <- x * Ht(y / H x) [/ norm]; NaN -> 0       */

typedef struct flf_ctx flf_ctx;

/* Create a context on CUDA device `device` for a PSF with lenslet size
 * `nnum` (odd) and `num_planes` z planes.  Replaces the module-level state
 * of py_light_field (gFHCache, gNumThreadsToUse; py_light_field.cpp:15-32,
 * 1319-1385). */
int flf_ctx_create(flf_ctx **out, int device, int nnum, int num_planes);

/* Free every device allocation of the context. */
int flf_ctx_destroy(flf_ctx *ctx);

/* Copy the last error message (NUL-terminated, truncated to len) of `ctx`,
 * or of the calling thread's last flf_ctx_create when ctx is NULL.
 * Replaces the PyErr_* exceptions of py_light_field.cpp:1425-1493. */
int flf_last_error(const flf_ctx *ctx, char *buf, size_t len);

/* Upload the stored PSF quadrant of one plane and direction: host array
 * [n_h][n_h][h][h] float32 with n_h = (nnum+1)/2 and h odd.  This is the
 * per-plane `hMatrix.Hcc(cc, useHt)` array the reference passes to
 * ProjectForZList (projector.py:813-815, 855-857; psfmatrix.py:46-66).
 * Invalidates transfer matrices built from an earlier upload. */
int flf_psf_upload(flf_ctx *ctx, int plane, int direction, const float *H_host,
                   int n_h, int h);

/* Build (or reuse) the transfer matrices for images of Y x X pixels:
 * the PSF spectrum precompute that the reference redoes on every call in
 * FHWorkItem::Run (py_light_field.cpp:781-812, 829-867) unless cacheFH.
 * `fft_size` 0 picks the transform size automatically; `fp64` nonzero
 * runs the precompute in double precision.  Optional: projections call it
 * themselves when the shape changes. */
int flf_prepare(flf_ctx *ctx, int Y, int X, int fft_size, int fp64);

/* Forward projection H x: vol_dev [Z][T][Y][X] -> img_dev [T][Y][X]
 * (sum over `planes`).  Replaces Projector_allC.ForwardProjectACC's
 * ProjectForZList + InverseRFFTList + CropAfterFFT + plane sum
 * (projector.py:851-896; py_light_field.cpp:1417-1635, 1663-1740). */
int flf_forward(flf_ctx *ctx, const float *vol_dev, float *img_dev, int T, int Y,
                int X, const int *planes, int nplanes, void *stream);

/* Back projection Ht y: img_dev [T][Y][X] -> vol_dev [Z][T][Y][X]; only the
 * listed planes are written.  Replaces Projector_allC.BackwardProjectACC
 * (projector.py:806-849). */
int flf_backward(flf_ctx *ctx, const float *img_dev, float *vol_dev, int T, int Y,
                 int X, const int *planes, int nplanes, void *stream);

/* Size of the fixed device scratch used by flf_backward_noalloc. */
#define FLF_NOALLOC_SCRATCH_BYTES (16u * 1024u * 1024u)

/* Back projection that allocates nothing: the same result as flf_backward
 * over all planes, for callers that cannot ask the CUDA driver for memory
 * while they run - for example a real-time acquisition loop that must never
 * wait on the device allocator, or a plug-in whose host application hands
 * out all device memory from its own pool and forbids cudaMalloc.  This entry
 * point has no counterpart in the reference.
 *  - The caller passes the image and the output volume; the transfer matrices
 *    must already exist for this Y x X (call flf_prepare earlier), otherwise
 *    FLF_E_STATE is returned instead of building them.
 *  - The intermediate spectra and channel images live in one fixed device
 *    array of FLF_NOALLOC_SCRATCH_BYTES (16 MiB) inside the library: one
 *    frame's channel images and spectra plus the output spectra and channel
 *    images of as many planes as fit.  A GPU holds this array from the first
 *    flf_ctx_create on it until the process exits.  Geometries that need more
 *    (2 * (Nnum^2 * f * (f/2+1) * 8 + Nnum^2 * Ly * Lxp * 4) bytes, Lxp =
 *    ceil(X/Nnum) rounded up to 4; e.g. the 1005 x 1005 full field) are
 *    rejected with FLF_E_ARG; use flf_backward.
 *  - The array is set up when the context is created: flf_ctx_create looks
 *    up its device address with the context's device current, which (under
 *    CUDA's lazy module loading) is also when the 16 MiB is committed on that
 *    GPU.  The call itself does no set-up, but under lazy loading its first
 *    launch of each kernel makes the driver load that kernel's code into
 *    device memory: make one call at set-up time (or run with
 *    CUDA_MODULE_LOADING=EAGER) before the loop that must not allocate.
 *    The address belongs to the device's primary context; after
 *    cudaDeviceReset create a new context.
 *  - All calls share the one array and nothing in it needs to start at zero
 *    (every element read is written first by the same call); calls whose
 *    work overlaps on the GPU, on any stream or context, race on it.
 *  - Like flf_backward, the call only enqueues work: a bounded device wait
 *    that gave up is reported by the next flf_synchronize (FLF_E_TIMEOUT),
 *    so check that before using the result. */
int flf_backward_noalloc(flf_ctx *ctx, const float *img_dev, float *vol_dev, int T, int Y,
                         int X, void *stream);

/* `iters` Richardson-Lucy iterations in place on x_dev [Z][T][Y][X] over all
 * planes of the context (the loop of DeconvRL, lfdeconv.py:185-196).
 *  FLF_RL_PREVEDEL: ref_dev = Htf [Z][T][Y][X]; norm_dev ignored.
 *  FLF_RL_STANDARD: ref_dev = camera image [T][Y][X]; norm_dev = Ht(mask)
 *    [Z][1][Y][X] or NULL (no normaliser). */
int flf_rl_iterate(flf_ctx *ctx, float *x_dev, const float *ref_dev,
                   const float *norm_dev, int variant, int iters, int T, int Y,
                   int X, void *stream);

/* Bytes of device memory the context holds (PSFs, transfer matrices,
 * workspaces).  Counterpart of gMemoryUsage (py_light_field.cpp:654-670). */
int flf_memory_usage(const flf_ctx *ctx, size_t *bytes);

/* A count the context bumps whenever it frees a workspace, transfer matrix or
 * PSF buffer.  A CUDA graph a caller captured around calls of this library
 * (rather than through flf_rl_graph_create) refers to the context's buffers
 * only while the count is unchanged: compare before each replay. */
int flf_memory_epoch(const flf_ctx *ctx, unsigned long long *epoch);

/* Drop the transfer matrices and workspaces (keeps the uploaded PSFs).
 * Counterpart of ClearFHCache (py_light_field.cpp:1370-1385). */
int flf_clear_cache(flf_ctx *ctx);

/* Transform sizes and precompute precision chosen by the last prepare:
 * out[0] = largest lenslet-grid FFT size f, out[1] = largest kernel radius R
 * (lenslets), out[2] = fp64 flag, out[3] = number of transform groups
 * (planes with equal f share one). */
int flf_geometry(const flf_ctx *ctx, int *out4);

/* Per-kernel statistics.  flf_profile(ctx, 1) clears the counters and
 * brackets every subsequent kernel launch with CUDA events on its stream;
 * flf_profile(ctx, 0) clears them and stops the event timing (launch counts
 * are always kept).  flf_profile_read writes one line per kernel:
 * "<name> <launches> <total_ms> <algorithmic_bytes>".  The reference's
 * counterparts are its per-work-item timeline and stats files
 * (SetThreadFileName / SetStatsFile, py_light_field.cpp:171-282). */
int flf_profile(flf_ctx *ctx, int enable);
int flf_profile_read(flf_ctx *ctx, char *buf, size_t len);

/* Tunable launch parameters (the GB300 counterpart of the reference's
 * block-shape knobs gBlockSelection / gCalculateRowsBlocks,
 * projector.py:26-36).  Options: "mac_stages" (shared-memory pipeline
 * stages of the multiply-accumulate, 2..16), "mac_chunk_rows" (stored rows
 * per stage, even, 2..64, both directions; "mac_chunk_rows_forward" and
 * "mac_chunk_rows_backward" set one), "mac_split" (threads sharing an orbit's rows,
 * 1..4; the CTA has two such groups, one per frequency pair of a quad, of at
 * most 256 threads in all), "mac_ctas_per_sm" (1..64, default 16: the CTAs
 * per SM the grouping of planes per CTA aims at; fewer CTAs stream more planes
 * each), "plane_transform_sizes" (1: each plane uses the smallest
 * transform its PSF allows, planes grouped by size - the default; 0: one
 * size for all planes) and "geometry_cache" (0..16, default 2: how many
 * transfer-matrix sets of other image shapes stay resident, most recent
 * first, so that a series alternating image sizes does not rebuild them) and
 * "streams" (1 or 2, default 2: the transform groups of a projection
 * alternate over this many streams, so one group's transforms overlap the
 * next group's multiply-accumulate) and "release_psf" (0 or 1, default 0:
 * free the uploaded PSF quadrants once both directions' transfer matrices of
 * the current image shape are built, for PSF sets whose quadrants and
 * matrices do not both fit; another image shape then needs the PSFs uploaded
 * again).  Results agree to rounding whatever the values.
 * Two options exist to test the bounded waits of the multiply-accumulate:
 * "mac_wait_limit_us" (100..1e7, default 1e6: how long a wait for a ring
 * slot may last before the kernel gives up, sets the error flag that the next
 * flf_synchronize reports as FLF_E_TIMEOUT, and returns) and
 * "test_drop_chunk" (-1 default; k >= 0: the first CTA of each
 * multiply-accumulate launch never issues its k-th bulk copy, so its wait
 * for that slot runs out).  Neither faults or hangs the GPU; results of a
 * launch that gave up are incomplete. */
int flf_set_option(flf_ctx *ctx, const char *name, long long value);

/* Wait for `stream` and report any failure of earlier launches, including a
 * bounded device-side wait that gave up (FLF_E_TIMEOUT).  Counterpart of the
 * reference's synchronous return from ProjectForZList. */
int flf_synchronize(flf_ctx *ctx, void *stream);

/* Library self-description for diagnostics: writes a short text (build
 * arch, kernel list) into buf. */
int flf_version(char *buf, size_t len);

/* PSF generation (the reference's generate_psf.py GeneratePSF, :63-737), as
 * four kernels a host driver chains with FFTs.  All arrays are device
 * pointers; complex arrays are interleaved (re, im) doubles, 16-byte aligned.
 *
 * flf_psf_debye: Debye integral of the objective's field (generate_psf.py:
 *   96-144, 263-315) at image-side points, out[t] = Koi * sum_q cw[q] *
 *   J0(s[q] * vFactor(t)), vFactor = k r sin(alpha) / sin(alpha), r =
 *   sqrt(x1^2 + x2^2) / M, x = dx * offset.  mode 0: the octant of offsets
 *   (m1, m2), 0 <= m2 <= m1, t = m1 (m1 + 1) / 2 + m2 (npoints = (n+1)(n+2)/2
 *   for offsets up to n); mode 1: the line (t, 0).  s / cw: nodes of a
 *   quadrature over theta in [0, alpha] (sin theta; weight x smooth
 *   integrand x depth phase).  out: npoints complex.
 * flf_psf_lf_input: for lenslet offsets q = q0 .. q0+nq-1 (a = q / nh,
 *   b = q % nh), out[q-q0][i][j] = wave(i - sx, j - sy) * lens(nearest lens
 *   centre), sx = osr (a + 1 - nh); wave from the octant array of flf_psf_debye
 *   (mode 0, up to `support`), zero outside; max_bug applies the reference's
 *   z = 0 maximum over rotations (generate_psf.py:338-341).  lens: the
 *   (2 lens_h + 1)^2 phase of one microlens.  out: nq L L complex (L odd).
 * flf_psf_lf_bin: after the Fresnel propagation of those fields, out[q-q0][I][J]
 *   = sum over an osr x osr block at (first + I osr, first + J osr) of
 *   |field[i + sx][j + sy]|^2 inside the aperture window [lo, hi]^2
 *   (generate_psf.py:529-546, pixelBinning :479-513).  out: nq S S floats.
 * flf_psf_ht: Ht from H (generate_psf.py:624-690), both [Z][nh][nh][S][S]
 *   floats, nh = (N+1)/2, S odd with (S/2) % N == 0. */
int flf_psf_debye(double *out_dev, int mode, long long npoints, double dx, double M, double k, double sin_alpha,
                  const double *s_dev, const double *cw_dev, int nodes, double koi_re, double koi_im,
                  void *stream);
int flf_psf_lf_input(double *out_dev, const double *wave_dev, int support, int max_bug, const double *lens_dev,
                     int lens_h, int L, int nh, int osr, int q0, int nq, void *stream);
int flf_psf_lf_bin(float *out_dev, const double *field_dev, int L, int S, int nh, int osr, int q0, int nq, int lo,
                   int hi, int first, void *stream);
int flf_psf_ht(float *Ht_dev, const float *H_dev, int Z, int nh, int S, int N, void *stream);

/* Learned warm start: kernels of a 3-D U-Net on channels-last BF16 volumes
 * [B][Z][Y][X][C] (C a multiple of 16), FP32 accumulation.  All pointers are
 * device pointers; volumes and weights 16-byte aligned.  These are the
 * network's own forward and backward kernels (the reference has no learned
 * part; its DeconvRL starts from Htf or a given guess, lfdeconv.py:72-202).
 *
 * flf_conv3d: y = act(conv3x3x3(x, w) + bias), zero padding, w [27][Ci][Co]
 *   (tap = (dz+1)*9 + (dy+1)*3 + (dx+1)), bias [Co] float or NULL, act = ReLU
 *   when relu != 0; with mask != NULL ([..][Co] bf16) entries whose mask is
 *   not > 0 are zeroed (the ReLU derivative in a backward pass).  ws (float,
 *   or NULL) lets layers with few output tiles split their K loop across
 *   CTAs, each split into its own B Z Y X Co slice (as many splits as fit,
 *   at least 2), summed in split order; it must not be shared by concurrent
 *   calls.  wp (or NULL): the same weights as flf_conv3d_pack writes them;
 *   with it the layers of 32 to 128 channels with a side of 64 or more (and
 *   X <= 254) run on the tcgen05 tensor cores (flf_net_conv_wide_tcgen05(0)
 *   selects the mma.sync kernel instead).
 * flf_conv3d_wgrad: dw [27][Ci][Co] float += sum_v x[v + tap][ci] dy[v][co].
 *   The voxels are cut into chunks whose partial gradients go to ws (float,
 *   27 Ci Co per chunk; as many chunks as ws holds, one without ws) and are
 *   added to dw in chunk order.
 * Every reduction of these kernels runs in a fixed order (no floating-point
 *   atomics), so training repeats bit for bit on the same device; the loss
 *   value of flf_mse_grad alone is summed with atomics.
 * flf_conv3d_flip: w2[26 - tap][co][ci] = w[tap][ci][co]; conv3d with w2 is
 *   the data gradient.
 * flf_conv3d_pack: wp = w [27][Ci][Co] (Ci a multiple of 16) as the B operand
 *   blocks of the tcgen05 wide-layer kernel: per tap and 16 input channels
 *   one [2][Co][8] block (27 Ci Co bf16 in all, 16-byte aligned).
 * flf_bias_grad: db[c] += sum over the M rows of g[M][C] (C <= 128); row
 *   blocks of 2048 have their sums in ws (float, C per block; as many blocks as
 *   ws holds, one without ws), added in block order.
 * flf_pool2 / flf_pool2_bwd: 2x2x2 average pooling (Z, Y, X even) and its
 *   adjoint plus an optional second gradient gskip, times (act > 0) if act.
 * flf_up2_add / flf_up2_bwd: out = nearest 2x upsampling of low (+ skip);
 *   adjoint: 2x2x2 block sums times (act > 0) if act.  Shapes are those of
 *   the full-resolution tensor; flf_up2_add takes C / 8 a power of two.
 * flf_mse_grad: loss += mean((y[:, 0] - target)^2), g = its gradient in
 *   channel 0 (other channels 0); M voxels, y / g [M][C] bf16.
 * flf_adam: Adam step on FP32 weights w with gradient g and moments m, v
 *   (bias corrections c1, c2, decoupled weight decay wd); writes the BF16
 *   copy wb when not NULL.
 * flf_render_blobs: vol [Z][Y][X] float += amp exp(-d^2 / 2 sigma^2) within
 *   3 sigma of each pts[k] = (z, y, x, amp) (float4 array).  With acc (Z Y X
 *   int64, 8-byte aligned, overwritten) the terms are summed exactly as 32.32
 *   fixed-point integers, so the result does not depend on the order of
 *   arrival (per-voxel totals below 2^31); without it, FP32 atomics. */
int flf_conv3d(const void *x, const void *w, const float *bias, const void *mask, void *y, int B, int Z, int Y, int X,
               int Ci, int Co, int relu, float *ws, long long ws_elems, const void *wp, void *stream);
int flf_conv3d_wgrad(const void *x, const void *dy, float *dw, int B, int Z, int Y, int X, int Ci, int Co,
                     float *ws, long long ws_elems, void *stream);
/* flf_conv3d_tc: flf_conv3d for 16 -> 16 channels on the tcgen05 tensor cores
 * (accumulators in TMEM).  rows = 0: the warp-specialised kernel (TMA loads
 * of input slabs into a shared-memory ring, one MMA-issuing thread, two TMEM
 * accumulator stages, 4 epilogue warps; 4 x 128-voxel tiles walking z);
 * rows = 1, 4 or 5: single-role kernels with tiles of 1 or 4 rows x 128
 * voxels (5 = 4 rows, double-buffered).  flf_net_status: FLF_OK, or
 * FLF_E_TIMEOUT when a bounded wait inside one gave up since the last call.
 * flf_net_conv16_tcgen05(mode): the kernels flf_conv3d and flf_ws_head use for
 * 16 / 32 -> 16 / 32 channels: 0 = the mma.sync kernels; 1 = the
 * warp-specialised tcgen05 kernel (32-byte swizzled TMA slabs, z taps folded
 * into N) for 16 -> 16 and mma.sync for the 32-channel layers; 2 (default) =
 * tcgen05 for all of them.  Returns the previous setting. */
int flf_conv3d_tc(const void *x, const void *w, const float *bias, const void *mask, void *y, int B, int Z, int Y,
                  int X, int relu, int rows, void *stream);
/* flf_conv3d_x1: the 3x3x1 convolution (the 9 taps (dz, dy) at the centre x
 * offset, tap index dx = 1) of a 16 -> 16 channel layer whose input carries
 * the x neighbours as channels (the warm start's first layer): y = act(conv +
 * bias).  The taps with dx != 1 of w [27][16][16] are ignored by the tcgen05
 * kernel and must be zero for the mma.sync kernel (flf_net_conv16_tcgen05(0)),
 * which computes the full 3x3x3 sum. */
int flf_conv3d_x1(const void *x, const void *w, const float *bias, void *y, int B, int Z, int Y, int X, int relu,
                  void *stream);
/* flf_conv3d_pool: y = act(conv3x3x3(x, w) + bias) for 16 -> 16 channels and
 * pooled [B][Z/2][Y/2][X/2][16] = the 2x2x2 average pooling of y (flf_pool2 of
 * y, the same bits), written from the convolution's epilogue on the tcgen05
 * kernel (the encoder's last full-resolution layer and its pooling).  Z, Y, X
 * even. */
int flf_conv3d_pool(const void *x, const void *w, const float *bias, void *y, void *pooled, int B, int Z, int Y,
                    int X, int relu, void *stream);
int flf_net_status(void);
int flf_net_conv16_tcgen05(int mode);
/* Number of kernel launches the network entry points above have made since
 * the library was loaded (all threads). */
long long flf_net_launches(void);
/* Wide layers (a side of 64 or 128 channels) when flf_conv3d gets packed
 * weights: 0 = the mma.sync kernel; 1 (default) = the tcgen05 kernel with the
 * rows per work item chosen from the shape; 2..5 = the tcgen05 kernel with
 * 1..4 tiles of 128 padded-row positions per work item.  Returns the previous
 * value. */
int flf_net_conv_wide_tcgen05(int mode);
int flf_conv3d_flip(const void *w, void *w2, int Ci, int Co, void *stream);
int flf_conv3d_pack(const void *w, void *wp, int Ci, int Co, void *stream);
int flf_bias_grad(const void *g, float *db, long long M, int C, float *ws, long long ws_elems, void *stream);
int flf_pool2(const void *in, void *out, int B, int Z, int Y, int X, int C, void *stream);
int flf_pool2_bwd(const void *gpool, const void *gskip, const void *act, void *gin, int B, int Z, int Y, int X, int C,
                  void *stream);
int flf_up2_add(const void *low, const void *skip, void *out, int B, int Z, int Y, int X, int C, void *stream);
int flf_up2_bwd(const void *g, const void *act, void *glow, int B, int Z, int Y, int X, int C, void *stream);
int flf_mse_grad(const void *y, const float *target, void *g, float *loss, long long M, int C, void *stream);
int flf_adam(float *w, const float *g, float *m, float *v, void *wb, long long n, float lr, float b1, float b2,
             float eps, float c1, float c2, float wd, void *stream);
int flf_render_blobs(float *vol, int Z, int Y, int X, const float *pts, int npts, float sigma, void *acc,
                     void *stream);
/* Warm-start inference glue.  flf_ws_input: network input [T][Zp][Yp][Xp][16]
 * bf16 from Htf [Z][T][Y][X] float and the sensitivity maps HtH1, Ht1
 * [Z][Y][X]: with the features f0 = Htf / HtH1 / m_t (m_t = frame mean of
 * Htf / HtH1, whose sums are left in sum_x1 [T]), f1 = Htf / Ht1 / m_t,
 * f2 = HtH1 * c2, f3 = Ht1 * c3, channel 4k + j (k = 0..2) holds f_j at
 * x + k - 1 (the x neighbours as channels, for the 3x3x1 first layer
 * flf_conv3d_x1), channels 12..15 and the padding 0.  flf_ws_head: the start volume
 * x0 [Z][T][Y][X] = max(conv3x3x3(d, w)[0] + bias, floor) * m_t from the last
 * features d [T][Zp][Yp][Xp][16] and the head's BF16 weights w [27][16][16]
 * (output channel 0 is used). */
int flf_ws_input(const float *htf, const float *hth1, const float *ht1, float *sum_x1, void *out, int T, int Z,
                 int Y, int X, int Zp, int Yp, int Xp, float c2, float c3, void *stream);
int flf_ws_head(const void *d, const void *w, float bias, float floor_, const float *sum_x1, float *x0, int T, int Z,
                int Y, int X, int Zp, int Yp, int Xp, void *stream);

/* CUDA graph of a whole RL run (the replay form of flf_rl_iterate): the
 * launches of `iters` iterations over T frames of Y x X images are captured
 * once, with these pointers baked in, and each flf_graph_launch replays them
 * with one call, as one unit of stream work.  Create builds the transfer
 * matrices and sizes every workspace first; the context must outlive the
 * graph, and its workspaces must not shrink meanwhile (flf_clear_cache
 * invalidates graphs).  Replays on one context must not overlap.  Replaces the
 * per-iteration calls of the DeconvRL loop (lfdeconv.py:185-196). */
typedef struct flf_graph flf_graph;
int flf_rl_graph_create(flf_ctx *ctx, flf_graph **out, float *x_dev, const float *ref_dev,
                        const float *norm_dev, int variant, int iters, int T, int Y, int X);
/* The whole deconvolution of T frames as one graph: the back projection of
 * img_dev [T][Y][X] into htf_dev [Z][T][Y][X], the start volume x = Htf (as
 * the reference's time-series driver starts, deconvolve_time_series.py:28) and
 * `iters` Prevedel iterations on x_dev, with these pointers baked in. */
int flf_deconv_graph_create(flf_ctx *ctx, flf_graph **out, const float *img_dev, float *htf_dev, float *x_dev,
                            int iters, int T, int Y, int X);
/* One graph that runs `parts` (graphs of one context, e.g. the deconvolution
 * graphs of several image sizes, whose transfer matrices the geometry cache
 * keeps resident) in order: one flf_graph_launch for all of them.  The parts
 * stay owned by the caller; destroy the combined graph with
 * flf_graph_destroy. */
int flf_graph_combine(flf_graph **out, flf_graph *const *parts, int n);
int flf_graph_launch(flf_graph *graph, void *stream);
int flf_graph_kernels(const flf_graph *graph);   /* kernels per replay */
int flf_graph_destroy(flf_graph *graph);

/* Autotuner (the GB300 counterpart of the reference's FFTW planning mode,
 * SetPlanningMode, and of its block-shape knobs, projector.py:26-36): for
 * T frames of Y x X images, builds the transfer matrices if needed, then
 * times the multiply-accumulate of both directions on the transform group
 * that streams the most bytes, over ring stages {2, 3} x rows per chunk
 * {8, 10, 12, 16, 20} x row split {1, 2} (shapes that fit shared memory).
 * The fastest shape is kept with this image shape's transfer matrices and
 * used by every later call on it; out4 = {stages, rows per chunk forward,
 * rows per chunk backward, split}.  Runs work on `stream` and waits for it.
 * Results do not depend on the launch shape beyond rounding. */
int flf_autotune(flf_ctx *ctx, int T, int Y, int X, int *out4, void *stream);

/* Apply a launch shape found earlier by flf_autotune (for example read back
 * from a cache file) to the prepared geometry of Y x X images. */
int flf_set_tuned(flf_ctx *ctx, int Y, int X, const int *in4);

/* Rectification resample (replaces the interpolation of the reference's
 * rectify.RectifyImage, rectify.py:56-57, a RectBivariateSpline with
 * kx = ky = 1, i.e. bilinear): out[r][c] = bilinear value of the image
 * img [H][W] (float, row-major) at (yq[r], xq[c]), 0-based pixel
 * coordinates, in double precision; coordinates outside the image are
 * clamped to its edge.  The query grids are built by the caller exactly as
 * the reference builds them.  Device pointers; no context; allocates
 * nothing.  Errors are read with flf_last_error(NULL, ...). */
int flf_resample_bilinear(const float *img_dev, int H, int W, const double *yq_dev, int ny,
                          const double *xq_dev, int nx, double *out_dev, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* FLF_H */
