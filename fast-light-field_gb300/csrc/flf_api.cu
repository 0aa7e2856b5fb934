// C ABI of libflf.so (declared in include/flf.h): context, PSF upload,
// transfer-matrix precompute, and the forward / back projection and
// Richardson-Lucy sequences built from the kernels in flf_kernels.cu.
#include "flf_internal.cuh"
#include "../../include/flf.h"

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <map>
#include <string>
#include <vector>

using namespace flf;

namespace {

thread_local std::string g_create_error;

struct Workspace {
  void *p = nullptr;
  size_t bytes = 0;
};

// Planes sharing one lenslet-grid transform size.  Every plane uses the
// smallest size its own kernel radius allows; planes with equal sizes share
// one group (one set of launches per projection).
struct Group {
  int f = 0, fh = 0, fq = 0, nkp = 0, nquads = 0, R = 0;   // nkp = fq^2 half blocks, nquads = fq(fq+1)/2
  FftPlan plan{};
  float2 *tw = nullptr;       // float twiddles [f]
  double2 *tw64 = nullptr;    // double twiddles [f]
  float2 *P[2] = {nullptr, nullptr};   // packed matrices [slot][nkp half blocks][nrow][RS]
  bool built[2] = {false, false};
  std::vector<int> planes;    // plane ids of the group, ascending (slot = index)
  int *d_ids = nullptr;       // device copy of `planes`
  int *d_slots = nullptr;     // 0..n-1
};

struct Geometry {
  bool valid = false;
  int Y = 0, X = 0, Ly = 0, Lx = 0, fp64 = 0, uniform_f = 0;
  int tuned[4] = {0, 0, 0, 0};   // multiply-accumulate launch shape chosen by flf_autotune
                                 // (stages, chunk rows forward, backward, split); 0: context options
  std::vector<Group> groups;
  std::vector<int> plane_group, plane_slot;
  bool built(int dir) const {
    for (const Group &g : groups)
      if (!g.built[dir]) return false;
    return !groups.empty();
  }
  int max_f() const {
    int m = 0;
    for (const Group &g : groups) m = std::max(m, g.f);
    return m;
  }
};

}  // namespace

struct flf_ctx {
  int device = 0, N = 0, nz = 0;
  Layout L{};
  std::vector<float *> dH[2];
  std::vector<int> h[2];
  Geometry geo;
  // index tables (device)
  short4 *d_rowS = nullptr, *d_oslots = nullptr;
  short *d_rowF = nullptr;
  short *d_slotcol = nullptr, *d_colslot = nullptr;
  int *d_rep_ch = nullptr, *d_rep_row = nullptr, *d_rep_kind = nullptr;
  int *d_planes_all = nullptr;
  int *d_planes_user = nullptr;   // per-call plane subsets: ids then slots, per group
  int planes_user_cap = 0;
  int *d_zero = nullptr;
  std::vector<int> rep_ch, rep_row, rep_kind;
  Workspace wsS, wsO;             // channel spectra in / out of the multiply-accumulate
  Workspace wsCvol;               // channel-major volume side (forward input, back projection output)
  Workspace wsCimg;               // channel-major image side (back projection input, forward output)
  Workspace wsCy;                 // channel-major measured image (standard RL numerator)
  int num_sms = 0;
  int req_f = 0, req_fp64 = 0;   // transform size / precision asked for by flf_prepare
  int opt_stages = 2;            // tunable: MAC shared-memory pipeline stages
  int opt_chunk_rows[2] = {12, 12};   // tunable: stored rows per pipeline stage (forward, backward)
  int opt_split = 1;             // tunable: threads sharing one orbit's rows
  int opt_ctas_per_sm = 16;      // tunable: multiply-accumulate CTAs per SM the plane grouping aims at
  int opt_plane_sizes = 1;       // 1: transform size per plane (grouped); 0: one size for all
  int opt_geometry_cache = 2;    // geometries of other image shapes kept resident (most recent first)
  std::vector<Geometry> parked;  // those geometries
  unsigned long long mem_epoch = 0;   // bumped whenever a workspace or geometry buffer is freed
  int opt_streams = 2;           // transform groups alternate over this many streams (1 or 2)
  int opt_release_psf = 0;       // free the PSF quadrants after the precompute of both directions
  long long opt_wait_us = 1000000;   // limit of the multiply-accumulate's waits for a ring slot
  int opt_drop_chunk = -1;       // test of the bounded waits: a chunk the first CTA never issues
  bool psf_released = false;
  cudaStream_t s2 = nullptr;     // the second stream, and the events that fork / chain / join it
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr, ev_chain = nullptr;
  void *noalloc_scratch = nullptr;   // device address of the fixed scratch of flf_backward_noalloc
  int *h_err = nullptr;          // host-mapped flag set by bounded device waits
  int *d_err = nullptr;
  // per-kernel launch statistics; event timing when profiling is on
  struct KStat { long long launches = 0; double ms = 0, bytes = 0; };
  struct Pending { std::string name; cudaEvent_t a, b; };
  std::map<std::string, KStat> kstats;
  std::vector<Pending> pending;
  std::vector<cudaEvent_t> evpool;
  bool profiling = false;
  std::string err;
};

namespace {

int fail(flf_ctx *ctx, int code, const char *fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  if (ctx) ctx->err = buf;
  else g_create_error = buf;
  return code;
}

#define CUDA_TRY(ctx, call)                                                                   \
  do {                                                                                        \
    cudaError_t e_ = (call);                                                                  \
    if (e_ != cudaSuccess)                                                                    \
      return fail(ctx, FLF_E_CUDA, "%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_),   \
                  __FILE__, __LINE__);                                                        \
  } while (0)

cudaEvent_t get_event(flf_ctx *ctx) {
  if (!ctx->evpool.empty()) {
    cudaEvent_t e = ctx->evpool.back();
    ctx->evpool.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  cudaEventCreate(&e);
  return e;
}

void resolve_pending(flf_ctx *ctx) {
  for (auto &p : ctx->pending) {
    float ms = 0.f;
    if (cudaEventSynchronize(p.b) == cudaSuccess && cudaEventElapsedTime(&ms, p.a, p.b) == cudaSuccess)
      ctx->kstats[p.name].ms += ms;
    ctx->evpool.push_back(p.a);
    ctx->evpool.push_back(p.b);
  }
  ctx->pending.clear();
}

// Launches `fn` (returning cudaError_t), counts it under `name` with its
// algorithmic bytes, and brackets it with events on `s` when profiling.
template <typename F>
int counted_launch(flf_ctx *ctx, const char *name, double bytes, cudaStream_t s, F &&fn) {
  cudaEvent_t a = nullptr, b = nullptr;
  if (ctx->profiling) {
    if (ctx->pending.size() > 8192) resolve_pending(ctx);
    a = get_event(ctx);
    b = get_event(ctx);
    cudaEventRecord(a, s);
  }
  cudaError_t e = fn();
  if (e != cudaSuccess)
    return fail(ctx, FLF_E_CUDA, "launch of %s failed: %s", name, cudaGetErrorString(e));
  if (ctx->profiling) {
    cudaEventRecord(b, s);
    ctx->pending.push_back({name, a, b});
  }
  auto &k = ctx->kstats[name];
  k.launches++;
  k.bytes += bytes;
  return FLF_OK;
}

#define LAUNCH(ctx, name, bytes, s, expr)                                  \
  do {                                                                     \
    int rc_ = counted_launch(ctx, name, (double)(bytes), s, [&]() { return (expr); }); \
    if (rc_ != FLF_OK) return rc_;                                         \
  } while (0)

// Report a bounded device wait that gave up in an earlier launch.
int check_device_flag(flf_ctx *ctx) {
  if (ctx->h_err && *(volatile int *)ctx->h_err) {
    const int code = *(volatile int *)ctx->h_err;
    *(volatile int *)ctx->h_err = 0;
    return fail(ctx, FLF_E_TIMEOUT, "a bounded wait in the multiply-accumulate pipeline gave up (code %d)", code);
  }
  return FLF_OK;
}

bool is_smooth_even(int n) {
  if (n < 2 || (n & 1)) return false;
  for (int p : {2, 3, 5, 7})
    while (n % p == 0) n /= p;
  return n == 1;
}

FftPlan make_plan(int n) {
  FftPlan pl{};
  pl.n = n;
  int m = n, k = 0;
  while (m % 4 == 0) { pl.rad[k++] = 4; m /= 4; }
  while (m % 2 == 0) { pl.rad[k++] = 2; m /= 2; }
  for (int p : {3, 5, 7})
    while (m % p == 0) { pl.rad[k++] = p; m /= p; }
  pl.nst = k;
  return pl;
}

int ensure_ws(flf_ctx *ctx, Workspace &w, size_t bytes) {
  if (w.bytes >= bytes) return FLF_OK;
  if (w.p) {
    cudaFree(w.p);
    ctx->mem_epoch++;
  }
  w.p = nullptr;
  w.bytes = 0;
  cudaError_t e = cudaMalloc(&w.p, bytes);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return fail(ctx, FLF_E_NOMEM, "cudaMalloc(%zu bytes) for workspace failed: %s", bytes,
                cudaGetErrorString(e));
  }
  w.bytes = bytes;
  return FLF_OK;
}

void free_geometry(Geometry &G) {
  for (Group &g : G.groups) {
    void *ptrs[] = {g.tw, g.tw64, g.P[0], g.P[1], g.d_ids, g.d_slots};
    for (void *p : ptrs)
      if (p) cudaFree(p);
  }
  G = Geometry();
}

// Keep a geometry of another image shape resident (most recent first), within
// opt_geometry_cache entries; the oldest beyond that is freed.
void park_geometry(flf_ctx *ctx, Geometry &&G) {
  if (!G.valid || ctx->opt_geometry_cache <= 0) {
    free_geometry(G);
    ctx->mem_epoch++;
    return;
  }
  ctx->parked.insert(ctx->parked.begin(), std::move(G));
  G = Geometry();
  while ((int)ctx->parked.size() > ctx->opt_geometry_cache) {
    ctx->mem_epoch++;
    free_geometry(ctx->parked.back());
    ctx->parked.pop_back();
  }
}

// Free the active geometry and every parked one (the PSFs or the size rule changed).
void free_all_geometries(flf_ctx *ctx) {
  ctx->mem_epoch++;
  free_geometry(ctx->geo);
  for (Geometry &g : ctx->parked) free_geometry(g);
  ctx->parked.clear();
}

// Host-side index tables of the packed layout (see flf_internal.cuh).
int build_tables(flf_ctx *ctx) {
  const int N = ctx->N, NN = N * N, c = N / 2;
  const Layout &L = ctx->L;
  auto My = [&](int i) { return (N - 1 - i / N) * N + i % N; };
  auto Mx = [&](int i) { return (i / N) * N + (N - 1 - i % N); };
  auto Mxy = [&](int i) { return NN - 1 - i; };
  // Slot order of a stored row: for the c^2 generic orbits o = be*c + al,
  // four blocks of c^2 slots (q, My q, Mx q, Mxy q of every orbit), then the
  // c orbits [q, My q] (alpha = c) as two blocks of c, the c orbits [q, Mx q]
  // (beta = c) as two blocks of c, then the centre.  A warp's threads (one
  // orbit each) read each block with consecutive addresses.
  const int c2 = c * c;
  std::vector<short> slotcol(NN, -1);
  for (int be = 0; be < c; be++)
    for (int al = 0; al < c; al++) {
      const int o = be * c + al, q = be * N + al;
      slotcol[o] = q; slotcol[c2 + o] = My(q); slotcol[2 * c2 + o] = Mx(q); slotcol[3 * c2 + o] = Mxy(q);
    }
  for (int j = 0; j < c; j++) {
    const int qa = j * N + c, qb = c * N + j;
    slotcol[4 * c2 + j] = qa; slotcol[4 * c2 + c + j] = My(qa);
    slotcol[4 * c2 + 2 * c + j] = qb; slotcol[4 * c2 + 3 * c + j] = Mx(qb);
  }
  slotcol[4 * c2 + 4 * c] = c * N + c;
  for (int sl = 0; sl < NN; sl++)
    if (slotcol[sl] < 0) return fail(ctx, FLF_E_STATE, "internal: slot table");
  std::vector<short> colslot(NN, -1);
  for (int s = 0; s < NN; s++) colslot[slotcol[s]] = s;

  auto Tr = [&](int i) { return (i % N) * N + i / N; };
  // virtual slots [q, My q, Mx q, Mxy q] of each output orbit (degenerate orbits
  // repeat their entries) and the slots of the transposed channels in the same order
  std::vector<short4> oslots(2 * L.nthr);
  for (int o = 0; o < L.nthr; o++) {
    int off[4];
    if (o < c2) {
      off[0] = o; off[1] = c2 + o; off[2] = 2 * c2 + o; off[3] = 3 * c2 + o;
    } else if (o < c2 + c) {
      const int j = o - c2;
      off[0] = off[2] = 4 * c2 + j; off[1] = off[3] = 4 * c2 + c + j;
    } else if (o < c2 + 2 * c) {
      const int j = o - c2 - c;
      off[0] = off[1] = 4 * c2 + 2 * c + j; off[2] = off[3] = 4 * c2 + 3 * c + j;
    } else {
      off[0] = off[1] = off[2] = off[3] = NN - 1;
    }
    int offT[4];
    for (int k = 0; k < 4; k++) offT[k] = colslot[Tr(slotcol[off[k]])];
    oslots[o] = make_short4(off[0], off[1], off[2], off[3]);
    oslots[L.nthr + o] = make_short4(offT[0], offT[1], offT[2], offT[3]);
  }
  // row groups of a half block with their operands for the own frequency pair
  // (use 0) and, through the transpose, for the other one of the quad (use 1)
  std::vector<short4> rowS(2 * L.ngrp, make_short4(0, 0, 0, 0));
  std::vector<short> rowF(2 * L.ngrp, 0);
  ctx->rep_ch.clear(); ctx->rep_row.clear(); ctx->rep_kind.clear();
  auto generic_ops = [&](int x, bool mxrow, short4 &si, short &fl) {
    si = make_short4(x, Mxy(x), NN + My(x), NN + Mx(x));
    fl = (short)((1 << 1) | (1 << 3) | (mxrow ? 0xF0 : 0));
  };
  int row = 0, grp = 0;
  std::vector<std::pair<int, int>> orbits;   // transposable orbits (a' < b) first, then the diagonal ones
  for (int b = 0; b < c; b++)
    for (int ap = 0; ap < b; ap++) orbits.push_back({b, ap});
  for (int b = 0; b < c; b++) orbits.push_back({b, b});
  for (const auto &ob : orbits) {
    const int b = ob.first, ap = ob.second;
    for (int a : {ap, N - 1 - ap}) {
        const int i = b * N + a;
        const bool trans = ap < b, mxrow = a > c;
        generic_ops(i, mxrow, rowS[grp], rowF[grp]);
        if (trans) {
          generic_ops(Tr(i), mxrow, rowS[L.ngrp + grp], rowF[L.ngrp + grp]);
          rowF[grp] |= kRowTransposable;
          rowF[L.ngrp + grp] |= kRowTransposable;
        }
        ctx->rep_ch.push_back(i); ctx->rep_row.push_back(row); ctx->rep_kind.push_back(0);
        row++; grp++;
      }
  }
  if (row != L.nrowG) return fail(ctx, FLF_E_STATE, "internal: generic row table size");
  for (int k = 0; k <= c; k++) {
    const bool centre = k == c;
    const int i = centre ? c * N + c : k * N + c;
    if (centre) {
      rowS[grp] = make_short4(i, NN + i, 0, 0);
      rowF[grp] = (short)((1 << 5) | (1 << 10) | (1 << 11));
    } else {
      rowS[grp] = make_short4(i, NN + i, NN + My(i), My(i));
      rowF[grp] = (short)((1 << 5) | (1 << 7) | kRowTransposable);
      const int x = Tr(i);   // (c, b): the row pair read through the transpose, conjugated u* terms
      rowS[L.ngrp + grp] = make_short4(x, NN + x, NN + Mx(x), Mx(x));
      rowF[L.ngrp + grp] = (short)((1 << 1) | (1 << 2) | (1 << 5) | (1 << 7) | kRowTransposable);
    }
    ctx->rep_ch.push_back(i); ctx->rep_row.push_back(row); ctx->rep_kind.push_back(1);
    row += 2; grp++;
  }
  if (row != L.nrow || grp != L.ngrp) return fail(ctx, FLF_E_STATE, "internal: row table size");
  const int nrepAll = (int)ctx->rep_ch.size();
  CUDA_TRY(ctx, cudaMalloc(&ctx->d_rowS, sizeof(short4) * rowS.size()));
  CUDA_TRY(ctx, cudaMemcpy(ctx->d_rowS, rowS.data(), sizeof(short4) * rowS.size(), cudaMemcpyHostToDevice));
  CUDA_TRY(ctx, cudaMalloc(&ctx->d_rowF, sizeof(short) * rowF.size()));
  CUDA_TRY(ctx, cudaMemcpy(ctx->d_rowF, rowF.data(), sizeof(short) * rowF.size(), cudaMemcpyHostToDevice));
  CUDA_TRY(ctx, cudaMalloc(&ctx->d_oslots, sizeof(short4) * oslots.size()));
  CUDA_TRY(ctx, cudaMemcpy(ctx->d_oslots, oslots.data(), sizeof(short4) * oslots.size(), cudaMemcpyHostToDevice));
  CUDA_TRY(ctx, cudaMalloc(&ctx->d_slotcol, sizeof(short) * NN));
  CUDA_TRY(ctx, cudaMemcpy(ctx->d_slotcol, slotcol.data(), sizeof(short) * NN, cudaMemcpyHostToDevice));
  CUDA_TRY(ctx, cudaMalloc(&ctx->d_colslot, sizeof(short) * NN));
  CUDA_TRY(ctx, cudaMemcpy(ctx->d_colslot, colslot.data(), sizeof(short) * NN, cudaMemcpyHostToDevice));
  CUDA_TRY(ctx, cudaMalloc(&ctx->d_rep_ch, sizeof(int) * nrepAll));
  CUDA_TRY(ctx, cudaMemcpy(ctx->d_rep_ch, ctx->rep_ch.data(), sizeof(int) * nrepAll, cudaMemcpyHostToDevice));
  CUDA_TRY(ctx, cudaMalloc(&ctx->d_rep_row, sizeof(int) * nrepAll));
  CUDA_TRY(ctx, cudaMemcpy(ctx->d_rep_row, ctx->rep_row.data(), sizeof(int) * nrepAll, cudaMemcpyHostToDevice));
  CUDA_TRY(ctx, cudaMalloc(&ctx->d_rep_kind, sizeof(int) * nrepAll));
  CUDA_TRY(ctx, cudaMemcpy(ctx->d_rep_kind, ctx->rep_kind.data(), sizeof(int) * nrepAll, cudaMemcpyHostToDevice));
  std::vector<int> all(ctx->nz);
  for (int z = 0; z < ctx->nz; z++) all[z] = z;
  CUDA_TRY(ctx, cudaMalloc(&ctx->d_planes_all, sizeof(int) * std::max(1, ctx->nz)));
  CUDA_TRY(ctx, cudaMemcpy(ctx->d_planes_all, all.data(), sizeof(int) * ctx->nz, cudaMemcpyHostToDevice));
  CUDA_TRY(ctx, cudaMalloc(&ctx->d_zero, sizeof(int)));
  CUDA_TRY(ctx, cudaMemset(ctx->d_zero, 0, sizeof(int)));
  return FLF_OK;
}

int kernel_radius(const flf_ctx *ctx, int hh) { return ((hh - 1) / 2 + ctx->N - 1) / ctx->N; }

int imgs_per_cta(int f, int fp64, size_t budget) {
  int b = 1;
  while (b < 16 && rfft2_smem_bytes(f, b + 1, fp64) <= budget) b++;
  return b;
}

// Transfer matrices of one direction for the planes of one group.
int build_group(flf_ctx *ctx, Group &G, int fp64, int dir, cudaStream_t s) {
  const Layout &L = ctx->L;
  const int NN = L.NN, f = G.f, fh = G.fh, ng = (int)G.planes.size();
  const size_t plane_elems = (size_t)G.nkp * L.nrow * L.RS;
  const size_t bytes = plane_elems * ng * sizeof(float2);
  if (!G.P[dir]) {
    cudaError_t e = cudaMalloc(&G.P[dir], bytes);
    if (e != cudaSuccess) {
      cudaGetLastError();
      return fail(ctx, FLF_E_NOMEM,
                  "cudaMalloc(%zu bytes) for the transfer matrices of direction %d failed: %s",
                  bytes, dir, cudaGetErrorString(e));
    }
  }
  CUDA_TRY(ctx, cudaMemsetAsync(G.P[dir], 0, bytes, s));
  const size_t rsz = fp64 ? sizeof(double) : sizeof(float);
  const size_t per_rep = (size_t)NN * ((size_t)f * f * rsz + (size_t)f * fh * 2 * rsz);
  const int nrepAll = (int)ctx->rep_ch.size();
  int chunk = (int)std::max<size_t>(1, std::min<size_t>(nrepAll, (size_t)(512u << 20) / per_rep));
  Workspace wk, wspec;
  int rc = ensure_ws(ctx, wk, (size_t)chunk * NN * f * f * rsz);
  if (rc == FLF_OK) rc = ensure_ws(ctx, wspec, (size_t)chunk * NN * f * fh * 2 * rsz);
  if (rc != FLF_OK) {
    if (wk.p) cudaFree(wk.p);
    if (wspec.p) cudaFree(wspec.p);
    return rc;
  }
  const int ipc = imgs_per_cta(f, fp64, 200 * 1024);
  for (int sl = 0; sl < ng && rc == FLF_OK; sl++) {
    const int z = G.planes[sl];
    const int hh = ctx->h[dir][z];
    for (int r0 = 0; r0 < nrepAll && rc == FLF_OK; r0 += chunk) {
      const int nr = std::min(chunk, nrepAll - r0);
      BuildKParams bk{};
      bk.N = ctx->N; bk.h = hh; bk.ch = (hh - 1) / 2; bk.R = kernel_radius(ctx, hh); bk.f = f;
      bk.H = ctx->dH[dir][z]; bk.rep_ch = ctx->d_rep_ch; bk.rep0 = r0; bk.nrep_chunk = nr;
      bk.dst = wk.p; bk.fp64 = fp64;
      cudaError_t e = launch_build_k(bk, nr * NN, s);
      if (e == cudaSuccess) {
        Rfft2Params rp{};
        rp.plan = G.plan; rp.N = ctx->N; rp.nimg = nr * NN; rp.mode = 1;
        rp.src_img = wk.p; rp.dst = wspec.p;
        rp.twiddle = fp64 ? (const void *)G.tw64 : (const void *)G.tw;
        rp.imgs_per_cta = ipc; rp.nq_rows = f / 2;
        e = launch_rfft2(rp, fp64, s);
      }
      if (e == cudaSuccess) {
        PackParams pp{};
        pp.L = L; pp.f = f; pp.fh = fh; pp.fq = G.fq; pp.nkp = G.nkp;
        pp.spec = wspec.p; pp.rep0 = r0; pp.nrep_chunk = nr;
        pp.rep_row = ctx->d_rep_row; pp.rep_kind = ctx->d_rep_kind; pp.rep_ch = ctx->d_rep_ch;
        pp.col_slot = ctx->d_colslot;
        pp.P = G.P[dir] + plane_elems * sl;
        pp.scale = 1.0 / ((double)f * (double)f);
        pp.fp64 = fp64;
        e = launch_pack(pp, s);
      }
      if (e != cudaSuccess)
        rc = fail(ctx, FLF_E_CUDA, "precompute launch failed: %s", cudaGetErrorString(e));
    }
  }
  cudaError_t es = cudaStreamSynchronize(s);
  if (wk.p) cudaFree(wk.p);
  if (wspec.p) cudaFree(wspec.p);
  if (rc != FLF_OK) return rc;
  if (es != cudaSuccess) return fail(ctx, FLF_E_CUDA, "precompute failed: %s", cudaGetErrorString(es));
  G.built[dir] = true;
  return FLF_OK;
}

// Transfer matrices of one direction for all uploaded planes.
int build_direction(flf_ctx *ctx, int dir, cudaStream_t s) {
  for (int z = 0; z < ctx->nz; z++)
    if (!ctx->dH[dir][z])
      return fail(ctx, FLF_E_STATE, "PSF for plane %d direction %d was not uploaded%s", z, dir,
                  ctx->psf_released ? " (the PSFs were released after the last precompute: upload them again "
                                      "to build transfer matrices for another image shape)" : "");
  ctx->psf_released = false;
  for (Group &g : ctx->geo.groups)
    if (!g.built[dir])
      if (int rc = build_group(ctx, g, ctx->geo.fp64, dir, s)) return rc;
  return FLF_OK;
}

// Every PSF of the directions in dmask (bit d) is uploaded, or they were
// released after a precompute (a rebuild then fails with that explanation).
int check_psfs(flf_ctx *ctx, int dmask) {
  for (int d = 0; d < 2; d++)
    if ((dmask >> d) & 1)
      for (int z = 0; z < ctx->nz; z++)
        if (!ctx->dH[d][z] && !ctx->psf_released)
          return fail(ctx, FLF_E_STATE, "%s PSF for plane %d was not uploaded", d ? "backward" : "forward", z);
  return FLF_OK;
}

// With the option "release_psf", free the uploaded PSF quadrants once both
// directions' transfer matrices of the current image shape exist (they are
// only read by the precompute); the sizes are kept.
void maybe_release_psfs(flf_ctx *ctx) {
  if (!ctx->opt_release_psf || !ctx->geo.built(FLF_DIR_FORWARD) || !ctx->geo.built(FLF_DIR_BACKWARD)) return;
  bool any = false;
  for (int d = 0; d < 2; d++)
    for (float *&p : ctx->dH[d])
      if (p) {
        if (!any) cudaDeviceSynchronize();
        cudaFree(p);
        p = nullptr;
        any = true;
      }
  if (any) {
    ctx->psf_released = true;
    ctx->mem_epoch++;
  }
}

int smooth_at_least(int n) {
  int f = std::max(n, 2);
  while (!is_smooth_even(f)) f++;
  return f;
}

// Kernel radius of plane z in lenslets.  Released PSFs keep their sizes, so
// the radius (and with it the geometry of every image shape) stays the one the
// transfer matrices were built with.
int plane_radius(const flf_ctx *ctx, int z) {
  int R = 0;
  for (int d = 0; d < 2; d++)
    if (ctx->dH[d][z] || ctx->psf_released) R = std::max(R, kernel_radius(ctx, ctx->h[d][z]));
  return R;
}

int prepare(flf_ctx *ctx, int Y, int X, int fft_size, int fp64) {
  if (Y <= 0 || X <= 0) return fail(ctx, FLF_E_ARG, "image shape must be positive (got %d x %d)", Y, X);
  const int N = ctx->N, nz = ctx->nz;
  const int Ly = (Y + N - 1) / N, Lx = (X + N - 1) / N, Lm = std::max(Ly, Lx);
  int Rmax = 0;
  for (int z = 0; z < nz; z++) Rmax = std::max(Rmax, plane_radius(ctx, z));
  std::vector<int> fz(nz);
  if (fft_size > 0) {
    if (!is_smooth_even(fft_size))
      return fail(ctx, FLF_E_ARG, "fft_size %d must be even with prime factors in {2,3,5,7}", fft_size);
    const int need = std::max(Lm + Rmax, 2 * Rmax + 1);
    if (fft_size < need) return fail(ctx, FLF_E_ARG, "fft_size %d too small: need >= %d", fft_size, need);
    std::fill(fz.begin(), fz.end(), fft_size);
  } else if (!ctx->opt_plane_sizes) {
    std::fill(fz.begin(), fz.end(), smooth_at_least(std::max(Lm + Rmax, 2 * Rmax + 1)));
  } else {
    for (int z = 0; z < nz; z++) {
      const int R = plane_radius(ctx, z);
      fz[z] = smooth_at_least(std::max(Lm + R, 2 * R + 1));
    }
  }
  const int fmax = *std::max_element(fz.begin(), fz.end());
  if (fmax > kMaxF)
    return fail(ctx, FLF_E_ARG, "lenslet-grid transform size %d exceeds the supported maximum %d "
                "(image %d x %d, Nnum %d, kernel radius %d lenslets)", fmax, kMaxF, Y, X, N, Rmax);
  if (fp64 && fmax > kMaxF64) fp64 = 0;   // double buffers do not fit shared memory
  Geometry &G = ctx->geo;
  auto matches = [&](const Geometry &g) {
    if (!g.valid || g.Ly != Ly || g.Lx != Lx || g.fp64 != fp64 || (int)g.plane_group.size() != nz) return false;
    for (int z = 0; z < nz; z++)
      if (g.groups[g.plane_group[z]].f != fz[z]) return false;
    return true;
  };
  if (matches(G)) {
    G.Y = Y; G.X = X;
    return FLF_OK;
  }
  // another image shape: park the active geometry; reuse a parked one that fits
  for (size_t i = 0; i < ctx->parked.size(); i++)
    if (matches(ctx->parked[i])) {
      Geometry found = std::move(ctx->parked[i]);
      ctx->parked.erase(ctx->parked.begin() + i);
      park_geometry(ctx, std::move(G));
      G = std::move(found);
      G.Y = Y; G.X = X;
      return FLF_OK;
    }
  park_geometry(ctx, std::move(G));
  G.Y = Y; G.X = X; G.Ly = Ly; G.Lx = Lx; G.fp64 = fp64; G.uniform_f = fft_size;
  G.plane_group.assign(nz, -1);
  G.plane_slot.assign(nz, -1);
  std::vector<int> sizes(fz);
  std::sort(sizes.begin(), sizes.end());
  sizes.erase(std::unique(sizes.begin(), sizes.end()), sizes.end());
  for (int f : sizes) {
    Group g;
    g.f = f; g.fh = f / 2 + 1; g.fq = f / 2 + 1; g.nkp = g.fq * g.fq; g.nquads = g.fq * (g.fq + 1) / 2;
    g.plan = make_plan(f);
    for (int z = 0; z < nz; z++)
      if (fz[z] == f) {
        G.plane_group[z] = (int)G.groups.size();
        G.plane_slot[z] = (int)g.planes.size();
        g.planes.push_back(z);
        g.R = std::max(g.R, plane_radius(ctx, z));
      }
    G.groups.push_back(g);
  }
  for (Group &g : G.groups) {
    const int f = g.f;
    std::vector<float2> tw(f);
    std::vector<double2> tw64(f);
    for (int k = 0; k < f; k++) {
      // exp(-2 pi i k / f) in double, rounded once
      const double ang = -2.0 * M_PI * (double)k / (double)f;
      tw64[k] = make_double2(std::cos(ang), std::sin(ang));
      tw[k] = make_float2((float)tw64[k].x, (float)tw64[k].y);
    }
    std::vector<int> slots(g.planes.size());
    for (size_t i = 0; i < slots.size(); i++) slots[i] = (int)i;
    CUDA_TRY(ctx, cudaMalloc(&g.tw, sizeof(float2) * f));
    CUDA_TRY(ctx, cudaMemcpy(g.tw, tw.data(), sizeof(float2) * f, cudaMemcpyHostToDevice));
    CUDA_TRY(ctx, cudaMalloc(&g.tw64, sizeof(double2) * f));
    CUDA_TRY(ctx, cudaMemcpy(g.tw64, tw64.data(), sizeof(double2) * f, cudaMemcpyHostToDevice));
    CUDA_TRY(ctx, cudaMalloc(&g.d_ids, sizeof(int) * g.planes.size()));
    CUDA_TRY(ctx, cudaMemcpy(g.d_ids, g.planes.data(), sizeof(int) * g.planes.size(), cudaMemcpyHostToDevice));
    CUDA_TRY(ctx, cudaMalloc(&g.d_slots, sizeof(int) * slots.size()));
    CUDA_TRY(ctx, cudaMemcpy(g.d_slots, slots.data(), sizeof(int) * slots.size(), cudaMemcpyHostToDevice));
  }
  G.valid = true;
  return FLF_OK;
}

// The planes one projection call works on, split by transform group:
// for group g, n[g] planes with ids ids[g] (volume addressing) and slots
// slots[g] (rows of the group's packed matrices), both device arrays.
struct PlaneSet {
  std::vector<int> n;
  std::vector<const int *> ids, slots;
};

int check_planes_arg(flf_ctx *ctx, const int *planes, int nplanes) {
  if (!planes) {
    if (nplanes != ctx->nz) return fail(ctx, FLF_E_ARG, "planes == NULL requires nplanes == num_planes");
    return FLF_OK;
  }
  if (nplanes <= 0 || nplanes > ctx->nz) return fail(ctx, FLF_E_ARG, "nplanes %d out of range", nplanes);
  std::vector<char> seen(ctx->nz, 0);
  for (int i = 0; i < nplanes; i++) {
    if (planes[i] < 0 || planes[i] >= ctx->nz)
      return fail(ctx, FLF_E_ARG, "plane id %d out of range [0, %d)", planes[i], ctx->nz);
    if (seen[planes[i]]) return fail(ctx, FLF_E_ARG, "plane id %d listed twice", planes[i]);
    seen[planes[i]] = 1;
  }
  return FLF_OK;
}

// Requires a valid geometry.  planes == NULL: every plane.
int make_plane_set(flf_ctx *ctx, const int *planes, int nplanes, cudaStream_t s, PlaneSet &ps) {
  const Geometry &G = ctx->geo;
  const int ng = (int)G.groups.size();
  ps.n.assign(ng, 0);
  ps.ids.assign(ng, nullptr);
  ps.slots.assign(ng, nullptr);
  if (!planes) {
    for (int g = 0; g < ng; g++) {
      ps.n[g] = (int)G.groups[g].planes.size();
      ps.ids[g] = G.groups[g].d_ids;
      ps.slots[g] = G.groups[g].d_slots;
    }
    return FLF_OK;
  }
  std::vector<std::vector<int>> ids(ng), slots(ng);
  for (int i = 0; i < nplanes; i++) {
    const int z = planes[i], g = G.plane_group[z];
    ids[g].push_back(z);
    slots[g].push_back(G.plane_slot[z]);
  }
  std::vector<int> host;   // per group: ids then slots
  std::vector<int> off(ng);
  for (int g = 0; g < ng; g++) {
    off[g] = (int)host.size();
    host.insert(host.end(), ids[g].begin(), ids[g].end());
    host.insert(host.end(), slots[g].begin(), slots[g].end());
  }
  if (ctx->planes_user_cap < (int)host.size()) {
    if (ctx->d_planes_user) cudaFree(ctx->d_planes_user);
    ctx->d_planes_user = nullptr;
    CUDA_TRY(ctx, cudaMalloc(&ctx->d_planes_user, sizeof(int) * 2 * ctx->nz));
    ctx->planes_user_cap = 2 * ctx->nz;
  }
  // the synchronous copy orders against earlier work on every stream
  CUDA_TRY(ctx, cudaStreamSynchronize(s));
  CUDA_TRY(ctx, cudaMemcpy(ctx->d_planes_user, host.data(), sizeof(int) * host.size(), cudaMemcpyHostToDevice));
  for (int g = 0; g < ng; g++) {
    ps.n[g] = (int)ids[g].size();
    ps.ids[g] = ctx->d_planes_user + off[g];
    ps.slots[g] = ctx->d_planes_user + off[g] + ps.n[g];
  }
  return FLF_OK;
}

int check_ready(flf_ctx *ctx, int T, int Y, int X, int dir, cudaStream_t s) {
  if (!ctx) return FLF_E_ARG;
  if (int rc0 = check_device_flag(ctx)) return rc0;
  if (T <= 0) return fail(ctx, FLF_E_ARG, "frame count must be positive (got %d)", T);
  int f_req = ctx->req_f;
  if (f_req > 0) {
    const int N = ctx->N, Ly = (Y + N - 1) / N, Lx = (X + N - 1) / N;
    int R = 0;
    for (int z = 0; z < ctx->nz; z++) R = std::max(R, plane_radius(ctx, z));
    if (f_req < std::max(Ly, Lx) + R || f_req < 2 * R + 1) f_req = 0;   // not valid for this shape
  }
  int rc = prepare(ctx, Y, X, f_req, ctx->req_fp64);
  if (rc != FLF_OK) return rc;
  if (!ctx->geo.built(dir)) rc = build_direction(ctx, dir, s);
  if (rc == FLF_OK) maybe_release_psfs(ctx);
  return rc;
}

// Planes per multiply-accumulate CTA: enough plane groups to give about
// opt_ctas_per_sm (16) CTAs per SM over the nquads frequency quads.
int zgroup_for(const flf_ctx *ctx, int nz, int nquads) {
  const int target = ctx->opt_ctas_per_sm * std::max(1, ctx->num_sms);
  const int nzg_needed = std::min(nz, std::max(1, (target + nquads - 1) / nquads));
  return std::min(kMacMaxZgroup, std::max(1, (nz + nzg_needed - 1) / nzg_needed));
}

// Floats of one channel-major image set (NN channel images of Ly x Lxp).
size_t chan_set_floats(const flf_ctx *ctx) {
  const Geometry &G = ctx->geo;
  return (size_t)ctx->L.NN * G.Ly * channel_pitch(G.Lx);
}

// Workspace bytes of one projection of nt frames over the plane set ps.
void ws_needs(const flf_ctx *ctx, const PlaneSet &ps, int nt, bool fwd, size_t &sS, size_t &sO, size_t &sCv) {
  const Geometry &G = ctx->geo;
  const int NN = ctx->L.NN;
  const size_t cset = sizeof(float) * chan_set_floats(ctx);
  sS = sO = sCv = 0;
  for (size_t g = 0; g < G.groups.size(); g++) {
    if (!ps.n[g]) continue;
    const size_t spec = sizeof(float2) * (size_t)NN * G.groups[g].f * G.groups[g].fh;
    const int n = ps.n[g];
    sCv = std::max(sCv, cset * nt * n);
    if (fwd) {
      const int zg = zgroup_for(ctx, n, G.groups[g].nquads);
      sS = std::max(sS, spec * nt * n);
      sO = std::max(sO, spec * nt * ((n + zg - 1) / zg));
    } else {
      sS = std::max(sS, spec * nt);
      sO = std::max(sO, spec * nt * n);
    }
  }
}

// Workspace slots: one per stream the transform groups alternate over.
int ws_slots(const flf_ctx *ctx) { return ctx->opt_streams > 1 ? 2 : 1; }
size_t slot_bytes(size_t b) { return (b + 255) / 256 * 256; }

// The second stream and its events (created on first use).
int ensure_streams(flf_ctx *ctx) {
  if (ctx->opt_streams < 2 || ctx->s2) return FLF_OK;
  CUDA_TRY(ctx, cudaStreamCreateWithFlags(&ctx->s2, cudaStreamNonBlocking));
  CUDA_TRY(ctx, cudaEventCreateWithFlags(&ctx->ev_fork, cudaEventDisableTiming));
  CUDA_TRY(ctx, cudaEventCreateWithFlags(&ctx->ev_join, cudaEventDisableTiming));
  CUDA_TRY(ctx, cudaEventCreateWithFlags(&ctx->ev_chain, cudaEventDisableTiming));
  return FLF_OK;
}

// Streams of a per-group loop: st[0] = s, st[1] = the second stream forked from s
// (or s again with one stream).  join_streams makes s wait for the second.
int fork_streams(flf_ctx *ctx, cudaStream_t s, cudaStream_t st[2]) {
  st[0] = st[1] = s;
  if (ctx->opt_streams < 2) return FLF_OK;
  if (int rc = ensure_streams(ctx)) return rc;
  CUDA_TRY(ctx, cudaEventRecord(ctx->ev_fork, s));
  CUDA_TRY(ctx, cudaStreamWaitEvent(ctx->s2, ctx->ev_fork, 0));
  st[1] = ctx->s2;
  return FLF_OK;
}
int join_streams(flf_ctx *ctx, cudaStream_t s) {
  if (ctx->opt_streams < 2 || !ctx->s2) return FLF_OK;
  CUDA_TRY(ctx, cudaEventRecord(ctx->ev_join, ctx->s2));
  CUDA_TRY(ctx, cudaStreamWaitEvent(s, ctx->ev_join, 0));
  return FLF_OK;
}

// Launch shape of the multiply-accumulate in direction dir: the image shape's
// tuned shape where one was set, else the options.
void mac_shape(const flf_ctx *ctx, int dir, int &stages, int &chunk_rows, int &split) {
  const int *tn = ctx->geo.tuned;
  stages = tn[0] ? tn[0] : ctx->opt_stages;
  chunk_rows = tn[1 + dir] ? tn[1 + dir] : ctx->opt_chunk_rows[dir];
  split = tn[3] ? tn[3] : ctx->opt_split;
  const int ntp = (ctx->L.nthr + 31) / 32 * 32;
  while (split > 1 && 2 * split * ntp > 256) split--;   // at most 256 threads per block
}

// Frames one multiply-accumulate pass takes: mac_max_frames(), or fewer where
// the ring, the staged spectra and the operand tables of that many frames do
// not fit shared memory with the current launch shape (Nnum 19 at 12 rows per
// stage: 2 frames).
int frames_per_pass(const flf_ctx *ctx) {
  for (int tf = mac_max_frames(); tf > 1; tf /= 2) {
    bool fits = true;
    for (int d = 0; d < 2; d++) {
      int st, cr, sp;
      mac_shape(ctx, d, st, cr, sp);
      if (mac_smem_bytes(ctx->L, tf, st, cr, sp, d == FLF_DIR_FORWARD) > kMacSmemMax) fits = false;
    }
    if (fits) return tf;
  }
  return 1;
}

MacParams mac_params(const flf_ctx *ctx, const Group &G, int dir, int nt) {
  MacParams mp{};
  mp.L = ctx->L; mp.f = G.f; mp.fh = G.fh; mp.fq = G.fq; mp.nkp = G.nkp; mp.nquads = G.nquads; mp.T = nt;
  mp.P = G.P[dir];
  mp.rowS = ctx->d_rowS; mp.rowF = ctx->d_rowF; mp.oslots = ctx->d_oslots; mp.slotcol = ctx->d_slotcol;
  mac_shape(ctx, dir, mp.stages, mp.chunk_rows, mp.split);
  mp.err = ctx->d_err;
  mp.wait_ns = (unsigned long long)ctx->opt_wait_us * 1000ull;
  mp.drop_chunk = ctx->opt_drop_chunk;
  return mp;
}

// One multiply-accumulate launch of group gi over all its planes for nt
// frames, on the workspaces (flf_autotune's timing unit).
cudaError_t mac_group_launch(flf_ctx *ctx, size_t gi, int dir, int nt, const PlaneSet &ps, int stages, int chunk,
                             int split, cudaStream_t s) {
  const Group &G = ctx->geo.groups[gi];
  const int nplanes = ps.n[gi];
  const int zg = zgroup_for(ctx, nplanes, G.nquads);
  MacParams mp = mac_params(ctx, G, dir, nt);
  mp.stages = stages; mp.chunk_rows = chunk; mp.split = split;
  mp.planes = ps.slots[gi]; mp.nz = nplanes; mp.zgroup = zg;
  mp.S = (const float2 *)ctx->wsS.p; mp.O = (float2 *)ctx->wsO.p;
  if (dir == FLF_DIR_FORWARD) {
    mp.nzS = nplanes; mp.nzo = (nplanes + zg - 1) / zg; mp.nzo_grid = mp.nzo;
  } else {
    mp.nzS = 1; mp.nzo = nplanes; mp.nzo_grid = (nplanes + zg - 1) / zg;
  }
  return launch_mac(mp, dir == FLF_DIR_FORWARD, s);
}

SplitParams split_params(const flf_ctx *ctx, const float *src, long long src_sz, long long src_st,
                         const int *planes, int nz, int nt, float *dst) {
  const Geometry &Gm = ctx->geo;
  SplitParams sp{};
  sp.src = src; sp.src_sz = src_sz; sp.src_st = src_st; sp.planes = planes;
  sp.nz = nz; sp.nsets = nz * nt;
  sp.N = ctx->N; sp.Y = Gm.Y; sp.X = Gm.X; sp.Ly = Gm.Ly; sp.Lx = Gm.Lx; sp.Lxp = channel_pitch(Gm.Lx);
  sp.dst = dst;
  return sp;
}

Rfft2Params rfft2_params(const flf_ctx *ctx, const Group &G, const float *chan, int nimg, void *dst) {
  const Geometry &Gm = ctx->geo;
  Rfft2Params rp{};
  rp.plan = G.plan; rp.N = ctx->N; rp.Y = Gm.Y; rp.X = Gm.X; rp.Ly = Gm.Ly; rp.Lx = Gm.Lx;
  rp.nimg = nimg; rp.mode = 0; rp.chan = chan; rp.Lxp = channel_pitch(Gm.Lx);
  rp.dst = dst; rp.twiddle = G.tw;
  return rp;
}

Irfft2Params irfft2_params(const flf_ctx *ctx, const Group &G, const float2 *src, int nimg, float *chan) {
  const Geometry &Gm = ctx->geo;
  Irfft2Params ip{};
  ip.plan = G.plan; ip.N = ctx->N; ip.Y = Gm.Y; ip.X = Gm.X; ip.Ly = Gm.Ly; ip.Lx = Gm.Lx;
  ip.nimg = nimg; ip.src = src; ip.sum_stride = 0; ip.nsum = 1;
  ip.chan = chan; ip.Lxp = channel_pitch(Gm.Lx); ip.twiddle = G.tw;
  return ip;
}

MergeParams merge_params(const flf_ctx *ctx, const float *src, const int *planes, int nzo, int nt, int epi,
                         Strided out, Strided aux, Strided norm) {
  const Geometry &Gm = ctx->geo;
  MergeParams mg{};
  mg.src = src; mg.nzo = nzo; mg.nsets = nzo * nt; mg.planes = planes;
  mg.N = ctx->N; mg.Y = Gm.Y; mg.X = Gm.X; mg.Ly = Gm.Ly; mg.Lx = Gm.Lx; mg.Lxp = channel_pitch(Gm.Lx);
  mg.epi = epi; mg.out = out; mg.aux = aux; mg.norm = norm;
  return mg;
}

// Bytes of nsets channel-major image sets.
double chan_bytes(const flf_ctx *ctx, int nsets) { return 4.0 * chan_set_floats(ctx) * nsets; }

// Forward projection of frames [t0, t0+nt) of vol into the channel-major
// image set `chan` ([nt][NN][Ly][Lxp]): each transform group is projected and
// summed in Fourier space over its planes; the groups are added in the
// channel-major domain.  The last group's pass zeroes the samples outside the
// image and, with `num`, stores num / (H x) (the standard RL error image).
int forward_chunk(flf_ctx *ctx, const float *vol, long long vol_sz, const PlaneSet &ps, int t0, int nt,
                  float *chan, const float *num, cudaStream_t s) {
  Geometry &Gm = ctx->geo;
  const Layout &L = ctx->L;
  const int NN = L.NN, Y = Gm.Y, X = Gm.X;
  size_t sS, sO, sCv;
  ws_needs(ctx, ps, nt, true, sS, sO, sCv);
  sS = slot_bytes(sS), sO = slot_bytes(sO), sCv = slot_bytes(sCv);
  const int nslot = ws_slots(ctx);
  int rc = ensure_ws(ctx, ctx->wsS, nslot * sS);
  if (rc == FLF_OK) rc = ensure_ws(ctx, ctx->wsO, nslot * sO);
  if (rc == FLF_OK) rc = ensure_ws(ctx, ctx->wsCvol, nslot * sCv);
  if (rc != FLF_OK) return rc;
  int last = -1;
  for (size_t gi = 0; gi < Gm.groups.size(); gi++)
    if (ps.n[gi]) last = (int)gi;
  bool first = true;
  // groups alternate over two streams with their own workspace slots; the
  // inverse transforms, which accumulate into chan, stay in group order
  cudaStream_t st[2];
  if ((rc = fork_streams(ctx, s, st))) return rc;
  const cudaStream_t s_caller = s;
  int k = 0;
  for (size_t gi = 0; gi < Gm.groups.size(); gi++) {
    const int nplanes = ps.n[gi];
    if (!nplanes) continue;
    const int slot = k & (nslot - 1);
    const cudaStream_t s = st[k & 1];
    float *cvol = (float *)((char *)ctx->wsCvol.p + slot * sCv);
    void *wS = (char *)ctx->wsS.p + slot * sS;
    float2 *wO = (float2 *)((char *)ctx->wsO.p + slot * sO);
    const Group &G = Gm.groups[gi];
    const int ffh = G.f * G.fh;
    const int zgroup = zgroup_for(ctx, nplanes, G.nquads);
    const int nzg = (nplanes + zgroup - 1) / zgroup;

    SplitParams sp = split_params(ctx, vol + (long long)t0 * Y * X, vol_sz, (long long)Y * X, ps.ids[gi],
                                  nplanes, nt, cvol);
    LAUNCH(ctx, "k_split", chan_bytes(ctx, nt * nplanes) + 4.0 * Y * X * nt * nplanes, s, launch_split(sp, s));

    Rfft2Params rp = rfft2_params(ctx, G, cvol, nt * nplanes * NN, wS);
    LAUNCH(ctx, "k_rfft2", chan_bytes(ctx, nt * nplanes) + 8.0 * ffh * NN * nt * nplanes, s, launch_rfft2(rp, 0, s));

    const double pbytes = (double)nplanes * G.nkp * L.nrow * L.RS * sizeof(float2);
    MacParams mp = mac_params(ctx, G, FLF_DIR_FORWARD, nt);
    mp.planes = ps.slots[gi]; mp.nz = nplanes; mp.zgroup = zgroup;
    mp.S = (const float2 *)wS; mp.nzS = nplanes; mp.O = wO; mp.nzo = nzg;
    mp.nzo_grid = nzg;
    LAUNCH(ctx, "k_mac_fwd", pbytes + 8.0 * ffh * NN * nt * ((double)nplanes + nzg), s, launch_mac(mp, true, s));

    if (k > 0 && nslot > 1) CUDA_TRY(ctx, cudaStreamWaitEvent(s, ctx->ev_chain, 0));
    Irfft2Params ip = irfft2_params(ctx, G, wO, nt * NN, chan);
    ip.sum_stride = (long long)nt * NN * ffh; ip.nsum = nzg;
    ip.add = !first; ip.final_pass = (int)gi == last; ip.num = ip.final_pass ? num : nullptr;
    const double cb = chan_bytes(ctx, nt) * (1 + ip.add + (ip.num ? 1 : 0));
    LAUNCH(ctx, "k_irfft2", 8.0 * ffh * NN * nt * nzg + cb, s, launch_irfft2(ip, s));
    if (nslot > 1) CUDA_TRY(ctx, cudaEventRecord(ctx->ev_chain, s));
    first = false;
    k++;
  }
  return join_streams(ctx, s_caller);
}

// Back projection of frames [t0, t0+nt) of the channel-major image set
// `chan` into the volume `out` (planes of ps) with the epilogue `epi`
// (aux / norm address volumes).
int backward_chunk(flf_ctx *ctx, const float *chan, const PlaneSet &ps, int nt, Strided out, Strided aux,
                   Strided norm, int epi, cudaStream_t s) {
  Geometry &Gm = ctx->geo;
  const Layout &L = ctx->L;
  const int NN = L.NN, Y = Gm.Y, X = Gm.X;
  size_t sS, sO, sCv;
  ws_needs(ctx, ps, nt, false, sS, sO, sCv);
  sS = slot_bytes(sS), sO = slot_bytes(sO), sCv = slot_bytes(sCv);
  const int nslot = ws_slots(ctx);
  int rc = ensure_ws(ctx, ctx->wsS, nslot * sS);
  if (rc == FLF_OK) rc = ensure_ws(ctx, ctx->wsO, nslot * sO);
  if (rc == FLF_OK) rc = ensure_ws(ctx, ctx->wsCvol, nslot * sCv);
  if (rc != FLF_OK) return rc;
  // groups alternate over two streams with their own workspace slots (their
  // planes, and so their outputs, are disjoint)
  cudaStream_t st[2];
  if ((rc = fork_streams(ctx, s, st))) return rc;
  const cudaStream_t s_caller = s;
  int k = 0;
  for (size_t gi = 0; gi < Gm.groups.size(); gi++) {
    const int nplanes = ps.n[gi];
    if (!nplanes) continue;
    const int slot = k & (nslot - 1);
    const cudaStream_t s = st[k & 1];
    k++;
    float *cvol = (float *)((char *)ctx->wsCvol.p + slot * sCv);
    void *wS = (char *)ctx->wsS.p + slot * sS;
    float2 *wO = (float2 *)((char *)ctx->wsO.p + slot * sO);
    const Group &G = Gm.groups[gi];
    const int ffh = G.f * G.fh;

    Rfft2Params rp = rfft2_params(ctx, G, chan, nt * NN, wS);
    LAUNCH(ctx, "k_rfft2", chan_bytes(ctx, nt) + 8.0 * ffh * NN * nt, s, launch_rfft2(rp, 0, s));

    const double pbytes = (double)nplanes * G.nkp * L.nrow * L.RS * sizeof(float2);
    const int zgb = zgroup_for(ctx, nplanes, G.nquads);
    MacParams mp = mac_params(ctx, G, FLF_DIR_BACKWARD, nt);
    mp.planes = ps.slots[gi]; mp.nz = nplanes; mp.zgroup = zgb;
    mp.S = (const float2 *)wS; mp.nzS = 1; mp.O = wO; mp.nzo = nplanes;
    mp.nzo_grid = (nplanes + zgb - 1) / zgb;
    LAUNCH(ctx, "k_mac_bwd", pbytes + 8.0 * ffh * NN * nt * (1.0 + nplanes), s, launch_mac(mp, false, s));

    Irfft2Params ip = irfft2_params(ctx, G, wO, nt * nplanes * NN, cvol);
    ip.final_pass = 1;
    LAUNCH(ctx, "k_irfft2", 8.0 * ffh * NN * nt * nplanes + chan_bytes(ctx, nt * nplanes), s, launch_irfft2(ip, s));

    MergeParams mg = merge_params(ctx, cvol, ps.ids[gi], nplanes, nt, epi, out, aux, norm);
    const int npix = epi == EPI_STORE ? 1 : (epi == EPI_RL_STANDARD && norm.p ? 4 : 3);
    LAUNCH(ctx, "k_merge", chan_bytes(ctx, nt * nplanes) + 4.0 * npix * Y * X * nt * nplanes, s,
           launch_merge(mg, s));
  }
  return join_streams(ctx, s_caller);
}

// ----------------------------------------------------------------------------
// Fixed scratch for flf_backward_noalloc: a file-scope device array, so that
// entry point never asks the driver for memory.  With CUDA's lazy module
// loading the array is committed when this file's module loads, which
// flf_ctx_create forces by looking up the array's address (below): from then
// on the GPU holds FLF_NOALLOC_SCRATCH_BYTES of it until the process exits.
// ----------------------------------------------------------------------------
static __device__ __align__(256) unsigned char g_noalloc_scratch[FLF_NOALLOC_SCRATCH_BYTES];

// Device address of the scratch array in the current CUDA context.  The
// host-side symbol is only a stand-in and must never reach a kernel.  Called
// by flf_ctx_create with the context's device current; the address is kept in
// the context, which is valid only in the primary context of that device.
int noalloc_scratch_lookup(flf_ctx *ctx) {
  void *ptr = nullptr;
  cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
  if (e != cudaSuccess || !ptr) {
    cudaGetLastError();
    return fail(ctx, FLF_E_CUDA, "cudaGetSymbolAddress of the fixed scratch failed: %s", cudaGetErrorString(e));
  }
  ctx->noalloc_scratch = ptr;
  return FLF_OK;
}

int backward_run(flf_ctx *ctx, const float *img_dev, float *vol_dev, int T, int Y, int X, const PlaneSet &ps,
                 cudaStream_t s);

}  // namespace

// ============================================================================
// C ABI
// ============================================================================
extern "C" {

int flf_ctx_create(flf_ctx **out, int device, int nnum, int num_planes) {
  if (!out) return fail(nullptr, FLF_E_ARG, "out pointer is NULL");
  *out = nullptr;
  if (nnum < 3 || (nnum % 2) == 0 || nnum > 31)
    return fail(nullptr, FLF_E_ARG, "Nnum must be odd and in [3, 31] (got %d)", nnum);
  if (num_planes <= 0 || num_planes > 4096)
    return fail(nullptr, FLF_E_ARG, "num_planes out of range (got %d)", num_planes);
  int ndev = 0;
  cudaError_t e = cudaGetDeviceCount(&ndev);
  if (e != cudaSuccess || ndev == 0)
    return fail(nullptr, FLF_E_CUDA, "no CUDA device available: %s", cudaGetErrorString(e));
  if (device < 0 || device >= ndev) return fail(nullptr, FLF_E_ARG, "device %d out of range", device);
  e = cudaSetDevice(device);
  if (e != cudaSuccess) return fail(nullptr, FLF_E_CUDA, "cudaSetDevice: %s", cudaGetErrorString(e));
  flf_ctx *ctx = new flf_ctx();
  ctx->device = device;
  ctx->N = nnum;
  ctx->nz = num_planes;
  ctx->L = make_layout(nnum);
  for (int d = 0; d < 2; d++) {
    ctx->dH[d].assign(num_planes, nullptr);
    ctx->h[d].assign(num_planes, 0);
  }
  cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount, device);
  int rc = FLF_OK;
  if (cudaHostAlloc((void **)&ctx->h_err, sizeof(int), cudaHostAllocMapped) != cudaSuccess ||
      cudaHostGetDevicePointer((void **)&ctx->d_err, ctx->h_err, 0) != cudaSuccess) {
    cudaGetLastError();
    rc = fail(ctx, FLF_E_CUDA, "mapped host allocation for the error flag failed");
  } else {
    *ctx->h_err = 0;
  }
  if (rc == FLF_OK) rc = build_tables(ctx);
  if (rc == FLF_OK) rc = noalloc_scratch_lookup(ctx);
  if (rc != FLF_OK) {
    g_create_error = ctx->err;
    flf_ctx_destroy(ctx);
    return rc;
  }
  *out = ctx;
  return FLF_OK;
}

int flf_ctx_destroy(flf_ctx *ctx) {
  if (!ctx) return FLF_OK;
  cudaSetDevice(ctx->device);
  for (int d = 0; d < 2; d++)
    for (float *p : ctx->dH[d])
      if (p) cudaFree(p);
  resolve_pending(ctx);
  for (cudaEvent_t e : ctx->evpool) cudaEventDestroy(e);
  free_all_geometries(ctx);
  void *ptrs[] = {ctx->d_rowS, ctx->d_rowF, ctx->d_oslots, ctx->d_slotcol, ctx->d_colslot, ctx->d_rep_ch, ctx->d_rep_row,
                  ctx->d_rep_kind, ctx->d_planes_all, ctx->d_planes_user, ctx->d_zero,
                  ctx->wsS.p, ctx->wsO.p, ctx->wsCvol.p, ctx->wsCimg.p, ctx->wsCy.p};
  for (void *p : ptrs)
    if (p) cudaFree(p);
  if (ctx->h_err) cudaFreeHost(ctx->h_err);
  cudaEvent_t evs[] = {ctx->ev_fork, ctx->ev_join, ctx->ev_chain};
  for (cudaEvent_t e : evs)
    if (e) cudaEventDestroy(e);
  if (ctx->s2) cudaStreamDestroy(ctx->s2);
  delete ctx;
  return FLF_OK;
}

int flf_last_error(const flf_ctx *ctx, char *buf, size_t len) {
  if (!buf || len == 0) return FLF_E_ARG;
  const std::string &s = ctx ? ctx->err : g_create_error;
  const size_t n = std::min(len - 1, s.size());
  memcpy(buf, s.data(), n);
  buf[n] = 0;
  return FLF_OK;
}

int flf_psf_upload(flf_ctx *ctx, int plane, int direction, const float *H_host, int n_h, int h) {
  if (!ctx) return FLF_E_ARG;
  if (plane < 0 || plane >= ctx->nz) return fail(ctx, FLF_E_ARG, "plane %d out of range [0, %d)", plane, ctx->nz);
  if (direction != FLF_DIR_FORWARD && direction != FLF_DIR_BACKWARD)
    return fail(ctx, FLF_E_ARG, "direction must be 0 (H) or 1 (Ht), got %d", direction);
  if (!H_host) return fail(ctx, FLF_E_ARG, "H pointer is NULL");
  if (n_h != ctx->L.nh) return fail(ctx, FLF_E_ARG, "n_h %d does not match Nnum %d (expected %d)", n_h, ctx->N, ctx->L.nh);
  if (h <= 0 || (h % 2) == 0) return fail(ctx, FLF_E_ARG, "PSF size h must be odd and positive (got %d)", h);
  cudaSetDevice(ctx->device);
  float *&dst = ctx->dH[direction][plane];
  if (dst && ctx->h[direction][plane] != h) { cudaFree(dst); dst = nullptr; }
  const size_t bytes = sizeof(float) * (size_t)n_h * n_h * h * h;
  if (!dst) {
    cudaError_t e = cudaMalloc(&dst, bytes);
    if (e != cudaSuccess) { cudaGetLastError(); dst = nullptr; return fail(ctx, FLF_E_NOMEM, "cudaMalloc for PSF failed: %s", cudaGetErrorString(e)); }
  }
  CUDA_TRY(ctx, cudaMemcpy(dst, H_host, bytes, cudaMemcpyHostToDevice));
  ctx->h[direction][plane] = h;
  // transfer matrices depend on the PSF and on the kernel radius
  free_all_geometries(ctx);
  return FLF_OK;
}

int flf_prepare(flf_ctx *ctx, int Y, int X, int fft_size, int fp64) {
  if (!ctx) return FLF_E_ARG;
  cudaSetDevice(ctx->device);
  for (int d = 0; d < 2; d++)
    for (int z = 0; z < ctx->nz; z++)
      if (!ctx->dH[d][z] && !(ctx->psf_released && ctx->geo.valid && ctx->geo.Y == Y && ctx->geo.X == X))
        return fail(ctx, FLF_E_STATE, "PSF for plane %d direction %d was not uploaded%s", z, d,
                    ctx->psf_released ? " (released after the last precompute)" : "");
  int rc = prepare(ctx, Y, X, fft_size, fp64);
  if (rc != FLF_OK) return rc;
  ctx->req_f = fft_size;
  ctx->req_fp64 = fp64;
  for (int d = 0; d < 2 && rc == FLF_OK; d++)
    if (!ctx->geo.built(d)) rc = build_direction(ctx, d, 0);
  if (rc == FLF_OK) maybe_release_psfs(ctx);
  return rc;
}

int flf_forward(flf_ctx *ctx, const float *vol_dev, float *img_dev, int T, int Y, int X,
                const int *planes, int nplanes, void *stream) {
  if (!ctx) return FLF_E_ARG;
  if (!vol_dev || !img_dev) return fail(ctx, FLF_E_ARG, "NULL array pointer");
  cudaSetDevice(ctx->device);
  cudaStream_t s = (cudaStream_t)stream;
  if (int rc0 = check_psfs(ctx, 1 << FLF_DIR_FORWARD)) return rc0;
  int rc = check_planes_arg(ctx, planes, nplanes);
  if (rc == FLF_OK) rc = check_ready(ctx, T, Y, X, FLF_DIR_FORWARD, s);
  PlaneSet ps;
  if (rc == FLF_OK) rc = make_plane_set(ctx, planes, nplanes, s, ps);
  if (rc != FLF_OK) return rc;
  const int TF = frames_per_pass(ctx);
  const long long vol_sz = (long long)T * Y * X;
  rc = ensure_ws(ctx, ctx->wsCimg, sizeof(float) * chan_set_floats(ctx) * std::min(T, TF));
  float *cimg = (float *)ctx->wsCimg.p;
  for (int t0 = 0; t0 < T && rc == FLF_OK; t0 += TF) {
    const int nt = std::min(TF, T - t0);
    rc = forward_chunk(ctx, vol_dev, vol_sz, ps, t0, nt, cimg, nullptr, s);
    if (rc != FLF_OK) break;
    const Strided out{img_dev + (long long)t0 * Y * X, 0, (long long)Y * X};
    MergeParams mg = merge_params(ctx, cimg, nullptr, 1, nt, EPI_STORE, out, Strided{nullptr, 0, 0},
                                  Strided{nullptr, 0, 0});
    LAUNCH(ctx, "k_merge", chan_bytes(ctx, nt) + 4.0 * Y * X * nt, s, launch_merge(mg, s));
  }
  return rc;
}

int flf_backward(flf_ctx *ctx, const float *img_dev, float *vol_dev, int T, int Y, int X,
                 const int *planes, int nplanes, void *stream) {
  if (!ctx) return FLF_E_ARG;
  if (!vol_dev || !img_dev) return fail(ctx, FLF_E_ARG, "NULL array pointer");
  cudaSetDevice(ctx->device);
  cudaStream_t s = (cudaStream_t)stream;
  if (int rc0 = check_psfs(ctx, 1 << FLF_DIR_BACKWARD)) return rc0;
  int rc = check_planes_arg(ctx, planes, nplanes);
  if (rc == FLF_OK) rc = check_ready(ctx, T, Y, X, FLF_DIR_BACKWARD, s);
  PlaneSet ps;
  if (rc == FLF_OK) rc = make_plane_set(ctx, planes, nplanes, s, ps);
  if (rc != FLF_OK) return rc;
  rc = ensure_ws(ctx, ctx->wsCimg, sizeof(float) * chan_set_floats(ctx) * std::min(T, frames_per_pass(ctx)));
  if (rc != FLF_OK) return rc;
  return backward_run(ctx, img_dev, vol_dev, T, Y, X, ps, s);
}

int flf_backward_noalloc(flf_ctx *ctx, const float *img_dev, float *vol_dev, int T, int Y, int X,
                         void *stream) {
  if (!ctx) return FLF_E_ARG;
  if (!vol_dev || !img_dev) return fail(ctx, FLF_E_ARG, "NULL array pointer");
  if (T <= 0) return fail(ctx, FLF_E_ARG, "frame count must be positive (got %d)", T);
  cudaSetDevice(ctx->device);
  if (int rc0 = check_device_flag(ctx)) return rc0;
  Geometry &Gm = ctx->geo;
  if (!Gm.valid || Gm.Y != Y || Gm.X != X || !Gm.built(FLF_DIR_BACKWARD))
    return fail(ctx, FLF_E_STATE,
                "flf_backward_noalloc needs transfer matrices for %d x %d built beforehand: call flf_prepare "
                "with this image shape first", Y, X);
  const Layout &L = ctx->L;
  const int NN = L.NN;
  // scratch: S (one frame's channel spectra) | C (its channel-major image) |
  // blocks of zb planes of O (output spectra) and their channel-major images
  auto up = [](size_t b) { return (b + 255) & ~(size_t)255; };
  const size_t cimg = up(sizeof(float) * chan_set_floats(ctx));
  size_t need = 0;
  for (const Group &G : Gm.groups) {
    const size_t spec = up(sizeof(float2) * (size_t)NN * G.f * G.fh);
    need = std::max(need, spec + cimg + spec + cimg);
  }
  if (need > FLF_NOALLOC_SCRATCH_BYTES)
    return fail(ctx, FLF_E_ARG,
                "flf_backward_noalloc needs %zu bytes of scratch for this geometry (Nnum %d, transform %d), "
                "more than its fixed %u bytes; use flf_backward", need, ctx->N, Gm.max_f(),
                (unsigned)FLF_NOALLOC_SCRATCH_BYTES);
  void *scratch = ctx->noalloc_scratch;
  if (!scratch) return fail(ctx, FLF_E_STATE, "the fixed scratch was not set up by flf_ctx_create");
  cudaStream_t s = (cudaStream_t)stream;
  const long long YX = (long long)Y * X;
  char *base = (char *)scratch;
  float *C = (float *)base;
  for (int t = 0; t < T; t++) {
    cudaError_t e = launch_split(split_params(ctx, img_dev + t * YX, 0, YX, nullptr, 1, 1, C), s);
    for (size_t gi = 0; gi < Gm.groups.size() && e == cudaSuccess; gi++) {
      const Group &G = Gm.groups[gi];
      const size_t spec = up(sizeof(float2) * (size_t)NN * G.f * G.fh);   // one frame or one plane
      float2 *S = (float2 *)(base + cimg);
      char *blocks = base + cimg + spec;
      const size_t per_plane = spec + cimg;
      const int ng = (int)G.planes.size();
      const int zb = std::max(1, std::min(ng, (int)((FLF_NOALLOC_SCRATCH_BYTES - cimg - spec) / per_plane)));
      float2 *O = (float2 *)blocks;
      float *Co = (float *)(blocks + spec * zb);
      e = launch_rfft2(rfft2_params(ctx, G, C, NN, S), 0, s);
      for (int z0 = 0; z0 < ng && e == cudaSuccess; z0 += zb) {
        const int nzl = std::min(zb, ng - z0);
        const int zg = zgroup_for(ctx, nzl, G.nquads);
        MacParams mp = mac_params(ctx, G, FLF_DIR_BACKWARD, 1);
        mp.planes = G.d_slots + z0; mp.nz = nzl; mp.zgroup = zg;
        mp.S = S; mp.nzS = 1; mp.O = O; mp.nzo = nzl; mp.nzo_grid = (nzl + zg - 1) / zg;
        e = launch_mac(mp, false, s);
        if (e != cudaSuccess) break;
        Irfft2Params ip = irfft2_params(ctx, G, O, nzl * NN, Co);
        ip.final_pass = 1;
        e = launch_irfft2(ip, s);
        if (e != cudaSuccess) break;
        const Strided out{vol_dev + t * YX, (long long)T * YX, YX};
        e = launch_merge(merge_params(ctx, Co, G.d_ids + z0, nzl, 1, EPI_STORE, out, Strided{nullptr, 0, 0},
                                      Strided{nullptr, 0, 0}), s);
      }
    }
    if (e != cudaSuccess) return fail(ctx, FLF_E_CUDA, "flf_backward_noalloc launch failed: %s", cudaGetErrorString(e));
  }
  return FLF_OK;
}

}  // extern "C"

namespace {

// Argument checks, transfer matrices and every workspace of an RL run of T
// frames of Y x X images, so that the loop itself allocates nothing.
int rl_setup(flf_ctx *ctx, float *x_dev, const float *ref_dev, int variant, int iters, int T, int Y, int X,
             cudaStream_t s, PlaneSet &ps) {
  if (!x_dev || !ref_dev) return fail(ctx, FLF_E_ARG, "NULL array pointer");
  if (variant != FLF_RL_PREVEDEL && variant != FLF_RL_STANDARD)
    return fail(ctx, FLF_E_ARG, "unknown RL variant %d", variant);
  if (iters < 0) return fail(ctx, FLF_E_ARG, "iters must be >= 0");
  if (int rc0 = check_psfs(ctx, 3)) return rc0;
  int rc = check_ready(ctx, T, Y, X, FLF_DIR_FORWARD, s);
  if (rc == FLF_OK) rc = check_ready(ctx, T, Y, X, FLF_DIR_BACKWARD, s);
  if (rc != FLF_OK) return rc;
  const int nt = std::min(T, frames_per_pass(ctx));
  const size_t cset = sizeof(float) * chan_set_floats(ctx) * nt;
  rc = ensure_ws(ctx, ctx->wsCimg, cset);
  if (rc == FLF_OK && variant == FLF_RL_STANDARD) rc = ensure_ws(ctx, ctx->wsCy, cset);
  if (rc == FLF_OK) rc = make_plane_set(ctx, nullptr, ctx->nz, s, ps);
  if (rc != FLF_OK) return rc;
  size_t a, b, c, a2, b2, c2;
  ws_needs(ctx, ps, nt, true, a, b, c);
  ws_needs(ctx, ps, nt, false, a2, b2, c2);
  const int nslot = ws_slots(ctx);
  rc = ensure_ws(ctx, ctx->wsS, nslot * slot_bytes(std::max(a, a2)));
  if (rc == FLF_OK) rc = ensure_ws(ctx, ctx->wsO, nslot * slot_bytes(std::max(b, b2)));
  if (rc == FLF_OK) rc = ensure_ws(ctx, ctx->wsCvol, nslot * slot_bytes(std::max(c, c2)));
  if (rc == FLF_OK) rc = ensure_streams(ctx);
  return rc;
}

// Back projection of T frames into vol_dev over the plane set ps (workspaces
// sized beforehand).
int backward_run(flf_ctx *ctx, const float *img_dev, float *vol_dev, int T, int Y, int X, const PlaneSet &ps,
                 cudaStream_t s) {
  const int TF = frames_per_pass(ctx);
  const long long YX = (long long)Y * X;
  float *cimg = (float *)ctx->wsCimg.p;
  int rc = FLF_OK;
  for (int t0 = 0; t0 < T && rc == FLF_OK; t0 += TF) {
    const int nt = std::min(TF, T - t0);
    SplitParams sp = split_params(ctx, img_dev + t0 * YX, 0, YX, nullptr, 1, nt, cimg);
    LAUNCH(ctx, "k_split", chan_bytes(ctx, nt) + 4.0 * YX * nt, s, launch_split(sp, s));
    const Strided out{vol_dev + t0 * YX, (long long)T * YX, YX};
    rc = backward_chunk(ctx, cimg, ps, nt, out, Strided{nullptr, 0, 0}, Strided{nullptr, 0, 0}, EPI_STORE, s);
  }
  return rc;
}

// The RL loop on stream s (after rl_setup).
int rl_run(flf_ctx *ctx, float *x_dev, const float *ref_dev, const float *norm_dev, int variant, int iters, int T,
           int Y, int X, const PlaneSet &ps, cudaStream_t s) {
  const int TF = frames_per_pass(ctx);
  const long long YX = (long long)Y * X;
  float *cimg = (float *)ctx->wsCimg.p;
  float *cy = (float *)ctx->wsCy.p;
  int rc = FLF_OK;
  for (int t0 = 0; t0 < T && rc == FLF_OK; t0 += TF) {
    const int nt = std::min(TF, T - t0);
    const Strided xs{x_dev + t0 * YX, (long long)T * YX, YX};
    if (variant == FLF_RL_STANDARD && iters > 0) {
      SplitParams sp = split_params(ctx, ref_dev + t0 * YX, 0, YX, nullptr, 1, nt, cy);
      LAUNCH(ctx, "k_split", chan_bytes(ctx, nt) + 4.0 * YX * nt, s, launch_split(sp, s));
    }
    for (int it = 0; it < iters && rc == FLF_OK; it++) {
      // H x (Prevedel) or y / H x (standard) as channel-major images, then the
      // back projection with the update fused into its pixel epilogue
      rc = forward_chunk(ctx, x_dev, (long long)T * YX, ps, t0, nt, cimg,
                         variant == FLF_RL_STANDARD ? cy : nullptr, s);
      if (rc != FLF_OK) break;
      if (variant == FLF_RL_PREVEDEL) {
        const Strided htf{const_cast<float *>(ref_dev) + t0 * YX, (long long)T * YX, YX};
        rc = backward_chunk(ctx, cimg, ps, nt, xs, htf, Strided{nullptr, 0, 0}, EPI_RL_PREVEDEL, s);
      } else {
        const Strided nrm{const_cast<float *>(norm_dev), YX, 0};
        rc = backward_chunk(ctx, cimg, ps, nt, xs, Strided{nullptr, 0, 0}, nrm, EPI_RL_STANDARD, s);
      }
    }
  }
  return rc;
}

}  // namespace

struct flf_graph {
  flf_ctx *ctx = nullptr;
  int device = 0;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  int launches = 0;
  unsigned long long epoch = 0;   // ctx->mem_epoch at capture: the buffers baked into the graph
};

extern "C" {

int flf_rl_iterate(flf_ctx *ctx, float *x_dev, const float *ref_dev, const float *norm_dev,
                   int variant, int iters, int T, int Y, int X, void *stream) {
  if (!ctx) return FLF_E_ARG;
  cudaSetDevice(ctx->device);
  cudaStream_t s = (cudaStream_t)stream;
  PlaneSet ps;
  int rc = rl_setup(ctx, x_dev, ref_dev, variant, iters, T, Y, X, s, ps);
  if (rc != FLF_OK) return rc;
  return rl_run(ctx, x_dev, ref_dev, norm_dev, variant, iters, T, Y, X, ps, s);
}

}  // extern "C"

namespace {

// Capture `body(stream)` (launches only: every buffer exists already) into a
// new graph of this context.
template <typename Body>
int capture_graph(flf_ctx *ctx, flf_graph **out, const char *what, Body body) {
  CUDA_TRY(ctx, cudaDeviceSynchronize());
  cudaStream_t cs = nullptr;
  CUDA_TRY(ctx, cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
  const bool prof = ctx->profiling;
  ctx->profiling = false;           // no per-launch events inside the graph
  long long before = 0;
  for (auto &kv : ctx->kstats) before += kv.second.launches;
  cudaError_t e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeRelaxed);
  int rc = FLF_OK;
  if (e == cudaSuccess) rc = body(cs);
  cudaGraph_t g = nullptr;
  const cudaError_t e2 = e == cudaSuccess ? cudaStreamEndCapture(cs, &g) : e;
  ctx->profiling = prof;
  long long after = 0;
  for (auto &kv : ctx->kstats) after += kv.second.launches;
  cudaStreamDestroy(cs);
  if (e != cudaSuccess || e2 != cudaSuccess || rc != FLF_OK) {
    if (g) cudaGraphDestroy(g);
    cudaGetLastError();
    if (rc != FLF_OK) return rc;
    return fail(ctx, FLF_E_CUDA, "capture of the %s failed: %s", what, cudaGetErrorString(e != cudaSuccess ? e : e2));
  }
  cudaGraphExec_t ex = nullptr;
  e = cudaGraphInstantiate(&ex, g, 0);
  if (e != cudaSuccess) {
    cudaGraphDestroy(g);
    return fail(ctx, FLF_E_CUDA, "instantiating the %s graph failed: %s", what, cudaGetErrorString(e));
  }
  flf_graph *gr = new flf_graph;
  gr->ctx = ctx; gr->graph = g; gr->exec = ex; gr->launches = (int)(after - before);
  gr->epoch = ctx->mem_epoch;
  gr->device = ctx->device;
  *out = gr;
  return FLF_OK;
}

}  // namespace

extern "C" {

int flf_deconv_graph_create(flf_ctx *ctx, flf_graph **out, const float *img_dev, float *htf_dev, float *x_dev,
                            int iters, int T, int Y, int X) {
  if (!ctx || !out) return FLF_E_ARG;
  *out = nullptr;
  if (!img_dev) return fail(ctx, FLF_E_ARG, "NULL array pointer");
  cudaSetDevice(ctx->device);
  PlaneSet ps;
  int rc = rl_setup(ctx, x_dev, htf_dev, FLF_RL_PREVEDEL, iters, T, Y, X, nullptr, ps);
  if (rc != FLF_OK) return rc;
  const size_t vbytes = sizeof(float) * (size_t)ctx->nz * T * Y * X;
  return capture_graph(ctx, out, "deconvolution", [&](cudaStream_t cs) {
    int r = backward_run(ctx, img_dev, htf_dev, T, Y, X, ps, cs);
    if (r != FLF_OK) return r;
    if (cudaMemcpyAsync(x_dev, htf_dev, vbytes, cudaMemcpyDeviceToDevice, cs) != cudaSuccess)
      return fail(ctx, FLF_E_CUDA, "copy of Htf into the start volume failed");
    return rl_run(ctx, x_dev, htf_dev, nullptr, FLF_RL_PREVEDEL, iters, T, Y, X, ps, cs);
  });
}

int flf_graph_combine(flf_graph **out, flf_graph *const *parts, int n) {
  if (!out || !parts || n <= 0) return FLF_E_ARG;
  *out = nullptr;
  flf_ctx *ctx = parts[0] ? parts[0]->ctx : nullptr;
  if (!ctx) return FLF_E_ARG;
  for (int i = 0; i < n; i++) {
    if (!parts[i] || parts[i]->ctx != ctx) return fail(ctx, FLF_E_ARG, "graphs to combine must share one context");
    if (parts[i]->epoch != ctx->mem_epoch)
      return fail(ctx, FLF_E_STATE, "graph %d refers to buffers freed since its capture: create it again", i);
  }
  cudaSetDevice(ctx->device);
  cudaGraph_t g = nullptr;
  CUDA_TRY(ctx, cudaGraphCreate(&g, 0));
  cudaGraphNode_t prev = nullptr;
  int launches = 0;
  cudaError_t e = cudaSuccess;
  for (int i = 0; i < n && e == cudaSuccess; i++) {
    cudaGraphNode_t node = nullptr;
    e = cudaGraphAddChildGraphNode(&node, g, prev ? &prev : nullptr, prev ? 1 : 0, parts[i]->graph);
    prev = node;
    launches += parts[i]->launches;
  }
  cudaGraphExec_t ex = nullptr;
  if (e == cudaSuccess) e = cudaGraphInstantiate(&ex, g, 0);
  if (e != cudaSuccess) {
    cudaGraphDestroy(g);
    return fail(ctx, FLF_E_CUDA, "combining graphs failed: %s", cudaGetErrorString(e));
  }
  flf_graph *gr = new flf_graph;
  gr->ctx = ctx; gr->graph = g; gr->exec = ex; gr->launches = launches;
  gr->epoch = ctx->mem_epoch;
  gr->device = ctx->device;
  *out = gr;
  return FLF_OK;
}

int flf_rl_graph_create(flf_ctx *ctx, flf_graph **out, float *x_dev, const float *ref_dev, const float *norm_dev,
                        int variant, int iters, int T, int Y, int X) {
  if (!ctx || !out) return FLF_E_ARG;
  *out = nullptr;
  cudaSetDevice(ctx->device);
  PlaneSet ps;
  int rc = rl_setup(ctx, x_dev, ref_dev, variant, iters, T, Y, X, nullptr, ps);
  if (rc != FLF_OK) return rc;
  return capture_graph(ctx, out, "RL loop", [&](cudaStream_t cs) {
    return rl_run(ctx, x_dev, ref_dev, norm_dev, variant, iters, T, Y, X, ps, cs);
  });
}

int flf_graph_launch(flf_graph *g, void *stream) {
  if (!g || !g->exec) return FLF_E_ARG;
  cudaSetDevice(g->ctx->device);
  if (g->epoch != g->ctx->mem_epoch)
    return fail(g->ctx, FLF_E_STATE, "the RL graph refers to workspaces or transfer matrices that were freed "
                                     "since its capture (clear_cache, new PSFs or larger images): create it again");
  if (int rc = check_device_flag(g->ctx)) return rc;
  CUDA_TRY(g->ctx, cudaGraphLaunch(g->exec, (cudaStream_t)stream));
  return FLF_OK;
}

int flf_graph_kernels(const flf_graph *g) { return g ? g->launches : -1; }

int flf_graph_destroy(flf_graph *g) {
  if (!g) return FLF_OK;
  cudaSetDevice(g->device);   // the context may already be gone
  if (g->exec) cudaGraphExecDestroy(g->exec);
  if (g->graph) cudaGraphDestroy(g->graph);
  delete g;
  return FLF_OK;
}

int flf_memory_epoch(const flf_ctx *ctx, unsigned long long *epoch) {
  if (!ctx || !epoch) return FLF_E_ARG;
  *epoch = ctx->mem_epoch;
  return FLF_OK;
}

int flf_memory_usage(const flf_ctx *ctx, size_t *bytes) {
  if (!ctx || !bytes) return FLF_E_ARG;
  size_t b = 0;
  for (int d = 0; d < 2; d++)
    for (int z = 0; z < ctx->nz; z++)
      if (ctx->dH[d][z]) b += sizeof(float) * (size_t)ctx->L.nh * ctx->L.nh * ctx->h[d][z] * ctx->h[d][z];
  std::vector<const Geometry *> geos{&ctx->geo};
  for (const Geometry &g : ctx->parked) geos.push_back(&g);
  for (const Geometry *Gm : geos)
    for (const Group &G : Gm->groups) {
      const size_t pe = (size_t)G.nkp * ctx->L.nrow * ctx->L.RS * G.planes.size() * sizeof(float2);
      for (int d = 0; d < 2; d++)
        if (G.P[d]) b += pe;
    }
  b += ctx->wsS.bytes + ctx->wsO.bytes + ctx->wsCvol.bytes + ctx->wsCimg.bytes + ctx->wsCy.bytes;
  *bytes = b;
  return FLF_OK;
}

int flf_clear_cache(flf_ctx *ctx) {
  if (!ctx) return FLF_E_ARG;
  cudaSetDevice(ctx->device);
  cudaDeviceSynchronize();
  free_all_geometries(ctx);
  Workspace *ws[] = {&ctx->wsS, &ctx->wsO, &ctx->wsCvol, &ctx->wsCimg, &ctx->wsCy};
  for (Workspace *w : ws) {
    if (w->p) cudaFree(w->p);
    *w = Workspace();
  }
  return FLF_OK;
}

int flf_geometry(const flf_ctx *ctx, int *out4) {
  if (!ctx || !out4) return FLF_E_ARG;
  const Geometry &G = ctx->geo;
  int R = 0;
  for (const Group &g : G.groups) R = std::max(R, g.R);
  out4[0] = G.valid ? G.max_f() : 0;
  out4[1] = G.valid ? R : 0;
  out4[2] = G.valid ? G.fp64 : 0;
  out4[3] = G.valid ? (int)G.groups.size() : 0;
  return FLF_OK;
}

int flf_profile(flf_ctx *ctx, int enable) {
  if (!ctx) return FLF_E_ARG;
  cudaSetDevice(ctx->device);
  resolve_pending(ctx);
  ctx->kstats.clear();
  ctx->profiling = enable != 0;
  return FLF_OK;
}

int flf_profile_read(flf_ctx *ctx, char *buf, size_t len) {
  if (!ctx || !buf || len == 0) return FLF_E_ARG;
  cudaSetDevice(ctx->device);
  resolve_pending(ctx);
  std::string out;
  char line[256];
  for (auto &kv : ctx->kstats) {
    snprintf(line, sizeof(line), "%s %lld %.6f %.0f\n", kv.first.c_str(), kv.second.launches, kv.second.ms,
             kv.second.bytes);
    out += line;
  }
  const size_t n = std::min(len - 1, out.size());
  memcpy(buf, out.data(), n);
  buf[n] = 0;
  return out.size() < len ? FLF_OK : FLF_E_ARG;
}

int flf_synchronize(flf_ctx *ctx, void *stream) {
  if (!ctx) return FLF_E_ARG;
  cudaSetDevice(ctx->device);
  CUDA_TRY(ctx, cudaStreamSynchronize((cudaStream_t)stream));
  return check_device_flag(ctx);
}

int flf_set_option(flf_ctx *ctx, const char *name, long long value) {
  if (!ctx || !name) return FLF_E_ARG;
  if (!strcmp(name, "plane_transform_sizes")) {
    if (value != 0 && value != 1) return fail(ctx, FLF_E_ARG, "plane_transform_sizes must be 0 or 1");
    if (ctx->opt_plane_sizes != (int)value) {
      ctx->opt_plane_sizes = (int)value;
      cudaDeviceSynchronize();
      free_all_geometries(ctx);   // rebuilt on the next call
    }
    return FLF_OK;
  }
  if (!strcmp(name, "mac_wait_limit_us")) {
    if (value < 100 || value > 10000000) return fail(ctx, FLF_E_ARG, "mac_wait_limit_us must be in [100, 1e7]");
    ctx->opt_wait_us = value;
    return FLF_OK;
  }
  if (!strcmp(name, "test_drop_chunk")) {
    if (value < -1 || value > 1000000) return fail(ctx, FLF_E_ARG, "test_drop_chunk must be -1 or a chunk index");
    ctx->opt_drop_chunk = (int)value;
    return FLF_OK;
  }
  if (!strcmp(name, "release_psf")) {
    if (value != 0 && value != 1) return fail(ctx, FLF_E_ARG, "release_psf must be 0 or 1");
    ctx->opt_release_psf = (int)value;
    if (value) maybe_release_psfs(ctx);
    return FLF_OK;
  }
  if (!strcmp(name, "mac_ctas_per_sm")) {
    if (value < 1 || value > 64) return fail(ctx, FLF_E_ARG, "mac_ctas_per_sm must be in [1, 64]");
    ctx->opt_ctas_per_sm = (int)value;
    return FLF_OK;
  }
  if (!strcmp(name, "geometry_cache")) {
    if (value < 0 || value > 16) return fail(ctx, FLF_E_ARG, "geometry_cache must be in [0, 16]");
    ctx->opt_geometry_cache = (int)value;
    while ((int)ctx->parked.size() > ctx->opt_geometry_cache) {
      cudaDeviceSynchronize();
      ctx->mem_epoch++;
      free_geometry(ctx->parked.back());
      ctx->parked.pop_back();
    }
    return FLF_OK;
  }
  if (!strcmp(name, "streams")) {
    if (value != 1 && value != 2) return fail(ctx, FLF_E_ARG, "streams must be 1 or 2");
    ctx->opt_streams = (int)value;
    return FLF_OK;
  }
  const bool cr_all = !strcmp(name, "mac_chunk_rows");
  const bool cr_fwd = !strcmp(name, "mac_chunk_rows_forward"), cr_bwd = !strcmp(name, "mac_chunk_rows_backward");
  if (!strcmp(name, "mac_stages") || cr_all || cr_fwd || cr_bwd || !strcmp(name, "mac_split")) {
    const int st = !strcmp(name, "mac_stages") ? (int)value : ctx->opt_stages;
    const int crf = (cr_all || cr_fwd) ? (int)value : ctx->opt_chunk_rows[FLF_DIR_FORWARD];
    const int crb = (cr_all || cr_bwd) ? (int)value : ctx->opt_chunk_rows[FLF_DIR_BACKWARD];
    const int sp = !strcmp(name, "mac_split") ? (int)value : ctx->opt_split;
    if (st < 2 || st > 16) return fail(ctx, FLF_E_ARG, "mac_stages must be in [2, 16]");
    for (int cr : {crf, crb})
      if (cr < 2 || cr > 64 || (cr & 1)) return fail(ctx, FLF_E_ARG, "mac_chunk_rows must be even, in [2, 64]");
    const int ntp = (ctx->L.nthr + 31) / 32 * 32;
    if (sp < 1 || sp > 4 || 2 * sp * ntp > 256)
      return fail(ctx, FLF_E_ARG, "mac_split must be in [1, 4] with at most 256 threads per block "
                                  "(2 frequency pairs x split x %d orbit threads)", ntp);
    for (int cr : {crf, crb})
      if (mac_smem_bytes(ctx->L, 1, st, cr, sp, true) > kMacSmemMax)
        return fail(ctx, FLF_E_ARG, "pipeline of %d stages x %d rows exceeds shared memory", st, cr);
    ctx->opt_stages = st;
    ctx->opt_chunk_rows[FLF_DIR_FORWARD] = crf;
    ctx->opt_chunk_rows[FLF_DIR_BACKWARD] = crb;
    ctx->opt_split = sp;
    return FLF_OK;
  }
  return fail(ctx, FLF_E_ARG, "unknown option '%s'", name);
}

int flf_autotune(flf_ctx *ctx, int T, int Y, int X, int *out4, void *stream) {
  if (!ctx || !out4) return FLF_E_ARG;
  cudaSetDevice(ctx->device);
  cudaStream_t s = (cudaStream_t)stream;
  if (int rc0 = check_psfs(ctx, 3)) return rc0;
  int rc = check_ready(ctx, T, Y, X, FLF_DIR_FORWARD, s);
  if (rc == FLF_OK) rc = check_ready(ctx, T, Y, X, FLF_DIR_BACKWARD, s);
  PlaneSet ps;
  if (rc == FLF_OK) rc = make_plane_set(ctx, nullptr, ctx->nz, s, ps);
  if (rc != FLF_OK) return rc;
  Geometry &Gm = ctx->geo;
  const int nt = std::min(T, frames_per_pass(ctx));
  size_t sSf, sOf, sCf, sSb, sOb, sCb;
  ws_needs(ctx, ps, nt, true, sSf, sOf, sCf);
  ws_needs(ctx, ps, nt, false, sSb, sOb, sCb);
  rc = ensure_ws(ctx, ctx->wsS, std::max(sSf, sSb));
  if (rc == FLF_OK) rc = ensure_ws(ctx, ctx->wsO, std::max(sOf, sOb));
  if (rc != FLF_OK) return rc;
  CUDA_TRY(ctx, cudaMemsetAsync(ctx->wsS.p, 0, ctx->wsS.bytes, s));
  // time the group that streams the most matrix bytes
  size_t gi = 0;
  double most = -1;
  for (size_t g = 0; g < Gm.groups.size(); g++) {
    const double b = (double)Gm.groups[g].nkp * ps.n[g];
    if (b > most) { most = b; gi = g; }
  }
  const int ntp = (ctx->L.nthr + 31) / 32 * 32;
  const int stages_c[] = {2, 3};
  const int chunk_c[] = {8, 10, 12, 16, 20};
  const int split_c[] = {1, 2};
  cudaEvent_t e0, e1;
  CUDA_TRY(ctx, cudaEventCreate(&e0));
  CUDA_TRY(ctx, cudaEventCreate(&e1));
  // best[dir][stages][split] = (time, chunk)
  double bt[2][2][2];
  int bc[2][2][2];
  for (int d = 0; d < 2; d++)
    for (int a = 0; a < 2; a++)
      for (int b = 0; b < 2; b++) { bt[d][a][b] = 1e30; bc[d][a][b] = 0; }
  cudaError_t e = cudaSuccess;
  for (int d = 0; d < 2 && e == cudaSuccess; d++)
    for (int a = 0; a < 2 && e == cudaSuccess; a++)
      for (int b = 0; b < 2 && e == cudaSuccess; b++) {
        if (2 * split_c[b] * ntp > 256) continue;
        for (int ch : chunk_c) {
          if (mac_smem_bytes(ctx->L, nt <= 1 ? 1 : (nt <= 2 ? 2 : 4), stages_c[a], ch, split_c[b], true) > kMacSmemMax)
            continue;
          e = mac_group_launch(ctx, gi, d, nt, ps, stages_c[a], ch, split_c[b], s);   // warm-up
          if (e == cudaSuccess) e = cudaEventRecord(e0, s);
          for (int k = 0; k < 3 && e == cudaSuccess; k++) e = mac_group_launch(ctx, gi, d, nt, ps, stages_c[a], ch, split_c[b], s);
          if (e == cudaSuccess) e = cudaEventRecord(e1, s);
          if (e == cudaSuccess) e = cudaEventSynchronize(e1);
          float ms = 0;
          if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
          if (e != cudaSuccess) break;
          if (ms < bt[d][a][b]) { bt[d][a][b] = ms; bc[d][a][b] = ch; }
        }
      }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (e != cudaSuccess) return fail(ctx, FLF_E_CUDA, "autotune launch failed: %s", cudaGetErrorString(e));
  if ((rc = check_device_flag(ctx)) != FLF_OK) return rc;
  int ba = 0, bb = 0;
  double best = 1e30;
  for (int a = 0; a < 2; a++)
    for (int b = 0; b < 2; b++)
      if (bc[0][a][b] && bc[1][a][b] && bt[0][a][b] + bt[1][a][b] < best) {
        best = bt[0][a][b] + bt[1][a][b];
        ba = a; bb = b;
      }
  if (best >= 1e30) return fail(ctx, FLF_E_STATE, "autotune found no launch shape that fits this geometry");
  Gm.tuned[0] = stages_c[ba];
  Gm.tuned[1] = bc[FLF_DIR_FORWARD][ba][bb];
  Gm.tuned[2] = bc[FLF_DIR_BACKWARD][ba][bb];
  Gm.tuned[3] = split_c[bb];
  for (int i = 0; i < 4; i++) out4[i] = Gm.tuned[i];
  return FLF_OK;
}

int flf_set_tuned(flf_ctx *ctx, int Y, int X, const int *in4) {
  if (!ctx || !in4) return FLF_E_ARG;
  Geometry &Gm = ctx->geo;
  if (!Gm.valid || Gm.Y != Y || Gm.X != X)
    return fail(ctx, FLF_E_STATE, "no prepared geometry for %d x %d: call flf_prepare first", Y, X);
  const int ntp = (ctx->L.nthr + 31) / 32 * 32;
  if (in4[0] < 2 || in4[0] > 16 || in4[3] < 1 || in4[3] > 4 || in4[3] * ntp > 256)
    return fail(ctx, FLF_E_ARG, "invalid launch shape");
  for (int d = 1; d <= 2; d++)
    if (in4[d] < 2 || in4[d] > 64 || (in4[d] & 1) ||
        mac_smem_bytes(ctx->L, 1, in4[0], in4[d], in4[3], true) > kMacSmemMax)
      return fail(ctx, FLF_E_ARG, "invalid rows per chunk %d", in4[d]);
  for (int i = 0; i < 4; i++) Gm.tuned[i] = in4[i];
  return FLF_OK;
}

int flf_resample_bilinear(const float *img_dev, int H, int W, const double *yq_dev, int ny, const double *xq_dev,
                          int nx, double *out_dev, void *stream) {
  if (!img_dev || !yq_dev || !xq_dev || !out_dev) return fail(nullptr, FLF_E_ARG, "NULL array pointer");
  if (H <= 0 || W <= 0 || ny < 0 || nx < 0)
    return fail(nullptr, FLF_E_ARG, "invalid sizes (image %d x %d, queries %d x %d)", H, W, ny, nx);
  ResampleParams rp{img_dev, H, W, yq_dev, xq_dev, ny, nx, out_dev};
  const cudaError_t e = launch_resample_bilinear(rp, (cudaStream_t)stream);
  if (e != cudaSuccess) return fail(nullptr, FLF_E_CUDA, "resample launch failed: %s", cudaGetErrorString(e));
  return FLF_OK;
}

static bool aligned16(const void *p) { return ((uintptr_t)p & 15) == 0; }

int flf_psf_debye(double *out_dev, int mode, long long npoints, double dx, double M, double k, double sin_alpha,
                  const double *s_dev, const double *cw_dev, int nodes, double koi_re, double koi_im,
                  void *stream) {
  if (!out_dev || !s_dev || !cw_dev) return fail(nullptr, FLF_E_ARG, "NULL array pointer");
  if ((mode != 0 && mode != 1) || npoints < 0 || nodes <= 0 || !(M > 0) || !(sin_alpha > 0))
    return fail(nullptr, FLF_E_ARG, "invalid Debye arguments (mode %d, points %lld, nodes %d)", mode, npoints,
                nodes);
  if (!aligned16(out_dev) || !aligned16(cw_dev))
    return fail(nullptr, FLF_E_ARG, "complex arrays must be 16-byte aligned");
  PsfDebyeParams p{(double2 *)out_dev, mode, npoints, dx, M, k, sin_alpha, s_dev, (const double2 *)cw_dev,
                   nodes, koi_re, koi_im};
  const cudaError_t e = launch_psf_debye(p, (cudaStream_t)stream);
  if (e != cudaSuccess) return fail(nullptr, FLF_E_CUDA, "Debye launch failed: %s", cudaGetErrorString(e));
  return FLF_OK;
}

int flf_psf_lf_input(double *out_dev, const double *wave_dev, int support, int max_bug, const double *lens_dev,
                     int lens_h, int L, int nh, int osr, int q0, int nq, void *stream) {
  if (!out_dev || !wave_dev || !lens_dev) return fail(nullptr, FLF_E_ARG, "NULL array pointer");
  if (L <= 0 || (L % 2) == 0 || support < 0 || support > (L - 1) / 2 || lens_h < 0 || nh <= 0 || osr <= 0 ||
      q0 < 0 || nq < 0 || q0 + nq > nh * nh || nq > 65535)
    return fail(nullptr, FLF_E_ARG, "invalid light-field input arguments (L %d, support %d, offsets %d+%d)", L,
                support, q0, nq);
  if (!aligned16(out_dev) || !aligned16(wave_dev) || !aligned16(lens_dev))
    return fail(nullptr, FLF_E_ARG, "complex arrays must be 16-byte aligned");
  PsfInputParams p{(double2 *)out_dev, (const double2 *)wave_dev, support, max_bug ? 1 : 0,
                   (const double2 *)lens_dev, lens_h, L, nh, osr, q0, nq};
  const cudaError_t e = launch_psf_lf_input(p, (cudaStream_t)stream);
  if (e != cudaSuccess) return fail(nullptr, FLF_E_CUDA, "light-field input launch failed: %s", cudaGetErrorString(e));
  return FLF_OK;
}

int flf_psf_lf_bin(float *out_dev, const double *field_dev, int L, int S, int nh, int osr, int q0, int nq, int lo,
                   int hi, int first, void *stream) {
  if (!out_dev || !field_dev) return fail(nullptr, FLF_E_ARG, "NULL array pointer");
  if (L <= 0 || S <= 0 || nh <= 0 || osr <= 0 || q0 < 0 || nq < 0 || q0 + nq > nh * nh || nq > 65535 ||
      first < 0 || first + S * osr > L)
    return fail(nullptr, FLF_E_ARG, "invalid binning arguments (L %d, S %d, OSR %d, first %d)", L, S, osr, first);
  if (!aligned16(field_dev)) return fail(nullptr, FLF_E_ARG, "complex arrays must be 16-byte aligned");
  PsfBinParams p{out_dev, (const double2 *)field_dev, L, S, nh, osr, q0, nq, lo, hi, first};
  const cudaError_t e = launch_psf_lf_bin(p, (cudaStream_t)stream);
  if (e != cudaSuccess) return fail(nullptr, FLF_E_CUDA, "binning launch failed: %s", cudaGetErrorString(e));
  return FLF_OK;
}

int flf_psf_ht(float *Ht_dev, const float *H_dev, int Z, int nh, int S, int N, void *stream) {
  if (!Ht_dev || !H_dev) return fail(nullptr, FLF_E_ARG, "NULL array pointer");
  if (Z <= 0 || N <= 0 || (N % 2) == 0 || nh != (N + 1) / 2 || S <= 0 || (S % 2) == 0 || ((S / 2) % N) != 0 ||
      (long long)Z * nh * nh > 65535)
    return fail(nullptr, FLF_E_ARG, "invalid Ht arguments (Z %d, N %d, S %d)", Z, N, S);
  PsfHtParams p{Ht_dev, H_dev, Z, nh, S, N};
  const cudaError_t e = launch_psf_ht(p, (cudaStream_t)stream);
  if (e != cudaSuccess) return fail(nullptr, FLF_E_CUDA, "Ht launch failed: %s", cudaGetErrorString(e));
  return FLF_OK;
}

static int net_sms() {
  static int sms = 0;
  if (!sms) {
    int dev = 0;
    cudaGetDevice(&dev);
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms <= 0) sms = 132;
  }
  return sms;
}

static int net_shape(int B, int Z, int Y, int X, int C) {
  if (B <= 0 || Z <= 0 || Y <= 0 || X <= 0 || C <= 0 || (C % 16) != 0)
    return fail(nullptr, FLF_E_ARG, "invalid volume shape %d x %d x %d x %d x %d (channels a multiple of 16)", B, Z,
                Y, X, C);
  return FLF_OK;
}

#define NET_CHECK(call)                                                                          \
  do {                                                                                           \
    const cudaError_t e_ = (call);                                                               \
    if (e_ != cudaSuccess) return fail(nullptr, FLF_E_CUDA, "%s: %s", #call, cudaGetErrorString(e_)); \
  } while (0)

int flf_conv3d(const void *x, const void *w, const float *bias, const void *mask, void *y, int B, int Z, int Y, int X,
               int Ci, int Co, int relu, float *ws, long long ws_elems, const void *wp, void *stream) {
  if (!x || !w || !y) return fail(nullptr, FLF_E_ARG, "NULL array pointer");
  if (int rc = net_shape(B, Z, Y, X, Ci)) return rc;
  if (int rc = net_shape(B, Z, Y, X, Co)) return rc;
  if (!aligned16(x) || !aligned16(w) || !aligned16(y) || (mask && !aligned16(mask)))
    return fail(nullptr, FLF_E_ARG, "volumes and weights must be 16-byte aligned");
  if (ws && !aligned16(ws)) return fail(nullptr, FLF_E_ARG, "workspace must be 16-byte aligned");
  if (wp && !aligned16(wp)) return fail(nullptr, FLF_E_ARG, "packed weights must be 16-byte aligned");
  ConvParams p{(const __nv_bfloat16 *)x, (const __nv_bfloat16 *)w, bias, (const __nv_bfloat16 *)mask,
               (__nv_bfloat16 *)y, B, Z, Y, X, Ci, Co, relu ? 1 : 0, ws, 1, (const __nv_bfloat16 *)wp};
  NET_CHECK(launch_conv3d(p, ws ? ws_elems : 0, (cudaStream_t)stream));
  return FLF_OK;
}

int flf_conv3d_x1(const void *x, const void *w, const float *bias, void *y, int B, int Z, int Y, int X, int relu,
                  void *stream) {
  if (!x || !w || !y) return fail(nullptr, FLF_E_ARG, "NULL array pointer");
  if (int rc = net_shape(B, Z, Y, X, 16)) return rc;
  if (!aligned16(x) || !aligned16(y)) return fail(nullptr, FLF_E_ARG, "volumes must be 16-byte aligned");
  ConvParams p{(const __nv_bfloat16 *)x, (const __nv_bfloat16 *)w, bias, nullptr, (__nv_bfloat16 *)y, B, Z, Y, X, 16, 16,
               relu ? 1 : 0, nullptr, 1};
  NET_CHECK(launch_conv3d_x1(p, (cudaStream_t)stream));
  return FLF_OK;
}

int flf_conv3d_pool(const void *x, const void *w, const float *bias, void *y, void *pooled, int B, int Z, int Y,
                    int X, int relu, void *stream) {
  if (!x || !w || !y || !pooled) return fail(nullptr, FLF_E_ARG, "NULL array pointer");
  if (int rc = net_shape(B, Z, Y, X, 16)) return rc;
  if ((Z | Y | X) & 1) return fail(nullptr, FLF_E_ARG, "Z, Y and X must be even (%d x %d x %d)", Z, Y, X);
  if (!aligned16(x) || !aligned16(y) || !aligned16(pooled))
    return fail(nullptr, FLF_E_ARG, "volumes must be 16-byte aligned");
  ConvParams p{(const __nv_bfloat16 *)x, (const __nv_bfloat16 *)w, bias, nullptr, (__nv_bfloat16 *)y, B, Z, Y, X, 16, 16,
               relu ? 1 : 0, nullptr, 1};
  p.pool = (__nv_bfloat16 *)pooled;
  NET_CHECK(launch_conv3d_pool(p, (cudaStream_t)stream));
  return FLF_OK;
}

int flf_conv3d_tc(const void *x, const void *w, const float *bias, const void *mask, void *y, int B, int Z, int Y,
                  int X, int relu, int rows, void *stream) {
  if (!x || !w || !y) return fail(nullptr, FLF_E_ARG, "NULL array pointer");
  if (int rc = net_shape(B, Z, Y, X, 16)) return rc;
  if (!aligned16(x) || !aligned16(y) || (mask && !aligned16(mask)))
    return fail(nullptr, FLF_E_ARG, "volumes must be 16-byte aligned");
  ConvParams p{(const __nv_bfloat16 *)x, (const __nv_bfloat16 *)w, bias, (const __nv_bfloat16 *)mask,
               (__nv_bfloat16 *)y, B, Z, Y, X, 16, 16, relu ? 1 : 0, nullptr, rows};
  if (rows != 0 && rows != -1 && rows != 1 && rows != 4 && rows != 5)
    return fail(nullptr, FLF_E_ARG,
                "tile choice must be 0 or -1 (warp-specialised, TMA-staged; -1 with 32-byte swizzled slabs), "
                "1, 4 or 5 (4 rows, double-buffered)");
  if (rows <= 0) NET_CHECK(launch_conv3d_tma16(p, (cudaStream_t)stream, rows < 0));
  else NET_CHECK(launch_conv3d_tc16(p, (cudaStream_t)stream));
  return FLF_OK;
}

int flf_net_conv16_tcgen05(int mode) { return net_set_conv16_tcgen05(mode); }

long long flf_net_launches(void) { return net_launches(); }

int flf_net_conv_wide_tcgen05(int mode) { return net_set_conv_wide_tcgen05(mode); }

int flf_net_status(void) {
  const int v = net_status_read_and_clear();
  if (v < 0) return fail(nullptr, FLF_E_CUDA, "reading the network status flag failed");
  if (v) return fail(nullptr, FLF_E_TIMEOUT, "a bounded wait in a tensor-core convolution gave up (code %d)", v);
  return FLF_OK;
}

int flf_conv3d_wgrad(const void *x, const void *dy, float *dw, int B, int Z, int Y, int X, int Ci, int Co,
                     float *ws, long long ws_elems, void *stream) {
  if (!x || !dy || !dw) return fail(nullptr, FLF_E_ARG, "NULL array pointer");
  if (int rc = net_shape(B, Z, Y, X, Ci)) return rc;
  if (int rc = net_shape(B, Z, Y, X, Co)) return rc;
  if (!aligned16(x) || !aligned16(dy)) return fail(nullptr, FLF_E_ARG, "volumes must be 16-byte aligned");
  if (ws && ws_elems < 0) return fail(nullptr, FLF_E_ARG, "negative workspace size");
  WgradParams p{(const __nv_bfloat16 *)x, (const __nv_bfloat16 *)dy, dw, B, Z, Y, X, Ci, Co, 0, ws};
  NET_CHECK(launch_conv3d_wgrad(p, ws ? ws_elems : 0, (cudaStream_t)stream, net_sms()));
  return FLF_OK;
}

int flf_conv3d_flip(const void *w, void *w2, int Ci, int Co, void *stream) {
  if (!w || !w2 || Ci <= 0 || Co <= 0) return fail(nullptr, FLF_E_ARG, "invalid weight flip arguments");
  NET_CHECK(launch_conv3d_flip(w, w2, Ci, Co, (cudaStream_t)stream));
  return FLF_OK;
}

int flf_conv3d_pack(const void *w, void *wp, int Ci, int Co, void *stream) {
  if (!w || !wp || Ci <= 0 || Co <= 0 || Ci % 16 || Co % 8)
    return fail(nullptr, FLF_E_ARG, "invalid weight packing arguments (Ci a multiple of 16, Co of 8)");
  if (!aligned16(wp)) return fail(nullptr, FLF_E_ARG, "packed weights must be 16-byte aligned");
  NET_CHECK(launch_conv3d_pack(w, wp, Ci, Co, (cudaStream_t)stream));
  return FLF_OK;
}

int flf_bias_grad(const void *g, float *db, long long M, int C, float *ws, long long ws_elems, void *stream) {
  if (!g || !db || M < 0 || C <= 0 || C > 128 || (ws && ws_elems < 0))
    return fail(nullptr, FLF_E_ARG, "invalid bias gradient arguments");
  if (M > 0) NET_CHECK(launch_bias_grad(g, db, ws, ws ? ws_elems : 0, M, C, (cudaStream_t)stream));
  return FLF_OK;
}

static int even_shape(int B, int Z, int Y, int X, int C) {
  if (B <= 0 || Z <= 0 || Y <= 0 || X <= 0 || C <= 0 || (Z | Y | X) & 1)
    return fail(nullptr, FLF_E_ARG, "pooling needs positive, even Z / Y / X (got %d x %d x %d)", Z, Y, X);
  return FLF_OK;
}

int flf_pool2(const void *in, void *out, int B, int Z, int Y, int X, int C, void *stream) {
  if (!in || !out) return fail(nullptr, FLF_E_ARG, "NULL array pointer");
  if (int rc = even_shape(B, Z, Y, X, C)) return rc;
  NET_CHECK(launch_pool2(in, out, B, Z, Y, X, C, (cudaStream_t)stream));
  return FLF_OK;
}

int flf_pool2_bwd(const void *gpool, const void *gskip, const void *act, void *gin, int B, int Z, int Y, int X, int C,
                  void *stream) {
  if (!gpool || !gin) return fail(nullptr, FLF_E_ARG, "NULL array pointer");
  if (int rc = even_shape(B, Z, Y, X, C)) return rc;
  NET_CHECK(launch_pool2_bwd(gpool, gskip, act, gin, B, Z, Y, X, C, (cudaStream_t)stream));
  return FLF_OK;
}

int flf_up2_add(const void *low, const void *skip, void *out, int B, int Z, int Y, int X, int C, void *stream) {
  if (!low || !out) return fail(nullptr, FLF_E_ARG, "NULL array pointer");
  if (int rc = even_shape(B, Z, Y, X, C)) return rc;
  if (C % 8 || ((C / 8) & (C / 8 - 1)))
    return fail(nullptr, FLF_E_ARG, "upsampling needs C / 8 a power of two (got C = %d)", C);
  NET_CHECK(launch_up2_add(low, skip, out, B, Z, Y, X, C, (cudaStream_t)stream));
  return FLF_OK;
}

int flf_up2_bwd(const void *g, const void *act, void *glow, int B, int Z, int Y, int X, int C, void *stream) {
  if (!g || !glow) return fail(nullptr, FLF_E_ARG, "NULL array pointer");
  if (int rc = even_shape(B, Z, Y, X, C)) return rc;
  NET_CHECK(launch_up2_bwd(g, act, glow, B, Z, Y, X, C, (cudaStream_t)stream));
  return FLF_OK;
}

int flf_mse_grad(const void *y, const float *target, void *g, float *loss, long long M, int C, void *stream) {
  if (!y || !target || !g || !loss || M <= 0 || C <= 0) return fail(nullptr, FLF_E_ARG, "invalid loss arguments");
  NET_CHECK(launch_mse_grad(y, target, g, loss, M, C, (cudaStream_t)stream));
  return FLF_OK;
}

int flf_adam(float *w, const float *g, float *m, float *v, void *wb, long long n, float lr, float b1, float b2,
             float eps, float c1, float c2, float wd, void *stream) {
  if (!w || !g || !m || !v || n < 0) return fail(nullptr, FLF_E_ARG, "invalid Adam arguments");
  if (n > 0) NET_CHECK(launch_adam(w, g, m, v, wb, n, lr, b1, b2, eps, c1, c2, wd, (cudaStream_t)stream));
  return FLF_OK;
}

int flf_render_blobs(float *vol, int Z, int Y, int X, const float *pts, int npts, float sigma, void *acc,
                     void *stream) {
  if (!vol || (!pts && npts > 0) || Z <= 0 || Y <= 0 || X <= 0 || npts < 0 || !(sigma > 0) || sigma > 8)
    return fail(nullptr, FLF_E_ARG, "invalid blob rendering arguments");
  if (!aligned16(pts)) return fail(nullptr, FLF_E_ARG, "blob array must be 16-byte aligned");
  if (acc && (reinterpret_cast<uintptr_t>(acc) & 7)) return fail(nullptr, FLF_E_ARG, "accumulator must be 8-byte aligned");
  NET_CHECK(launch_render_blobs(vol, acc, Z, Y, X, pts, npts, sigma, (cudaStream_t)stream));
  return FLF_OK;
}

int flf_ws_input(const float *htf, const float *hth1, const float *ht1, float *sum_x1, void *out, int T, int Z,
                 int Y, int X, int Zp, int Yp, int Xp, float c2, float c3, void *stream) {
  if (!htf || !hth1 || !ht1 || !sum_x1 || !out) return fail(nullptr, FLF_E_ARG, "NULL array pointer");
  if (T <= 0 || Z <= 0 || Y <= 0 || X <= 0 || Zp < Z || Yp < Y || Xp < X || T > 65535)
    return fail(nullptr, FLF_E_ARG, "invalid warm-start input shape");
  if (!aligned16(out)) return fail(nullptr, FLF_E_ARG, "network input must be 16-byte aligned");
  WsInputParams p{htf, hth1, ht1, sum_x1, (__nv_bfloat16 *)out, T, Z, Y, X, Zp, Yp, Xp, (float)Z * Y * X, c2, c3};
  NET_CHECK(launch_ws_input(p, (cudaStream_t)stream));
  return FLF_OK;
}

int flf_ws_head(const void *d, const void *w, float bias, float floor_, const float *sum_x1, float *x0, int T, int Z,
                int Y, int X, int Zp, int Yp, int Xp, void *stream) {
  if (!d || !w || !sum_x1 || !x0) return fail(nullptr, FLF_E_ARG, "NULL array pointer");
  if (T <= 0 || Z <= 0 || Y <= 0 || X <= 0 || Zp < Z || Yp < Y || Xp < X)
    return fail(nullptr, FLF_E_ARG, "invalid warm-start head shape");
  if (!aligned16(d) || !aligned16(w)) return fail(nullptr, FLF_E_ARG, "features and weights must be 16-byte aligned");
  NET_CHECK(launch_ws_head(d, w, bias, floor_, sum_x1, x0, T, Z, Y, X, Zp, Yp, Xp, (cudaStream_t)stream));
  return FLF_OK;
}

int flf_version(char *buf, size_t len) {
  if (!buf || len == 0) return FLF_E_ARG;
  snprintf(buf, len, "libflf 0.3 sm_103a kernels: k_split k_rfft2_sized k_mac k_irfft2_sized k_merge k_build_k k_rfft2 k_pack k_resample_bilinear k_psf_debye k_psf_lf_input k_psf_lf_bin k_psf_ht k_conv3d k_conv3d_wgrad");
  return FLF_OK;
}

}  // extern "C"
