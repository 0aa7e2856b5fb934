// Kernels of the learned warm start: a 3-D U-Net on channels-last BF16
// volumes [B][Z][Y][X][C] with FP32 accumulation.
//
//   k_conv3d<BN>      3x3x3 'same' convolution as an implicit GEMM
//                     (M = voxels, N = output channels, K = 27 taps x input
//                     channels) on the BF16 tensor cores (mma.sync m16n8k16),
//                     4-stage cp.async ring, swizzled shared tiles read with
//                     ldmatrix; epilogue: bias, ReLU, gradient mask, BF16.
//                     The data gradient is the same kernel on the flipped,
//                     transposed weights (k_conv3d_flip_weights).
//   k_conv3d_tiled    the same for 16 / 32 channels in and out: persistent
//                     CTAs with the weights resident in shared memory and
//                     one staged input patch per output tile for all taps.
//   k_conv3d_t16      16 -> 16 channels: 16 x 16-voxel tiles, 4 rows per warp,
//                     one z slice of weight fragments in registers at a time;
//                     with HEAD, the warm-start head writing the start volume.
//   k_conv3d_tma16    16 / 32 -> 16 / 32 channels on tcgen05 (the default for
//                     these layers): warp-specialised producer / MMA /
//                     epilogue roles, TMA-staged input slabs, the z taps
//                     folded into N and summed from a TMEM accumulator ring;
//                     variants: the 3x3x1 first layer (X1), the folded head
//                     (HEAD) and the output's 2x2x2 pooling from the epilogue
//                     (POOL).
//   k_conv3d_tc16     the first single-role tcgen05 16 -> 16 kernel.
//   k_conv3d_wide     32..128 -> 32..128 channels (a side of 64 or more) on
//                     tcgen05: padded-row implicit GEMM over TMA-staged input
//                     slabs, packed weights streamed by bulk copies, persistent
//                     CTAs with two TMEM accumulator buffers.
//   k_conv3d_wgrad    weight gradient dW[tap][ci][co] = sum_v x[v+tap][ci]
//                     dy[v][co]: per (voxel chunk, tap, channel tile) one CTA,
//                     split-K over its 4 warps; each chunk writes a partial
//                     sum and k_wgrad_reduce adds them in chunk order (no
//                     atomics, so training repeats bit for bit).
//   small kernels     bias gradient, 2x2x2 average pooling and its adjoint,
//                     nearest 2x2x2 upsampling + skip and its adjoint with the
//                     ReLU mask, MSE loss gradient, Adam, bead rendering.
#include "flf_internal.cuh"

#include <atomic>

#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>

namespace flf {

// Kernel launches made by this file since the library was loaded (flf_net_launches).
static std::atomic<long long> g_net_launches{0};
#define FLF_NET_LAUNCH(...)  \
  do {                       \
    __VA_ARGS__;             \
    ++g_net_launches;        \
  } while (0)

long long net_launches() { return g_net_launches.load(); }

namespace {

typedef __nv_bfloat16 bf16;

__device__ __forceinline__ uint32_t su32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void cp16(uint32_t dst, const void *src, bool valid) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(dst), "l"(src), "r"(valid ? 16 : 0)
               : "memory");
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

__device__ __forceinline__ void ldsm4(uint32_t a, uint32_t &r0, uint32_t &r1, uint32_t &r2, uint32_t &r3) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
               : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3)
               : "r"(a));
}
__device__ __forceinline__ void ldsm4t(uint32_t a, uint32_t &r0, uint32_t &r1, uint32_t &r2, uint32_t &r3) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];\n"
               : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3)
               : "r"(a));
}
__device__ __forceinline__ void mma_bf16(float *c, const uint32_t *a, uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// XOR swizzle of 16-byte chunks in rows of R chunks: the 8 consecutive rows an
// ldmatrix reads at one logical chunk land in 8 distinct 4-bank groups.
template <int R>
__device__ __forceinline__ int swz(int row) {
  return R == 8 ? (row & 7) : R == 4 ? ((row >> 1) & 3) : ((row >> 2) & 1);
}

struct Vox {
  int b, z, y, x;
};
__device__ __forceinline__ Vox decode(long long m, int Z, int Y, int X) {
  Vox v;
  v.x = (int)(m % X);
  m /= X;
  v.y = (int)(m % Y);
  m /= Y;
  v.z = (int)(m % Z);
  v.b = (int)(m / Z);
  return v;
}

}  // namespace

template <int BN>
__global__ void __launch_bounds__(128) k_conv3d(ConvParams p) {
  constexpr int BM = 128, NS = 4, RB = BN / 8;
  __shared__ __align__(128) bf16 As[NS][BM * 16];
  __shared__ __align__(128) bf16 Bs[NS][16 * BN];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const long long M = (long long)p.B * p.Z * p.Y * p.X;
  const long long m0 = (long long)blockIdx.x * BM;
  const int n0 = blockIdx.y * BN;
  const long long mrow = m0 + tid;
  const bool rowok = mrow < M;
  const Vox v = decode(rowok ? mrow : 0, p.Z, p.Y, p.X);
  const int cch = p.Ci / 16;
  const int KT = 27 * cch;
  const int kb = (int)((long long)blockIdx.z * KT / p.splits), ke = (int)((long long)(blockIdx.z + 1) * KT / p.splits);
  const int KS = ke - kb;

  auto load = [&](int kr, int st) {
    const int ks = kb + kr;
    const int tap = ks / cch, c0 = (ks - tap * cch) * 16;
    const int z = v.z + tap / 9 - 1, y = v.y + (tap / 3) % 3 - 1, x = v.x + tap % 3 - 1;
    const bool ok = rowok && z >= 0 && z < p.Z && y >= 0 && y < p.Y && x >= 0 && x < p.X;
    const bf16 *src = ok ? p.x + ((((long long)v.b * p.Z + z) * p.Y + y) * p.X + x) * p.Ci + c0 : p.x;
    const uint32_t base = su32(&As[st][tid * 16]);
    const int s = swz<2>(tid);
    cp16(base + ((0 ^ s) << 4), src, ok);
    cp16(base + ((1 ^ s) << 4), ok ? src + 8 : p.x, ok);
    if (tid < 16 * RB) {
      const int k = tid / RB, c = tid - k * RB;
      const bf16 *wsrc = p.w + ((long long)tap * p.Ci + c0 + k) * p.Co + n0 + c * 8;
      cp16(su32(&Bs[st][k * BN]) + ((c ^ swz<RB>(k)) << 4), wsrc, true);
    }
  };

  float acc[2][BN / 8][4];
#pragma unroll
  for (int i = 0; i < 2; i++)
#pragma unroll
    for (int j = 0; j < BN / 8; j++)
#pragma unroll
      for (int e = 0; e < 4; e++) acc[i][j][e] = 0.f;

#pragma unroll
  for (int s = 0; s < NS - 1; s++) {
    if (s < KS) load(s, s);
    cp_commit();
  }
  const int mat = lane >> 3, r8 = lane & 7;
  for (int ks = 0; ks < KS; ks++) {
    cp_wait<NS - 2>();
    __syncthreads();
    const int st = ks % NS;
    uint32_t a[2][4];
#pragma unroll
    for (int mt = 0; mt < 2; mt++) {
      const int row = warp * 32 + mt * 16 + r8 + 8 * (mat & 1);
      const int chunk = mat >> 1;
      ldsm4(su32(&As[st][row * 16]) + ((chunk ^ swz<2>(row)) << 4), a[mt][0], a[mt][1], a[mt][2], a[mt][3]);
    }
#pragma unroll
    for (int n2 = 0; n2 < BN / 16; n2++) {
      const int k = r8 + 8 * (mat & 1);
      const int c = n2 * 2 + (mat >> 1);
      uint32_t b0, b1, b2, b3;
      ldsm4t(su32(&Bs[st][k * BN]) + ((c ^ swz<RB>(k)) << 4), b0, b1, b2, b3);
#pragma unroll
      for (int mt = 0; mt < 2; mt++) {
        mma_bf16(acc[mt][2 * n2], a[mt], b0, b1);
        mma_bf16(acc[mt][2 * n2 + 1], a[mt], b2, b3);
      }
    }
    const int nk = ks + NS - 1;
    if (nk < KS) load(nk, nk % NS);
    cp_commit();
  }
  cp_wait<0>();

  if (p.splits > 1) {   // partial sums of this CTA's K range, in its own slice of ws
    float *slice = p.ws + (long long)blockIdx.z * M * p.Co;
#pragma unroll
    for (int mt = 0; mt < 2; mt++)
#pragma unroll
      for (int nt = 0; nt < BN / 8; nt++)
#pragma unroll
        for (int h = 0; h < 2; h++) {
          const long long row = m0 + warp * 32 + mt * 16 + (lane >> 2) + 8 * h;
          if (row >= M) continue;
          const int col = n0 + nt * 8 + 2 * (lane & 3);
          *reinterpret_cast<float2 *>(slice + row * p.Co + col) = make_float2(acc[mt][nt][2 * h], acc[mt][nt][2 * h + 1]);
        }
    return;
  }
#pragma unroll
  for (int mt = 0; mt < 2; mt++)
#pragma unroll
    for (int nt = 0; nt < BN / 8; nt++) {
      const int col = n0 + nt * 8 + 2 * (lane & 3);
      const float b0 = p.bias ? p.bias[col] : 0.f, b1 = p.bias ? p.bias[col + 1] : 0.f;
#pragma unroll
      for (int h = 0; h < 2; h++) {
        const long long row = m0 + warp * 32 + mt * 16 + (lane >> 2) + 8 * h;
        if (row >= M) continue;
        float v0 = acc[mt][nt][2 * h] + b0, v1 = acc[mt][nt][2 * h + 1] + b1;
        if (p.relu) {
          v0 = fmaxf(v0, 0.f);
          v1 = fmaxf(v1, 0.f);
        }
        const long long o = row * p.Co + col;
        if (p.mask) {
          const __nv_bfloat162 mk = *reinterpret_cast<const __nv_bfloat162 *>(p.mask + o);
          if (!(__bfloat162float(mk.x) > 0.f)) v0 = 0.f;
          if (!(__bfloat162float(mk.y) > 0.f)) v1 = 0.f;
        }
        *reinterpret_cast<__nv_bfloat162 *>(p.y + o) = __floats2bfloat162_rn(v0, v1);
      }
    }
}

// Persistent variant for the wide, shallow layers (Ci, Co in {16, 32}): all
// 27 x Ci x Co weights stay in shared memory; each CTA walks output tiles of
// one z slice, 8 rows x 16 columns, staging the 3 x 10 x 18 input patch of a
// tile (one buffer; two CTAs per SM overlap loads and math) and reading every tap's A fragments
// straight from the patch with shifted ldmatrix row addresses.  Each input
// voxel is fetched about 4 times instead of 27.
template <int CI, int CO>
__global__ void __launch_bounds__(128, 2) k_conv3d_tiled(ConvParams p, int tiles_x, int tiles_y, long long ntiles) {
  extern __shared__ __align__(128) unsigned char smem[];
  constexpr int PY = 10, PX = 18, PR = 3 * PY * PX;
  constexpr int RA = CI / 8, RB = CO / 8;
  bf16 *Ws = reinterpret_cast<bf16 *>(smem);     // [27 * CI][CO]
  bf16 *Ps = Ws + 27 * CI * CO;                   // [PR][CI] (one buffer: several CTAs per SM overlap)
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;

  for (int i = tid; i < 27 * CI * RB; i += 128) {
    const int row = i / RB, c = i - row * RB;
    cp16(su32(Ws + row * CO) + ((c ^ swz<RB>(row)) << 4), p.w + (long long)row * CO + c * 8, true);
  }
  auto tile_pos = [&](long long t, int &b, int &z, int &y0, int &x0) {
    const int tx = (int)(t % tiles_x);
    t /= tiles_x;
    const int ty = (int)(t % tiles_y);
    t /= tiles_y;
    z = (int)(t % p.Z);
    b = (int)(t / p.Z);
    y0 = ty * 8;
    x0 = tx * 16;
  };
  auto load_patch = [&](long long t, int buf) {
    int b, z, y0, x0;
    tile_pos(t, b, z, y0, x0);
    bf16 *P = Ps + buf * PR * CI;
    for (int i = tid; i < PR * RA; i += 128) {
      const int r = i / RA, c = i - r * RA;
      const int pz = r / (PY * PX), py = (r / PX) % PY, px = r % PX;
      const int gz = z + pz - 1, gy = y0 + py - 1, gx = x0 + px - 1;
      const bool ok = gz >= 0 && gz < p.Z && gy >= 0 && gy < p.Y && gx >= 0 && gx < p.X;
      const bf16 *src = ok ? p.x + ((((long long)b * p.Z + gz) * p.Y + gy) * p.X + gx) * CI + c * 8 : p.x;
      cp16(su32(P + r * CI) + ((c ^ swz<RA>(r)) << 4), src, ok);
    }
  };

  const int mat = lane >> 3, r8 = lane & 7;
  for (long long t = blockIdx.x; t < ntiles; t += gridDim.x) {
    load_patch(t, 0);
    cp_commit();
    cp_wait<0>();
    __syncthreads();
    const bf16 *P = Ps;
    float acc[2][CO / 8][4];
#pragma unroll
    for (int i = 0; i < 2; i++)
#pragma unroll
      for (int j = 0; j < CO / 8; j++)
#pragma unroll
        for (int e = 0; e < 4; e++) acc[i][j][e] = 0.f;
#pragma unroll 1
    for (int tap = 0; tap < 27; tap++) {
      const int dz = tap / 9, dy = (tap / 3) % 3, dx = tap % 3;
#pragma unroll
      for (int kc = 0; kc < CI / 16; kc++) {
        uint32_t a[2][4];
#pragma unroll
        for (int mt = 0; mt < 2; mt++) {
          const int yy = 2 * warp + mt, xx = r8 + 8 * (mat & 1);
          const int pr = (dz * PY + yy + dy) * PX + xx + dx;
          const int chunk = 2 * kc + (mat >> 1);
          ldsm4(su32(P + pr * CI) + ((chunk ^ swz<RA>(pr)) << 4), a[mt][0], a[mt][1], a[mt][2], a[mt][3]);
        }
#pragma unroll
        for (int n2 = 0; n2 < CO / 16; n2++) {
          const int row = tap * CI + kc * 16 + r8 + 8 * (mat & 1);
          const int c = n2 * 2 + (mat >> 1);
          uint32_t b0, b1, b2, b3;
          ldsm4t(su32(Ws + row * CO) + ((c ^ swz<RB>(row)) << 4), b0, b1, b2, b3);
#pragma unroll
          for (int mt = 0; mt < 2; mt++) {
            mma_bf16(acc[mt][2 * n2], a[mt], b0, b1);
            mma_bf16(acc[mt][2 * n2 + 1], a[mt], b2, b3);
          }
        }
      }
    }
    __syncthreads();   // the patch is refilled for the next tile
    int b, z, y0, x0;
    tile_pos(t, b, z, y0, x0);
#pragma unroll
    for (int mt = 0; mt < 2; mt++)
#pragma unroll
      for (int nt = 0; nt < CO / 8; nt++) {
        const int col = nt * 8 + 2 * (lane & 3);
        const float b0 = p.bias ? p.bias[col] : 0.f, b1 = p.bias ? p.bias[col + 1] : 0.f;
        const int y = y0 + 2 * warp + mt;
#pragma unroll
        for (int h = 0; h < 2; h++) {
          const int x = x0 + (lane >> 2) + 8 * h;
          if (y >= p.Y || x >= p.X) continue;
          float v0 = acc[mt][nt][2 * h] + b0, v1 = acc[mt][nt][2 * h + 1] + b1;
          if (p.relu) {
            v0 = fmaxf(v0, 0.f);
            v1 = fmaxf(v1, 0.f);
          }
          const long long o = ((((long long)b * p.Z + z) * p.Y + y) * p.X + x) * CO + col;
          if (p.mask) {
            const __nv_bfloat162 mk = *reinterpret_cast<const __nv_bfloat162 *>(p.mask + o);
            if (!(__bfloat162float(mk.x) > 0.f)) v0 = 0.f;
            if (!(__bfloat162float(mk.y) > 0.f)) v1 = 0.f;
          }
          *reinterpret_cast<__nv_bfloat162 *>(p.y + o) = __floats2bfloat162_rn(v0, v1);
        }
      }
  }
  cp_wait<0>();
}

// 16 -> 16 channels (the full-resolution layers).  A tile is 16 rows x 16
// columns of one z slice, 4 rows per warp (8 independent accumulator chains),
// staged as a 3 x 18 x 18 input patch; the weights stay in shared memory and
// the B fragments of one z slice of taps (9 taps) are held in registers while
// they are used.  Single-buffered patches keep shared memory and registers low
// enough for several CTAs per SM, whose loads overlap one another's math.
// HEAD: the warm-start head -- only output channel 0 is kept, written as the
// start volume max(v + bias, floor) * mean_t into x0 [Zr][T][Yr][Xr].
template <bool HEAD>
__global__ void __launch_bounds__(128, 4) k_conv3d_t16(ConvParams p, HeadOut h, int tiles_x, int tiles_y,
                                                       long long ntiles) {
  extern __shared__ __align__(128) unsigned char smem[];
  constexpr int PY = 18, PX = 18, PR = 3 * PY * PX;
  bf16 *Ws = reinterpret_cast<bf16 *>(smem);     // [27 * 16][16]
  bf16 *P = Ws + 27 * 16 * 16;                    // [PR][16]
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  for (int i = tid; i < 27 * 16 * 2; i += 128) {
    const int row = i >> 1, c = i & 1;
    cp16(su32(Ws + row * 16) + ((c ^ swz<2>(row)) << 4), p.w + (long long)row * 16 + c * 8, true);
  }
  cp_commit();
  const int mat = lane >> 3, r8 = lane & 7;
  const int xx = r8 + 8 * (mat & 1), chunk = mat >> 1;
  for (long long t = blockIdx.x; t < ntiles; t += gridDim.x) {
    long long q = t;
    const int tx = (int)(q % tiles_x);
    q /= tiles_x;
    const int ty = (int)(q % tiles_y);
    q /= tiles_y;
    const int z = (int)(q % p.Z), b = (int)(q / p.Z);
    const int y0 = ty * 16, x0 = tx * 16;
    for (int i = tid; i < PR * 2; i += 128) {
      const int r = i >> 1, c = i & 1;
      const int pz = r / (PY * PX), py = (r / PX) % PY, px = r % PX;
      const int gz = z + pz - 1, gy = y0 + py - 1, gx = x0 + px - 1;
      const bool ok = gz >= 0 && gz < p.Z && gy >= 0 && gy < p.Y && gx >= 0 && gx < p.X;
      const bf16 *src = ok ? p.x + ((((long long)b * p.Z + gz) * p.Y + gy) * p.X + gx) * 16 + c * 8 : p.x;
      cp16(su32(P + r * 16) + ((c ^ swz<2>(r)) << 4), src, ok);
    }
    cp_commit();
    cp_wait<0>();
    __syncthreads();
    float acc[4][2][4];
#pragma unroll
    for (int i = 0; i < 4; i++)
#pragma unroll
      for (int j = 0; j < 2; j++)
#pragma unroll
        for (int e = 0; e < 4; e++) acc[i][j][e] = 0.f;
#pragma unroll 1
    for (int dz = 0; dz < 3; dz++) {
      uint32_t bw[9][4];
#pragma unroll
      for (int k = 0; k < 9; k++) {
        const int row = (dz * 9 + k) * 16 + r8 + 8 * (mat & 1);
        ldsm4t(su32(Ws + row * 16) + (((mat >> 1) ^ swz<2>(row)) << 4), bw[k][0], bw[k][1], bw[k][2], bw[k][3]);
      }
#pragma unroll
      for (int k = 0; k < 9; k++) {
        const int dy = k / 3, dx = k % 3;
#pragma unroll
        for (int mt = 0; mt < 4; mt++) {
          const int pr = (dz * PY + 4 * warp + mt + dy) * PX + xx + dx;
          uint32_t a[4];
          ldsm4(su32(P + pr * 16) + ((chunk ^ swz<2>(pr)) << 4), a[0], a[1], a[2], a[3]);
          mma_bf16(acc[mt][0], a, bw[k][0], bw[k][1]);
          if (!HEAD) mma_bf16(acc[mt][1], a, bw[k][2], bw[k][3]);
        }
      }
    }
    __syncthreads();   // the patch is refilled for the next tile
    if (HEAD) {
      // channel 0 sits in lanes with (lane & 3) == 0: rows lane/4 and lane/4 + 8
      if ((lane & 3) == 0 && b < h.T && z < h.Zr) {
        const float sc = h.sum_x1[b] / h.count;
#pragma unroll
        for (int mt = 0; mt < 4; mt++) {
          const int y = y0 + 4 * warp + mt;
#pragma unroll
          for (int hh = 0; hh < 2; hh++) {
            const int x = x0 + (lane >> 2) + 8 * hh;
            if (y >= h.Yr || x >= h.Xr) continue;
            const float v = acc[mt][0][2 * hh] + h.bias;
            h.x0[(((long long)z * h.T + b) * h.Yr + y) * h.Xr + x] = fmaxf(v, h.floor) * sc;
          }
        }
      }
    } else {
#pragma unroll
    for (int mt = 0; mt < 4; mt++)
#pragma unroll
      for (int nt = 0; nt < 2; nt++) {
        const int col = nt * 8 + 2 * (lane & 3);
        const float b0 = p.bias ? p.bias[col] : 0.f, b1 = p.bias ? p.bias[col + 1] : 0.f;
        const int y = y0 + 4 * warp + mt;
#pragma unroll
        for (int hh = 0; hh < 2; hh++) {
          const int x = x0 + (lane >> 2) + 8 * hh;
          if (y >= p.Y || x >= p.X) continue;
          float v0 = acc[mt][nt][2 * hh] + b0, v1 = acc[mt][nt][2 * hh + 1] + b1;
          if (p.relu) {
            v0 = fmaxf(v0, 0.f);
            v1 = fmaxf(v1, 0.f);
          }
          const long long o = ((((long long)b * p.Z + z) * p.Y + y) * p.X + x) * 16 + col;
          if (p.mask) {
            const __nv_bfloat162 mk = *reinterpret_cast<const __nv_bfloat162 *>(p.mask + o);
            if (!(__bfloat162float(mk.x) > 0.f)) v0 = 0.f;
            if (!(__bfloat162float(mk.y) > 0.f)) v1 = 0.f;
          }
          *reinterpret_cast<__nv_bfloat162 *>(p.y + o) = __floats2bfloat162_rn(v0, v1);
        }
      }
    }
  }
  cp_wait<0>();
}

// ---------------------------------------------------------------------------
// 16 -> 16 channels on the 5th-generation tensor cores (tcgen05).  A tile is
// 128 consecutive voxels of one x row (M = 128); each of the 27 taps is one
// tcgen05.mma (M 128, N 16, K 16, BF16 in, FP32 accumulate in TMEM) issued by
// one thread with both operands read from shared memory through matrix
// descriptors in the canonical K-major, no-swizzle layout (8-row x 16-byte
// core matrices).  The 3 x 3 x 130-voxel input patch is stored as two planes
// of 8 channels, so the A tile of every tap is a uniformly strided window of
// it (start + (dz*3+dy)*130 + dx voxels; core matrices 128 B apart along M,
// one plane apart along K).  The accumulator is read back with tcgen05.ld
// (warp w holds rows 32w..32w+31).  Every wait is bounded; a wait that gives
// up sets g_net_err (flf_net_status) and the kernel stops cleanly.
// ---------------------------------------------------------------------------
__device__ int g_net_err;

namespace {

__device__ __forceinline__ uint64_t umma_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = (uint64_t)((saddr >> 4) & 0x3FFFu);
  d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
  d |= (uint64_t)1 << 46;                          // descriptor version (bits 46-48 = 0b001); no swizzle
  return d;
}
__device__ __forceinline__ void umma_f16(uint32_t tmem_d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
      "l"(a), "l"(b), "r"(idesc), "r"(acc)
      : "memory");
}
__device__ __forceinline__ void umma_commit(uint32_t mbar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(mbar)
               : "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory"); }
__device__ __forceinline__ void net_mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(bar), "r"(count) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
}
__device__ __forceinline__ bool net_mbar_wait(uint32_t bar, uint32_t parity, unsigned long long limit_ns) {
  unsigned long long t0 = 0;
  for (int it = 0;; it++) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    if (ok) return true;
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;\n" : "=l"(t));
    if (it == 0) t0 = t;
    else if (t - t0 > limit_ns) return false;
  }
}

}  // namespace

template <int ROWS, int NBUF>
__global__ void __launch_bounds__(128) k_conv3d_tc16(ConvParams p, int tiles_x, long long ntiles) {
  extern __shared__ __align__(1024) unsigned char smem[];
  constexpr int PXW = 130, PYH = ROWS + 2, PV = 3 * PYH * PXW;   // patch voxels: 3 (z) x (ROWS+2) (y) x 130 (x)
  constexpr uint32_t PLANE = PV * 16;                            // bytes of one 8-channel plane
  // layout: [B: 27 taps x 512 B][patch buffers x 2 planes][mbarrier 8 B][tmem address 4 B]
  unsigned char *Wb = smem;
  unsigned char *Pb = smem + 27 * 512;
  unsigned long long *bar = reinterpret_cast<unsigned long long *>(Pb + NBUF * 2 * PLANE);
  uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(bar + 1);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const uint32_t wb_s = su32(Wb), pb_s = su32(Pb), bar_s = su32(bar);
  constexpr uint32_t TCOLS = ROWS * 16 <= 32 ? 32 : (ROWS * 16 <= 64 ? 64 : 128);

  // B operands: per tap, co-major rows of 16 ci: core matrix (co/8, ci/8) at
  // (ci/8)*128 + (co/8)*256, row co%8 at 16 B, element ci%8 at 2 B.
  for (int i = tid; i < 27 * 16; i += 128) {
    const int tap = i >> 4, co = i & 15;
    uint32_t pk[8];
#pragma unroll
    for (int c = 0; c < 8; c++) {
      const unsigned short lo = __bfloat16_as_ushort(p.w[((long long)tap * 16 + 2 * c) * 16 + co]);
      const unsigned short hi = __bfloat16_as_ushort(p.w[((long long)tap * 16 + 2 * c + 1) * 16 + co]);
      pk[c] = (uint32_t)lo | ((uint32_t)hi << 16);
    }
    unsigned char *row = Wb + tap * 512 + (co >> 3) * 256 + (co & 7) * 16;
    *reinterpret_cast<uint4 *>(row) = make_uint4(pk[0], pk[1], pk[2], pk[3]);
    *reinterpret_cast<uint4 *>(row + 128) = make_uint4(pk[4], pk[5], pk[6], pk[7]);
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(su32(tmem_slot)),
                 "r"(TCOLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
  }
  if (tid == 0) net_mbar_init(bar_s, 1);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;
  // instruction descriptor: F32 accumulate, BF16 A and B, both K-major, N = 16, M = 128
  const uint32_t idesc = (1u << 4) | (1u << 7) | (1u << 10) | ((16u >> 3) << 17) | ((128u >> 4) << 24);
  bool ok = true;
  uint32_t phase = 0;
  const int tiles_y = (p.Y + ROWS - 1) / ROWS;
  auto tile_of = [&](long long t, int &b, int &z, int &y0, int &x0) {
    long long q = t;
    const int tx = (int)(q % tiles_x);
    q /= tiles_x;
    y0 = (int)(q % tiles_y) * ROWS;
    q /= tiles_y;
    z = (int)(q % p.Z);
    b = (int)(q / p.Z);
    x0 = tx * 128;
  };
  auto load_patch = [&](long long t, int buf) {
    int b, z, y0, x0;
    tile_of(t, b, z, y0, x0);
    const uint32_t base = pb_s + buf * 2 * PLANE;
    for (int i = tid; i < PV * 2; i += 128) {
      const int v = i >> 1, pl = i & 1;
      const int pz = v / (PYH * PXW), py = (v / PXW) % PYH, px = v % PXW;
      const int gz = z + pz - 1, gy = y0 + py - 1, gx = x0 + px - 1;
      const bool in = gz >= 0 && gz < p.Z && gy >= 0 && gy < p.Y && gx >= 0 && gx < p.X;
      const bf16 *src = in ? p.x + ((((long long)b * p.Z + gz) * p.Y + gy) * p.X + gx) * 16 + pl * 8 : p.x;
      cp16(base + pl * PLANE + v * 16, src, in);
    }
  };
  int buf = 0;
  if (NBUF == 2 && (long long)blockIdx.x < ntiles) load_patch(blockIdx.x, 0);
  cp_commit();
  for (long long t = blockIdx.x; t < ntiles && ok; t += gridDim.x) {
    int b, z, y0, x0;
    tile_of(t, b, z, y0, x0);
    if (NBUF == 2) {
      // the next tile's patch streams in while this tile multiplies
      if (t + gridDim.x < ntiles) load_patch(t + gridDim.x, buf ^ 1);
      cp_commit();
      cp_wait<1>();
    } else {
      load_patch(t, 0);
      cp_commit();
      cp_wait<0>();
    }
    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
    __syncthreads();
    const uint32_t pbuf = pb_s + buf * 2 * PLANE;
    if (tid == 0) {
      tc_fence_after();
#pragma unroll 1
      for (int tap = 0; tap < 27; tap++) {
        const int dz = tap / 9, dy = (tap / 3) % 3, dx = tap % 3;
        const uint64_t bd = umma_desc(wb_s + tap * 512, 128, 256);
#pragma unroll
        for (int r = 0; r < ROWS; r++) {   // independent accumulators, one per output row
          const uint64_t ad = umma_desc(pbuf + ((dz * PYH + r + dy) * PXW + dx) * 16, PLANE, 128);
          umma_f16(tmem + r * 16, ad, bd, idesc, tap > 0 ? 1u : 0u);
        }
      }
      umma_commit(bar_s);
    }
    const int late = net_mbar_wait(bar_s, phase, 1000000000ULL) ? 0 : 1;
    if (__syncthreads_or(late)) {     // one decision for the whole CTA
      if (tid == 0) atomicExch(&g_net_err, 2);
      ok = false;
      break;
    }
    phase ^= 1;
    tc_fence_after();
#pragma unroll 1
    for (int r = 0; r < ROWS; r++) {
      uint32_t v[16];
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
          : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
            "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
          : "r"(tmem + ((uint32_t)(warp * 32) << 16) + r * 16));
      asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
      const int x = x0 + warp * 32 + lane, y = y0 + r;
      if (x < p.X && y < p.Y) {
        const long long o = ((((long long)b * p.Z + z) * p.Y + y) * p.X + x) * 16;
        uint4 mk[2];
        if (p.mask) {
          mk[0] = *reinterpret_cast<const uint4 *>(p.mask + o);
          mk[1] = *reinterpret_cast<const uint4 *>(p.mask + o + 8);
        }
        uint4 outv[2];
        __nv_bfloat162 *h = reinterpret_cast<__nv_bfloat162 *>(outv);
        const __nv_bfloat162 *m2 = reinterpret_cast<const __nv_bfloat162 *>(mk);
#pragma unroll
        for (int k = 0; k < 8; k++) {
          float v0 = __uint_as_float(v[2 * k]) + (p.bias ? p.bias[2 * k] : 0.f);
          float v1 = __uint_as_float(v[2 * k + 1]) + (p.bias ? p.bias[2 * k + 1] : 0.f);
          if (p.relu) {
            v0 = fmaxf(v0, 0.f);
            v1 = fmaxf(v1, 0.f);
          }
          if (p.mask) {
            const float2 mf = __bfloat1622float2(m2[k]);
            if (!(mf.x > 0.f)) v0 = 0.f;
            if (!(mf.y > 0.f)) v1 = 0.f;
          }
          h[k] = __floats2bfloat162_rn(v0, v1);
        }
        *reinterpret_cast<uint4 *>(p.y + o) = outv[0];
        *reinterpret_cast<uint4 *>(p.y + o + 8) = outv[1];
      }
    }
    tc_fence_before();
    __syncthreads();   // TMEM and the patch buffer are reused
    if (NBUF == 2) buf ^= 1;
  }
  cp_wait<0>();
  if (!ok) {
    // let any MMA still in flight finish before the accumulator is released
    if (!net_mbar_wait(bar_s, phase, 1000000000ULL)) atomicExch(&g_net_err, 3);
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(TCOLS) : "memory");
  }
}

// ---------------------------------------------------------------------------
// 16 / 32 -> 16 / 32 channels, warp-specialised on tcgen05 with TMA staging
// (written here for CI = CO = 16; CI = 32 adds a second K step of 16
// channels, CO = 32 makes N = 96 and an item one row).  A work
// item is a column of output, R rows (y) x 128 voxels (x), over a run of z
// planes.  The CTA walks the input planes z' of the column: each is one slab,
// (R+2) rows of the voxels x0-1 .. (the x / y halo included), that TMA loads
// into a ring of S shared-memory slots through a tensor map over
// [B][Z][Y][X][16] BF16.  Two slab layouts (SW32):
//   true   one load per slab, box 16 channels x 136 x (R+2) x 1 x 1 with the
//          32-byte swizzle: a voxel is one 32-byte row whose 16-byte halves
//          are swapped where smem address bit 7 is set, rows 256-byte aligned,
//          which is the 32-byte-swizzled K-major A layout (8-row groups 256
//          bytes apart).  A tap's x shift moves the start 32 bytes per voxel;
//          the tensor cores apply the swizzle to the absolute address, as TMA
//          does, so shifted windows read correctly (checked by the tests);
//   false  two loads per slab, box 8 channels x 130 x (R+2) x 1 x 1, one per
//          8-channel plane: the canonical no-swizzle K-major layout, 8-voxel
//          x 16-byte core matrices, the planes one LBO apart.
// Coordinates outside the volume read zeros: the 'same' padding in x and y.
// The three z taps are folded into N.  For output row r of slab z', one
//   tcgen05.mma  M 128 (voxels x) x N 48 (dz, co) x K 16 (ci)
// per (dy, dx), with A the slab row r+dy shifted by dx, accumulates
//   D[z'][r][x][dz][co] = sum over (dy, dx, ci) of in[z'][r+dy][x+dx][ci] w[dz][dy][dx][ci][co]
// into one of 5 TMEM accumulator slots (R x N columns each), and
//   out[z][r][x][co] = D[z-1][r][x][0][co] + D[z][r][x][1][co] + D[z+1][r][x][2][co]
// adds three column groups of the same TMEM lane: no data moves between
// lanes.  A slab's shared memory is free as soon as its MMAs complete; its
// accumulator slot is free after the last output plane that reads it.
// Planes outside the volume contribute nothing: their MMAs are skipped and
// the epilogue leaves their terms out.
// The head (HEAD; only output channel 0 is used) folds (dz, dy) into N
// instead: one MMA of N 16 (9 columns used) per input row ri of a slab and dx,
//   D[z'][ri][x][dz*3 + dy] = sum over (dx, ci) of in[z'][y0-1+ri][x+dx-1][ci] w[dz*9 + dy*3 + dx][ci][0],
// and out[z][y0+r][x] = sum over (dz, dy) of D[z-1+dz][r+dy][x][dz*3+dy], so a
// slab of R+2 input rows costs 3 (R+2) MMAs for R output rows instead of 9 R.
//   warp 0     producer: one thread issues the TMA loads;
//   warps 1-2  MMA issuers: one thread each issues the 9 MMAs of half of the
//              rows per slab, then commits to the slab's accumulator barrier
//              and to its shared-memory slot; before a slab's MMAs it tests
//              the next slab's barriers without blocking, so that test's
//              latency overlaps the MMAs (a blocking wait follows only if a
//              phase was not complete yet);
//   warps 3-10 epilogue: warp w reads TMEM lane quarter w % 4 (tcgen05.ld)
//              for 8 of the 16 output channels, sums the three z terms, then
//              bias / ReLU / mask and BF16 stores, or with HEAD the clamped,
//              scaled start volume from output channel 0.  With POOL it also
//              writes the 2x2x2 average of the stored outputs (x pairs from
//              neighbouring lanes, row pairs of the item, plane pairs of
//              consecutive planes; z chunks of even length).
// Every mbarrier wait is bounded (1 s).  A wait that gives up sets g_net_err
// and a shared abort flag that every role polls; the CTA then waits (bounded)
// for its copies and MMAs in flight before TMEM is released.
// ---------------------------------------------------------------------------
struct Tma16Grid {   // work items: [B][zchunks][yblocks][xsegs] columns of R x 128 voxels over zc planes
  int xsegs, yblocks, zchunks, zc;
  long long items;
};

constexpr int TMA16_NACC = 5;   // TMEM accumulator slots (R x 3 CO columns each)

namespace {

__device__ __forceinline__ void net_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(bar), "r"(bytes) : "memory");
}
__device__ __forceinline__ void net_arrive(uint32_t bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];\n" ::"r"(bar) : "memory");
}
// non-blocking test of a phase (1 = the phase with this parity has completed)
__device__ __forceinline__ uint32_t mbar_test(uint32_t bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok;
}
__device__ __forceinline__ void tma_load_5d(uint32_t dst, const CUtensorMap *map, int c0, int c1, int c2, int c3,
                                            int c4, uint32_t bar) {
  asm volatile(
      "cp.async.bulk.tensor.5d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5, "
      "%6}], [%7];\n" ::"r"(dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(c4), "r"(bar)
      : "memory");
}
// bounded wait that also gives up when another role has aborted
__device__ __forceinline__ bool role_wait(uint32_t bar, uint32_t parity, volatile int *abort_s, int code) {
  unsigned long long t0 = 0;
  for (int it = 0;; it++) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    if (ok) return true;
    if (*abort_s) return false;
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;\n" : "=l"(t));
    if (it == 0) {
      t0 = t;
    } else if (t - t0 > 1000000000ULL) {
      *abort_s = 1;
      atomicExch(&g_net_err, code);
      return false;
    }
  }
}
__device__ __forceinline__ void tmem_ld16(uint32_t addr, float *v) {
  uint32_t u[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
      : "=r"(u[0]), "=r"(u[1]), "=r"(u[2]), "=r"(u[3]), "=r"(u[4]), "=r"(u[5]), "=r"(u[6]), "=r"(u[7]), "=r"(u[8]),
        "=r"(u[9]), "=r"(u[10]), "=r"(u[11]), "=r"(u[12]), "=r"(u[13]), "=r"(u[14]), "=r"(u[15])
      : "r"(addr));
#pragma unroll
  for (int k = 0; k < 16; k++) v[k] = __uint_as_float(u[k]);
}
__device__ __forceinline__ void tmem_ld8(uint32_t addr, float *v) {
  uint32_t u[8];
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];\n"
               : "=r"(u[0]), "=r"(u[1]), "=r"(u[2]), "=r"(u[3]), "=r"(u[4]), "=r"(u[5]), "=r"(u[6]), "=r"(u[7])
               : "r"(addr));
#pragma unroll
  for (int k = 0; k < 8; k++) v[k] = __uint_as_float(u[k]);
}

}  // namespace

// Head epilogue: add column dz*3 + dy of input row r + dy (dy = 0..2) to output row r.
template <int RH, int DZ>
__device__ __forceinline__ void head_rows(float (&o)[RH], const float (&v)[RH + 2][16], bool in) {
#pragma unroll
  for (int r = 0; r < RH; r++)
#pragma unroll
    for (int dy = 0; dy < 3; dy++) o[r] += in ? v[r + dy][DZ * 3 + dy] : 0.f;
}

template <int CI, int CO, int R, int S, bool HEAD, bool SW32, bool X1 = false, bool POOL = false>
__global__ void __launch_bounds__(352, 1)
    k_conv3d_tma16(const __grid_constant__ CUtensorMap tx, ConvParams p, HeadOut h, Tma16Grid g) {
  extern __shared__ __align__(1024) unsigned char smem[];
  constexpr int PYH = R + 2, NACC = TMA16_NACC;
  constexpr int KS = CI / 16;                 // K steps of 16 input channels
  // N of one MMA: (dz, co); the head, whose only output channel is 0, folds (dz, dy) into N
  // instead (9 of 16 columns) and issues one MMA per input row and dx
  constexpr int NN = HEAD ? 16 : 3 * CO;
  // B blocks per K step: (dy, dx); dx for the head; dy for X1, a 3x3x1 convolution (the taps
  // dx != 1 of w are ignored: the first layer, whose input carries the x neighbours as channels)
  constexpr int NBLK = (HEAD || X1) ? 3 : 9;
  static_assert(!(HEAD && X1), "the head is a full 3x3x3 convolution");
  static_assert(!POOL || (CO == 16 && R == 2 && !HEAD && !X1),
                "the pooled output is for 16 output channels and two rows per item");
  constexpr int NISS = (HEAD ? PYH : R) % 2 == 0 ? 2 : 1;   // MMA-issuing threads (warps 1 .. NISS)
  constexpr int CH = CO / 2;                  // output channels per epilogue warp
  static_assert((CI == 16 || CI == 32) && (CO == 16 || CO == 32), "16 or 32 channels in and out");
  static_assert(SW32 || CI == 16, "the unswizzled slab layout is for 16 input channels");
  static_assert(!HEAD || (CI == 16 && CO == 16), "the head is a 16 -> 16 convolution");
  // SW32: per slab one load per 16 input channels of rows of 136 voxels x 32 bytes, written with
  // the 32-byte swizzle (16-byte halves of a voxel swapped where address bit 7 is set); otherwise
  // two loads of 130-voxel rows x 16 bytes, one per 8-channel plane
  constexpr int PXW = SW32 ? 136 : 130;
  constexpr uint32_t PLANE_TX = SW32 ? PYH * PXW * 32 : PYH * PXW * 16;   // bytes one TMA load writes
  constexpr uint32_t PLANE = SW32 ? (PLANE_TX + 1023) / 1024 * 1024 : (PLANE_TX + 127) / 128 * 128;
  constexpr uint32_t LOADS = SW32 ? KS : 2;
  constexpr uint32_t SLOT = LOADS * PLANE;
  constexpr uint32_t BBLK = NN * 16 * 2;                     // B operand of one (dy, dx, K step)
  constexpr uint32_t SLAB0 = (NBLK * KS * BBLK + 1023) / 1024 * 1024;
  constexpr uint32_t ACOLS = (HEAD ? PYH : R) * NN;          // one accumulator slot (per output / input row)
  constexpr uint32_t TCOLS = NACC * ACOLS <= 256 ? 256 : 512;
  static_assert(NACC * ACOLS <= 512, "the accumulator slots fit the 512 TMEM columns");
  // layout: [B operands][S slots][mbarriers][tmem address][abort flag]
  unsigned char *Wb = smem;
  uint64_t *bars = reinterpret_cast<uint64_t *>(smem + SLAB0 + S * SLOT);
  uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(bars + 2 * S + 2 * NACC + 1);
  volatile int *abort_s = reinterpret_cast<volatile int *>(tmem_slot + 1);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const uint32_t wb_s = su32(Wb), slab_s = su32(smem + SLAB0), bar_s = su32(bars);
  auto full = [&](uint32_t k) { return bar_s + 8u * k; };                  // slab k loaded
  auto empty = [&](uint32_t k) { return bar_s + 8u * (S + k); };           // slab k's MMAs done
  auto tfull = [&](uint32_t k) { return bar_s + 8u * (2 * S + k); };       // accumulator slot k written
  auto tempty = [&](uint32_t k) { return bar_s + 8u * (2 * S + NACC + k); };   // accumulator slot k read
  const uint32_t fin = bar_s + 8u * (2 * S + 2 * NACC);

  // B operands: block (dy, dx, K step kh) holds B[n = dz*CO + co][k = ci - 16 kh] =
  // w[tap = dz*9 + dy*3 + dx][ci][co]; for the head, block (dx, kh) holds B[n = dz*3 + dy][k] =
  // w[tap = dz*9 + dy*3 + dx][ci][0] (n < 9, zero above); core matrix (n/8, k/8) at
  // (n/8)*256 + (k/8)*128, row n%8 at 16 B, element k%8 at 2 B
  for (int i = tid; i < NBLK * KS * NN; i += blockDim.x) {
    const int bk = i / NN, n = i % NN;
    const int blk = bk / KS, kh = bk % KS;
    const bool used = !HEAD || n < 9;
    const int tap = HEAD ? (n / 3) * 9 + (n % 3) * 3 + blk : (n / CO) * 9 + (X1 ? blk * 3 + 1 : blk);
    const int co = HEAD ? 0 : n % CO;
    uint32_t pk[8];
#pragma unroll
    for (int c = 0; c < 8; c++) {
      const int ci = kh * 16 + 2 * c;
      const unsigned short lo = used ? __bfloat16_as_ushort(p.w[((long long)tap * CI + ci) * CO + co]) : 0;
      const unsigned short hi = used ? __bfloat16_as_ushort(p.w[((long long)tap * CI + ci + 1) * CO + co]) : 0;
      pk[c] = (uint32_t)lo | ((uint32_t)hi << 16);
    }
    unsigned char *row = Wb + bk * BBLK + (n >> 3) * 256 + (n & 7) * 16;
    *reinterpret_cast<uint4 *>(row) = make_uint4(pk[0], pk[1], pk[2], pk[3]);
    *reinterpret_cast<uint4 *>(row + 128) = make_uint4(pk[4], pk[5], pk[6], pk[7]);
  }
  if (tid == 0) {
    for (int k = 0; k < S; k++) {
      net_mbar_init(full(k), 1);
      net_mbar_init(empty(k), NISS);
    }
    for (int k = 0; k < NACC; k++) {
      net_mbar_init(tfull(k), NISS);
      net_mbar_init(tempty(k), 256);
    }
    net_mbar_init(fin, NISS);
    *abort_s = 0;
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(su32(tmem_slot)),
                 "r"(TCOLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
  }
  asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");   // the B operands, for the tensor cores
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  auto decode = [&](long long it, int &b, int &zlo, int &nz, int &y0, int &x0) {
    long long q = it;
    x0 = (int)(q % g.xsegs) * 128;
    q /= g.xsegs;
    y0 = (int)(q % g.yblocks) * R;
    q /= g.yblocks;
    zlo = (int)(q % g.zchunks) * g.zc;
    b = (int)(q / g.zchunks);
    nz = min(p.Z - zlo, g.zc);
  };

  uint32_t nload = 0;
  if (warp == 0) {
    if (lane == 0) {
      // ---- producer: slabs zlo-1 .. zlo+nz of every item ----
      for (long long it = blockIdx.x; it < g.items && !*abort_s; it += gridDim.x) {
        int b, zlo, nz, y0, x0;
        decode(it, b, zlo, nz, y0, x0);
        for (int k = 0; k < nz + 2; k++) {
          const uint32_t slot = nload % S;
          if (nload >= S && !role_wait(empty(slot), ((nload / S) - 1) & 1, abort_s, 4)) break;
          net_expect_tx(full(slot), LOADS * PLANE_TX);
          const uint32_t dst = slab_s + slot * SLOT;
#pragma unroll
          for (int l = 0; l < (int)LOADS; l++)
            tma_load_5d(dst + l * PLANE, &tx, l * (SW32 ? 16 : 8), x0 - 1, y0 - 1, zlo - 1 + k, b, full(slot));
          nload++;
        }
      }
    }
  } else if (warp <= 2) {
    if (lane == 0 && warp <= NISS) {
      // ---- MMA issuers: warp 1 + j takes rows j*RR/NISS .. (j+1)*RR/NISS - 1 (output rows, or for
      // the head input rows) ----
      constexpr int RI = (HEAD ? PYH : R) / NISS;
      const int r0 = (warp - 1) * RI;
      // instruction descriptor: F32 accumulate, BF16 A and B, both K-major, N = 3 CO, M = 128
      const uint32_t idesc =
          (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(NN >> 3) << 17) | ((128u >> 4) << 24);
      const uint64_t b_desc = umma_desc(wb_s, 128, 256);
      const uint32_t b_lo = (uint32_t)b_desc, b_hi = (uint32_t)(b_desc >> 32);
      // A: slot 0, row 0.  SW32: K-major with the 32-byte swizzle (layout type 6 in bits 61-63),
      // 8-row groups 256 bytes apart, K within one swizzle row (leading offset unused, 16 bytes);
      // otherwise canonical no-swizzle, the two 8-channel planes one LBO apart
      const uint64_t a_desc = SW32 ? (umma_desc(slab_s, 16, 256) | (6ull << 61)) : umma_desc(slab_s, PLANE, 128);
      const uint32_t a_lo = (uint32_t)a_desc, a_hi = (uint32_t)(a_desc >> 32);
      constexpr uint32_t VOX = SW32 ? 2 : 1;   // one voxel in 16-byte units
      uint32_t n = 0;   // slabs consumed (= accumulator slots written)
      bool ok = true;
      uint32_t pre_full = 0, pre_empty = 0;   // the next slab's barriers, tested ahead
      for (long long it = blockIdx.x; it < g.items && ok; it += gridDim.x) {
        int b, zlo, nz, y0, x0;
        decode(it, b, zlo, nz, y0, x0);
        for (int k = 0; k < nz + 2; k++, n++) {
          const uint32_t acc = n % NACC;
          ok = (pre_full & pre_empty) ||
               (role_wait(full(n % S), (n / S) & 1, abort_s, 5) &&
                (n < NACC || role_wait(tempty(acc), ((n / NACC) - 1) & 1, abort_s, 6)));
          if (!ok) break;
          {
            // test slab n+1's barriers now, without blocking: the results are read at the next slab,
            // so their latency overlaps this slab's MMAs (a blocking wait follows only if a phase
            // was not yet complete).  A phase seen complete stays complete until this thread's own
            // commits let the slot be refilled.
            const uint32_t n1 = n + 1;
            pre_full = mbar_test(full(n1 % S), (n1 / S) & 1);
            pre_empty = n1 < NACC ? 1u : mbar_test(tempty(n1 % NACC), ((n1 / NACC) - 1) & 1);
          }
          const int zin = zlo - 1 + k;
          if (zin >= 0 && zin < p.Z) {
            tc_fence_after();
            // low descriptor word of the slab (start address >> 4 | LBO >> 4 << 16); a slab row of
            // PXW voxels is PXW * VOX units of 16 bytes
            const uint32_t al = a_lo + (n % S) * (SLOT >> 4);
            const uint32_t dcol = tmem + acc * ACOLS;
#pragma unroll
            for (int blk = 0; blk < NBLK; blk++) {
              // head: block dx, slab row = the input row; X1: block dy, dx = 1; otherwise block
              // (dy, dx), slab row r + dy
              const int dy = HEAD ? 0 : (X1 ? blk : blk / 3), dx = HEAD ? blk : (X1 ? 1 : blk % 3);
#pragma unroll
              for (int kh = 0; kh < KS; kh++) {
                const uint64_t bd = ((uint64_t)b_hi << 32) | (uint64_t)(b_lo + (blk * KS + kh) * (BBLK >> 4));
#pragma unroll
                for (int r = 0; r < RI; r++) {
                  const uint64_t ad = ((uint64_t)a_hi << 32) |
                                      (uint64_t)(al + kh * (PLANE >> 4) +
                                                 (uint32_t)(((r0 + r + dy) * PXW + dx) * VOX));
                  umma_f16(dcol + (r0 + r) * NN, ad, bd, idesc, (blk > 0 || kh > 0) ? 1u : 0u);
                }
              }
            }
          }
          umma_commit(tfull(acc));
          umma_commit(empty(n % S));   // the slab's shared memory is free
        }
      }
    }
  } else {
    // ---- epilogue: warps 3..10; warp w owns TMEM lane quarter w % 4 and output channels CH*hf .. ----
    const int qd = warp & 3, hf = (warp - 3) >> 2;
    const uint32_t lane_base = (uint32_t)(qd * 32) << 16;
    float bias[CH];
#pragma unroll
    for (int c = 0; c < CH; c++) bias[c] = (!HEAD && p.bias) ? p.bias[hf * CH + c] : 0.f;
    uint32_t n = 0;   // first slab of the current item
    bool ok = true;
    for (long long it = blockIdx.x; it < g.items && ok; it += gridDim.x) {
      int b, zlo, nz, y0, x0;
      decode(it, b, zlo, nz, y0, x0);
      const int x = x0 + qd * 32 + lane;
      float pacc[POOL ? CH : 1];   // POOL: the 2x2x2 average of the output, summed over a plane pair
      for (int i = 0; i < nz; i++) {
        // output plane z = zlo + i reads slabs n+i (dz 0), n+i+1 (dz 1), n+i+2 (dz 2); each issuer's
        // commits complete in order, so slab n+i+2's barrier covers the other two
        const uint32_t m = n + i + 2;
        // tcgen05.ld is .sync.aligned: the whole warp takes one decision
        if (!__all_sync(0xffffffffu, role_wait(tfull(m % NACC), (m / NACC) & 1, abort_s, 7) ? 1 : 0)) {
          ok = false;
          break;
        }
        tc_fence_after();
        const int z = zlo + i;
        const bool lo_in = z > 0, hi_in = z + 1 < p.Z;
        if constexpr (HEAD) {
          // out[z][y0 + r] = sum over (dz, dy) of column dz*3 + dy of input row r + dy of slab z-1+dz.
          // Channel half hf takes output rows hf*R/2 .. : input rows hf*R/2 .. hf*R/2 + R/2 + 1
          constexpr int RH = R / 2;
          static_assert(!HEAD || R % 2 == 0, "the head's rows split between the two warp halves");
          float o[RH];
#pragma unroll
          for (int r = 0; r < RH; r++) o[r] = 0.f;
          const int rb = hf * RH;
          // one plane's rows at a time (planes outside the volume had no MMAs: their slot holds
          // stale values, selected away); the column index is a constant in each call
          float v[RH + 2][16];
          auto rows = [&](int dz) {
            const uint32_t slot = tmem + lane_base + ((n + i + dz) % NACC) * ACOLS + rb * NN;
#pragma unroll
            for (int j = 0; j < RH + 2; j++) tmem_ld16(slot + j * NN, v[j]);
            asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
          };
          rows(0);
          head_rows<RH, 0>(o, v, lo_in);
          rows(1);
          head_rows<RH, 1>(o, v, true);
          rows(2);
          head_rows<RH, 2>(o, v, hi_in);
          tc_fence_before();
          net_arrive(tempty((n + i) % NACC));   // slab n+i has no later reader
          if (b < h.T && z < h.Zr && x < h.Xr) {
            const float sc = h.sum_x1[b] / h.count;
#pragma unroll
            for (int r = 0; r < RH; r++) {
              const int y = y0 + rb + r;
              if (y < h.Yr) h.x0[(((long long)z * h.T + b) * h.Yr + y) * h.Xr + x] = fmaxf(o[r] + h.bias, h.floor) * sc;
            }
          }
        } else {
          float d[R][3][CH];
#pragma unroll
          for (int r = 0; r < R; r++)
#pragma unroll
            for (int dz = 0; dz < 3; dz++) {
              const uint32_t a = tmem + lane_base + ((n + i + dz) % NACC) * ACOLS + r * NN + dz * CO + hf * CH;
              if constexpr (CH == 16) tmem_ld16(a, d[r][dz]);
              else tmem_ld8(a, d[r][dz]);
            }
          asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
          tc_fence_before();
          net_arrive(tempty((n + i) % NACC));   // slab n+i has no later reader
          uint4 kept[POOL ? R : 1];   // POOL: the BF16 outputs of this lane's rows
          if constexpr (POOL) {
#pragma unroll
            for (int r = 0; r < R; r++) kept[r] = make_uint4(0u, 0u, 0u, 0u);
          }
#pragma unroll
          for (int r = 0; r < R; r++) {
            const int y = y0 + r;
            float o[CH];
#pragma unroll
            for (int c = 0; c < CH; c++)
              o[c] = (lo_in ? d[r][0][c] : 0.f) + d[r][1][c] + (hi_in ? d[r][2][c] : 0.f);
            if (x >= p.X || y >= p.Y) continue;
            const long long off = ((((long long)b * p.Z + z) * p.Y + y) * p.X + x) * CO + hf * CH;
#pragma unroll
            for (int v = 0; v < CH / 8; v++) {
              uint4 mk;
              if (p.mask) mk = *reinterpret_cast<const uint4 *>(p.mask + off + v * 8);
              uint4 outv;
              __nv_bfloat162 *hv = reinterpret_cast<__nv_bfloat162 *>(&outv);
              const __nv_bfloat162 *m2 = reinterpret_cast<const __nv_bfloat162 *>(&mk);
#pragma unroll
              for (int k = 0; k < 4; k++) {
                float v0 = o[v * 8 + 2 * k] + bias[v * 8 + 2 * k];
                float v1 = o[v * 8 + 2 * k + 1] + bias[v * 8 + 2 * k + 1];
                if (p.relu) {
                  v0 = fmaxf(v0, 0.f);
                  v1 = fmaxf(v1, 0.f);
                }
                if (p.mask) {
                  const float2 mf = __bfloat1622float2(m2[k]);
                  if (!(mf.x > 0.f)) v0 = 0.f;
                  if (!(mf.y > 0.f)) v1 = 0.f;
                }
                hv[k] = __floats2bfloat162_rn(v0, v1);
              }
              *reinterpret_cast<uint4 *>(p.y + off + v * 8) = outv;
              if constexpr (POOL) kept[r] = outv;
            }
          }
          if constexpr (POOL) {
            // k_pool2's sum in its order: (y0, x), (y0, x+1), (y0+1, x), (y0+1, x+1) of plane 2zp,
            // then of plane 2zp+1, times 1/8; x+1 comes from the next lane (x0 and the item's first
            // plane are even, so lane pairs and plane pairs are pooling pairs)
            float pv[R][CH], nb[R][CH];
#pragma unroll
            for (int r = 0; r < R; r++) {
              const __nv_bfloat162 *k2 = reinterpret_cast<const __nv_bfloat162 *>(&kept[r]);
#pragma unroll
              for (int c = 0; c < CH / 2; c++) {
                const float2 f = __bfloat1622float2(k2[c]);
                pv[r][2 * c] = f.x;
                pv[r][2 * c + 1] = f.y;
              }
#pragma unroll
              for (int c = 0; c < CH; c++) nb[r][c] = __shfl_down_sync(0xffffffffu, pv[r][c], 1);
            }
            if ((i & 1) == 0) {
#pragma unroll
              for (int c = 0; c < CH; c++) pacc[c] = 0.f;
            }
#pragma unroll
            for (int c = 0; c < CH; c++) {
              pacc[c] += pv[0][c];
              pacc[c] += nb[0][c];
              pacc[c] += pv[1][c];
              pacc[c] += nb[1][c];
            }
            if ((i & 1) && !(lane & 1) && x < p.X && y0 < p.Y) {
              uint4 pw;
              __nv_bfloat162 *h2 = reinterpret_cast<__nv_bfloat162 *>(&pw);
#pragma unroll
              for (int c = 0; c < CH / 2; c++) h2[c] = __floats2bfloat162_rn(pacc[2 * c] * 0.125f, pacc[2 * c + 1] * 0.125f);
              const long long po =
                  ((((long long)b * (p.Z / 2) + (z >> 1)) * (p.Y / 2) + (y0 >> 1)) * (p.X / 2) + (x >> 1)) * CO + hf * CH;
              *reinterpret_cast<uint4 *>(p.pool + po) = pw;
            }
          }
        }
      }
      if (!ok) break;
      // the item's last two slabs have no later reader
      net_arrive(tempty((n + nz) % NACC));
      net_arrive(tempty((n + nz + 1) % NACC));
      n += nz + 2;
    }
  }

  __syncthreads();   // every role has left its loop (normally, or on an abort)
  if (warp == 0 && lane == 0 && *abort_s) {
    // copies still in flight land before the CTA exits: wait for the last load of every slot
    for (uint32_t sl = 0; sl < (uint32_t)S && sl < nload; sl++) {
      const uint32_t last = sl + ((nload - 1 - sl) / S) * S;
      if (!net_mbar_wait(full(sl), (last / S) & 1, 1000000000ULL)) atomicExch(&g_net_err, 8);
    }
  }
  if (warp >= 1 && warp <= NISS && lane == 0) {
    // every MMA issued has completed before the accumulators are released
    umma_commit(fin);
    if (!net_mbar_wait(fin, 0, 1000000000ULL)) atomicExch(&g_net_err, 9);
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(TCOLS) : "memory");
  }
}

// Weight gradient.  CTA = (voxel chunk, tap) x (ci tile CM, co tile CN); the 4
// warps take alternate k16 steps of its voxels (split-K) and are summed in
// shared memory at the end.  The tile goes to its chunk's slice of p.part,
// and k_wgrad_reduce adds the chunks to dW in chunk order, so the gradient is
// the same bits on every run; with one chunk (p.part null) the CTA adds its
// tile to dW itself (one writer per element).
template <int CM, int CN>
__global__ void __launch_bounds__(128) k_conv3d_wgrad(WgradParams p) {
  constexpr int BK = 64, NS = 3, RA = CM / 8, RBc = CN / 8;
  __shared__ __align__(128) bf16 Xs[NS][BK * CM];
  __shared__ __align__(128) bf16 Ds[NS][BK * CN];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const long long M = (long long)p.B * p.Z * p.Y * p.X;
  const int tap = blockIdx.x % 27;
  const long long chunk = blockIdx.x / 27;
  const int ctiles = p.Co / CN;
  const int ci0 = (blockIdx.y / ctiles) * CM, co0 = (blockIdx.y % ctiles) * CN;
  const long long v0 = chunk * p.chunk;
  const long long v1 = v0 + p.chunk < M ? v0 + p.chunk : M;
  const int dz = tap / 9 - 1, dy = (tap / 3) % 3 - 1, dx = tap % 3 - 1;
  const int KS = (int)((v1 - v0 + BK - 1) / BK);

  auto load = [&](int ks, int st) {
    for (int i = tid; i < BK * (RA + RBc); i += 128) {
      const int row = i / (RA + RBc), c = i - row * (RA + RBc);
      const long long vv = v0 + (long long)ks * BK + row;
      const bool in = vv < v1;
      if (c < RA) {
        bool ok = false;
        const bf16 *src = p.x;
        if (in) {
          const Vox q = decode(vv, p.Z, p.Y, p.X);
          const int z = q.z + dz, y = q.y + dy, x = q.x + dx;
          ok = z >= 0 && z < p.Z && y >= 0 && y < p.Y && x >= 0 && x < p.X;
          if (ok) src = p.x + ((((long long)q.b * p.Z + z) * p.Y + y) * p.X + x) * p.Ci + ci0 + c * 8;
        }
        cp16(su32(&Xs[st][row * CM]) + ((c ^ swz<RA>(row)) << 4), src, ok);
      } else {
        const int cc = c - RA;
        const bf16 *src = in ? p.dy + vv * p.Co + co0 + cc * 8 : p.dy;
        cp16(su32(&Ds[st][row * CN]) + ((cc ^ swz<RBc>(row)) << 4), src, in);
      }
    }
  };

  float acc[CM / 16][CN / 8][4];
#pragma unroll
  for (int i = 0; i < CM / 16; i++)
#pragma unroll
    for (int j = 0; j < CN / 8; j++)
#pragma unroll
      for (int e = 0; e < 4; e++) acc[i][j][e] = 0.f;

#pragma unroll
  for (int s = 0; s < NS - 1; s++) {
    if (s < KS) load(s, s);
    cp_commit();
  }
  const int mat = lane >> 3, r8 = lane & 7;
  for (int ks = 0; ks < KS; ks++) {
    cp_wait<NS - 2>();
    __syncthreads();
    const int st = ks % NS;
    const int kr = warp * 16;   // this warp's 16 voxels of the stage
    uint32_t a[CM / 16][4];
#pragma unroll
    for (int mt = 0; mt < CM / 16; mt++) {
      // A[ci][k] from Xs[k][ci]: transposed 8x8 blocks (k rows, ci chunk)
      const int row = kr + r8 + 8 * (mat >> 1);
      const int c = mt * 2 + (mat & 1);
      ldsm4t(su32(&Xs[st][row * CM]) + ((c ^ swz<RA>(row)) << 4), a[mt][0], a[mt][1], a[mt][2], a[mt][3]);
    }
#pragma unroll
    for (int n2 = 0; n2 < CN / 16; n2++) {
      const int row = kr + r8 + 8 * (mat & 1);
      const int c = n2 * 2 + (mat >> 1);
      uint32_t b0, b1, b2, b3;
      ldsm4t(su32(&Ds[st][row * CN]) + ((c ^ swz<RBc>(row)) << 4), b0, b1, b2, b3);
#pragma unroll
      for (int mt = 0; mt < CM / 16; mt++) {
        mma_bf16(acc[mt][2 * n2], a[mt], b0, b1);
        mma_bf16(acc[mt][2 * n2 + 1], a[mt], b2, b3);
      }
    }
    const int nk = ks + NS - 1;
    if (nk < KS) load(nk, nk % NS);
    cp_commit();
  }
  cp_wait<0>();
  __syncthreads();
  // sum the 4 warps' partial tiles in shared memory (reuses the ring)
  float *red = reinterpret_cast<float *>(&Xs[0][0]);
  static_assert(sizeof(Xs) >= sizeof(float) * CM * CN, "reduction buffer");
  for (int i = tid; i < CM * CN; i += 128) red[i] = 0.f;
  __syncthreads();
  for (int w = 0; w < 4; w++) {
    if (warp == w) {
#pragma unroll
      for (int mt = 0; mt < CM / 16; mt++)
#pragma unroll
        for (int nt = 0; nt < CN / 8; nt++)
#pragma unroll
          for (int e = 0; e < 4; e++) {
            const int ci = mt * 16 + (lane >> 2) + 8 * (e >> 1);
            const int co = nt * 8 + 2 * (lane & 3) + (e & 1);
            red[ci * CN + co] += acc[mt][nt][e];
          }
    }
    __syncthreads();
  }
  const long long nw = 27LL * p.Ci * p.Co;
  for (int i = tid; i < CM * CN; i += 128) {
    const int ci = i / CN, co = i - ci * CN;
    const long long o = ((long long)tap * p.Ci + ci0 + ci) * p.Co + co0 + co;
    if (p.part) p.part[chunk * nw + o] = red[i];
    else p.dw[o] += red[i];
  }
}

// dw[i] += sum over the chunks of part[chunk][i], in chunk order.
__global__ void k_wgrad_reduce(const float *part, float *dw, long long n, int chunks) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    float s = 0.f;
    for (int c = 0; c < chunks; c++) s += part[(long long)c * n + i];
    dw[i] += s;
  }
}

// w2[26 - tap][co][ci] = w[tap][ci][co]: the data-gradient convolution's weights.
__global__ void k_conv3d_flip_weights(const bf16 *w, bf16 *w2, int Ci, int Co) {
  const long long n = 27LL * Ci * Co;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const int co = (int)(i % Co);
    const long long t = i / Co;
    const int ci = (int)(t % Ci), tap = (int)(t / Ci);
    w2[((long long)(26 - tap) * Co + co) * Ci + ci] = w[i];
  }
}

// Sums over rows of g[M][C], one row block per CTA: into part[block][c] (then
// k_bias_reduce adds the blocks in order), or with a single block (part null)
// straight into db[c].
__global__ void k_bias_grad(const bf16 *g, float *db, float *part, long long M, int C, long long rows_per_block) {
  const int c = threadIdx.x;
  if (c >= C) return;
  const long long r0 = (long long)blockIdx.x * rows_per_block;
  const long long r1 = r0 + rows_per_block < M ? r0 + rows_per_block : M;
  float s = 0.f;
  for (long long r = r0; r < r1; r++) s += __bfloat162float(g[r * C + c]);
  if (part) part[(long long)blockIdx.x * C + c] = s;
  else db[c] += s;
}

__global__ void k_bias_reduce(const float *part, float *db, int blocks, int C) {
  const int c = threadIdx.x;
  if (c >= C) return;
  float s = 0.f;
  for (int b = 0; b < blocks; b++) s += part[(long long)b * C + c];
  db[c] += s;
}

// Epilogue of a split convolution: y = act(ws + bias) (* (mask > 0)), 8 channels per thread.
__global__ void k_conv3d_finish(ConvParams p, long long M) {
  const int G = p.Co / 8;
  const long long n = M * G;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const int c0 = (int)(i % G) * 8;
    const long long o = (i / G) * p.Co + c0;
    float v[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    for (int sp = 0; sp < p.splits; sp++) {   // the K slices in order
      const float *src = p.ws + (long long)sp * M * p.Co + o;
      const float4 a = *reinterpret_cast<const float4 *>(src);
      const float4 b = *reinterpret_cast<const float4 *>(src + 4);
      v[0] += a.x; v[1] += a.y; v[2] += a.z; v[3] += a.w;
      v[4] += b.x; v[5] += b.y; v[6] += b.z; v[7] += b.w;
    }
    uint4 mk;
    if (p.mask) mk = *reinterpret_cast<const uint4 *>(p.mask + o);
    const __nv_bfloat162 *m2 = reinterpret_cast<const __nv_bfloat162 *>(&mk);
    uint4 u;
    __nv_bfloat162 *h = reinterpret_cast<__nv_bfloat162 *>(&u);
#pragma unroll
    for (int k = 0; k < 4; k++) {
      float v0 = v[2 * k] + (p.bias ? p.bias[c0 + 2 * k] : 0.f);
      float v1 = v[2 * k + 1] + (p.bias ? p.bias[c0 + 2 * k + 1] : 0.f);
      if (p.relu) {
        v0 = fmaxf(v0, 0.f);
        v1 = fmaxf(v1, 0.f);
      }
      if (p.mask) {
        const float2 mf = __bfloat1622float2(m2[k]);
        if (!(mf.x > 0.f)) v0 = 0.f;
        if (!(mf.y > 0.f)) v1 = 0.f;
      }
      h[k] = __floats2bfloat162_rn(v0, v1);
    }
    *reinterpret_cast<uint4 *>(p.y + o) = u;
  }
}

// 8 BF16 channels as one 16-byte vector.
struct V8 {
  float v[8];
  __device__ __forceinline__ void load(const bf16 *p) {
    const uint4 u = *reinterpret_cast<const uint4 *>(p);
    const __nv_bfloat162 *h = reinterpret_cast<const __nv_bfloat162 *>(&u);
#pragma unroll
    for (int k = 0; k < 4; k++) {
      const float2 f = __bfloat1622float2(h[k]);
      v[2 * k] = f.x;
      v[2 * k + 1] = f.y;
    }
  }
  __device__ __forceinline__ void store(bf16 *p) const {
    uint4 u;
    __nv_bfloat162 *h = reinterpret_cast<__nv_bfloat162 *>(&u);
#pragma unroll
    for (int k = 0; k < 4; k++) h[k] = __floats2bfloat162_rn(v[2 * k], v[2 * k + 1]);
    *reinterpret_cast<uint4 *>(p) = u;
  }
};

__device__ __forceinline__ long long half_index(const Vox &v, int Z, int Y, int X, int C) {
  return ((((long long)v.b * (Z / 2) + v.z / 2) * (Y / 2) + v.y / 2) * (X / 2) + v.x / 2) * C;
}

// out[b][z][y][x][c] = mean of the 2x2x2 block of in (Z, Y, X even); one thread
// per output voxel and 8 channels.
__global__ void k_pool2(const bf16 *in, bf16 *out, int B, int Z, int Y, int X, int C) {
  const int Zo = Z / 2, Yo = Y / 2, Xo = X / 2, G = C / 8;
  const long long n = (long long)B * Zo * Yo * Xo * G;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const int g = (int)(i % G);
    const Vox o = decode(i / G, Zo, Yo, Xo);
    V8 acc;
#pragma unroll
    for (int k = 0; k < 8; k++) acc.v[k] = 0.f;
    for (int d = 0; d < 8; d++) {
      V8 q;
      q.load(in + ((((long long)o.b * Z + 2 * o.z + (d >> 2)) * Y + 2 * o.y + ((d >> 1) & 1)) * X + 2 * o.x + (d & 1)) *
                      C + g * 8);
#pragma unroll
      for (int k = 0; k < 8; k++) acc.v[k] += q.v[k];
    }
#pragma unroll
    for (int k = 0; k < 8; k++) acc.v[k] *= 0.125f;
    acc.store(out + (i / G) * C + g * 8);
  }
}

// Adjoint of k_pool2 plus a second gradient, under a ReLU mask:
// gin[v] = (gpool[v/2] / 8 + gskip[v]) * (act[v] > 0)   (gskip, act may be null)
__global__ void k_pool2_bwd(const bf16 *gpool, const bf16 *gskip, const bf16 *act, bf16 *gin, int B, int Z, int Y,
                            int X, int C) {
  const int G = C / 8;
  const long long n = (long long)B * Z * Y * X * G;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const int g = (int)(i % G);
    const long long vox = i / G;
    const Vox v = decode(vox, Z, Y, X);
    V8 r, q;
    r.load(gpool + half_index(v, Z, Y, X, C) + g * 8);
#pragma unroll
    for (int k = 0; k < 8; k++) r.v[k] *= 0.125f;
    if (gskip) {
      q.load(gskip + vox * C + g * 8);
#pragma unroll
      for (int k = 0; k < 8; k++) r.v[k] += q.v[k];
    }
    if (act) {
      q.load(act + vox * C + g * 8);
#pragma unroll
      for (int k = 0; k < 8; k++)
        if (!(q.v[k] > 0.f)) r.v[k] = 0.f;
    }
    r.store(gin + vox * C + g * 8);
  }
}

// out[v] = low[v/2] + skip[v]  (nearest 2x2x2 upsampling; low has C channels)
// One CTA per output row (b, z, y): the row's coordinates are decoded once and
// the threads walk its X * C / 8 vectors of 8 channels (C / 8 a power of two),
// so the per-vector index work is a shift and a mask.
__global__ void k_up2_add(const bf16 *low, const bf16 *skip, bf16 *out, int B, int Z, int Y, int X, int C) {
  const int G = C / 8, gsh = __ffs(G) - 1;
  const long long row = blockIdx.x;                    // (b * Z + z) * Y + y
  const int y = (int)(row % Y);
  const long long bz = row / Y;
  const int z = (int)(bz % Z), b = (int)(bz / Z);
  const bf16 *lrow = low + ((((long long)b * (Z / 2) + z / 2) * (Y / 2) + y / 2) * (long long)(X / 2)) * C;
  const long long o = row * X * C;
  for (int i = threadIdx.x; i < X * G; i += blockDim.x) {
    const int x = i >> gsh, g = i & (G - 1);
    V8 r, q;
    r.load(lrow + (long long)(x >> 1) * C + g * 8);
    if (skip) {
      q.load(skip + o + (long long)i * 8);
#pragma unroll
      for (int k = 0; k < 8; k++) r.v[k] += q.v[k];
    }
    r.store(out + o + (long long)i * 8);
  }
}

// Adjoint of the upsampling: glow[u] = sum of g over its 2x2x2 block, times (act[u] > 0)
__global__ void k_up2_bwd(const bf16 *g, const bf16 *act, bf16 *glow, int B, int Z, int Y, int X, int C) {
  const int Zo = Z / 2, Yo = Y / 2, Xo = X / 2, G = C / 8;
  const long long n = (long long)B * Zo * Yo * Xo * G;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const int gi = (int)(i % G);
    const Vox o = decode(i / G, Zo, Yo, Xo);
    V8 acc, q;
#pragma unroll
    for (int k = 0; k < 8; k++) acc.v[k] = 0.f;
    for (int d = 0; d < 8; d++) {
      q.load(g + ((((long long)o.b * Z + 2 * o.z + (d >> 2)) * Y + 2 * o.y + ((d >> 1) & 1)) * X + 2 * o.x + (d & 1)) *
                     C + gi * 8);
#pragma unroll
      for (int k = 0; k < 8; k++) acc.v[k] += q.v[k];
    }
    if (act) {
      q.load(act + (i / G) * C + gi * 8);
#pragma unroll
      for (int k = 0; k < 8; k++)
        if (!(q.v[k] > 0.f)) acc.v[k] = 0.f;
    }
    acc.store(glow + (i / G) * C + gi * 8);
  }
}

// Prediction = channel 0 of y (C channels); loss terms and the gradient of
// mean((pred - target)^2) into channel 0 of g (other channels 0).
__global__ void k_mse_grad(const bf16 *y, const float *target, bf16 *g, float *loss, long long M, int C) {
  float s = 0.f;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < M; i += (long long)gridDim.x * blockDim.x) {
    const float d = __bfloat162float(y[i * C]) - target[i];
    s += d * d;
    g[i * C] = __float2bfloat16_rn(2.f * d / (float)M);
    for (int c = 1; c < C; c++) g[i * C + c] = __float2bfloat16_rn(0.f);
  }
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) atomicAdd(loss, s / (float)M);
}

// Adam on FP32 master weights; writes the BF16 copy the kernels read.
__global__ void k_adam(float *w, const float *g, float *m, float *v, bf16 *wb, long long n, float lr, float b1,
                       float b2, float eps, float c1, float c2, float wd) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const float gi = g[i] + wd * w[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    const float wi = w[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    w[i] = wi;
    if (wb) wb[i] = __float2bfloat16_rn(wi);
  }
}

// Gaussian blobs: vol[z][y][x] += amp exp(-|p - c|^2 / (2 sigma^2)) within 3 sigma;
// pts[k] = (z, y, x, amp), one warp per blob.  With acc (an int64 per voxel,
// zeroed) the terms are added as 32.32 fixed-point integers, whose sum does
// not depend on the order the warps arrive in; k_blobs_add then adds the
// totals to vol.  Without acc they go to vol through FP32 atomics.
__global__ void k_render_blobs(float *vol, unsigned long long *acc, int Z, int Y, int X, const float4 *pts, int npts,
                               float sigma) {
  const int k = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (k >= npts) return;
  const float4 q = pts[k];
  const int r = (int)ceilf(3.f * sigma);
  const int w = 2 * r + 1;
  const float inv = 1.f / (2.f * sigma * sigma);
  for (int t = lane; t < w * w * w; t += 32) {
    const int dz = t / (w * w) - r, dy = (t / w) % w - r, dx = t % w - r;
    const int z = (int)floorf(q.x + 0.5f) + dz, y = (int)floorf(q.y + 0.5f) + dy, x = (int)floorf(q.z + 0.5f) + dx;
    if (z < 0 || z >= Z || y < 0 || y >= Y || x < 0 || x >= X) continue;
    const float d2 = (z - q.x) * (z - q.x) + (y - q.y) * (y - q.y) + (x - q.z) * (x - q.z);
    const float v = q.w * __expf(-d2 * inv);
    const long long o = ((long long)z * Y + y) * X + x;
    if (acc) atomicAdd(acc + o, (unsigned long long)__double2ll_rn((double)v * 4294967296.0));
    else atomicAdd(vol + o, v);
  }
}

__global__ void k_blobs_add(float *vol, const unsigned long long *acc, long long n) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    vol[i] += (float)((double)(long long)acc[i] * (1.0 / 4294967296.0));
}

// Frame sums of the first RL iterate Htf / HtH1 (Htf [Z][T][Y][X], HtH1 [Z][Y][X]):
// one partial per (block, frame) into part[t][block]; k_ws_sum_final adds them
// in block order.
__global__ void __launch_bounds__(256) k_ws_sum(const float *htf, const float *hth1, float *partial, int T,
                                                long long V, long long YX) {
  __shared__ float red[8];
  const int t = blockIdx.y;
  const int Z = (int)(V / YX);
  float part = 0.f;
  // a thread owns pixels yx (strided over the grid) of every plane: no division per element
  for (long long yx = (long long)blockIdx.x * blockDim.x + threadIdx.x; yx < YX; yx += (long long)gridDim.x * blockDim.x)
    for (int z = 0; z < Z; z++) part += htf[((long long)z * T + t) * YX + yx] / hth1[(long long)z * YX + yx];
  for (int o = 16; o > 0; o >>= 1) part += __shfl_down_sync(0xffffffffu, part, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = part;
  __syncthreads();
  if (threadIdx.x == 0) {
    float b = 0.f;
    for (int w = 0; w < 8; w++) b += red[w];
    partial[(long long)t * gridDim.x + blockIdx.x] = b;
  }
}

__global__ void k_ws_sum_final(const float *part, float *sum, int T, int blocks) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= T) return;
  float s = 0.f;
  for (int b = 0; b < blocks; b++) s += part[(long long)t * blocks + b];
  sum[t] = s;
}

// Network input, channels-last [T][Zp][Yp][Xp][16] from Htf [Z][T][Y][X]: with
// the features f0 = Htf / HtH1 / m[t] (the first RL iterate over its frame
// mean m), f1 = Htf / Ht1 / m[t], f2 = HtH1 * c2, f3 = Ht1 * c3, channel 4k + j
// (k = 0..2) holds f_j at x + k - 1, so that the first layer's x taps are
// channels and it runs as a 3x3x1 convolution; 12..15 = 0; zero in the padding.
// One CTA per padded output row (t, z, y), its coordinates decoded once; the
// threads walk x.
__global__ void __launch_bounds__(256) k_ws_input(WsInputParams p) {
  const long long row = blockIdx.x;                    // ((t * Zp) + z) * Yp + y
  const int y = (int)(row % p.Yp);
  const long long tz = row / p.Yp;
  const int z = (int)(tz % p.Zp), t = (int)(tz / p.Zp);
  for (int x = threadIdx.x; x < p.Xp; x += blockDim.x) {
    const long long i = row * p.Xp + x;
    __nv_bfloat162 c[8];
    for (int k = 0; k < 8; k++) c[k] = __floats2bfloat162_rn(0.f, 0.f);
    if (z < p.Z && y < p.Y) {
      const float inv = p.count / fmaxf(p.sum_x1[t], 1e-30f);
#pragma unroll
      for (int k = 0; k < 3; k++) {
        const int xs = x + k - 1;
        if (xs < 0 || xs >= p.X) continue;
        const long long v = ((long long)z * p.Y + y) * p.X + xs;
        const float h = p.htf[(((long long)z * p.T + t) * p.Y + y) * p.X + xs];
        const float a = p.hth1[v], b = p.ht1[v];
        c[2 * k] = __floats2bfloat162_rn(h / a * inv, h / b * inv);
        c[2 * k + 1] = __floats2bfloat162_rn(a * p.c2, b * p.c3);
      }
    }
    uint4 *dst = reinterpret_cast<uint4 *>(p.out + i * 16);
    dst[0] = *reinterpret_cast<uint4 *>(&c[0]);
    dst[1] = *reinterpret_cast<uint4 *>(&c[4]);
  }
}

static unsigned grid_for(long long n, int block) {
  long long g = (n + block - 1) / block;
  return (unsigned)(g < 152LL * 32 ? (g < 1 ? 1 : g) : 152LL * 32);
}

template <int CI, int CO>
static cudaError_t launch_tiled(const ConvParams &p, cudaStream_t s) {
  static int grid_cap = 0;
  const size_t smem = sizeof(bf16) * (27 * CI * CO + 540 * CI);
  if (!grid_cap) {
    cudaError_t e = cudaFuncSetAttribute(k_conv3d_tiled<CI, CO>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    if (e != cudaSuccess) return e;
    int per_sm = 0, dev = 0, sms = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_conv3d_tiled<CI, CO>, 128, smem);
    if (e != cudaSuccess) return e;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    grid_cap = (per_sm > 0 ? per_sm : 1) * (sms > 0 ? sms : 1);
  }
  const int tiles_x = (p.X + 15) / 16, tiles_y = (p.Y + 7) / 8;
  const long long ntiles = (long long)p.B * p.Z * tiles_y * tiles_x;
  const unsigned grid = (unsigned)(ntiles < grid_cap ? ntiles : grid_cap);
  FLF_NET_LAUNCH(k_conv3d_tiled<CI, CO><<<grid, 128, smem, s>>>(p, tiles_x, tiles_y, ntiles));
  return cudaGetLastError();
}

template <bool HEAD>
static cudaError_t launch_t16(const ConvParams &p, const HeadOut &h, cudaStream_t s) {
  static int grid_cap = 0;
  const size_t smem = sizeof(bf16) * (27 * 16 * 16 + 972 * 16);
  if (!grid_cap) {
    cudaError_t e = cudaFuncSetAttribute(k_conv3d_t16<HEAD>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    int per_sm = 0, dev = 0, sms = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_conv3d_t16<HEAD>, 128, smem);
    if (e != cudaSuccess) return e;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    grid_cap = (per_sm > 0 ? per_sm : 1) * (sms > 0 ? sms : 1);
  }
  const int tiles_x = (p.X + 15) / 16, tiles_y = (p.Y + 15) / 16;
  const long long ntiles = (long long)p.B * p.Z * tiles_y * tiles_x;
  const unsigned grid = (unsigned)(ntiles < grid_cap ? ntiles : grid_cap);
  FLF_NET_LAUNCH(k_conv3d_t16<HEAD><<<grid, 128, smem, s>>>(p, h, tiles_x, tiles_y, ntiles));
  return cudaGetLastError();
}

// cuTensorMapEncodeTiled through the runtime's driver entry point (no link to libcuda)
static PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  if (!fn) {
    void *f = nullptr;
    cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(f);
  }
  return fn;
}

template <int CI, int CO, int R, int S, bool HEAD, bool SW32, bool X1 = false, bool POOL = false>
static cudaError_t launch_tma16(const ConvParams &p, const HeadOut &h, cudaStream_t s) {
  constexpr int KS = CI / 16;
  constexpr size_t SLOT = SW32 ? KS * (((R + 2) * 136 * 32 + 1023) / 1024 * 1024)
                               : 2 * (((R + 2) * 130 * 16 + 127) / 128 * 128);
  constexpr size_t SMEM =
      (9 * KS * 3 * CO * 32 + 1023) / 1024 * 1024 + S * SLOT + (2 * S + 2 * TMA16_NACC + 1) * 8 + 8;
  static_assert(SMEM <= 227 * 1024, "shared memory of one CTA");
  static int sms = 0;
  if (!sms) {
    cudaError_t e = cudaFuncSetAttribute(k_conv3d_tma16<CI, CO, R, S, HEAD, SW32, X1, POOL>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMEM);
    if (e != cudaSuccess) return e;
    int dev = 0, n = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    sms = n > 0 ? n : 1;
  }
  const long long M = (long long)p.B * p.Z * p.Y * p.X;
  if (M == 0) return cudaSuccess;
  PFN_cuTensorMapEncodeTiled_v12000 enc = tensor_map_encoder();
  if (!enc) return cudaErrorNotSupported;
  if (reinterpret_cast<uintptr_t>(p.x) % 16) return cudaErrorMisalignedAddress;
  // [B][Z][Y][X][CI] BF16, innermost first; one box = 16 channels (SW32) or one 8-channel plane of a slab
  CUtensorMap map;
  const cuuint64_t vb = 2ull * CI;   // bytes per voxel
  const cuuint64_t dims[5] = {(cuuint64_t)CI, (cuuint64_t)p.X, (cuuint64_t)p.Y, (cuuint64_t)p.Z, (cuuint64_t)p.B};
  const cuuint64_t strides[4] = {vb, vb * p.X, vb * p.X * p.Y, vb * p.X * p.Y * p.Z};
  const cuuint32_t box[5] = {SW32 ? 16u : 8u, SW32 ? 136u : 130u, (cuuint32_t)(R + 2), 1, 1};
  const cuuint32_t estr[5] = {1, 1, 1, 1, 1};
  if (enc(&map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 5, const_cast<bf16 *>(p.x), dims, strides, box, estr,
          CU_TENSOR_MAP_INTERLEAVE_NONE, SW32 ? CU_TENSOR_MAP_SWIZZLE_32B : CU_TENSOR_MAP_SWIZZLE_NONE,
          CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
          CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
    return cudaErrorInvalidValue;
  Tma16Grid g;
  g.xsegs = (p.X + 127) / 128;
  g.yblocks = (p.Y + R - 1) / R;
  // split z into chunks when whole columns fill the GPU unevenly (each chunk reloads 2 halo slabs)
  long long best = -1;
  int zc_best = p.Z;
  for (int c = 1; c <= 8 && c <= p.Z; c++) {
    int zc = (p.Z + c - 1) / c;
    if (POOL) zc += zc & 1;   // plane pairs stay in one item
    const long long items = (long long)p.B * ((p.Z + zc - 1) / zc) * g.yblocks * g.xsegs;
    const long long cost = (items + sms - 1) / sms * (zc + 2);
    if (best < 0 || cost < best) {
      best = cost;
      zc_best = zc;
    }
  }
  g.zc = zc_best;
  g.zchunks = (p.Z + g.zc - 1) / g.zc;
  g.items = (long long)p.B * g.zchunks * g.yblocks * g.xsegs;
  const unsigned grid = (unsigned)(g.items < sms ? g.items : sms);
  FLF_NET_LAUNCH(k_conv3d_tma16<CI, CO, R, S, HEAD, SW32, X1, POOL><<<grid, 352, SMEM, s>>>(map, p, h, g));
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Wide layers (32..128 channels in and out, at least one side 64 or more) on
// tcgen05, as an implicit GEMM over "padded rows".  A work item is one output
// plane z of one volume b and a block of R rows y0 .. y0+R-1.  Input slabs
// (R+2 rows x Xp = X+2 voxels, the halo included, zeros outside the volume)
// arrive by TMA in the canonical no-swizzle K-major layout: one 16-byte row
// per voxel and 8 channels, the 8-channel groups LBO apart.  In such a slab
// the voxel at (row r, column c) is row r*Xp + c, so for output position
// q = r*Xp + x (x < Xp) the tap (dy, dx) is slab row q + dy*Xp + dx: every
// tap's A operand is the slab seen from another start row, a legal operand
// address (16-byte aligned).  An item's M = nM x 128 positions q cover its R
// rows (positions with x >= X or beyond the R rows are computed and dropped).
//   chunk = one input plane z+dz x KC (<= 64) input channels: KC/8 TMA loads
//           into one of 2 slab slots;
//   B     = the KC/16 blocks of one (tap, chunk) of the packed weights
//           (flf_conv3d_pack: per 16 input channels a [2 k8][CO][8] BF16
//           block), one 1-D bulk copy per ring slot;
//   MMA   = M 128 x N CO x K 16, nM per B block, into one of 2 TMEM
//           accumulator buffers (nM x CO <= 256 columns each); the issuing
//           thread moves only the start-address words of the descriptors.
//   warp 0      slab producer (one thread);
//   warp 1      MMA issuer (one thread), TMEM allocation;
//   warp 2      B producer (one thread);
//   warps 4-7   epilogue: warp w reads TMEM lanes 32 (w % 4) .. +31 of every
//               M tile, adds the bias, ReLU / mask, stores BF16.
// Items are dealt round-robin to persistent CTAs (one per SM); the epilogue of
// an item overlaps the MMAs of the next.  Every mbarrier wait is bounded; a
// give-up sets g_net_err and a shared abort flag, and the CTA drains its copies
// and MMAs before TMEM is released.
// ---------------------------------------------------------------------------
struct WideGrid {
  int Xp, R, nM, nyb;   // padded row, rows per item, M tiles per item, y blocks
  int slab_rows;        // rows of one 8-channel group of a slab slot (LBO / 16)
  int sb;               // B ring slots (the shared memory the slabs leave)
  int tps;              // taps per B ring slot (3: a row of dx taps, one wait and one commit)
  int splits;           // 1, or 3: work unit = (item, input plane z-1+s) writing FP32 partials to ws[s]
  long long items;      // B * Z * nyb * splits (work units)
};

constexpr int WIDE_SB_MAX = 64;      // B block ring: barriers for at most this many blocks
constexpr int WIDE_SB = 12;          // taps of B blocks in flight at most
constexpr int WIDE_ACC_COLS = 256;   // columns of one TMEM accumulator buffer

template <int CI, int CO>
__global__ void __launch_bounds__(256, 1)
    k_conv3d_wide(const __grid_constant__ CUtensorMap tx, ConvParams p, const bf16 *__restrict__ wp, WideGrid g) {
  extern __shared__ __align__(1024) unsigned char smem[];
  constexpr int KC = CI < 64 ? CI : 64;   // input channels of one chunk
  constexpr int NCG = CI / KC;            // chunks per input plane
  constexpr bool SW = KC == 64;           // 128-byte rows, 128-byte swizzle (else 8-channel groups)
  constexpr int NBOX = SW ? 1 : KC / 8;   // TMA loads per chunk
  constexpr int KS = KC / 16;             // K steps per chunk
  constexpr uint32_t BBLK = 32u * CO;     // one packed B block
  static_assert(CI % 32 == 0 && CO % 32 == 0 && CO <= 128 && CI <= 128, "32..128 channels");
  // SW: a slab slot is slab_rows rows of 128 bytes (64 channels), written by one TMA load with the
  // 128-byte swizzle; otherwise KC/8 groups of slab_rows 16-byte rows, LBO apart
  const uint32_t LBO = (uint32_t)g.slab_rows * 16u;
  const uint32_t SLOT = SW ? (uint32_t)g.slab_rows * 128u : (uint32_t)(KC / 8) * LBO;
  const uint32_t box_tx = (SW ? 128u : 16u) * (uint32_t)g.Xp * (uint32_t)(g.R + 2);
  // layout: [2 slab slots][B ring][mbarriers][tmem address][abort flag]
  const uint32_t smem_s = su32(smem);
  const uint32_t slab_s = smem_s, bring_s = smem_s + 2 * SLOT;
  const uint32_t SB = (uint32_t)g.sb;          // B ring slots
  constexpr uint32_t TB = KS * BBLK;            // one tap's B blocks (KC input channels)
  const int TPS = g.tps;                        // taps per slot
  const uint32_t SLOTB = (uint32_t)TPS * TB;
  uint64_t *bars = reinterpret_cast<uint64_t *>(smem + 2 * SLOT + SB * SLOTB);
  uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(bars + 4 + 2 * WIDE_SB_MAX + 4 + 1);
  volatile int *abort_s = reinterpret_cast<volatile int *>(tmem_slot + 1);
  const uint32_t bar_s = su32(bars);
  auto sfull = [&](uint32_t k) { return bar_s + 8u * k; };                           // slab slot loaded
  auto sempty = [&](uint32_t k) { return bar_s + 8u * (2 + k); };                    // slab slot read
  auto bfull = [&](uint32_t k) { return bar_s + 8u * (4 + k); };                     // B block loaded
  auto bempty = [&](uint32_t k) { return bar_s + 8u * (4 + WIDE_SB_MAX + k); };      // B block read
  auto afull = [&](uint32_t k) { return bar_s + 8u * (4 + 2 * WIDE_SB_MAX + k); };   // accumulator done
  auto aempty = [&](uint32_t k) { return bar_s + 8u * (6 + 2 * WIDE_SB_MAX + k); };  // accumulator read
  const uint32_t fin = bar_s + 8u * (8 + 2 * WIDE_SB_MAX);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const long long Mv = (long long)p.B * p.Z * p.Y * p.X;   // voxels (the stride of a partial-sum slice)

  if (tid == 0) {
    for (int k = 0; k < 2; k++) {
      net_mbar_init(sfull(k), 1);
      net_mbar_init(sempty(k), 1);
      net_mbar_init(afull(k), 1);
      net_mbar_init(aempty(k), 4);
    }
    for (uint32_t k = 0; k < SB; k++) {
      net_mbar_init(bfull(k), 1);
      net_mbar_init(bempty(k), 1);
    }
    net_mbar_init(fin, 1);
    *abort_s = 0;
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");   // visible to TMA and the MMAs
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(su32(tmem_slot)),
                 "r"(2 * WIDE_ACC_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  // work unit it -> volume b, output plane z, first row y0 and, with splits, the one input
  // plane offset dz1 (-1..1) it covers (splits == 1: all three, dz1 = 2)
  auto decode = [&](long long it, int &b, int &z, int &y0, int &dz1) {
    long long q = it;
    dz1 = 2;
    if (g.splits > 1) {
      dz1 = (int)(q % g.splits) - 1;
      q /= g.splits;
    }
    const int yb = (int)(q % g.nyb);
    q /= g.nyb;
    z = (int)(q % p.Z);
    b = (int)(q / p.Z);
    y0 = yb * g.R;
  };
  // the input planes a unit reads: in the volume, and its own with splits
  auto plane_used = [&](int z, int dz, int dz1) {
    return z + dz >= 0 && z + dz < p.Z && (dz1 == 2 || dz == dz1);
  };

  uint32_t nslab = 0, nbb = 0;   // slab chunks / B blocks issued (producers)
  if (warp == 0) {
    if (lane == 0) {
      // ---- slab producer ----
      for (long long it = blockIdx.x; it < g.items && !*abort_s; it += gridDim.x) {
        int b, z, y0, dz1;
        decode(it, b, z, y0, dz1);
        bool ok = true;
        for (int dz = -1; dz <= 1 && ok; dz++) {
          if (!plane_used(z, dz, dz1)) continue;
          for (int cg = 0; cg < NCG; cg++) {
            const uint32_t sl = nslab & 1;
            if (nslab >= 2 && !role_wait(sempty(sl), ((nslab >> 1) - 1) & 1, abort_s, 21)) {
              ok = false;
              break;
            }
            net_expect_tx(sfull(sl), NBOX * box_tx);
            for (int k = 0; k < NBOX; k++)
              tma_load_5d(slab_s + sl * SLOT + k * LBO, &tx, cg * KC + 8 * k, -1, y0 - 1, z + dz, b, sfull(sl));
            nslab++;
          }
        }
        if (!ok) break;
      }
    }
  } else if (warp == 2) {
    if (lane == 0) {
      // ---- B producer: one tap's KS blocks per ring slot, in the issuer's order ----
      for (long long it = blockIdx.x; it < g.items && !*abort_s; it += gridDim.x) {
        int b, z, y0, dz1;
        decode(it, b, z, y0, dz1);
        bool ok = true;
        for (int dz = -1; dz <= 1 && ok; dz++) {
          if (!plane_used(z, dz, dz1)) continue;
          for (int cg = 0; cg < NCG && ok; cg++)
            for (int t9 = 0; t9 < 9; t9 += TPS) {
              const uint32_t sl = nbb % SB;
              if (nbb >= SB && !role_wait(bempty(sl), ((nbb / SB) - 1) & 1, abort_s, 22)) {
                ok = false;
                break;
              }
              net_expect_tx(bfull(sl), SLOTB);
              // taps t9 .. t9+TPS-1 (contiguous in the packed weights when one chunk covers CI)
              for (int u = 0; u < TPS; u += (NCG == 1 ? TPS : 1)) {
                const int tap = (dz + 1) * 9 + t9 + u;
                const bf16 *src = wp + ((long long)tap * (CI / 16) + cg * KS) * (BBLK / 2);
                const uint32_t bytes = NCG == 1 ? SLOTB : TB;
                asm volatile(
                    "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::"r"(
                        bring_s + sl * SLOTB + u * TB),
                    "l"(src), "r"(bytes), "r"(bfull(sl))
                    : "memory");
              }
              nbb++;
            }
        }
        if (!ok) break;
      }
    }
  } else if (warp == 1) {
    if (lane == 0) {
      // ---- MMA issuer ----
      // instruction descriptor: F32 accumulate, BF16 A and B, both K-major, N = CO, M = 128
      const uint32_t idesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(CO >> 3) << 17) | ((128u >> 4) << 24);
      // operand descriptors: only the start-address field (low word, 16-byte units) moves.
      // A (SW): 128-byte swizzle, 8-row groups 1024 bytes apart, a row 8 units, a K step 2 units;
      // A (otherwise): 8-channel groups LBO apart, a row 1 unit, a K step 2 LBO; B: N-adjacent
      // core matrices 128 bytes apart, K-adjacent ones 16 CO bytes apart, a K step 2 CO units
      const uint64_t a0d = SW ? (umma_desc(slab_s, 16, 1024) | (2ull << 61)) : umma_desc(slab_s, LBO, 128);
      const uint64_t b0d = umma_desc(bring_s, 16u * CO, 128);
      const uint32_t a_lo0 = (uint32_t)a0d, a_hi = (uint32_t)(a0d >> 32);
      const uint32_t b_lo0 = (uint32_t)b0d, b_hi = (uint32_t)(b0d >> 32);
      const uint32_t a_row = SW ? 8u : 1u, a_ks = SW ? 2u : 2u * (LBO >> 4), a_slot = SLOT >> 4;
      const uint32_t a_m = 128u * a_row, b_ks = (2u * CO * 16u) >> 4, b_slot = SLOTB >> 4, b_tap = TB >> 4;
      const int nM = g.nM;
      uint32_t ns = 0, nb = 0, li = 0;
      bool ok = true;
      for (long long it = blockIdx.x; it < g.items && ok; it += gridDim.x, li++) {
        int b, z, y0, dz1;
        decode(it, b, z, y0, dz1);
        const uint32_t ab = li & 1;
        if (li >= 2 && !role_wait(aempty(ab), ((li >> 1) - 1) & 1, abort_s, 23)) {
          ok = false;
          break;
        }
        tc_fence_after();
        const uint32_t dcol = tmem + ab * WIDE_ACC_COLS;
        uint32_t acc = 0;   // the item's first MMA of each tile overwrites
        for (int dz = -1; dz <= 1 && ok; dz++) {
          if (!plane_used(z, dz, dz1)) continue;
          for (int cg = 0; cg < NCG && ok; cg++) {
            const uint32_t sl = ns & 1;
            if (!role_wait(sfull(sl), (ns >> 1) & 1, abort_s, 24)) {
              ok = false;
              break;
            }
            const uint32_t a_c = a_lo0 + sl * a_slot;
            for (int t9 = 0; t9 < 9; t9 += TPS) {
              const uint32_t bs = nb % SB;
              if (!role_wait(bfull(bs), (nb / SB) & 1, abort_s, 25)) {
                ok = false;
                break;
              }
              tc_fence_after();
              for (int u = 0; u < TPS; u++) {
                const int t = t9 + u;
                const uint32_t a_t = a_c + (uint32_t)((t / 3) * g.Xp + (t % 3)) * a_row;
                const uint32_t b_t = b_lo0 + bs * b_slot + u * b_tap;
#pragma unroll
                for (int ks = 0; ks < KS; ks++) {
                  const uint64_t bd = ((uint64_t)b_hi << 32) | (b_t + ks * b_ks);
#pragma unroll
                  for (int m = 0; m < 4; m++)
                    if (m < nM)
                      umma_f16(dcol + m * CO, ((uint64_t)a_hi << 32) | (a_t + ks * a_ks + m * a_m), bd, idesc, acc);
                  acc = 1;
                }
              }
              umma_commit(bempty(bs));   // the slot's B blocks are free once these MMAs complete
              nb++;
            }
            if (!ok) break;
            umma_commit(sempty(sl));     // the slab slot likewise
            ns++;
          }
        }
        if (!ok) break;
        umma_commit(afull(ab));
      }
    }
  } else if (warp >= 4) {
    // ---- epilogue ----
    const int qd = warp & 3;
    const uint32_t lane_base = (uint32_t)(qd * 32) << 16;
    uint32_t li = 0;
    for (long long it = blockIdx.x; it < g.items; it += gridDim.x, li++) {
      int b, z, y0, dz1;
      decode(it, b, z, y0, dz1);
      const uint32_t ab = li & 1;
      // tcgen05.ld is .sync.aligned: the whole warp takes one decision
      if (!__all_sync(0xffffffffu, role_wait(afull(ab), (li >> 1) & 1, abort_s, 26) ? 1 : 0)) break;
      tc_fence_after();
      // with splits a unit whose input plane lies outside the volume issued no MMA: zeros
      const bool none = g.splits > 1 && !plane_used(z, dz1, dz1);
      for (int m = 0; m < g.nM; m++) {
        const int q = m * 128 + qd * 32 + lane;
        const int yl = q / g.Xp, x = q - yl * g.Xp;
        const int y = y0 + yl;
        const bool valid = yl < g.R && y < p.Y && x < p.X;
        const long long vox = (((long long)b * p.Z + z) * p.Y + y) * p.X + x;
        const long long off = vox * CO;
#pragma unroll 1
        for (int c0 = 0; c0 < CO; c0 += 16) {
          float d[16];
          tmem_ld16(tmem + lane_base + ab * WIDE_ACC_COLS + m * CO + c0, d);
          asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
          if (!valid) continue;
          if (g.splits > 1) {   // FP32 partial sum of this input plane; bias, ReLU and mask come later
            float *dst = p.ws + (long long)(dz1 + 1) * Mv * CO + off + c0;
#pragma unroll
            for (int k = 0; k < 16; k += 4)
              *reinterpret_cast<float4 *>(dst + k) =
                  none ? make_float4(0.f, 0.f, 0.f, 0.f) : make_float4(d[k], d[k + 1], d[k + 2], d[k + 3]);
            continue;
          }
          uint4 mk[2];
          if (p.mask) {
            mk[0] = *reinterpret_cast<const uint4 *>(p.mask + off + c0);
            mk[1] = *reinterpret_cast<const uint4 *>(p.mask + off + c0 + 8);
          }
          const __nv_bfloat162 *m2 = reinterpret_cast<const __nv_bfloat162 *>(mk);
          uint4 outv[2];
          __nv_bfloat162 *hv = reinterpret_cast<__nv_bfloat162 *>(outv);
#pragma unroll
          for (int k = 0; k < 8; k++) {
            float v0 = d[2 * k] + (p.bias ? p.bias[c0 + 2 * k] : 0.f);
            float v1 = d[2 * k + 1] + (p.bias ? p.bias[c0 + 2 * k + 1] : 0.f);
            if (p.relu) {
              v0 = fmaxf(v0, 0.f);
              v1 = fmaxf(v1, 0.f);
            }
            if (p.mask) {
              const float2 mf = __bfloat1622float2(m2[k]);
              if (!(mf.x > 0.f)) v0 = 0.f;
              if (!(mf.y > 0.f)) v1 = 0.f;
            }
            hv[k] = __floats2bfloat162_rn(v0, v1);
          }
          *reinterpret_cast<uint4 *>(p.y + off + c0) = outv[0];
          *reinterpret_cast<uint4 *>(p.y + off + c0 + 8) = outv[1];
        }
      }
      tc_fence_before();
      __syncwarp();
      if (lane == 0) net_arrive(aempty(ab));
    }
  }

  __syncthreads();   // every role has left its loop (normally, or on an abort)
  if (*abort_s) {
    // copies still in flight land before the CTA exits: wait for the last load of every slot
    if (warp == 0 && lane == 0)
      for (uint32_t sl = 0; sl < 2 && sl < nslab; sl++) {
        const uint32_t last = sl + ((nslab - 1 - sl) / 2) * 2;
        if (!net_mbar_wait(sfull(sl), (last >> 1) & 1, 1000000000ULL)) atomicExch(&g_net_err, 27);
      }
    if (warp == 2 && lane == 0)
      for (uint32_t sl = 0; sl < SB && sl < nbb; sl++) {
        const uint32_t last = sl + ((nbb - 1 - sl) / SB) * SB;
        if (!net_mbar_wait(bfull(sl), (last / SB) & 1, 1000000000ULL)) atomicExch(&g_net_err, 28);
      }
  }
  if (warp == 1 && lane == 0) {
    // every MMA issued has completed before the accumulators are released
    umma_commit(fin);
    if (!net_mbar_wait(fin, 0, 1000000000ULL)) atomicExch(&g_net_err, 29);
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(2 * WIDE_ACC_COLS)
                 : "memory");
  }
}

// Packed B blocks of the wide kernel: wp[((tap * Ci/16 + ks) * 2 + k8) * Co + co][j]
// = w[tap][ci = 16 ks + 8 k8 + j][co], i.e. per (tap, 16 input channels) one
// [2][Co][8] block, the canonical no-swizzle K-major layout of an N = Co x
// K = 16 operand (K-adjacent core matrices 16 Co bytes apart).
__global__ void k_conv3d_pack_weights(const bf16 *w, bf16 *wp, int Ci, int Co) {
  const long long n = 27LL * Ci * Co;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const int co = (int)(i % Co);
    const long long t = i / Co;
    const int ci = (int)(t % Ci), tap = (int)(t / Ci);
    const int ks = ci >> 4, k8 = (ci >> 3) & 1, j = ci & 7;
    wp[((((long long)tap * (Ci / 16) + ks) * 2 + k8) * Co + co) * 8 + j] = w[i];
  }
}

// 0: the wide layers on mma.sync; 1 (default): on k_conv3d_wide with the rows
// per item chosen from the shape; 2..5: k_conv3d_wide with 1..4 M tiles per
// item (a sweep of the choice)
static int g_conv_wide_tc = 1;

int net_set_conv_wide_tcgen05(int mode) {
  const int old = g_conv_wide_tc;
  g_conv_wide_tc = mode < 0 ? 0 : (mode > 5 ? 5 : mode);
  return old;
}

// Shared memory of k_conv3d_wide: the two slab slots of slab_rows rows of KC
// channels, sb B blocks, the mbarriers, the TMEM address and abort flag.
static size_t wide_smem(int CI, int CO, int slab_rows, int sb, int tps) {
  const int KC = CI < 64 ? CI : 64;
  return (size_t)2 * KC * 2 * slab_rows + (size_t)sb * tps * (KC / 16) * 32 * CO + 8 * (8 + 2 * WIDE_SB_MAX + 1) +
         16;
}

// The item shape for nM M tiles: rows per item R (balanced over the y blocks),
// its slab rows, the taps of B blocks the rest of the shared memory holds, and
// the shared memory; false when nM tiles hold no full row or fewer than 3 taps
// fit beside the slabs.
static bool wide_shape(int CI, int CO, int Y, int X, int nM, WideGrid &g, size_t &smem) {
  g.Xp = X + 2;
  const int rmax = nM * 128 / g.Xp;
  if (rmax < 1 || g.Xp > 256 || nM * CO > WIDE_ACC_COLS) return false;
  g.nyb = (Y + rmax - 1) / rmax;
  g.R = (Y + g.nyb - 1) / g.nyb;
  if (g.R + 2 > 256) return false;
  g.nM = (g.R * g.Xp + 127) / 128;
  g.slab_rows = (g.nM * 128 + 2 * g.Xp + 2 + 7) / 8 * 8;
  const size_t fixed = wide_smem(CI, CO, g.slab_rows, 0, 1);
  const size_t tb = (size_t)((CI < 64 ? CI : 64) / 16) * 32 * CO;   // one tap's B blocks
  // a row of 3 taps per ring slot where 2 such slots fit, else one tap per slot (3 slots at least)
  g.tps = fixed + 2 * 3 * tb <= 227 * 1024 ? 3 : 1;
  if (fixed + 3 * tb > 227 * 1024) return false;
  g.sb = (int)((227 * 1024 - fixed) / (g.tps * tb));
  const int cap = g.tps == 3 ? WIDE_SB / 3 : WIDE_SB;
  if (g.sb > cap) g.sb = cap;
  smem = wide_smem(CI, CO, g.slab_rows, g.sb, g.tps);
  return true;
}

template <int CI, int CO>
static cudaError_t launch_wide(ConvParams p, long long ws_elems, cudaStream_t s, bool &done) {
  done = false;
  if (!p.wp) return cudaSuccess;
  static int sms = 0;
  if (!sms) {
    int dev = 0, n = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    sms = n > 0 ? n : 1;
  }
  const long long Mv = (long long)p.B * p.Z * p.Y * p.X;
  const bool can_split = p.ws && ws_elems >= 3 * Mv * CO;
  // work-unit shape: M tiles per item forced (modes 2..5) or chosen, and whether each item
  // splits over its three input planes (FP32 partials in ws, summed by k_conv3d_finish): the
  // least estimated time, ties to more M tiles.  Measured: a unit's time follows its weight
  // blocks (~320 cycles each, whatever the number of M tiles they feed; ~15 % less with three
  // taps per ring slot), plus a fixed cost per unit; a split also writes and reads three FP32
  // partial sets (~3000 bytes per cycle) and launches the finish kernel.
  WideGrid g{};
  size_t smem = 0;
  bool found = false;
  double best = 0;
  for (int nM = 1; nM <= 4; nM++) {
    if (g_conv_wide_tc >= 2 && nM != g_conv_wide_tc - 1) continue;
    WideGrid c{};
    size_t sm = 0;
    if (!wide_shape(CI, CO, p.Y, p.X, nM, c, sm)) continue;
    for (int sp = 1; sp <= (can_split ? 3 : 1); sp += 2) {
      c.splits = sp;
      c.items = (long long)p.B * p.Z * c.nyb * sp;
      const double waves = (double)((c.items + sms - 1) / sms);
      const double blocks = 27.0 * (CI / 16) / sp;
      const double partials = sp > 1 ? 4000.0 + 2.0 * 3.0 * (double)Mv * CO * 4.0 / 3000.0 : 0.0;
      const double cost = waves * (blocks * (c.tps == 3 ? 272.0 : 320.0) + 3000.0) + partials;
      if (!found || cost <= best) {
        found = true;
        best = cost;
        g = c;
        smem = sm;
      }
    }
  }
  if (!found) return cudaSuccess;   // the mma.sync kernel takes this shape
  done = true;
  if (reinterpret_cast<uintptr_t>(p.x) % 16 || reinterpret_cast<uintptr_t>(p.wp) % 16) return cudaErrorMisalignedAddress;
  PFN_cuTensorMapEncodeTiled_v12000 enc = tensor_map_encoder();
  if (!enc) return cudaErrorNotSupported;
  CUtensorMap map;
  const cuuint64_t vb = 2ull * CI;   // bytes per voxel
  const cuuint64_t dims[5] = {(cuuint64_t)CI, (cuuint64_t)p.X, (cuuint64_t)p.Y, (cuuint64_t)p.Z, (cuuint64_t)p.B};
  const cuuint64_t strides[4] = {vb, vb * p.X, vb * p.X * p.Y, vb * p.X * p.Y * p.Z};
  // 64-channel chunks: one box of 64 channels (128-byte rows, 128-byte swizzle); 32: 8-channel boxes
  constexpr bool SW = CI >= 64;
  const cuuint32_t box[5] = {SW ? 64u : 8u, (cuuint32_t)g.Xp, (cuuint32_t)(g.R + 2), 1, 1};
  const cuuint32_t estr[5] = {1, 1, 1, 1, 1};
  if (enc(&map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 5, const_cast<bf16 *>(p.x), dims, strides, box, estr,
          CU_TENSOR_MAP_INTERLEAVE_NONE, SW ? CU_TENSOR_MAP_SWIZZLE_128B : CU_TENSOR_MAP_SWIZZLE_NONE,
          CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
    return cudaErrorInvalidValue;
  // one CTA per SM (its 512 TMEM columns): ask for at least half the shared memory
  const size_t sm_launch = smem < 116 * 1024 ? 116 * 1024 : smem;
  static size_t attr = 0;
  if (attr < sm_launch) {
    cudaError_t e = cudaFuncSetAttribute(k_conv3d_wide<CI, CO>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)(227 * 1024));
    if (e != cudaSuccess) return e;
    attr = 227 * 1024;
  }
  const unsigned grid = (unsigned)(g.items < sms ? g.items : sms);
  p.splits = g.splits;
  FLF_NET_LAUNCH(k_conv3d_wide<CI, CO><<<grid, 256, sm_launch, s>>>(map, p, p.wp, g));
  if (g.splits > 1) FLF_NET_LAUNCH(k_conv3d_finish<<<grid_for(Mv * CO / 8, 256), 256, 0, s>>>(p, Mv));
  return cudaGetLastError();
}

static cudaError_t launch_wide_tc(const ConvParams &p, long long ws_elems, cudaStream_t s, bool &done) {
  done = false;
#define FLF_WD(a, b) if (p.Ci == a && p.Co == b) return launch_wide<a, b>(p, ws_elems, s, done);
  FLF_WD(32, 64) FLF_WD(64, 32) FLF_WD(64, 64) FLF_WD(64, 128) FLF_WD(128, 64) FLF_WD(128, 128)
  FLF_WD(32, 128) FLF_WD(128, 32)
#undef FLF_WD
  return cudaSuccess;
}

// kernels of the 16 / 32-channel convolutions: 0 = mma.sync tiles; 1 = tcgen05 with TMA staging
// for 16 -> 16, mma.sync for the 32-channel layers; 2 (default) = tcgen05 for all of them
static int g_conv16_tc = 2;

int net_set_conv16_tcgen05(int mode) {
  const int old = g_conv16_tc;
  g_conv16_tc = mode < 0 ? 0 : (mode > 2 ? 2 : mode);
  return old;
}

// 3x3x1 convolution (16 -> 16 channels; the taps dx != 1 of w ignored) on the
// tcgen05 kernel, or the 3x3x3 mma.sync kernel (those taps must then be zero)
cudaError_t launch_conv3d_x1(const ConvParams &p, cudaStream_t s) {
  if (p.Ci != 16 || p.Co != 16) return cudaErrorInvalidValue;
  return g_conv16_tc ? launch_tma16<16, 16, 2, 8, false, true, true>(p, HeadOut{}, s) : launch_t16<false>(p, HeadOut{}, s);
}

// 16 -> 16 channels with the output's 2x2x2 average pooling written as well (p.pool): the pooled
// values come from the epilogue of the tcgen05 kernel, or from k_pool2 after the mma.sync kernel
cudaError_t launch_conv3d_pool(const ConvParams &p, cudaStream_t s) {
  if (p.Ci != 16 || p.Co != 16 || !p.pool || ((p.Z | p.Y | p.X) & 1)) return cudaErrorInvalidValue;
  if (g_conv16_tc) return launch_tma16<16, 16, 2, 8, false, true, false, true>(p, HeadOut{}, s);
  const cudaError_t e = launch_t16<false>(p, HeadOut{}, s);
  if (e != cudaSuccess) return e;
  return launch_pool2(p.y, p.pool, p.B, p.Z, p.Y, p.X, 16, s);
}

cudaError_t launch_conv3d_tma16(const ConvParams &p, cudaStream_t s, bool sw32) {
  return sw32 ? launch_tma16<16, 16, 2, 8, false, true>(p, HeadOut{}, s)
              : launch_tma16<16, 16, 2, 8, false, false>(p, HeadOut{}, s);
}

cudaError_t launch_conv3d(ConvParams p, long long ws_elems, cudaStream_t s) {
  const long long M = (long long)p.B * p.Z * p.Y * p.X;
  if (M == 0) return cudaSuccess;
  p.splits = 1;
  if (p.Ci == 16 && p.Co == 16)
    return g_conv16_tc ? launch_tma16<16, 16, 2, 8, false, true>(p, HeadOut{}, s) : launch_t16<false>(p, HeadOut{}, s);
  if (p.Ci == 16 && p.Co == 32)
    return g_conv16_tc == 2 ? launch_tma16<16, 32, 1, 8, false, true>(p, HeadOut{}, s) : launch_tiled<16, 32>(p, s);
  if (p.Ci == 32 && p.Co == 16)
    return g_conv16_tc == 2 ? launch_tma16<32, 16, 2, 4, false, true>(p, HeadOut{}, s) : launch_tiled<32, 16>(p, s);
  if (p.Ci == 32 && p.Co == 32)
    return g_conv16_tc == 2 ? launch_tma16<32, 32, 1, 5, false, true>(p, HeadOut{}, s) : launch_tiled<32, 32>(p, s);
  if (p.wp && g_conv_wide_tc) {
    bool done = false;
    const cudaError_t e = launch_wide_tc(p, ws_elems, s, done);
    if (done) return e;
  }
  const int BN = p.Co >= 64 ? 64 : p.Co;
  const long long ctas = (M + 127) / 128 * (p.Co / BN);
  const int KT = 27 * (p.Ci / 16);
  static int sms = 0;
  if (!sms) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (sms <= 0) sms = 1;
  }
  // few CTAs with long K loops (the coarse levels): split K over up to 3 waves,
  // each split writing its own [M][Co] slice of ws (as many as ws holds)
  if (p.ws && ws_elems >= 2 * M * p.Co && ctas < 2LL * sms) {
    long long sp = (3LL * sms + ctas - 1) / ctas;
    if (sp > KT / 8) sp = KT / 8;
    if (sp > ws_elems / (M * p.Co)) sp = ws_elems / (M * p.Co);
    if (sp > 1) p.splits = (int)sp;
  }
  dim3 grid((unsigned)((M + 127) / 128), (unsigned)(p.Co / BN), (unsigned)p.splits);
  if (BN == 64) FLF_NET_LAUNCH(k_conv3d<64><<<grid, 128, 0, s>>>(p));
  else if (BN == 32) FLF_NET_LAUNCH(k_conv3d<32><<<grid, 128, 0, s>>>(p));
  else FLF_NET_LAUNCH(k_conv3d<16><<<grid, 128, 0, s>>>(p));
  if (p.splits > 1) FLF_NET_LAUNCH(k_conv3d_finish<<<grid_for(M * p.Co / 8, 256), 256, 0, s>>>(p, M));
  return cudaGetLastError();
}

cudaError_t launch_conv3d_wgrad(WgradParams p, long long ws_elems, cudaStream_t s, int num_sms) {
  const long long M = (long long)p.B * p.Z * p.Y * p.X;
  if (M == 0) return cudaSuccess;
  const int CM = p.Ci >= 32 ? 32 : 16, CN = p.Co >= 64 ? 64 : p.Co;
  const int tiles = (p.Ci / CM) * (p.Co / CN);
  const long long nw = 27LL * p.Ci * p.Co;
  long long chunks = (4LL * num_sms + 27 * tiles - 1) / (27 * tiles);
  if (!p.part) chunks = 1;                                         // no workspace: one writer per element
  else if (chunks > ws_elems / nw) chunks = ws_elems / nw;         // partial tiles must fit the workspace
  if (chunks < 1) chunks = 1;
  long long per = (M + chunks - 1) / chunks;
  per = (per + 63) / 64 * 64;
  chunks = (M + per - 1) / per;
  p.chunk = per;
  if (chunks == 1) p.part = nullptr;
  dim3 grid((unsigned)(chunks * 27), (unsigned)tiles);
#define FLF_WG(a, b) else if (CM == a && CN == b) FLF_NET_LAUNCH(k_conv3d_wgrad<a, b><<<grid, 128, 0, s>>>(p));
  if (false) {
  }
  FLF_WG(16, 16) FLF_WG(16, 32) FLF_WG(16, 64) FLF_WG(32, 16) FLF_WG(32, 32) FLF_WG(32, 64)
#undef FLF_WG
  if (p.part) FLF_NET_LAUNCH(k_wgrad_reduce<<<grid_for(nw, 256), 256, 0, s>>>(p.part, p.dw, nw, (int)chunks));
  return cudaGetLastError();
}

template <int ROWS, int NBUF>
static cudaError_t launch_tc16_rows(const ConvParams &p, cudaStream_t s) {
  static int grid_cap = 0;
  const size_t smem = 27 * 512 + (size_t)NBUF * 2 * 3 * (ROWS + 2) * 130 * 16 + 16;
  if (!grid_cap) {
    cudaError_t e = cudaFuncSetAttribute(k_conv3d_tc16<ROWS, NBUF>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    if (e != cudaSuccess) return e;
    e = cudaFuncSetAttribute(k_conv3d_tc16<ROWS, NBUF>, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
    if (e != cudaSuccess) return e;
    int per_sm = 0, dev = 0, sms = 0, smem_sm = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_conv3d_tc16<ROWS, NBUF>, 128, smem);
    if (e != cudaSuccess) return e;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
    const int by_smem = smem_sm > 0 ? (int)(smem_sm / (smem + 1024)) : 1;
    if (per_sm < by_smem) per_sm = by_smem;
    // TMEM: at most 512 columns per SM
    const int cols = ROWS * 16 <= 32 ? 32 : (ROWS * 16 <= 64 ? 64 : 128);
    if (per_sm > 512 / cols) per_sm = 512 / cols;
    if (per_sm < 1) per_sm = 1;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    grid_cap = per_sm * (sms > 0 ? sms : 1);
  }
  const long long M = (long long)p.B * p.Z * p.Y * p.X;
  if (M == 0) return cudaSuccess;
  const int tiles_x = (p.X + 127) / 128;
  const long long ntiles = (long long)p.B * p.Z * ((p.Y + ROWS - 1) / ROWS) * tiles_x;
  const unsigned grid = (unsigned)(ntiles < grid_cap ? ntiles : grid_cap);
  FLF_NET_LAUNCH(k_conv3d_tc16<ROWS, NBUF><<<grid, 128, smem, s>>>(p, tiles_x, ntiles));
  return cudaGetLastError();
}

cudaError_t launch_conv3d_tc16(const ConvParams &p, cudaStream_t s) {
  // p.splits selects the tile: 1 = 1 row x 128 (double-buffered), 4 = 4 rows (single buffer),
  // 5 = 4 rows double-buffered
  if (p.splits == 4) return launch_tc16_rows<4, 1>(p, s);
  if (p.splits == 5) return launch_tc16_rows<4, 2>(p, s);
  return launch_tc16_rows<1, 2>(p, s);
}

int net_status_read_and_clear() {
  int v = 0, z = 0;
  if (cudaMemcpyFromSymbol(&v, g_net_err, sizeof(int)) != cudaSuccess) return -1;
  if (v) cudaMemcpyToSymbol(g_net_err, &z, sizeof(int));
  return v;
}

cudaError_t launch_conv3d_flip(const void *w, void *w2, int Ci, int Co, cudaStream_t s) {
  FLF_NET_LAUNCH(k_conv3d_flip_weights<<<grid_for(27LL * Ci * Co, 256), 256, 0, s>>>((const bf16 *)w, (bf16 *)w2, Ci, Co));
  return cudaGetLastError();
}

cudaError_t launch_conv3d_pack(const void *w, void *wp, int Ci, int Co, cudaStream_t s) {
  FLF_NET_LAUNCH(k_conv3d_pack_weights<<<grid_for(27LL * Ci * Co, 256), 256, 0, s>>>((const bf16 *)w, (bf16 *)wp, Ci,
                                                                                      Co));
  return cudaGetLastError();
}

cudaError_t launch_bias_grad(const void *g, float *db, float *ws, long long ws_elems, long long M, int C,
                             cudaStream_t s) {
  long long blocks = (M + 2047) / 2048;
  if (!ws || blocks > ws_elems / C) blocks = ws ? ws_elems / C : 1;
  if (blocks > 65535) blocks = 65535;
  if (blocks < 1) blocks = 1;
  const long long rows = (M + blocks - 1) / blocks;
  blocks = (M + rows - 1) / rows;
  float *part = blocks > 1 ? ws : nullptr;
  FLF_NET_LAUNCH(k_bias_grad<<<(unsigned)blocks, 128, 0, s>>>((const bf16 *)g, db, part, M, C, rows));
  if (part) FLF_NET_LAUNCH(k_bias_reduce<<<1, 128, 0, s>>>(part, db, (int)blocks, C));
  return cudaGetLastError();
}

cudaError_t launch_pool2(const void *in, void *out, int B, int Z, int Y, int X, int C, cudaStream_t s) {
  FLF_NET_LAUNCH(k_pool2<<<grid_for((long long)B * Z * Y * X * C / 64, 256), 256, 0, s>>>((const bf16 *)in, (bf16 *)out, B, Z, Y, X, C));
  return cudaGetLastError();
}

cudaError_t launch_pool2_bwd(const void *gpool, const void *gskip, const void *act, void *gin, int B, int Z, int Y,
                             int X, int C, cudaStream_t s) {
  FLF_NET_LAUNCH(k_pool2_bwd<<<grid_for((long long)B * Z * Y * X * C / 8, 256), 256, 0, s>>>(
      (const bf16 *)gpool, (const bf16 *)gskip, (const bf16 *)act, (bf16 *)gin, B, Z, Y, X, C));
  return cudaGetLastError();
}

cudaError_t launch_up2_add(const void *low, const void *skip, void *out, int B, int Z, int Y, int X, int C,
                           cudaStream_t s) {
  if ((C / 8) & (C / 8 - 1)) return cudaErrorInvalidValue;   // C / 8 a power of two
  const long long rows = (long long)B * Z * Y;
  if (rows == 0 || X == 0) return cudaSuccess;
  const int threads = X * (C / 8) >= 256 ? 256 : 128;
  FLF_NET_LAUNCH(k_up2_add<<<(unsigned)rows, threads, 0, s>>>((const bf16 *)low, (const bf16 *)skip, (bf16 *)out, B, Z,
                                                            Y, X, C));
  return cudaGetLastError();
}

cudaError_t launch_up2_bwd(const void *g, const void *act, void *glow, int B, int Z, int Y, int X, int C,
                           cudaStream_t s) {
  FLF_NET_LAUNCH(k_up2_bwd<<<grid_for((long long)B * Z * Y * X * C / 64, 256), 256, 0, s>>>((const bf16 *)g, (const bf16 *)act,
                                                                              (bf16 *)glow, B, Z, Y, X, C));
  return cudaGetLastError();
}

cudaError_t launch_mse_grad(const void *y, const float *target, void *g, float *loss, long long M, int C,
                            cudaStream_t s) {
  FLF_NET_LAUNCH(k_mse_grad<<<grid_for(M, 256), 256, 0, s>>>((const bf16 *)y, target, (bf16 *)g, loss, M, C));
  return cudaGetLastError();
}

cudaError_t launch_adam(float *w, const float *g, float *m, float *v, void *wb, long long n, float lr, float b1,
                        float b2, float eps, float c1, float c2, float wd, cudaStream_t s) {
  FLF_NET_LAUNCH(k_adam<<<grid_for(n, 256), 256, 0, s>>>(w, g, m, v, (bf16 *)wb, n, lr, b1, b2, eps, c1, c2, wd));
  return cudaGetLastError();
}

cudaError_t launch_ws_input(const WsInputParams &p, cudaStream_t s) {
  const long long n = (long long)p.T * p.Zp * p.Yp * p.Xp;
  if (n == 0) return cudaSuccess;
  const long long V = (long long)p.Z * p.Y * p.X;
  const long long YX = (long long)p.Y * p.X;
  long long blocks = (YX + 255) / 256;   // a thread per pixel of a plane, all planes in its loop
  if (blocks > 1024) blocks = 1024;
  // the per-block partial sums go to the start of `out` (T * blocks floats fit:
  // out holds 32 bytes per padded voxel), which k_ws_input overwrites afterwards
  float *part = reinterpret_cast<float *>(p.out);
  FLF_NET_LAUNCH(k_ws_sum<<<dim3((unsigned)blocks, (unsigned)p.T), 256, 0, s>>>(p.htf, p.hth1, part, p.T, V, (long long)p.Y * p.X));
  FLF_NET_LAUNCH(k_ws_sum_final<<<(p.T + 127) / 128, 128, 0, s>>>(part, p.sum_x1, p.T, (int)blocks));
  FLF_NET_LAUNCH(k_ws_input<<<(unsigned)((long long)p.T * p.Zp * p.Yp), p.Xp >= 256 ? 256 : 128, 0, s>>>(p));
  return cudaGetLastError();
}

cudaError_t launch_ws_head(const void *d, const void *w, float bias, float floor_, const float *sum_x1, float *x0,
                           int T, int Z, int Y, int X, int Zp, int Yp, int Xp, cudaStream_t s) {
  ConvParams p{(const bf16 *)d, (const bf16 *)w, nullptr, nullptr, nullptr, T, Zp, Yp, Xp, 16, 16, 0, nullptr, 1};
  HeadOut h{x0, sum_x1, (float)Z * Y * X, bias, floor_, T, Z, Y, X};
  return g_conv16_tc ? launch_tma16<16, 16, 4, 8, true, true>(p, h, s) : launch_t16<true>(p, h, s);
}

cudaError_t launch_render_blobs(float *vol, void *acc, int Z, int Y, int X, const float *pts, int npts, float sigma,
                                cudaStream_t s) {
  if (npts <= 0) return cudaSuccess;
  const long long n = (long long)Z * Y * X;
  if (acc) {
    cudaError_t e = cudaMemsetAsync(acc, 0, sizeof(unsigned long long) * n, s);
    if (e != cudaSuccess) return e;
  }
  FLF_NET_LAUNCH(k_render_blobs<<<(unsigned)((npts * 32 + 255) / 256), 256, 0, s>>>(vol, (unsigned long long *)acc, Z, Y, X,
                                                                      (const float4 *)pts, npts, sigma));
  if (acc) FLF_NET_LAUNCH(k_blobs_add<<<grid_for(n, 256), 256, 0, s>>>(vol, (const unsigned long long *)acc, n));
  return cudaGetLastError();
}

}  // namespace flf
