// Learned heterogeneity correction: the 3-D U-Net's BF16 training and inference
// kernels on the fifth-generation tensor cores (tcgen05, FP32 accumulation in
// tensor memory), plus the memory-bound layers around them.
//
// Activation layout ("plane" layout): a tensor of C channels (C a multiple of
// 16) on a D x H x W grid is C/8 planes; a plane is `rows` rows of 16 bytes
// (8 BF16 channels of one voxel).  Rows index the zero-haloed grid
// (D+2) x (H+2) x (W+2) flattened in C order, offset by `margin` zero rows on
// both sides.  Halo and margin rows are zero in every tensor, so a 3x3x3 tap is
// a constant row offset and a tile of 128 consecutive rows of one tap is one
// contiguous 2 KB block per plane - exactly the no-swizzle core-matrix layout
// the tensor core reads (8 rows x 16 bytes per core matrix).
//
// Convolution as implicit GEMM (forward and data gradient):
//   Y[p, n] = sum_{tap, k} X[p + off(tap), k] * Wt[tap][n][k]   (M = 128 rows p,
//   N = output channels, K = 27 x input channels), one tcgen05.mma per 16 K.
// For each (dz, dy) the CTA stages a 130-row slab per plane; the three dx taps
// read it at row offsets 0, 1, 2 (descriptor start +16 bytes each).
// Weight gradient: dW[tap][k][n] = sum_p X[p + off(tap), k] G[p, n]: M = 128
// (tap, input-channel) pairs, N = output channels, K = rows, both operands
// MN-major straight from the plane layout; split over rows, partial sums
// reduced in a fixed order (deterministic).
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <mutex>
#include <string>

#include "pvd_common.cuh"
#include "umma.cuh"

namespace pvd {
namespace unet {

constexpr int TILE_M = 128;
constexpr int SLAB_ROWS = TILE_M + 2;
constexpr uint32_t SLAB_PITCH = SLAB_ROWS * 16;  // bytes of one plane's slab
constexpr int WG_KT = 64;                        // rows per weight-gradient stage
constexpr uint64_t WAIT_NS = 2000000000ull;      // bound of every mbarrier wait (2 s)
constexpr int CONV_THREADS = 192;                // warp 0 loads, warp 1 MMA, warps 2-5 epilogue
constexpr int MAX_SMEM = 232448;                 // 227 KB opt-in dynamic shared memory

enum { ST_TIMEOUT_LOAD = 1, ST_TIMEOUT_MMA = 2, ST_TIMEOUT_EPI = 3 };

__device__ int g_unet_status;  // first failure code seen by any kernel (0 = none)

__device__ __forceinline__ void fail(int code) { atomicCAS(&g_unet_status, 0, code); }

struct Geo {
  int D, H, W, Hp, Wp;
  long long np, np_tiles, margin, rows;
};

static Geo make_geo(const pvd_unet_geom* g) {
  Geo o;
  o.D = g->dims[0];
  o.H = g->dims[1];
  o.W = g->dims[2];
  o.Hp = o.H + 2;
  o.Wp = o.W + 2;
  o.np = g->padded;
  o.np_tiles = g->padded_tiles;
  o.margin = g->margin;
  o.rows = g->rows;
  return o;
}

__device__ __forceinline__ bool interior(const Geo& g, long long p) {
  if (p >= g.np) return false;
  int x, y, z;
  if (g.np < (1LL << 31)) {  // 32-bit division (the 64-bit one is emulated and slow)
    const uint32_t q = (uint32_t)p, t = q / (uint32_t)g.Wp;
    x = (int)(q - t * (uint32_t)g.Wp);
    z = (int)(t / (uint32_t)g.Hp);
    y = (int)(t - (uint32_t)z * (uint32_t)g.Hp);
  } else {
    x = (int)(p % g.Wp);
    const long long t = p / g.Wp;
    y = (int)(t % g.Hp);
    z = (int)(t / g.Hp);
  }
  return x >= 1 && x <= g.W && y >= 1 && y <= g.H && z >= 1 && z <= g.D;
}

__device__ __forceinline__ long long tap_offset(const Geo& g, int tap) {
  int dz = tap / 9, dy = (tap / 3) % 3, dx = tap % 3;
  return (long long)(dz - 1) * g.Hp * g.Wp + (long long)(dy - 1) * g.Wp + (dx - 1);
}

__device__ __forceinline__ float leaky_grad(float m, float slope) { return m > 0.f ? 1.f : slope; }

__device__ __forceinline__ void unpack8(uint4 u, float* f) {
  const __nv_bfloat162* h = reinterpret_cast<const __nv_bfloat162*>(&u);
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    float2 t = __bfloat1622float2(h[i]);
    f[2 * i] = t.x;
    f[2 * i + 1] = t.y;
  }
}
__device__ __forceinline__ uint4 pack8(const float* f) {
  uint4 u;
  __nv_bfloat162* h = reinterpret_cast<__nv_bfloat162*>(&u);
#pragma unroll
  for (int i = 0; i < 4; ++i) h[i] = __floats2bfloat162_rn(f[2 * i], f[2 * i + 1]);
  return u;
}

// ---------------------------------------------------------------------------
// 3x3x3 convolution (forward / data gradient), persistent, warp-specialised
// ---------------------------------------------------------------------------
struct ConvArgs {
  const uint8_t* x;     // input plane 0
  const uint8_t* w;     // packed weights [27][cin/8][cout][8] BF16
  const float* bias;    // [cout] or null
  uint8_t* y;           // output plane 0
  const uint8_t* mask;  // plane 0 of a cout-channel tensor whose LeakyReLU derivative scales the result, or null
  int cin, cout, flags, na, nb, resident, n_tiles;
  float slope;
  long long plane;  // bytes per plane (rows * 16), same for x, y, mask
  Geo g;
};

__global__ void __launch_bounds__(CONV_THREADS, 1) k_conv3(const ConvArgs a) {
  extern __shared__ __align__(128) uint8_t sm[];
  const int cin8 = a.cin >> 3;
  const uint32_t a_bytes = (uint32_t)cin8 * SLAB_PITCH;
  const uint32_t b_bytes = (uint32_t)a.cin * a.cout * 2;
  const int na = a.na, nb = a.nb;
  const bool resident = a.resident != 0;  // all 27 taps' weights loaded once into nb == 27 slots
  uint8_t* sa = sm;
  uint8_t* sb = sm + (size_t)na * a_bytes;
  uint64_t* full_a = reinterpret_cast<uint64_t*>(sb + (size_t)nb * b_bytes);
  uint64_t* empty_a = full_a + na;
  uint64_t* full_b = empty_a + na;
  uint64_t* empty_b = full_b + nb;
  uint64_t* acc_full = empty_b + nb;
  uint64_t* acc_empty = acc_full + 2;
  uint32_t* tslot = reinterpret_cast<uint32_t*>(acc_empty + 2);
  float* bias_s = reinterpret_cast<float*>(tslot + 4);  // [cout] bias (0 without one)
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint32_t ncols = umma::tmem_cols(2 * a.cout);

  for (int i = threadIdx.x; i < a.cout; i += blockDim.x) bias_s[i] = a.bias ? __ldg(a.bias + i) : 0.f;
  if (threadIdx.x == 0) {
    for (int i = 0; i < na; ++i) {
      mbar_init(&full_a[i], 1);
      mbar_init(&empty_a[i], 1);
    }
    for (int i = 0; i < 2; ++i) {
      mbar_init(&acc_full[i], 1);
      mbar_init(&acc_empty[i], 128);
    }
    for (int i = 0; i < nb; ++i) {
      mbar_init(&full_b[i], 1);
      mbar_init(&empty_b[i], 1);
    }
    fence_mbar_init();
  }
  if (warp == 1) umma::tmem_alloc(tslot, ncols);
  umma::fence_before_sync();
  __syncthreads();
  umma::fence_after_sync();
  const uint32_t tmem = *tslot;
  const Geo& g = a.g;

  if (warp == 0) {
    // load warp: lane 0 waits and arms the barrier, lane c copies plane c of the slab
    if (resident) {  // every tap's weights once, completing on full_b[0]
      if (lane == 0) mbar_arrive_expect_tx(&full_b[0], 27 * b_bytes);
      __syncwarp();
      if (lane < 27) umma::bulk_g2s(sb + (size_t)lane * b_bytes, a.w + (size_t)lane * b_bytes, b_bytes, &full_b[0]);
    }
    int it_a = 0, it_b = 0;
    for (int tile = blockIdx.x; tile < a.n_tiles; tile += gridDim.x) {
      const long long p0 = (long long)tile * TILE_M;
      for (int grp = 0; grp < 9; ++grp) {
        const int dz = grp / 3, dy = grp % 3;
        const long long row0 = g.margin + p0 + (long long)(dz - 1) * g.Hp * g.Wp + (long long)(dy - 1) * g.Wp - 1;
        const int s = it_a % na;
        if (!umma::warp_wait(&empty_a[s], ((it_a / na) & 1) ^ 1, WAIT_NS)) {
          if (lane == 0) fail(ST_TIMEOUT_LOAD);
          goto done;
        }
        if (lane == 0) mbar_arrive_expect_tx(&full_a[s], a_bytes);
        __syncwarp();
        for (int c = lane; c < cin8; c += 32)
          umma::bulk_g2s(sa + (size_t)s * a_bytes + (size_t)c * SLAB_PITCH, a.x + c * a.plane + row0 * 16, SLAB_PITCH,
                         &full_a[s]);
        ++it_a;
        if (resident) continue;
        for (int dx = 0; dx < 3; ++dx) {
          const int tap = grp * 3 + dx;
          const int sbi = it_b % nb;
          if (!umma::warp_wait(&empty_b[sbi], ((it_b / nb) & 1) ^ 1, WAIT_NS)) {
            if (lane == 0) fail(ST_TIMEOUT_LOAD);
            goto done;
          }
          if (lane == 0) {
            mbar_arrive_expect_tx(&full_b[sbi], b_bytes);
            umma::bulk_g2s(sb + (size_t)sbi * b_bytes, a.w + (size_t)tap * b_bytes, b_bytes, &full_b[sbi]);
          }
          __syncwarp();
          ++it_b;
        }
      }
    }
  } else if (warp == 1) {
    // MMA warp: the whole warp walks the loop (uniform descriptors), one elected lane issues
    const uint32_t idesc = umma::idesc_bf16(a.cout, false, false);
    const uint32_t b_lbo = (uint32_t)a.cout * 16;
    const uint64_t a_kstep = (2 * SLAB_PITCH) >> 4;  // descriptor start-address units per 16 channels
    const uint64_t b_kstep = (2 * b_lbo) >> 4;
    const int ksteps = a.cin / 16;
    int it_a = 0, it_b = 0, t_local = 0;
    if (resident && !umma::warp_wait(&full_b[0], 0, WAIT_NS)) {
      if (lane == 0) fail(ST_TIMEOUT_MMA);
      goto done;
    }
    for (int tile = blockIdx.x; tile < a.n_tiles; tile += gridDim.x, ++t_local) {
      const int acc = t_local & 1;
      if (!umma::warp_wait(&acc_empty[acc], ((t_local >> 1) & 1) ^ 1, WAIT_NS)) {
        if (lane == 0) fail(ST_TIMEOUT_MMA);
        goto done;
      }
      umma::fence_after_sync();
      const uint32_t d = tmem + (uint32_t)(acc * a.cout);
      for (int grp = 0; grp < 9; ++grp) {
        const int s = it_a % na;
        if (!umma::warp_wait(&full_a[s], (it_a / na) & 1, WAIT_NS)) {
          if (lane == 0) fail(ST_TIMEOUT_MMA);
          goto done;
        }
        umma::fence_after_sync();
        const uint64_t a0 = umma::smem_desc(smem_u32(sa + (size_t)s * a_bytes), SLAB_PITCH, 128);
        for (int dx = 0; dx < 3; ++dx) {
          const int sbi = resident ? grp * 3 + dx : it_b % nb;
          if (!resident) {
            if (!umma::warp_wait(&full_b[sbi], (it_b / nb) & 1, WAIT_NS)) {
              if (lane == 0) fail(ST_TIMEOUT_MMA);
              goto done;
            }
            umma::fence_after_sync();
          }
          uint64_t ad = a0 + (uint64_t)dx;  // +16 bytes per dx tap
          uint64_t bd = umma::smem_desc(smem_u32(sb + (size_t)sbi * b_bytes), b_lbo, 128);
          for (int kc = 0; kc < ksteps; ++kc, ad += a_kstep, bd += b_kstep)
            umma::mma_bf16_elect(d, ad, bd, idesc, (grp | dx | kc) != 0);
          if (!resident) {
            umma::commit_elect(&empty_b[sbi]);
            ++it_b;
          }
        }
        umma::commit_elect(&empty_a[s]);
        ++it_a;
      }
      umma::commit_elect(&acc_full[acc]);
    }
  } else {
    // epilogue: warp w reads TMEM lanes 32*(w%4) .. +31, one output row per thread
    const int q = warp & 3;
    const int r = 32 * q + lane;
    int t_local = 0;
    for (int tile = blockIdx.x; tile < a.n_tiles; tile += gridDim.x, ++t_local) {
      const int acc = t_local & 1;
      if (!mbar_wait_bounded(&acc_full[acc], (t_local >> 1) & 1, WAIT_NS)) {
        fail(ST_TIMEOUT_EPI);
        goto done;
      }
      umma::fence_after_sync();
      const long long p = (long long)tile * TILE_M + r;
      const bool in = interior(g, p);
      const long long roff = (g.margin + p) * 16;
      auto finish16 = [&](int c0, float* v) {
#pragma unroll
        for (int j = 0; j < 16; ++j) v[j] += bias_s[c0 + j];
        if (a.flags & PVD_UNET_ACT_LEAKY) {
#pragma unroll
          for (int j = 0; j < 16; ++j) v[j] = v[j] > 0.f ? v[j] : v[j] * a.slope;
        }
        const int pl = c0 >> 3;
        if (in && a.mask) {
          float m[16];
          unpack8(*reinterpret_cast<const uint4*>(a.mask + pl * a.plane + roff), m);
          unpack8(*reinterpret_cast<const uint4*>(a.mask + (pl + 1) * a.plane + roff), m + 8);
#pragma unroll
          for (int j = 0; j < 16; ++j) v[j] *= leaky_grad(m[j], a.slope);
        }
        if (in && (a.flags & PVD_UNET_ACCUMULATE)) {
          float o[16];
          unpack8(*reinterpret_cast<const uint4*>(a.y + pl * a.plane + roff), o);
          unpack8(*reinterpret_cast<const uint4*>(a.y + (pl + 1) * a.plane + roff), o + 8);
#pragma unroll
          for (int j = 0; j < 16; ++j) v[j] += o[j];
        }
        if (!in) {
#pragma unroll
          for (int j = 0; j < 16; ++j) v[j] = 0.f;
        }
        *reinterpret_cast<uint4*>(a.y + pl * a.plane + roff) = pack8(v);
        *reinterpret_cast<uint4*>(a.y + (pl + 1) * a.plane + roff) = pack8(v + 8);
      };
      const uint32_t trow = tmem + ((uint32_t)(32 * q) << 16) + (uint32_t)(acc * a.cout);
      for (int c0 = 0; c0 < a.cout; c0 += 32) {  // two column groups of 16 in flight per wait
        uint32_t t0[16], t1[16];
        const bool two = c0 + 16 < a.cout;  // uniform: cout is a kernel argument
        __syncwarp();
        umma::tmem_ld16_issue(trow + (uint32_t)c0, t0);
        if (two) umma::tmem_ld16_issue(trow + (uint32_t)(c0 + 16), t1);
        umma::tmem_wait_ld_tied(t0);
        umma::tmem_tie(t1);
        float v[16];
#pragma unroll
        for (int j = 0; j < 16; ++j) v[j] = __uint_as_float(t0[j]);
        finish16(c0, v);
        if (two) {
#pragma unroll
          for (int j = 0; j < 16; ++j) v[j] = __uint_as_float(t1[j]);
          finish16(c0 + 16, v);
        }
      }
      umma::fence_before_sync();
      umma::mbar_arrive(&acc_empty[acc]);
    }
  }
done:
  umma::fence_before_sync();
  __syncthreads();
  if (warp == 1) {
    umma::fence_after_sync();
    umma::tmem_dealloc(tmem, ncols);
  }
}

// ---------------------------------------------------------------------------
// 3x3x3 convolution with the three dx taps stacked along N (for 16 or 32 output
// channels, where an MMA costs the same ~40 cycles whatever its N up to 64):
// for each (dz, dy) and 16 input channels, one MMA of 128 unshifted slab rows x
// (3 x cout) columns gives P[r][dx][n]; the output row r of the tile is
// P[r][0] + P[r+1][1] + P[r+2][2], summed by the epilogue through shared memory.
// A tile therefore yields 126 output rows; 9 x cin/16 MMAs per tile instead of 27 x cin/16.
// ---------------------------------------------------------------------------
constexpr int STK_ROWS = 128;                      // slab rows = MMA rows
constexpr int STK_OUT = STK_ROWS - 2;              // output rows per tile
constexpr uint32_t STK_PITCH = STK_ROWS * 16;      // bytes of one plane's slab

template <int CO>
__global__ void __launch_bounds__(CONV_THREADS, CO == 16 ? 4 : 3) k_conv3s(const ConvArgs a) {
  extern __shared__ __align__(128) uint8_t sm[];
  const int cin8 = a.cin >> 3;
  constexpr int n3 = 3 * CO;
  const uint32_t a_bytes = (uint32_t)cin8 * STK_PITCH;
  const uint32_t g_bytes = (uint32_t)a.cin * n3 * 2;  // one (dz, dy) group's weights
  const int na = a.na;
  uint8_t* sa = sm;
  uint8_t* sb = sm + (size_t)na * a_bytes;
  constexpr int xp = CO + 4;  // exchange row pitch: 16-byte rows, 8 consecutive rows on distinct banks
  float* xch = reinterpret_cast<float*>(sb + (size_t)9 * g_bytes);  // [2][128][cout + 1] exchange
  uint64_t* full_a = reinterpret_cast<uint64_t*>(xch + 2 * STK_ROWS * xp);
  uint64_t* empty_a = full_a + na;
  uint64_t* full_w = empty_a + na;
  uint64_t* acc_full = full_w + 1;
  uint64_t* acc_empty = acc_full + 2;
  uint32_t* tslot = reinterpret_cast<uint32_t*>(acc_empty + 2);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(tslot + 1);  // an epilogue warp timed out
  float* bias_s = reinterpret_cast<float*>(tslot + 4);                    // [CO] bias (0 without one)
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint32_t ncols = umma::tmem_cols(2 * n3);

  if (threadIdx.x == 0) {
    *abort_flag = 0;
    for (int i = 0; i < na; ++i) {
      mbar_init(&full_a[i], 1);
      mbar_init(&empty_a[i], 1);
    }
    mbar_init(full_w, 1);
    for (int i = 0; i < 2; ++i) {
      mbar_init(&acc_full[i], 1);
      mbar_init(&acc_empty[i], 128);
    }
    fence_mbar_init();
  }
  if (warp == 1) umma::tmem_alloc(tslot, ncols);
  umma::fence_before_sync();
  __syncthreads();
  umma::fence_after_sync();
  const uint32_t tmem = *tslot;
  const Geo& g = a.g;

  if (warp == 0) {
    // load warp: all 9 groups' weights once (lanes 0-8), then the slabs (lane c: plane c)
    if (lane == 0) mbar_arrive_expect_tx(full_w, 9 * g_bytes);
    __syncwarp();
    if (lane < 9) umma::bulk_g2s(sb + (size_t)lane * g_bytes, a.w + (size_t)lane * g_bytes, g_bytes, full_w);
    int it_a = 0;
    for (int tile = blockIdx.x; tile < a.n_tiles; tile += gridDim.x) {
      const long long p0 = (long long)tile * STK_OUT;
      for (int grp = 0; grp < 9; ++grp) {
        const int dz = grp / 3, dy = grp % 3;
        const long long row0 = g.margin + p0 + (long long)(dz - 1) * g.Hp * g.Wp + (long long)(dy - 1) * g.Wp - 1;
        const int s = it_a % na;
        if (!umma::warp_wait(&empty_a[s], ((it_a / na) & 1) ^ 1, WAIT_NS)) {
          if (lane == 0) fail(ST_TIMEOUT_LOAD);
          goto done;
        }
        if (lane == 0) mbar_arrive_expect_tx(&full_a[s], a_bytes);
        __syncwarp();
        for (int c = lane; c < cin8; c += 32)
          umma::bulk_g2s(sa + (size_t)s * a_bytes + (size_t)c * STK_PITCH, a.x + c * a.plane + row0 * 16, STK_PITCH,
                         &full_a[s]);
        ++it_a;
      }
    }
  } else if (warp == 1) {
    const uint32_t idesc = umma::idesc_bf16(n3, false, false);
    const uint32_t b_lbo = (uint32_t)n3 * 16;
    const uint64_t a_kstep = (2 * STK_PITCH) >> 4;
    const uint64_t b_kstep = (2 * b_lbo) >> 4;
    const int ksteps = a.cin / 16;
    int it_a = 0, t_local = 0;
    if (!umma::warp_wait(full_w, 0, WAIT_NS)) {
      if (lane == 0) fail(ST_TIMEOUT_MMA);
      goto done;
    }
    for (int tile = blockIdx.x; tile < a.n_tiles; tile += gridDim.x, ++t_local) {
      const int acc = t_local & 1;
      if (!umma::warp_wait(&acc_empty[acc], ((t_local >> 1) & 1) ^ 1, WAIT_NS)) {
        if (lane == 0) fail(ST_TIMEOUT_MMA);
        goto done;
      }
      umma::fence_after_sync();
      const uint32_t d = tmem + (uint32_t)(acc * n3);
      for (int grp = 0; grp < 9; ++grp) {
        const int s = it_a % na;
        if (!umma::warp_wait(&full_a[s], (it_a / na) & 1, WAIT_NS)) {
          if (lane == 0) fail(ST_TIMEOUT_MMA);
          goto done;
        }
        umma::fence_after_sync();
        uint64_t ad = umma::smem_desc(smem_u32(sa + (size_t)s * a_bytes), STK_PITCH, 128);
        uint64_t bd = umma::smem_desc(smem_u32(sb + (size_t)grp * g_bytes), b_lbo, 128);
        for (int kc = 0; kc < ksteps; ++kc, ad += a_kstep, bd += b_kstep)
          umma::mma_bf16_elect(d, ad, bd, idesc, (grp | kc) != 0);
        umma::commit_elect(&empty_a[s]);
        ++it_a;
      }
      umma::commit_elect(&acc_full[acc]);
    }
  } else {
    // epilogue: thread r holds P[r][dx][n]; it publishes P[r][1] and P[r][2], then
    // sums P[r][0] + P[r+1][1] + P[r+2][2] for output row p0 + r (r < 126).  The four
    // warps meet at named barriers; a warp whose wait timed out still takes part and
    // raises the abort flag, so all four leave the loop together.
    const int q = warp & 3;
    const int r = 32 * q + lane;
    constexpr int co = CO;
    float* x1 = xch;                 // [128][cout + 4]: P[.][1]
    float* x2 = xch + STK_ROWS * xp; // [128][cout + 4]: P[.][2]
    if (r < CO) bias_s[r] = a.bias ? __ldg(a.bias + r) : 0.f;  // the bias, loaded once
    asm volatile("bar.sync 1, 128;" ::: "memory");
    int t_local = 0;
    for (int tile = blockIdx.x; tile < a.n_tiles; tile += gridDim.x, ++t_local) {
      const int acc = t_local & 1;
      const bool ok = umma::warp_wait(&acc_full[acc], (t_local >> 1) & 1, WAIT_NS);
      float v0[CO];
      if (ok) {
        umma::fence_after_sync();
        const uint32_t trow = tmem + ((uint32_t)(32 * q) << 16) + (uint32_t)(acc * n3);
        // P[r][1] and P[r][2] of 16 columns in flight together (one wait), to the exchange
#pragma unroll
        for (int c0 = 0; c0 < co; c0 += 16) {
          uint32_t t1[16], t2[16];
          umma::tmem_ld16_issue(trow + (uint32_t)(co + c0), t1);
          umma::tmem_ld16_issue(trow + (uint32_t)(2 * co + c0), t2);
          umma::tmem_wait_ld_tied(t1);
          umma::tmem_tie(t2);
#pragma unroll
          for (int j = 0; j < 16; j += 4) {
            *reinterpret_cast<uint4*>(x1 + r * xp + c0 + j) = make_uint4(t1[j], t1[j + 1], t1[j + 2], t1[j + 3]);
            *reinterpret_cast<uint4*>(x2 + r * xp + c0 + j) = make_uint4(t2[j], t2[j + 1], t2[j + 2], t2[j + 3]);
          }
        }
        // P[r][0], kept in registers across the exchange
#pragma unroll
        for (int c0 = 0; c0 < co; c0 += 16) {
          uint32_t t0[16];
          umma::tmem_ld16_issue(trow + (uint32_t)c0, t0);
          umma::tmem_wait_ld_tied(t0);
#pragma unroll
          for (int j = 0; j < 16; ++j) v0[c0 + j] = __uint_as_float(t0[j]);
        }
        umma::fence_before_sync();
        umma::mbar_arrive(&acc_empty[acc]);  // TMEM read: the MMA warp may reuse it
      } else if (lane == 0) {
        fail(ST_TIMEOUT_EPI);
        *abort_flag = 1;
      }
      asm volatile("bar.sync 1, 128;" ::: "memory");
      const bool stop = *abort_flag != 0;
      const long long p = (long long)tile * STK_OUT + r;
      if (!stop && r < STK_OUT && p < g.np) {
        const bool in = interior(g, p);
        const long long roff = (g.margin + p) * 16;
#pragma unroll
        for (int c0 = 0; c0 < co; c0 += 16) {
          float v[16];
#pragma unroll
          for (int j = 0; j < 16; j += 4) {
            const float4 u1 = *reinterpret_cast<const float4*>(x1 + (r + 1) * xp + c0 + j);
            const float4 u2 = *reinterpret_cast<const float4*>(x2 + (r + 2) * xp + c0 + j);
            v[j] = v0[c0 + j] + u1.x + u2.x;
            v[j + 1] = v0[c0 + j + 1] + u1.y + u2.y;
            v[j + 2] = v0[c0 + j + 2] + u1.z + u2.z;
            v[j + 3] = v0[c0 + j + 3] + u1.w + u2.w;
          }
#pragma unroll
          for (int j = 0; j < 16; ++j) v[j] += bias_s[c0 + j];
          if (a.flags & PVD_UNET_ACT_LEAKY) {
#pragma unroll
            for (int j = 0; j < 16; ++j) v[j] = v[j] > 0.f ? v[j] : v[j] * a.slope;
          }
          const int pl = c0 >> 3;
          if (in && a.mask) {
            float m[16];
            unpack8(*reinterpret_cast<const uint4*>(a.mask + pl * a.plane + roff), m);
            unpack8(*reinterpret_cast<const uint4*>(a.mask + (pl + 1) * a.plane + roff), m + 8);
#pragma unroll
            for (int j = 0; j < 16; ++j) v[j] *= leaky_grad(m[j], a.slope);
          }
          if (in && (a.flags & PVD_UNET_ACCUMULATE)) {
            float o[16];
            unpack8(*reinterpret_cast<const uint4*>(a.y + pl * a.plane + roff), o);
            unpack8(*reinterpret_cast<const uint4*>(a.y + (pl + 1) * a.plane + roff), o + 8);
#pragma unroll
            for (int j = 0; j < 16; ++j) v[j] += o[j];
          }
          if (!in) {
#pragma unroll
            for (int j = 0; j < 16; ++j) v[j] = 0.f;
          }
          *reinterpret_cast<uint4*>(a.y + pl * a.plane + roff) = pack8(v);
          *reinterpret_cast<uint4*>(a.y + (pl + 1) * a.plane + roff) = pack8(v + 8);
        }
      }
      asm volatile("bar.sync 1, 128;" ::: "memory");  // exchange buffer free for the next tile
      if (stop) break;
    }
  }
done:
  umma::fence_before_sync();
  __syncthreads();
  if (warp == 1) {
    umma::fence_after_sync();
    umma::tmem_dealloc(tmem, ncols);
  }
}

// ---------------------------------------------------------------------------
// weight gradient: partial[split][mt][m][n] = sum over this split's rows
// ---------------------------------------------------------------------------
struct WgradArgs {
  const uint8_t* x;  // input planes (cin channels)
  const uint8_t* g;  // output-gradient planes (cout channels)
  float* partial;
  int cin, cout, m_tiles, splits, ns;
  long long rows_per_split, plane;
  Geo geo;
};

__global__ void __launch_bounds__(CONV_THREADS, 1) k_wgrad(const WgradArgs a) {
  extern __shared__ __align__(128) uint8_t sm[];
  const uint32_t plane_tile = WG_KT * 16;  // bytes of one 8-channel group of a stage
  const uint32_t a_bytes = 16 * plane_tile;
  const uint32_t b_bytes = (uint32_t)(a.cout / 8) * plane_tile;
  const uint32_t st_bytes = a_bytes + b_bytes;
  const int ns = a.ns;
  uint64_t* full = reinterpret_cast<uint64_t*>(sm + (size_t)ns * st_bytes);
  uint64_t* empty = full + ns;
  uint64_t* acc_full = empty + ns;
  uint32_t* tslot = reinterpret_cast<uint32_t*>(acc_full + 1);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int mt = blockIdx.x, split = blockIdx.y;
  const uint32_t ncols = umma::tmem_cols(a.cout);
  const Geo& g = a.geo;
  const long long k_begin = (long long)split * a.rows_per_split;
  const long long k_end = min(g.np_tiles, k_begin + a.rows_per_split);
  const int n_st = k_end > k_begin ? (int)((k_end - k_begin) / WG_KT) : 0;

  if (threadIdx.x == 0) {
    for (int i = 0; i < ns; ++i) {
      mbar_init(&full[i], 1);
      mbar_init(&empty[i], 1);
    }
    mbar_init(acc_full, 1);
    fence_mbar_init();
  }
  if (warp == 1) umma::tmem_alloc(tslot, ncols);
  umma::fence_before_sync();
  __syncthreads();
  umma::fence_after_sync();
  const uint32_t tmem = *tslot;

  if (warp == 0) {
    // load warp: lane 0 waits and arms the barrier; lanes copy the 16 A groups and the
    // cout/8 B planes of a stage in parallel
    long long a_off = 0;
    int a_pl = 0;
    if (lane < 16) {  // source rows of A group `lane` (tap, 8-channel chunk) of this M tile
      const int mg = mt * 128 + lane * 8;
      int tap = mg / a.cin, ch = (mg % a.cin) / 8;
      if (tap >= 27) tap = 0, ch = 0;  // rows beyond 27 x cin: loaded but never stored
      a_off = tap_offset(g, tap);
      a_pl = ch;
    }
    const int n_copies = 16 + a.cout / 8;
    for (int st = 0; st < n_st; ++st) {
      const int s = st % ns;
      if (!umma::warp_wait(&empty[s], ((st / ns) & 1) ^ 1, WAIT_NS)) {
        if (lane == 0) fail(ST_TIMEOUT_LOAD);
        goto done;
      }
      if (lane == 0) mbar_arrive_expect_tx(&full[s], st_bytes);
      __syncwarp();
      const long long k0 = k_begin + (long long)st * WG_KT;
      uint8_t* dst = sm + (size_t)s * st_bytes;
      for (int c = lane; c < n_copies; c += 32) {
        if (c < 16)
          umma::bulk_g2s(dst + c * plane_tile, a.x + a_pl * a.plane + (g.margin + k0 + a_off) * 16, plane_tile,
                         &full[s]);
        else
          umma::bulk_g2s(dst + a_bytes + (c - 16) * plane_tile, a.g + (c - 16) * a.plane + (g.margin + k0) * 16,
                         plane_tile, &full[s]);
      }
    }
  } else if (warp == 1) {
    // MMA warp: whole warp walks the loop, one elected lane issues
    const uint32_t idesc = umma::idesc_bf16(a.cout, true, true);
    for (int st = 0; st < n_st; ++st) {
      const int s = st % ns;
      if (!umma::warp_wait(&full[s], (st / ns) & 1, WAIT_NS)) {
        if (lane == 0) fail(ST_TIMEOUT_MMA);
        goto done;
      }
      umma::fence_after_sync();
      const uint32_t base = smem_u32(sm + (size_t)s * st_bytes);
      uint64_t ad = umma::smem_desc(base, 128, plane_tile);
      uint64_t bd = umma::smem_desc(base + a_bytes, 128, plane_tile);
      for (int j = 0; j < WG_KT / 16; ++j, ad += 16, bd += 16)  // +256 bytes (16 rows) per K step
        umma::mma_bf16_elect(tmem, ad, bd, idesc, (st | j) != 0);
      umma::commit_elect(&empty[s]);
    }
    if (n_st > 0) umma::commit_elect(acc_full);
  } else {
    const int q = warp & 3;
    const int r = 32 * q + lane;
    float* out = a.partial + (((size_t)split * a.m_tiles + mt) * 128 + r) * a.cout;
    if (n_st == 0) {
      for (int c = 0; c < a.cout; ++c) out[c] = 0.f;
    } else {
      if (!mbar_wait_bounded(acc_full, 0, WAIT_NS)) {
        fail(ST_TIMEOUT_EPI);
        goto done;
      }
      umma::fence_after_sync();
      for (int c0 = 0; c0 < a.cout; c0 += 16) {
        float v[16];
        umma::tmem_ld16(tmem + ((uint32_t)(32 * q) << 16) + (uint32_t)c0, v);
#pragma unroll
        for (int j = 0; j < 16; j += 4) *reinterpret_cast<float4*>(out + c0 + j) = make_float4(v[j], v[j + 1], v[j + 2], v[j + 3]);
      }
    }
  }
done:
  umma::fence_before_sync();
  __syncthreads();
  if (warp == 1) {
    umma::fence_after_sync();
    umma::tmem_dealloc(tmem, ncols);
  }
}

// dw[n][k][tap] = sum over splits of partial[split][mt][m][n], m_global = tap*cin + k = mt*128 + m
// (threads run along n, so every split's partial row is read contiguously)
__global__ void k_wgrad_reduce(const float* __restrict__ partial, float* __restrict__ dw, int cin, int cout,
                               int m_tiles, int splits, int accumulate) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int total = cout * cin * 27;
  if (i >= total) return;
  const int n = i % cout, mgl = i / cout;
  const int tap = mgl / cin, k = mgl % cin;
  const size_t stride = (size_t)m_tiles * 128 * cout;
  const float* src = partial + (size_t)mgl * cout + n;  // mt * 128 + m == mgl
  float s = 0.f;
  for (int sp = 0; sp < splits; ++sp) s += src[sp * stride];
  const size_t o = ((size_t)n * cin + k) * 27 + tap;
  dw[o] = accumulate ? dw[o] + s : s;
}

// ---------------------------------------------------------------------------
// weight packing: FP32 [cout][cin][27] -> BF16 forward [27][cin/8][cout][8] and
// data-gradient [27][cout/8][cin][8] with the taps mirrored
// ---------------------------------------------------------------------------
// index of element (tap t, K channel kk, N channel nn) of a packed weight buffer for a
// convolution kernel with CI input and CO output channels: per-tap layout
// [27][CI/8][CO][8], or dx-stacked layout [9 (dz,dy)][CI/8][3 dx x CO][8]
__device__ __forceinline__ size_t packed_index(int t, int kk, int nn, int CI, int CO, bool stacked) {
  if (!stacked) return (((size_t)t * (CI / 8) + kk / 8) * CO + nn) * 8 + (kk % 8);
  return (((size_t)(t / 3) * (CI / 8) + kk / 8) * (3 * CO) + (t % 3) * CO + nn) * 8 + (kk % 8);
}

// FP32 [cout][cin][27] -> BF16 forward weights (kernel cin -> cout) and data-gradient
// weights (kernel cout -> cin, taps mirrored)
__global__ void k_pack_weights(const float* __restrict__ w, int cin, int cout, __nv_bfloat16* fwd,
                               __nv_bfloat16* bwd, int fwd_stacked, int bwd_stacked) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= cout * cin * 27) return;
  const int tap = i % 27, k = (i / 27) % cin, n = i / (27 * cin);
  const __nv_bfloat16 v = __float2bfloat16_rn(w[i]);
  if (fwd) fwd[packed_index(tap, k, n, cin, cout, fwd_stacked)] = v;
  if (bwd) bwd[packed_index(26 - tap, n, k, cout, cin, bwd_stacked)] = v;
}

// ---------------------------------------------------------------------------
// memory-bound layers (one thread per voxel and 8-channel plane)
// ---------------------------------------------------------------------------
__device__ __forceinline__ long long row_of(const Geo& g, int z, int y, int x) {
  return g.margin + ((long long)(z + 1) * g.Hp + (y + 1)) * g.Wp + (x + 1);
}

// Grid symmetry: U = flip(transpose(V, perm), flips).  U's axis k is V's axis perm[k],
// read backwards when flip[k]; U's dims are V's dims permuted.
struct Sym {
  int perm[3], flip[3];
};

__host__ __device__ inline Sym sym_of(int code) {
  Sym t;
  const int p = code / 8, f = code % 8;
  // the six permutations of (0, 1, 2) in lexicographic order
  t.perm[0] = p / 2;
  const int r0 = p / 2 == 0 ? 1 : 0, r1 = p / 2 == 2 ? 1 : 2;  // the two axes left, ascending
  t.perm[1] = (p & 1) ? r1 : r0;
  t.perm[2] = (p & 1) ? r0 : r1;
  for (int k = 0; k < 3; ++k) t.flip[k] = (f >> k) & 1;
  return t;
}

// V-coordinate of U's point u along V's axes: v[perm[k]] = flip[k] ? dim - 1 - u[k] : u[k]
__device__ __forceinline__ void sym_to_v(const Sym& t, const int* vdim, const int u[3], int v[3]) {
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const int ax = t.perm[k];
    v[ax] = t.flip[k] ? vdim[ax] - 1 - u[k] : u[k];
  }
}

// network input: channel c of the first n_in volumes (float32, C order, full grid
// vd x vh x vw) read at origin + voxel of the transformed volume U, scaled and
// mapped, others zero
struct InputArgs {
  const float* vol[4];
  float scale[4];
  const float* scale_d;  // device scales (n_in floats) overriding scale[], or null
  int mode[4];
  int n_in, origin[3], vdim[3];
  Sym sym;
  uint8_t* x;
  long long plane;
  Geo g;
};

__global__ void k_pack_input(const InputArgs a) {
  const long long n = (long long)a.g.D * a.g.H * a.g.W;
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int x = (int)(i % a.g.W), y = (int)((i / a.g.W) % a.g.H), z = (int)(i / ((long long)a.g.W * a.g.H));
  const int u[3] = {z + a.origin[0], y + a.origin[1], x + a.origin[2]};
  bool inside = true;
#pragma unroll
  for (int k = 0; k < 3; ++k) inside = inside && u[k] >= 0 && u[k] < a.vdim[a.sym.perm[k]];
  int v[3] = {0, 0, 0};
  if (inside) sym_to_v(a.sym, a.vdim, u, v);
  const long long src = inside ? ((long long)v[0] * a.vdim[1] + v[1]) * a.vdim[2] + v[2] : 0;
  float f[16];
#pragma unroll
  for (int c = 0; c < 16; ++c) f[c] = 0.f;
  for (int c = 0; c < a.n_in; ++c) {
    const float sc = a.scale_d ? a.scale_d[c] : a.scale[c];
    float v = inside ? a.vol[c][src] * sc : 0.f;
    if (a.mode[c] == 1) v = sqrtf(fmaxf(v, 0.f));
    else if (a.mode[c] == 2) v = log1pf(fmaxf(v, 0.f));
    f[c] = v;
  }
  const long long r = row_of(a.g, z, y, x) * 16;
  *reinterpret_cast<uint4*>(a.x + r) = pack8(f);
  *reinterpret_cast<uint4*>(a.x + a.plane + r) = pack8(f + 8);
}

// 2x2x2 average pooling, fine -> coarse
__global__ void k_pool(const uint8_t* __restrict__ xf, Geo gf, long long plane_f, uint8_t* yc, Geo gc,
                       long long plane_c, int c8) {
  const long long n = (long long)gc.D * gc.H * gc.W * c8;
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int pl = (int)(i % c8);
  const long long v = i / c8;
  const int x = (int)(v % gc.W), y = (int)((v / gc.W) % gc.H), z = (int)(v / ((long long)gc.W * gc.H));
  float s[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  for (int d = 0; d < 8; ++d) {
    float f[8];
    unpack8(*reinterpret_cast<const uint4*>(xf + pl * plane_f +
                                            row_of(gf, 2 * z + (d >> 2), 2 * y + ((d >> 1) & 1), 2 * x + (d & 1)) * 16),
            f);
#pragma unroll
    for (int j = 0; j < 8; ++j) s[j] += f[j];
  }
#pragma unroll
  for (int j = 0; j < 8; ++j) s[j] *= 0.125f;
  *reinterpret_cast<uint4*>(yc + pl * plane_c + row_of(gc, z, y, x) * 16) = pack8(s);
}

// pooling backward: dxf = ((accumulate ? dxf : 0) + dyc[parent] / 8) * leaky'(mask)
__global__ void k_pool_bwd(const uint8_t* __restrict__ dyc, Geo gc, long long plane_c, uint8_t* dxf,
                           const uint8_t* __restrict__ mask, Geo gf, long long plane_f, int c8, int accumulate,
                           float slope) {
  const long long n = (long long)gf.D * gf.H * gf.W * c8;
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int pl = (int)(i % c8);
  const long long v = i / c8;
  const int x = (int)(v % gf.W), y = (int)((v / gf.W) % gf.H), z = (int)(v / ((long long)gf.W * gf.H));
  float d[8], o[8];
  unpack8(*reinterpret_cast<const uint4*>(dyc + pl * plane_c + row_of(gc, z >> 1, y >> 1, x >> 1) * 16), d);
  const long long r = pl * plane_f + row_of(gf, z, y, x) * 16;
  if (accumulate) unpack8(*reinterpret_cast<const uint4*>(dxf + r), o);
#pragma unroll
  for (int j = 0; j < 8; ++j) d[j] = d[j] * 0.125f + (accumulate ? o[j] : 0.f);
  if (mask) {
    float m[8];
    unpack8(*reinterpret_cast<const uint4*>(mask + r), m);
#pragma unroll
    for (int j = 0; j < 8; ++j) d[j] *= leaky_grad(m[j], slope);
  }
  *reinterpret_cast<uint4*>(dxf + r) = pack8(d);
}

// nearest-neighbour 2x upsampling, coarse -> fine
__global__ void k_upsample(const uint8_t* __restrict__ xc, Geo gc, long long plane_c, uint8_t* yf, Geo gf,
                           long long plane_f, int c8) {
  const long long n = (long long)gf.D * gf.H * gf.W * c8;
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int pl = (int)(i % c8);
  const long long v = i / c8;
  const int x = (int)(v % gf.W), y = (int)((v / gf.W) % gf.H), z = (int)(v / ((long long)gf.W * gf.H));
  *reinterpret_cast<uint4*>(yf + pl * plane_f + row_of(gf, z, y, x) * 16) =
      *reinterpret_cast<const uint4*>(xc + pl * plane_c + row_of(gc, z >> 1, y >> 1, x >> 1) * 16);
}

// upsampling backward: dxc = sum of the 8 children's dyf, times leaky'(mask)
__global__ void k_upsample_bwd(const uint8_t* __restrict__ dyf, Geo gf, long long plane_f, uint8_t* dxc,
                               const uint8_t* __restrict__ mask, Geo gc, long long plane_c, int c8, float slope) {
  const long long n = (long long)gc.D * gc.H * gc.W * c8;
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int pl = (int)(i % c8);
  const long long v = i / c8;
  const int x = (int)(v % gc.W), y = (int)((v / gc.W) % gc.H), z = (int)(v / ((long long)gc.W * gc.H));
  float s[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  for (int d = 0; d < 8; ++d) {
    float f[8];
    unpack8(*reinterpret_cast<const uint4*>(dyf + pl * plane_f +
                                            row_of(gf, 2 * z + (d >> 2), 2 * y + ((d >> 1) & 1), 2 * x + (d & 1)) * 16),
            f);
#pragma unroll
    for (int j = 0; j < 8; ++j) s[j] += f[j];
  }
  const long long r = pl * plane_c + row_of(gc, z, y, x) * 16;
  if (mask) {
    float m[8];
    unpack8(*reinterpret_cast<const uint4*>(mask + r), m);
#pragma unroll
    for (int j = 0; j < 8; ++j) s[j] *= leaky_grad(m[j], slope);
  }
  *reinterpret_cast<uint4*>(dxc + r) = pack8(s);
}

// head: out[k][voxel] = b[k] + sum_c w[k][c] x[voxel][c], k = 0 (log dose ratio), 1 (log squared error)
__global__ void k_head(const uint8_t* __restrict__ x, long long plane, Geo g, const float* __restrict__ w,
                       float* __restrict__ out) {
  const long long n = (long long)g.D * g.H * g.W;
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int xx = (int)(i % g.W), y = (int)((i / g.W) % g.H), z = (int)(i / ((long long)g.W * g.H));
  const long long r = row_of(g, z, y, xx) * 16;
  float f[16];
  unpack8(*reinterpret_cast<const uint4*>(x + r), f);
  unpack8(*reinterpret_cast<const uint4*>(x + plane + r), f + 8);
  float o0 = w[32], o1 = w[33];
#pragma unroll
  for (int c = 0; c < 16; ++c) {
    o0 += w[c] * f[c];
    o1 += w[16 + c] * f[c];
  }
  out[i] = o0;
  out[n + i] = o1;
}

// loss and head backward.  pred: [2][n] from k_head; target/weight: full volumes
// read at origin.  Per voxel e = mu - t, l = log(e^2 + eps):
//   loss0 = sum w e^2 / n,  loss1 = sum w (s - l)^2 / n  (l taken as constant)
// gx (16-channel planes) = g_mu w0 * leaky'(x): the error head s learns from the
// features without passing its gradient into the network; per-block partial sums
// of [dw0(16) dw1(16) db0 db1 loss0 loss1] go to part[block][36].
constexpr int HEAD_THREADS = 256;
__global__ void __launch_bounds__(HEAD_THREADS) k_head_loss(const uint8_t* __restrict__ x, long long plane, Geo g,
                                                           const float* __restrict__ w, const float* __restrict__ pred,
                                                           const float* __restrict__ target,
                                                           const float* __restrict__ weight, int o0, int o1, int o2,
                                                           int vd, int vh, int vw, Sym t_sym, float inv_n, float eps,
                                                           float slope, uint8_t* gx, float* __restrict__ part) {
  __shared__ float red[HEAD_THREADS / 32][36];
  const long long n = (long long)g.D * g.H * g.W;
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  float acc[36];
#pragma unroll
  for (int j = 0; j < 36; ++j) acc[j] = 0.f;
  if (i < n) {
    const int xx = (int)(i % g.W), y = (int)((i / g.W) % g.H), z = (int)(i / ((long long)g.W * g.H));
    // crop voxel -> point u of the transformed volume U -> voxel v of the target volumes
    const int u[3] = {z + o0, y + o1, xx + o2};
    const int vdim[3] = {vd, vh, vw};
    bool inside = true;
#pragma unroll
    for (int k = 0; k < 3; ++k) inside = inside && u[k] >= 0 && u[k] < vdim[t_sym.perm[k]];
    int v[3] = {0, 0, 0};
    if (inside) sym_to_v(t_sym, vdim, u, v);
    const long long src = inside ? ((long long)v[0] * vh + v[1]) * vw + v[2] : 0;
    const float t = inside ? target[src] : 0.f, wt = inside ? weight[src] : 0.f;
    const float mu = pred[i], s = pred[n + i];
    const float e = mu - t;
    const float l = logf(e * e + eps);
    const float gm = 2.f * wt * e * inv_n, gs = 2.f * wt * (s - l) * inv_n;
    const long long r = row_of(g, z, y, xx) * 16;
    float f[16], gv[16];
    unpack8(*reinterpret_cast<const uint4*>(x + r), f);
    unpack8(*reinterpret_cast<const uint4*>(x + plane + r), f + 8);
#pragma unroll
    for (int c = 0; c < 16; ++c) {
      gv[c] = gm * w[c] * leaky_grad(f[c], slope);
      acc[c] = gm * f[c];
      acc[16 + c] = gs * f[c];
    }
    acc[32] = gm;
    acc[33] = gs;
    acc[34] = wt * e * e * inv_n;
    acc[35] = wt * (s - l) * (s - l) * inv_n;
    *reinterpret_cast<uint4*>(gx + r) = pack8(gv);
    *reinterpret_cast<uint4*>(gx + plane + r) = pack8(gv + 8);
  }
  const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5;
#pragma unroll
  for (int j = 0; j < 36; ++j) {
    float v = acc[j];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) red[wp][j] = v;
  }
  __syncthreads();
  if (threadIdx.x < 36) {
    float v = 0.f;
    for (int k = 0; k < HEAD_THREADS / 32; ++k) v += red[k][threadIdx.x];
    part[(size_t)blockIdx.x * 36 + threadIdx.x] = v;
  }
}

// sum of per-block rows, fixed order: out[j] = sum_b part[b][j]
__global__ void k_sum_rows(const float* __restrict__ part, int n_rows, int n_cols, float* __restrict__ out) {
  const int j = blockIdx.x;
  float s = 0.f;
  for (int b = threadIdx.x; b < n_rows; b += blockDim.x) s += part[(size_t)b * n_cols + j];
  __shared__ float red[32];
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x < 32) {
    float v = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.f;
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (threadIdx.x == 0) out[j] = v;
  }
}

// bias gradient partials: part[block][c] = sum over this block's interior voxels of G[voxel][c]
constexpr int BIAS_VOX = 256;
__global__ void k_bias_grad(const uint8_t* __restrict__ gt, long long plane, Geo g, int c8, float* __restrict__ part) {
  // block: 256 voxels x all planes; thread t handles voxel t for each plane
  const long long n = (long long)g.D * g.H * g.W;
  const long long i = (long long)blockIdx.x * BIAS_VOX + threadIdx.x;
  __shared__ float red[BIAS_VOX / 32][8];
  const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5;
  long long r = -1;
  if (i < n) {
    const int xx = (int)(i % g.W), y = (int)((i / g.W) % g.H), z = (int)(i / ((long long)g.W * g.H));
    r = row_of(g, z, y, xx) * 16;
  }
  for (int pl = 0; pl < c8; ++pl) {
    float f[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    if (r >= 0) unpack8(*reinterpret_cast<const uint4*>(gt + pl * plane + r), f);
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      float v = f[j];
      for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
      if (lane == 0) red[wp][j] = v;
    }
    __syncthreads();
    if (threadIdx.x < 8) {
      float v = 0.f;
      for (int k = 0; k < BIAS_VOX / 32; ++k) v += red[k][threadIdx.x];
      part[(size_t)blockIdx.x * (c8 * 8) + pl * 8 + threadIdx.x] = v;
    }
    __syncthreads();
  }
}

// corrected dose on the volume voxels the crop covers: dose_conv * exp(clamp(mu)),
// or dose_conv itself where the predicted error sqrt(exp(s)) exceeds sigma_max
__global__ void k_apply(const float* __restrict__ pred, Geo g, const float* __restrict__ dose, int o0, int o1, int o2,
                        int vd, int vh, int vw, float sigma_max, float mu_clamp, float* __restrict__ out,
                        uint8_t* __restrict__ fallback) {
  const long long n = (long long)g.D * g.H * g.W;
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int xx = (int)(i % g.W), y = (int)((i / g.W) % g.H), z = (int)(i / ((long long)g.W * g.H));
  const int sz = z + o0, sy = y + o1, sx = xx + o2;
  if (sz < 0 || sz >= vd || sy < 0 || sy >= vh || sx < 0 || sx >= vw) return;
  const long long v = ((long long)sz * vh + sy) * vw + sx;
  const float mu = fminf(fmaxf(pred[i], -mu_clamp), mu_clamp);
  const bool fb = !(expf(0.5f * pred[n + i]) <= sigma_max);
  out[v] = fb ? dose[v] : dose[v] * expf(mu);
  if (fallback) fallback[v] = fb ? 1 : 0;
}

// pred_avg[c][v] (+)= w * pred_sym[c][T(v)] over the voxels v of V (dims vd), T(v) in
// U = flip(transpose(V, perm)); both predictions dense [2][crop dims] at origin 0
__global__ void k_sym_accumulate(const float* __restrict__ ps, Geo gs, float* __restrict__ acc, Geo g, int vd0,
                                 int vd1, int vd2, Sym t, float w, int accumulate) {
  const long long n = (long long)vd0 * vd1 * vd2;
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int v[3] = {(int)(i / ((long long)vd1 * vd2)), (int)((i / vd2) % vd1), (int)(i % vd2)};
  const int vdim[3] = {vd0, vd1, vd2};
  int u[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const int ax = t.perm[k];
    u[k] = t.flip[k] ? vdim[ax] - 1 - v[ax] : v[ax];
  }
  const long long ns = (long long)gs.D * gs.H * gs.W, na = (long long)g.D * g.H * g.W;
  const long long is = ((long long)u[0] * gs.H + u[1]) * gs.W + u[2];
  const long long ia = ((long long)v[0] * g.H + v[1]) * g.W + v[2];
#pragma unroll
  for (int c = 0; c < 2; ++c) {
    const float val = w * ps[c * ns + is];
    acc[c * na + ia] = accumulate ? acc[c * na + ia] + val : val;
  }
}

// maxima[0] = max activity, maxima[1] = max dose over voxels with density >= rho_min
// (both over non-negative finite values; maxima zeroed first)
__global__ void k_input_maxima(const float* __restrict__ act, const float* __restrict__ rho,
                               const float* __restrict__ dose, long long n, float rho_min, float* maxima) {
  float ma = 0.f, md = 0.f;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const float a = act[i];
    if (a > ma && a <= 3.4e38f) ma = a;
    const float d = dose[i];
    if (rho[i] >= rho_min && d > md && d <= 3.4e38f) md = d;
  }
  for (int o = 16; o > 0; o >>= 1) {
    ma = fmaxf(ma, __shfl_xor_sync(0xffffffffu, ma, o));
    md = fmaxf(md, __shfl_xor_sync(0xffffffffu, md, o));
  }
  if ((threadIdx.x & 31) == 0) {
    // non-negative floats order like their bit patterns
    atomicMax(reinterpret_cast<int*>(maxima), __float_as_int(ma));
    atomicMax(reinterpret_cast<int*>(maxima) + 1, __float_as_int(md));
  }
}

// out[2..4] = network input scales from the maxima in out[0..1]: 1/max activity, 1, 1/max dose
__global__ void k_input_scales(float* out) {
  out[2] = out[0] > 0.f ? 1.f / out[0] : 0.f;
  out[3] = 1.f;
  out[4] = out[1] > 0.f ? 1.f / out[1] : 0.f;
}

// Adam with decoupled weight decay on FP32 parameters
__global__ void k_adam(float* __restrict__ p, const float* __restrict__ gr, float* __restrict__ m,
                       float* __restrict__ v, long long n, float lr, float b1, float b2, float eps, float wd,
                       float c1, float c2) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float gg = gr[i];
  const float mi = b1 * m[i] + (1.f - b1) * gg;
  const float vi = b2 * v[i] + (1.f - b2) * gg * gg;
  m[i] = mi;
  v[i] = vi;
  p[i] -= lr * ((mi / c1) / (sqrtf(vi / c2) + eps) + wd * p[i]);
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
static int g_sms = 0;
static int sm_count() {
  if (g_sms == 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&g_sms, cudaDevAttrMultiProcessorCount, dev);
    if (g_sms <= 0) g_sms = 1;
  }
  return g_sms;
}

static bool ch_ok(int c) { return c >= 16 && c <= 256 && c % 16 == 0; }
static bool al16(const void* p) { return ((uintptr_t)p & 15) == 0; }

static size_t conv_smem(int cin, int cout, int na, int nb) {
  return (size_t)na * (cin / 8) * SLAB_PITCH + (size_t)nb * cin * cout * 2 + (size_t)(4 + 2 * na + 2 * nb) * 8 + 16 +
         (size_t)cout * 4 + 16;
}

// Shared-memory plan of a convolution: all 27 taps' weights resident with up to
// four input slabs in flight when they fit, else a ring of tap-weight slots.
struct ConvPlanSm {
  int na, nb, resident, occ;
  size_t smem;
  int stacked;  // dx taps stacked along N (k_conv3s)
};

static size_t conv_smem_stacked(int cin, int cout, int na) {
  return (size_t)na * (cin / 8) * STK_PITCH + (size_t)27 * cin * cout * 2 + (size_t)2 * STK_ROWS * (cout + 4) * 4 +
         (size_t)(2 * na + 5) * 8 + 16 + (size_t)cout * 4 + 16;
}

static ConvPlanSm conv_plan(int cin, int cout) {
  ConvPlanSm p{0, 0, 0, 0, 0, 0};
  // 16 or 32 output channels: dx taps stacked along N, weights resident, the deepest
  // slab ring that lets 4, else 2, else 1 CTAs share an SM
  if (cout == 16 || cout == 32) {
    for (int target : {4, 2, 1}) {
      const size_t budget = std::min((size_t)MAX_SMEM, (size_t)(233472 / target) - 2048);
      for (int na = 9; na >= 2 && !p.na; --na)
        if (conv_smem_stacked(cin, cout, na) <= budget) p = {na, 0, 1, 0, conv_smem_stacked(cin, cout, na), 1};
      if (p.na) return p;
    }
  }
  // resident weights: the deepest input-slab ring (up to a whole tile's 9 slabs) that
  // still lets 4, else 2, else 1 CTAs share an SM
  for (int target : {4, 2, 1}) {
    const size_t budget = std::min((size_t)MAX_SMEM, (size_t)(233472 / target) - 2048);
    for (int na = 9; na >= 2 && !p.na; --na)
      if (conv_smem(cin, cout, na, 27) <= budget) p = {na, 27, 1, 0, conv_smem(cin, cout, na, 27), 0};
    if (p.na) break;
  }
  if (!p.na) {
    int nb = 4;
    while (nb > 2 && conv_smem(cin, cout, 2, nb) > (size_t)MAX_SMEM) --nb;
    p = {2, nb, 0, 0, conv_smem(cin, cout, 2, nb), 0};
  }
  return p;
}

static pvd_status geo_check(const pvd_unet_geom* g) {
  if (!g) return set_error(PVD_ERR_ARG, "unet: null geometry");
  pvd_unet_geom ref;
  if (pvd_unet_geometry(g->dims[0], g->dims[1], g->dims[2], &ref) != PVD_OK) return PVD_ERR_ARG;
  if (ref.rows != g->rows || ref.margin != g->margin || ref.padded != g->padded || ref.padded_tiles != g->padded_tiles)
    return set_error(PVD_ERR_ARG, "unet: geometry not produced by pvd_unet_geometry");
  return PVD_OK;
}

static unsigned blocks_for(long long n, int t) { return (unsigned)((n + t - 1) / t); }

}  // namespace unet
}  // namespace pvd

using namespace pvd;
using namespace pvd::unet;

extern "C" pvd_status pvd_unet_geometry(int d, int h, int w, pvd_unet_geom* out) {
  if (!out) return set_error(PVD_ERR_ARG, "pvd_unet_geometry: null output");
  if (d < 1 || h < 1 || w < 1 || d > 4096 || h > 4096 || w > 4096)
    return set_error(PVD_ERR_ARG, "pvd_unet_geometry: dims must be in [1, 4096]");
  const long long hp = h + 2, wp = w + 2, dp = d + 2;
  out->dims[0] = d;
  out->dims[1] = h;
  out->dims[2] = w;
  out->padded = dp * hp * wp;
  out->padded_tiles = (out->padded + TILE_M - 1) / TILE_M * TILE_M;
  // zero rows either side: the largest tap offset plus one 128-row tile, so every
  // slab a convolution tile reads lies inside the plane
  out->margin = (hp * wp + wp + 2 + 7) / 8 * 8 + TILE_M;
  out->rows = out->margin + out->padded_tiles + out->margin;
  return PVD_OK;
}

// the kernel a plan launches
static const void* conv_kernel(const ConvPlanSm& pl, int cout) {
  if (!pl.stacked) return (const void*)k_conv3;
  return cout == 16 ? (const void*)k_conv3s<16> : (const void*)k_conv3s<32>;
}

extern "C" pvd_status pvd_unet_conv3d(const pvd_unet_geom* geom, const void* x, int cin, const void* w_packed,
                                      const float* bias, void* y, int cout, const void* mask, int flags, float slope,
                                      pvd_stream stream) {
  pvd_status st = geo_check(geom);
  if (st != PVD_OK) return st;
  if (!ch_ok(cin) || !ch_ok(cout)) return set_error(PVD_ERR_ARG, "pvd_unet_conv3d: channels must be multiples of 16 in [16, 256]");
  if (!x || !w_packed || !y || !al16(x) || !al16(w_packed) || !al16(y) || (mask && !al16(mask)))
    return set_error(PVD_ERR_ARG, "pvd_unet_conv3d: tensors must be non-null and 16-byte aligned");
  if (flags & ~(PVD_UNET_ACT_LEAKY | PVD_UNET_ACCUMULATE)) return set_error(PVD_ERR_ARG, "pvd_unet_conv3d: unknown flags");
  // launch configuration per (cin, cout), computed once per process (one device)
  static ConvPlanSm plans[17][17];
  static bool have[17][17];
  static std::mutex plans_mu;
  std::unique_lock<std::mutex> lock(plans_mu);
  if (!have[cin / 16][cout / 16]) {
    ConvPlanSm np = conv_plan(cin, cout);
    if (np.smem > (size_t)MAX_SMEM)
      return set_error(PVD_ERR_UNSUPPORTED, "pvd_unet_conv3d: channel counts need more shared memory than a CTA has");
    const void* kern = conv_kernel(np, cout);
    PVD_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)MAX_SMEM));
    // CTAs that can be resident on one SM at once: registers (allocated per warp in
    // units of 256), shared memory (228 KB per SM, 1 KB reserved per CTA), threads,
    // and TMEM (512 columns per SM; a CTA holds two accumulators)
    cudaFuncAttributes fa;
    PVD_CUDA_TRY(cudaFuncGetAttributes(&fa, kern));
    const int regs_warp = (fa.numRegs * 32 + 255) / 256 * 256;
    const int by_regs = 65536 / (regs_warp * (CONV_THREADS / 32));
    const int by_smem = (int)(233472 / (np.smem + fa.sharedSizeBytes + 1024));
    const int by_threads = 2048 / CONV_THREADS;
    const int by_tmem = (int)(512 / umma::tmem_cols(2 * cout * (np.stacked ? 3 : 1)));
    np.occ = std::max(1, std::min(std::min(by_regs, by_smem), std::min(by_threads, by_tmem)));
    // when TMEM is the binding limit, request enough shared memory that no more CTAs
    // than that can be co-resident (an extra CTA would wait in tcgen05.alloc for a
    // persistent CTA to finish)
    if (by_tmem < std::min(std::min(by_regs, by_smem), by_threads))
      np.smem = std::max(np.smem, (size_t)(233472 / by_tmem) - 1024 - fa.sharedSizeBytes);
    plans[cin / 16][cout / 16] = np;
    have[cin / 16][cout / 16] = true;
  }
  const ConvPlanSm pl = plans[cin / 16][cout / 16];
  lock.unlock();
  const size_t smem = pl.smem;
  ConvArgs a;
  a.x = (const uint8_t*)x;
  a.w = (const uint8_t*)w_packed;
  a.bias = bias;
  a.y = (uint8_t*)y;
  a.mask = (const uint8_t*)mask;
  a.cin = cin;
  a.cout = cout;
  a.flags = flags;
  a.na = pl.na;
  a.nb = pl.nb;
  a.resident = pl.resident;
  a.slope = slope;
  a.g = make_geo(geom);
  a.plane = a.g.rows * 16;
  if (pl.stacked) {
    a.n_tiles = (int)((a.g.np + STK_OUT - 1) / STK_OUT);
    const int grid = std::min(a.n_tiles, sm_count() * pl.occ);
    if (cout == 16)
      k_conv3s<16><<<grid, CONV_THREADS, smem, (cudaStream_t)stream>>>(a);
    else
      k_conv3s<32><<<grid, CONV_THREADS, smem, (cudaStream_t)stream>>>(a);
    PVD_LAUNCH_CHECK("k_conv3s");
    return PVD_OK;
  }
  a.n_tiles = (int)(a.g.np_tiles / TILE_M);
  const int grid = std::min(a.n_tiles, sm_count() * pl.occ);
  k_conv3<<<grid, CONV_THREADS, smem, (cudaStream_t)stream>>>(a);
  PVD_LAUNCH_CHECK("k_conv3");
  return PVD_OK;
}

static void wgrad_plan(const Geo& g, int cin, int cout, int* m_tiles, int* splits, long long* per, int* ns) {
  *m_tiles = (27 * cin + 127) / 128;
  const long long n_k = g.np_tiles / WG_KT;
  long long want = std::max<long long>(1, (2LL * sm_count() + *m_tiles - 1) / *m_tiles);
  want = std::min(want, n_k);
  const long long per_k = (n_k + want - 1) / want;
  *per = per_k * WG_KT;
  *splits = (int)((n_k + per_k - 1) / per_k);
  const size_t st_bytes = 16 * WG_KT * 16 + (size_t)(cout / 8) * WG_KT * 16;
  int s = 6;
  while (s > 2 && (size_t)s * st_bytes + (2 * s + 1) * 8 + 16 > (size_t)MAX_SMEM) --s;
  *ns = s;
}

extern "C" pvd_status pvd_unet_wgrad_workspace(const pvd_unet_geom* geom, int cin, int cout, size_t* bytes) {
  pvd_status st = geo_check(geom);
  if (st != PVD_OK) return st;
  if (!bytes || !ch_ok(cin) || !ch_ok(cout)) return set_error(PVD_ERR_ARG, "pvd_unet_wgrad_workspace: bad arguments");
  int mt, sp, ns;
  long long per;
  wgrad_plan(make_geo(geom), cin, cout, &mt, &sp, &per, &ns);
  *bytes = (size_t)sp * mt * 128 * cout * sizeof(float);
  return PVD_OK;
}

extern "C" pvd_status pvd_unet_conv3d_wgrad(const pvd_unet_geom* geom, const void* x, int cin, const void* grad,
                                            int cout, float* dw, int accumulate, void* workspace,
                                            size_t workspace_bytes, pvd_stream stream) {
  pvd_status st = geo_check(geom);
  if (st != PVD_OK) return st;
  if (!ch_ok(cin) || !ch_ok(cout)) return set_error(PVD_ERR_ARG, "pvd_unet_conv3d_wgrad: channels must be multiples of 16 in [16, 256]");
  if (!x || !grad || !dw || !workspace || !al16(x) || !al16(grad) || !al16(workspace))
    return set_error(PVD_ERR_ARG, "pvd_unet_conv3d_wgrad: tensors must be non-null and 16-byte aligned");
  WgradArgs a;
  a.geo = make_geo(geom);
  wgrad_plan(a.geo, cin, cout, &a.m_tiles, &a.splits, &a.rows_per_split, &a.ns);
  const size_t need = (size_t)a.splits * a.m_tiles * 128 * cout * sizeof(float);
  if (workspace_bytes < need) return set_error(PVD_ERR_ARG, "pvd_unet_conv3d_wgrad: workspace smaller than pvd_unet_wgrad_workspace");
  a.x = (const uint8_t*)x;
  a.g = (const uint8_t*)grad;
  a.partial = (float*)workspace;
  a.cin = cin;
  a.cout = cout;
  a.plane = a.geo.rows * 16;
  const size_t st_bytes = 16 * WG_KT * 16 + (size_t)(cout / 8) * WG_KT * 16;
  const size_t smem = (size_t)a.ns * st_bytes + (2 * a.ns + 1) * 8 + 16;
  {
    // raised only when a larger stage ring is needed: after the first call per layer shape no
    // attribute call remains, so a training step can be captured in a CUDA graph
    static size_t smem_set = 0;
    static std::mutex mu;
    std::lock_guard<std::mutex> lock(mu);
    if (smem > smem_set) {
      PVD_CUDA_TRY(cudaFuncSetAttribute(k_wgrad, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
      smem_set = smem;
    }
  }
  k_wgrad<<<dim3(a.m_tiles, a.splits), CONV_THREADS, smem, (cudaStream_t)stream>>>(a);
  PVD_LAUNCH_CHECK("k_wgrad");
  const int total = cout * cin * 27;
  k_wgrad_reduce<<<blocks_for(total, 256), 256, 0, (cudaStream_t)stream>>>(a.partial, dw, cin, cout, a.m_tiles,
                                                                          a.splits, accumulate);
  PVD_LAUNCH_CHECK("k_wgrad_reduce");
  return PVD_OK;
}

extern "C" pvd_status pvd_unet_pack_weights(const float* w, int cin, int cout, void* fwd_packed, void* bwd_packed,
                                            pvd_stream stream) {
  if (!w || (!fwd_packed && !bwd_packed) || !ch_ok(cin) || !ch_ok(cout))
    return set_error(PVD_ERR_ARG, "pvd_unet_pack_weights: bad arguments");
  const int total = cout * cin * 27;
  // each buffer in the layout the convolution of those channels will read
  const int fs = conv_plan(cin, cout).stacked, bs = conv_plan(cout, cin).stacked;
  k_pack_weights<<<blocks_for(total, 256), 256, 0, (cudaStream_t)stream>>>(w, cin, cout, (__nv_bfloat16*)fwd_packed,
                                                                          (__nv_bfloat16*)bwd_packed, fs, bs);
  PVD_LAUNCH_CHECK("k_pack_weights");
  return PVD_OK;
}

extern "C" pvd_status pvd_unet_pack_input(const pvd_unet_geom* geom, const float* const* volumes, const float* scales,
                                          const float* scales_d, const int* modes, int n_in, const int* vol_dims,
                                          const int* origin, void* x, pvd_stream stream) {
  return pvd_unet_pack_input_sym(geom, volumes, scales, scales_d, modes, n_in, vol_dims, origin, 0, x, stream);
}

extern "C" pvd_status pvd_unet_pack_input_sym(const pvd_unet_geom* geom, const float* const* volumes,
                                              const float* scales, const float* scales_d, const int* modes, int n_in,
                                              const int* vol_dims, const int* origin, int sym, void* x,
                                              pvd_stream stream) {
  pvd_status st = geo_check(geom);
  if (st != PVD_OK) return st;
  if (n_in < 1 || n_in > 4 || !volumes || (!scales && !scales_d) || !modes || !vol_dims || !origin || !x || !al16(x))
    return set_error(PVD_ERR_ARG, "pvd_unet_pack_input: bad arguments");
  if (sym < 0 || sym >= PVD_UNET_SYMMETRIES) return set_error(PVD_ERR_ARG, "pvd_unet_pack_input_sym: sym out of range");
  InputArgs a;
  a.g = make_geo(geom);
  a.sym = sym_of(sym);
  for (int i = 0; i < 3; ++i) {
    a.origin[i] = origin[i];
    a.vdim[i] = vol_dims[i];
    if (vol_dims[i] < 1) return set_error(PVD_ERR_ARG, "pvd_unet_pack_input: bad volume dims");
  }
  for (int c = 0; c < 4; ++c) {
    a.vol[c] = c < n_in ? volumes[c] : nullptr;
    a.scale[c] = (c < n_in && scales) ? scales[c] : 0.f;
    a.mode[c] = c < n_in ? modes[c] : 0;
    if (c < n_in && (!volumes[c] || modes[c] < 0 || modes[c] > 2))
      return set_error(PVD_ERR_ARG, "pvd_unet_pack_input: null volume or unknown mode");
  }
  a.n_in = n_in;
  a.scale_d = scales_d;
  a.x = (uint8_t*)x;
  a.plane = a.g.rows * 16;
  const long long n = (long long)a.g.D * a.g.H * a.g.W;
  k_pack_input<<<blocks_for(n, 256), 256, 0, (cudaStream_t)stream>>>(a);
  PVD_LAUNCH_CHECK("k_pack_input");
  return PVD_OK;
}

static pvd_status pair_check(const pvd_unet_geom* fine, const pvd_unet_geom* coarse, int c, const void* p, const void* q,
                             const char* who) {
  pvd_status st = geo_check(fine);
  if (st != PVD_OK) return st;
  st = geo_check(coarse);
  if (st != PVD_OK) return st;
  for (int i = 0; i < 3; ++i)
    if (fine->dims[i] != 2 * coarse->dims[i]) return set_error(PVD_ERR_ARG, std::string(who) + ": fine dims must be twice the coarse dims");
  if (c < 8 || c % 8 || !p || !q || !al16(p) || !al16(q))
    return set_error(PVD_ERR_ARG, std::string(who) + ": bad channel count or tensor");
  return PVD_OK;
}

extern "C" pvd_status pvd_unet_pool(const pvd_unet_geom* fine, const void* x, const pvd_unet_geom* coarse, void* y,
                                    int channels, pvd_stream stream) {
  pvd_status st = pair_check(fine, coarse, channels, x, y, "pvd_unet_pool");
  if (st != PVD_OK) return st;
  const Geo gf = make_geo(fine), gc = make_geo(coarse);
  const long long n = (long long)gc.D * gc.H * gc.W * (channels / 8);
  k_pool<<<blocks_for(n, 256), 256, 0, (cudaStream_t)stream>>>((const uint8_t*)x, gf, gf.rows * 16, (uint8_t*)y, gc,
                                                              gc.rows * 16, channels / 8);
  PVD_LAUNCH_CHECK("k_pool");
  return PVD_OK;
}

extern "C" pvd_status pvd_unet_pool_backward(const pvd_unet_geom* coarse, const void* dy, const pvd_unet_geom* fine,
                                             void* dx, const void* mask, int channels, int accumulate, float slope,
                                             pvd_stream stream) {
  pvd_status st = pair_check(fine, coarse, channels, dy, dx, "pvd_unet_pool_backward");
  if (st != PVD_OK) return st;
  const Geo gf = make_geo(fine), gc = make_geo(coarse);
  const long long n = (long long)gf.D * gf.H * gf.W * (channels / 8);
  k_pool_bwd<<<blocks_for(n, 256), 256, 0, (cudaStream_t)stream>>>((const uint8_t*)dy, gc, gc.rows * 16, (uint8_t*)dx,
                                                                  (const uint8_t*)mask, gf, gf.rows * 16,
                                                                  channels / 8, accumulate, slope);
  PVD_LAUNCH_CHECK("k_pool_bwd");
  return PVD_OK;
}

extern "C" pvd_status pvd_unet_upsample(const pvd_unet_geom* coarse, const void* x, const pvd_unet_geom* fine, void* y,
                                        int channels, pvd_stream stream) {
  pvd_status st = pair_check(fine, coarse, channels, x, y, "pvd_unet_upsample");
  if (st != PVD_OK) return st;
  const Geo gf = make_geo(fine), gc = make_geo(coarse);
  const long long n = (long long)gf.D * gf.H * gf.W * (channels / 8);
  k_upsample<<<blocks_for(n, 256), 256, 0, (cudaStream_t)stream>>>((const uint8_t*)x, gc, gc.rows * 16, (uint8_t*)y,
                                                                  gf, gf.rows * 16, channels / 8);
  PVD_LAUNCH_CHECK("k_upsample");
  return PVD_OK;
}

extern "C" pvd_status pvd_unet_upsample_backward(const pvd_unet_geom* fine, const void* dy, const pvd_unet_geom* coarse,
                                                 void* dx, const void* mask, int channels, float slope,
                                                 pvd_stream stream) {
  pvd_status st = pair_check(fine, coarse, channels, dy, dx, "pvd_unet_upsample_backward");
  if (st != PVD_OK) return st;
  const Geo gf = make_geo(fine), gc = make_geo(coarse);
  const long long n = (long long)gc.D * gc.H * gc.W * (channels / 8);
  k_upsample_bwd<<<blocks_for(n, 256), 256, 0, (cudaStream_t)stream>>>((const uint8_t*)dy, gf, gf.rows * 16,
                                                                      (uint8_t*)dx, (const uint8_t*)mask, gc,
                                                                      gc.rows * 16, channels / 8, slope);
  PVD_LAUNCH_CHECK("k_upsample_bwd");
  return PVD_OK;
}

extern "C" pvd_status pvd_unet_head(const pvd_unet_geom* geom, const void* x, const float* w_head, float* out,
                                    pvd_stream stream) {
  pvd_status st = geo_check(geom);
  if (st != PVD_OK) return st;
  if (!x || !w_head || !out || !al16(x)) return set_error(PVD_ERR_ARG, "pvd_unet_head: bad arguments");
  const Geo g = make_geo(geom);
  const long long n = (long long)g.D * g.H * g.W;
  k_head<<<blocks_for(n, 256), 256, 0, (cudaStream_t)stream>>>((const uint8_t*)x, g.rows * 16, g, w_head, out);
  PVD_LAUNCH_CHECK("k_head");
  return PVD_OK;
}

extern "C" pvd_status pvd_unet_head_loss_workspace(const pvd_unet_geom* geom, size_t* bytes) {
  pvd_status st = geo_check(geom);
  if (st != PVD_OK) return st;
  if (!bytes) return set_error(PVD_ERR_ARG, "pvd_unet_head_loss_workspace: null output");
  const long long n = (long long)geom->dims[0] * geom->dims[1] * geom->dims[2];
  *bytes = (size_t)blocks_for(n, HEAD_THREADS) * 36 * sizeof(float);
  return PVD_OK;
}

extern "C" pvd_status pvd_unet_head_loss(const pvd_unet_geom* geom, const void* x, const float* w_head,
                                         const float* pred, const float* target, const float* weight,
                                         const int* vol_dims, const int* origin, float eps, float slope, void* grad_x,
                                         float* grads_and_loss, void* workspace, size_t workspace_bytes,
                                         pvd_stream stream) {
  return pvd_unet_head_loss_sym(geom, x, w_head, pred, target, weight, vol_dims, origin, 0, eps, slope, grad_x,
                                grads_and_loss, workspace, workspace_bytes, stream);
}

extern "C" pvd_status pvd_unet_head_loss_sym(const pvd_unet_geom* geom, const void* x, const float* w_head,
                                             const float* pred, const float* target, const float* weight,
                                             const int* vol_dims, const int* origin, int sym, float eps, float slope,
                                             void* grad_x, float* grads_and_loss, void* workspace,
                                             size_t workspace_bytes, pvd_stream stream) {
  pvd_status st = geo_check(geom);
  if (st != PVD_OK) return st;
  if (!x || !w_head || !pred || !target || !weight || !vol_dims || !origin || !grad_x || !grads_and_loss ||
      !workspace || !al16(x) || !al16(grad_x))
    return set_error(PVD_ERR_ARG, "pvd_unet_head_loss: bad arguments");
  if (sym < 0 || sym >= PVD_UNET_SYMMETRIES) return set_error(PVD_ERR_ARG, "pvd_unet_head_loss_sym: sym out of range");
  for (int i = 0; i < 3; ++i)
    if (vol_dims[i] < 1) return set_error(PVD_ERR_ARG, "pvd_unet_head_loss: bad volume dims");
  const Geo g = make_geo(geom);
  const long long n = (long long)g.D * g.H * g.W;
  const unsigned nblk = blocks_for(n, HEAD_THREADS);
  if (workspace_bytes < (size_t)nblk * 36 * sizeof(float))
    return set_error(PVD_ERR_ARG, "pvd_unet_head_loss: workspace smaller than pvd_unet_head_loss_workspace");
  k_head_loss<<<nblk, HEAD_THREADS, 0, (cudaStream_t)stream>>>(
      (const uint8_t*)x, g.rows * 16, g, w_head, pred, target, weight, origin[0], origin[1], origin[2], vol_dims[0],
      vol_dims[1], vol_dims[2], sym_of(sym), (float)(1.0 / (double)n), eps, slope, (uint8_t*)grad_x,
      (float*)workspace);
  PVD_LAUNCH_CHECK("k_head_loss");
  k_sum_rows<<<36, 256, 0, (cudaStream_t)stream>>>((const float*)workspace, (int)nblk, 36, grads_and_loss);
  PVD_LAUNCH_CHECK("k_sum_rows");
  return PVD_OK;
}

extern "C" pvd_status pvd_unet_bias_grad_workspace(const pvd_unet_geom* geom, int channels, size_t* bytes) {
  pvd_status st = geo_check(geom);
  if (st != PVD_OK) return st;
  if (!bytes || channels < 8 || channels % 8) return set_error(PVD_ERR_ARG, "pvd_unet_bias_grad_workspace: bad arguments");
  const long long n = (long long)geom->dims[0] * geom->dims[1] * geom->dims[2];
  *bytes = (size_t)blocks_for(n, BIAS_VOX) * channels * sizeof(float);
  return PVD_OK;
}

extern "C" pvd_status pvd_unet_bias_grad(const pvd_unet_geom* geom, const void* grad, int channels, float* db,
                                         void* workspace, size_t workspace_bytes, pvd_stream stream) {
  pvd_status st = geo_check(geom);
  if (st != PVD_OK) return st;
  if (!grad || !db || !workspace || channels < 8 || channels % 8 || !al16(grad))
    return set_error(PVD_ERR_ARG, "pvd_unet_bias_grad: bad arguments");
  const Geo g = make_geo(geom);
  const long long n = (long long)g.D * g.H * g.W;
  const unsigned nblk = blocks_for(n, BIAS_VOX);
  if (workspace_bytes < (size_t)nblk * channels * sizeof(float))
    return set_error(PVD_ERR_ARG, "pvd_unet_bias_grad: workspace smaller than pvd_unet_bias_grad_workspace");
  k_bias_grad<<<nblk, BIAS_VOX, 0, (cudaStream_t)stream>>>((const uint8_t*)grad, g.rows * 16, g, channels / 8,
                                                          (float*)workspace);
  PVD_LAUNCH_CHECK("k_bias_grad");
  k_sum_rows<<<channels, 256, 0, (cudaStream_t)stream>>>((const float*)workspace, (int)nblk, channels, db);
  PVD_LAUNCH_CHECK("k_sum_rows");
  return PVD_OK;
}

extern "C" pvd_status pvd_unet_symmetry_accumulate(const pvd_unet_geom* geom_sym, const float* pred_sym,
                                                   const pvd_unet_geom* geom, const int* vol_dims, int sym,
                                                   float weight, int accumulate, float* pred_avg, pvd_stream stream) {
  pvd_status st = geo_check(geom_sym);
  if (st == PVD_OK) st = geo_check(geom);
  if (st != PVD_OK) return st;
  if (!pred_sym || !pred_avg || !vol_dims || sym < 0 || sym >= PVD_UNET_SYMMETRIES || !std::isfinite(weight))
    return set_error(PVD_ERR_ARG, "pvd_unet_symmetry_accumulate: bad arguments");
  const Geo gs = make_geo(geom_sym), g = make_geo(geom);
  const Sym t = sym_of(sym);
  const int cs[3] = {gs.D, gs.H, gs.W}, ca[3] = {g.D, g.H, g.W};
  for (int k = 0; k < 3; ++k)
    if (vol_dims[k] < 1 || vol_dims[k] > ca[k] || vol_dims[t.perm[k]] > cs[k])
      return set_error(PVD_ERR_ARG, "pvd_unet_symmetry_accumulate: a crop does not cover its volume");
  const long long n = (long long)vol_dims[0] * vol_dims[1] * vol_dims[2];
  k_sym_accumulate<<<blocks_for(n, 256), 256, 0, (cudaStream_t)stream>>>(
      pred_sym, gs, pred_avg, g, vol_dims[0], vol_dims[1], vol_dims[2], t, weight, accumulate ? 1 : 0);
  PVD_LAUNCH_CHECK("k_sym_accumulate");
  return PVD_OK;
}

extern "C" pvd_status pvd_unet_apply_correction(const pvd_unet_geom* geom, const float* pred, const float* dose_conv,
                                                const int* vol_dims, const int* origin, float sigma_max,
                                                float mu_clamp, float* dose_out, uint8_t* fallback,
                                                pvd_stream stream) {
  pvd_status st = geo_check(geom);
  if (st != PVD_OK) return st;
  if (!pred || !dose_conv || !vol_dims || !origin || !dose_out || !(mu_clamp > 0.f))
    return set_error(PVD_ERR_ARG, "pvd_unet_apply_correction: bad arguments");
  for (int i = 0; i < 3; ++i)
    if (vol_dims[i] < 1) return set_error(PVD_ERR_ARG, "pvd_unet_apply_correction: bad volume dims");
  const Geo g = make_geo(geom);
  const long long n = (long long)g.D * g.H * g.W;
  k_apply<<<blocks_for(n, 256), 256, 0, (cudaStream_t)stream>>>(pred, g, dose_conv, origin[0], origin[1], origin[2],
                                                               vol_dims[0], vol_dims[1], vol_dims[2], sigma_max,
                                                               mu_clamp, dose_out, fallback);
  PVD_LAUNCH_CHECK("k_apply");
  return PVD_OK;
}

extern "C" pvd_status pvd_unet_input_maxima(const float* activity, const float* density, const float* dose, int64_t n,
                                            float rho_min, float* maxima, pvd_stream stream) {
  if (!activity || !density || !dose || !maxima || n < 0) return set_error(PVD_ERR_ARG, "pvd_unet_input_maxima: bad arguments");
  PVD_CUDA_TRY(cudaMemsetAsync(maxima, 0, 2 * sizeof(float), (cudaStream_t)stream));
  if (n == 0) {
    k_input_scales<<<1, 1, 0, (cudaStream_t)stream>>>(maxima);
    PVD_LAUNCH_CHECK("k_input_scales");
    return PVD_OK;
  }
  const unsigned grid = (unsigned)std::min<long long>(blocks_for(n, 256), 4LL * sm_count());
  k_input_maxima<<<grid, 256, 0, (cudaStream_t)stream>>>(activity, density, dose, n, rho_min, maxima);
  PVD_LAUNCH_CHECK("k_input_maxima");
  k_input_scales<<<1, 1, 0, (cudaStream_t)stream>>>(maxima);
  PVD_LAUNCH_CHECK("k_input_scales");
  return PVD_OK;
}

extern "C" pvd_status pvd_adam_step(float* params, const float* grads, float* m, float* v, int64_t n, float lr,
                                    float beta1, float beta2, float eps, float weight_decay, int step,
                                    pvd_stream stream) {
  if (!params || !grads || !m || !v || n < 0 || step < 1) return set_error(PVD_ERR_ARG, "pvd_adam_step: bad arguments");
  if (n == 0) return PVD_OK;
  const float c1 = (float)(1.0 - std::pow((double)beta1, step));
  const float c2 = (float)(1.0 - std::pow((double)beta2, step));
  k_adam<<<blocks_for(n, 256), 256, 0, (cudaStream_t)stream>>>(params, grads, m, v, n, lr, beta1, beta2, eps,
                                                              weight_decay, c1, c2);
  PVD_LAUNCH_CHECK("k_adam");
  return PVD_OK;
}

namespace pvd {
namespace {
constexpr int kClipParts = 1024;

// partial sums of squares of contiguous chunks, each a fixed-order tree sum
__global__ void __launch_bounds__(256) k_sumsq_parts(const float* __restrict__ g, int64_t n, float* __restrict__ parts) {
  __shared__ double red[256];
  const int64_t chunk = (n + gridDim.x - 1) / gridDim.x;
  const int64_t i0 = (int64_t)blockIdx.x * chunk, i1 = min(n, i0 + chunk);
  double s = 0.0;
  for (int64_t i = i0 + threadIdx.x; i < i1; i += blockDim.x) s += (double)g[i] * (double)g[i];
  red[threadIdx.x] = s;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) parts[blockIdx.x] = (float)red[0];
}

// norm = sqrt(sum of the parts); limit = max_norm, lowered to spike_factor times the
// running mean of the (limited) norms when spike_factor > 0 (work[kClipParts + 2]);
// scale = min(1, limit / norm), counted in work[kClipParts + 3] when the running-mean
// limit bit; 0 (the step's gradient dropped) only for a non-finite norm.  A limited
// gradient keeps its direction: dropping it instead lets Adam's momentum carry the
// weights on, unopposed, when a rising loss makes every gradient look large.
__global__ void __launch_bounds__(kClipParts) k_clip_scale(float* __restrict__ work, float max_norm,
                                                           float spike_factor) {
  __shared__ double red[kClipParts];
  red[threadIdx.x] = (double)work[threadIdx.x];
  __syncthreads();
  for (int w = kClipParts / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    const double nrm = sqrt(red[0]);
    const float mean = work[kClipParts + 2];
    double limit = (double)max_norm;
    const bool adaptive = spike_factor > 0.f && mean > 0.f && (double)spike_factor * mean < limit;
    if (adaptive) limit = (double)spike_factor * mean;
    work[kClipParts] = (float)nrm;
    if (!isfinite(nrm)) {
      work[kClipParts + 1] = 0.f;
      work[kClipParts + 3] += 1.f;
    } else {
      work[kClipParts + 1] = (float)fmin(1.0, limit / fmax(nrm, 1e-30));
      if (adaptive && nrm > limit) work[kClipParts + 3] += 1.f;
      const float used = (float)fmin(nrm, limit);
      work[kClipParts + 2] = mean > 0.f ? 0.98f * mean + 0.02f * used : used;
    }
  }
}

__global__ void k_clip_apply(float* __restrict__ g, int64_t n, const float* __restrict__ work) {
  const float sc = work[kClipParts + 1];
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    g[i] = (sc == 0.f) ? 0.f : g[i] * sc;  // a non-finite gradient is dropped, not propagated
}
}  // namespace
}  // namespace pvd

extern "C" pvd_status pvd_grad_clip(float* grads, int64_t n, float max_norm, float spike_factor, float* work,
                                    pvd_stream stream) {
  if (!grads || !work || n < 0) return set_error(PVD_ERR_ARG, "pvd_grad_clip: bad arguments");
  if (!(max_norm > 0.f) || !std::isfinite(max_norm)) return set_error(PVD_ERR_ARG, "pvd_grad_clip: max_norm must be > 0");
  if (!(spike_factor >= 0.f) || !std::isfinite(spike_factor))
    return set_error(PVD_ERR_ARG, "pvd_grad_clip: spike_factor must be >= 0");
  if (n == 0) return PVD_OK;
  cudaStream_t st = (cudaStream_t)stream;
  k_sumsq_parts<<<kClipParts, 256, 0, st>>>(grads, n, work);
  PVD_LAUNCH_CHECK("k_sumsq_parts");
  k_clip_scale<<<1, kClipParts, 0, st>>>(work, max_norm, spike_factor);
  PVD_LAUNCH_CHECK("k_clip_scale");
  k_clip_apply<<<blocks_for(n, 256), 256, 0, st>>>(grads, n, work);
  PVD_LAUNCH_CHECK("k_clip_apply");
  return PVD_OK;
}

namespace pvd {
namespace {
// One warp waits, through the pipeline's own warp-wide bounded wait, on a barrier
// phase that nothing completes (no bulk copy or MMA is issued), and records the
// timeout like the load warp does.
__global__ void k_unet_wait_check(uint64_t limit_ns) {
  __shared__ uint64_t bar;
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);
    fence_mbar_init();
  }
  __syncthreads();
  if (!umma::warp_wait(&bar, 0, limit_ns)) {
    if ((threadIdx.x & 31) == 0) fail(ST_TIMEOUT_LOAD);
  }
}
}  // namespace

pvd_status unet_wait_check(unsigned long long limit_ns, cudaStream_t st) {
  k_unet_wait_check<<<1, 32, 0, st>>>(limit_ns);
  PVD_LAUNCH_CHECK("k_unet_wait_check");
  return PVD_OK;
}
}  // namespace pvd

extern "C" pvd_status pvd_unet_status(int* code, int reset) {
  if (!code) return set_error(PVD_ERR_ARG, "pvd_unet_status: null output");
  PVD_CUDA_TRY(cudaMemcpyFromSymbol(code, g_unet_status, sizeof(int)));
  if (reset) {
    const int z = 0;
    PVD_CUDA_TRY(cudaMemcpyToSymbol(g_unet_status, &z, sizeof(int)));
  }
  if (*code != 0) return set_error(PVD_ERR_TIMEOUT, "unet: a bounded tensor-core pipeline wait ran out (code " + std::to_string(*code) + ")");
  return PVD_OK;
}
