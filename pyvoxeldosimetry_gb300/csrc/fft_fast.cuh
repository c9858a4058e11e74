// Fast convolution pass kernels for FFT lengths L = A * B (A, B <= 32), built on
// the register four-step FFT of fft_reg.cuh.  One shared-memory exchange per
// 1D transform; column passes load global memory straight into registers
// (TXX consecutive complex columns = one 128-byte segment per row); row passes
// stage rows through shared memory for coalescing and for the two-real-rows-
// in-one-complex-transform packing.
//
// Instantiated for a fixed list of lengths (fft_fast_inst.cu); the plan uses
// them for every axis whose FFT length is in the list and the generic
// Stockham kernels otherwise.
#pragma once

#include "conv_types.cuh"
#include "fft_reg.cuh"
#include "tma.cuh"

namespace pvd {

constexpr int FTX = 16;        // transforms (columns / row pairs) per CTA
constexpr int FTXP = FTX + 1;  // padded stride of row-pass staging tiles
constexpr int FZ_SLOTS = 4;    // kernel slots per z-pass launch

__host__ __device__ constexpr int cmax(int a, int b) { return a > b ? a : b; }

typedef void (*KxFwdFn)(ActIn, float2*, int, int, int, const float2*);
typedef void (*KxInvFn)(XInvSet, const float*, int, int, int, int, int, float, const float2*);
typedef void (*KyFn)(ColSet, int, int, int, const float2*);
typedef void (*KzFn)(const float2*, OutSet, int, int, int, const float2*);
// TMA-staged persistent column passes
typedef void (*KtyFn)(const __grid_constant__ CUtensorMap, float2*, int, int, int, int, int, int, long long, int,
                      int, const float2*, int*);
typedef void (*KtzFn)(const __grid_constant__ CUtensorMap, OutSet, int, int, int, int, int, int, const float2*, int*);

constexpr unsigned long long TMA_WAIT_NS = 2000000000ull;  // a tile that has not landed after 2 s is an error

struct FastLen {
  int L, A, B, threads;
  size_t smem_col, smem_row, smem_z;
  KxFwdFn x_fwd;
  KxInvFn x_inv;
  KyFn y_fwd, y_inv;
  KzFn z;
  KtyFn ty_fwd, ty_inv;
  KtzFn tz;
};

// shared-memory layout helpers: twiddle table first (rounded to 2 float2 = 16 B)
__host__ __device__ constexpr int tw_slots(int L) { return (L + 1) & ~1; }

template <int L>
__device__ __forceinline__ void load_tw(float2* tw, const float2* __restrict__ twg, int nthreads) {
  for (int i = threadIdx.x; i < L; i += nthreads) tw[i] = twg[i];
}

// ---------------------------------------------------------------------------
// column pass (y axis): blockIdx.x = column tile, blockIdx.y = z slab,
// blockIdx.z = kernel slot.  Loads bypass L1 (ld.global.cg): the inverse pass
// writes its output over its own input.
// ---------------------------------------------------------------------------
template <int A, int B, bool INV>
__global__ void __launch_bounds__(FTX* cmax(A, B)) kf_y(ColSet io, int nin, int nout, int HS,
                                                         const float2* __restrict__ twg) {
  constexpr int L = A * B, NTH = FTX * cmax(A, B);
  extern __shared__ float2 sm[];
  float2* tw = sm;
  float2* ex = sm + tw_slots(L);
  const int c = threadIdx.x % FTX, j = threadIdx.x / FTX;
  const int kx0 = blockIdx.x * FTX;
  const float2* src = pick(io.in, blockIdx.z) + (long long)blockIdx.y * io.in_slab + kx0 + c;
  float2* dst = pick(io.out, blockIdx.z) + (long long)blockIdx.y * io.out_slab + kx0 + c;
  float2 v[B];
  if (j < A) {
    static_for<B>([&](auto ib) {
      constexpr int b = decltype(ib)::value;
      const int n = j + A * b;
      v[b] = (n < nin) ? __ldcg(src + (long long)n * HS) : make_float2(0.f, 0.f);
    });
  }
  load_tw<L>(tw, twg, NTH);
  __syncthreads();
  float2 w[A];
  four_step<A, B, INV, FTX, false>(v, w, ex, tw, c, j);
  if (j < B) {
    static_for<A>([&](auto iq) {
      constexpr int q = decltype(iq)::value;
      const int k = j + B * q;
      if (k < nout) dst[(long long)k * HS] = w[q];
    });
  }
}

// ---------------------------------------------------------------------------
// z pass: forward, spectrum multiply, inverse, crop — every kernel slot.
// blockIdx.x = column tile, blockIdx.y = ky.
// ---------------------------------------------------------------------------
// enough resident CTAs for ~960 threads per SM where the register arrays allow it
// without spilling (A + B <= 36 fits in 64 registers); the compiler's choice otherwise
__host__ __device__ constexpr int z_min_blocks(int a, int b) {
  return (a + b <= 36 && cmax(a, b) <= 20) ? 960 / (FTX * cmax(a, b)) : 1;
}

template <int A, int B>
__global__ void __launch_bounds__(FTX* cmax(A, B), z_min_blocks(A, B)) kf_z(const float2* __restrict__ in, OutSet os, int N0, int P1,
                                                         int HS, const float2* __restrict__ twg) {
  constexpr int L = A * B, NTH = FTX * cmax(A, B);
  extern __shared__ float2 sm[];
  float2* tw = sm;
  float2* ex = sm + tw_slots(L);
  float2* xs = ex + L * FTX;  // forward spectrum of the tile, kept for every slot
  const int c = threadIdx.x % FTX, j = threadIdx.x / FTX;
  const int kx0 = blockIdx.x * FTX;
  const int ky = blockIdx.y;
  const long long zstride = (long long)P1 * HS;
  const long long base = (long long)ky * HS + kx0 + c;
  float2 v[B];
  if (j < A) {
    static_for<B>([&](auto ib) {
      constexpr int b = decltype(ib)::value;
      const int n = j + A * b;
      v[b] = (n < N0) ? in[n * zstride + base] : make_float2(0.f, 0.f);
    });
  }
  load_tw<L>(tw, twg, NTH);
  __syncthreads();
  {
    float2 X[A];
    four_step<A, B, false, FTX, false>(v, X, ex, tw, c, j);
    if (j < B) {
      static_for<A>([&](auto iq) {
        constexpr int q = decltype(iq)::value;
        xs[(j + B * q) * FTX + c] = X[q];
      });
    }
  }
  // kernel slots of this launch, unrolled so the slot arguments stay in the
  // parameter bank; the forward spectrum is re-read from shared memory per
  // slot (each thread reads back what it wrote), which keeps registers low
  static_for<FZ_SLOTS>([&](auto is) {
    constexpr int sl = decltype(is)::value;
    if (sl < os.n) {
      float2 X[A], Y[A];
      if (j < B) {
        static_for<A>([&](auto iq) {
          constexpr int q = decltype(iq)::value;
          X[q] = xs[(j + B * q) * FTX + c];
        });
        if (os.mode[sl] == SPEC_REAL_EVEN) {
          const float* S = (const float*)os.s[sl];
          static_for<A>([&](auto iq) {
            constexpr int q = decltype(iq)::value;
            const int kz = j + B * q;
            const int kzq = min(kz, os.P0 - kz), kyq = min(ky, P1 - ky);
            Y[q] = cscale(X[q], __ldg(S + ((long long)kzq * os.P1h + kyq) * HS + kx0 + c));
          });
        } else {
          const float2* S = (const float2*)os.s[sl];
          static_for<A>([&](auto iq) {
            constexpr int q = decltype(iq)::value;
            const int kz = j + B * q;
            Y[q] = cmul(X[q], __ldg(S + ((long long)kz * P1 + ky) * HS + kx0 + c));
          });
        }
      }
      __syncthreads();  // previous exchange reads are done
      float2 Z[B];
      four_step<B, A, true, FTX, false>(Y, Z, ex, tw, c, j);
      if (j < A) {
        float2* dst = os.p[sl] + base;
        static_for<B>([&](auto ir) {
          constexpr int r = decltype(ir)::value;
          const int z = j + A * r;
          if (z < N0) dst[z * zstride] = Z[r];
        });
      }
    }
  });
}

// ---------------------------------------------------------------------------
// TMA-staged persistent column passes.  Each CTA walks tiles t = blockIdx.x,
// blockIdx.x + gridDim.x, ...; while it transforms tile t from one shared
// stage, one elected thread has already issued the bulk tensor load of the
// next tile into the other stage (mbarrier-completed), so HBM latency overlaps
// the FFT arithmetic.  A stage is (chunks * boxr) rows of FTX complex (128 B
// per row), at least L rows so it can double as the exchange tile.  Waits are
// bounded: a load that has not landed after TMA_WAIT_NS sets *err and the CTA
// leaves.
// ---------------------------------------------------------------------------
// Every chunk of a stage starts at a multiple of one 128-byte row, the alignment
// bulk tensor copies need for their shared-memory destination.
static_assert(FTX * sizeof(float2) % 128 == 0, "TMA stage rows must be multiples of 128 bytes");

// Bounded wait of the whole CTA for a TMA stage's barrier phase.  On timeout every
// thread learns of it and thread 0 records PVD_ERR_TIMEOUT in *err (read by
// pvd_plan_status); the caller then leaves the kernel.
__device__ __forceinline__ bool cta_stage_wait(uint64_t* bar, uint32_t parity, uint64_t limit_ns, int* err) {
  const bool ok = mbar_wait_bounded(bar, parity, limit_ns);
  if (__syncthreads_or(!ok)) {
    if (threadIdx.x == 0) atomicExch(err, (int)PVD_ERR_TIMEOUT);
    return false;
  }
  return true;
}

__device__ __forceinline__ void tma_issue_rows(float2* dst, const CUtensorMap* map, int c0, int c2_or_row,
                                               bool rows_on_dim1, int chunks, int boxr, uint64_t* bar) {
  fence_proxy_async_shared();
  mbar_arrive_expect_tx(bar, (uint32_t)(chunks * boxr * FTX * sizeof(float2)));
  for (int k = 0; k < chunks; ++k) {
    if (rows_on_dim1)
      tma_load_3d(dst + k * boxr * FTX, map, c0, k * boxr, c2_or_row, bar);
    else
      tma_load_3d(dst + k * boxr * FTX, map, c0, c2_or_row, k * boxr, bar);
  }
}

// y pass: tiles (column tile, z slab) of a [nslab][nin][HS] tensor -> [nslab][nout][HS]
template <int A, int B, bool INV>
__global__ void __launch_bounds__(FTX* cmax(A, B)) kt_y(const __grid_constant__ CUtensorMap tin,
                                                         float2* __restrict__ out, int nin, int nout, int slab0,
                                                         int nslab, int ctiles, int HS, long long out_slab,
                                                         int chunks, int boxr, const float2* __restrict__ twg,
                                                         int* __restrict__ err) {
  constexpr int L = A * B, NTH = FTX * cmax(A, B);
  extern __shared__ __align__(128) float2 sm[];
  const int SR = max(chunks * boxr, L);
  float2* tw = sm + 2 * SR * FTX;
  uint64_t* bar = reinterpret_cast<uint64_t*>(tw + tw_slots(L));
  const int c = threadIdx.x % FTX, j = threadIdx.x / FTX;
  const int total = ctiles * nslab;
  if (threadIdx.x == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    fence_mbar_init();
  }
  load_tw<L>(tw, twg, NTH);
  __syncthreads();
  int t = blockIdx.x;
  if (threadIdx.x == 0 && t < total)
    tma_issue_rows(sm, &tin, (t % ctiles) * FTX, slab0 + t / ctiles, true, chunks, boxr, &bar[0]);
  for (int i = 0; t < total; ++i, t += gridDim.x) {
    const int s = i & 1;
    const int tn = t + gridDim.x;
    if (threadIdx.x == 0 && tn < total)
      tma_issue_rows(sm + (s ^ 1) * SR * FTX, &tin, (tn % ctiles) * FTX, slab0 + tn / ctiles, true, chunks, boxr,
                     &bar[s ^ 1]);
    if (!cta_stage_wait(&bar[s], (i >> 1) & 1, TMA_WAIT_NS, err)) return;
    float2* stage = sm + s * SR * FTX;
    float2 v[B];
    if (j < A) {
      static_for<B>([&](auto ib) {
        constexpr int b = decltype(ib)::value;
        const int n = j + A * b;
        v[b] = (n < nin) ? stage[n * FTX + c] : make_float2(0.f, 0.f);
      });
    }
    float2 w[A];
    four_step<A, B, INV, FTX, true>(v, w, stage, tw, c, j);
    float2* dst = out + (long long)(slab0 + t / ctiles) * out_slab + (t % ctiles) * FTX + c;
    if (j < B) {
      static_for<A>([&](auto iq) {
        constexpr int q = decltype(iq)::value;
        const int k = j + B * q;
        if (k < nout) dst[(long long)k * HS] = w[q];
      });
    }
    __syncthreads();  // the stage (also the exchange tile) is free for the load after next
  }
}

// z pass: tiles (column tile, ky) of a [N0][P1][HS] tensor, rows along z
template <int A, int B>
__global__ void __launch_bounds__(FTX* cmax(A, B), z_min_blocks(A, B)) kt_z(const __grid_constant__ CUtensorMap tin,
                                                                            OutSet os, int N0, int P1, int HS,
                                                                            int ctiles, int chunks, int boxr,
                                                                            const float2* __restrict__ twg,
                                                                            int* __restrict__ err) {
  constexpr int L = A * B, NTH = FTX * cmax(A, B);
  extern __shared__ __align__(128) float2 sm[];
  const int SR = max(chunks * boxr, L);
  float2* ex = sm + 2 * SR * FTX;
  float2* tw = ex + L * FTX;
  uint64_t* bar = reinterpret_cast<uint64_t*>(tw + tw_slots(L));
  const int c = threadIdx.x % FTX, j = threadIdx.x / FTX;
  const int total = ctiles * P1;
  const long long zstride = (long long)P1 * HS;
  if (threadIdx.x == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    fence_mbar_init();
  }
  load_tw<L>(tw, twg, NTH);
  __syncthreads();
  int t = blockIdx.x;
  if (threadIdx.x == 0 && t < total) tma_issue_rows(sm, &tin, (t % ctiles) * FTX, t / ctiles, false, chunks, boxr, &bar[0]);
  for (int i = 0; t < total; ++i, t += gridDim.x) {
    const int s = i & 1;
    const int tn = t + gridDim.x;
    if (threadIdx.x == 0 && tn < total)
      tma_issue_rows(sm + (s ^ 1) * SR * FTX, &tin, (tn % ctiles) * FTX, tn / ctiles, false, chunks, boxr,
                     &bar[s ^ 1]);
    if (!cta_stage_wait(&bar[s], (i >> 1) & 1, TMA_WAIT_NS, err)) return;
    float2* stage = sm + s * SR * FTX;
    const int kx0 = (t % ctiles) * FTX, ky = t / ctiles;
    const long long base = (long long)ky * HS + kx0 + c;
    float2 v[B];
    if (j < A) {
      static_for<B>([&](auto ib) {
        constexpr int b = decltype(ib)::value;
        const int n = j + A * b;
        v[b] = (n < N0) ? stage[n * FTX + c] : make_float2(0.f, 0.f);
      });
    }
    {
      float2 X[A];
      four_step<A, B, false, FTX, false>(v, X, ex, tw, c, j);
      // every stage read happened before four_step's barrier: the stage now keeps the spectrum
      if (j < B) {
        static_for<A>([&](auto iq) {
          constexpr int q = decltype(iq)::value;
          stage[(j + B * q) * FTX + c] = X[q];
        });
      }
    }
    static_for<FZ_SLOTS>([&](auto is) {
      constexpr int sl = decltype(is)::value;
      if (sl < os.n) {
        float2 X[A], Y[A];
        if (j < B) {
          static_for<A>([&](auto iq) {
            constexpr int q = decltype(iq)::value;
            X[q] = stage[(j + B * q) * FTX + c];
          });
          if (os.mode[sl] == SPEC_REAL_EVEN) {
            const float* S = (const float*)os.s[sl];
            static_for<A>([&](auto iq) {
              constexpr int q = decltype(iq)::value;
              const int kz = j + B * q;
              const int kzq = min(kz, os.P0 - kz), kyq = min(ky, P1 - ky);
              Y[q] = cscale(X[q], __ldg(S + ((long long)kzq * os.P1h + kyq) * HS + kx0 + c));
            });
          } else {
            const float2* S = (const float2*)os.s[sl];
            static_for<A>([&](auto iq) {
              constexpr int q = decltype(iq)::value;
              const int kz = j + B * q;
              Y[q] = cmul(X[q], __ldg(S + ((long long)kz * P1 + ky) * HS + kx0 + c));
            });
          }
        }
        __syncthreads();  // previous exchange reads are done
        float2 Z[B];
        four_step<B, A, true, FTX, false>(Y, Z, ex, tw, c, j);
        if (j < A) {
          float2* dst = os.p[sl] + base;
          static_for<B>([&](auto ir) {
            constexpr int r = decltype(ir)::value;
            const int z = j + A * r;
            if (z < N0) dst[z * zstride] = Z[r];
          });
        }
      }
    });
    __syncthreads();  // stage and exchange free
  }
}

// shared bytes of the TMA passes (stages of SR rows, twiddles, two barriers)
inline size_t tma_y_smem(int L, int chunks, int boxr) {
  const int SR = chunks * boxr > L ? chunks * boxr : L;
  return sizeof(float2) * ((size_t)2 * SR * FTX + tw_slots(L)) + 2 * sizeof(uint64_t);
}
inline size_t tma_z_smem(int L, int chunks, int boxr) {
  const int SR = chunks * boxr > L ? chunks * boxr : L;
  return sizeof(float2) * ((size_t)2 * SR * FTX + (size_t)L * FTX + tw_slots(L)) + 2 * sizeof(uint64_t);
}

// ---------------------------------------------------------------------------
// Row passes (x axis, contiguous).  A CTA owns ROWS = 2*FTX consecutive rows:
// a contiguous block of global memory, moved with fully coalesced loads that
// keep all of a row's loads per lane in flight (trip counts are compile-time,
// from L).  Shared tiles use odd row strides so the
// transposed per-transform reads of the four-step FFT are bank-conflict free.
// Real rows 2m and 2m+1 form the real and imaginary part of transform m.
// ---------------------------------------------------------------------------

// x forward: weighted timepoint sum, zero pad, R2C, half spectra [row][HS].
// row passes of up to 320 threads keep ~1280 threads resident per SM (4 CTAs of
// 320: <= 51 registers); larger tiles are left to the compiler
__host__ __device__ constexpr int x_min_blocks(int a, int b) {
  return FTX * cmax(a, b) <= 320 ? 1280 / (FTX * cmax(a, b)) : 1;
}

template <int A, int B>
__global__ void __launch_bounds__(FTX* cmax(A, B), x_min_blocks(A, B)) kf_x_fwd(ActIn in, float2* __restrict__ out, int nrows, int N2,
                                                             int HS, const float2* __restrict__ twg) {
  constexpr int L = A * B, NTH = FTX * cmax(A, B), H = L / 2 + 1, ROWS = 2 * FTX;
  constexpr int NWF = NTH / 32;  // full warps (the last warp is partial when max(A, B) is odd)
  constexpr int S2 = L | 1;  // odd float2 stride of the spectrum tile
  extern __shared__ float2 sm[];
  float2* tw = sm;
  float2* buf = sm + tw_slots(L);               // chunk / exchange / spectrum tile (aliased in turn)
  float* chunk = reinterpret_cast<float*>(buf);  // [ROWS][S] real rows
  const int S = N2 | 1;
  const long long row0 = (long long)blockIdx.x * ROWS;
  const int nr = (int)min((long long)ROWS, (long long)nrows - row0);
  load_tw<L>(tw, twg, NTH);
  // whole warps take whole rows: lane-contiguous loads, the row's loads all in flight
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  constexpr int NU = (L + 31) / 32;  // N2 <= L: row slots per lane
  if (warp < NWF) {
    for (int rr = warp; rr < nr; rr += NWF) {
      float r[NU];
      if (in.n == 1) {  // one activity map (the common case): asynchronous copies, all rows in flight
        const float* src = in.p[0] + (row0 + rr) * N2;
#pragma unroll
        for (int u = 0; u < NU; ++u) {
          const int n = 32 * u + lane;
          if (n < N2) cp_async4(chunk + rr * S + n, src + n);
        }
        continue;
      } else {
#pragma unroll
        for (int u = 0; u < NU; ++u) r[u] = 0.f;
        for (int t = 0; t < in.n; ++t) {
          const float* src = in.p[t] + (row0 + rr) * N2;
          const float w = in.w[t];
#pragma unroll
          for (int u = 0; u < NU; ++u) {
            const int n = 32 * u + lane;
            if (n < N2) r[u] += w * __ldg(src + n);
          }
        }
      }
#pragma unroll
      for (int u = 0; u < NU; ++u) {
        const int n = 32 * u + lane;
        if (n < N2) chunk[rr * S + n] = r[u];
      }
    }
  }
  cp_async_wait_all();
  __syncthreads();
  const int c = threadIdx.x % FTX, j = threadIdx.x / FTX;
  float2 v[B];
  if (j < A) {
    const bool va = 2 * c < nr, vb = 2 * c + 1 < nr;
    static_for<B>([&](auto ib) {
      constexpr int b = decltype(ib)::value;
      const int n = j + A * b;
      float xa = 0.f, xb = 0.f;
      if (n < N2) {
        if (va) xa = chunk[(2 * c) * S + n];
        if (vb) xb = chunk[(2 * c + 1) * S + n];
      }
      v[b] = make_float2(xa, xb);
    });
  }
  float2 X[A];
  four_step<A, B, false, FTX, true>(v, X, buf, tw, c, j);
  __syncthreads();
  if (j < B) {
    static_for<A>([&](auto iq) {
      constexpr int q = decltype(iq)::value;
      buf[c * S2 + j + B * q] = X[q];
    });
  }
  __syncthreads();
  if (warp < NWF) {
    for (int rr = warp; rr < nr; rr += NWF) {
      const int m = rr >> 1;
      const bool odd = rr & 1;
      float2* dst = out + (row0 + rr) * HS;
      constexpr int KU = (H + 31) / 32;
#pragma unroll
      for (int u = 0; u < KU; ++u) {
        const int k = 32 * u + lane;
        if (k < H) {
          const float2 z1 = buf[m * S2 + k];
          const float2 z2 = buf[m * S2 + (k ? L - k : 0)];
          // Xa = (Z[k] + conj Z[-k]) / 2 ;  Xb = (Z[k] - conj Z[-k]) / (2i)
          dst[k] = odd ? make_float2(0.5f * (z1.y + z2.y), -0.5f * (z1.x - z2.x))
                       : make_float2(0.5f * (z1.x + z2.x), 0.5f * (z1.y - z2.y));
        }
      }
    }
  }
}

// x inverse: C2R of pairs of half-spectrum rows, crop, scale, density, for up to
// XINV_SLOTS kernel slots in turn (one launch per row block and slot group: the
// twiddles are loaded once and the density rows come from HBM once, the later
// slots finding them in cache).  Row r = z * N1 + y of slot s is read at
// io.in[s] + (z * pitch + y) * HS.
template <int A, int B>
__global__ void __launch_bounds__(FTX* cmax(A, B), x_min_blocks(A, B)) kf_x_inv(XInvSet io, const float* __restrict__ rho,
                                                             int nrows, int N1, int pitch, int N2, int HS,
                                                             float scale, const float2* __restrict__ twg) {
  constexpr int L = A * B, NTH = FTX * cmax(A, B), H = L / 2 + 1, ROWS = 2 * FTX;
  constexpr int NWF = NTH / 32;  // full warps (the last warp is partial when max(A, B) is odd)
  constexpr int S2 = H | 1;  // odd float2 stride of the half-spectrum tiles
  extern __shared__ float2 sm[];
  float2* tw = sm;
  float2* buf = sm + tw_slots(L);
  float2* ha = buf;              // even rows  [FTX][S2]
  float2* hb = buf + FTX * S2;   // odd rows   [FTX][S2]
  float* oc = reinterpret_cast<float*>(buf);  // output rows [ROWS][S] (aliases the tiles later)
  const int S = N2 | 1;
  const long long row0 = (long long)blockIdx.x * ROWS;
  const int nr = (int)min((long long)ROWS, (long long)nrows - row0);
  __shared__ long long roff[ROWS];  // element offset of each row of the tile in a slot's buffer
  if (threadIdx.x < ROWS) {         // rows of a launch fit in 32 bits (n0 n1 <= 4096^2)
    const int r = (int)row0 + threadIdx.x, z = r / N1;
    roff[threadIdx.x] = ((long long)z * pitch + (r - z * N1)) * HS;
  }
  load_tw<L>(tw, twg, NTH);
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int c = threadIdx.x % FTX, j = threadIdx.x / FTX;
  static_for<XINV_SLOTS>([&](auto is) {
    constexpr int sl = decltype(is)::value;
    if (sl < io.n) {
      const float2* in = io.in[sl];
      // every row of the tile in flight at once: asynchronous copies straight into shared memory
      if (warp < NWF) {
        for (int rr = warp; rr < nr; rr += NWF) {
          const float2* src = in + roff[rr];
          float2* dsm = ((rr & 1) ? hb : ha) + (rr >> 1) * S2;
          constexpr int KU = (H + 31) / 32;
#pragma unroll
          for (int u = 0; u < KU; ++u) {
            const int k = 32 * u + lane;
            if (k < H) cp_async8(dsm + k, src + k);
          }
        }
      }
      cp_async_wait_all();
      __syncthreads();
      float2 v[B];
      if (j < A) {
        const bool va = 2 * c < nr, vb = 2 * c + 1 < nr;
        static_for<B>([&](auto ib) {
          constexpr int b = decltype(ib)::value;
          const int n = j + A * b;
          const bool lo = n < H;
          const int k = lo ? n : L - n;
          float2 xa = va ? ha[c * S2 + k] : make_float2(0.f, 0.f);
          float2 xb = vb ? hb[c * S2 + k] : make_float2(0.f, 0.f);
          if (k == 0 || 2 * k == L) {  // DC / Nyquist bins of a real row are real
            xa.y = 0.f;
            xb.y = 0.f;
          }
          // Z[n] = Xa[n] + i Xb[n] for n < H, conj Xa[L-n] + i conj Xb[L-n] above
          v[b] = lo ? make_float2(xa.x - xb.y, xa.y + xb.x) : make_float2(xa.x + xb.y, xb.x - xa.y);
        });
      }
      float2 X[A];
      four_step<A, B, true, FTX, true>(v, X, buf, tw, c, j);
      __syncthreads();
      if (j < B) {
        static_for<A>([&](auto iq) {
          constexpr int q = decltype(iq)::value;
          const int n = j + B * q;
          if (n < N2) {
            oc[(2 * c) * S + n] = X[q].x * scale;
            oc[(2 * c + 1) * S + n] = X[q].y * scale;
          }
        });
      }
      __syncthreads();
      if (warp < NWF) {
        float* out = io.out[sl];
        for (int rr = warp; rr < nr; rr += NWF) {
          float* dst = out + (row0 + rr) * N2;
          const float* dr = rho ? rho + (row0 + rr) * N2 : nullptr;
          constexpr int NU = (L + 31) / 32;  // N2 <= L
          float d[NU];
          if (dr) {
#pragma unroll
            for (int u = 0; u < NU; ++u) {
              const int n = 32 * u + lane;
              d[u] = (n < N2) ? __ldg(dr + n) : 1.f;
            }
          }
#pragma unroll
          for (int u = 0; u < NU; ++u) {
            const int n = 32 * u + lane;
            if (n < N2) {
              float val = oc[rr * S + n];
              // 2-ulp division (x * rcp.approx(d)): far inside the 1e-5 parity bound, and a
              // fraction of the instructions of a correctly rounded one
              if (dr) val = (d[u] > 0.f) ? __fdividef(val, d[u]) : 0.f;
              dst[n] = val;
            }
          }
        }
      }
      __syncthreads();  // the output tile (aliasing the row tiles) is read out before the next slot's rows land
    }
  });
}

template <int A, int B>
FastLen make_fast_len() {
  constexpr int L = A * B;
  FastLen f;
  f.L = L;
  f.A = A;
  f.B = B;
  f.threads = FTX * cmax(A, B);
  f.smem_col = sizeof(float2) * (size_t)(tw_slots(L) + L * FTX);
  f.smem_z = sizeof(float2) * (size_t)(tw_slots(L) + 2 * L * FTX);
  f.smem_row = sizeof(float2) * (size_t)(tw_slots(L) + L * FTXP);
  f.x_fwd = kf_x_fwd<A, B>;
  f.x_inv = kf_x_inv<A, B>;
  f.y_fwd = kf_y<A, B, false>;
  f.y_inv = kf_y<A, B, true>;
  f.z = kf_z<A, B>;
  f.ty_fwd = kt_y<A, B, false>;
  f.ty_inv = kt_y<A, B, true>;
  f.tz = kt_z<A, B>;
  return f;
}

// Registry of instantiated lengths (fft_fast_inst.cu); nullptr if L is not fast.
const FastLen* fast_len(int L);
// Smallest fast length >= n, or 0 if none.
int fast_len_at_least(int n);

}  // namespace pvd
