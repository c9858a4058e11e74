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

namespace pvd {

constexpr int FTX = 16;        // transforms per CTA
constexpr int FTXP = FTX + 1;  // padded stride of row-pass staging tiles
constexpr int FZ_SLOTS = 4;    // kernel slots per z-pass launch

__host__ __device__ constexpr int cmax(int a, int b) { return a > b ? a : b; }

typedef void (*KxFwdFn)(ActIn, float2*, int, int, int, const float2*);
typedef void (*KxInvFn)(const float2*, float*, const float*, int, int, int, float, const float2*);
typedef void (*KyFn)(const float2*, float2*, int, int, int, const float2*);
typedef void (*KzFn)(const float2*, OutSet, int, int, int, const float2*);

struct FastLen {
  int L, A, B, threads;
  size_t smem_col, smem_row;
  KxFwdFn x_fwd;
  KxInvFn x_inv;
  KyFn y_fwd, y_inv;
  KzFn z;
};

// shared-memory layout helpers: twiddle table first (rounded to 2 float2 = 16 B)
__host__ __device__ constexpr int tw_slots(int L) { return (L + 1) & ~1; }

template <int L>
__device__ __forceinline__ void load_tw(float2* tw, const float2* __restrict__ twg, int nthreads) {
  for (int i = threadIdx.x; i < L; i += nthreads) tw[i] = twg[i];
}

// ---------------------------------------------------------------------------
// column pass (y axis): blockIdx.x = column tile, blockIdx.y = z slab
// ---------------------------------------------------------------------------
template <int A, int B, bool INV>
__global__ void __launch_bounds__(FTX* cmax(A, B)) kf_y(const float2* __restrict__ in, float2* __restrict__ out,
                                                         int nin, int nout, int HS, const float2* __restrict__ twg) {
  constexpr int L = A * B, NTH = FTX * cmax(A, B);
  extern __shared__ float2 sm[];
  float2* tw = sm;
  float2* ex = sm + tw_slots(L);
  const int c = threadIdx.x % FTX, j = threadIdx.x / FTX;
  const int kx0 = blockIdx.x * FTX;
  const float2* src = in + (long long)blockIdx.y * nin * HS + kx0 + c;
  float2* dst = out + (long long)blockIdx.y * nout * HS + kx0 + c;
  float2 v[B];
  if (j < A) {
    static_for<B>([&](auto ib) {
      constexpr int b = decltype(ib)::value;
      const int n = j + A * b;
      v[b] = (n < nin) ? src[(long long)n * HS] : make_float2(0.f, 0.f);
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
template <int A, int B>
__global__ void __launch_bounds__(FTX* cmax(A, B)) kf_z(const float2* __restrict__ in, OutSet os, int N0, int P1,
                                                         int HS, const float2* __restrict__ twg) {
  constexpr int L = A * B, NTH = FTX * cmax(A, B);
  extern __shared__ float2 sm[];
  float2* tw = sm;
  float2* ex = sm + tw_slots(L);
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
  float2 X[A];
  four_step<A, B, false, FTX, false>(v, X, ex, tw, c, j);
  // kernel slots [s0, s0 + FZ_SLOTS) of this launch, unrolled so the slot
  // arguments stay in the parameter bank
  static_for<FZ_SLOTS>([&](auto is) {
    constexpr int sl = decltype(is)::value;
    if (sl < os.n) {
      float2 Y[A];
      if (j < B) {
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
// x forward: weighted timepoint sum, zero pad, R2C of 2*FTX real rows packed
// as FTX complex rows, written as [row][HS] half spectra.
// ---------------------------------------------------------------------------
template <int A, int B>
__global__ void __launch_bounds__(FTX* cmax(A, B)) kf_x_fwd(ActIn in, float2* __restrict__ out, int nrows, int N2,
                                                             int HS, const float2* __restrict__ twg) {
  constexpr int L = A * B, NTH = FTX * cmax(A, B), H = L / 2 + 1;
  extern __shared__ float2 sm[];
  float2* tw = sm;
  float2* buf = sm + tw_slots(L);  // [L][FTXP] staging, also the exchange tile
  const long long row0 = (long long)blockIdx.x * (2 * FTX);
  load_tw<L>(tw, twg, NTH);
  for (int idx = threadIdx.x; idx < FTX * L; idx += NTH) {
    const int m = idx / L, n = idx - m * L;
    float2 val = make_float2(0.f, 0.f);
    if (n < N2) {
      const long long ra = row0 + 2 * m, rb = ra + 1;
      if (ra < nrows) {
        const long long o = ra * N2 + n;
        float s = 0.f;
        for (int t = 0; t < in.n; ++t) s += in.w[t] * __ldg(in.p[t] + o);
        val.x = s;
      }
      if (rb < nrows) {
        const long long o = rb * N2 + n;
        float s = 0.f;
        for (int t = 0; t < in.n; ++t) s += in.w[t] * __ldg(in.p[t] + o);
        val.y = s;
      }
    }
    buf[n * FTXP + m] = val;
  }
  __syncthreads();
  const int c = threadIdx.x % FTX, j = threadIdx.x / FTX;
  float2 v[B];
  if (j < A) {
    static_for<B>([&](auto ib) {
      constexpr int b = decltype(ib)::value;
      v[b] = buf[(j + A * b) * FTXP + c];
    });
  }
  float2 X[A];
  four_step<A, B, false, FTX, true>(v, X, buf, tw, c, j);
  __syncthreads();
  if (j < B) {
    static_for<A>([&](auto iq) {
      constexpr int q = decltype(iq)::value;
      buf[(j + B * q) * FTXP + c] = X[q];
    });
  }
  __syncthreads();
  for (int idx = threadIdx.x; idx < FTX * H; idx += NTH) {
    const int m = idx / H, k = idx - m * H;
    const long long ra = row0 + 2 * m, rb = ra + 1;
    const int kk = (k == 0) ? 0 : L - k;
    const float2 z1 = buf[k * FTXP + m];
    const float2 z2 = buf[kk * FTXP + m];
    if (ra < nrows) out[ra * HS + k] = make_float2(0.5f * (z1.x + z2.x), 0.5f * (z1.y - z2.y));
    if (rb < nrows) out[rb * HS + k] = make_float2(0.5f * (z1.y + z2.y), -0.5f * (z1.x - z2.x));
  }
}

// ---------------------------------------------------------------------------
// x inverse: C2R of pairs of half-spectrum rows, crop, scale, density.
// ---------------------------------------------------------------------------
template <int A, int B>
__global__ void __launch_bounds__(FTX* cmax(A, B)) kf_x_inv(const float2* __restrict__ in, float* __restrict__ out,
                                                             const float* __restrict__ rho, int nrows, int N2, int HS,
                                                             float scale, const float2* __restrict__ twg) {
  constexpr int L = A * B, NTH = FTX * cmax(A, B), H = L / 2 + 1;
  extern __shared__ float2 sm[];
  float2* tw = sm;
  float2* buf = sm + tw_slots(L);
  const long long row0 = (long long)blockIdx.x * (2 * FTX);
  load_tw<L>(tw, twg, NTH);
  for (int idx = threadIdx.x; idx < FTX * H; idx += NTH) {
    const int m = idx / H, k = idx - m * H;
    const long long ra = row0 + 2 * m, rb = ra + 1;
    float2 xa = (ra < nrows) ? in[ra * HS + k] : make_float2(0.f, 0.f);
    float2 xb = (rb < nrows) ? in[rb * HS + k] : make_float2(0.f, 0.f);
    if (k == 0 || 2 * k == L) {
      xa.y = 0.f;
      xb.y = 0.f;
    }
    buf[k * FTXP + m] = make_float2(xa.x - xb.y, xa.y + xb.x);
    const int kk = L - k;
    if (k > 0 && kk >= H) buf[kk * FTXP + m] = make_float2(xa.x + xb.y, xb.x - xa.y);
  }
  __syncthreads();
  const int c = threadIdx.x % FTX, j = threadIdx.x / FTX;
  float2 v[B];
  if (j < A) {
    static_for<B>([&](auto ib) {
      constexpr int b = decltype(ib)::value;
      v[b] = buf[(j + A * b) * FTXP + c];
    });
  }
  float2 X[A];
  four_step<A, B, true, FTX, true>(v, X, buf, tw, c, j);
  __syncthreads();
  if (j < B) {
    static_for<A>([&](auto iq) {
      constexpr int q = decltype(iq)::value;
      buf[(j + B * q) * FTXP + c] = X[q];
    });
  }
  __syncthreads();
  for (int idx = threadIdx.x; idx < FTX * N2; idx += NTH) {
    const int m = idx / N2, n = idx - m * N2;
    const long long ra = row0 + 2 * m, rb = ra + 1;
    const float2 z = buf[n * FTXP + m];
    if (ra < nrows) {
      float val = z.x * scale;
      if (rho) {
        const float d = __ldg(rho + ra * N2 + n);
        val = (d > 0.f) ? val / d : 0.f;
      }
      out[ra * N2 + n] = val;
    }
    if (rb < nrows) {
      float val = z.y * scale;
      if (rho) {
        const float d = __ldg(rho + rb * N2 + n);
        val = (d > 0.f) ? val / d : 0.f;
      }
      out[rb * N2 + n] = val;
    }
  }
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
  f.smem_row = sizeof(float2) * (size_t)(tw_slots(L) + L * FTXP);
  f.x_fwd = kf_x_fwd<A, B>;
  f.x_inv = kf_x_inv<A, B>;
  f.y_fwd = kf_y<A, B, false>;
  f.y_inv = kf_y<A, B, true>;
  f.z = kf_z<A, B>;
  return f;
}

// Registry of instantiated lengths (fft_fast_inst.cu); nullptr if L is not fast.
const FastLen* fast_len(int L);
// Smallest fast length >= n, or 0 if none.
int fast_len_at_least(int n);

}  // namespace pvd
