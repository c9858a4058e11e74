// Dose-point-kernel convolution as a pruned, fused 3D real FFT pipeline.
//
// Replaces the reference operator
//   np.fft.ifftn(np.fft.fftn(A) * np.fft.fftn(K, A.shape)).real
// (pyvoxeldosimetry/core/kernel_convolution.py:71-74) with five passes over
// HBM, each a batch of 1D mixed-radix (2,3,4,5,7,8) Stockham FFTs done in
// shared memory:
//
//   pass 1  x  : weighted sum of timepoints -> zero-pad -> R2C      act  -> B1[N0][N1][HS]
//   pass 2  y  : zero-pad -> C2C forward                            B1   -> B2[N0][P1][HS]
//   pass 3  z  : zero-pad -> C2C forward -> * S_k -> C2C inverse     B2   -> B3_k[N0][P1][HS]
//                -> crop     (one forward, one multiply+inverse per kernel slot k)
//   pass 4  y  : C2C inverse -> crop                                B3_k -> B1[N0][N1][HS]
//   pass 5  x  : C2R -> crop -> * out_scale / rho                   B1   -> dose_k[N0][N1][N2]
//
// Axis 2 (x) is the contiguous axis of the C-ordered volume.  Zero padding is
// never materialised: rows that are all zero are skipped (pruned) and the pad
// region of each transform is filled in shared memory.  Two real rows are
// packed into one complex transform on the x axis.
//
// Kernel placement: LINEAR mode puts kernel index m at padded index
// (m - k//2) mod P (kernel centred at the origin) so the output needs no shift
// and a symmetric kernel has a real spectrum; CIRCULAR mode puts it at m
// (the reference's corner placement, truncated to P) which reproduces the
// reference's K//2 output shift exactly.
#include <cudaTypedefs.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "conv_types.cuh"
#include "fft_fast.cuh"
#include "pvd_common.cuh"

namespace pvd {

constexpr int TX = 16;        // transforms (columns) per CTA
constexpr int TXP = TX + 1;   // padded shared-memory row stride (complex)
constexpr int NT = 256;       // threads per CTA
constexpr int NL = NT / TX;   // lanes per transform
constexpr int MAX_STAGES = 16;
constexpr int PVD_HOST_CHUNKS = 4;  // activity upload chunks overlapped with the forward passes
constexpr int PVD_DOSE_CHUNKS = 4;  // density upload / inverse-x / dose copy-back chunks (z ranges)

struct FftLen {
  int L;
  int nst;
  int rad[MAX_STAGES];
};

// ---------------------------------------------------------------------------
// host-side length helpers
// ---------------------------------------------------------------------------
static bool factorize(int L, FftLen* f) {
  f->L = L;
  f->nst = 0;
  int r = L;
  std::vector<int> rad;
  while (r % 8 == 0) { rad.push_back(8); r /= 8; }
  while (r % 4 == 0) { rad.push_back(4); r /= 4; }
  while (r % 2 == 0) { rad.push_back(2); r /= 2; }
  while (r % 3 == 0) { rad.push_back(3); r /= 3; }
  while (r % 5 == 0) { rad.push_back(5); r /= 5; }
  while (r % 7 == 0) { rad.push_back(7); r /= 7; }
  if (r != 1 || (int)rad.size() > MAX_STAGES) return false;
  for (size_t i = 0; i < rad.size(); ++i) f->rad[i] = rad[i];
  f->nst = (int)rad.size();
  return true;
}

static bool is_smooth7(int n) {
  if (n < 1) return false;
  for (int p : {2, 3, 5, 7})
    while (n % p == 0) n /= p;
  return n == 1;
}

static int next_smooth7(int n) {
  int m = std::max(n, 1);
  while (!is_smooth7(m)) ++m;
  return m;
}

// ---------------------------------------------------------------------------
// device: Stockham stage and tile FFT along the row index of a [L][TXP] tile
// ---------------------------------------------------------------------------
template <int R, bool INV>
__device__ __forceinline__ void stockham_stage(const float2* __restrict__ a, float2* __restrict__ b, int L, int ns,
                                               const float2* __restrict__ tw, int col, int lane) {
  const int m = L / R;
  const int tstep = L / (ns * R);
  for (int j = lane; j < m; j += NL) {
    const int k = j % ns;
    float2 v[R];
#pragma unroll
    for (int q = 0; q < R; ++q) v[q] = a[(j + q * m) * TXP + col];
    if (ns > 1) {
#pragma unroll
      for (int q = 1; q < R; ++q) {
        float2 w = tw[q * k * tstep];
        if (INV) w.y = -w.y;
        v[q] = cmul(v[q], w);
      }
    }
    Dft<R, INV>::run(v);
    const int base = (j - k) * R + k;
#pragma unroll
    for (int q = 0; q < R; ++q) b[(base + q * ns) * TXP + col] = v[q];
  }
}

// FFT of TX columns of length f.L held in `a`; ping-pongs with `b`; returns
// the buffer holding the natural-order result.  Caller syncs before the call.
template <bool INV>
__device__ float2* fft_tile(float2* a, float2* b, const FftLen& f, const float2* tw) {
  const int col = threadIdx.x % TX;
  const int lane = threadIdx.x / TX;
  int ns = 1;
  for (int s = 0; s < f.nst; ++s) {
    const int r = f.rad[s];
    switch (r) {
      case 2: stockham_stage<2, INV>(a, b, f.L, ns, tw, col, lane); break;
      case 3: stockham_stage<3, INV>(a, b, f.L, ns, tw, col, lane); break;
      case 4: stockham_stage<4, INV>(a, b, f.L, ns, tw, col, lane); break;
      case 5: stockham_stage<5, INV>(a, b, f.L, ns, tw, col, lane); break;
      case 7: stockham_stage<7, INV>(a, b, f.L, ns, tw, col, lane); break;
      default: stockham_stage<8, INV>(a, b, f.L, ns, tw, col, lane); break;
    }
    __syncthreads();
    float2* t = a;
    a = b;
    b = t;
    ns *= r;
  }
  return a;
}

__device__ __forceinline__ void load_twiddles(float2* tw_s, const float2* __restrict__ tw_g, int L) {
  for (int i = threadIdx.x; i < L; i += NT) tw_s[i] = tw_g[i];
}

// ---------------------------------------------------------------------------
// pass 1: x-axis forward R2C of pairs of real rows (weighted timepoint sum)
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(NT) k_x_fwd(ActIn in, float2* __restrict__ out, int nrows, int N2, int HS, FftLen f,
                                              const float2* __restrict__ twg) {
  extern __shared__ float2 sm[];
  float2* tw = sm;
  float2* a = sm + f.L;
  float2* b = a + f.L * TXP;
  load_twiddles(tw, twg, f.L);
  const long long row0 = (long long)blockIdx.x * (2 * TX);
  for (int idx = threadIdx.x; idx < TX * f.L; idx += NT) {
    const int m = idx / f.L, n = idx - (idx / f.L) * f.L;
    float2 v = make_float2(0.f, 0.f);
    if (n < N2) {
      const long long ra = row0 + 2 * m, rb = ra + 1;
      if (ra < nrows) {
        const long long o = ra * N2 + n;
        float s = 0.f;
        for (int t = 0; t < in.n; ++t) s += in.w[t] * __ldg(in.p[t] + o);
        v.x = s;
      }
      if (rb < nrows) {
        const long long o = rb * N2 + n;
        float s = 0.f;
        for (int t = 0; t < in.n; ++t) s += in.w[t] * __ldg(in.p[t] + o);
        v.y = s;
      }
    }
    a[n * TXP + m] = v;
  }
  __syncthreads();
  float2* r = fft_tile<false>(a, b, f, tw);
  const int H = f.L / 2 + 1;
  for (int idx = threadIdx.x; idx < TX * H; idx += NT) {
    const int m = idx / H, k = idx - (idx / H) * H;
    const long long ra = row0 + 2 * m, rb = ra + 1;
    const int kk = (k == 0) ? 0 : f.L - k;
    const float2 z1 = r[k * TXP + m];
    const float2 z2 = r[kk * TXP + m];
    // Xa = (Z[k] + conj Z[-k]) / 2 ;  Xb = (Z[k] - conj Z[-k]) / (2i)
    const float2 xa = make_float2(0.5f * (z1.x + z2.x), 0.5f * (z1.y - z2.y));
    const float2 xb = make_float2(0.5f * (z1.y + z2.y), -0.5f * (z1.x - z2.x));
    if (ra < nrows) out[ra * HS + k] = xa;
    if (rb < nrows) out[rb * HS + k] = xb;
  }
}

// ---------------------------------------------------------------------------
// passes 2 and 4: y-axis C2C over columns, zero-pad input rows >= nin, keep
// output rows < nout.  blockIdx.x: column tile, blockIdx.y: z slab, blockIdx.z:
// kernel slot (the inverse pass runs in place in each slot's buffer).
// ---------------------------------------------------------------------------
template <bool INV>
__global__ void __launch_bounds__(NT) k_y(ColSet io, int nin, int nout, int HS, FftLen f,
                                          const float2* __restrict__ twg) {
  extern __shared__ float2 sm[];
  float2* tw = sm;
  float2* a = sm + f.L;
  float2* b = a + f.L * TXP;
  load_twiddles(tw, twg, f.L);
  const int kx0 = blockIdx.x * TX;
  const float2* src = pick(io.in, blockIdx.z) + (long long)blockIdx.y * io.in_slab + kx0;
  float2* dst = pick(io.out, blockIdx.z) + (long long)blockIdx.y * io.out_slab + kx0;
  for (int idx = threadIdx.x; idx < TX * f.L; idx += NT) {
    const int n = idx / TX, c = idx % TX;
    a[n * TXP + c] = (n < nin) ? __ldcg(src + (long long)n * HS + c) : make_float2(0.f, 0.f);
  }
  __syncthreads();
  float2* r = fft_tile<INV>(a, b, f, tw);
  for (int idx = threadIdx.x; idx < TX * nout; idx += NT) {
    const int n = idx / TX, c = idx % TX;
    dst[(long long)n * HS + c] = r[n * TXP + c];
  }
}

// ---------------------------------------------------------------------------
// pass 3: z-axis forward, spectrum multiply, inverse, crop — per kernel slot.
// in:  [N0][P1][HS] (rows z < N0 valid);  out_k: [N0][P1][HS].
// blockIdx.x: column tile, blockIdx.y: ky.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(NT) k_z(const float2* __restrict__ in, OutSet os, int N0, int P1, int HS, FftLen f,
                                          const float2* __restrict__ twg) {
  extern __shared__ float2 sm[];
  float2* tw = sm;
  float2* bufs[3];
  bufs[0] = sm + f.L;
  bufs[1] = bufs[0] + f.L * TXP;
  bufs[2] = bufs[1] + f.L * TXP;
  load_twiddles(tw, twg, f.L);
  const int kx0 = blockIdx.x * TX;
  const int ky = blockIdx.y;
  const long long zstride = (long long)P1 * HS;
  const long long base = (long long)ky * HS + kx0;
  for (int idx = threadIdx.x; idx < TX * f.L; idx += NT) {
    const int z = idx / TX, c = idx % TX;
    bufs[0][z * TXP + c] = (z < N0) ? in[z * zstride + base + c] : make_float2(0.f, 0.f);
  }
  __syncthreads();
  float2* X = fft_tile<false>(bufs[0], bufs[1], f, tw);
  const int xi = (X == bufs[0]) ? 0 : 1;
  for (int s = 0; s < os.n; ++s) {
    float2* A;
    float2* B;
    if (os.n == 1) {
      A = X;
      B = bufs[1 - xi];
    } else {
      A = bufs[1 - xi];
      B = bufs[2];
    }
    if (os.mode[s] == SPEC_REAL_EVEN) {
      const float* S = (const float*)os.s[s];
      const int kyq = min(ky, P1 - ky);
      for (int idx = threadIdx.x; idx < TX * f.L; idx += NT) {
        const int z = idx / TX, c = idx % TX;
        const int kzq = min(z, os.P0 - z);
        A[z * TXP + c] = cscale(X[z * TXP + c], __ldg(S + ((long long)kzq * os.P1h + kyq) * HS + kx0 + c));
      }
    } else {
      const float2* S = (const float2*)os.s[s];
      for (int idx = threadIdx.x; idx < TX * f.L; idx += NT) {
        const int z = idx / TX, c = idx % TX;
        A[z * TXP + c] = cmul(X[z * TXP + c], __ldg(S + z * zstride + (long long)ky * HS + kx0 + c));
      }
    }
    __syncthreads();
    float2* r = fft_tile<true>(A, B, f, tw);
    float2* dst = os.p[s];
    for (int idx = threadIdx.x; idx < TX * N0; idx += NT) {
      const int z = idx / TX, c = idx % TX;
      dst[z * zstride + base + c] = r[z * TXP + c];
    }
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------
// pass 5: x-axis inverse C2R of pairs of rows, crop, scale, density, for the
// kernel slots of `io` in turn (row r = z * N1 + y of slot s at
// io.in[s] + (z * pitch + y) * HS).
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(NT) k_x_inv(XInvSet io, const float* __restrict__ rho, int nrows, int N1,
                                              int pitch, int N2, int HS, float scale, FftLen f,
                                              const float2* __restrict__ twg) {
  extern __shared__ float2 sm[];
  float2* tw = sm;
  float2* a = sm + f.L;
  float2* b = a + f.L * TXP;
  load_twiddles(tw, twg, f.L);
  const long long row0 = (long long)blockIdx.x * (2 * TX);
  const int H = f.L / 2 + 1;
  for (int sl = 0; sl < io.n; ++sl) {
    const float2* in = pick(io.in, sl);
    float* out = pick(io.out, sl);
    for (int idx = threadIdx.x; idx < TX * H; idx += NT) {
      const int m = idx / H, k = idx - (idx / H) * H;
      const long long ra = row0 + 2 * m, rb = ra + 1;
      const long long za = ra / N1, zb = rb / N1;
      float2 xa = (ra < nrows) ? in[(za * pitch + (ra - za * N1)) * HS + k] : make_float2(0.f, 0.f);
      float2 xb = (rb < nrows) ? in[(zb * pitch + (rb - zb * N1)) * HS + k] : make_float2(0.f, 0.f);
      if (k == 0 || 2 * k == f.L) {  // DC / Nyquist bins of a real row are real
        xa.y = 0.f;
        xb.y = 0.f;
      }
      a[k * TXP + m] = make_float2(xa.x - xb.y, xa.y + xb.x);  // Xa + i Xb
      const int kk = f.L - k;
      if (k > 0 && kk >= H) a[kk * TXP + m] = make_float2(xa.x + xb.y, xb.x - xa.y);  // conj Xa + i conj Xb
    }
    __syncthreads();
    float2* r = fft_tile<true>(a, b, f, tw);
    for (int idx = threadIdx.x; idx < TX * N2; idx += NT) {
      const int m = idx / N2, n = idx - (idx / N2) * N2;
      const long long ra = row0 + 2 * m, rb = ra + 1;
      const float2 z = r[n * TXP + m];
      if (ra < nrows) {
        float v = z.x * scale;
        if (rho) {
          const float d = __ldg(rho + ra * N2 + n);
          v = (d > 0.f) ? v / d : 0.f;
        }
        out[ra * N2 + n] = v;
      }
      if (rb < nrows) {
        float v = z.y * scale;
        if (rho) {
          const float d = __ldg(rho + rb * N2 + n);
          v = (d > 0.f) ? v / d : 0.f;
        }
        out[rb * N2 + n] = v;
      }
    }
    __syncthreads();  // the tiles are free for the next slot
  }
}

// ---------------------------------------------------------------------------
// kernel spectrum: FP64 normalisation sum, scale, and a separable direct DFT
// of the (small) placed kernel into the padded spectral layout.
// ---------------------------------------------------------------------------
__global__ void k_sum_f64(const double* __restrict__ k, long long n, double* __restrict__ out) {
  __shared__ double red[NT];
  double s = 0.0;
  for (long long i = threadIdx.x; i < n; i += NT) s += k[i];
  red[threadIdx.x] = s;
  __syncthreads();
  for (int w = NT / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = red[0];
}

// kf = float(k * factor) where factor = scale / sum (or scale) / (P0 P1 P2), all FP64
__global__ void k_scale_to_f32(const double* __restrict__ k, long long n, const double* __restrict__ sum,
                               double scale_over_p, float* __restrict__ kf) {
  const double fac = sum ? scale_over_p / *sum : scale_over_p;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    kf[i] = (float)(k[i] * fac);
}

// Placement of kernel index m along one axis of length P: at (m - o) mod P, and, when
// img > 0, a second copy at (m + img) mod P.  The copy makes a convolution of period
// P >= 2N into the circular convolution of period N (img = P - N): for an input that
// is zero beyond N, output index i < N then receives A[(i - m) mod N] * K[m] exactly.
// Returns the summed twiddle of the placed copies for frequency k.
__device__ __forceinline__ float2 placed_twiddle(const float2* __restrict__ tw, int k, int m, int o, int img, int P) {
  const int p = ((m - o) % P + P) % P;
  float2 w = tw[(int)(((long long)k * p) % P)];
  if (img > 0) w = cadd(w, tw[(int)(((long long)k * ((m + img) % P)) % P)]);
  return w;
}

// T1[m0][m1][kx] = sum_m2 k[m0][m1][m2] w2^(kx * place(m2))
__global__ void k_spec_x(const float* __restrict__ kf, float2* __restrict__ t1, int K0, int K1, int K2, int K2e,
                         int o2, int img2, int P2, int H, const float2* __restrict__ tw2) {
  const long long total = (long long)K0 * K1 * H;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total; i += (long long)gridDim.x * blockDim.x) {
    const int kx = (int)(i % H);
    const long long row = i / H;
    float2 acc = make_float2(0.f, 0.f);
    for (int m = 0; m < K2e; ++m) {
      const float v = kf[row * K2 + m];
      const float2 w = placed_twiddle(tw2, kx, m, o2, img2, P2);
      acc.x += v * w.x;
      acc.y += v * w.y;
    }
    t1[i] = acc;
  }
}

// T2[m0][ky][kx] = sum_m1 T1[m0][m1][kx] w1^(ky * place(m1))
__global__ void k_spec_y(const float2* __restrict__ t1, float2* __restrict__ t2, int K0, int K1, int K1e, int o1,
                         int img1, int P1, int H, const float2* __restrict__ tw1) {
  const long long total = (long long)K0 * P1 * H;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total; i += (long long)gridDim.x * blockDim.x) {
    const int kx = (int)(i % H);
    const int ky = (int)((i / H) % P1);
    const int m0 = (int)(i / ((long long)H * P1));
    float2 acc = make_float2(0.f, 0.f);
    for (int m = 0; m < K1e; ++m) {
      const float2 v = t1[((long long)m0 * K1 + m) * H + kx];
      acc = cadd(acc, cmul(v, placed_twiddle(tw1, ky, m, o1, img1, P1)));
    }
    t2[i] = acc;
  }
}

// S[kz][ky][kx] = sum_m0 T2[m0][ky][kx] w0^(kz * place(m0)); kx in [H, HS) -> 0.
// SPEC_REAL_EVEN stores the real part for kz <= P0/2, ky <= P1/2 only.
__global__ void k_spec_z(const float2* __restrict__ t2, void* __restrict__ spec, int mode, int K0e, int o0, int img0,
                         int P0, int P1, int H, int HS, const float2* __restrict__ tw0) {
  const int nz = (mode == SPEC_REAL_EVEN) ? P0 / 2 + 1 : P0;
  const int ny = (mode == SPEC_REAL_EVEN) ? P1 / 2 + 1 : P1;
  const long long total = (long long)nz * ny * HS;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total; i += (long long)gridDim.x * blockDim.x) {
    const int kx = (int)(i % HS);
    const int ky = (int)((i / HS) % ny);
    const int kz = (int)(i / ((long long)HS * ny));
    float2 acc = make_float2(0.f, 0.f);
    if (kx < H) {
      for (int m = 0; m < K0e; ++m) {
        const float2 v = t2[((long long)m * P1 + ky) * H + kx];
        acc = cadd(acc, cmul(v, placed_twiddle(tw0, kz, m, o0, img0, P0)));
      }
    }
    if (mode == SPEC_REAL_EVEN)
      ((float*)spec)[i] = acc.x;
    else
      ((float2*)spec)[i] = acc;
  }
}

}  // namespace pvd

// ===========================================================================
// plan object and C ABI
// ===========================================================================
using namespace pvd;

struct pvd_plan {
  int dev = 0;
  int mode = PVD_MODE_LINEAR;
  int N[3] = {0, 0, 0};
  int P[3] = {0, 0, 0};
  int kmax[3] = {0, 0, 0};
  int img[3] = {0, 0, 0};  // CIRCULAR axes with P >= 2N: offset of the kernel's image copy (P - N)
  int H = 0, HS = 0, nk = 0;
  FftLen f[3];
  float2* tw[3] = {nullptr, nullptr, nullptr};
  float2* buf1 = nullptr;
  float2* buf2 = nullptr;
  float2* buf3[PVD_MAX_KERNELS] = {};
  const FastLen* fl[3] = {nullptr, nullptr, nullptr};  // register four-step kernels per axis (or generic)
  void* spec[PVD_MAX_KERNELS] = {};
  int spec_mode[PVD_MAX_KERNELS] = {};
  size_t spec_bytes[PVD_MAX_KERNELS] = {};
  int spec_set[PVD_MAX_KERNELS] = {};
  size_t ws_bytes = 0;
  size_t smem_x = 0, smem_y = 0, smem_z = 0;
  std::vector<void*> allocs;
  // per-pass event timing (instrumentation, off by default)
  int prof = 0;
  // TMA-staged persistent column passes (register four-step lengths only)
  int tma = 0;
  int* d_err = nullptr;
  CUtensorMap m_yf, m_z;
  CUtensorMap m_yi[PVD_MAX_KERNELS];
  int yf_chunks = 1, yf_boxr = 1, yi_chunks = 1, yi_boxr = 1, z_chunks = 1, z_boxr = 1;
  int grid_yf = 0, grid_yi = 0, grid_z = 0;
  size_t smem_tyf = 0, smem_tyi = 0, smem_tz = 0;
  // host-buffer execution (pvd_conv_execute_host): device staging and copy streams
  float* io_act = nullptr;
  float* io_rho = nullptr;
  float* io_dose = nullptr;
  cudaStream_t s_h2d = nullptr, s_d2h = nullptr;
  cudaEvent_t ev_start = nullptr, ev_done = nullptr;
  cudaEvent_t ev_act[PVD_HOST_CHUNKS] = {};
  cudaEvent_t ev_rho[PVD_DOSE_CHUNKS] = {};
  cudaEvent_t ev_dose[PVD_MAX_KERNELS * PVD_DOSE_CHUNKS] = {};
  std::vector<cudaEvent_t> ev_pool;
  size_t ev_used = 0;
  struct Rec { int kind; cudaEvent_t a, b; };
  std::vector<Rec> recs;
};

namespace {

// Cap on the device bytes one plan may hold (0 = none): instrumentation that lets a
// test make plan creation fail the way an exhausted device does, without exhausting it.
std::atomic<size_t> g_plan_alloc_cap{0};

pvd_status plan_alloc(pvd_plan* p, size_t bytes, void** out) {
  const size_t cap = g_plan_alloc_cap.load();
  if (cap && p->ws_bytes + bytes > cap)
    return set_error(PVD_ERR_OOM, "plan workspace: " + std::to_string(p->ws_bytes + bytes) +
                                      " bytes exceed the allocation cap of " + std::to_string(cap) + " bytes");
  void* ptr = nullptr;
  cudaError_t e = cudaMalloc(&ptr, bytes);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return cuda_error(e, "cudaMalloc(plan workspace)");
  }
  p->allocs.push_back(ptr);
  p->ws_bytes += bytes;
  *out = ptr;
  return PVD_OK;
}

void plan_free(pvd_plan* p) {
  for (void* a : p->allocs) cudaFree(a);
  p->allocs.clear();
  if (p->s_h2d) cudaStreamDestroy(p->s_h2d);
  if (p->s_d2h) cudaStreamDestroy(p->s_d2h);
  for (cudaEvent_t e : {p->ev_start, p->ev_done})
    if (e) cudaEventDestroy(e);
  for (cudaEvent_t e : p->ev_act)
    if (e) cudaEventDestroy(e);
  for (cudaEvent_t e : p->ev_rho)
    if (e) cudaEventDestroy(e);
  for (cudaEvent_t e : p->ev_dose)
    if (e) cudaEventDestroy(e);
  for (cudaEvent_t e : p->ev_pool) cudaEventDestroy(e);
  p->ev_pool.clear();
}

cudaEvent_t prof_event(pvd_plan* p) {
  if (p->ev_used == p->ev_pool.size()) {
    cudaEvent_t e;
    if (cudaEventCreate(&e) != cudaSuccess) return nullptr;
    p->ev_pool.push_back(e);
  }
  return p->ev_pool[p->ev_used++];
}

// Brackets one pass launch with events on `st` when profiling is enabled.
struct PassTimer {
  pvd_plan* p;
  int kind;
  cudaStream_t st;
  cudaEvent_t a = nullptr;
  PassTimer(pvd_plan* p_, int kind_, cudaStream_t st_) : p(p_), kind(kind_), st(st_) {
    if (p->prof && (a = prof_event(p))) cudaEventRecord(a, st);
  }
  ~PassTimer() {
    if (!a) return;
    cudaEvent_t b = prof_event(p);
    if (!b) return;
    cudaEventRecord(b, st);
    p->recs.push_back({kind, a, b});
  }
};

size_t smem_bytes(int L, int nbuf) { return (size_t)(L + nbuf * L * TXP) * sizeof(float2); }

}  // namespace

namespace {

// rows of one TMA box (<= 256) and the number of boxes covering n rows
void box_rows(int n, int* chunks, int* boxr) {
  *chunks = (n + 255) / 256;
  *boxr = (n + *chunks - 1) / *chunks;
}

PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = [] {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      f = nullptr;
    return (PFN_cuTensorMapEncodeTiled_v12000)f;
  }();
  return fn;
}

// [dim2][dim1][HS] complex buffer as 8-byte elements; box {16, b1, b2}
bool encode_cols(CUtensorMap* m, void* base, int HS, int dim1, int dim2, int b1, int b2) {
  auto enc = tensor_map_encoder();
  if (!enc) return false;
  const cuuint64_t dims[3] = {(cuuint64_t)HS, (cuuint64_t)dim1, (cuuint64_t)dim2};
  const cuuint64_t strides[2] = {(cuuint64_t)HS * 8, (cuuint64_t)HS * 8 * dim1};
  const cuuint32_t box[3] = {(cuuint32_t)FTX, (cuuint32_t)b1, (cuuint32_t)b2};
  const cuuint32_t es[3] = {1, 1, 1};
  return enc(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 3, base, dims, strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
             CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) ==
         CUDA_SUCCESS;
}

int persistent_grid(const void* fn, int threads, size_t smem, int dev) {
  int nb = 0, sms = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, fn, threads, smem) != cudaSuccess) return 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  return nb * sms;
}

// Lets f take the largest dynamic shared memory the device allows beside f's own static
// shared memory; returns that allowance (0 when the attribute could not be set).
size_t allow_dyn_smem(const void* f, int smem_max) {
  cudaFuncAttributes a{};
  if (cudaFuncGetAttributes(&a, f) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  const int allow = smem_max - (int)a.sharedSizeBytes;
  if (allow <= 0 || cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, allow) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return (size_t)allow;
}

// Opts the pass kernels a plan launches (the register kernels of its fast lengths, else the
// generic ones) into large tiles; false if a pass's tile does not fit beside its kernel's
// static shared memory.  fl[i] serves axis i: x (rows) is axis 2, y axis 1, z axis 0.
bool pass_tiles_fit(const FastLen* const fl[3], size_t smem_x, size_t smem_y, size_t smem_z, int smem_max) {
  auto fits = [smem_max](const void* f, size_t need) { return need <= allow_dyn_smem(f, smem_max); };
  bool ok = true;
  if (fl[2]) {
    ok = fits((const void*)fl[2]->x_fwd, fl[2]->smem_row) && ok;
    ok = fits((const void*)fl[2]->x_inv, fl[2]->smem_row) && ok;
  } else {
    ok = fits((const void*)k_x_fwd, smem_x) && ok;
    ok = fits((const void*)k_x_inv, smem_x) && ok;
  }
  if (fl[1]) {
    ok = fits((const void*)fl[1]->y_fwd, fl[1]->smem_col) && ok;
    ok = fits((const void*)fl[1]->y_inv, fl[1]->smem_col) && ok;
  } else {
    ok = fits((const void*)k_y<false>, smem_y) && ok;
    ok = fits((const void*)k_y<true>, smem_y) && ok;
  }
  if (fl[0]) ok = fits((const void*)fl[0]->z, fl[0]->smem_z) && ok;
  else ok = fits((const void*)k_z, smem_z) && ok;
  return ok;
}

// Enables the TMA-staged y and z passes when both axes have register kernels;
// leaves p->tma = 0 (plain register passes) if anything does not fit.
pvd_status setup_tma(pvd_plan* p, int smem_max) {
  const FastLen* fy = p->fl[1];
  const FastLen* fz = p->fl[0];
  if (!fy || !fz) return PVD_OK;
  box_rows(p->N[1], &p->yf_chunks, &p->yf_boxr);
  box_rows(p->P[1], &p->yi_chunks, &p->yi_boxr);
  box_rows(p->N[0], &p->z_chunks, &p->z_boxr);
  // each box lands at stage + k * boxr rows: 128-byte aligned only if a box of rows is
  for (int br : {p->yf_boxr, p->yi_boxr, p->z_boxr})
    if (((size_t)br * FTX * sizeof(float2)) % 128 != 0) return PVD_OK;
  p->smem_tyf = tma_y_smem(fy->L, p->yf_chunks, p->yf_boxr);
  p->smem_tyi = tma_y_smem(fy->L, p->yi_chunks, p->yi_boxr);
  p->smem_tz = tma_z_smem(fz->L, p->z_chunks, p->z_boxr);
  if (p->smem_tyf > allow_dyn_smem((const void*)fy->ty_fwd, smem_max) ||
      p->smem_tyi > allow_dyn_smem((const void*)fy->ty_inv, smem_max) ||
      p->smem_tz > allow_dyn_smem((const void*)fz->tz, smem_max))
    return PVD_OK;
  bool ok = encode_cols(&p->m_yf, p->buf1, p->HS, p->N[1], p->N[0], p->yf_boxr, 1) &&
            encode_cols(&p->m_z, p->buf2, p->HS, p->P[1], p->N[0], 1, p->z_boxr);
  for (int s = 0; s < p->nk && ok; ++s) ok = encode_cols(&p->m_yi[s], p->buf3[s], p->HS, p->P[1], p->N[0], p->yi_boxr, 1);
  if (!ok) return PVD_OK;
  p->grid_yf = persistent_grid((const void*)fy->ty_fwd, fy->threads, p->smem_tyf, p->dev);
  p->grid_yi = persistent_grid((const void*)fy->ty_inv, fy->threads, p->smem_tyi, p->dev);
  p->grid_z = persistent_grid((const void*)fz->tz, fz->threads, p->smem_tz, p->dev);
  if (p->grid_yf <= 0 || p->grid_yi <= 0 || p->grid_z <= 0) return PVD_OK;
  p->tma = 1;
  return PVD_OK;
}

}  // namespace

extern "C" pvd_status pvd_plan_create(const pvd_conv_desc* d, pvd_plan** out) {
  if (!d || !out) return set_error(PVD_ERR_ARG, "pvd_plan_create: null argument");
  *out = nullptr;
  if (d->flags & ~PVD_PLAN_TMA) return set_error(PVD_ERR_ARG, "pvd_plan_create: unknown flags");
  if (d->mode != PVD_MODE_LINEAR && d->mode != PVD_MODE_CIRCULAR)
    return set_error(PVD_ERR_ARG, "pvd_plan_create: unknown mode");
  if (d->n_kernels < 1 || d->n_kernels > PVD_MAX_KERNELS)
    return set_error(PVD_ERR_ARG, "pvd_plan_create: n_kernels must be in [1, 8]");
  for (int i = 0; i < 3; ++i) {
    if (d->n[i] < 1 || d->n[i] > 4096) return set_error(PVD_ERR_ARG, "pvd_plan_create: volume dims must be in [1, 4096]");
    if (d->mode == PVD_MODE_LINEAR && (d->kmax[i] < 1 || d->kmax[i] > 1024))
      return set_error(PVD_ERR_ARG, "pvd_plan_create: kmax must be in [1, 1024] for LINEAR mode");
  }
  pvd_plan* p = new pvd_plan();
  p->mode = d->mode;
  p->nk = d->n_kernels;
  cudaGetDevice(&p->dev);
  for (int i = 0; i < 3; ++i) {
    p->N[i] = d->n[i];
    p->kmax[i] = d->kmax[i];
    const int n = d->n[i];
    int L = d->pad[i];
    if (d->mode == PVD_MODE_CIRCULAR) {
      // period n directly when n is 7-smooth; otherwise a zero-padded length >= 2n with
      // the kernel's image copy at P - n, which gives the same period-n convolution
      if (!L) {
        if (is_smooth7(n)) {
          L = n;
        } else {
          const int lf = fast_len_at_least(2 * n), ls = next_smooth7(2 * n);
          L = (lf && lf <= ls) ? lf : ls;
        }
      }
      if (L != n && L < 2 * n) {
        delete p;
        return set_error(PVD_ERR_ARG, "pvd_plan_create: CIRCULAR pad must be n or at least 2n");
      }
      p->img[i] = (L == n) ? 0 : L - n;
    } else {
      const int need = n + d->kmax[i] - 1;
      if (!L) {  // prefer a length with register four-step kernels when it pads by <= 25 %
        const int lf = fast_len_at_least(need), ls = next_smooth7(need);
        L = (lf && (lf == ls || 4 * lf <= 5 * need)) ? lf : ls;
      }
      if (L < need) {
        delete p;
        return set_error(PVD_ERR_ARG, "pvd_plan_create: explicit pad too small (LINEAR needs n+kmax-1)");
      }
    }
    if (!factorize(L, &p->f[i])) {
      delete p;
      return set_error(PVD_ERR_UNSUPPORTED, "pvd_plan_create: FFT length " + std::to_string(L) +
                                                " has a prime factor > 7 (explicit pads must be 7-smooth)");
    }
    p->P[i] = L;
    p->fl[i] = fast_len(L);
  }
  p->H = p->P[2] / 2 + 1;
  p->HS = (p->H + TX - 1) / TX * TX;
  p->smem_x = smem_bytes(p->P[2], 2);
  p->smem_y = smem_bytes(p->P[1], 2);
  p->smem_z = smem_bytes(p->P[0], p->nk > 1 ? 3 : 2);
  int smem_max = 0;
  cudaDeviceGetAttribute(&smem_max, cudaDevAttrMaxSharedMemoryPerBlockOptin, p->dev);
  if (!pass_tiles_fit(p->fl, p->smem_x, p->smem_y, p->smem_z, smem_max)) {
    delete p;
    return set_error(PVD_ERR_UNSUPPORTED, "pvd_plan_create: FFT length too large for one shared-memory tile");
  }

  pvd_status st = PVD_OK;
  // twiddle tables exp(-2 pi i n / L), computed in FP64 on the host
  for (int i = 0; i < 3 && st == PVD_OK; ++i) {
    int L = p->P[i];
    std::vector<float2> h(L);
    for (int n = 0; n < L; ++n) {
      double a = -2.0 * M_PI * (double)n / (double)L;
      h[n] = make_float2((float)std::cos(a), (float)std::sin(a));
    }
    void* ptr = nullptr;
    st = plan_alloc(p, sizeof(float2) * L, &ptr);
    if (st == PVD_OK) {
      p->tw[i] = (float2*)ptr;
      cudaError_t e = cudaMemcpy(ptr, h.data(), sizeof(float2) * L, cudaMemcpyHostToDevice);
      if (e != cudaSuccess) st = cuda_error(e, "cudaMemcpy(twiddles)");
    }
  }
  const size_t b1 = sizeof(float2) * (size_t)p->N[0] * p->N[1] * p->HS;
  const size_t b2 = sizeof(float2) * (size_t)p->N[0] * p->P[1] * p->HS;
  void* ptr = nullptr;
  if (st == PVD_OK) st = plan_alloc(p, b1, &ptr), p->buf1 = (float2*)ptr;
  if (st == PVD_OK) st = plan_alloc(p, b2, &ptr), p->buf2 = (float2*)ptr;
  if (st == PVD_OK) p->buf3[0] = p->buf2;  // slot 0 transforms in place
  for (int s = 1; s < p->nk && st == PVD_OK; ++s) st = plan_alloc(p, b2, &ptr), p->buf3[s] = (float2*)ptr;
  if (st == PVD_OK) {
    // padding columns [H, HS) are carried through the column passes; keep them defined
    cudaError_t e = cudaMemset(p->buf1, 0, b1);
    if (e == cudaSuccess) e = cudaMemset(p->buf2, 0, b2);
    for (int s = 1; s < p->nk && e == cudaSuccess; ++s) e = cudaMemset(p->buf3[s], 0, b2);
    if (e != cudaSuccess) st = cuda_error(e, "cudaMemset(workspace)");
  }
  if (st == PVD_OK) {  // device status word of the plan's passes (bounded waits record here)
    st = plan_alloc(p, sizeof(int), &ptr);
    if (st == PVD_OK) {
      p->d_err = (int*)ptr;
      cudaError_t e = cudaMemset(p->d_err, 0, sizeof(int));
      if (e != cudaSuccess) st = cuda_error(e, "cudaMemset(status word)");
    }
  }
  if (st == PVD_OK && (d->flags & PVD_PLAN_TMA)) st = setup_tma(p, smem_max);
  if (st != PVD_OK) {
    plan_free(p);
    delete p;
    return st;
  }
  *out = p;
  return PVD_OK;
}

extern "C" pvd_status pvd_plan_get_info(const pvd_plan* p, pvd_plan_info* info) {
  if (!p || !info) return set_error(PVD_ERR_ARG, "pvd_plan_get_info: null argument");
  for (int i = 0; i < 3; ++i) {
    info->n[i] = p->N[i];
    info->p[i] = p->P[i];
  }
  info->h = p->H;
  info->hs = p->HS;
  info->n_kernels = p->nk;
  info->workspace_bytes = p->ws_bytes;
  return PVD_OK;
}

extern "C" pvd_status pvd_plan_set_kernel(pvd_plan* p, int slot, const double* kh, int k0, int k1, int k2,
                                          double scale, int flags) {
  if (!p || !kh) return set_error(PVD_ERR_ARG, "pvd_plan_set_kernel: null argument");
  if (slot < 0 || slot >= p->nk) return set_error(PVD_ERR_ARG, "pvd_plan_set_kernel: slot out of range");
  if (flags & ~PVD_KERNEL_NORMALIZE) return set_error(PVD_ERR_ARG, "pvd_plan_set_kernel: unknown flags");
  const int K[3] = {k0, k1, k2};
  for (int i = 0; i < 3; ++i) {
    if (K[i] < 1) return set_error(PVD_ERR_ARG, "pvd_plan_set_kernel: kernel dims must be >= 1");
    if (p->mode == PVD_MODE_LINEAR && K[i] > p->kmax[i])
      return set_error(PVD_ERR_ARG, "pvd_plan_set_kernel: kernel larger than the plan's kmax");
  }
  if (!std::isfinite(scale)) return set_error(PVD_ERR_NUMERIC, "pvd_plan_set_kernel: non-finite scale");
  const long long nk = (long long)k0 * k1 * k2;
  for (long long i = 0; i < nk; ++i)
    if (!std::isfinite(kh[i]))
      return set_error(PVD_ERR_NUMERIC, "pvd_plan_set_kernel: kernel has a non-finite value at flat index " +
                                            std::to_string(i));
  // placement offsets; a LINEAR-mode kernel with odd dims that is even along
  // every axis separately (any radial kernel) has a real spectrum that is even
  // in kz and ky: only a quarter of it is stored.
  int o[3], Ke[3];
  bool sym = (p->mode == PVD_MODE_LINEAR);
  for (int i = 0; i < 3; ++i) {
    o[i] = (p->mode == PVD_MODE_LINEAR) ? K[i] / 2 : 0;
    // CIRCULAR: the reference's fftn(K, A.shape) keeps the first n entries per axis
    Ke[i] = std::min(K[i], (p->mode == PVD_MODE_LINEAR) ? p->P[i] : p->N[i]);
    if (K[i] % 2 == 0) sym = false;
  }
  for (long long i = 0; sym && i < nk; ++i) {
    const int a = (int)(i / ((long long)k1 * k2)), b = (int)((i / k2) % k1), c = (int)(i % k2);
    const long long jz = ((long long)(k0 - 1 - a) * k1 + b) * k2 + c;
    const long long jy = ((long long)a * k1 + (k1 - 1 - b)) * k2 + c;
    const long long jx = ((long long)a * k1 + b) * k2 + (k2 - 1 - c);
    if (kh[i] != kh[jz] || kh[i] != kh[jy] || kh[i] != kh[jx]) sym = false;
  }
  const int smode = sym ? SPEC_REAL_EVEN : SPEC_COMPLEX;
  const size_t spec_bytes = sym ? sizeof(float) * (size_t)(p->P[0] / 2 + 1) * (p->P[1] / 2 + 1) * p->HS
                                : sizeof(float2) * (size_t)p->P[0] * p->P[1] * p->HS;
  const double inv_p = 1.0 / ((double)p->P[0] * p->P[1] * p->P[2]);

  double* kd = nullptr;
  double* sumd = nullptr;
  float* kf = nullptr;
  float2* t1 = nullptr;
  float2* t2 = nullptr;
  pvd_status st = PVD_OK;
  auto cleanup = [&]() {
    cudaFree(kd);
    cudaFree(sumd);
    cudaFree(kf);
    cudaFree(t1);
    cudaFree(t2);
  };
  cudaError_t e = cudaMalloc(&kd, sizeof(double) * nk);
  if (e == cudaSuccess) e = cudaMalloc(&sumd, sizeof(double));
  if (e == cudaSuccess) e = cudaMalloc(&kf, sizeof(float) * nk);
  if (e == cudaSuccess) e = cudaMalloc(&t1, sizeof(float2) * (size_t)k0 * k1 * p->H);
  if (e == cudaSuccess) e = cudaMalloc(&t2, sizeof(float2) * (size_t)k0 * p->P[1] * p->H);
  if (e != cudaSuccess) {
    cudaGetLastError();
    cleanup();
    return cuda_error(e, "cudaMalloc(kernel staging)");
  }
  if (p->spec[slot]) {  // replace the slot's previous spectrum
    for (auto it = p->allocs.begin(); it != p->allocs.end(); ++it)
      if (*it == p->spec[slot]) {
        p->allocs.erase(it);
        break;
      }
    cudaFree(p->spec[slot]);
    p->ws_bytes -= p->spec_bytes[slot];
    p->spec[slot] = nullptr;
    p->spec_set[slot] = 0;
  }
  {
    void* sp = nullptr;
    pvd_status as = plan_alloc(p, spec_bytes, &sp);
    if (as != PVD_OK) {
      cleanup();
      return as;
    }
    p->spec[slot] = sp;
    p->spec_bytes[slot] = spec_bytes;
  }
  e = cudaMemcpy(kd, kh, sizeof(double) * nk, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    cleanup();
    return cuda_error(e, "cudaMemcpy(kernel)");
  }
  const bool norm = (flags & PVD_KERNEL_NORMALIZE) != 0;
  if (norm) {
    k_sum_f64<<<1, NT>>>(kd, nk, sumd);
    count_launch();
    double hsum = 0.0;
    e = cudaMemcpy(&hsum, sumd, sizeof(double), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) {
      cleanup();
      return cuda_error(e, "k_sum_f64");
    }
    if (!(std::isfinite(hsum) && hsum != 0.0)) {
      cleanup();
      return set_error(PVD_ERR_NUMERIC, "pvd_plan_set_kernel: kernel sum is zero or non-finite; cannot normalise");
    }
  }
  const int gs = 152 * 8;
  k_scale_to_f32<<<gs, NT>>>(kd, nk, norm ? sumd : nullptr, scale * inv_p, kf);
  count_launch();
  k_spec_x<<<gs, NT>>>(kf, t1, k0, k1, k2, Ke[2], o[2], p->img[2], p->P[2], p->H, p->tw[2]);
  count_launch();
  k_spec_y<<<gs, NT>>>(t1, t2, k0, k1, Ke[1], o[1], p->img[1], p->P[1], p->H, p->tw[1]);
  count_launch();
  k_spec_z<<<gs, NT>>>(t2, p->spec[slot], smode, Ke[0], o[0], p->img[0], p->P[0], p->P[1], p->H, p->HS, p->tw[0]);
  count_launch();
  e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  if (e != cudaSuccess) st = cuda_error(e, "kernel spectrum");
  cleanup();
  if (st == PVD_OK) {
    p->spec_mode[slot] = smode;
    p->spec_set[slot] = 1;
  }
  return st;
}

// Host buffers of one pvd_conv_execute_host call (device staging lives in the plan).
struct HostIO {
  const float* act;
  const float* rho;
  float* dose;
};

static pvd_status conv_run(pvd_plan* p, const ActIn& in, const float* rho, float* dose, float out_scale,
                           pvd_stream stream, const HostIO* hio = nullptr) {
  for (int s = 0; s < p->nk; ++s)
    if (!p->spec_set[s]) return set_error(PVD_ERR_STATE, "pvd_conv_execute: kernel slot " + std::to_string(s) + " not set");
  if (!dose) return set_error(PVD_ERR_ARG, "pvd_conv_execute: null dose pointer");
  if (!std::isfinite(out_scale)) return set_error(PVD_ERR_NUMERIC, "pvd_conv_execute: non-finite out_scale");
  cudaStream_t st = (cudaStream_t)stream;
  const int N0 = p->N[0], N1 = p->N[1], N2 = p->N[2];
  const int nrows = N0 * N1;
  const long long vox = (long long)nrows * N2;
  const FastLen* fx = p->fl[2];
  const FastLen* fy = p->fl[1];
  const FastLen* fz = p->fl[0];
  // column tiles and row blocks differ between the register (FTX) and generic (TX) kernels
  const int ctiles_y = p->HS / (fy ? FTX : TX);
  const int ctiles_z = p->HS / (fz ? FTX : TX);
  const int rows_x = 2 * (fx ? FTX : TX);
  // forward x and y passes, in z chunks when the activity arrives from the host
  // in pieces (each chunk waits for its own upload)
  const int nchunks = hio ? std::min(PVD_HOST_CHUNKS, N0) : 1;
  for (int c = 0; c < nchunks; ++c) {
    const int z0 = (int)((long long)N0 * c / nchunks), z1 = (int)((long long)N0 * (c + 1) / nchunks);
    if (z1 <= z0) continue;
    if (hio) PVD_CUDA_TRY(cudaStreamWaitEvent(st, p->ev_act[c], 0));
    ActIn ic = in;
    for (int t = 0; t < ic.n; ++t) ic.p[t] = in.p[t] + (long long)z0 * N1 * N2;
    const int rows = (z1 - z0) * N1;
    const int xb = (rows + rows_x - 1) / rows_x;
    float2* b1 = p->buf1 + (long long)z0 * N1 * p->HS;
    float2* b2 = p->buf2 + (long long)z0 * p->P[1] * p->HS;
    {
      PassTimer t(p, 0, st);
      if (fx)
        fx->x_fwd<<<xb, fx->threads, fx->smem_row, st>>>(ic, b1, rows, N2, p->HS, p->tw[2]);
      else
        k_x_fwd<<<xb, NT, p->smem_x, st>>>(ic, b1, rows, N2, p->HS, p->f[2], p->tw[2]);
      PVD_LAUNCH_CHECK("x_fwd");
    }
    {
      PassTimer t(p, 1, st);
      ColSet io;
      std::memset(&io, 0, sizeof(io));
      io.in[0] = b1;
      io.out[0] = b2;
      io.in_slab = (long long)N1 * p->HS;
      io.out_slab = (long long)p->P[1] * p->HS;
      if (p->tma)
        fy->ty_fwd<<<std::min(p->grid_yf, ctiles_y * (z1 - z0)), fy->threads, p->smem_tyf, st>>>(
            p->m_yf, p->buf2, N1, p->P[1], z0, z1 - z0, ctiles_y, p->HS, io.out_slab, p->yf_chunks, p->yf_boxr,
            p->tw[1], p->d_err);
      else if (fy)
        fy->y_fwd<<<dim3(ctiles_y, z1 - z0), fy->threads, fy->smem_col, st>>>(io, N1, p->P[1], p->HS, p->tw[1]);
      else
        k_y<false><<<dim3(ctiles_y, z1 - z0), NT, p->smem_y, st>>>(io, N1, p->P[1], p->HS, p->f[1], p->tw[1]);
      PVD_LAUNCH_CHECK("y_fwd");
    }
  }
  // z pass: the fast kernel takes up to FZ_SLOTS kernel slots per launch (each
  // launch reads the forward data again); the generic one takes all of them.
  // Slot 0 transforms in place, so it goes last.
  const int group = fz ? FZ_SLOTS : PVD_MAX_KERNELS;
  int order[PVD_MAX_KERNELS];
  for (int s = 0; s < p->nk; ++s) order[s] = (s + 1) % p->nk;
  for (int g0 = 0; g0 < p->nk; g0 += group) {
    OutSet os;
    std::memset(&os, 0, sizeof(os));
    os.n = std::min(group, p->nk - g0);
    os.P0 = p->P[0];
    os.P0h = p->P[0] / 2 + 1;
    os.P1h = p->P[1] / 2 + 1;
    for (int i = 0; i < os.n; ++i) {
      const int s = (p->nk <= group) ? i : order[g0 + i];
      os.p[i] = p->buf3[s];
      os.s[i] = p->spec[s];
      os.mode[i] = p->spec_mode[s];
    }
    PassTimer t(p, 2, st);
    if (p->tma)
      fz->tz<<<std::min(p->grid_z, ctiles_z * p->P[1]), fz->threads, p->smem_tz, st>>>(
          p->m_z, os, N0, p->P[1], p->HS, ctiles_z, p->z_chunks, p->z_boxr, p->tw[0], p->d_err);
    else if (fz)
      fz->z<<<dim3(ctiles_z, p->P[1]), fz->threads, fz->smem_z, st>>>(p->buf2, os, N0, p->P[1], p->HS, p->tw[0]);
    else
      k_z<<<dim3(ctiles_z, p->P[1]), NT, p->smem_z, st>>>(p->buf2, os, N0, p->P[1], p->HS, p->f[0], p->tw[0]);
    PVD_LAUNCH_CHECK("z");
  }
  // y inverse of every slot in one launch (blockIdx.z = slot), in place: rows 0..N1-1
  // of each z slab of the slot's z-pass buffer
  const long long zslab = (long long)p->P[1] * p->HS;
  {
    PassTimer t(p, 3, st);
    if (p->tma) {
      for (int s = 0; s < p->nk; ++s) {
        fy->ty_inv<<<std::min(p->grid_yi, ctiles_y * N0), fy->threads, p->smem_tyi, st>>>(
            p->m_yi[s], p->buf3[s], p->P[1], N1, 0, N0, ctiles_y, p->HS, zslab, p->yi_chunks, p->yi_boxr, p->tw[1],
            p->d_err);
        PVD_LAUNCH_CHECK("y_inv");
      }
    } else {
      ColSet io;
      std::memset(&io, 0, sizeof(io));
      for (int s = 0; s < p->nk; ++s) io.in[s] = io.out[s] = p->buf3[s];
      io.in_slab = io.out_slab = zslab;
      if (fy)
        fy->y_inv<<<dim3(ctiles_y, N0, p->nk), fy->threads, fy->smem_col, st>>>(io, p->P[1], N1, p->HS, p->tw[1]);
      else
        k_y<true><<<dim3(ctiles_y, N0, p->nk), NT, p->smem_y, st>>>(io, p->P[1], N1, p->HS, p->f[1], p->tw[1]);
      PVD_LAUNCH_CHECK("y_inv");
    }
  }
  // x inverse of every slot (up to XINV_SLOTS per launch): the density rows are read
  // from HBM once per row block.  With host buffers it runs in z chunks: chunk c
  // waits only for density chunk c, and each chunk's dose goes back as soon as it is
  // written.
  const int dchunks = hio ? std::min(PVD_DOSE_CHUNKS, N0) : 1;
  PassTimer t(p, 4, st);
  for (int c = 0; c < dchunks; ++c) {
    const long long z0 = (long long)N0 * c / dchunks, z1 = (long long)N0 * (c + 1) / dchunks;
    const long long r0 = z0 * N1, nr = (z1 - z0) * N1;  // rows of this chunk
    if (nr == 0) continue;
    if (hio && hio->rho) PVD_CUDA_TRY(cudaStreamWaitEvent(st, p->ev_rho[c], 0));
    const float* rho_c = rho ? rho + r0 * N2 : nullptr;
    const int xb = (int)((nr + rows_x - 1) / rows_x);
    for (int g0 = 0; g0 < p->nk; g0 += XINV_SLOTS) {
      XInvSet xs;
      std::memset(&xs, 0, sizeof(xs));
      xs.n = std::min(XINV_SLOTS, p->nk - g0);
      for (int i = 0; i < xs.n; ++i) {
        xs.in[i] = p->buf3[g0 + i] + z0 * zslab;
        xs.out[i] = dose + (g0 + i) * vox + r0 * N2;
      }
      if (fx)
        fx->x_inv<<<xb, fx->threads, fx->smem_row, st>>>(xs, rho_c, (int)nr, N1, p->P[1], N2, p->HS, out_scale,
                                                         p->tw[2]);
      else
        k_x_inv<<<xb, NT, p->smem_x, st>>>(xs, rho_c, (int)nr, N1, p->P[1], N2, p->HS, out_scale, p->f[2], p->tw[2]);
      PVD_LAUNCH_CHECK("x_inv");
    }
    if (hio) {  // this chunk goes back while the next one computes
      cudaEvent_t ev = p->ev_dose[c];
      PVD_CUDA_TRY(cudaEventRecord(ev, st));
      PVD_CUDA_TRY(cudaStreamWaitEvent(p->s_d2h, ev, 0));
      for (int s = 0; s < p->nk; ++s)
        PVD_CUDA_TRY(cudaMemcpyAsync(hio->dose + s * vox + r0 * N2, dose + s * vox + r0 * N2, sizeof(float) * nr * N2,
                                     cudaMemcpyDeviceToHost, p->s_d2h));
    }
  }
  if (hio) {  // the caller's stream completes only after the last copy back
    PVD_CUDA_TRY(cudaEventRecord(p->ev_done, p->s_d2h));
    PVD_CUDA_TRY(cudaStreamWaitEvent(st, p->ev_done, 0));
  }
  return PVD_OK;
}

extern "C" pvd_status pvd_conv_execute(pvd_plan* p, const float* act, const float* rho, float* dose, float out_scale,
                                       pvd_stream stream) {
  if (!p || !act) return set_error(PVD_ERR_ARG, "pvd_conv_execute: null argument");
  ActIn in;
  std::memset(&in, 0, sizeof(in));
  in.n = 1;
  in.p[0] = act;
  in.w[0] = 1.0f;
  return conv_run(p, in, rho, dose, out_scale, stream);
}

extern "C" pvd_status pvd_conv_execute_host(pvd_plan* p, const float* act_h, const float* rho_h, float* dose_h,
                                            float out_scale, pvd_stream stream) {
  if (!p || !act_h || !dose_h) return set_error(PVD_ERR_ARG, "pvd_conv_execute_host: null argument");
  cudaStream_t st = (cudaStream_t)stream;
  const int N0 = p->N[0], N1 = p->N[1], N2 = p->N[2];
  const long long vox = (long long)N0 * N1 * N2;
  const size_t vb = sizeof(float) * (size_t)vox;
  // lazily created staging buffers, streams and events (kept for later calls)
  void* ptr = nullptr;
  pvd_status as = PVD_OK;
  if (!p->io_act) {
    if ((as = plan_alloc(p, vb, &ptr)) != PVD_OK) return as;
    p->io_act = (float*)ptr;
  }
  if (rho_h && !p->io_rho) {
    if ((as = plan_alloc(p, vb, &ptr)) != PVD_OK) return as;
    p->io_rho = (float*)ptr;
  }
  if (!p->io_dose) {
    if ((as = plan_alloc(p, vb * p->nk, &ptr)) != PVD_OK) return as;
    p->io_dose = (float*)ptr;
  }
  if (!p->s_h2d) {
    PVD_CUDA_TRY(cudaStreamCreateWithFlags(&p->s_h2d, cudaStreamNonBlocking));
    PVD_CUDA_TRY(cudaStreamCreateWithFlags(&p->s_d2h, cudaStreamNonBlocking));
    PVD_CUDA_TRY(cudaEventCreateWithFlags(&p->ev_start, cudaEventDisableTiming));
    for (auto& e : p->ev_rho) PVD_CUDA_TRY(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    PVD_CUDA_TRY(cudaEventCreateWithFlags(&p->ev_done, cudaEventDisableTiming));
    for (auto& e : p->ev_act) PVD_CUDA_TRY(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    for (auto& e : p->ev_dose) PVD_CUDA_TRY(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  }
  // uploads start after everything already queued on the caller's stream (which
  // may still read the staging buffers of a previous call)
  PVD_CUDA_TRY(cudaEventRecord(p->ev_start, st));
  PVD_CUDA_TRY(cudaStreamWaitEvent(p->s_h2d, p->ev_start, 0));
  const int nchunks = std::min(PVD_HOST_CHUNKS, N0);
  for (int c = 0; c < nchunks; ++c) {
    const long long z0 = (long long)N0 * c / nchunks, z1 = (long long)N0 * (c + 1) / nchunks;
    const long long off = z0 * N1 * N2, n = (z1 - z0) * N1 * N2;
    if (n > 0)
      PVD_CUDA_TRY(cudaMemcpyAsync(p->io_act + off, act_h + off, sizeof(float) * n, cudaMemcpyHostToDevice, p->s_h2d));
    PVD_CUDA_TRY(cudaEventRecord(p->ev_act[c], p->s_h2d));
  }
  if (rho_h) {  // in the z chunks the inverse x pass consumes them in
    const int dchunks = std::min(PVD_DOSE_CHUNKS, N0);
    for (int c = 0; c < dchunks; ++c) {
      const long long z0 = (long long)N0 * c / dchunks, z1 = (long long)N0 * (c + 1) / dchunks;
      const long long off = z0 * N1 * N2, n = (z1 - z0) * N1 * N2;
      if (n > 0)
        PVD_CUDA_TRY(cudaMemcpyAsync(p->io_rho + off, rho_h + off, sizeof(float) * n, cudaMemcpyHostToDevice,
                                     p->s_h2d));
      PVD_CUDA_TRY(cudaEventRecord(p->ev_rho[c], p->s_h2d));
    }
  }
  ActIn in;
  std::memset(&in, 0, sizeof(in));
  in.n = 1;
  in.p[0] = p->io_act;
  in.w[0] = 1.0f;
  HostIO hio{act_h, rho_h, dose_h};
  return conv_run(p, in, rho_h ? p->io_rho : nullptr, p->io_dose, out_scale, stream, &hio);
}

extern "C" pvd_status pvd_conv_execute_weighted(pvd_plan* p, const float* const* act, const float* w, int n_act,
                                                const float* rho, float* dose, float out_scale, pvd_stream stream) {
  if (!p || !act || !w) return set_error(PVD_ERR_ARG, "pvd_conv_execute_weighted: null argument");
  if (n_act < 1 || n_act > PVD_MAX_TIMEPOINTS)
    return set_error(PVD_ERR_ARG, "pvd_conv_execute_weighted: n_act must be in [1, 16]");
  ActIn in;
  std::memset(&in, 0, sizeof(in));
  in.n = n_act;
  for (int t = 0; t < n_act; ++t) {
    if (!act[t]) return set_error(PVD_ERR_ARG, "pvd_conv_execute_weighted: null activity pointer");
    if (!std::isfinite(w[t])) return set_error(PVD_ERR_NUMERIC, "pvd_conv_execute_weighted: non-finite weight");
    in.p[t] = act[t];
    in.w[t] = w[t];
  }
  return conv_run(p, in, rho, dose, out_scale, stream);
}

extern "C" pvd_status pvd_plan_profile(pvd_plan* p, int enable) {
  if (!p) return set_error(PVD_ERR_ARG, "pvd_plan_profile: null plan");
  p->prof = enable ? 1 : 0;
  p->recs.clear();
  p->ev_used = 0;
  return PVD_OK;
}

extern "C" pvd_status pvd_plan_pass_times(pvd_plan* p, double* ms, int* launches) {
  if (!p || !ms || !launches) return set_error(PVD_ERR_ARG, "pvd_plan_pass_times: null argument");
  for (int i = 0; i < PVD_NUM_PASSES; ++i) {
    ms[i] = 0.0;
    launches[i] = 0;
  }
  for (const auto& r : p->recs) {
    cudaError_t e = cudaEventSynchronize(r.b);
    if (e != cudaSuccess) return cuda_error(e, "pvd_plan_pass_times");
    float t = 0.f;
    e = cudaEventElapsedTime(&t, r.a, r.b);
    if (e != cudaSuccess) return cuda_error(e, "pvd_plan_pass_times");
    ms[r.kind] += t;
    launches[r.kind] += 1;
  }
  return PVD_OK;
}

extern "C" pvd_status pvd_plan_status(const pvd_plan* p) {
  if (!p) return set_error(PVD_ERR_ARG, "pvd_plan_status: null plan");
  if (!p->d_err) return PVD_OK;
  int v = 0;
  PVD_CUDA_TRY(cudaMemcpy(&v, p->d_err, sizeof(int), cudaMemcpyDeviceToHost));
  if (v) {  // reported once: the word is cleared for the plan's later work
    PVD_CUDA_TRY(cudaMemset(p->d_err, 0, sizeof(int)));
    return set_error((pvd_status)v, "pvd_plan_status: a bounded wait of a pass ran out (TMA tile load not complete)");
  }
  return PVD_OK;
}

namespace {
// One CTA waits, through the TMA passes' own bounded wait, on a barrier phase that
// nothing completes: no copy is issued, so nothing is in flight when the wait ends.
__global__ void k_plan_wait_check(uint64_t limit_ns, int* err) {
  __shared__ uint64_t bar;
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);
    fence_mbar_init();
  }
  __syncthreads();
  if (!cta_stage_wait(&bar, 0, limit_ns, err)) return;
}
}  // namespace

namespace pvd {
pvd_status plan_wait_check(pvd_plan* p, unsigned long long limit_ns, cudaStream_t st) {
  if (!p) return set_error(PVD_ERR_ARG, "pvd_wait_check: null plan");
  k_plan_wait_check<<<1, 128, 0, st>>>(limit_ns, p->d_err);
  PVD_LAUNCH_CHECK("k_plan_wait_check");
  return PVD_OK;
}
}  // namespace pvd

extern "C" pvd_status pvd_set_plan_alloc_cap(size_t bytes) {
  g_plan_alloc_cap.store(bytes);
  return PVD_OK;
}

extern "C" pvd_status pvd_plan_destroy(pvd_plan* p) {
  if (!p) return PVD_OK;
  plan_free(p);
  delete p;
  return PVD_OK;
}

// ===========================================================================
// Allocation-free convolution (no counterpart in the reference).
//
// Some callers cannot allocate device memory: code that runs under a memory
// budget enforced by a host framework that owns the allocator, or plugins that
// must not call cudaMalloc/cudaFree (they synchronise the device and would
// stall the host application's streams).
// pvd_conv_execute_static runs the same five-pass pipeline as a plan, with all
// of its scratch (twiddles, kernel staging, spectrum, the two spectral work
// buffers) carved out of one file-scope device array of PVD_STATIC_SCRATCH_BYTES.
// The host code below never uses the array's name as an address: on the first
// call on a device (with that device current) it asks the runtime for the
// array's device address with cudaGetSymbolAddress and caches it per device.
// ===========================================================================

namespace {

__device__ __align__(256) unsigned char g_conv_scratch[PVD_STATIC_SCRATCH_BYTES];

std::mutex g_scratch_mu;
void* g_scratch_addr[PVD_STATIC_MAX_DEVICES] = {};

// Device address of g_conv_scratch on the current device (looked up once per device).
pvd_status static_scratch_address(void** out) {
  int dev = 0;
  PVD_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= PVD_STATIC_MAX_DEVICES)
    return set_error(PVD_ERR_UNSUPPORTED, "pvd_conv_execute_static: device ordinal out of range");
  std::lock_guard<std::mutex> lock(g_scratch_mu);
  if (!g_scratch_addr[dev]) {
    void* addr = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&addr, g_conv_scratch);
    if (e != cudaSuccess) return cuda_error(e, "cudaGetSymbolAddress(g_conv_scratch)");
    g_scratch_addr[dev] = addr;
  }
  *out = g_scratch_addr[dev];
  return PVD_OK;
}

// twiddles exp(-2 pi i n / L) computed on the device (no host staging buffer)
__global__ void k_twiddle(float2* __restrict__ tw, int L) {
  for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < L; n += gridDim.x * blockDim.x) {
    float s, c;
    sincospif(-2.0f * (float)n / (float)L, &s, &c);
    tw[n] = make_float2(c, s);
  }
}

size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

}  // namespace

extern "C" pvd_status pvd_conv_execute_static(const float* activity_d, const float* density_d, float* dose_d,
                                              int n0, int n1, int n2, const double* kernel_h, int k0, int k1,
                                              int k2, double scale, int flags, float out_scale, pvd_stream stream) {
  if (!activity_d || !dose_d || !kernel_h) return set_error(PVD_ERR_ARG, "pvd_conv_execute_static: null argument");
  if (flags & ~PVD_KERNEL_NORMALIZE) return set_error(PVD_ERR_ARG, "pvd_conv_execute_static: unknown flags");
  const int N[3] = {n0, n1, n2}, K[3] = {k0, k1, k2};
  for (int i = 0; i < 3; ++i) {
    if (N[i] < 1 || N[i] > 4096) return set_error(PVD_ERR_ARG, "pvd_conv_execute_static: volume dims must be in [1, 4096]");
    if (K[i] < 1 || K[i] > 1024) return set_error(PVD_ERR_ARG, "pvd_conv_execute_static: kernel dims must be in [1, 1024]");
  }
  if (!std::isfinite(scale) || !std::isfinite(out_scale))
    return set_error(PVD_ERR_NUMERIC, "pvd_conv_execute_static: non-finite scale");
  const long long nk = (long long)k0 * k1 * k2;
  double host_sum = 0.0;
  for (long long i = 0; i < nk; ++i) {
    if (!std::isfinite(kernel_h[i])) return set_error(PVD_ERR_NUMERIC, "pvd_conv_execute_static: non-finite kernel value");
    host_sum += kernel_h[i];
  }
  // the same rule as pvd_plan_set_kernel: a kernel that sums to zero (or overflows) cannot
  // be normalised; the device still computes the normalisation sum itself in FP64
  if ((flags & PVD_KERNEL_NORMALIZE) && !(std::isfinite(host_sum) && host_sum != 0.0))
    return set_error(PVD_ERR_NUMERIC, "pvd_conv_execute_static: kernel sum is zero or non-finite; cannot normalise");

  // plan on the stack: same length choice and pass kernels as pvd_plan_create (LINEAR, one slot)
  pvd_plan p;
  p.mode = PVD_MODE_LINEAR;
  p.nk = 1;
  for (int i = 0; i < 3; ++i) {
    p.N[i] = N[i];
    p.kmax[i] = K[i];
    const int need = N[i] + K[i] - 1;
    const int lf = fast_len_at_least(need), ls = next_smooth7(need);
    const int L = (lf && (lf == ls || 4 * lf <= 5 * need)) ? lf : ls;
    if (!factorize(L, &p.f[i])) return set_error(PVD_ERR_UNSUPPORTED, "pvd_conv_execute_static: FFT length not 7-smooth");
    p.P[i] = L;
    p.fl[i] = fast_len(L);
  }
  p.H = p.P[2] / 2 + 1;
  p.HS = (p.H + TX - 1) / TX * TX;
  p.smem_x = smem_bytes(p.P[2], 2);
  p.smem_y = smem_bytes(p.P[1], 2);
  p.smem_z = smem_bytes(p.P[0], 2);

  // real-even spectrum for kernels that are even along every axis (as pvd_plan_set_kernel)
  bool sym = true;
  for (int i = 0; i < 3; ++i)
    if (K[i] % 2 == 0) sym = false;
  for (long long i = 0; sym && i < nk; ++i) {
    const int a = (int)(i / ((long long)k1 * k2)), b = (int)((i / k2) % k1), c = (int)(i % k2);
    const long long jz = ((long long)(k0 - 1 - a) * k1 + b) * k2 + c;
    const long long jy = ((long long)a * k1 + (k1 - 1 - b)) * k2 + c;
    const long long jx = ((long long)a * k1 + b) * k2 + (k2 - 1 - c);
    if (kernel_h[i] != kernel_h[jz] || kernel_h[i] != kernel_h[jy] || kernel_h[i] != kernel_h[jx]) sym = false;
  }
  const int smode = sym ? SPEC_REAL_EVEN : SPEC_COMPLEX;

  // scratch layout (256-byte aligned regions); T1 / T2 of the spectrum build
  // share the two spectral work buffers, which the pipeline fills afterwards
  const size_t b_tw0 = sizeof(float2) * p.P[0], b_tw1 = sizeof(float2) * p.P[1], b_tw2 = sizeof(float2) * p.P[2];
  const size_t b_spec = sym ? sizeof(float) * (size_t)(p.P[0] / 2 + 1) * (p.P[1] / 2 + 1) * p.HS
                            : sizeof(float2) * (size_t)p.P[0] * p.P[1] * p.HS;
  const size_t b_buf1 = std::max(sizeof(float2) * (size_t)n0 * n1 * p.HS, sizeof(float2) * (size_t)k0 * p.P[1] * p.H);
  const size_t b_buf2 = std::max(sizeof(float2) * (size_t)n0 * p.P[1] * p.HS, sizeof(float2) * (size_t)k0 * k1 * p.H);
  const size_t b_kd = sizeof(double) * (size_t)nk, b_kf = sizeof(float) * (size_t)nk, b_sum = sizeof(double);
  size_t off = 0;
  const size_t o_tw0 = off; off += align256(b_tw0);
  const size_t o_tw1 = off; off += align256(b_tw1);
  const size_t o_tw2 = off; off += align256(b_tw2);
  const size_t o_spec = off; off += align256(b_spec);
  const size_t o_buf1 = off; off += align256(b_buf1);
  const size_t o_buf2 = off; off += align256(b_buf2);
  const size_t o_kd = off; off += align256(b_kd);
  const size_t o_kf = off; off += align256(b_kf);
  const size_t o_sum = off; off += align256(b_sum);
  if (off > PVD_STATIC_SCRATCH_BYTES)
    return set_error(PVD_ERR_UNSUPPORTED, "pvd_conv_execute_static: this volume/kernel needs " + std::to_string(off) +
                                              " bytes of scratch, more than the static maximum of " +
                                              std::to_string((size_t)PVD_STATIC_SCRATCH_BYTES) +
                                              " bytes; use a plan (pvd_plan_create)");
  void* base = nullptr;
  pvd_status st0 = static_scratch_address(&base);
  if (st0 != PVD_OK) return st0;
  unsigned char* sb = (unsigned char*)base;
  p.tw[0] = (float2*)(sb + o_tw0);
  p.tw[1] = (float2*)(sb + o_tw1);
  p.tw[2] = (float2*)(sb + o_tw2);
  p.spec[0] = sb + o_spec;
  p.spec_mode[0] = smode;
  p.spec_set[0] = 1;
  p.buf1 = (float2*)(sb + o_buf1);
  p.buf2 = (float2*)(sb + o_buf2);
  p.buf3[0] = p.buf2;
  double* kd = (double*)(sb + o_kd);
  float* kf = (float*)(sb + o_kf);
  double* sumd = (double*)(sb + o_sum);

  int smem_max = 0, cur = 0;
  PVD_CUDA_TRY(cudaGetDevice(&cur));
  PVD_CUDA_TRY(cudaDeviceGetAttribute(&smem_max, cudaDevAttrMaxSharedMemoryPerBlockOptin, cur));
  if (!pass_tiles_fit(p.fl, p.smem_x, p.smem_y, p.smem_z, smem_max))
    return set_error(PVD_ERR_UNSUPPORTED, "pvd_conv_execute_static: FFT length too large for one shared-memory tile");

  cudaStream_t st = (cudaStream_t)stream;
  for (int i = 0; i < 3; ++i) {
    k_twiddle<<<(p.P[i] + 255) / 256, 256, 0, st>>>(p.tw[i], p.P[i]);
    PVD_LAUNCH_CHECK("k_twiddle");
  }
  // kernel spectrum (FP64 normalisation sum on the GPU when asked), into scratch
  PVD_CUDA_TRY(cudaMemcpyAsync(kd, kernel_h, b_kd, cudaMemcpyHostToDevice, st));
  const bool norm = (flags & PVD_KERNEL_NORMALIZE) != 0;
  if (norm) {
    k_sum_f64<<<1, NT, 0, st>>>(kd, nk, sumd);
    PVD_LAUNCH_CHECK("k_sum_f64");
  }
  const double inv_p = 1.0 / ((double)p.P[0] * p.P[1] * p.P[2]);
  const int o[3] = {k0 / 2, k1 / 2, k2 / 2};
  const int Ke[3] = {std::min(k0, p.P[0]), std::min(k1, p.P[1]), std::min(k2, p.P[2])};
  const int gs = 152 * 8;
  float2* t1 = p.buf2;
  float2* t2 = p.buf1;
  k_scale_to_f32<<<gs, NT, 0, st>>>(kd, nk, norm ? sumd : nullptr, scale * inv_p, kf);
  PVD_LAUNCH_CHECK("k_scale_to_f32");
  k_spec_x<<<gs, NT, 0, st>>>(kf, t1, k0, k1, k2, Ke[2], o[2], 0, p.P[2], p.H, p.tw[2]);
  PVD_LAUNCH_CHECK("k_spec_x");
  k_spec_y<<<gs, NT, 0, st>>>(t1, t2, k0, k1, Ke[1], o[1], 0, p.P[1], p.H, p.tw[1]);
  PVD_LAUNCH_CHECK("k_spec_y");
  k_spec_z<<<gs, NT, 0, st>>>(t2, p.spec[0], smode, Ke[0], o[0], 0, p.P[0], p.P[1], p.H, p.HS, p.tw[0]);
  PVD_LAUNCH_CHECK("k_spec_z");
  // the array keeps the previous call's contents: the padding columns [H, HS)
  // of the first work buffer must start at zero
  PVD_CUDA_TRY(cudaMemsetAsync(p.buf1, 0, sizeof(float2) * (size_t)n0 * n1 * p.HS, st));

  ActIn in;
  std::memset(&in, 0, sizeof(in));
  in.n = 1;
  in.p[0] = activity_d;
  in.w[0] = 1.0f;
  return conv_run(&p, in, density_d, dose_d, out_scale, stream);
}
