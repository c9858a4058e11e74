// Dose-volume histogram on the GPU.
//
// Replaces calculate_dvh (pyvoxeldosimetry/core/utils.py:233-262): the doses
// inside an ROI (mask > 0) are histogrammed with np.histogram(roi, bins) — bins
// uniform between the ROI's minimum and maximum — and turned into 1 - cumsum / n.
// Two HBM-bound passes over the volume:
//   k_roi_stats  min, max, count and non-finite count of the ROI doses
//                (numpy raises for a non-finite range; the host does too);
//   k_histogram  the bin of every ROI dose by numpy's own arithmetic for
//                uniform bins (numpy/lib/_histograms_impl.py, `histogram`):
//                f = ((x - first) / (last - first)) * bins in the dose's type,
//                truncated; index bins -> bins - 1; one step down if
//                x < edge[i], one step up if x >= edge[i+1] and i != bins - 1,
//                with the edges numpy's linspace produced (given by the host).
//                Every operation is an IEEE round-to-nearest intrinsic, so the
//                counts are the ones np.histogram returns, bit for bit.
// Counts are accumulated per block in shared memory (bins <= kSmemBins), then
// added to 64-bit global counters.
#include <algorithm>
#include <cstdint>
#include <cstring>

#include "pvd_common.cuh"

namespace pvd {

constexpr int kSmemBins = 12288;  // 48 KB of 32-bit counters
constexpr int kDvhThreads = 256;

__device__ __forceinline__ unsigned long long order_key(float x) {
  const unsigned int b = __float_as_uint(x);
  return (unsigned long long)((b & 0x80000000u) ? ~b : (b | 0x80000000u));
}
__device__ __forceinline__ unsigned long long order_key(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  return (b & 0x8000000000000000ull) ? ~b : (b | 0x8000000000000000ull);
}

template <typename M>
__device__ __forceinline__ bool in_roi(const M* mask, long long i) {
  return mask == nullptr || __ldg(mask + i) > (M)0;
}

// Four consecutive voxels per load: float4 / two double2 for the dose, uchar4 / float4
// for the mask (VEC: the pointers are 16-byte aligned), else four scalar loads.
// Dose and mask are loaded together, so each thread keeps both in flight.
template <typename T, bool VEC>
__device__ __forceinline__ void load4(const T* __restrict__ p, long long i, T* x) {
  if constexpr (VEC && sizeof(T) == 4) {
    const float4 v = __ldg(reinterpret_cast<const float4*>(p + i));
    x[0] = v.x, x[1] = v.y, x[2] = v.z, x[3] = v.w;
  } else if constexpr (VEC) {
    const double2 a = __ldg(reinterpret_cast<const double2*>(p + i));
    const double2 b = __ldg(reinterpret_cast<const double2*>(p + i + 2));
    x[0] = a.x, x[1] = a.y, x[2] = b.x, x[3] = b.y;
  } else {
#pragma unroll
    for (int k = 0; k < 4; ++k) x[k] = __ldg(p + i + k);
  }
}
template <typename M, bool VEC>
__device__ __forceinline__ void roi4(const M* __restrict__ m, long long i, bool* in) {
  if (m == nullptr) {
    in[0] = in[1] = in[2] = in[3] = true;
  } else if constexpr (VEC && sizeof(M) == 1) {
    const uchar4 v = __ldg(reinterpret_cast<const uchar4*>(m + i));
    in[0] = v.x > 0, in[1] = v.y > 0, in[2] = v.z > 0, in[3] = v.w > 0;
  } else if constexpr (VEC) {
    const float4 v = __ldg(reinterpret_cast<const float4*>(m + i));
    in[0] = v.x > 0.f, in[1] = v.y > 0.f, in[2] = v.z > 0.f, in[3] = v.w > 0.f;
  } else {
#pragma unroll
    for (int k = 0; k < 4; ++k) in[k] = __ldg(m + i + k) > (M)0;
  }
}

// out[0] = min key, out[1] = max key, out[2] = ROI count, out[3] = non-finite ROI count
template <typename T, typename M, bool VEC>
__global__ void __launch_bounds__(kDvhThreads) k_roi_stats(const T* __restrict__ dose, const M* __restrict__ mask,
                                                           long long n, unsigned long long* __restrict__ out) {
  unsigned long long kmin = ~0ull, kmax = 0ull, cnt = 0ull, bad = 0ull;
  const long long stride = (long long)gridDim.x * blockDim.x;
  const long long tid = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  auto take = [&](T x) {
    ++cnt;
    if (!isfinite(x)) {
      ++bad;
      return;
    }
    const unsigned long long k = order_key(x);
    kmin = min(kmin, k);
    kmax = max(kmax, k);
  };
  const long long n4 = n / 4;
  for (long long q = tid; q < n4; q += stride) {
    T x[4];
    bool in[4];
    load4<T, VEC>(dose, 4 * q, x);
    roi4<M, VEC>(mask, 4 * q, in);
#pragma unroll
    for (int k = 0; k < 4; ++k)
      if (in[k]) take(x[k]);
  }
  for (long long i = 4 * n4 + tid; i < n; i += stride)
    if (in_roi(mask, i)) take(__ldg(dose + i));
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    kmin = min(kmin, __shfl_xor_sync(0xffffffffu, kmin, o));
    kmax = max(kmax, __shfl_xor_sync(0xffffffffu, kmax, o));
    cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
    bad += __shfl_xor_sync(0xffffffffu, bad, o);
  }
  if ((threadIdx.x & 31) == 0) {
    if (cnt > bad) {
      atomicMin(out + 0, kmin);
      atomicMax(out + 1, kmax);
    }
    if (cnt) atomicAdd(out + 2, cnt);
    if (bad) atomicAdd(out + 3, bad);
  }
}

__device__ __forceinline__ float sub_rn(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float div_rn(float a, float b) { return __fdiv_rn(a, b); }
__device__ __forceinline__ float mul_rn(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double sub_rn(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double div_rn(double a, double b) { return __ddiv_rn(a, b); }
__device__ __forceinline__ double mul_rn(double a, double b) { return __dmul_rn(a, b); }

__device__ __forceinline__ float add_rn(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ double add_rn(double a, double b) { return __dadd_rn(a, b); }

template <typename T> __device__ __forceinline__ T key_value(unsigned long long k);
template <> __device__ __forceinline__ float key_value<float>(unsigned long long k) {
  const unsigned int u = (unsigned int)k;
  return __uint_as_float((u & 0x80000000u) ? (u & 0x7fffffffu) : ~u);
}
template <> __device__ __forceinline__ double key_value<double>(unsigned long long k) {
  return __longlong_as_double((long long)((k & 0x8000000000000000ull) ? (k & 0x7fffffffffffffffull) : ~k));
}

// The bins+1 edges numpy's histogram uses, from the ROI statistics: range widened by
// 0.5 on each side when empty, then np.linspace(first, last, bins + 1) in the dose's
// type (numpy/_core/function_base.py `linspace`: step = (last - first) / bins,
// edge i = i * step + first, the last edge = last; (i / bins) * (last - first) + first
// when the step underflows to 0).  Nothing is written for an empty or non-finite ROI.
template <typename T>
__global__ void k_dvh_edges(const unsigned long long* __restrict__ acc, int bins, T* __restrict__ edges) {
  if (acc[2] == 0ull || acc[3] != 0ull) return;
  T first = key_value<T>(acc[0]), last = key_value<T>(acc[1]);
  if (first == last) {
    first = sub_rn(first, (T)0.5);
    last = add_rn(last, (T)0.5);
  }
  const T delta = sub_rn(last, first);
  const T div = (T)bins;
  const T step = div_rn(delta, div);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i <= bins; i += gridDim.x * blockDim.x) {
    T y;
    if (i == bins)
      y = last;
    else if (step == (T)0)
      y = add_rn(mul_rn(div_rn((T)i, div), delta), first);
    else
      y = add_rn(mul_rn((T)i, step), first);
    edges[i] = y;
  }
}

template <typename T>
__device__ __forceinline__ int bin_of(T x, T first, T denom, T nb, int bins, const T* __restrict__ edges) {
  const T f = mul_rn(div_rn(sub_rn(x, first), denom), nb);
  long long i = (long long)f;  // f >= 0: truncation, as astype(intp)
  if (i >= bins) i = bins - 1;
  if (i > 0 && x < __ldg(edges + i)) --i;
  if (i != bins - 1 && x >= __ldg(edges + i + 1)) ++i;
  return (int)i;
}

// acc (nullable): ROI statistics of k_roi_stats; nothing is counted for an empty or non-finite ROI
template <typename T, typename M, bool SMEM, bool VEC>
__global__ void __launch_bounds__(kDvhThreads) k_histogram(const T* __restrict__ dose, const M* __restrict__ mask,
                                                           long long n, const T* __restrict__ edges, int bins,
                                                           unsigned long long* __restrict__ counts,
                                                           const unsigned long long* __restrict__ acc) {
  if (acc && (acc[2] == 0ull || acc[3] != 0ull)) return;
  __shared__ unsigned int h[SMEM ? kSmemBins : 1];
  if (SMEM) {
    for (int b = threadIdx.x; b < bins; b += blockDim.x) h[b] = 0u;
    __syncthreads();
  }
  const T first = __ldg(edges), last = __ldg(edges + bins);
  const T denom = sub_rn(last, first), nb = (T)bins;
  const long long stride = (long long)gridDim.x * blockDim.x;
  const long long tid = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  auto count = [&](T x) {
    if (!(x >= first && x <= last)) return;  // numpy keeps [first, last] only
    const int b = bin_of<T>(x, first, denom, nb, bins, edges);
    if (SMEM)
      atomicAdd(h + b, 1u);
    else
      atomicAdd(counts + b, 1ull);
  };
  const long long n4 = n / 4;
  for (long long q = tid; q < n4; q += stride) {
    T x[4];
    bool in[4];
    load4<T, VEC>(dose, 4 * q, x);
    roi4<M, VEC>(mask, 4 * q, in);
#pragma unroll
    for (int k = 0; k < 4; ++k)
      if (in[k]) count(x[k]);
  }
  for (long long i = 4 * n4 + tid; i < n; i += stride)
    if (in_roi(mask, i)) count(__ldg(dose + i));
  if (SMEM) {
    __syncthreads();
    for (int b = threadIdx.x; b < bins; b += blockDim.x)
      if (h[b]) atomicAdd(counts + b, (unsigned long long)h[b]);
  }
}

static int grid_for(long long n) {
  return (int)std::max<long long>(1, std::min<long long>((n + kDvhThreads - 1) / kDvhThreads, 152LL * 8));
}

static bool aligned16(const void* p) { return ((uintptr_t)p & 15u) == 0; }

// vector loads when dose and mask start on 16-byte boundaries (4 voxels of the mask
// span 4 or 16 bytes, and every group starts at a multiple of 4 voxels)
static bool vec_ok(const void* dose, const void* mask) { return aligned16(dose) && (!mask || aligned16(mask)); }

template <typename T, typename M>
static void launch_stats(const void* dose, const void* mask, long long n, unsigned long long* out, cudaStream_t st) {
  const int g = grid_for((n + 3) / 4);
  if (vec_ok(dose, mask))
    k_roi_stats<T, M, true><<<g, kDvhThreads, 0, st>>>((const T*)dose, (const M*)mask, n, out);
  else
    k_roi_stats<T, M, false><<<g, kDvhThreads, 0, st>>>((const T*)dose, (const M*)mask, n, out);
}

template <typename T, typename M>
static void launch_hist(const void* dose, const void* mask, long long n, const void* edges, int bins,
                        unsigned long long* counts, cudaStream_t st, const unsigned long long* acc = nullptr) {
  const int g = grid_for((n + 3) / 4);
  const bool v = vec_ok(dose, mask);
#define PVD_HIST(SM, VE)                                                                                     \
  k_histogram<T, M, SM, VE><<<g, kDvhThreads, 0, st>>>((const T*)dose, (const M*)mask, n, (const T*)edges, bins, \
                                                       counts, acc)
  if (bins <= kSmemBins) {
    if (v)
      PVD_HIST(true, true);
    else
      PVD_HIST(true, false);
  } else {
    if (v)
      PVD_HIST(false, true);
    else
      PVD_HIST(false, false);
  }
#undef PVD_HIST
}

template <typename T, typename M>
static void launch_dvh(const void* dose, const void* mask, long long n, int bins, void* edges,
                       unsigned long long* res, cudaStream_t st) {
  launch_stats<T, M>(dose, mask, n, res, st);
  k_dvh_edges<T><<<(bins + 256) / 256, 256, 0, st>>>(res, bins, (T*)edges);
  launch_hist<T, M>(dose, mask, n, edges, bins, res + 4, st, res);
}

static double key_to_value(unsigned long long k, int dtype) {
  if (dtype == PVD_DTYPE_F32) {
    const unsigned int u = (unsigned int)k;
    const unsigned int b = (u & 0x80000000u) ? (u & 0x7fffffffu) : ~u;
    float f;
    std::memcpy(&f, &b, 4);
    return (double)f;
  }
  const unsigned long long b = (k & 0x8000000000000000ull) ? (k & 0x7fffffffffffffffull) : ~k;
  double d;
  std::memcpy(&d, &b, 8);
  return d;
}

static bool dtypes_ok(int dose_dtype, int mask_dtype) {
  return (dose_dtype == PVD_DTYPE_F32 || dose_dtype == PVD_DTYPE_F64) &&
         (mask_dtype == PVD_DTYPE_U8 || mask_dtype == PVD_DTYPE_F32);
}

}  // namespace pvd

using namespace pvd;

extern "C" pvd_status pvd_roi_stats(const void* dose_d, int dose_dtype, const void* mask_d, int mask_dtype, long long n,
                                    pvd_roi_stats_t* out, pvd_stream stream) {
  if (!dose_d || !out) return set_error(PVD_ERR_ARG, "pvd_roi_stats: null argument");
  if (n < 0) return set_error(PVD_ERR_ARG, "pvd_roi_stats: negative voxel count");
  if (!dtypes_ok(dose_dtype, mask_dtype))
    return set_error(PVD_ERR_ARG, "pvd_roi_stats: dose must be PVD_DTYPE_F32/F64, mask PVD_DTYPE_U8/F32");
  out->min = 0.0;
  out->max = 0.0;
  out->count = 0;
  out->nonfinite = 0;
  if (n == 0) return PVD_OK;
  cudaStream_t st = (cudaStream_t)stream;
  unsigned long long* acc = nullptr;
  cudaError_t e = cudaMallocAsync((void**)&acc, 4 * sizeof(unsigned long long), st);
  if (e != cudaSuccess) return set_error(PVD_ERR_OOM, std::string("pvd_roi_stats: ") + cudaGetErrorString(e));
  const unsigned long long init[4] = {~0ull, 0ull, 0ull, 0ull};
  unsigned long long host[4];
  e = cudaMemcpyAsync(acc, init, sizeof(init), cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) {
    if (dose_dtype == PVD_DTYPE_F32)
      (mask_dtype == PVD_DTYPE_U8) ? launch_stats<float, unsigned char>(dose_d, mask_d, n, acc, st)
                                   : launch_stats<float, float>(dose_d, mask_d, n, acc, st);
    else
      (mask_dtype == PVD_DTYPE_U8) ? launch_stats<double, unsigned char>(dose_d, mask_d, n, acc, st)
                                   : launch_stats<double, float>(dose_d, mask_d, n, acc, st);
    count_launch();
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(host, acc, sizeof(host), cudaMemcpyDeviceToHost, st);
  cudaFreeAsync(acc, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return set_error(PVD_ERR_CUDA, std::string("pvd_roi_stats: ") + cudaGetErrorString(e));
  out->count = (long long)host[2];
  out->nonfinite = (long long)host[3];
  if (host[2] > host[3]) {
    out->min = key_to_value(host[0], dose_dtype);
    out->max = key_to_value(host[1], dose_dtype);
  }
  return PVD_OK;
}

extern "C" pvd_status pvd_histogram(const void* dose_d, int dose_dtype, const void* mask_d, int mask_dtype, long long n,
                                    const void* edges_d, int bins, long long* counts_d, pvd_stream stream) {
  if (!dose_d || !edges_d || !counts_d) return set_error(PVD_ERR_ARG, "pvd_histogram: null argument");
  if (n < 0 || bins < 1) return set_error(PVD_ERR_ARG, "pvd_histogram: need n >= 0 and bins >= 1");
  if (!dtypes_ok(dose_dtype, mask_dtype))
    return set_error(PVD_ERR_ARG, "pvd_histogram: dose must be PVD_DTYPE_F32/F64, mask PVD_DTYPE_U8/F32");
  cudaStream_t st = (cudaStream_t)stream;
  cudaError_t e = cudaMemsetAsync(counts_d, 0, sizeof(long long) * (size_t)bins, st);
  if (e != cudaSuccess) return set_error(PVD_ERR_CUDA, std::string("pvd_histogram: ") + cudaGetErrorString(e));
  if (n == 0) return PVD_OK;
  unsigned long long* c = (unsigned long long*)counts_d;
  if (dose_dtype == PVD_DTYPE_F32)
    (mask_dtype == PVD_DTYPE_U8) ? launch_hist<float, unsigned char>(dose_d, mask_d, n, edges_d, bins, c, st)
                                 : launch_hist<float, float>(dose_d, mask_d, n, edges_d, bins, c, st);
  else
    (mask_dtype == PVD_DTYPE_U8) ? launch_hist<double, unsigned char>(dose_d, mask_d, n, edges_d, bins, c, st)
                                 : launch_hist<double, float>(dose_d, mask_d, n, edges_d, bins, c, st);
  PVD_LAUNCH_CHECK("k_histogram");
  return PVD_OK;
}

extern "C" pvd_status pvd_dvh(const void* dose_d, int dose_dtype, const void* mask_d, int mask_dtype, long long n,
                              int bins, void* edges_d, long long* result_d, pvd_stream stream) {
  if (!dose_d || !edges_d || !result_d) return set_error(PVD_ERR_ARG, "pvd_dvh: null argument");
  if (n < 1 || bins < 1) return set_error(PVD_ERR_ARG, "pvd_dvh: need n >= 1 and bins >= 1");
  if (!dtypes_ok(dose_dtype, mask_dtype))
    return set_error(PVD_ERR_ARG, "pvd_dvh: dose must be PVD_DTYPE_F32/F64, mask PVD_DTYPE_U8/F32");
  cudaStream_t st = (cudaStream_t)stream;
  cudaError_t e = cudaMemsetAsync(result_d, 0xff, sizeof(long long), st);  // min key starts at all ones
  if (e == cudaSuccess) e = cudaMemsetAsync(result_d + 1, 0, sizeof(long long) * (size_t)(3 + bins), st);
  if (e != cudaSuccess) return set_error(PVD_ERR_CUDA, std::string("pvd_dvh: ") + cudaGetErrorString(e));
  unsigned long long* res = (unsigned long long*)result_d;
  if (dose_dtype == PVD_DTYPE_F32)
    (mask_dtype == PVD_DTYPE_U8) ? launch_dvh<float, unsigned char>(dose_d, mask_d, n, bins, edges_d, res, st)
                                 : launch_dvh<float, float>(dose_d, mask_d, n, bins, edges_d, res, st);
  else
    (mask_dtype == PVD_DTYPE_U8) ? launch_dvh<double, unsigned char>(dose_d, mask_d, n, bins, edges_d, res, st)
                                 : launch_dvh<double, float>(dose_d, mask_d, n, bins, edges_d, res, st);
  count_launch(2);
  PVD_LAUNCH_CHECK("k_histogram");
  return PVD_OK;
}
