// Volume resampling on the GPU: cubic B-spline (order 3) or trilinear (order 1)
// interpolation at an axis-aligned grid of sample points.
//
// Replaces the resampling the reference leaves to a stub on the convolution
// path (_resample_activity, core/kernel_convolution.py:108-114) and to
// nibabel's order-3 spline conform in resample_dose_map (core/utils.py:193-231).
// The spline is scipy.ndimage's: interpolating cubic B-spline with mirror
// boundaries (d c b | a b c d | c b a), i.e. map_coordinates(order=3,
// mode='mirror').
//
// k_prefilter: the coefficients.  The recursive cubic B-spline filter (Unser,
//   Aldroubi & Eden, IEEE Trans. Signal Process. 41, 1993) with the exact
//   mirror-boundary initial values equals the symmetric convolution
//   c[i] = sqrt(3) * sum_k z^|k| x~[i - k] over the mirror-extended line x~,
//   z = sqrt(3) - 2.  |z|^17 / (1 - |z|) < 1e-9, so the sum is cut at
//   |k| <= 16: a separable 33-tap filter, one pass per axis, every output
//   independent (staged in shared-memory tiles, coalesced along x) instead of
//   a sequential recursion per line.  Within 5e-10 of the recursion in exact arithmetic.
//   Three passes src -> coef -> scratch -> coef.
// k_resample: one thread per output voxel; u_a = j_a * step_a + origin_a in
//   input voxel units; 4 (order 3) or 2 (order 1) taps per axis at mirrored
//   indices; result times value_scale.  Output writes coalesced along x;
//   tap reads are gathers served mostly from L1/L2.
#include <algorithm>
#include <cmath>

#include "pvd_common.cuh"

namespace pvd {

constexpr int kResampleThreads = 256;

__device__ __forceinline__ int mirror_index(int k, int n) {
  if (n == 1) return 0;
  const int period = 2 * n - 2;
  k = k < 0 ? -k : k;
  k %= period;
  return k >= n ? period - k : k;
}

constexpr int kFirHalf = 16;
// sqrt(3) z^k for k = 0..16, z = sqrt(3) - 2, rounded to float
__device__ constexpr float c_fir[kFirHalf + 1] = {
    1.7320507764816284f,     -0.4641016125679016f,    0.12435565143823624f,    -0.03332099691033363f,
    0.008928334340453148f,   -0.002392339985817671f,  0.0006410255446098745f,  -0.0001717622799333185f,
    4.6023564209463075e-05f, -1.2331976904533803e-05f, 3.3043431812984636e-06f, -8.853961048771453e-07f,
    2.3724116715584387e-07f, -6.356857795708493e-08f, 1.7033150001566355e-08f, -4.564018496466815e-09f,
    1.22292509452393e-09f};

// out = 33-tap B-spline prefilter of src along AXIS (0 slowest, 2 contiguous).
// Shared-memory tiles: a block stages kPfT outputs plus a kFirHalf-sample
// mirrored halo on each side along the axis, 32 wide across it, so every input
// crosses L2 (kPfT + 32) / kPfT times instead of 33.
//   AXIS 0/1: tile[axis position][32 consecutive x]; blockIdx = (x tile, axis
//             tile, index of the remaining axis); 8 warps, each warp one axis row.
//   AXIS 2:   tile[8 rows][segment of kPfT2 + 32 along x]; blockIdx = (x
//             segment, row group).
constexpr int kPfT = 64, kPfT2 = 128, kPfRows = 8;

template <int AXIS>
__global__ void __launch_bounds__(256) k_prefilter(const float* __restrict__ src, float* __restrict__ out, int n0,
                                                   int n1, int n2) {
  const int tx = threadIdx.x, ty = threadIdx.y;
  if constexpr (AXIS == 2) {
    __shared__ __align__(16) float tile[kPfRows][kPfT2 + 2 * kFirHalf];  // rows of 160 floats: 16-byte aligned
    const long long rows = (long long)n0 * n1;
    const int x0 = blockIdx.x * kPfT2;
    const long long row = (long long)blockIdx.y * kPfRows + ty;
    const bool row_ok = row < rows;
    const float* in = src + (row_ok ? row : 0) * n2;
    for (int c = tx; c < kPfT2 + 2 * kFirHalf; c += 32)
      tile[ty][c] = row_ok ? __ldg(in + mirror_index(x0 - kFirHalf + c, n2)) : 0.0f;
    __syncthreads();
    if (!row_ok) return;
    // 4 consecutive outputs per thread from one 36-sample window (nine 16-byte reads)
    constexpr int OX = kPfT2 / 32;  // 4
    float win[OX + 2 * kFirHalf];
#pragma unroll
    for (int q = 0; q < (OX + 2 * kFirHalf) / 4; ++q) {
      const float4 v = *reinterpret_cast<const float4*>(&tile[ty][tx * OX + 4 * q]);
      win[4 * q] = v.x, win[4 * q + 1] = v.y, win[4 * q + 2] = v.z, win[4 * q + 3] = v.w;
    }
#pragma unroll
    for (int o = 0; o < OX; ++o) {
      const int x = x0 + tx * OX + o;
      if (x >= n2) break;
      float acc = c_fir[0] * win[o + kFirHalf];
#pragma unroll
      for (int k = 1; k <= kFirHalf; ++k) acc += c_fir[k] * (win[o + kFirHalf - k] + win[o + kFirHalf + k]);
      out[row * n2 + x] = acc;
    }
  } else {
    __shared__ float tile[kPfT + 2 * kFirHalf][33];
    const int n = AXIS == 0 ? n0 : n1;
    const long long stride = AXIS == 0 ? (long long)n1 * n2 : (long long)n2;
    const int x = blockIdx.x * 32 + tx;
    const int a0 = blockIdx.y * kPfT;
    const int other = blockIdx.z;  // i1 for AXIS 0, i0 for AXIS 1
    const long long base = (AXIS == 0 ? (long long)other * n2 : (long long)other * n1 * n2) + x;
    const bool x_ok = x < n2;
    for (int r = ty; r < kPfT + 2 * kFirHalf; r += blockDim.y)
      tile[r][tx] = x_ok ? __ldg(src + base + (long long)mirror_index(a0 - kFirHalf + r, n) * stride) : 0.0f;
    __syncthreads();
    if (!x_ok) return;
    // 8 consecutive outputs per thread from one 40-sample window of its column
    constexpr int OY = kPfT / kPfRows;  // 8
    float win[OY + 2 * kFirHalf];
#pragma unroll
    for (int k = 0; k < OY + 2 * kFirHalf; ++k) win[k] = tile[ty * OY + k][tx];
#pragma unroll
    for (int o = 0; o < OY; ++o) {
      const int i = a0 + ty * OY + o;
      if (i >= n) break;
      float acc = c_fir[0] * win[o + kFirHalf];
#pragma unroll
      for (int k = 1; k <= kFirHalf; ++k) acc += c_fir[k] * (win[o + kFirHalf - k] + win[o + kFirHalf + k]);
      out[base + (long long)i * stride] = acc;
    }
  }
}

struct ResampleArgs {
  int n[3], m[3];
  double step[3], origin[3];
  float value_scale;
};

template <int ORDER>
__device__ __forceinline__ void taps_of(double u, int n, int* idx, float* w) {
  const double fl = floor(u);
  const float t = (float)(u - fl);
  const int b = (int)fl;
  if (ORDER == 3) {
    const float t2 = t * t, t3 = t2 * t, s = 1.0f - t;
    w[0] = s * s * s * (1.0f / 6.0f);
    w[1] = (4.0f - 6.0f * t2 + 3.0f * t3) * (1.0f / 6.0f);
    w[2] = (1.0f + 3.0f * t + 3.0f * t2 - 3.0f * t3) * (1.0f / 6.0f);
    w[3] = t3 * (1.0f / 6.0f);
    if (b >= 1 && b + 2 < n) {
#pragma unroll
      for (int k = 0; k < 4; ++k) idx[k] = b - 1 + k;
    } else {
#pragma unroll
      for (int k = 0; k < 4; ++k) idx[k] = mirror_index(b - 1 + k, n);
    }
  } else {
    w[0] = 1.0f - t;
    w[1] = t;
    idx[0] = mirror_index(b, n);
    idx[1] = mirror_index(b + 1, n);
  }
}

// One output row (j0, j1) per block iteration; the axis-0/1 taps and weights are
// the same for the whole row, threads run along j2.
template <int ORDER>
__global__ void __launch_bounds__(kResampleThreads) k_resample(const float* __restrict__ src, float* __restrict__ out,
                                                               ResampleArgs a) {
  constexpr int TAPS = ORDER == 3 ? 4 : 2;
  const long long rows = (long long)a.m[0] * a.m[1];
  for (long long row = blockIdx.x; row < rows; row += gridDim.x) {
    const int j0 = (int)(row / a.m[1]), j1 = (int)(row % a.m[1]);
    int id0[TAPS], id1[TAPS];
    float w0[TAPS], w1[TAPS];
    taps_of<ORDER>(j0 * a.step[0] + a.origin[0], a.n[0], id0, w0);
    taps_of<ORDER>(j1 * a.step[1] + a.origin[1], a.n[1], id1, w1);
    for (int j2 = threadIdx.x; j2 < a.m[2]; j2 += blockDim.x) {
      int id2[TAPS];
      float w2[TAPS];
      taps_of<ORDER>(j2 * a.step[2] + a.origin[2], a.n[2], id2, w2);
      float acc = 0.0f;
#pragma unroll
      for (int i0 = 0; i0 < TAPS; ++i0) {
        const long long b0 = (long long)id0[i0] * a.n[1];
        float acc1 = 0.0f;
#pragma unroll
        for (int i1 = 0; i1 < TAPS; ++i1) {
          const float* r = src + (b0 + id1[i1]) * a.n[2];
          float acc2 = 0.0f;
#pragma unroll
          for (int i2 = 0; i2 < TAPS; ++i2) acc2 += w2[i2] * __ldg(r + id2[i2]);
          acc1 += w1[i1] * acc2;
        }
        acc += w0[i0] * acc1;
      }
      out[row * a.m[2] + j2] = acc * a.value_scale;
    }
  }
}

// Taps of one output coordinate: 4 input indices (mirrored) and weights; order 1
// fills two and leaves zero weights on a repeated valid index.
struct Tap4 {
  int idx[4];
  float w[4];
};

// tab[j] = the taps of u = j * step + origin (FP64 once per coordinate, not per voxel)
template <int ORDER>
__global__ void k_taps(Tap4* __restrict__ tab, int m, int n, double step, double origin) {
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < m; j += gridDim.x * blockDim.x) {
    Tap4 t;
    if (ORDER == 3) {
      taps_of<3>(j * step + origin, n, t.idx, t.w);
    } else {
      taps_of<1>(j * step + origin, n, t.idx, t.w);
      t.idx[2] = t.idx[3] = t.idx[1];
      t.w[2] = t.w[3] = 0.0f;
    }
    tab[j] = t;
  }
}

// One 1-D evaluation along AXIS of a volume whose output shape is (s0, s1, s2) and
// whose input has length n along AXIS (the other two axes as in the output):
// out = scale * sum_k w_k in[idx_k] with the taps of the output coordinate from
// tab.  The cubic B-spline of a volume is the tensor product of its axes'
// splines, so three such passes over the coefficients (x, then y, then z) give
// the 3-D interpolant with 4 taps per output and pass instead of 64 per output.
// Blocks take output rows (j0, j1); along y and z the taps are the row's.
template <int AXIS>
__global__ void __launch_bounds__(kResampleThreads) k_eval_axis(const float* __restrict__ in, float* __restrict__ out,
                                                                int s0, int s1, int s2, int n,
                                                                const Tap4* __restrict__ tab, float scale) {
  const long long rows = (long long)s0 * s1;
  for (long long row = blockIdx.x; row < rows; row += gridDim.x) {
    const int j0 = (int)(row / s1), j1 = (int)(row % s1);
    float* orow = out + row * s2;
    if constexpr (AXIS == 2) {
      const float* irow = in + row * n;
      for (int j2 = threadIdx.x; j2 < s2; j2 += blockDim.x) {
        const Tap4 t = tab[j2];
        float acc = 0.0f;
#pragma unroll
        for (int k = 0; k < 4; ++k) acc += t.w[k] * __ldg(irow + t.idx[k]);
        orow[j2] = acc * scale;
      }
    } else {
      const Tap4 t = tab[AXIS == 1 ? j1 : j0];
      const float* base[4];
#pragma unroll
      for (int k = 0; k < 4; ++k)
        base[k] = AXIS == 1 ? in + ((long long)j0 * n + t.idx[k]) * s2 : in + ((long long)t.idx[k] * s1 + j1) * s2;
      for (int j2 = threadIdx.x; j2 < s2; j2 += blockDim.x) {
        float acc = 0.0f;
#pragma unroll
        for (int k = 0; k < 4; ++k) acc += t.w[k] * __ldg(base[k] + j2);
        orow[j2] = acc * scale;
      }
    }
  }
}

// blocks over rows, threads along x: the row length rounded up to whole warps, at most 256
static int rows_grid(long long rows) { return (int)std::max<long long>(1, std::min<long long>(rows, 152LL * 16)); }
static int row_threads(int len) { return std::min(kResampleThreads, std::max(32, (len + 31) / 32 * 32)); }

}  // namespace pvd

using namespace pvd;

extern "C" pvd_status pvd_bspline_prefilter(const float* src_d, float* coef_d, float* scratch_d, int n0, int n1,
                                            int n2, pvd_stream stream) {
  if (!src_d || !coef_d || !scratch_d) return set_error(PVD_ERR_ARG, "pvd_bspline_prefilter: null argument");
  if (n0 < 1 || n1 < 1 || n2 < 1) return set_error(PVD_ERR_ARG, "pvd_bspline_prefilter: dims must be >= 1");
  if (coef_d == src_d || scratch_d == src_d || scratch_d == coef_d)
    return set_error(PVD_ERR_ARG, "pvd_bspline_prefilter: src, coef and scratch must be distinct buffers");
  cudaStream_t st = (cudaStream_t)stream;
  if (n0 > 65535 || n1 > 65535 || ((long long)n0 * n1 + kPfRows - 1) / kPfRows > 65535)
    return set_error(PVD_ERR_UNSUPPORTED, "pvd_bspline_prefilter: volume too large for the tiled grid");
  const dim3 blk(32, kPfRows);
  const int xt = (n2 + 31) / 32;
  k_prefilter<0><<<dim3(xt, (n0 + kPfT - 1) / kPfT, n1), blk, 0, st>>>(src_d, coef_d, n0, n1, n2);
  PVD_LAUNCH_CHECK("k_prefilter<0>");
  k_prefilter<1><<<dim3(xt, (n1 + kPfT - 1) / kPfT, n0), blk, 0, st>>>(coef_d, scratch_d, n0, n1, n2);
  PVD_LAUNCH_CHECK("k_prefilter<1>");
  k_prefilter<2><<<dim3((n2 + kPfT2 - 1) / kPfT2, (int)(((long long)n0 * n1 + kPfRows - 1) / kPfRows)), blk, 0, st>>>(
      scratch_d, coef_d, n0, n1, n2);
  PVD_LAUNCH_CHECK("k_prefilter<2>");
  return PVD_OK;
}

extern "C" pvd_status pvd_resample(const float* src_d, int n0, int n1, int n2, float* out_d, int m0, int m1, int m2,
                                   const double* step, const double* origin, int order, float value_scale,
                                   pvd_stream stream) {
  if (!src_d || !out_d || !step || !origin) return set_error(PVD_ERR_ARG, "pvd_resample: null argument");
  if (n0 < 1 || n1 < 1 || n2 < 1 || m0 < 0 || m1 < 0 || m2 < 0)
    return set_error(PVD_ERR_ARG, "pvd_resample: bad dims");
  if (order != 1 && order != 3) return set_error(PVD_ERR_ARG, "pvd_resample: order must be 1 or 3");
  ResampleArgs a;
  a.n[0] = n0, a.n[1] = n1, a.n[2] = n2;
  a.m[0] = m0, a.m[1] = m1, a.m[2] = m2;
  for (int i = 0; i < 3; ++i) {
    if (!std::isfinite(step[i]) || !std::isfinite(origin[i]))
      return set_error(PVD_ERR_ARG, "pvd_resample: step and origin must be finite");
    // every sample coordinate must fit an int after flooring
    const double far = std::fabs(origin[i]) + std::fabs(step[i]) * (double)std::max(1, a.m[i]);
    if (far > 1e9) return set_error(PVD_ERR_ARG, "pvd_resample: sample coordinates out of range");
    a.step[i] = step[i];
    a.origin[i] = origin[i];
  }
  a.value_scale = value_scale;
  const long long total = (long long)m0 * m1 * m2;
  if (total == 0) return PVD_OK;
  cudaStream_t st = (cudaStream_t)stream;
  const int grid = rows_grid((long long)m0 * m1), threads = row_threads(m2);
  if (order == 3)
    k_resample<3><<<grid, threads, 0, st>>>(src_d, out_d, a);
  else
    k_resample<1><<<grid, threads, 0, st>>>(src_d, out_d, a);
  PVD_LAUNCH_CHECK("k_resample");
  return PVD_OK;
}

extern "C" pvd_status pvd_resample_separable(const float* src_d, int n0, int n1, int n2, float* out_d, int m0, int m1,
                                             int m2, const double* step, const double* origin, int order,
                                             float value_scale, float* scratch_d, long long scratch_elems,
                                             pvd_stream stream) {
  if (!src_d || !out_d || !step || !origin || !scratch_d)
    return set_error(PVD_ERR_ARG, "pvd_resample_separable: null argument");
  if (n0 < 1 || n1 < 1 || n2 < 1 || m0 < 0 || m1 < 0 || m2 < 0)
    return set_error(PVD_ERR_ARG, "pvd_resample_separable: bad dims");
  if (order != 1 && order != 3) return set_error(PVD_ERR_ARG, "pvd_resample_separable: order must be 1 or 3");
  for (int i = 0; i < 3; ++i) {
    if (!std::isfinite(step[i]) || !std::isfinite(origin[i]))
      return set_error(PVD_ERR_ARG, "pvd_resample_separable: step and origin must be finite");
    const int m = i == 0 ? m0 : (i == 1 ? m1 : m2);
    if (std::fabs(origin[i]) + std::fabs(step[i]) * (double)std::max(1, m) > 1e9)
      return set_error(PVD_ERR_ARG, "pvd_resample_separable: sample coordinates out of range");
  }
  const long long a_elems = (long long)n0 * n1 * m2, b_elems = (long long)n0 * m1 * m2;
  const long long tab_elems = 8LL * ((long long)m0 + m1 + m2);  // Tap4 = 8 four-byte words
  if (scratch_elems < a_elems + b_elems + tab_elems)
    return set_error(PVD_ERR_ARG, "pvd_resample_separable: scratch needs n0*n1*m2 + n0*m1*m2 + 8*(m0+m1+m2) floats");
  if ((long long)m0 * m1 * m2 == 0) return PVD_OK;
  cudaStream_t st = (cudaStream_t)stream;
  float* ta = scratch_d;            // (n0, n1, m2)
  float* tb = scratch_d + a_elems;  // (n0, m1, m2)
  Tap4* tab = reinterpret_cast<Tap4*>(scratch_d + a_elems + b_elems);
  Tap4* tab_ax[3] = {tab, tab + m0, tab + m0 + m1};
  const int m[3] = {m0, m1, m2}, n[3] = {n0, n1, n2};
  for (int ax = 0; ax < 3; ++ax) {
    const int blocks = (m[ax] + 255) / 256;
    if (order == 3)
      k_taps<3><<<blocks, 256, 0, st>>>(tab_ax[ax], m[ax], n[ax], step[ax], origin[ax]);
    else
      k_taps<1><<<blocks, 256, 0, st>>>(tab_ax[ax], m[ax], n[ax], step[ax], origin[ax]);
    PVD_LAUNCH_CHECK("k_taps");
  }
  const int thr = row_threads(m2);
  k_eval_axis<2><<<rows_grid((long long)n0 * n1), thr, 0, st>>>(src_d, ta, n0, n1, m2, n2, tab_ax[2], 1.0f);
  PVD_LAUNCH_CHECK("k_eval_axis<2>");
  k_eval_axis<1><<<rows_grid((long long)n0 * m1), thr, 0, st>>>(ta, tb, n0, m1, m2, n1, tab_ax[1], 1.0f);
  PVD_LAUNCH_CHECK("k_eval_axis<1>");
  k_eval_axis<0><<<rows_grid((long long)m0 * m1), thr, 0, st>>>(tb, out_d, m0, m1, m2, n0, tab_ax[0], value_scale);
  PVD_LAUNCH_CHECK("k_eval_axis<0>");
  return PVD_OK;
}
