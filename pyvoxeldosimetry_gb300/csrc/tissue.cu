// CT Hounsfield units -> tissue masks and mass density, one pass over the volume.
//
// Replaces TissueComposition.calculate_composition with its artefact handling
// (pyvoxeldosimetry/tissue/composition.py:48-93):
//   * metal (HU > 2000) is replaced by the Gaussian-smoothed image (sigma 1 voxel,
//     scipy.ndimage.gaussian_filter: radius 4, weights exp(-k^2/2) normalised over
//     k in [-4, 4], 'reflect' boundary) of the image whose metal voxels (and NaNs)
//     are 0;
//   * masks: HU in the closed ranges air [-1000, -900], lung [-900, -500], soft
//     tissue [-100, 100], bone [300, 3000], water [-10, 10] (ranges overlap and
//     leave gaps exactly as the reference's do; NaN is in none).
// The mass density map that the density-scaled convolution divides by is not in
// the reference (its tissue_densities hook is unused, core/dose_calculator.py:90):
// a piecewise-linear calibration through caller-given (HU, g/cc) anchors, clamped
// at the ends, NaN -> 0 (dose 0 there).
//
// Memory-bound: 4 voxels per thread per iteration (float4 in, uchar4 masks and
// float4 density out); a metal voxel takes the 9^3-tap smoothing sum in FP64 on
// its own (metal voxels are rare).
#include <cuda_runtime.h>

#include <cmath>
#include <string>

#include "pvd_common.cuh"

namespace pvd {
namespace {

constexpr int MAX_ANCHORS = 16;
constexpr float METAL_HU = 2000.0f;

struct Calib {
  float hu[MAX_ANCHORS];
  float rho[MAX_ANCHORS];
  int n;
};

// Gaussian weights of scipy.ndimage.gaussian_filter(sigma = 1): exp(-k^2 / 2) / sum
__constant__ double c_gw[9];

__device__ __forceinline__ int reflect(int i, int n) {
  // scipy 'reflect' (d c b a | a b c d | d c b a); the radius (4) may exceed n
  while (i < 0 || i >= n) i = (i < 0) ? -i - 1 : 2 * n - i - 1;
  return i;
}

// smoothed value of the metal-free image at (z, y, x)
__device__ double smoothed(const float* __restrict__ ct, int n0, int n1, int n2, int z, int y, int x) {
  double acc = 0.0;
  for (int dz = -4; dz <= 4; ++dz) {
    const long long oz = (long long)reflect(z + dz, n0) * n1;
    double az = 0.0;
    for (int dy = -4; dy <= 4; ++dy) {
      const long long oy = (oz + reflect(y + dy, n1)) * n2;
      double ay = 0.0;
      for (int dx = -4; dx <= 4; ++dx) {
        const float v = __ldg(ct + oy + reflect(x + dx, n2));
        // metal and NaN are 0 in the image that is smoothed; +-inf become +-DBL_MAX
        double d = (v > METAL_HU || v != v) ? 0.0 : (double)v;
        if (isinf(d)) d = d > 0 ? 1.7976931348623157e308 : -1.7976931348623157e308;
        ay += c_gw[dx + 4] * d;
      }
      az += c_gw[dy + 4] * ay;
    }
    acc += c_gw[dz + 4] * az;
  }
  return acc;
}

__device__ __forceinline__ float density_of(float hu, const Calib& c) {
  if (hu != hu) return 0.f;
  if (hu <= c.hu[0]) return c.rho[0];
  for (int i = 1; i < c.n; ++i)
    if (hu <= c.hu[i]) {
      const float t = (hu - c.hu[i - 1]) / (c.hu[i] - c.hu[i - 1]);
      return c.rho[i - 1] + t * (c.rho[i] - c.rho[i - 1]);
    }
  return c.rho[c.n - 1];
}

__device__ __forceinline__ unsigned char in_range(float v, float lo, float hi) { return (v >= lo && v <= hi) ? 1 : 0; }

__global__ void k_hu_composition(const float* __restrict__ ct, long long n, int n0, int n1, int n2, int artifacts,
                                 unsigned char* __restrict__ masks, float* __restrict__ rho, float* __restrict__ hu_out,
                                 Calib cal) {
  const long long n4 = n / 4;
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < (n + 3) / 4; q += stride) {
    float v[4];
    const long long i0 = 4 * q;
    if (q < n4) {
      const float4 f = __ldg(reinterpret_cast<const float4*>(ct) + q);
      v[0] = f.x, v[1] = f.y, v[2] = f.z, v[3] = f.w;
    } else {
      for (int k = 0; k < 4; ++k) v[k] = (i0 + k < n) ? __ldg(ct + i0 + k) : 0.f;
    }
    if (artifacts) {
      for (int k = 0; k < 4; ++k)
        if (v[k] > METAL_HU && i0 + k < n) {
          const long long i = i0 + k;
          const int x = (int)(i % n2), y = (int)((i / n2) % n1), z = (int)(i / ((long long)n1 * n2));
          v[k] = (float)smoothed(ct, n0, n1, n2, z, y, x);
        }
    }
    unsigned char m[5][4];
    float d[4];
    for (int k = 0; k < 4; ++k) {
      m[0][k] = in_range(v[k], -1000.f, -900.f);  // air
      m[1][k] = in_range(v[k], -900.f, -500.f);   // lung
      m[2][k] = in_range(v[k], -100.f, 100.f);    // soft tissue
      m[3][k] = in_range(v[k], 300.f, 3000.f);    // bone
      m[4][k] = in_range(v[k], -10.f, 10.f);      // water
      d[k] = density_of(v[k], cal);
    }
    if (q < n4) {
      if (masks) {
        if ((n & 3) == 0) {  // every plane starts on a 4-byte boundary
          for (int t = 0; t < 5; ++t)
            reinterpret_cast<uchar4*>(masks + t * n)[q] = make_uchar4(m[t][0], m[t][1], m[t][2], m[t][3]);
        } else {
          for (int t = 0; t < 5; ++t)
            for (int k = 0; k < 4; ++k) masks[t * n + i0 + k] = m[t][k];
        }
      }
      if (rho) reinterpret_cast<float4*>(rho)[q] = make_float4(d[0], d[1], d[2], d[3]);
      if (hu_out) reinterpret_cast<float4*>(hu_out)[q] = make_float4(v[0], v[1], v[2], v[3]);
    } else {
      for (int k = 0; k < 4 && i0 + k < n; ++k) {
        if (masks)
          for (int t = 0; t < 5; ++t) masks[t * n + i0 + k] = m[t][k];
        if (rho) rho[i0 + k] = d[k];
        if (hu_out) hu_out[i0 + k] = v[k];
      }
    }
  }
}

}  // namespace
}  // namespace pvd

using namespace pvd;

extern "C" pvd_status pvd_hu_composition(const float* ct_d, int n0, int n1, int n2, int flags,
                                         const float* anchor_hu, const float* anchor_rho, int n_anchor,
                                         unsigned char* masks_d, float* density_d, float* hu_d, pvd_stream stream) {
  if (!ct_d) return set_error(PVD_ERR_ARG, "pvd_hu_composition: null CT");
  if (n0 < 1 || n1 < 1 || n2 < 1) return set_error(PVD_ERR_ARG, "pvd_hu_composition: dims must be >= 1");
  if (flags & ~PVD_HU_ARTIFACTS) return set_error(PVD_ERR_ARG, "pvd_hu_composition: unknown flags");
  const long long n = (long long)n0 * n1 * n2;
  for (const void* p : {(const void*)ct_d, (const void*)masks_d, (const void*)density_d, (const void*)hu_d})
    if (((uintptr_t)p) % 16) return set_error(PVD_ERR_ARG, "pvd_hu_composition: buffers must be 16-byte aligned");
  Calib cal{};
  if (density_d) {
    if (!anchor_hu || !anchor_rho || n_anchor < 1 || n_anchor > MAX_ANCHORS)
      return set_error(PVD_ERR_ARG, "pvd_hu_composition: density needs 1..16 calibration anchors");
    for (int i = 0; i < n_anchor; ++i) {
      if (!std::isfinite(anchor_hu[i]) || !std::isfinite(anchor_rho[i]) || anchor_rho[i] < 0.f)
        return set_error(PVD_ERR_NUMERIC, "pvd_hu_composition: calibration anchors must be finite, density >= 0");
      if (i && !(anchor_hu[i] > anchor_hu[i - 1]))
        return set_error(PVD_ERR_ARG, "pvd_hu_composition: calibration HU must increase");
      cal.hu[i] = anchor_hu[i];
      cal.rho[i] = anchor_rho[i];
    }
    cal.n = n_anchor;
  }
  static const double* gw = [] {
    static double w[9];
    double s = 0.0;
    for (int k = -4; k <= 4; ++k) s += w[k + 4] = std::exp(-0.5 * k * k);
    for (double& x : w) x /= s;
    return w;
  }();
  PVD_CUDA_TRY(cudaMemcpyToSymbolAsync(c_gw, gw, sizeof(double) * 9, 0, cudaMemcpyHostToDevice,
                                       (cudaStream_t)stream));
  int dev = 0, sms = 0;
  PVD_CUDA_TRY(cudaGetDevice(&dev));
  PVD_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  const long long quads = (n + 3) / 4;
  const int grid = (int)std::min<long long>((quads + 255) / 256, (long long)sms * 8);
  k_hu_composition<<<grid, 256, 0, (cudaStream_t)stream>>>(ct_d, n, n0, n1, n2, flags & PVD_HU_ARTIFACTS, masks_d,
                                                          density_d, hu_d, cal);
  PVD_LAUNCH_CHECK("k_hu_composition");
  return PVD_OK;
}
