// Time integration on the GPU: the weighted sum of timepoint maps (trapezoid)
// and, in tac_fit.cu, the per-voxel time-activity-curve fits.
//
// pvd_weighted_sum replaces ActivitySampler._trapezoid_integration
// (pyvoxeldosimetry/core/activity_sampler.py:69-78): out = sum_t w_t A_t with
// w_t the trapezoid weights of the timepoints.  One HBM-bound pass: T reads and
// one write of 4 bytes per voxel, float4-vectorised where the pointers allow.
#include <algorithm>

#include "pvd_common.cuh"

namespace pvd {

struct MapSet {
  const float* p[PVD_MAX_TIMEPOINTS];
  float w[PVD_MAX_TIMEPOINTS];
  int n;
};

__global__ void k_weighted_sum4(MapSet m, float4* __restrict__ out, long long n4) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n4; i += (long long)gridDim.x * blockDim.x) {
    float4 s = make_float4(0.f, 0.f, 0.f, 0.f);
    for (int t = 0; t < m.n; ++t) {
      const float4 v = __ldg(reinterpret_cast<const float4*>(m.p[t]) + i);
      const float w = m.w[t];
      s.x += w * v.x;
      s.y += w * v.y;
      s.z += w * v.z;
      s.w += w * v.w;
    }
    out[i] = s;
  }
}

__global__ void k_weighted_sum1(MapSet m, float* __restrict__ out, long long begin, long long n) {
  for (long long i = begin + blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    float s = 0.f;
    for (int t = 0; t < m.n; ++t) s += m.w[t] * __ldg(m.p[t] + i);
    out[i] = s;
  }
}

}  // namespace pvd

using namespace pvd;

extern "C" pvd_status pvd_weighted_sum(const float* const* maps, const float* weights, int n_maps, long long n_voxels,
                                       float* out, pvd_stream stream) {
  if (!maps || !weights || !out) return set_error(PVD_ERR_ARG, "pvd_weighted_sum: null argument");
  if (n_maps < 1 || n_maps > PVD_MAX_TIMEPOINTS) return set_error(PVD_ERR_ARG, "pvd_weighted_sum: n_maps must be in [1, 16]");
  if (n_voxels < 0) return set_error(PVD_ERR_ARG, "pvd_weighted_sum: negative size");
  if (n_voxels == 0) return PVD_OK;
  MapSet m;
  m.n = n_maps;
  bool aligned = (reinterpret_cast<uintptr_t>(out) % 16) == 0;
  for (int t = 0; t < n_maps; ++t) {
    if (!maps[t]) return set_error(PVD_ERR_ARG, "pvd_weighted_sum: null map pointer");
    m.p[t] = maps[t];
    m.w[t] = weights[t];
    aligned = aligned && (reinterpret_cast<uintptr_t>(maps[t]) % 16) == 0;
  }
  cudaStream_t st = (cudaStream_t)stream;
  long long done = 0;
  if (aligned && n_voxels >= 4) {
    const long long n4 = n_voxels / 4;
    const int blocks = (int)std::min<long long>((n4 + 255) / 256, 152LL * 16);
    k_weighted_sum4<<<blocks, 256, 0, st>>>(m, reinterpret_cast<float4*>(out), n4);
    PVD_LAUNCH_CHECK("k_weighted_sum4");
    done = n4 * 4;
  }
  if (done < n_voxels) {
    const long long rem = n_voxels - done;
    const int blocks = (int)std::min<long long>((rem + 255) / 256, 152LL * 16);
    k_weighted_sum1<<<blocks, 256, 0, st>>>(m, out, done, n_voxels);
    PVD_LAUNCH_CHECK("k_weighted_sum1");
  }
  return PVD_OK;
}
