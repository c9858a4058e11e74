// Kernel-argument structs shared by the convolution pass kernels.
#pragma once

#include "pvd_common.cuh"

namespace pvd {

// Activity input of the first pass: sum_t w[t] * p[t] (one map: n = 1, w = 1).
struct ActIn {
  const float* p[PVD_MAX_TIMEPOINTS];
  float w[PVD_MAX_TIMEPOINTS];
  int n;
};

// Spectrum storage modes.
enum SpecMode {
  SPEC_COMPLEX = 0,  // float2 [P0][P1][HS]
  SPEC_REAL_EVEN = 1 // float  [P0/2+1][P1/2+1][HS]: real and even along z and y
};

// Outputs of the z pass: one spectrum and one destination per kernel slot.
struct OutSet {
  float2* p[PVD_MAX_KERNELS];
  const void* s[PVD_MAX_KERNELS];
  int mode[PVD_MAX_KERNELS];
  int n;
  int P0, P0h, P1h;
};

// Spectrum value at (kz, ky, kx) for slot s.
__device__ __forceinline__ float2 spec_at(const OutSet& os, int s, int kz, int ky, int kx, int P1, int HS) {
  if (os.mode[s] == SPEC_REAL_EVEN) {
    const int kzq = min(kz, os.P0 - kz);
    const int kyq = min(ky, P1 - ky);
    const float v = __ldg((const float*)os.s[s] + ((long long)kzq * os.P1h + kyq) * HS + kx);
    return make_float2(v, 0.f);
  }
  return __ldg((const float2*)os.s[s] + ((long long)kz * P1 + ky) * HS + kx);
}

}  // namespace pvd
