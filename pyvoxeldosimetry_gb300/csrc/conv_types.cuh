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

// Column (y) pass inputs and outputs per kernel slot, blockIdx.z = slot.  A z slab
// of the input starts every in_slab complex elements, one of the output every
// out_slab; input and output may be the same buffer (the inverse pass runs in
// place: every CTA reads its whole tile before it writes any of it).
struct ColSet {
  const float2* in[PVD_MAX_KERNELS];
  float2* out[PVD_MAX_KERNELS];
  long long in_slab, out_slab;
};

// Inverse x pass over several kernel slots in one launch: slot s reads its
// half-spectrum rows from in[s] (row r = z * N1 + y stored at (z * pitch + y) * HS,
// i.e. in place in the slot's z-pass buffer) and writes dose rows to out[s].
constexpr int XINV_SLOTS = 4;  // slots per inverse-x launch
struct XInvSet {
  const float2* in[XINV_SLOTS];
  float* out[XINV_SLOTS];
  int n;
};

// a[i] for a runtime i, by compile-time indexing (keeps a kernel-parameter array in
// the parameter bank instead of copying it to local memory)
template <class T, int N>
__device__ __forceinline__ T pick(const T (&a)[N], int i) {
  T r = a[0];
#pragma unroll
  for (int k = 1; k < N; ++k)
    if (i == k) r = a[k];
  return r;
}

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
