// Dose-point kernels on the GPU in FP64: a sum of radial terms evaluated at
// every voxel of a (k0, k1, k2) grid centred on voxel (k0/2, k1/2, k2/2).
//
// The terms are the building blocks of the reference's generators
// (pyvoxeldosimetry/data/dose_kernels/*_kernel.py):
//   COLE    w (1 - r/R)^2 exp(-2 r/R), r <= R    beta / positron (y90_kernel.py:93-117,
//                                                  lu177_kernel.py:129-154, ga68_kernel.py:54-66)
//   PHOTON  w exp(-mu r/10) / (4 pi r^2)           photons, mu in 1/cm, r in mm
//                                                  (y90_kernel.py:119-140, ga68_kernel.py:68-83,
//                                                  lu177_kernel.py:156-184, ac225_kernel.py:168-184)
//   ALPHA   w (1 - (r/R)^p) exp(-c r/R), r <= R   alphas (ac225_kernel.py:140-166)
//   EXP_R2  w exp(-r/lambda) / r^2                 the analytic profile of the dose path
// At r = 0 a PHOTON / EXP_R2 term takes the radius of the sphere of the voxel's
// volume, 0, or NaN (the reference's 0 * inf) as its `center` field says.
// Each term's operations follow the reference's numpy expression left to right.
#include <algorithm>
#include <cmath>

#include "pvd_common.cuh"

namespace pvd {

struct TermSet {
  pvd_radial_term t[PVD_MAX_RADIAL_TERMS];
  int n;
  double scale, v0, v1, v2, r0;
  int k0, k1, k2;
};

__device__ __forceinline__ double term_value(const pvd_radial_term& t, double r, double r0) {
  const double pi4 = 4.0 * 3.14159265358979323846;
  switch (t.type) {
    case PVD_TERM_COLE: {
      if (!(r <= t.p1)) return 0.0;
      const double u = 1.0 - r / t.p1;
      return u * u * exp(-2.0 * r / t.p1) * t.weight;
    }
    case PVD_TERM_ALPHA: {
      if (!(r <= t.p1)) return 0.0;
      return (1.0 - pow(r / t.p1, t.p2)) * exp(-t.p3 * r / t.p1) * t.weight;
    }
    case PVD_TERM_PHOTON:
    case PVD_TERM_EXP_R2: {
      double rc = r;
      if (r == 0.0) {
        if (t.center == PVD_CENTER_ZERO) return 0.0;
        if (t.center == PVD_CENTER_NAN) return __longlong_as_double(0x7ff8000000000000ll);
        rc = r0;
      }
      if (t.type == PVD_TERM_PHOTON) return t.weight * exp(-t.p1 * rc / 10.0) / (pi4 * (rc * rc));
      return t.weight * exp(-rc / t.p1) / (rc * rc);
    }
    default:
      return 0.0;
  }
}

__global__ void k_radial_kernel(TermSet s, double* __restrict__ out) {
  const long long total = (long long)s.k0 * s.k1 * s.k2;
  for (long long o = blockIdx.x * (long long)blockDim.x + threadIdx.x; o < total;
       o += (long long)gridDim.x * blockDim.x) {
    const int i2 = (int)(o % s.k2);
    const long long q = o / s.k2;
    const int i1 = (int)(q % s.k1), i0 = (int)(q / s.k1);
    const double x = (double)(i0 - s.k0 / 2) * s.v0, y = (double)(i1 - s.k1 / 2) * s.v1,
                 z = (double)(i2 - s.k2 / 2) * s.v2;
    const double r = sqrt(x * x + y * y + z * z);
    double k = 0.0;
    for (int j = 0; j < s.n; ++j) k += term_value(s.t[j], r, s.r0);
    out[o] = k * s.scale;
  }
}

}  // namespace pvd

using namespace pvd;

extern "C" pvd_status pvd_radial_kernel(const pvd_radial_term* terms, int n_terms, double scale, int k0, int k1,
                                        int k2, const double* voxel_mm, double* out_d, pvd_stream stream) {
  if (!terms || !voxel_mm || !out_d) return set_error(PVD_ERR_ARG, "pvd_radial_kernel: null argument");
  if (n_terms < 1 || n_terms > PVD_MAX_RADIAL_TERMS)
    return set_error(PVD_ERR_ARG, "pvd_radial_kernel: n_terms must be in [1, PVD_MAX_RADIAL_TERMS]");
  if (k0 < 1 || k1 < 1 || k2 < 1) return set_error(PVD_ERR_ARG, "pvd_radial_kernel: grid dims must be >= 1");
  TermSet s;
  for (int j = 0; j < n_terms; ++j) {
    const pvd_radial_term& t = terms[j];
    if (t.type < PVD_TERM_COLE || t.type > PVD_TERM_EXP_R2)
      return set_error(PVD_ERR_ARG, "pvd_radial_kernel: unknown term type");
    if ((t.type == PVD_TERM_COLE || t.type == PVD_TERM_ALPHA || t.type == PVD_TERM_EXP_R2) && !(t.p1 > 0.0))
      return set_error(PVD_ERR_ARG, "pvd_radial_kernel: range / decay length must be > 0");
    s.t[j] = t;
  }
  for (int i = 0; i < 3; ++i)
    if (!(voxel_mm[i] > 0.0)) return set_error(PVD_ERR_ARG, "pvd_radial_kernel: voxel size must be > 0");
  s.n = n_terms;
  s.scale = scale;
  s.v0 = voxel_mm[0], s.v1 = voxel_mm[1], s.v2 = voxel_mm[2];
  s.r0 = std::cbrt(3.0 * s.v0 * s.v1 * s.v2 / (4.0 * 3.14159265358979323846));
  s.k0 = k0, s.k1 = k1, s.k2 = k2;
  const long long total = (long long)k0 * k1 * k2;
  const int threads = 256;
  const int blocks = (int)std::min<long long>((total + threads - 1) / threads, 152LL * 16);
  k_radial_kernel<<<blocks, threads, 0, (cudaStream_t)stream>>>(s, out_d);
  PVD_LAUNCH_CHECK("k_radial_kernel");
  return PVD_OK;
}
