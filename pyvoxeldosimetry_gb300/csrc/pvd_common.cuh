// Shared helpers of the sm_103a dose kernels: status/error plumbing, complex
// arithmetic and the small fixed-radix DFTs used by the shared-memory FFTs.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <string>

#include "../../include/pvd.h"

namespace pvd {

// ---------------------------------------------------------------------------
// error plumbing (thread-local last error, never aborts)
// ---------------------------------------------------------------------------
pvd_status set_error(pvd_status st, const std::string& msg);
pvd_status cuda_error(cudaError_t e, const char* what);
void count_launch(int n = 1);

// Failure-path checks behind pvd_wait_check: one small kernel that waits, through the
// bounded wait of the plan's TMA passes or of the U-Net's tensor-core pipeline, on an
// mbarrier phase that nothing completes, and records the timeout where those do.
pvd_status plan_wait_check(pvd_plan* p, unsigned long long limit_ns, cudaStream_t st);
pvd_status unet_wait_check(unsigned long long limit_ns, cudaStream_t st);

#define PVD_CUDA_TRY(expr)                                        \
  do {                                                            \
    cudaError_t _e = (expr);                                      \
    if (_e != cudaSuccess) return ::pvd::cuda_error(_e, #expr);   \
  } while (0)

// Check a kernel launch that just happened.
#define PVD_LAUNCH_CHECK(name)                                    \
  do {                                                            \
    ::pvd::count_launch();                                        \
    cudaError_t _e = cudaGetLastError();                          \
    if (_e != cudaSuccess) return ::pvd::cuda_error(_e, name);    \
  } while (0)

// ---------------------------------------------------------------------------
// complex helpers (float2 = re, im)
// ---------------------------------------------------------------------------
__host__ __device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__host__ __device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__host__ __device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__host__ __device__ __forceinline__ float2 cscale(float2 a, float s) { return make_float2(a.x * s, a.y * s); }
// multiply by -i (forward) or +i (inverse)
template <bool INV>
__host__ __device__ __forceinline__ float2 mul_mi(float2 a) {
  return INV ? make_float2(-a.y, a.x) : make_float2(a.y, -a.x);
}

// ---------------------------------------------------------------------------
// fixed-radix DFTs in registers.  Forward: X[p] = sum_q v[q] exp(-2 pi i p q / R);
// INV uses the conjugate roots.  Constants are cos/sin of 2 pi k / R.
// ---------------------------------------------------------------------------
template <int R, bool INV> struct Dft;

template <bool INV> struct Dft<2, INV> {
  static __device__ __forceinline__ void run(float2* v) {
    float2 a = v[0], b = v[1];
    v[0] = cadd(a, b);
    v[1] = csub(a, b);
  }
};

template <bool INV> struct Dft<3, INV> {
  static __device__ __forceinline__ void run(float2* v) {
    const float s3 = 0.86602540378443865f;  // sin(2 pi / 3)
    float2 t1 = cadd(v[1], v[2]);
    float2 t2 = make_float2(v[0].x - 0.5f * t1.x, v[0].y - 0.5f * t1.y);
    float2 d = cscale(csub(v[1], v[2]), s3);
    float2 md = mul_mi<INV>(d);
    v[0] = cadd(v[0], t1);
    v[1] = cadd(t2, md);
    v[2] = csub(t2, md);
  }
};

template <bool INV> struct Dft<4, INV> {
  static __device__ __forceinline__ void run(float2* v) {
    float2 s02 = cadd(v[0], v[2]), d02 = csub(v[0], v[2]);
    float2 s13 = cadd(v[1], v[3]), d13 = mul_mi<INV>(csub(v[1], v[3]));
    v[0] = cadd(s02, s13);
    v[2] = csub(s02, s13);
    v[1] = cadd(d02, d13);
    v[3] = csub(d02, d13);
  }
};

template <bool INV> struct Dft<5, INV> {
  static __device__ __forceinline__ void run(float2* v) {
    const float c1 = 0.30901699437494742f;   // cos(2 pi/5)
    const float c2 = -0.80901699437494742f;  // cos(4 pi/5)
    const float s1 = 0.95105651629515357f;   // sin(2 pi/5)
    const float s2 = 0.58778525229247313f;   // sin(4 pi/5)
    float2 a1 = cadd(v[1], v[4]), b1 = csub(v[1], v[4]);
    float2 a2 = cadd(v[2], v[3]), b2 = csub(v[2], v[3]);
    float2 x0 = v[0];
    float2 r1 = make_float2(x0.x + c1 * a1.x + c2 * a2.x, x0.y + c1 * a1.y + c2 * a2.y);
    float2 r2 = make_float2(x0.x + c2 * a1.x + c1 * a2.x, x0.y + c2 * a1.y + c1 * a2.y);
    float2 i1 = mul_mi<INV>(make_float2(s1 * b1.x + s2 * b2.x, s1 * b1.y + s2 * b2.y));
    float2 i2 = mul_mi<INV>(make_float2(s2 * b1.x - s1 * b2.x, s2 * b1.y - s1 * b2.y));
    v[0] = make_float2(x0.x + a1.x + a2.x, x0.y + a1.y + a2.y);
    v[1] = cadd(r1, i1);
    v[4] = csub(r1, i1);
    v[2] = cadd(r2, i2);
    v[3] = csub(r2, i2);
  }
};

template <bool INV> struct Dft<7, INV> {
  static __device__ __forceinline__ void run(float2* v) {
    const float C1 = 0.62348980185873353f, C2 = -0.22252093395631440f, C3 = -0.90096886790241913f;
    const float S1 = 0.78183148246802981f, S2 = 0.97492791218182361f, S3 = 0.43388373911755812f;
    float2 a1 = cadd(v[1], v[6]), b1 = csub(v[1], v[6]);
    float2 a2 = cadd(v[2], v[5]), b2 = csub(v[2], v[5]);
    float2 a3 = cadd(v[3], v[4]), b3 = csub(v[3], v[4]);
    float2 x0 = v[0];
    // k = 1: cos(2pi jk/7) -> C1,C2,C3 ; sin -> S1,S2,S3
    // k = 2: C2,C3(=cos 12pi/7 = C1?) -- use explicit (jk mod 7) tables:
    //   jk mod 7 for k=2: 2,4,6 -> cos: C2, C3, C1 ; sin: S2, -S3, -S1
    //   k=3: 3,6,2 -> cos: C3, C1, C2 ; sin: S3, -S1, S2
    float2 r1 = make_float2(x0.x + C1 * a1.x + C2 * a2.x + C3 * a3.x, x0.y + C1 * a1.y + C2 * a2.y + C3 * a3.y);
    float2 r2 = make_float2(x0.x + C2 * a1.x + C3 * a2.x + C1 * a3.x, x0.y + C2 * a1.y + C3 * a2.y + C1 * a3.y);
    float2 r3 = make_float2(x0.x + C3 * a1.x + C1 * a2.x + C2 * a3.x, x0.y + C3 * a1.y + C1 * a2.y + C2 * a3.y);
    float2 i1 = mul_mi<INV>(make_float2(S1 * b1.x + S2 * b2.x + S3 * b3.x, S1 * b1.y + S2 * b2.y + S3 * b3.y));
    float2 i2 = mul_mi<INV>(make_float2(S2 * b1.x - S3 * b2.x - S1 * b3.x, S2 * b1.y - S3 * b2.y - S1 * b3.y));
    float2 i3 = mul_mi<INV>(make_float2(S3 * b1.x - S1 * b2.x + S2 * b3.x, S3 * b1.y - S1 * b2.y + S2 * b3.y));
    v[0] = make_float2(x0.x + a1.x + a2.x + a3.x, x0.y + a1.y + a2.y + a3.y);
    v[1] = cadd(r1, i1);
    v[6] = csub(r1, i1);
    v[2] = cadd(r2, i2);
    v[5] = csub(r2, i2);
    v[3] = cadd(r3, i3);
    v[4] = csub(r3, i3);
  }
};

template <bool INV> struct Dft<8, INV> {
  static __device__ __forceinline__ void run(float2* v) {
    const float h = 0.70710678118654752f;
    float2 e[4] = {v[0], v[2], v[4], v[6]};
    float2 o[4] = {v[1], v[3], v[5], v[7]};
    Dft<4, INV>::run(e);
    Dft<4, INV>::run(o);
    // w^k, w = exp(-+2 pi i / 8)
    float2 o1 = INV ? make_float2(h * (o[1].x - o[1].y), h * (o[1].x + o[1].y))
                    : make_float2(h * (o[1].x + o[1].y), h * (o[1].y - o[1].x));
    float2 o2 = mul_mi<INV>(o[2]);
    float2 o3 = INV ? make_float2(-h * (o[3].x + o[3].y), h * (o[3].x - o[3].y))
                    : make_float2(h * (o[3].y - o[3].x), -h * (o[3].x + o[3].y));
    v[0] = cadd(e[0], o[0]);
    v[4] = csub(e[0], o[0]);
    v[1] = cadd(e[1], o1);
    v[5] = csub(e[1], o1);
    v[2] = cadd(e[2], o2);
    v[6] = csub(e[2], o2);
    v[3] = cadd(e[3], o3);
    v[7] = csub(e[3], o3);
  }
};

}  // namespace pvd
