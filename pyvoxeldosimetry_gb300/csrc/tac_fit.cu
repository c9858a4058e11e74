// Per-voxel time-activity-curve fits in FP64, one thread per voxel.
//
// Replaces the Python loops over scipy.optimize.curve_fit of
//   TimeCurveFitting.fit_time_activity_curve      (time_integration/curve_fitting.py:19-65)
//   TimeCurveFitting._calculate_accumulated_dose  (curve_fitting.py:74-84)
//   TimeCurveFitting.fit_time_activity_curve_advanced (curve_fitting.py:112-219)
// with the same models, initial guesses, sigma = 1/weight residual scaling,
// failure fallbacks and AUC formulas.  The minimiser restates Moré's scaled
// trust-region Levenberg-Marquardt (the published algorithm behind MINPACK
// lmdif, which curve_fit runs) on the normal equations in FP64 with an
// analytic Jacobian where lmdif uses forward differences; initial trust
// region, scaling, step control, convergence tests and info codes follow the
// algorithm, so success/failure match curve_fit's on the same curves.  Non-finite samples or
// fewer samples than parameters are failures, as curve_fit raises for them.
//
// Layout: activities [T][n_vox] float32 (time-major, the stacked maps);
// params [n_par][n_vox] float64; auc [n_vox] float64; ok [n_vox] uint8.
// HBM traffic per voxel: 4T bytes read, 8(n_par+1)+1 bytes written; the
// kernel is FP64-throughput bound (exp and the normal equations per iteration).
#include <algorithm>
#include <map>
#include <mutex>
#include <type_traits>
#include <cmath>

#include "pvd_common.cuh"
#include "sched.cuh"

namespace pvd {

#define PVD_LN2 0.69314718055994530942

enum Model {
  M_MONO_LAMBDA = 0,  // A0 exp(-lam t)                     (fit_time_activity_curve)
  M_F2 = 1, M_F3 = 2, M_F3A = 3, M_F4A = 4, M_F4B = 5, M_F4C = 6,  // NUKFIT
  M_LM_MONO = 7, M_LM_BI = 8, M_LM_TRI = 9                          // "lmfit" table
};

struct FitArgs {
  double t[PVD_MAX_TIMEPOINTS];
  double w[PVD_MAX_TIMEPOINTS];  // residual multipliers (1 / sigma)
  float tf[PVD_MAX_TIMEPOINTS];  // float copies for the FP32 iterations (a conversion from
  float wf[PVD_MAX_TIMEPOINTS];  // double per use would run on GB300's slow FP64 pipe)
  float lam_phys_f;
  double p0[5];
  int T;
  double lam_phys;               // ln2 / physical half-life (models with lambda_phys)
  double auc_limit;              // mono-lambda model: integration limit (same time unit)
  int max_fev;                  // model-evaluation budget (curve_fit's maxfev)
  int force_zero_at_t0;
  int p0_from_data;              // mono-lambda: p0 = [y(t0), lam_phys] per voxel
  int p0_peel;                   // f4a: p0 from exponential peeling of the samples
  int auc_inf;                   // f2 / f4a / mono: analytic integral to infinity
  double f32_scale;              // scale of the optional float32 copy of the AUC
  int mixed;                     // FP32 Levenberg-Marquardt, then FP64 from its end point
};

// sample time, residual weight and physical decay constant in the iteration's precision
template <typename R> __device__ __forceinline__ R t_at(const FitArgs& a, int k);
template <> __device__ __forceinline__ double t_at<double>(const FitArgs& a, int k) { return a.t[k]; }
template <> __device__ __forceinline__ float t_at<float>(const FitArgs& a, int k) { return a.tf[k]; }
template <typename R> __device__ __forceinline__ R w_at(const FitArgs& a, int k);
template <> __device__ __forceinline__ double w_at<double>(const FitArgs& a, int k) { return a.w[k]; }
template <> __device__ __forceinline__ float w_at<float>(const FitArgs& a, int k) { return a.wf[k]; }
template <typename R> __device__ __forceinline__ R lp_of(const FitArgs& a);
template <> __device__ __forceinline__ double lp_of<double>(const FitArgs& a) { return a.lam_phys; }
template <> __device__ __forceinline__ float lp_of<float>(const FitArgs& a) { return a.lam_phys_f; }

// Start for the two-exponential model f4a from "exponential peeling": the slow
// rate from the last two samples (yA at tA, yB at tB), the fast one from what it
// leaves at the first two.  Rates are total (physical + biological); returned
// params subtract lp.
__device__ void peel_biexp4(const FitArgs& a, double y0, double y1, double yA, double yB, double tA, double tB,
                            double* p) {
  const double t0 = a.t[0], t1 = a.t[1];
  double k2 = PVD_LN2 / (10.0 * tB);
  if (yA > 0.0 && yB > 0.0 && yA > yB) k2 = log(yA / yB) / (tB - tA);
  const double A2 = yB * exp(k2 * tB);
  const double r0 = y0 - A2 * exp(-k2 * t0), r1 = y1 - A2 * exp(-k2 * t1);
  double k1 = 4.0 * k2 + PVD_LN2 / t1, A1 = 0.0;
  if (r0 > 0.0 && r1 > 0.0 && r0 > r1) {
    const double kk = log(r0 / r1) / (t1 - t0);
    if (kk > k2) k1 = kk;
  }
  if (r0 > 0.0) A1 = r0 * exp(k1 * t0);
  p[0] = A1;
  p[1] = k1 - a.lam_phys;
  p[2] = A2;
  p[3] = k2 - a.lam_phys;
}

__device__ void peel_biexp(const FitArgs& a, const double* y, double* p) {
  const int T = a.T;
  peel_biexp4(a, y[0], y[1], y[T - 2], y[T - 1], a.t[T - 2], a.t[T - 1], p);
}

template <int M> struct ModelTraits;

// value and gradient of each model at time t
template <> struct ModelTraits<M_MONO_LAMBDA> {
  static constexpr int N = 2;
  template <typename R>
  static __device__ R eval(const R* p, R t, R, R* g) {
    const R e = exp(-p[1] * t);
    g[0] = e;
    g[1] = -t * p[0] * e;
    return p[0] * e;
  }
};
template <> struct ModelTraits<M_F2> {
  static constexpr int N = 2;
  template <typename R>
  static __device__ R eval(const R* p, R t, R lp, R* g) {
    const R e = exp(-(p[1] + lp) * t);
    g[0] = e;
    g[1] = -t * p[0] * e;
    return p[0] * e;
  }
};
template <> struct ModelTraits<M_F3> {
  static constexpr int N = 3;
  template <typename R>
  static __device__ R eval(const R* p, R t, R lp, R* g) {
    const R e1 = exp(-(p[1] + lp) * t), e2 = exp(-(p[2] + lp) * t);
    g[0] = e1 - e2;
    g[1] = -t * p[0] * e1;
    g[2] = t * p[0] * e2;
    return p[0] * (e1 - e2);
  }
};
template <> struct ModelTraits<M_F3A> {
  static constexpr int N = 3;
  template <typename R>
  static __device__ R eval(const R* p, R t, R lp, R* g) {
    const R e1 = exp(-(p[2] + lp) * t), ep = exp(-lp * t);
    g[0] = p[1] * e1 + ((R)1 - p[1]) * ep;
    g[1] = p[0] * (e1 - ep);
    g[2] = -t * p[0] * p[1] * e1;
    return p[0] * (p[1] * e1 + ((R)1 - p[1]) * ep);
  }
};
template <> struct ModelTraits<M_F4A> {
  static constexpr int N = 4;
  template <typename R>
  static __device__ R eval(const R* p, R t, R lp, R* g) {
    const R e1 = exp(-(p[1] + lp) * t), e2 = exp(-(p[3] + lp) * t);
    g[0] = e1;
    g[1] = -t * p[0] * e1;
    g[2] = e2;
    g[3] = -t * p[2] * e2;
    return p[0] * e1 + p[2] * e2;
  }
};
template <> struct ModelTraits<M_F4B> {
  static constexpr int N = 5;
  template <typename R>
  static __device__ R eval(const R* p, R t, R lp, R* g) {
    const R e1 = exp(-(p[1] + lp) * t), e2 = exp(-(p[3] + lp) * t), eb = exp(-(p[4] + lp) * t);
    g[0] = e1 - eb;
    g[1] = -t * p[0] * e1;
    g[2] = -e2 + eb;
    g[3] = t * p[2] * e2;
    g[4] = t * (p[0] - p[2]) * eb;
    return p[0] * e1 - p[2] * e2 - (p[0] - p[2]) * eb;
  }
};
template <> struct ModelTraits<M_F4C> {
  static constexpr int N = 5;
  template <typename R>
  static __device__ R eval(const R* p, R t, R lp, R* g) {
    const R e1 = exp(-(p[1] + lp) * t), e2 = exp(-(p[3] + lp) * t), eb = exp(-(p[4] + lp) * t);
    g[0] = e1 - eb;
    g[1] = -t * p[0] * e1;
    g[2] = e2 - eb;
    g[3] = -t * p[2] * e2;
    g[4] = t * (p[0] + p[2]) * eb;
    return p[0] * e1 + p[2] * e2 - (p[0] + p[2]) * eb;
  }
};
template <> struct ModelTraits<M_LM_MONO> {
  static constexpr int N = 2;
  template <typename R>
  static __device__ R eval(const R* p, R t, R, R* g) {
    const R e = exp(-(R)PVD_LN2 * t / p[1]);
    g[0] = e;
    g[1] = p[0] * e * (R)PVD_LN2 * t / (p[1] * p[1]);
    return p[0] * e;
  }
};
template <> struct ModelTraits<M_LM_BI> {
  static constexpr int N = 3;
  template <typename R>
  static __device__ R eval(const R* p, R t, R, R* g) {
    const R e1 = exp(-(R)PVD_LN2 * t / p[1]), e2 = exp(-(R)PVD_LN2 * t / p[2]);
    g[0] = e1 - e2;
    g[1] = p[0] * e1 * (R)PVD_LN2 * t / (p[1] * p[1]);
    g[2] = -p[0] * e2 * (R)PVD_LN2 * t / (p[2] * p[2]);
    return p[0] * (e1 - e2);
  }
};
template <> struct ModelTraits<M_LM_TRI> {
  static constexpr int N = 5;
  template <typename R>
  static __device__ R eval(const R* p, R t, R, R* g) {
    const R e1 = exp(-(R)PVD_LN2 * t / p[1]), e2 = exp(-(R)PVD_LN2 * t / p[3]), e3 = exp(-(R)PVD_LN2 * t / p[4]);
    g[0] = e1 - e3;
    g[1] = p[0] * e1 * (R)PVD_LN2 * t / (p[1] * p[1]);
    g[2] = -e2 + e3;
    g[3] = -p[2] * e2 * (R)PVD_LN2 * t / (p[3] * p[3]);
    g[4] = -(p[0] - p[2]) * e3 * (R)PVD_LN2 * t / (p[4] * p[4]);
    return p[0] * e1 - p[2] * e2 - (p[0] - p[2]) * e3;
  }
};

// tolerances per precision: MINPACK's defaults (sqrt(eps) ftol/xtol) in double; the
// float iterations stop at 1e-6 and are followed by double ones
template <typename R> struct Lim;
template <> struct Lim<double> {
  static __device__ double tiny() { return 2.2250738585072014e-308; }
  static __device__ double tol() { return 1.49012e-8; }
  static __device__ double eps() { return 2.220446049250313e-16; }
};
template <> struct Lim<float> {
  static __device__ float tiny() { return 1.17549435e-38f; }
  static __device__ float tol() { return 1e-6f; }
  static __device__ float eps() { return 1.1920929e-7f; }
};

// Two-exponential model f4a by variable projection (Golub & Pereyra, SIAM J.
// Numer. Anal. 10, 1973): for rates p = (lam1, lam2) the amplitudes minimising
// the weighted residual are linear least squares, so the cost is
// 0.5 ||P_perp(p) w y||^2 with P_perp the projector onto the complement of
// span{w e1, w e2}, e_i = exp(-(lam_i + lp) t).  Its Jacobian is Kaufman's
// (BIT 15, 1975): column i = P_perp d(w e_i)/d lam_i c_i, exact at zero
// residual.  The basis is orthonormalised by Gram-Schmidt with one
// re-orthogonalisation, so nearly equal rates (cos(e1, e2) -> 1) keep a
// residual accurate to rounding; numerically dependent columns (r22 below
// 64 eps r11) give a non-finite cost, which the trust region rejects.
// TM is a compile-time bound on the number of samples, so the per-sample
// arrays stay in registers.  y is already multiplied by the weights.
constexpr int M_F4A_VP4 = 10, M_F4A_VP6 = 11, M_F4A_VP8 = 12, M_F4A_VP16 = 13;
template <int TM> struct VpTraits {
  static constexpr int N = 2;
  static constexpr bool VP = true;
  static constexpr int TMAX = TM;
};
template <> struct ModelTraits<M_F4A_VP4> : VpTraits<4> {};
template <> struct ModelTraits<M_F4A_VP6> : VpTraits<6> {};
template <> struct ModelTraits<M_F4A_VP8> : VpTraits<8> {};
template <> struct ModelTraits<M_F4A_VP16> : VpTraits<16> {};
template <int M, typename = void> struct IsVp { static constexpr bool value = false; };
template <int M> struct IsVp<M, decltype((void)ModelTraits<M>::VP)> { static constexpr bool value = ModelTraits<M>::VP; };

template <int TM, typename R>
struct VpBasis {
  R e1[TM], e2[TM];  // weighted exponentials, then the orthonormal basis q1, q2
  R r[TM];           // residual y - Phi c (weighted)
  R r11, r12, r22, c1, c2;
};

template <int TM, typename R>
__device__ __forceinline__ R vp_project(const FitArgs& a, const R* y, const R* p, VpBasis<TM, R>& b) {
  const R lp = lp_of<R>(a);
  R n1 = (R)0;
#pragma unroll
  for (int j = 0; j < TM; ++j) {
    if (j < a.T) {
      const R w = w_at<R>(a, j), t = t_at<R>(a, j);
      b.e1[j] = w * exp(-(p[0] + lp) * t);
      b.e2[j] = w * exp(-(p[1] + lp) * t);
    } else {
      b.e1[j] = (R)0;
      b.e2[j] = (R)0;
    }
    n1 += b.e1[j] * b.e1[j];
  }
  b.r11 = sqrt(n1);
  if (!(b.r11 > Lim<R>::tiny())) return (R)NAN;
  R d = (R)0;
#pragma unroll
  for (int j = 0; j < TM; ++j) {
    b.e1[j] /= b.r11;
    d += b.e1[j] * b.e2[j];
  }
  R d2 = (R)0;
#pragma unroll
  for (int j = 0; j < TM; ++j) {
    b.e2[j] -= d * b.e1[j];
    d2 += b.e1[j] * b.e2[j];
  }
  R n2 = (R)0;
#pragma unroll
  for (int j = 0; j < TM; ++j) {
    b.e2[j] -= d2 * b.e1[j];
    n2 += b.e2[j] * b.e2[j];
  }
  b.r12 = d + d2;
  b.r22 = sqrt(n2);
  if (!(b.r22 > (R)64 * Lim<R>::eps() * b.r11)) return (R)NAN;
  R s1 = (R)0;
#pragma unroll
  for (int j = 0; j < TM; ++j) {
    b.e2[j] /= b.r22;
    s1 += b.e1[j] * y[j];
  }
  R s2 = (R)0;
#pragma unroll
  for (int j = 0; j < TM; ++j) {
    b.r[j] = y[j] - s1 * b.e1[j];
    s2 += b.e2[j] * b.r[j];
  }
  R cost = (R)0;
#pragma unroll
  for (int j = 0; j < TM; ++j) {
    b.r[j] -= s2 * b.e2[j];
    cost += b.r[j] * b.r[j];
  }
  b.c2 = s2 / b.r22;
  b.c1 = (s1 - b.r12 * b.c2) / b.r11;
  return (R)0.5 * cost;
}

// normal equations of the projected problem; LM residual is Phi c - y = -r
template <int TM, typename R>
__device__ __forceinline__ R vp_normal_eq(const FitArgs& a, const R* y, const R* p, R* A, R* g) {
  VpBasis<TM, R> b;
  const R cost = vp_project<TM, R>(a, y, p, b);
  if (!isfinite(cost)) {
    A[0] = A[1] = A[2] = A[3] = g[0] = g[1] = (R)0;
    return cost;
  }
  // d(w e_i)/d lam_i * c_i = -t w e_i c_i, rebuilt from q1, q2 and R: w e1 = r11 q1,
  // w e2 = r12 q1 + r22 q2
  R j1[TM], j2[TM];
  R u1 = (R)0, u2 = (R)0, v1 = (R)0, v2 = (R)0;
#pragma unroll
  for (int j = 0; j < TM; ++j) {
    const R t = j < a.T ? t_at<R>(a, j) : (R)0;
    const R we1 = b.r11 * b.e1[j], we2 = b.r12 * b.e1[j] + b.r22 * b.e2[j];
    j1[j] = -t * we1 * b.c1;
    j2[j] = -t * we2 * b.c2;
    u1 += b.e1[j] * j1[j];
    u2 += b.e1[j] * j2[j];
  }
#pragma unroll
  for (int j = 0; j < TM; ++j) {
    j1[j] -= u1 * b.e1[j];
    j2[j] -= u2 * b.e1[j];
    v1 += b.e2[j] * j1[j];
    v2 += b.e2[j] * j2[j];
  }
  R a11 = (R)0, a12 = (R)0, a22 = (R)0, g1 = (R)0, g2 = (R)0;
#pragma unroll
  for (int j = 0; j < TM; ++j) {
    j1[j] -= v1 * b.e2[j];
    j2[j] -= v2 * b.e2[j];
    a11 += j1[j] * j1[j];
    a12 += j1[j] * j2[j];
    a22 += j2[j] * j2[j];
    g1 -= j1[j] * b.r[j];
    g2 -= j2[j] * b.r[j];
  }
  A[0] = a11;
  A[1] = a12;
  A[2] = a12;
  A[3] = a22;
  g[0] = g1;
  g[1] = g2;
  return cost;
}

// normal equations at p: A = J^T J (upper triangle), g = J^T r, returns 0.5 r^T r
template <int M, typename R>
__device__ R normal_eq(const FitArgs& a, const R* y, const R* p, R* A, R* g) {
  if constexpr (IsVp<M>::value) {
    return vp_normal_eq<ModelTraits<M>::TMAX, R>(a, y, p, A, g);
  } else {
  constexpr int N = ModelTraits<M>::N;
#pragma unroll
  for (int i = 0; i < N * N; ++i) A[i] = (R)0;
#pragma unroll
  for (int i = 0; i < N; ++i) g[i] = (R)0;
  R cost = (R)0;
  for (int k = 0; k < a.T; ++k) {
    R j[N];
    const R w = w_at<R>(a, k);
    const R f = ModelTraits<M>::template eval<R>(p, t_at<R>(a, k), lp_of<R>(a), j);
    const R r = w * (f - y[k]);
#pragma unroll
    for (int i = 0; i < N; ++i) j[i] *= w;
#pragma unroll
    for (int i = 0; i < N; ++i) {
      g[i] += j[i] * r;
#pragma unroll
      for (int c = i; c < N; ++c) A[i * N + c] += j[i] * j[c];
    }
    cost += r * r;
  }
  return (R)0.5 * cost;
  }
}

template <int M, typename R>
__device__ R cost_at(const FitArgs& a, const R* y, const R* p) {
  if constexpr (IsVp<M>::value) {
    VpBasis<ModelTraits<M>::TMAX, R> b;
    return vp_project<ModelTraits<M>::TMAX, R>(a, y, p, b);
  } else {
  constexpr int N = ModelTraits<M>::N;
  R cost = (R)0;
  for (int k = 0; k < a.T; ++k) {
    R j[N];
    const R r = w_at<R>(a, k) * (ModelTraits<M>::template eval<R>(p, t_at<R>(a, k), lp_of<R>(a), j) - y[k]);
    cost += r * r;
  }
  return (R)0.5 * cost;
  }
}

// Cholesky of (A + par diag(D^2)) (A symmetric, upper triangle stored in A[i*N+c], c >= i).
// L is lower triangular, row major.  false if not positive definite.
template <int N, typename R>
__device__ bool chol_damped(const R* A, const R* D, R par, R* L) {
#pragma unroll
  for (int i = 0; i < N; ++i) {
#pragma unroll
    for (int c = 0; c <= i; ++c) {
      R s = (c == i) ? A[i * N + i] + par * D[i] * D[i] : A[c * N + i];
      for (int k = 0; k < c; ++k) s -= L[i * N + k] * L[c * N + k];
      if (c == i) {
        if (!(s > (R)0.0)) return false;
        L[i * N + i] = sqrt(s);
      } else {
        L[i * N + c] = s / L[c * N + c];
      }
    }
  }
  return true;
}

template <int N, typename R>
__device__ void chol_fwd(const R* L, const R* b, R* z) {  // L z = b
#pragma unroll
  for (int i = 0; i < N; ++i) {
    R s = b[i];
    for (int k = 0; k < i; ++k) s -= L[i * N + k] * z[k];
    z[i] = s / L[i * N + i];
  }
}

template <int N, typename R>
__device__ void chol_solve_neg(const R* L, const R* g, R* p) {  // L L^T p = -g
  R z[N];
  R mg[N];
#pragma unroll
  for (int i = 0; i < N; ++i) mg[i] = -g[i];
  chol_fwd<N, R>(L, mg, z);
#pragma unroll
  for (int i = N - 1; i >= 0; --i) {
    R s = z[i];
    for (int k = i + 1; k < N; ++k) s -= L[k * N + i] * p[k];
    p[i] = s / L[i * N + i];
  }
}

template <int N, typename R>
__device__ R dnorm(const R* D, const R* v) {
  R s = (R)0.0;
#pragma unroll
  for (int i = 0; i < N; ++i) s += (D[i] * v[i]) * (D[i] * v[i]);
  return sqrt(s);
}

// Trust-region step (Moré, "The Levenberg-Marquardt algorithm: implementation
// and theory", 1978, the lmpar procedure) on the normal equations: find
// par >= 0 with ||D p|| within 10 % of delta, p = -(A + par D^2)^-1 g, or the
// Gauss-Newton step (par = 0) when it already fits in the region.
template <int N, typename R>
__device__ void lm_par(const R* A, const R* g, const R* D, R delta, R& par, R* p) {
  const R dwarf = Lim<R>::tiny();
  R L[N * N], w[N], q[N];
  R parl = (R)0.0;
  R fp;
  const bool have_gn = chol_damped<N, R>(A, D, (R)0.0, L);  // false: J^T J singular, no Gauss-Newton step
  if (have_gn) {
    chol_solve_neg<N, R>(L, g, p);
    const R dxn = dnorm<N, R>(D, p);
    fp = dxn - delta;
    if (fp <= (R)0.1 * delta) {
      par = (R)0.0;
      return;
    }
#pragma unroll
    for (int i = 0; i < N; ++i) q[i] = D[i] * (D[i] * p[i]) / dxn;
    chol_fwd<N, R>(L, q, w);
    R wn = (R)0.0;
#pragma unroll
    for (int i = 0; i < N; ++i) wn += w[i] * w[i];
    parl = (fp / delta) / wn;
  }
  R gn = (R)0.0;
#pragma unroll
  for (int i = 0; i < N; ++i) gn += (g[i] / D[i]) * (g[i] / D[i]);
  gn = sqrt(gn);
  R paru = gn / delta;
  if (paru == (R)0.0) paru = dwarf / fmin(delta, (R)0.1);
  par = fmax(par, parl);
  par = fmin(par, paru);
  if (par == (R)0.0 && have_gn) par = gn / fmax(dnorm<N, R>(D, p), dwarf);  // else 0.001 paru below
  fp = (R)0.0;
  for (int it = 1; it <= 10; ++it) {
    if (par == (R)0.0) par = fmax(dwarf, (R)0.001 * paru);
    if (!chol_damped<N, R>(A, D, par, L)) {  // only possible when D has zero entries
      par = fmax(par * (R)10.0, dwarf);
      continue;
    }
    chol_solve_neg<N, R>(L, g, p);
    const R dxn = dnorm<N, R>(D, p);
    const R temp = fp;
    fp = dxn - delta;
    if (fabs(fp) <= (R)0.1 * delta || (parl == (R)0.0 && fp <= temp && temp < (R)0.0) || it == 10) break;
#pragma unroll
    for (int i = 0; i < N; ++i) q[i] = D[i] * (D[i] * p[i]) / dxn;
    chol_fwd<N, R>(L, q, w);
    R wn = (R)0.0;
#pragma unroll
    for (int i = 0; i < N; ++i) wn += w[i] * w[i];
    const R parc = (fp / delta) / wn;
    if (fp > (R)0.0) parl = fmax(parl, par);
    if (fp < (R)0.0) paru = fmin(paru, par);
    par = fmax(parl, par + parc);
  }
}

// Moré's Levenberg-Marquardt outer iteration (scaled trust region) with an
// analytic Jacobian, as a resumable state machine: lm_begin, then lm_tick until
// it returns non-zero.  Each tick evaluates the normal equations when the last
// step was accepted and makes one trial step, so a lane can interleave voxels at
// tick granularity.  Info codes are MINPACK's: 1-4 success (ftol / xtol / both /
// gtol), 5 evaluation budget exhausted, 6-8 tolerances too small, -1 non-finite
// cost.  `maxfev` counts model evaluations as a forward-difference Jacobian
// would (N per Jacobian), so the budget matches curve_fit's.  fstop > 0 adds a
// success test (info 1): residual norm <= fstop.
template <int M, typename R>
struct LmState {
  static constexpr int N = ModelTraits<M>::N;
  R x[N], D[N], A[N * N], g[N];
  R fnorm, delta, xnorm, par, gnorm, fstop;
  int iter, nfev, maxfev;
  bool need_jac;
};

template <int M, typename R>
__device__ __forceinline__ int lm_begin(const FitArgs& a, const R* y, LmState<M, R>& s) {
  s.nfev = 1;
  s.fnorm = sqrt((R)2.0 * cost_at<M, R>(a, y, s.x));
  if (!isfinite(s.fnorm)) return -1;
  if (s.fnorm <= s.fstop) return 1;
  s.delta = (R)0.0;
  s.xnorm = (R)0.0;
  s.par = (R)0.0;
  s.gnorm = (R)0.0;
  s.iter = 1;
  s.need_jac = true;
  return 0;
}

template <int M, typename R>
__device__ __forceinline__ int lm_tick(const FitArgs& a, const R* y, LmState<M, R>& s) {
  constexpr int N = ModelTraits<M>::N;
  const R ftol = Lim<R>::tol(), xtol = Lim<R>::tol(), epsmch = Lim<R>::eps();
  if (s.need_jac) {
    normal_eq<M, R>(a, y, s.x, s.A, s.g);
    s.nfev += N;
    R acn[N];
#pragma unroll
    for (int j = 0; j < N; ++j) acn[j] = sqrt(s.A[j * N + j]);
    if (s.iter == 1) {
#pragma unroll
      for (int j = 0; j < N; ++j) s.D[j] = (acn[j] == (R)0.0) ? (R)1.0 : acn[j];
      s.xnorm = dnorm<N, R>(s.D, s.x);
      s.delta = (R)100.0 * s.xnorm;
      if (s.delta == (R)0.0) s.delta = (R)100.0;
    }
    R gnorm = (R)0.0;
    if (s.fnorm != (R)0.0) {
#pragma unroll
      for (int j = 0; j < N; ++j)
        if (acn[j] != (R)0.0) gnorm = fmax(gnorm, fabs(s.g[j] / s.fnorm) / acn[j]);
    }
    s.gnorm = gnorm;
    if (gnorm <= (R)0.0) return 4;  // gtol = 0
#pragma unroll
    for (int j = 0; j < N; ++j) s.D[j] = fmax(s.D[j], acn[j]);
    s.need_jac = false;
  }
  // one trial step of the inner loop
  R p[N], xt[N];
  lm_par<N, R>(s.A, s.g, s.D, s.delta, s.par, p);
#pragma unroll
  for (int j = 0; j < N; ++j) xt[j] = s.x[j] + p[j];
  const R pnorm = dnorm<N, R>(s.D, p);
  if (s.iter == 1) s.delta = fmin(s.delta, pnorm);
  const R fnorm1 = sqrt((R)2.0 * cost_at<M, R>(a, y, xt));
  s.nfev += 1;
  R actred = -(R)1.0;
  if ((R)0.1 * fnorm1 < s.fnorm) actred = (R)1.0 - (fnorm1 / s.fnorm) * (fnorm1 / s.fnorm);
  R jp2 = (R)0.0;  // ||J p||^2 = p^T A p
#pragma unroll
  for (int i = 0; i < N; ++i) {
    R row = (R)0.0;
#pragma unroll
    for (int c = 0; c < N; ++c) row += (c >= i ? s.A[i * N + c] : s.A[c * N + i]) * p[c];
    jp2 += p[i] * row;
  }
  const R t1 = sqrt(fmax(jp2, (R)0.0)) / s.fnorm;
  const R t2 = sqrt(s.par) * pnorm / s.fnorm;
  const R prered = t1 * t1 + t2 * t2 / (R)0.5;
  const R dirder = -(t1 * t1 + t2 * t2);
  R ratio = (prered != (R)0.0) ? actred / prered : (R)0.0;
  if (!isfinite(fnorm1)) ratio = (R)0.0;
  if (ratio <= (R)0.25) {
    R temp = (actred >= (R)0.0) ? (R)0.5 : (R)0.5 * dirder / (dirder + (R)0.5 * actred);
    if ((R)0.1 * fnorm1 >= s.fnorm || temp < (R)0.1 || !isfinite(fnorm1)) temp = (R)0.1;
    s.delta = temp * fmin(s.delta, pnorm / (R)0.1);
    s.par = s.par / temp;
  } else if (s.par == (R)0.0 || ratio >= (R)0.75) {
    s.delta = pnorm / (R)0.5;
    s.par = (R)0.5 * s.par;
  }
  const bool accepted = ratio >= (R)1e-4;
  if (accepted) {
#pragma unroll
    for (int j = 0; j < N; ++j) s.x[j] = xt[j];
    s.fnorm = fnorm1;
    s.xnorm = dnorm<N, R>(s.D, s.x);
    if (s.fnorm <= s.fstop) return 1;  // the curve reproduces the samples to their own precision
  }
  int info = 0;
  if (fabs(actred) <= ftol && prered <= ftol && (R)0.5 * ratio <= (R)1.0) info = 1;
  if (s.delta <= xtol * s.xnorm) info = (info == 1) ? 3 : 2;
  if (info) return info;
  if (s.nfev >= s.maxfev) return 5;
  if (fabs(actred) <= epsmch && prered <= epsmch && (R)0.5 * ratio <= (R)1.0) return 6;
  if (s.delta <= epsmch * s.xnorm) return 7;
  if (s.gnorm <= epsmch) return 8;
  if (accepted) {  // next outer iteration
    ++s.iter;
    s.need_jac = true;
  }
  return 0;
}

template <int M, typename R>
__device__ int lm_fit(const FitArgs& a, const R* y, R* x, int maxfev, R fstop = (R)0) {
  constexpr int N = ModelTraits<M>::N;
  LmState<M, R> s;
#pragma unroll
  for (int j = 0; j < N; ++j) s.x[j] = x[j];
  s.maxfev = maxfev;
  s.fstop = fstop;
  int info = lm_begin<M, R>(a, y, s);
  while (info == 0) info = lm_tick<M, R>(a, y, s);
#pragma unroll
  for (int j = 0; j < N; ++j) x[j] = s.x[j];
  return info;
}

// Fallbacks of a failed fit, the AUC and the stores of one voxel.  good: the
// minimiser converged (curve_fit raises for any other outcome).
template <int M>
__device__ __forceinline__ void store_fit(const FitArgs& a, double* p, bool good, double ymax, long long v, long long nvox,
                                          double* __restrict__ params, double* __restrict__ auc,
                                          unsigned char* __restrict__ ok, float* __restrict__ auc32) {
  constexpr int N = ModelTraits<M>::N;
  if (!good) {
    if (M == M_MONO_LAMBDA) {  // fallback [0, lam_phys] (curve_fitting.py:58-59)
      p[0] = 0.0;
      p[1] = a.lam_phys;
    } else {                   // fallback zeros (curve_fitting.py:210-213)
#pragma unroll
      for (int i = 0; i < N; ++i) p[i] = 0.0;
    }
  }
#pragma unroll
  for (int i = 0; i < N; ++i) params[(long long)i * nvox + v] = p[i];
  double s = 0.0;
  bool inf_done = false;
  if (a.auc_inf && good) {  // integral of the fitted curve from 0 to infinity
    if constexpr (M == M_MONO_LAMBDA) {
      if (p[1] > 0.0) {
        s = p[0] / p[1];
        inf_done = true;
      }
    } else if constexpr (M == M_F2) {
      const double k = p[1] + a.lam_phys;
      if (k > 0.0) {
        s = p[0] / k;
        inf_done = true;
      }
    } else if constexpr (M == M_F4A) {
      // A1 e^{-k1 t} + A2 e^{-k2 t} is >= 0 on [0, inf) iff the slow amplitude is
      // >= 0 and A1 + A2 >= 0.  The part before the first sample is an
      // extrapolation: a component that decays by orders of magnitude before
      // it (a runaway fast rate whose amplitude no sample constrains) would
      // dominate the integral, so the curve at t = 0 may not exceed 100 times
      // the largest sample.  Otherwise there is no meaningful cumulated activity.
      const double k1 = p[1] + a.lam_phys, k2 = p[3] + a.lam_phys;
      const double a_slow = (k1 < k2) ? p[0] : p[2];
      const double f0 = p[0] + p[2];
      const bool nonneg = a_slow >= 0.0 && f0 >= -1e-9 * (fabs(p[0]) + fabs(p[2]));
      if (k1 > 0.0 && k2 > 0.0 && nonneg && f0 <= 100.0 * ymax) {
        s = p[0] / k1 + p[2] / k2;
        inf_done = true;
      }
    }
    if (inf_done && !(isfinite(s) && isfinite((float)(s * a.f32_scale)))) inf_done = false;
    if (!inf_done) good = false;  // diverging or unsupported: the sampled-interval rule below
  }
  if (inf_done) {
  } else if (M == M_MONO_LAMBDA) {
    // A0 / lam * (1 - exp(-lam * limit))  (curve_fitting.py:74-84)
    s = p[0] / p[1] * (1.0 - exp(-p[1] * a.auc_limit));
  } else {
    // trapezoid of the fitted curve over the sampled times (curve_fitting.py:215)
    double j[N];
    s = 0.0;
    double fprev = ModelTraits<M>::template eval<double>(p, a.t[0], a.lam_phys, j);
    for (int k = 1; k < a.T; ++k) {
      const double f = ModelTraits<M>::template eval<double>(p, a.t[k], a.lam_phys, j);
      s += 0.5 * (f + fprev) * (a.t[k] - a.t[k - 1]);
      fprev = f;
    }
  }
  float s32 = (float)(s * a.f32_scale);
  if (!isfinite(s32)) {  // the float copy feeds a convolution: one inf would reach every voxel
    s32 = 0.0f;
    good = false;
  }
  auc[v] = s;
  if (auc32) auc32[v] = s32;
  if (ok) ok[v] = good ? 1 : 0;
}

// Evaluation budget of the FP64 stage that finishes an FP32 fit: from an FP32
// least-squares point the iteration converges quadratically in two or three
// steps; 60 evaluations also cover slow cases, and a voxel that needs more
// (FP64 runs at a small fraction of the FP32 rate, and one voxel holds its
// whole warp) is reported as not converged.
constexpr int kFinishFev = 60;

template <int M>
__global__ void k_tac_fit(FitArgs a, const float* __restrict__ acts, long long nvox, double* __restrict__ params,
                          double* __restrict__ auc, unsigned char* __restrict__ ok, float* __restrict__ auc32) {
  constexpr int N = ModelTraits<M>::N;
  for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < nvox; v += (long long)gridDim.x * blockDim.x) {
    double y[PVD_MAX_TIMEPOINTS];
    bool finite = true;
    for (int k = 0; k < a.T; ++k) {
      y[k] = (double)__ldg(acts + (long long)k * nvox + v);
      finite = finite && isfinite(y[k]);
    }
    if (a.force_zero_at_t0) {
      const double y0 = y[0];
      for (int k = 0; k < a.T; ++k) y[k] -= y0;
      y[0] = 0.0;
    }
    double p[N];
#pragma unroll
    for (int i = 0; i < N; ++i) p[i] = a.p0[i];
    if (M == M_MONO_LAMBDA && a.p0_from_data) {
      p[0] = y[0];
      p[1] = a.lam_phys;
    }
    if constexpr (M == M_F4A) {
      if (a.p0_peel && finite && a.T >= 4) peel_biexp(a, y, p);
    }
    int info = -1;
    if (!(finite && a.T >= N)) {
      info = -1;
    } else if (a.mixed) {
      float yf[PVD_MAX_TIMEPOINTS], pf[N];
      for (int k = 0; k < a.T; ++k) yf[k] = (float)y[k];
#pragma unroll
      for (int i = 0; i < N; ++i) pf[i] = (float)p[i];
      lm_fit<M, float>(a, yf, pf, a.max_fev);
      bool pf_finite = true;
#pragma unroll
      for (int i = 0; i < N; ++i) pf_finite = pf_finite && isfinite(pf[i]);
      if (pf_finite) {
#pragma unroll
        for (int i = 0; i < N; ++i) p[i] = (double)pf[i];
      }
      info = lm_fit<M, double>(a, y, p, min(a.max_fev, kFinishFev));  // FP64 from the FP32 end point decides
    } else {
      info = lm_fit<M, double>(a, y, p, a.max_fev);
    }
    double ymax = 0.0;
    for (int k = 0; k < a.T; ++k) ymax = fmax(ymax, fabs(y[k]));
    store_fit<M>(a, p, info >= 1 && info <= 4, ymax, v, nvox, params, auc, ok, auc32);
  }
}


// Other models, FP64 (the reference-parity path): one lane per voxel at a time with refill.
template <int M>
__global__ void __launch_bounds__(128) k_tac_fit_sched(FitArgs a, const float* __restrict__ acts, long long nvox,
                                                       long long per_block, double* __restrict__ params,
                                                       double* __restrict__ auc, unsigned char* __restrict__ ok,
                                                       float* __restrict__ auc32) {
  constexpr int N = ModelTraits<M>::N;
  __shared__ unsigned long long next;
  const long long r0 = (long long)blockIdx.x * per_block;
  const long long r1 = min(nvox, r0 + per_block);
  if (threadIdx.x == 0) next = (unsigned long long)r0;
  __syncthreads();
  double y[PVD_MAX_TIMEPOINTS];
  double ymax = 0.0;
  LmState<M, double> s;
  long long v = 0;
  auto init = [&](long long vv) -> int {
    v = vv;
    bool finite = true;
    ymax = 0.0;
    for (int k = 0; k < a.T; ++k) {
      y[k] = (double)__ldg(acts + (long long)k * nvox + v);
      finite = finite && isfinite(y[k]);
    }
    if (a.force_zero_at_t0) {
      const double y0 = y[0];
      for (int k = 0; k < a.T; ++k) y[k] -= y0;
      y[0] = 0.0;
    }
    for (int k = 0; k < a.T; ++k) ymax = fmax(ymax, fabs(y[k]));
#pragma unroll
    for (int i = 0; i < N; ++i) s.x[i] = a.p0[i];
    if (M == M_MONO_LAMBDA && a.p0_from_data) {
      s.x[0] = y[0];
      s.x[1] = a.lam_phys;
    }
    if constexpr (M == M_F4A) {
      if (a.p0_peel && finite && a.T >= 4) peel_biexp(a, y, s.x);
    }
    s.maxfev = a.max_fev;
    s.fstop = 0.0;
    if (!(finite && a.T >= N)) return -1;
    return lm_begin<M, double>(a, y, s);
  };
  auto tick = [&]() -> int { return lm_tick<M, double>(a, y, s); };
  auto finish = [&](int info) {
    double p[N];
#pragma unroll
    for (int i = 0; i < N; ++i) p[i] = s.x[i];
    store_fit<M>(a, p, info >= 1 && info <= 4, ymax, v, nvox, params, auc, ok, auc32);
  };
  refill_loop(r0, r1, &next, init, tick, finish);
}

// Variable-projection fit of f4a (PVD_FIT_VARPRO) with lane refill.  The number
// of trust-region steps differs widely between voxels (nearly equal rates make a
// long curved valley), so one voxel per thread leaves most lanes of a warp idle.
// Here every block owns a contiguous range of voxels and each lane steps its
// voxel one tick at a time (lm_tick); when a lane's voxel is done the warp takes
// the next voxels of the range from a shared-memory counter (one atomic per warp,
// lane offsets from the ballot), so lanes stay busy until the range is exhausted.
// FP32 and FP64 run as two launches (PVD_FIT_MIXED): the first from the
// exponential-peeling start, handing its rates to the second through params;
// a warp never mixes the two precisions.  FP64 iterations also stop once the
// curve reproduces the float32 samples to their rounding (2^-24 relative each).
// The amplitudes are then solved at the converged rates in FP64; the fast
// component is stored first.
constexpr int kVpThreads = 128;

template <int TM>
struct VpVoxel {
  double y[TM], yw[TM];
  double fstop;
  bool finite;
};

template <int TM>
__device__ __forceinline__ void vp_load(const FitArgs& a, const float* __restrict__ acts, long long nvox, long long v,
                                        VpVoxel<TM>& d) {
  d.finite = true;
#pragma unroll
  for (int k = 0; k < TM; ++k) {
    d.y[k] = k < a.T ? (double)__ldg(acts + (long long)k * nvox + v) : 0.0;
    d.finite = d.finite && isfinite(d.y[k]);
  }
  if (a.force_zero_at_t0) {
    const double y0 = d.y[0];
#pragma unroll
    for (int k = 1; k < TM; ++k)
      if (k < a.T) d.y[k] -= y0;
    d.y[0] = 0.0;
  }
  double yn = 0.0;
#pragma unroll
  for (int k = 0; k < TM; ++k) {
    d.yw[k] = k < a.T ? a.w[k] * d.y[k] : 0.0;
    yn += d.yw[k] * d.yw[k];
  }
  // float32 samples carry relative rounding <= 2^-24 each: a fitted curve within
  // twice that of the samples reproduces them to their own precision
  d.fstop = 2.0 * 5.9604644775390625e-8 * sqrt(yn);
}

// the starting rates: exponential peeling, or p0
template <int TM>
__device__ __forceinline__ void vp_start(const FitArgs& a, const VpVoxel<TM>& d, double* lam) {
  double p[4];
#pragma unroll
  for (int i = 0; i < 4; ++i) p[i] = a.p0[i];
  if (a.p0_peel && d.finite) {
    double yA = 0.0, yB = 0.0;
#pragma unroll
    for (int k = 0; k < TM; ++k) {
      if (k == a.T - 2) yA = d.y[k];
      if (k == a.T - 1) yB = d.y[k];
    }
    peel_biexp4(a, d.y[0], d.y[1], yA, yB, a.t[a.T - 2], a.t[a.T - 1], p);
  }
  lam[0] = p[1];
  lam[1] = p[3];
}

// amplitudes at the final rates, fallbacks, AUC and stores
template <int TM>
__device__ __forceinline__ void vp_store(const FitArgs& a, const VpVoxel<TM>& d, const double* lam, bool good,
                                         long long v, long long nvox, double* __restrict__ params,
                                         double* __restrict__ auc, unsigned char* __restrict__ ok,
                                         float* __restrict__ auc32) {
  double p[4] = {0.0, 0.0, 0.0, 0.0};
  if (good) {
    VpBasis<TM, double> b;
    good = isfinite(vp_project<TM, double>(a, d.yw, lam, b));
    const bool swap = lam[1] > lam[0];
    p[0] = swap ? b.c2 : b.c1;
    p[1] = swap ? lam[1] : lam[0];
    p[2] = swap ? b.c1 : b.c2;
    p[3] = swap ? lam[0] : lam[1];
  }
  double ymax = 0.0;
#pragma unroll
  for (int k = 0; k < TM; ++k) ymax = fmax(ymax, fabs(d.y[k]));
  store_fit<M_F4A>(a, p, good, ymax, v, nvox, params, auc, ok, auc32);
}

constexpr int kVpPolished = 100;  // init code of a voxel the polish already stored

// FP64 polish between the FP32 and the FP64 trust-region stages (PVD_FIT_MIXED): from
// the FP32 rates, at most three Gauss-Newton steps on the two rates of the projected
// problem (the same normal equations the trust region uses), each kept only if it
// lowers the cost.  A voxel whose curve then reproduces its float32 samples to their
// rounding (the FP64 stage's own stopping test, ||r|| <= fstop) is stored here; any
// other keeps its FP32 rates in params[1], params[3] and gets NaN in params[0], which
// sends it to the FP64 trust-region stage.  Near the minimum the Gauss-Newton steps
// converge quadratically, and a warp runs them without the trust region's branches.
template <int MV>
__global__ void __launch_bounds__(kVpThreads) k_tac_fit_vp_polish(FitArgs a, const float* __restrict__ acts,
                                                                  long long nvox, double* __restrict__ params,
                                                                  double* __restrict__ auc,
                                                                  unsigned char* __restrict__ ok,
                                                                  float* __restrict__ auc32) {
  constexpr int TM = ModelTraits<MV>::TMAX;
  for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < nvox;
       v += (long long)gridDim.x * blockDim.x) {
    VpVoxel<TM> d;
    vp_load<TM>(a, acts, nvox, v, d);
    double lam[2] = {params[1 * nvox + v], params[3 * nvox + v]};
    bool good = d.finite && a.T >= 4 && isfinite(lam[0]) && isfinite(lam[1]);
    bool done = false;
    if (good) {
      double A[4], g[2];
      double cost = vp_normal_eq<TM, double>(a, d.yw, lam, A, g);
      for (int it = 0; it < 3 && isfinite(cost) && !done; ++it) {
        if (sqrt(2.0 * cost) <= d.fstop) {
          done = true;
          break;
        }
        const double det = A[0] * A[3] - A[1] * A[1];
        if (!(det > 0.0) || !isfinite(det)) break;
        const double l1[2] = {lam[0] - (A[3] * g[0] - A[1] * g[1]) / det,
                              lam[1] - (A[0] * g[1] - A[1] * g[0]) / det};
        double A1[4], g1[2];
        const double c1 = vp_normal_eq<TM, double>(a, d.yw, l1, A1, g1);
        if (!(c1 < cost)) break;
        lam[0] = l1[0], lam[1] = l1[1], cost = c1;
        for (int i = 0; i < 4; ++i) A[i] = A1[i];
        g[0] = g1[0], g[1] = g1[1];
      }
      if (!done && isfinite(cost) && sqrt(2.0 * cost) <= d.fstop) done = true;
    }
    if (done) {
      vp_store<TM>(a, d, lam, true, v, nvox, params, auc, ok, auc32);
    } else {
      params[v] = (double)NAN;  // to the FP64 trust-region stage, from the FP32 rates
    }
  }
}

// STAGE 0: FP32 from the peeling start, rates handed over in params[1], params[3].
// STAGE 1: FP64 from those rates (PVD_FIT_MIXED; only the voxels the polish left,
// marked by NaN in params[0]) or from the start, then the stores.
template <int MV, int STAGE>
__global__ void __launch_bounds__(kVpThreads) k_tac_fit_vp(FitArgs a, const float* __restrict__ acts, long long nvox,
                                                           long long per_block, double* __restrict__ params,
                                                           double* __restrict__ auc, unsigned char* __restrict__ ok,
                                                           float* __restrict__ auc32) {
  constexpr int TM = ModelTraits<MV>::TMAX;
  using R = typename std::conditional<STAGE == 0, float, double>::type;
  __shared__ unsigned long long next;
  const long long r0 = (long long)blockIdx.x * per_block;
  const long long r1 = min(nvox, r0 + per_block);
  if (threadIdx.x == 0) next = (unsigned long long)r0;
  __syncthreads();
  VpVoxel<TM> d;
  LmState<MV, R> s;
  R yr[TM];
  double lam0[2] = {0.0, 0.0};  // start of the stage (STAGE 0 keeps it for a non-finite FP32 result)
  long long v = 0;
  auto init = [&](long long vv) -> int {
    v = vv;
    if (STAGE == 1 && a.mixed && !isnan(params[v])) return kVpPolished;
    vp_load<TM>(a, acts, nvox, v, d);
    if (STAGE == 1 && a.mixed) {
      lam0[0] = params[1 * nvox + v];
      lam0[1] = params[3 * nvox + v];
    } else {
      vp_start<TM>(a, d, lam0);
    }
#pragma unroll
    for (int k = 0; k < TM; ++k) yr[k] = (R)d.yw[k];
    s.x[0] = (R)lam0[0];
    s.x[1] = (R)lam0[1];
    s.maxfev = a.max_fev;
    s.fstop = STAGE == 0 ? (R)0 : (R)d.fstop;
    if (!(d.finite && a.T >= 4 && isfinite(lam0[0]) && isfinite(lam0[1]))) return -1;
    return lm_begin<MV, R>(a, yr, s);
  };
  auto tick = [&]() -> int { return lm_tick<MV, R>(a, yr, s); };
  auto finish = [&](int info) {
    if (info == kVpPolished) return;
    if (STAGE == 0) {
      const bool f = isfinite(s.x[0]) && isfinite(s.x[1]);
      params[1 * nvox + v] = f ? (double)s.x[0] : lam0[0];
      params[3 * nvox + v] = f ? (double)s.x[1] : lam0[1];
    } else {
      double lam[2] = {(double)s.x[0], (double)s.x[1]};
      vp_store<TM>(a, d, lam, info >= 1 && info <= 4, v, nvox, params, auc, ok, auc32);
    }
  };
  refill_loop(r0, r1, &next, init, tick, finish);
}

// Grid of a variable-projection stage: as many blocks as the device holds at once
// (SMs x resident blocks of the kernel, computed once per kernel), each owning an
// equal contiguous range of voxels.
struct VpGrid {
  int blocks;
  long long per_block;
};

inline VpGrid vp_grid(const void* kern, long long n_vox) {
  static std::mutex mu;
  static std::map<const void*, int> wave;
  int slots = 0;
  {
    std::lock_guard<std::mutex> lock(mu);
    auto it = wave.find(kern);
    if (it == wave.end()) {
      int dev = 0, sms = 0, occ = 0;
      if (cudaGetDevice(&dev) != cudaSuccess ||
          cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
          cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, kVpThreads, 0) != cudaSuccess) {
        cudaGetLastError();
        sms = 152, occ = 1;
      }
      it = wave.emplace(kern, std::max(1, sms) * std::max(1, occ)).first;
    }
    slots = it->second;
  }
  const long long nblk = std::max(1LL, std::min<long long>((n_vox + kVpThreads - 1) / kVpThreads, slots));
  const long long per_block = (n_vox + nblk - 1) / nblk;
  return VpGrid{(int)((n_vox + per_block - 1) / per_block), per_block};
}

}  // namespace pvd

using namespace pvd;

extern "C" pvd_status pvd_tac_fit(int model, const double* times, const double* weights, int n_times,
                                  const double* p0, double lam_phys, double auc_limit, int max_fev, int flags,
                                  const float* acts_d, long long n_vox, double* params_d, double* auc_d,
                                  unsigned char* ok_d, float* auc_f32_d, double auc_f32_scale, pvd_stream stream) {
  if (!times || !acts_d || !params_d || !auc_d) return set_error(PVD_ERR_ARG, "pvd_tac_fit: null argument");
  if (n_times < 1 || n_times > PVD_MAX_TIMEPOINTS) return set_error(PVD_ERR_ARG, "pvd_tac_fit: n_times must be in [1, 16]");
  if (n_vox < 0) return set_error(PVD_ERR_ARG, "pvd_tac_fit: negative voxel count");
  if (model < 0 || model > M_LM_TRI) return set_error(PVD_ERR_ARG, "pvd_tac_fit: unknown model");
  if (model != M_MONO_LAMBDA && !p0) return set_error(PVD_ERR_ARG, "pvd_tac_fit: p0 required for this model");
  if (max_fev < 1) return set_error(PVD_ERR_ARG, "pvd_tac_fit: max_fev must be >= 1");
  if (n_vox == 0) return PVD_OK;
  FitArgs a;
  a.T = n_times;
  for (int k = 0; k < n_times; ++k) {
    a.t[k] = times[k];
    a.w[k] = weights ? weights[k] : 1.0;
    a.tf[k] = (float)a.t[k];
    a.wf[k] = (float)a.w[k];
  }
  a.lam_phys_f = (float)lam_phys;
  for (int i = 0; i < 5; ++i) a.p0[i] = p0 ? p0[i] : 0.0;
  a.lam_phys = lam_phys;
  a.auc_limit = auc_limit;
  a.max_fev = max_fev;
  a.force_zero_at_t0 = (flags & PVD_FIT_FORCE_ZERO_AT_T0) ? 1 : 0;
  a.p0_from_data = (model == M_MONO_LAMBDA && !(flags & PVD_FIT_P0_GIVEN)) ? 1 : 0;
  a.p0_peel = (flags & PVD_FIT_P0_FROM_DATA) ? 1 : 0;
  a.auc_inf = (flags & PVD_FIT_AUC_INF) ? 1 : 0;
  a.f32_scale = auc_f32_scale;
  a.mixed = (flags & PVD_FIT_MIXED) ? 1 : 0;
  if ((flags & PVD_FIT_P0_FROM_DATA) && model != M_F4A)
    return set_error(PVD_ERR_ARG, "pvd_tac_fit: PVD_FIT_P0_FROM_DATA applies to PVD_FIT_F4A");
  if ((flags & PVD_FIT_AUC_INF) && model != M_MONO_LAMBDA && model != M_F2 && model != M_F4A)
    return set_error(PVD_ERR_ARG, "pvd_tac_fit: PVD_FIT_AUC_INF applies to the mono, f2 and f4a models");
  if ((flags & PVD_FIT_VARPRO) && model != M_F4A)
    return set_error(PVD_ERR_ARG, "pvd_tac_fit: PVD_FIT_VARPRO applies to PVD_FIT_F4A");
  cudaStream_t st = (cudaStream_t)stream;
  const int threads = 128;
  const int blocks = (int)std::min<long long>((n_vox + threads - 1) / threads, 152LL * 64);
  if (flags & PVD_FIT_VARPRO) {
    // blocks own contiguous voxel ranges, one resident wave of them per launch: a block's
    // range ends on its slowest voxel (up to max_fev evaluations on one lane), and a
    // second wave would pay that tail again
    const int pg = (int)std::min<long long>((n_vox + kVpThreads - 1) / kVpThreads, 152LL * 32);
#define PVD_VP_LAUNCH(MV)                                                                                   \
  {                                                                                                         \
    if (a.mixed) {                                                                                          \
      const VpGrid g0 = vp_grid((const void*)k_tac_fit_vp<MV, 0>, n_vox);                                   \
      k_tac_fit_vp<MV, 0><<<g0.blocks, kVpThreads, 0, st>>>(a, acts_d, n_vox, g0.per_block, params_d, auc_d, \
                                                            ok_d, auc_f32_d);                               \
      PVD_LAUNCH_CHECK("k_tac_fit_vp<fp32>");                                                               \
      k_tac_fit_vp_polish<MV><<<pg, kVpThreads, 0, st>>>(a, acts_d, n_vox, params_d, auc_d, ok_d, auc_f32_d); \
      PVD_LAUNCH_CHECK("k_tac_fit_vp_polish");                                                              \
    }                                                                                                       \
    const VpGrid g1 = vp_grid((const void*)k_tac_fit_vp<MV, 1>, n_vox);                                     \
    k_tac_fit_vp<MV, 1><<<g1.blocks, kVpThreads, 0, st>>>(a, acts_d, n_vox, g1.per_block, params_d, auc_d,   \
                                                          ok_d, auc_f32_d);                                 \
    PVD_LAUNCH_CHECK("k_tac_fit_vp<fp64>");                                                                 \
  }
    if (n_times == 4)
      PVD_VP_LAUNCH(M_F4A_VP4)
    else if (n_times <= 6)
      PVD_VP_LAUNCH(M_F4A_VP6)
    else if (n_times <= 8)
      PVD_VP_LAUNCH(M_F4A_VP8)
    else
      PVD_VP_LAUNCH(M_F4A_VP16)
#undef PVD_VP_LAUNCH
    return PVD_OK;
  }
  const long long sblk = std::min<long long>((n_vox + 127) / 128, 152LL * 8);
  const long long s_per = (n_vox + sblk - 1) / sblk;
  const int sgrid = (int)((n_vox + s_per - 1) / s_per);
  switch (model) {
#define PVD_FIT_CASE(M)                                                                                \
  case M:                                                                                              \
    if (a.mixed)                                                                                       \
      k_tac_fit<M><<<blocks, threads, 0, st>>>(a, acts_d, n_vox, params_d, auc_d, ok_d, auc_f32_d);    \
    else                                                                                               \
      k_tac_fit_sched<M><<<sgrid, 128, 0, st>>>(a, acts_d, n_vox, s_per, params_d, auc_d, ok_d, auc_f32_d); \
    break;
    PVD_FIT_CASE(M_MONO_LAMBDA)
    PVD_FIT_CASE(M_F2)
    PVD_FIT_CASE(M_F3)
    PVD_FIT_CASE(M_F3A)
    PVD_FIT_CASE(M_F4A)
    PVD_FIT_CASE(M_F4B)
    PVD_FIT_CASE(M_F4C)
    PVD_FIT_CASE(M_LM_MONO)
    PVD_FIT_CASE(M_LM_BI)
    PVD_FIT_CASE(M_LM_TRI)
#undef PVD_FIT_CASE
  }
  PVD_LAUNCH_CHECK("k_tac_fit");
  return PVD_OK;
}
