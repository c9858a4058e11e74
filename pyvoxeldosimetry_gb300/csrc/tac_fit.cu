// Per-voxel time-activity-curve fits in FP64, one thread per voxel.
//
// Replaces the Python loops over scipy.optimize.curve_fit of
//   TimeCurveFitting.fit_time_activity_curve      (time_integration/curve_fitting.py:19-65)
//   TimeCurveFitting._calculate_accumulated_dose  (curve_fitting.py:74-84)
//   TimeCurveFitting.fit_time_activity_curve_advanced (curve_fitting.py:112-219)
// with the same models, initial guesses, sigma = 1/weight residual scaling,
// failure fallbacks and AUC formulas.  The minimiser is a Levenberg-Marquardt
// iteration with Marquardt's diagonal scaling and an analytic Jacobian (the
// reference's MINPACK lmdif uses forward differences); both converge to the
// same least-squares minimum on well-posed curves.  Non-finite samples or
// fewer samples than parameters are failures, as curve_fit raises for them.
//
// Layout: activities [T][n_vox] float32 (time-major, the stacked maps);
// params [n_par][n_vox] float64; auc [n_vox] float64; ok [n_vox] uint8.
// HBM traffic per voxel: 4T bytes read, 8(n_par+1)+1 bytes written; the
// kernel is FP64-throughput bound (exp and the normal equations per iteration).
#include <algorithm>
#include <cmath>

#include "pvd_common.cuh"

namespace pvd {

enum Model {
  M_MONO_LAMBDA = 0,  // A0 exp(-lam t)                     (fit_time_activity_curve)
  M_F2 = 1, M_F3 = 2, M_F3A = 3, M_F4A = 4, M_F4B = 5, M_F4C = 6,  // NUKFIT
  M_LM_MONO = 7, M_LM_BI = 8, M_LM_TRI = 9                          // "lmfit" table
};

struct FitArgs {
  double t[PVD_MAX_TIMEPOINTS];
  double w[PVD_MAX_TIMEPOINTS];  // residual multipliers (1 / sigma)
  double p0[5];
  int T;
  double lam_phys;               // ln2 / physical half-life (models with lambda_phys)
  double auc_limit;              // mono-lambda model: integration limit (same time unit)
  int max_iter;
  int force_zero_at_t0;
  int p0_from_data;              // mono-lambda: p0 = [y(t0), lam_phys] per voxel
};

template <int M> struct ModelTraits;

#define PVD_LN2 0.69314718055994530942

// value and gradient of each model at time t
template <> struct ModelTraits<M_MONO_LAMBDA> {
  static constexpr int N = 2;
  static __device__ double eval(const double* p, double t, double, double* g) {
    const double e = exp(-p[1] * t);
    g[0] = e;
    g[1] = -t * p[0] * e;
    return p[0] * e;
  }
};
template <> struct ModelTraits<M_F2> {
  static constexpr int N = 2;
  static __device__ double eval(const double* p, double t, double lp, double* g) {
    const double e = exp(-(p[1] + lp) * t);
    g[0] = e;
    g[1] = -t * p[0] * e;
    return p[0] * e;
  }
};
template <> struct ModelTraits<M_F3> {
  static constexpr int N = 3;
  static __device__ double eval(const double* p, double t, double lp, double* g) {
    const double e1 = exp(-(p[1] + lp) * t), e2 = exp(-(p[2] + lp) * t);
    g[0] = e1 - e2;
    g[1] = -t * p[0] * e1;
    g[2] = t * p[0] * e2;
    return p[0] * (e1 - e2);
  }
};
template <> struct ModelTraits<M_F3A> {
  static constexpr int N = 3;
  static __device__ double eval(const double* p, double t, double lp, double* g) {
    const double e1 = exp(-(p[2] + lp) * t), ep = exp(-lp * t);
    g[0] = p[1] * e1 + (1 - p[1]) * ep;
    g[1] = p[0] * (e1 - ep);
    g[2] = -t * p[0] * p[1] * e1;
    return p[0] * (p[1] * e1 + (1 - p[1]) * ep);
  }
};
template <> struct ModelTraits<M_F4A> {
  static constexpr int N = 4;
  static __device__ double eval(const double* p, double t, double lp, double* g) {
    const double e1 = exp(-(p[1] + lp) * t), e2 = exp(-(p[3] + lp) * t);
    g[0] = e1;
    g[1] = -t * p[0] * e1;
    g[2] = e2;
    g[3] = -t * p[2] * e2;
    return p[0] * e1 + p[2] * e2;
  }
};
template <> struct ModelTraits<M_F4B> {
  static constexpr int N = 5;
  static __device__ double eval(const double* p, double t, double lp, double* g) {
    const double e1 = exp(-(p[1] + lp) * t), e2 = exp(-(p[3] + lp) * t), eb = exp(-(p[4] + lp) * t);
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
  static __device__ double eval(const double* p, double t, double lp, double* g) {
    const double e1 = exp(-(p[1] + lp) * t), e2 = exp(-(p[3] + lp) * t), eb = exp(-(p[4] + lp) * t);
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
  static __device__ double eval(const double* p, double t, double, double* g) {
    const double e = exp(-PVD_LN2 * t / p[1]);
    g[0] = e;
    g[1] = p[0] * e * PVD_LN2 * t / (p[1] * p[1]);
    return p[0] * e;
  }
};
template <> struct ModelTraits<M_LM_BI> {
  static constexpr int N = 3;
  static __device__ double eval(const double* p, double t, double, double* g) {
    const double e1 = exp(-PVD_LN2 * t / p[1]), e2 = exp(-PVD_LN2 * t / p[2]);
    g[0] = e1 - e2;
    g[1] = p[0] * e1 * PVD_LN2 * t / (p[1] * p[1]);
    g[2] = -p[0] * e2 * PVD_LN2 * t / (p[2] * p[2]);
    return p[0] * (e1 - e2);
  }
};
template <> struct ModelTraits<M_LM_TRI> {
  static constexpr int N = 5;
  static __device__ double eval(const double* p, double t, double, double* g) {
    const double e1 = exp(-PVD_LN2 * t / p[1]), e2 = exp(-PVD_LN2 * t / p[3]), e3 = exp(-PVD_LN2 * t / p[4]);
    g[0] = e1 - e3;
    g[1] = p[0] * e1 * PVD_LN2 * t / (p[1] * p[1]);
    g[2] = -e2 + e3;
    g[3] = -p[2] * e2 * PVD_LN2 * t / (p[3] * p[3]);
    g[4] = -(p[0] - p[2]) * e3 * PVD_LN2 * t / (p[4] * p[4]);
    return p[0] * e1 - p[2] * e2 - (p[0] - p[2]) * e3;
  }
};

// normal equations at p: A = J^T J (upper triangle), g = J^T r, returns 0.5 r^T r
template <int M>
__device__ double normal_eq(const FitArgs& a, const double* y, const double* p, double* A, double* g) {
  constexpr int N = ModelTraits<M>::N;
#pragma unroll
  for (int i = 0; i < N * N; ++i) A[i] = 0.0;
#pragma unroll
  for (int i = 0; i < N; ++i) g[i] = 0.0;
  double cost = 0.0;
  for (int k = 0; k < a.T; ++k) {
    double j[N];
    const double f = ModelTraits<M>::eval(p, a.t[k], a.lam_phys, j);
    const double r = a.w[k] * (f - y[k]);
#pragma unroll
    for (int i = 0; i < N; ++i) j[i] *= a.w[k];
#pragma unroll
    for (int i = 0; i < N; ++i) {
      g[i] += j[i] * r;
#pragma unroll
      for (int c = i; c < N; ++c) A[i * N + c] += j[i] * j[c];
    }
    cost += r * r;
  }
  return 0.5 * cost;
}

template <int M>
__device__ double cost_at(const FitArgs& a, const double* y, const double* p) {
  constexpr int N = ModelTraits<M>::N;
  double cost = 0.0;
  for (int k = 0; k < a.T; ++k) {
    double j[N];
    const double r = a.w[k] * (ModelTraits<M>::eval(p, a.t[k], a.lam_phys, j) - y[k]);
    cost += r * r;
  }
  return 0.5 * cost;
}

// solve (A + mu diag(A)) h = -g by Cholesky (A symmetric, upper triangle stored); false if not SPD
template <int N>
__device__ bool damped_solve(const double* A, const double* g, double mu, double* h) {
  double L[N * N];
#pragma unroll
  for (int i = 0; i < N; ++i) {
#pragma unroll
    for (int c = 0; c <= i; ++c) {
      double s = (c == i) ? A[i * N + i] * (1.0 + mu) + 1e-300 : A[c * N + i];
      for (int k = 0; k < c; ++k) s -= L[i * N + k] * L[c * N + k];
      if (c == i) {
        if (!(s > 0.0)) return false;
        L[i * N + i] = sqrt(s);
      } else {
        L[i * N + c] = s / L[c * N + c];
      }
    }
  }
  double z[N];
#pragma unroll
  for (int i = 0; i < N; ++i) {
    double s = -g[i];
    for (int k = 0; k < i; ++k) s -= L[i * N + k] * z[k];
    z[i] = s / L[i * N + i];
  }
#pragma unroll
  for (int i = N - 1; i >= 0; --i) {
    double s = z[i];
    for (int k = i + 1; k < N; ++k) s -= L[k * N + i] * h[k];
    h[i] = s / L[i * N + i];
  }
  return true;
}

// Levenberg-Marquardt from p (in/out); returns true on convergence.
template <int M>
__device__ bool lm_fit(const FitArgs& a, const double* y, double* p) {
  constexpr int N = ModelTraits<M>::N;
  double A[N * N], g[N], h[N], pn[N];
  double F = normal_eq<M>(a, y, p, A, g);
  if (!isfinite(F)) return false;
  double mu = 1e-3;
  double nu = 2.0;
  for (int it = 0; it < a.max_iter; ++it) {
    double gmax = 0.0, dmax = 0.0;
#pragma unroll
    for (int i = 0; i < N; ++i) {
      gmax = fmax(gmax, fabs(g[i]));
      dmax = fmax(dmax, A[i * N + i]);
    }
    if (F == 0.0 || gmax == 0.0) return true;   // exact fit / stationary point
    if (!damped_solve<N>(A, g, mu, h)) {
      mu *= nu;
      nu *= 2.0;
      if (mu > 1e30) return false;
      continue;
    }
    double hn = 0.0, pnrm = 0.0;
#pragma unroll
    for (int i = 0; i < N; ++i) {
      pn[i] = p[i] + h[i];
      hn += h[i] * h[i];
      pnrm += p[i] * p[i];
    }
    if (sqrt(hn) <= 1e-15 * (sqrt(pnrm) + 1e-300)) return true;
    const double Fn = cost_at<M>(a, y, pn);
    // predicted reduction of the damped quadratic model: 0.5 h^T (mu D h - g)
    double pred = 0.0;
#pragma unroll
    for (int i = 0; i < N; ++i) pred += h[i] * (mu * A[i * N + i] * h[i] - g[i]);
    pred *= 0.5;
    const double rho = (F - Fn) / pred;
    if (isfinite(Fn) && Fn < F && pred > 0.0) {
      const double rel = (F - Fn) / F;
#pragma unroll
      for (int i = 0; i < N; ++i) p[i] = pn[i];
      const double Fold = F;
      F = normal_eq<M>(a, y, p, A, g);
      const double t = 2.0 * rho - 1.0;
      mu *= fmax(1.0 / 3.0, 1.0 - t * t * t);
      nu = 2.0;
      if (rel <= 1e-15 || Fold - F <= 1e-15 * Fold) return true;
    } else {
      mu *= nu;
      nu *= 2.0;
      if (mu > 1e30) return true;  // no further decrease possible: at the minimum to working precision
    }
  }
  return false;
}

template <int M>
__global__ void k_tac_fit(FitArgs a, const float* __restrict__ acts, long long nvox, double* __restrict__ params,
                          double* __restrict__ auc, unsigned char* __restrict__ ok) {
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
    bool good = finite && a.T >= N && lm_fit<M>(a, y, p);
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
    double s;
    if (M == M_MONO_LAMBDA) {
      // A0 / lam * (1 - exp(-lam * limit))  (curve_fitting.py:74-84)
      s = p[0] / p[1] * (1.0 - exp(-p[1] * a.auc_limit));
    } else {
      // trapezoid of the fitted curve over the sampled times (curve_fitting.py:215)
      double j[N];
      s = 0.0;
      double fprev = ModelTraits<M>::eval(p, a.t[0], a.lam_phys, j);
      for (int k = 1; k < a.T; ++k) {
        const double f = ModelTraits<M>::eval(p, a.t[k], a.lam_phys, j);
        s += 0.5 * (f + fprev) * (a.t[k] - a.t[k - 1]);
        fprev = f;
      }
    }
    auc[v] = s;
    if (ok) ok[v] = good ? 1 : 0;
  }
}

}  // namespace pvd

using namespace pvd;

extern "C" pvd_status pvd_tac_fit(int model, const double* times, const double* weights, int n_times,
                                  const double* p0, double lam_phys, double auc_limit, int max_iter, int flags,
                                  const float* acts_d, long long n_vox, double* params_d, double* auc_d,
                                  unsigned char* ok_d, pvd_stream stream) {
  if (!times || !acts_d || !params_d || !auc_d) return set_error(PVD_ERR_ARG, "pvd_tac_fit: null argument");
  if (n_times < 1 || n_times > PVD_MAX_TIMEPOINTS) return set_error(PVD_ERR_ARG, "pvd_tac_fit: n_times must be in [1, 16]");
  if (n_vox < 0) return set_error(PVD_ERR_ARG, "pvd_tac_fit: negative voxel count");
  if (model < 0 || model > M_LM_TRI) return set_error(PVD_ERR_ARG, "pvd_tac_fit: unknown model");
  if (model != M_MONO_LAMBDA && !p0) return set_error(PVD_ERR_ARG, "pvd_tac_fit: p0 required for this model");
  if (max_iter < 1) return set_error(PVD_ERR_ARG, "pvd_tac_fit: max_iter must be >= 1");
  if (n_vox == 0) return PVD_OK;
  FitArgs a;
  a.T = n_times;
  for (int k = 0; k < n_times; ++k) {
    a.t[k] = times[k];
    a.w[k] = weights ? weights[k] : 1.0;
  }
  for (int i = 0; i < 5; ++i) a.p0[i] = p0 ? p0[i] : 0.0;
  a.lam_phys = lam_phys;
  a.auc_limit = auc_limit;
  a.max_iter = max_iter;
  a.force_zero_at_t0 = (flags & PVD_FIT_FORCE_ZERO_AT_T0) ? 1 : 0;
  a.p0_from_data = (model == M_MONO_LAMBDA && !(flags & PVD_FIT_P0_GIVEN)) ? 1 : 0;
  cudaStream_t st = (cudaStream_t)stream;
  const int threads = 128;
  const int blocks = (int)std::min<long long>((n_vox + threads - 1) / threads, 152LL * 64);
  switch (model) {
#define PVD_FIT_CASE(M)                                                                    \
  case M:                                                                                  \
    k_tac_fit<M><<<blocks, threads, 0, st>>>(a, acts_d, n_vox, params_d, auc_d, ok_d);    \
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
