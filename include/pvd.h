/*
 * pvd.h — C ABI of the GB300 (sm_103a) voxel-dosimetry hot path.
 *
 * Plain pointers, sizes and status codes only: no torch or CUDA types in the
 * signatures (`pvd_stream` is ABI-identical to `cudaStream_t`).  Every device
 * pointer argument must point to memory of the current CUDA device.  All calls
 * return a `pvd_status`; on failure a message is available from
 * `pvd_last_error` (thread-local).  No call aborts, traps or exits the process.
 *
 * Reference interfaces these entry points replace (devhliu/PyVoxelDosimetry,
 * paths within that project):
 *   - pvd_plan_create / pvd_plan_set_kernel:
 *       KernelConvolutionCalculator.__init__/_load_dose_kernel
 *       (pyvoxeldosimetry/core/kernel_convolution.py:27-46) and
 *       KernelFactory.get_kernel (data/dose_kernels/kernel_factory.py:37-75).
 *   - pvd_conv_execute:
 *       KernelConvolutionCalculator.calculate_dose_rate
 *       (pyvoxeldosimetry/core/kernel_convolution.py:48-76), the numpy
 *       `ifftn(fftn(A) * fftn(K, A.shape)).real` at :71-74; plus the density
 *       hook `tissue_densities` of DoseCalculator.calculate_dose
 *       (core/dose_calculator.py:90), which the reference accepts and ignores.
 *   - pvd_conv_execute_weighted:
 *       the trapezoid of ActivitySampler._trapezoid_integration
 *       (core/activity_sampler.py:69-78) and of
 *       KernelConvolutionCalculator.calculate_absorbed_dose
 *       (core/kernel_convolution.py:99-104), folded into the first pass.
 *   - pvd_tac_fit_mono / pvd_tac_fit_model:
 *       TimeCurveFitting.fit_time_activity_curve + _calculate_accumulated_dose
 *       (time_integration/curve_fitting.py:19-84) and
 *       fit_time_activity_curve_advanced (curve_fitting.py:112-219).
 *   - pvd_mc_run:
 *       MonteCarloCalculator.calculate_dose_rate (core/monte_carlo.py:104-137).
 */
#ifndef PVD_H_
#define PVD_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct CUstream_st* pvd_stream; /* == cudaStream_t; NULL = legacy default stream */

typedef enum {
  PVD_OK = 0,
  PVD_ERR_ARG = 1,         /* invalid argument (shape, pointer, flag) */
  PVD_ERR_CUDA = 2,        /* a CUDA runtime call failed */
  PVD_ERR_OOM = 3,         /* device allocation failed */
  PVD_ERR_TIMEOUT = 4,     /* a bounded device wait ran out */
  PVD_ERR_NUMERIC = 5,     /* non-finite or degenerate numeric input */
  PVD_ERR_UNSUPPORTED = 6, /* size / mode outside what the plan supports */
  PVD_ERR_STATE = 7        /* call order violated (e.g. kernel slot not set) */
} pvd_status;

/* ------------------------------------------------------------------------ */
/* Dose-point-kernel FFT convolution                                          */
/* ------------------------------------------------------------------------ */

/* Convolution semantics.
 *   PVD_MODE_LINEAR  : zero-padded linear convolution cropped to the input
 *                      grid ("same"), kernel centred at index k//2 per axis.
 *                      Equal to the reference operator applied to inputs
 *                      zero-padded to P >= N+K-1 and cropped at offset k//2.
 *   PVD_MODE_CIRCULAR: exactly the reference operator
 *                      ifftn(fftn(A) * fftn(K, A.shape)).real: circular,
 *                      unpadded, kernel placed at the array corner and
 *                      truncated to the volume shape where it is larger
 *                      (output shifted by k//2 relative to LINEAR).  Any
 *                      volume shape: an axis whose length n is 7-smooth is
 *                      transformed at length n; any other axis at a zero-
 *                      padded length P >= 2n with a second copy of the kernel
 *                      at offset P - n, which yields the same period-n
 *                      convolution (pad[i] may give n or a length >= 2n). */
enum { PVD_MODE_LINEAR = 0, PVD_MODE_CIRCULAR = 1 };

/* pvd_conv_desc flags */
enum {
  PVD_PLAN_TMA = 1 /* stage the column passes' tiles with TMA bulk tensor loads (persistent,
                      double-buffered); default: tiles loaded straight into registers */
};

/* pvd_plan_set_kernel flags */
enum {
  PVD_KERNEL_NORMALIZE = 1 /* divide the kernel by its FP64 sum (on the GPU) */
};

#define PVD_MAX_KERNELS 8
#define PVD_MAX_TIMEPOINTS 16

typedef struct {
  int n[3];           /* volume dims, slowest..fastest (C order of the numpy array) */
  int kmax[3];        /* largest kernel dims this plan will accept (LINEAR: sets padding) */
  int mode;           /* PVD_MODE_* */
  int n_kernels;      /* number of kernel slots (nuclides) sharing one forward transform */
  int pad[3];         /* explicit FFT lengths; 0 = choose automatically */
  int flags;          /* PVD_PLAN_* */
} pvd_conv_desc;

typedef struct {
  int n[3];
  int p[3];           /* FFT lengths actually used */
  int h;              /* p[2]/2+1 complex bins on the fastest axis */
  int hs;             /* row stride (complex) of the spectral buffers */
  int n_kernels;
  size_t workspace_bytes;  /* device bytes owned by the plan (buffers + spectra) */
} pvd_plan_info;

typedef struct pvd_plan pvd_plan;

/* Create a plan on the current device; allocates its workspace with cudaMalloc. */
pvd_status pvd_plan_create(const pvd_conv_desc* desc, pvd_plan** out);

/* Query sizes of a plan. */
pvd_status pvd_plan_get_info(const pvd_plan* plan, pvd_plan_info* info);

/* Load kernel `slot` from a host FP64 array (C order, dims k0,k1,k2).  The
 * kernel is copied to the device, optionally normalised by its FP64 sum on the
 * GPU, multiplied by `scale`, and transformed to the padded spectrum (FP32).
 * Synchronous with respect to the host.  Radially symmetric kernels in LINEAR
 * mode are stored as a real spectrum; any other kernel as a complex one. */
pvd_status pvd_plan_set_kernel(pvd_plan* plan, int slot, const double* kernel_host,
                               int k0, int k1, int k2, double scale, int flags);

/* dose[s] = out_scale * (activity (*) kernel[s]) / rho   for every slot s.
 *   activity_d : device float32 [n0*n1*n2]
 *   density_d  : device float32 [n0*n1*n2] or NULL (rho == 1); voxels with
 *                rho <= 0 (or NaN) get dose 0
 *   dose_d     : device float32 [n_kernels][n0*n1*n2] (slot-major)
 * Enqueued on `stream`; returns once queued. */
pvd_status pvd_conv_execute(pvd_plan* plan, const float* activity_d, const float* density_d,
                            float* dose_d, float out_scale, pvd_stream stream);

/* pvd_conv_execute with HOST buffers: activity_h / density_h (nullable) /
 * dose_h are host float32 arrays of the sizes above.  The plan stages them in
 * device buffers it owns and pipelines the copies with the passes: the
 * activity goes up in z chunks that each release their share of the forward
 * passes, the density goes up during the z pass, and the inverse x pass runs in
 * z chunks whose dose (every slot's) goes back while the next chunk computes.  Returns once queued; the copies back
 * are complete when `stream` is (cudaStreamSynchronize).  Page-locked host
 * memory makes the copies asynchronous; pageable memory works but copies
 * synchronously. */
pvd_status pvd_conv_execute_host(pvd_plan* plan, const float* activity_h, const float* density_h,
                                 float* dose_h, float out_scale, pvd_stream stream);

/* As pvd_conv_execute with activity = sum_t weights[t] * activity_d[t]
 * (t < n_act <= PVD_MAX_TIMEPOINTS), the weighted sum fused into the first
 * pass (trapezoid time integration without an extra pass over the volume). */
pvd_status pvd_conv_execute_weighted(pvd_plan* plan, const float* const* activity_d,
                                     const float* weights, int n_act, const float* density_d,
                                     float* dose_d, float out_scale, pvd_stream stream);

pvd_status pvd_plan_destroy(pvd_plan* plan);

/* Device-side status of the plan's passes: PVD_ERR_TIMEOUT if a TMA tile load
 * of a column pass did not complete within its bounded wait (the pass then
 * left its tiles unwritten); PVD_OK otherwise.  A failure is reported once: the
 * status word is cleared when it is read.  Synchronises with the device. */
pvd_status pvd_plan_status(const pvd_plan* plan);

/* Allocation-free convolution.  No counterpart in the reference.
 *
 * For callers that cannot allocate device memory themselves or let a library
 * do it (a host framework that owns the device allocator and its budget, a
 * plugin that must not call cudaMalloc/cudaFree because they synchronise the
 * device, code that must not grow the process's footprint per call).  It runs
 * the pvd_conv_execute pipeline (LINEAR mode, one kernel, density optional)
 * with every temporary (twiddles, kernel staging, spectrum, spectral work
 * buffers) placed in one static device array of PVD_STATIC_SCRATCH_BYTES that
 * each GPU loading this library holds until the process exits.  The caller
 * passes the inputs (device activity/density, host FP64 kernel) and the output
 * (device dose); nothing is allocated.  Volumes whose scratch would exceed the
 * array (about 128^3 with a 15^3 kernel fits) are rejected with
 * PVD_ERR_UNSUPPORTED and a message giving the bytes needed.
 *
 * The first call on a device looks up the array's device address
 * (cudaGetSymbolAddress, with that device current) and caches it for the life
 * of the process; make that first call before any stream capture, and do not
 * use this entry point across a cudaDeviceReset (or any destruction of the
 * device's primary context), after which the cached address is stale.  Every
 * call uses the same array: calls that can overlap on the GPU (other streams,
 * other host threads) race and must be serialised by the caller.  The kernel
 * upload is a plain host-to-device copy on `stream` from the caller's
 * `kernel_h`.  With PVD_KERNEL_NORMALIZE a kernel whose sum is zero or not
 * finite is rejected with PVD_ERR_NUMERIC, as pvd_plan_set_kernel does. */
#define PVD_STATIC_SCRATCH_BYTES (64ull << 20)
#define PVD_STATIC_MAX_DEVICES 64
pvd_status pvd_conv_execute_static(const float* activity_d, const float* density_d, float* dose_d,
                                   int n0, int n1, int n2, const double* kernel_h, int k0, int k1, int k2,
                                   double scale, int flags, float out_scale, pvd_stream stream);

/* FFT lengths that have register-resident (four-step) pass kernels; LINEAR
 * plans pad to one of them when it costs <= 25 % over the minimum.  Writes up
 * to `cap` lengths (ascending) and returns how many exist. */
int pvd_fast_lengths(int* out, int cap);

/* Per-pass timing (instrumentation; not part of the reference interface).
 * pvd_plan_profile(plan, 1) resets the records and brackets every later pass
 * launch of this plan with CUDA events on its stream; pvd_plan_pass_times
 * waits for the recorded events and returns, per pass kind, the summed
 * milliseconds and the number of launches:
 *   0 x-forward (R2C), 1 y-forward, 2 z (forward * spectrum * inverse),
 *   3 y-inverse, 4 x-inverse (C2R, crop, scale, density). */
#define PVD_NUM_PASSES 5
pvd_status pvd_plan_profile(pvd_plan* plan, int enable);
pvd_status pvd_plan_pass_times(pvd_plan* plan, double* ms, int* launches);

/* ------------------------------------------------------------------------ */
/* Time integration                                                           */
/* ------------------------------------------------------------------------ */

/* out[i] = sum_t weights[t] * maps[t][i] over n_voxels float32 voxels (device
 * pointers, t < n_maps <= PVD_MAX_TIMEPOINTS).  With trapezoid weights this is
 * ActivitySampler._trapezoid_integration (core/activity_sampler.py:69-78). */
pvd_status pvd_weighted_sum(const float* const* maps, const float* weights, int n_maps,
                            long long n_voxels, float* out, pvd_stream stream);

/* Per-voxel time-activity-curve fit (FP64, one thread per voxel).
 * Models (the reference's curve_fitting.py):
 *   PVD_FIT_MONO_LAMBDA  A0 exp(-lam t), p = [A0, lam]; p0 = [y(t0), lam_phys]
 *                        unless PVD_FIT_P0_GIVEN; failure -> [0, lam_phys];
 *                        auc = A0/lam (1 - exp(-lam auc_limit))      (:19-84)
 *   PVD_FIT_F2..F4C      NUKFIT f2, f3, f3a, f4a, f4b, f4c (lam_phys added to
 *                        every rate), PVD_FIT_LM_MONO/BI/TRI the "lmfit" table;
 *                        p0 required; failure -> zeros; auc = trapezoid of the
 *                        fitted curve over the sampled times              (:112-219)
 * Residuals are weights[k] * (f(t_k) - y_k) (curve_fit with sigma = 1/weights;
 * weights may be NULL = 1).  acts_d: device float32 [n_times][n_vox];
 * params_d: device float64 [n_par][n_vox]; auc_d: device float64 [n_vox];
 * ok_d: device uint8 [n_vox] (1 = converged) or NULL.  The minimiser is
 * Moré's scaled trust-region Levenberg-Marquardt (the algorithm of MINPACK
 * lmdif, which curve_fit runs); max_fev is curve_fit's maxfev (model
 * evaluations, a Jacobian counting n_par of them) and, as there, running out
 * of it or of attainable precision is a failure. */
enum {
  PVD_FIT_MONO_LAMBDA = 0, PVD_FIT_F2 = 1, PVD_FIT_F3 = 2, PVD_FIT_F3A = 3, PVD_FIT_F4A = 4,
  PVD_FIT_F4B = 5, PVD_FIT_F4C = 6, PVD_FIT_LM_MONO = 7, PVD_FIT_LM_BI = 8, PVD_FIT_LM_TRI = 9
};
/* Flags.  PVD_FIT_P0_FROM_DATA (f4a only): start from exponential peeling of
 * each voxel's samples instead of p0.  PVD_FIT_AUC_INF (mono, f2, f4a): the
 * AUC is the fitted curve's integral from 0 to infinity (all rates must come out
 * positive, the f4a curve non-negative on [0, inf) and at t = 0 at most 100
 * times the largest sample, and the integral finite;
 * otherwise the voxel is marked not ok and the model's own AUC rule is used).  PVD_FIT_MIXED runs the iterations in FP32, then the same minimiser
 * again in FP64 from where they stopped, with at most 60 evaluations; success
 * is decided by the FP64 run's convergence tests alone.  With PVD_FIT_VARPRO
 * the FP64 run starts with at most three Gauss-Newton steps from the FP32
 * rates; a voxel whose curve then reproduces its float32 samples to their
 * rounding (the FP64 run's own stopping test) is done, and only the others go
 * through the FP64 trust-region iteration.  PVD_FIT_VARPRO (f4a only) minimises the same
 * least-squares cost by variable projection: the two amplitudes are solved
 * linearly for given rates and the trust-region iteration runs over the two
 * rates only, which converges where the four-parameter iteration stalls in the
 * valley of nearly equal rates; params are ordered fast rate first.
 * None of these exists in the reference; they serve the time-integrated dose
 * of a whole batch of volumes.  auc_f32_d (nullable) receives
 * float(auc * auc_f32_scale), e.g. cumulated activity in Bq s for a convolution;
 * a value that is not finite in float32 is stored as 0 with the voxel not ok. */
enum {
  PVD_FIT_FORCE_ZERO_AT_T0 = 1,
  PVD_FIT_P0_GIVEN = 2,
  PVD_FIT_P0_FROM_DATA = 4,
  PVD_FIT_AUC_INF = 8,
  PVD_FIT_MIXED = 16, /* FP32 iterations, FP64 finish (GB300's FP64 rate is a small fraction of FP32's) */
  PVD_FIT_VARPRO = 32
};
pvd_status pvd_tac_fit(int model, const double* times, const double* weights, int n_times,
                       const double* p0, double lam_phys, double auc_limit, int max_fev, int flags,
                       const float* acts_d, long long n_vox, double* params_d, double* auc_d,
                       unsigned char* ok_d, float* auc_f32_d, double auc_f32_scale, pvd_stream stream);

/* ------------------------------------------------------------------------ */
/* Monte Carlo transport                                                      */
/* ------------------------------------------------------------------------ */

/* One thread per decay history: decays sampled in proportion to the activity
 * (voxel by an integer prefix sum, uniform position inside it), one beta with
 * probability beta_yield (energy from the inverse-CDF table) and each gamma line
 * with its yield, isotropic.  Electrons: continuous slowing down along voxel-
 * bounded steps (<= 1/4 of the residual CSDA range), range table scaled by the
 * local density, Highland multiple scattering in water.  Photons: Woodcock
 * tracking with the total mass attenuation table, absorption or Compton
 * (Klein-Nishina, Kahn's method) with the electron deposited locally.  Energy
 * is scored in unsigned 64-bit fixed point, 2^-32 MeV per unit, so results are
 * bit-reproducible for a given seed.  Tables are uniform in energy:
 * E_i = i * de.  Replaces MonteCarloCalculator (core/monte_carlo.py:10-172). */
#define PVD_MC_MAX_GAMMA 8
typedef struct {
  int n[3];                  /* volume dims (C order) */
  double voxel_mm[3];        /* voxel size per axis (mm) */
  const float* beta_icdf;    /* host: beta energy (MeV) at u = i/(n_beta-1) */
  int n_beta;
  const float* range;        /* host: electron CSDA range in water (g/cm^2) at E_i */
  int n_range;
  float range_de;
  const float* mu_rho;       /* host: photon total mass attenuation of water (cm^2/g) at E_i */
  const float* compton_frac; /* host: Compton share of mu_rho at E_i */
  int n_photon;
  float photon_de;
  int n_gamma;
  float gamma_e[PVD_MC_MAX_GAMMA];      /* MeV */
  float gamma_yield[PVD_MC_MAX_GAMMA];  /* photons per decay (<= 1) */
  float beta_yield;          /* betas per decay (<= 1) */
  float e_cut;               /* MeV: particles below it deposit locally */
} pvd_mc_desc;

typedef struct {
  unsigned long long total_weight;  /* sum of the fixed-point source weights */
  unsigned long long emitted;       /* emitted energy, 2^-32 MeV units */
  unsigned long long escaped;       /* energy leaving the volume, 2^-32 MeV units */
  unsigned long long steps;         /* transport steps taken */
  double activity_bq;               /* activity the histories represent (sum of the map) */
} pvd_mc_stats;

typedef struct pvd_mc_plan pvd_mc_plan;

/* Copy the tables to the device and allocate the source-sampling workspace. */
pvd_status pvd_mc_plan_create(const pvd_mc_desc* desc, pvd_mc_plan** out);

/* Run n_histories decays with Philox4x32-10 stream `seed`.
 *   activity_d : device float32 [n] (Bq per voxel; <= 0 and NaN count as 0)
 *   density_d  : device float32 [n] g/cc or NULL (water)
 *   edep_d     : device uint64 [n], zeroed then filled with deposited energy
 *   dose_rate_d: device float32 [n] or NULL: Gy/s = E / n_histories * activity
 *                * 1.602176634e-13 J/MeV / voxel mass (0 where density <= 0)
 *   stats      : host or NULL; when given, the call waits for the stream. */
pvd_status pvd_mc_run(pvd_mc_plan* plan, const float* activity_d, const float* density_d,
                      unsigned long long n_histories, unsigned long long seed,
                      unsigned long long* edep_d, float* dose_rate_d, pvd_mc_stats* stats,
                      pvd_stream stream);

pvd_status pvd_mc_plan_destroy(pvd_mc_plan* plan);

/* ------------------------------------------------------------------------ */
/* Batched time-integrated dose                                               */
/* ------------------------------------------------------------------------ */

/* One volume of a batch: n_times activity maps at their times, fitted per
 * voxel with the two-exponential model f4a from an exponential-peeling start
 * (pvd_tac_fit with PVD_FIT_P0_FROM_DATA | PVD_FIT_AUC_INF and the caller's
 * flags), the fit's integral from 0 to infinity times time_scale (e.g. 3600
 * for hours -> seconds) as float32 cumulated activity in cum_d, and that
 * convolved with every kernel slot of the plan into dose_d (pvd_conv_execute,
 * density-scaled when density_d is given).  The reference computes this one
 * volume at a time on the CPU: core/dose_calculator.py:85-164 with
 * time_integration/curve_fitting.py:112-219 and core/kernel_convolution.py:48-106. */
typedef struct {
  pvd_plan* plan;               /* plan of this volume's shape; items may share a plan */
  const float* activity_d;      /* device float32 [n_times][n_vox] */
  const double* times;          /* host, n_times entries (read during the call) */
  int n_times;                  /* 4 .. PVD_MAX_TIMEPOINTS */
  const float* density_d;       /* device float32 [n_vox] or NULL */
  double* params_d;             /* device float64 [4][n_vox] */
  double* auc_d;                /* device float64 [n_vox] */
  unsigned char* ok_d;          /* device uint8 [n_vox] or NULL */
  float* cum_d;                 /* device float32 [n_vox] */
  float* dose_d;                /* device float32 [n_kernels][n_vox] */
} pvd_batch_item;

/* Enqueue every item on `stream`, item by item (fit, then convolution).
 * fit_flags: further PVD_FIT_* flags (PVD_FIT_VARPRO, PVD_FIT_MIXED);
 * max_fev: the fit's evaluation budget per voxel.  All items are validated
 * before anything is enqueued.  May be recorded into a CUDA graph. */
pvd_status pvd_batch_execute(const pvd_batch_item* items, int n_items, int fit_flags, int max_fev,
                             double time_scale, pvd_stream stream);

typedef struct pvd_batch pvd_batch;

/* Run pvd_batch_execute of these items once on a private stream (loading every
 * kernel it uses), then record it into a CUDA graph owned by the returned
 * handle.  The items' buffers and plans must outlive the handle; their
 * contents may change between runs. */
pvd_status pvd_batch_create(const pvd_batch_item* items, int n_items, int fit_flags, int max_fev,
                            double time_scale, pvd_batch** out);

/* Launch the recorded graph on `stream`: the whole batch in one launch. */
pvd_status pvd_batch_run(pvd_batch* batch, pvd_stream stream);

pvd_status pvd_batch_destroy(pvd_batch* batch);

/* ------------------------------------------------------------------------ */
/* Dose-volume histogram                                                      */
/* ------------------------------------------------------------------------ */

/* Replaces calculate_dvh (core/utils.py:233-262): np.histogram(dose[mask > 0],
 * bins) with uniform bins between the ROI's minimum and maximum, then
 * 1 - cumsum(hist) / n.  The device computes the ROI statistics and the
 * counts; the caller computes the edges exactly as numpy does
 * (np.linspace(first, last, bins + 1) in the dose's type, after widening an
 * empty range by 0.5 on each side) and the cumulative sum.  The bin of every
 * dose follows numpy's arithmetic for uniform bins operation for operation,
 * so the counts equal np.histogram's.
 * dose_d: device float32 or float64 [n]; mask_d: device uint8 or float32 [n]
 * (voxels with mask > 0), or NULL for every voxel. */
enum { PVD_DTYPE_U8 = 0, PVD_DTYPE_F32 = 1, PVD_DTYPE_F64 = 2 };
typedef struct {
  double min, max;       /* of the finite ROI doses (exact in the dose's type) */
  long long count;       /* ROI voxels */
  long long nonfinite;   /* ROI voxels whose dose is NaN or infinite */
} pvd_roi_stats_t;

/* ROI statistics; synchronises `stream` and fills *out. */
pvd_status pvd_roi_stats(const void* dose_d, int dose_dtype, const void* mask_d, int mask_dtype, long long n,
                         pvd_roi_stats_t* out, pvd_stream stream);

/* counts_d[b] (device int64 [bins], overwritten) = ROI doses in bin b of the
 * edges edges_d (device, dose type, bins + 1 values); doses outside
 * [edges[0], edges[bins]] are not counted.  Enqueued on `stream`. */
pvd_status pvd_histogram(const void* dose_d, int dose_dtype, const void* mask_d, int mask_dtype, long long n,
                         const void* edges_d, int bins, long long* counts_d, pvd_stream stream);

/* Both steps without a host round trip: ROI statistics, numpy's edges computed on
 * the device (np.linspace(first, last, bins + 1) restated operation for operation),
 * counts.  result_d: device int64 [4 + bins] = [min key, max key, ROI count,
 * non-finite ROI count, counts...]; the keys are the doses' bit patterns made
 * order-preserving (negative values bit-inverted, positive ones with the sign bit
 * set; float32 in the low 32 bits).  With no ROI voxel or a non-finite ROI dose
 * nothing is counted (the caller raises, as numpy does).  edges_d: device
 * workspace of bins + 1 values of the dose's type.  Enqueued on `stream`. */
pvd_status pvd_dvh(const void* dose_d, int dose_dtype, const void* mask_d, int mask_dtype, long long n, int bins,
                   void* edges_d, long long* result_d, pvd_stream stream);

/* ------------------------------------------------------------------------ */
/* Resampling                                                                 */
/* ------------------------------------------------------------------------ */

/* Replaces the activity resampling the reference leaves as a stub on the
 * convolution path (_resample_activity, core/kernel_convolution.py:108-114)
 * and the order-3 spline resampling of resample_dose_map (core/utils.py:193-231,
 * through nibabel).  The spline is scipy.ndimage's interpolating cubic
 * B-spline with mirror boundaries (map_coordinates(order=3, mode='mirror')). */

/* coef_d = the cubic B-spline coefficients (mirror boundaries) of the float32
 * volume src_d [n0][n1][n2]; scratch_d is a third buffer of the same size.
 * All three are device buffers and must be distinct.  Enqueued on `stream`. */
pvd_status pvd_bspline_prefilter(const float* src_d, float* coef_d, float* scratch_d, int n0, int n1, int n2,
                                 pvd_stream stream);

/* out[j0][j1][j2] = value_scale * f(u), u_a = j_a * step[a] + origin[a] in input
 * voxel units (voxel centres at integers), f the cubic B-spline with the
 * coefficients src_d (order 3, after pvd_bspline_prefilter) or the trilinear
 * interpolant of src_d (order 1), both extended by mirroring.  step / origin:
 * host double[3].  Enqueued on `stream`. */
pvd_status pvd_resample(const float* src_d, int n0, int n1, int n2, float* out_d, int m0, int m1, int m2,
                        const double* step, const double* origin, int order, float value_scale,
                        pvd_stream stream);

/* pvd_resample as three one-axis passes (x, then y, then z; the spline is a tensor
 * product): 4 (order 3) or 2 (order 1) taps per output and pass.  scratch_d: device
 * float32 of at least n0*n1*m2 + n0*m1*m2 + 8*(m0+m1+m2) elements (scratch_elems). */
pvd_status pvd_resample_separable(const float* src_d, int n0, int n1, int n2, float* out_d, int m0, int m1,
                                  int m2, const double* step, const double* origin, int order, float value_scale,
                                  float* scratch_d, long long scratch_elems, pvd_stream stream);

/* ------------------------------------------------------------------------ */
/* CT Hounsfield units -> tissue masks and density                            */
/* ------------------------------------------------------------------------ */

/* Replaces TissueComposition.calculate_composition (tissue/composition.py:48-70)
 * with its artefact handling (:72-93): with PVD_HU_ARTIFACTS, voxels above 2000 HU
 * (metal) take the value of the Gaussian-smoothed image (sigma 1 voxel, as
 * scipy.ndimage.gaussian_filter with its default radius 4 and 'reflect' boundary)
 * of the image whose metal voxels and NaNs are 0, computed in FP64.  Then
 *   masks_d (device uint8 [5][n] or NULL): 1 where the (corrected) HU lies in the
 *     closed range of air [-1000, -900], lung [-900, -500], soft tissue [-100, 100],
 *     bone [300, 3000], water [-10, 10], in that plane order (ranges overlap and
 *     leave gaps exactly as the reference's do; NaN is in none);
 *   density_d (device float32 [n] or NULL): mass density (g/cc) by linear
 *     interpolation through the n_anchor (1..16, HU increasing) calibration points
 *     (anchor_hu[i], anchor_rho[i]) (host arrays), clamped to the end values, 0 for
 *     NaN.  The reference has no HU-to-density step; this map feeds the
 *     density-scaled convolution (pvd_conv_execute's density_d);
 *   hu_d (device float32 [n] or NULL): the corrected HU.
 * ct_d: device float32 [n0][n1][n2].  Device buffers 16-byte aligned.  Enqueued on
 * `stream`. */
enum { PVD_HU_ARTIFACTS = 1 };
pvd_status pvd_hu_composition(const float* ct_d, int n0, int n1, int n2, int flags, const float* anchor_hu,
                              const float* anchor_rho, int n_anchor, unsigned char* masks_d, float* density_d,
                              float* hu_d, pvd_stream stream);

/* ------------------------------------------------------------------------ */
/* Dose-point kernels                                                         */
/* ------------------------------------------------------------------------ */

/* The reference generates its kernels in numpy on the CPU
 * (data/dose_kernels/kernel_factory.py:37-75 and the *_kernel.py generators);
 * here a kernel is a sum of radial terms evaluated in FP64 on the device:
 *   PVD_TERM_COLE    weight (1 - r/p1)^2 exp(-2 r/p1) for r <= p1 (beta, positron)
 *   PVD_TERM_PHOTON  weight exp(-p1 r / 10) / (4 pi r^2), p1 = mu in 1/cm
 *   PVD_TERM_ALPHA   weight (1 - (r/p1)^p2) exp(-p3 r/p1) for r <= p1
 *   PVD_TERM_EXP_R2  weight exp(-r/p1) / r^2
 * with r in mm from the centre voxel (k/2 on each axis).  At r = 0 the PHOTON
 * and EXP_R2 terms use the radius of the sphere of the voxel's volume
 * (PVD_CENTER_R0), 0 (PVD_CENTER_ZERO) or NaN (PVD_CENTER_NAN, the reference's
 * 0 * inf for Y-90 and Ga-68). */
#define PVD_MAX_RADIAL_TERMS 16
enum { PVD_TERM_COLE = 0, PVD_TERM_PHOTON = 1, PVD_TERM_ALPHA = 2, PVD_TERM_EXP_R2 = 3 };
enum { PVD_CENTER_R0 = 0, PVD_CENTER_ZERO = 1, PVD_CENTER_NAN = 2 };
typedef struct {
  int type;       /* PVD_TERM_* */
  int center;     /* PVD_CENTER_*: value at r = 0 of PHOTON and EXP_R2 terms */
  double weight;
  double p1;      /* COLE / ALPHA: range (mm); PHOTON: mu (1/cm); EXP_R2: decay length (mm) */
  double p2;      /* ALPHA: exponent of r / range */
  double p3;      /* ALPHA: decay constant */
} pvd_radial_term;

/* out_d (device float64 [k0][k1][k2]) = scale * sum of the terms; voxel_mm: host
 * double[3].  Enqueued on `stream`. */
pvd_status pvd_radial_kernel(const pvd_radial_term* terms, int n_terms, double scale, int k0, int k1, int k2,
                             const double* voxel_mm, double* out_d, pvd_stream stream);

/* ------------------------------------------------------------------------ */
/* Learned heterogeneity correction: 3-D U-Net layers on tcgen05 (BF16, FP32   */
/* accumulation)                                                              */
/* ------------------------------------------------------------------------ */
/* No counterpart in the reference, whose correction of the water kernel for
 * tissue heterogeneity is the unused `tissue_densities` hook
 * (core/dose_calculator.py:90) and whose Monte Carlo cannot run
 * (core/monte_carlo.py:38-40).  These calls are the layers of a small 3-D
 * U-Net that predicts log(D_MC / D_conv) from activity, density and the
 * convolution dose; the network is trained on pairs produced by pvd_mc_run and
 * pvd_conv_execute.
 *
 * Tensor layout ("plane" layout): a tensor of C channels (C a multiple of 16
 * for convolutions, of 8 elsewhere) on a D x H x W grid is C/8 planes of
 * `rows` rows x 8 BF16 values (16 bytes per row), planes `rows * 16` bytes
 * apart.  Row `margin + p` holds voxel p of the zero-haloed grid
 * (D+2) x (H+2) x (W+2) flattened in C order.  Halo and margin rows must be
 * zero when a tensor is first used (allocate zeroed); every call here keeps
 * them zero.  A channel concatenation is two tensors whose planes are
 * adjacent in one allocation. */
typedef struct {
  int dims[3];          /* D, H, W interior voxels */
  int64_t padded;       /* (D+2)(H+2)(W+2) */
  int64_t padded_tiles; /* padded rounded up to a multiple of 128 */
  int64_t margin;       /* zero rows before (and after) the padded grid */
  int64_t rows;         /* rows of one plane: 2 * margin + padded_tiles */
} pvd_unet_geom;

enum {
  PVD_UNET_ACT_LEAKY = 1, /* apply LeakyReLU(slope) after the bias */
  PVD_UNET_ACCUMULATE = 2 /* add the result to the output tensor's contents */
};

pvd_status pvd_unet_geometry(int d, int h, int w, pvd_unet_geom* out);

/* 3x3x3 convolution, zero padding 1, as implicit GEMM on the tensor cores:
 *   y[v][n] = act( bias[n] + sum_{tap,k} x[v + tap][k] * W[n][k][tap] )
 *             * (mask ? leaky'(mask[v][n]) : 1)  (+ y[v][n] if ACCUMULATE)
 * with w_packed from pvd_unet_pack_weights (forward layout).  The same call
 * with the data-gradient layout, x = output gradient and mask = the layer's
 * input gives the input gradient times the previous LeakyReLU's derivative.
 * cin, cout: multiples of 16 in [16, 256]; bias may be NULL. */
pvd_status pvd_unet_conv3d(const pvd_unet_geom* geom, const void* x, int cin, const void* w_packed, const float* bias,
                           void* y, int cout, const void* mask, int flags, float slope, pvd_stream stream);

/* dw[n][k][tap] (+)= sum_v x[v + tap][k] * grad[v][n]  (FP32 [cout][cin][27],
 * the torch conv3d weight layout).  Deterministic: split over voxels on the
 * tensor cores, partial sums added in a fixed order.  workspace: device
 * memory of at least pvd_unet_wgrad_workspace bytes. */
pvd_status pvd_unet_wgrad_workspace(const pvd_unet_geom* geom, int cin, int cout, size_t* bytes);
pvd_status pvd_unet_conv3d_wgrad(const pvd_unet_geom* geom, const void* x, int cin, const void* grad, int cout,
                                 float* dw, int accumulate, void* workspace, size_t workspace_bytes,
                                 pvd_stream stream);

/* FP32 weights [cout][cin][27] -> BF16 packed weights (27 * cin * cout values
 * each) for the forward convolution cin -> cout (fwd_packed) and for the data
 * gradient cout -> cin with mirrored taps (bwd_packed); either output may be
 * NULL.  The packed layout is internal to this library and chosen per channel
 * pair the way pvd_unet_conv3d chooses its kernel: per tap [27][K/8][N][8], or,
 * for 16 or 32 output channels, with the three x taps stacked along N
 * [9][K/8][3N][8]. */
pvd_status pvd_unet_pack_weights(const float* w, int cin, int cout, void* fwd_packed, void* bwd_packed,
                                 pvd_stream stream);

/* Network input (16 channels): channel c < n_in (<= 4) is volumes[c] (device
 * float32, C order, vol_dims) read at origin + voxel, times scales[c] (host) or,
 * when scales_d is not NULL, scales_d[c] (device, read by the kernel), then
 * modes[c]: 0 linear, 1 sqrt, 2 log1p; channels >= n_in are zero, and so is
 * every channel of a voxel outside the volumes (a crop may overhang them). */
pvd_status pvd_unet_pack_input(const pvd_unet_geom* geom, const float* const* volumes, const float* scales,
                               const float* scales_d, const int* modes, int n_in, const int* vol_dims,
                               const int* origin, void* x, pvd_stream stream);

/* Symmetries of the voxel grid, for averaging the network's prediction over them
 * (the dose physics is invariant under flips, and under axis permutations of a grid
 * with equal voxel sizes along the permuted axes).  Code s in [0, 48): the axis
 * permutation s / 8 -- 0 (0,1,2), 1 (0,2,1), 2 (1,0,2), 3 (1,2,0), 4 (2,0,1),
 * 5 (2,1,0), C-order axes -- followed by flips of the permuted axes in the bits of
 * s % 8 (bit k: axis k).  The transformed volume is U = flip(transpose(V, perm),
 * flipped axes) in numpy's meaning, of dims vol_dims[perm[k]].  Codes 0..7 are the
 * flips alone. */
#define PVD_UNET_SYMMETRIES 48

/* pvd_unet_pack_input of the transformed volumes U (vol_dims: the dims of V, the
 * untransformed volumes; origin in U's coordinates; geom: a crop of U).  sym 0 is
 * pvd_unet_pack_input itself. */
pvd_status pvd_unet_pack_input_sym(const pvd_unet_geom* geom, const float* const* volumes, const float* scales,
                                   const float* scales_d, const int* modes, int n_in, const int* vol_dims,
                                   const int* origin, int sym, void* x, pvd_stream stream);

/* Average of predictions over symmetries, in the untransformed frame: for every
 * voxel v of V (vol_dims) and both channels c (mu, s),
 *   pred_avg[c][v] = (accumulate ? pred_avg[c][v] : 0) + weight * pred_sym[c][T(v)]
 * where T maps v to U's coordinates for `sym`.  pred_sym: [2][geom_sym dims], a
 * whole-volume prediction of U at origin 0 (pvd_unet_head on a crop of U, dims
 * >= U's); pred_avg: [2][geom dims] (dims >= V's), the layout
 * pvd_unet_apply_correction reads at origin 0.  Crop voxels outside V are not
 * written. */
pvd_status pvd_unet_symmetry_accumulate(const pvd_unet_geom* geom_sym, const float* pred_sym,
                                        const pvd_unet_geom* geom, const int* vol_dims, int sym, float weight,
                                        int accumulate, float* pred_avg, pvd_stream stream);

/* 2x2x2 average pooling (fine dims = 2 x coarse dims) and its backward:
 * dx = ((accumulate ? dx : 0) + dy[parent] / 8) * (mask ? leaky'(mask) : 1). */
pvd_status pvd_unet_pool(const pvd_unet_geom* fine, const void* x, const pvd_unet_geom* coarse, void* y, int channels,
                         pvd_stream stream);
pvd_status pvd_unet_pool_backward(const pvd_unet_geom* coarse, const void* dy, const pvd_unet_geom* fine, void* dx,
                                  const void* mask, int channels, int accumulate, float slope, pvd_stream stream);

/* Nearest-neighbour 2x upsampling and its backward: dx = (sum of the 8
 * children of dy) * (mask ? leaky'(mask) : 1). */
pvd_status pvd_unet_upsample(const pvd_unet_geom* coarse, const void* x, const pvd_unet_geom* fine, void* y,
                             int channels, pvd_stream stream);
pvd_status pvd_unet_upsample_backward(const pvd_unet_geom* fine, const void* dy, const pvd_unet_geom* coarse, void* dx,
                                      const void* mask, int channels, float slope, pvd_stream stream);

/* Output head (1x1x1, 16 -> 2): out[0][v] = mu (predicted log(D_MC/D_conv)),
 * out[1][v] = s (predicted log of its squared error); w_head = [w_mu(16),
 * w_s(16), b_mu, b_s]; out: device float32 [2][D][H][W]. */
pvd_status pvd_unet_head(const pvd_unet_geom* geom, const void* x, const float* w_head, float* out, pvd_stream stream);

/* Loss and head backward.  target, weight: device float32 volumes of vol_dims
 * read at origin (voxels outside them have weight 0).  With e = mu - target and l = log(e^2 + eps):
 *   loss_mu = sum weight e^2 / n,  loss_s = sum weight (s - l)^2 / n
 * (n = D*H*W; l treated as a constant).  Writes grad_x (16-channel tensor: the
 * gradient of loss_mu at the head input times leaky'(x); the error head s is
 * trained on the features without passing its gradient into the network) and
 * grads_and_loss[36] =
 * [d w_mu (16), d w_s (16), d b_mu, d b_s, loss_mu, loss_s]. */
pvd_status pvd_unet_head_loss_workspace(const pvd_unet_geom* geom, size_t* bytes);
pvd_status pvd_unet_head_loss(const pvd_unet_geom* geom, const void* x, const float* w_head, const float* pred,
                              const float* target, const float* weight, const int* vol_dims, const int* origin,
                              float eps, float slope, void* grad_x, float* grads_and_loss, void* workspace,
                              size_t workspace_bytes, pvd_stream stream);
/* pvd_unet_head_loss on a crop of the transformed volumes U of grid symmetry `sym`
 * (PVD_UNET_SYMMETRIES; origin in U's coordinates, vol_dims the untransformed dims):
 * target and weight are read at the voxel of V the crop voxel maps to, as
 * pvd_unet_pack_input_sym reads the inputs -- training on flipped crops.  sym 0 is
 * pvd_unet_head_loss. */
pvd_status pvd_unet_head_loss_sym(const pvd_unet_geom* geom, const void* x, const float* w_head, const float* pred,
                                  const float* target, const float* weight, const int* vol_dims, const int* origin,
                                  int sym, float eps, float slope, void* grad_x, float* grads_and_loss,
                                  void* workspace, size_t workspace_bytes, pvd_stream stream);

/* Corrected dose on the volume voxels that the crop at `origin` covers:
 * dose_out[v] = dose_conv[v] * exp(clamp(mu, +-mu_clamp)), or dose_conv[v]
 * itself (fallback[v] = 1, if fallback is not NULL) where the predicted error
 * sqrt(exp(s)) exceeds sigma_max or is not finite.  pred from pvd_unet_head. */
pvd_status pvd_unet_apply_correction(const pvd_unet_geom* geom, const float* pred, const float* dose_conv,
                                     const int* vol_dims, const int* origin, float sigma_max, float mu_clamp,
                                     float* dose_out, uint8_t* fallback, pvd_stream stream);

/* maxima_d (device, 5 floats): [0] = max activity, [1] = max dose over voxels
 * with density >= rho_min (device float32 volumes of n voxels; non-negative
 * finite values; 0 if none), [2..4] = the network input scales 1/[0], 1, 1/[1]
 * (0 where the maximum is 0), ready for pvd_unet_pack_input's scales_d. */
pvd_status pvd_unet_input_maxima(const float* activity, const float* density, const float* dose, int64_t n,
                                 float rho_min, float* maxima_d, pvd_stream stream);

/* db[c] = sum over interior voxels of grad[v][c] (fixed-order reduction). */
pvd_status pvd_unet_bias_grad_workspace(const pvd_unet_geom* geom, int channels, size_t* bytes);
pvd_status pvd_unet_bias_grad(const pvd_unet_geom* geom, const void* grad, int channels, float* db, void* workspace,
                              size_t workspace_bytes, pvd_stream stream);

/* Adam (bias-corrected, decoupled weight decay) on n FP32 parameters; step >= 1. */
pvd_status pvd_adam_step(float* params, const float* grads, float* m, float* v, int64_t n, float lr, float beta1,
                         float beta2, float eps, float weight_decay, int step, pvd_stream stream);

/* Global-norm gradient clipping before pvd_adam_step: norm = ||grads||_2 over n
 * FP32 values (fixed-order reduction, FP64 partial sums), then grads *= min(1,
 * limit / norm), limit = max_norm or, with spike_factor > 0, the smaller of
 * max_norm and spike_factor times the running mean of the limited norms (so one
 * outlying crop cannot throw Adam's second moments off, while its gradient still
 * acts).  A non-finite norm zeroes the gradients.  work: device float32 of
 * PVD_GRAD_CLIP_WORK values, zeroed before the first step and kept between steps:
 * work[1024] receives the norm, work[1025] the scale, work[1026] holds the
 * running mean, work[1027] counts the steps the running-mean limit (or a
 * non-finite norm) cut.  No host round trip. */
#define PVD_GRAD_CLIP_WORK 1028
pvd_status pvd_grad_clip(float* grads, int64_t n, float max_norm, float spike_factor, float* work,
                         pvd_stream stream);

/* First failure code recorded by a U-Net kernel (0: none; a bounded wait of
 * the tensor-core pipeline ran out otherwise, and PVD_ERR_TIMEOUT is
 * returned).  Synchronises the device; reset != 0 clears it. */
pvd_status pvd_unet_status(int* code, int reset);

/* ------------------------------------------------------------------------ */
/* Misc                                                                       */
/* ------------------------------------------------------------------------ */

/* Failure-path instrumentation (no counterpart in the reference, whose failure
 * handling is a try/except around curve_fit, time_integration/curve_fitting.py:58-59).
 *
 * pvd_wait_check launches one small kernel that waits on an mbarrier phase that
 * nothing will complete, through the same bounded wait and failure recording as
 * the plan's TMA column passes (PVD_WAITCHECK_PLAN: the plan's status word, read
 * and cleared by pvd_plan_status) or the U-Net's tensor-core pipeline
 * (PVD_WAITCHECK_UNET: read by pvd_unet_status; plan ignored), with `limit_ns`
 * (at most 2e9) in place of their 2 s bound.  No copy or MMA is issued, so
 * nothing is in flight when the wait runs out; the kernel records
 * PVD_ERR_TIMEOUT and returns, and the context stays usable.
 *
 * pvd_set_plan_alloc_cap caps the device bytes any one plan may hold (0 = no
 * cap): a plan creation or kernel load that would exceed it fails with
 * PVD_ERR_OOM exactly as a failed cudaMalloc does, freeing what it holds. */
enum { PVD_WAITCHECK_PLAN = 0, PVD_WAITCHECK_UNET = 1 };
pvd_status pvd_wait_check(int which, pvd_plan* plan, unsigned long long limit_ns, pvd_stream stream);
pvd_status pvd_set_plan_alloc_cap(size_t bytes);

/* Copy the calling thread's last error message into buf (NUL-terminated).
 * Returns the status of the last failing call on this thread (PVD_OK if none). */
pvd_status pvd_last_error(char* buf, size_t len);

/* Library version as MAJOR*10000 + MINOR*100 + PATCH. */
int pvd_version(void);

/* Number of kernel launches this library enqueued on this thread since the
 * last reset (instrumentation for benchmarks; monotone, never wraps in
 * practice). */
uint64_t pvd_launch_count(int reset);

#ifdef __cplusplus
}
#endif

#endif /* PVD_H_ */
