// Batched time-integrated dose: per-voxel two-exponential fit and kernel
// convolution of the fitted cumulated activity for many volumes of uneven
// sizes, enqueued item by item on one stream, or recorded once into a CUDA
// graph and replayed as a single launch.  The reference computes this one
// volume at a time on the CPU (core/dose_calculator.py:85-164 with
// time_integration/curve_fitting.py:112-219 and core/kernel_convolution.py:48-106).
#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "pvd_common.cuh"

struct pvd_batch {
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  int n_launches = 0;  // kernel launches recorded in the graph
};

namespace pvd {

static pvd_status validate(const pvd_batch_item* items, int n_items, int max_fev) {
  if (n_items < 0 || (n_items > 0 && !items)) return set_error(PVD_ERR_ARG, "pvd_batch: null or negative item list");
  if (max_fev < 1) return set_error(PVD_ERR_ARG, "pvd_batch: max_fev must be >= 1");
  for (int i = 0; i < n_items; ++i) {
    const pvd_batch_item& it = items[i];
    const std::string at = "pvd_batch: item " + std::to_string(i) + ": ";
    if (!it.plan || !it.activity_d || !it.times || !it.params_d || !it.auc_d || !it.cum_d || !it.dose_d)
      return set_error(PVD_ERR_ARG, at + "null plan, buffer or times");
    if (it.n_times < 4 || it.n_times > PVD_MAX_TIMEPOINTS)
      return set_error(PVD_ERR_ARG, at + "n_times must be in [4, 16] for the two-exponential fit");
    for (int k = 1; k < it.n_times; ++k)
      if (!(it.times[k] > it.times[k - 1])) return set_error(PVD_ERR_ARG, at + "times must increase");
    pvd_plan_info info;
    if (pvd_plan_get_info(it.plan, &info) != PVD_OK) return set_error(PVD_ERR_ARG, at + "invalid plan");
  }
  return PVD_OK;
}

static pvd_status enqueue(const pvd_batch_item* items, int n_items, int fit_flags, int max_fev, double time_scale,
                          cudaStream_t st) {
  const double p0[5] = {1.0, 0.1, 0.5, 0.01, 0.0};  // unused: every voxel starts from its own peeling
  const int flags = fit_flags | PVD_FIT_P0_FROM_DATA | PVD_FIT_AUC_INF;
  for (int i = 0; i < n_items; ++i) {
    const pvd_batch_item& it = items[i];
    pvd_plan_info info;
    pvd_plan_get_info(it.plan, &info);
    const long long nvox = (long long)info.n[0] * info.n[1] * info.n[2];
    pvd_status s = pvd_tac_fit(PVD_FIT_F4A, it.times, nullptr, it.n_times, p0, 0.0, 0.0, max_fev, flags,
                               it.activity_d, nvox, it.params_d, it.auc_d, it.ok_d, it.cum_d, time_scale,
                               (pvd_stream)st);
    if (s != PVD_OK) return s;
    s = pvd_conv_execute(it.plan, it.cum_d, it.density_d, it.dose_d, 1.0f, (pvd_stream)st);
    if (s != PVD_OK) return s;
  }
  return PVD_OK;
}

}  // namespace pvd

using namespace pvd;

extern "C" pvd_status pvd_batch_execute(const pvd_batch_item* items, int n_items, int fit_flags, int max_fev,
                                        double time_scale, pvd_stream stream) {
  pvd_status s = validate(items, n_items, max_fev);
  if (s != PVD_OK) return s;
  return enqueue(items, n_items, fit_flags, max_fev, time_scale, (cudaStream_t)stream);
}

extern "C" pvd_status pvd_batch_create(const pvd_batch_item* items, int n_items, int fit_flags, int max_fev,
                                       double time_scale, pvd_batch** out) {
  if (!out) return set_error(PVD_ERR_ARG, "pvd_batch_create: null output handle");
  *out = nullptr;
  pvd_status s = validate(items, n_items, max_fev);
  if (s != PVD_OK) return s;
  cudaStream_t cs = nullptr;
  if (cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking) != cudaSuccess)
    return set_error(PVD_ERR_CUDA, std::string("pvd_batch_create: stream: ") + cudaGetErrorString(cudaGetLastError()));
  // one eager pass: loads every kernel the batch uses before recording
  s = enqueue(items, n_items, fit_flags, max_fev, time_scale, cs);
  if (s == PVD_OK && cudaStreamSynchronize(cs) != cudaSuccess)
    s = set_error(PVD_ERR_CUDA, std::string("pvd_batch_create: eager pass: ") + cudaGetErrorString(cudaGetLastError()));
  if (s != PVD_OK) {
    cudaStreamDestroy(cs);
    return s;
  }
  pvd_batch* b = new pvd_batch();
  const uint64_t before = pvd_launch_count(0);
  cudaError_t e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
  if (e == cudaSuccess) {
    const pvd_status es = enqueue(items, n_items, fit_flags, max_fev, time_scale, cs);
    e = cudaStreamEndCapture(cs, &b->graph);  // always end the capture, also after a failed enqueue
    if (es != PVD_OK) s = es;
  }
  b->n_launches = (int)(pvd_launch_count(0) - before);
  if (s == PVD_OK && e == cudaSuccess) e = cudaGraphInstantiate(&b->exec, b->graph, 0);
  cudaStreamDestroy(cs);
  if (s == PVD_OK && e != cudaSuccess)
    s = set_error(PVD_ERR_CUDA, std::string("pvd_batch_create: graph: ") + cudaGetErrorString(e));
  if (s != PVD_OK) {
    cudaGetLastError();
    pvd_batch_destroy(b);
    return s;
  }
  *out = b;
  return PVD_OK;
}

extern "C" pvd_status pvd_batch_run(pvd_batch* b, pvd_stream stream) {
  if (!b || !b->exec) return set_error(PVD_ERR_ARG, "pvd_batch_run: invalid handle");
  const cudaError_t e = cudaGraphLaunch(b->exec, (cudaStream_t)stream);
  if (e != cudaSuccess) return set_error(PVD_ERR_CUDA, std::string("pvd_batch_run: ") + cudaGetErrorString(e));
  count_launch(b->n_launches);
  return PVD_OK;
}

extern "C" pvd_status pvd_batch_destroy(pvd_batch* b) {
  if (!b) return PVD_OK;
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  delete b;
  return PVD_OK;
}
