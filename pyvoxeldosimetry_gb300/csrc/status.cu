// Thread-local error state and launch counter behind the C ABI.
#include <cstdio>
#include <cstring>
#include <string>

#include "pvd_common.cuh"

namespace pvd {

namespace {
thread_local std::string g_msg;
thread_local pvd_status g_status = PVD_OK;
thread_local uint64_t g_launches = 0;
}  // namespace

pvd_status set_error(pvd_status st, const std::string& msg) {
  g_status = st;
  g_msg = msg;
  return st;
}

pvd_status cuda_error(cudaError_t e, const char* what) {
  std::string m = std::string(what) + ": " + cudaGetErrorName(e) + " (" + cudaGetErrorString(e) + ")";
  return set_error(e == cudaErrorMemoryAllocation ? PVD_ERR_OOM : PVD_ERR_CUDA, m);
}

void count_launch(int n) { g_launches += (uint64_t)n; }

}  // namespace pvd

extern "C" pvd_status pvd_last_error(char* buf, size_t len) {
  if (buf && len) {
    size_t n = pvd::g_msg.size() < len - 1 ? pvd::g_msg.size() : len - 1;
    std::memcpy(buf, pvd::g_msg.data(), n);
    buf[n] = '\0';
  }
  return pvd::g_status;
}

extern "C" int pvd_version(void) { return 100; }

extern "C" uint64_t pvd_launch_count(int reset) {
  uint64_t v = pvd::g_launches;
  if (reset) pvd::g_launches = 0;
  return v;
}

extern "C" pvd_status pvd_wait_check(int which, pvd_plan* plan, unsigned long long limit_ns, pvd_stream stream) {
  if (limit_ns == 0 || limit_ns > 2000000000ull)
    return pvd::set_error(PVD_ERR_ARG, "pvd_wait_check: limit_ns must be in (0, 2e9]");
  if (which == PVD_WAITCHECK_PLAN) return pvd::plan_wait_check(plan, limit_ns, (cudaStream_t)stream);
  if (which == PVD_WAITCHECK_UNET) return pvd::unet_wait_check(limit_ns, (cudaStream_t)stream);
  return pvd::set_error(PVD_ERR_ARG, "pvd_wait_check: unknown target");
}
