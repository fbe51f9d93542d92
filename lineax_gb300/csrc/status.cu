// Status strings, per-thread error text and device queries for the C ABI.
#include <stdarg.h>
#include <string.h>

#include <map>
#include <mutex>
#include <utility>

#include "common.cuh"

namespace lxgb {

static thread_local char g_last_error[512] = {0};

void set_last_error(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_last_error, sizeof(g_last_error), fmt, ap);
  va_end(ap);
}

int sm_count() {
  static int cached[16] = {0};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0) dev = 0;
  if (dev < 16 && cached[dev] > 0) return cached[dev];
  int sms = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
      sms <= 0)
    sms = 152;
  if (dev < 16) cached[dev] = sms;
  return sms;
}

cudaError_t ensure_dynamic_smem(const void* fn, int bytes) {
  static std::mutex mu;
  static std::map<std::pair<const void*, int>, int> given;  // (kernel, device) -> bytes
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) dev = 0;
  std::lock_guard<std::mutex> lock(mu);
  int& have = given[{fn, dev}];
  if (have >= bytes) return cudaSuccess;
  const cudaError_t e =
      cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  if (e == cudaSuccess) have = bytes;
  return e;
}

}  // namespace lxgb

extern "C" {

int lxgb_version(void) { return 100; }

const char* lxgb_status_string(int status) {
  switch (status) {
    case LXGB_SUCCESSFUL: return "successful";
    case LXGB_MAX_STEPS_REACHED: return "max_steps_reached";
    case LXGB_SINGULAR: return "singular";
    case LXGB_BREAKDOWN: return "breakdown";
    case LXGB_STAGNATION: return "stagnation";
    case LXGB_CONLIM: return "conlim";
    case LXGB_NONFINITE_INPUT: return "nonfinite_input";
    case LXGB_INVALID_ARG: return "invalid argument";
    case LXGB_CUDA_ERROR: return "CUDA error";
    case LXGB_NOT_SUPPORTED: return "not supported";
    case LXGB_TIMEOUT: return "timeout";
    case LXGB_WORKSPACE_TOO_SMALL: return "workspace too small";
    default: return "unknown status";
  }
}

const char* lxgb_last_error(void) { return lxgb::g_last_error; }

}  // extern "C"
