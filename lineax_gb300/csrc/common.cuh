// Shared helpers for the lxgb CUDA sources: status plumbing, launch checks,
// warp reductions.  Every entry point validates its arguments on the host,
// launches, and converts a launch error into LXGB_CUDA_ERROR with a message
// retrievable through lxgb_last_error().
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>

#include "../../include/lxgb.h"

namespace lxgb {

// Thread-local text of the last failure; defined in status.cu.
void set_last_error(const char* fmt, ...);

inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

// Returns LXGB_CUDA_ERROR (and records the message) if the last launch failed.
inline int check_launch(const char* what) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_last_error("%s: %s", what, cudaGetErrorString(e));
    return LXGB_CUDA_ERROR;
  }
  return LXGB_SUCCESSFUL;
}

inline int invalid(const char* fmt_msg) {
  set_last_error("%s", fmt_msg);
  return LXGB_INVALID_ARG;
}

#define LXGB_REQUIRE(cond, msg)            \
  do {                                     \
    if (!(cond)) return ::lxgb::invalid(msg); \
  } while (0)

#define LXGB_CUDA_TRY(expr, what)                                         \
  do {                                                                   \
    cudaError_t _e = (expr);                                             \
    if (_e != cudaSuccess) {                                             \
      ::lxgb::set_last_error("%s: %s", what, cudaGetErrorString(_e));    \
      return LXGB_CUDA_ERROR;                                            \
    }                                                                    \
  } while (0)

// Number of SMs of the current device (cached per process for device 0..15).
int sm_count();

// Raises kernel `fn`'s dynamic shared-memory limit to `bytes` on the current
// device.  The attribute persists in the context, so the driver is called only
// the first time a kernel needs more than it was last given (repeated driver
// calls cost microseconds of host time per launch).  Defined in status.cu.
cudaError_t ensure_dynamic_smem(const void* fn, int bytes);

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ double warp_max(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

// Arg-max of |value| with the lowest index winning ties: the combination rule
// of LAPACK idamax, which scans upward and only moves on a strictly larger
// magnitude.  Each lane first scans its own rows in increasing order with the
// same strict rule, so the warp result equals a sequential scan.
__device__ __forceinline__ void warp_argmax_first(double& v, int& idx) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    double ov = __shfl_xor_sync(0xffffffffu, v, o);
    int oi = __shfl_xor_sync(0xffffffffu, idx, o);
    if (ov > v || (ov == v && oi < idx)) {
      v = ov;
      idx = oi;
    }
  }
}

// Pivot-search key of x: |x| as its IEEE bit pattern, which orders like the
// value for every non-NaN x; NaN maps to -1 and never wins (as "|x| > v" never
// holds for NaN).  64-bit integer compares run on the integer pipe, not on
// GB300's narrow FP64 pipe.
__device__ __forceinline__ long long pivot_key(double x) {
  const long long b = __double_as_longlong(x) & 0x7FFFFFFFFFFFFFFFLL;
  return b > 0x7FF0000000000000LL ? -1LL : b;
}

// warp_argmax_first over pivot keys.
__device__ __forceinline__ void warp_argmax_first_key(long long& v, int& idx) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const long long ov = __shfl_xor_sync(0xffffffffu, v, o);
    const int oi = __shfl_xor_sync(0xffffffffu, idx, o);
    if (ov > v || (ov == v && oi < idx)) {
      v = ov;
      idx = oi;
    }
  }
}

}  // namespace lxgb
