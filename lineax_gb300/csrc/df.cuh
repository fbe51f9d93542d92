// Double-float helpers: FP64 values carried as an unevaluated sum of two
// FP32 values, so that FP64-accurate products and sums run on the FP32 pipe
// (GB300 issues FP32 at 64x its FP64 rate).
#pragma once

#include <cuda_runtime.h>

namespace lxgb {

// hi = a truncated to 24 significant bits, lo = the rest truncated to 24
// bits, by integer operations only; |a - hi - lo| <= 2^-46 |a|.  Nonzero
// values outside 2^-74 <= |a| < 2^128 (and inf, NaN) take a conversion path
// behind a warp-uniform branch: GB300 runs conversions on its narrow FP64
// pipe, and a predicated (if-converted) fallback would issue them for every
// element.
__device__ __forceinline__ void split_f64(double a, float& hi, float& lo) {
  const unsigned long long u = (unsigned long long)__double_as_longlong(a);
  const unsigned e = (unsigned)(u >> 52) & 0x7FFu;
  const unsigned sign = (unsigned)(u >> 32) & 0x80000000u;
  const unsigned mh = (unsigned)(u >> 29) & 0x7FFFFFu;
  const unsigned rem = (unsigned)u & 0x1FFFFFFFu;
  const int sh = __clz(rem | 1u) - 8;
  const unsigned m = (sh >= 0) ? (rem << sh) : (rem >> (-sh));
  const int ex = (int)e - 1052 - sh + 127;
  const bool zero = (u << 1) == 0ull;
  hi = zero ? __uint_as_float(sign) : __uint_as_float(sign | (((e - 1023u + 127u) & 0xFFu) << 23) | mh);
  lo = (rem == 0u) ? 0.0f : __uint_as_float(sign | (((unsigned)ex & 0xFFu) << 23) | (m & 0x7FFFFFu));
  const bool slow = !zero && ((e < 949u) || (e > 1150u));
  if (__any_sync(__activemask(), slow)) {
    if (slow) {
      hi = __double2float_rz(a);
      lo = __double2float_rn(a - (double)hi);
    }
  }
}

// FP32 copy of a for the factor (the hi part of split_f64, integer path).
__device__ __forceinline__ float to_f32(double a) {
  float hi, lo;
  split_f64(a, hi, lo);
  return hi;
}

// s + t exactly as (s', err) (Knuth TwoSum).
__device__ __forceinline__ void two_sum(float& s, float t, float& err) {
  const float r = s + t;
  const float z = r - s;
  err = (s - (r - z)) + (t - z);
  s = r;
}

// s + t as (s', err) when |s| >= |t| or s == 0 (Dekker's FastTwoSum).
__device__ __forceinline__ void fast_two_sum(float& s, float t, float& err) {
  const float r = s + t;
  err = t - (r - s);
  s = r;
}

}  // namespace lxgb
