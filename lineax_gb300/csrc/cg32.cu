// Mixed-precision CG for the 5-point Poisson operator, k right-hand sides:
// the iteration vectors p, r, Ap and the running correction x_lo are FP32
// (the HBM stream of the hot loop), the solution x and the right-hand side b
// FP64.  Every `check` iterations (16 by default) the host calls lxgb_cg32_refresh, which
// folds x_lo into x in FP64, recomputes the true residual r = b - A x in FP64
// (residual replacement: the recurrence residual restarts from it, the search
// direction is kept), evaluates lineax's stopping test on that true residual
// (max_i |r_i| / (atol + rtol |b_i|) <= 1, lineax/_solver/cg.py:149-160) and
// resets gamma = rᵀr.  Between refreshes an iteration is
//   Ap = A p, <p, Ap>          (one fused pass)
//   alpha = gamma / <p, Ap>    (lineax's breakdown guard)
//   x_lo += alpha p, r -= alpha Ap, <r, r>   (one fused pass)
//   beta = <r, r> / gamma, p = r + beta p
// Dot products accumulate FP32 products in FP32 over a thread's few elements
// and combine the per-thread sums in FP64, in a fixed order.  Each right-hand
// side carries its own flags; an inactive one is left untouched, so results do
// not depend on the other right-hand sides in the block.
#include <math.h>

#include "common.cuh"

namespace lxgb {

constexpr int kC32Threads = 256;
constexpr int kC32RowsPerCta = 16;  // grid rows per CTA of the stencil pass
constexpr int kC32MaxParts = 1024;  // partial sums per right-hand side

struct C32State {
  double* gamma;   // k: <r, r> of the current recurrence
  double* alpha;   // k
  double* beta;    // k
  int* act;        // k: not finished (the next refresh still folds x_lo)
  int* run;        // k: iterating
  int* steps;      // k
  int* conv;       // k: 1 converged, 2 breakdown or NaN test
  double* part;    // k * kC32MaxParts partial sums
};

static int64_t c32_state_bytes(int k) {
  return 256 + (int64_t)k * (3 * 8 + 4 * 4) + 256 + (int64_t)k * kC32MaxParts * 8;
}

static C32State c32_carve(void* work, int k) {
  C32State s;
  char* p = reinterpret_cast<char*>(work) + 256;
  s.gamma = reinterpret_cast<double*>(p); p += (int64_t)k * 8;
  s.alpha = reinterpret_cast<double*>(p); p += (int64_t)k * 8;
  s.beta = reinterpret_cast<double*>(p); p += (int64_t)k * 8;
  s.act = reinterpret_cast<int*>(p); p += (int64_t)k * 4;
  s.run = reinterpret_cast<int*>(p); p += (int64_t)k * 4;
  s.steps = reinterpret_cast<int*>(p); p += (int64_t)k * 4;
  s.conv = reinterpret_cast<int*>(p); p += (int64_t)k * 4;
  p = reinterpret_cast<char*>(((uintptr_t)p + 255) & ~(uintptr_t)255);
  s.part = reinterpret_cast<double*>(p);
  return s;
}

__device__ __forceinline__ double c32_block_sum(double v, double* sm) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  v = warp_sum(v);
  if (lane == 0) sm[warp] = v;
  __syncthreads();
  double t = 0.0;
  if (threadIdx.x == 0)
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += sm[w];
  return t;
}

// Partial count for the stencil pass over an nx×ny grid.
static int c32_parts(int64_t nx, int64_t ny) {
  return (int)(((ny + kC32Threads - 1) / kC32Threads) *
               ((nx + kC32RowsPerCta - 1) / kC32RowsPerCta));
}

// Ap = A p (FP32) and partial <p, Ap> for active right-hand sides.
__global__ void __launch_bounds__(kC32Threads)
c32_stencil_dot_kernel(int64_t nx, int64_t ny, C32State s, const float* __restrict__ p,
                       float* __restrict__ ap) {
  __shared__ double sm[kC32Threads / 32];
  const int c = blockIdx.z;
  const int part = blockIdx.y * gridDim.x + blockIdx.x;
  if (!s.run[c]) return;  // uniform per CTA
  const int64_t n = nx * ny;
  const float* pc = p + (int64_t)c * n;
  float* apc = ap + (int64_t)c * n;
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  float acc = 0.0f;
  if (j < ny) {
    const int64_t i0 = (int64_t)blockIdx.y * kC32RowsPerCta;
    const int64_t i1 = min(nx, i0 + kC32RowsPerCta);
    float up = (i0 > 0) ? pc[(i0 - 1) * ny + j] : 0.0f;
    float cen = pc[i0 * ny + j];
    for (int64_t i = i0; i < i1; ++i) {
      const int64_t o = i * ny + j;
      const float dn = (i + 1 < nx) ? pc[o + ny] : 0.0f;
      const float lf = (j > 0) ? pc[o - 1] : 0.0f;
      const float rt = (j + 1 < ny) ? pc[o + 1] : 0.0f;
      const float v = fmaf(4.0f, cen, -((up + dn) + (lf + rt)));
      apc[o] = v;
      acc = fmaf(cen, v, acc);
      up = cen;
      cen = dn;
    }
  }
  const double t = c32_block_sum((double)acc, sm);
  if (threadIdx.x == 0) s.part[(int64_t)c * kC32MaxParts + part] = t;
}

// Sum of vector c's partials in index order (one warp per right-hand side).
__device__ double c32_combine(const double* part, int P) {
  const int lane = threadIdx.x & 31;
  double v = 0.0;
  for (int i = lane; i < P; i += 32) v += part[i];
  return warp_sum(v);
}

// alpha = gamma / <p, Ap>; a non-positive or non-finite curvature stops the
// right-hand side (breakdown, as lineax's NaN alpha at cg.py:172-178).
__global__ void c32_alpha_kernel(int k, C32State s, int P) {
  const int c = blockIdx.x;
  if (!s.run[c]) return;
  const double pap = c32_combine(s.part + (int64_t)c * kC32MaxParts, P);
  if (threadIdx.x == 0) {
    const double a = s.gamma[c] / pap;
    if (!(pap > 0.0) || !isfinite(a)) {
      s.run[c] = 0;  // the next refresh folds x_lo and ends this right-hand side
      s.conv[c] = 2;
    }
    s.alpha[c] = a;
  }
}

// x_lo += alpha p; r -= alpha Ap; partial <r, r>.
__global__ void __launch_bounds__(kC32Threads)
c32_update_kernel(int64_t n, C32State s, const float* __restrict__ p,
                  const float* __restrict__ ap, float* __restrict__ xlo, float* __restrict__ r,
                  int P) {
  __shared__ double sm[kC32Threads / 32];
  const int c = blockIdx.y;
  if (!s.run[c]) return;
  const float a = (float)s.alpha[c];
  const int64_t o = (int64_t)c * n;
  float acc = 0.0f;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    xlo[o + i] = fmaf(a, p[o + i], xlo[o + i]);
    const float rn = fmaf(-a, ap[o + i], r[o + i]);
    r[o + i] = rn;
    acc = fmaf(rn, rn, acc);
  }
  const double t = c32_block_sum((double)acc, sm);
  if (threadIdx.x == 0) s.part[(int64_t)c * kC32MaxParts + blockIdx.x] = t;
}

// beta = <r, r> / gamma, gamma = <r, r>, steps += 1 (one warp per right-hand side).
__global__ void c32_beta_kernel(int k, C32State s, int P) {
  const int c = blockIdx.x;
  if (!s.run[c]) return;
  const double rr = c32_combine(s.part + (int64_t)c * kC32MaxParts, P);
  if (threadIdx.x == 0) {
    s.beta[c] = rr / s.gamma[c];
    s.gamma[c] = rr;
    s.steps[c] += 1;
  }
}

// p = r + beta p.
__global__ void __launch_bounds__(kC32Threads)
c32_direction_kernel(int64_t n, C32State s, const float* __restrict__ r, float* __restrict__ p) {
  const int c = blockIdx.y;
  if (!s.run[c]) return;
  const float b = (float)s.beta[c];
  const int64_t o = (int64_t)c * n;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    p[o + i] = fmaf(b, p[o + i], r[o + i]);
}

// |v| / s against 1 without a division: 0 (<= 1), 1 (> 1), 2 (NaN).
__device__ __forceinline__ int c32_ratio_code(double v, double sc) {
  const long long kInf = 0x7FF0000000000000LL;
  const long long av = __double_as_longlong(v) & 0x7FFFFFFFFFFFFFFFLL;
  const long long sb = __double_as_longlong(sc);
  const long long as = sb & 0x7FFFFFFFFFFFFFFFLL;
  if (av > kInf || as > kInf) return 2;
  if (as == 0) return av == 0 ? 2 : 1;
  if (as == kInf) return av == kInf ? 2 : 0;
  if (sb < 0) return 0;
  return av > sb ? 1 : 0;
}

// Refresh, first pass (active right-hand sides): x += x_lo, x_lo = 0.
__global__ void c32_fold_kernel(int64_t n, C32State s, double* __restrict__ x,
                                float* __restrict__ xlo) {
  const int c = blockIdx.y;
  if (!s.act[c]) return;
  const int64_t o = (int64_t)c * n;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    x[o + i] += (double)xlo[o + i];
    xlo[o + i] = 0.0f;
  }
}

// Refresh, second pass: r = b - A x in FP64 (stored as FP32), partial <r, r>
// and the stopping-test code per CTA.
__global__ void __launch_bounds__(kC32Threads)
c32_refresh_kernel(int64_t nx, int64_t ny, C32State s, const double* __restrict__ b,
                   const double* __restrict__ x, float* __restrict__ r,
                   int* __restrict__ codes, double rtol, double atol) {
  __shared__ double sm[kC32Threads / 32];
  __shared__ int s_code;
  const int c = blockIdx.z;
  const int part = blockIdx.y * gridDim.x + blockIdx.x;
  if (!s.act[c]) return;
  const int64_t n = nx * ny;
  const double* xc = x + (int64_t)c * n;
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (threadIdx.x == 0) s_code = 0;
  __syncthreads();
  const int64_t i0 = (int64_t)blockIdx.y * kC32RowsPerCta;
  const int64_t i1 = min(nx, i0 + kC32RowsPerCta);
  float acc = 0.0f;
  int code = 0;
  if (j < ny) {
    double up = (i0 > 0) ? xc[(i0 - 1) * ny + j] : 0.0;
    double cen = xc[i0 * ny + j];
    for (int64_t i = i0; i < i1; ++i) {
      const int64_t o = i * ny + j;
      const double dn = (i + 1 < nx) ? xc[o + ny] : 0.0;
      const double lf = (j > 0) ? xc[o - 1] : 0.0;
      const double rt = (j + 1 < ny) ? xc[o + 1] : 0.0;
      const double ax = fma(4.0, cen, -((up + dn) + (lf + rt)));
      const double bv = b[(int64_t)c * n + o];
      const double rv = bv - ax;
      const float rf = (float)rv;
      r[(int64_t)c * n + o] = rf;
      acc = fmaf(rf, rf, acc);
      code = max(code, c32_ratio_code(rv, fma(rtol, fabs(bv), atol)));
      up = cen;
      cen = dn;
    }
  }
  const double t = c32_block_sum((double)acc, sm);
  if (code) atomicMax(&s_code, code);
  __syncthreads();
  if (threadIdx.x == 0) {
    s.part[(int64_t)c * kC32MaxParts + part] = t;
    codes[(int64_t)c * kC32MaxParts + part] = s_code;
  }
}

// gamma = <r, r> of the replaced residual; the right-hand side ends when the
// test passes (max code 0), when it is NaN (lineax: a NaN norm ends the
// loop), after a breakdown, or at max_steps.
__global__ void c32_refresh_final_kernel(int k, C32State s, const int* __restrict__ codes, int P,
                                         int64_t max_steps) {
  const int c = blockIdx.x;
  if (!s.act[c]) return;
  const double rr = c32_combine(s.part + (int64_t)c * kC32MaxParts, P);
  const int lane = threadIdx.x & 31;
  int m = 0;
  for (int i = lane; i < P; i += 32) m = max(m, codes[(int64_t)c * kC32MaxParts + i]);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
  if (threadIdx.x == 0) {
    s.gamma[c] = rr;
    if (s.conv[c] == 2) {
      s.act[c] = s.run[c] = 0;
    } else if (m != 1) {
      s.act[c] = s.run[c] = 0;
      s.conv[c] = (m == 0) ? 1 : 2;
    } else if (s.steps[c] >= max_steps) {
      s.act[c] = s.run[c] = 0;
    }
  }
}

__global__ void c32_init_kernel(int k, C32State s, int64_t max_steps) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= k) return;
  s.act[c] = 1;
  s.run[c] = max_steps > 0 ? 1 : 0;
  s.steps[c] = 0;
  s.conv[c] = 0;
  s.gamma[c] = 0.0;
}

__global__ void c32_status_kernel(int k, C32State s, int32_t* out) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= k) return;
  out[3 * c] = s.act[c];
  out[3 * c + 1] = s.steps[c];
  out[3 * c + 2] = s.conv[c];  // 0: max steps (or running), 1 converged, 2 breakdown / NaN
}

}  // namespace lxgb

using namespace lxgb;

extern "C" int64_t lxgb_cg32_workspace_size(int32_t nrhs) {
  // state + partial codes
  return c32_state_bytes(nrhs > 0 ? nrhs : 1) + (int64_t)(nrhs > 0 ? nrhs : 1) * kC32MaxParts * 4 +
         256;
}

static int c32_check(int32_t k, int64_t nx, int64_t ny, void* work, int64_t wbytes) {
  LXGB_REQUIRE(k >= 1 && k <= 65535 && nx >= 1 && ny >= 1, "cg32: bad sizes");
  LXGB_REQUIRE(nx <= 65535 * (int64_t)kC32RowsPerCta, "cg32: grid too tall");
  LXGB_REQUIRE(c32_parts(nx, ny) <= kC32MaxParts, "cg32: grid too large for the partial sums");
  LXGB_REQUIRE(work && ((uintptr_t)work & 255) == 0, "cg32: workspace must be 256-byte aligned");
  if (wbytes < lxgb_cg32_workspace_size(k)) {
    set_last_error("cg32: workspace too small");
    return LXGB_WORKSPACE_TOO_SMALL;
  }
  return LXGB_SUCCESSFUL;
}

static int* c32_codes(void* work, int k) {
  return reinterpret_cast<int*>(reinterpret_cast<char*>(work) + c32_state_bytes(k));
}

static int c32_vec_grid(int64_t n) {
  const int64_t per = (n + kC32Threads * 8 - 1) / (kC32Threads * 8);
  return (int)(per < 1 ? 1 : (per > kC32MaxParts ? kC32MaxParts : per));
}

extern "C" int lxgb_cg32_init(int32_t k, int64_t nx, int64_t ny, int64_t max_steps, void* work,
                              int64_t wbytes, void* stream) {
  int rc = c32_check(k, nx, ny, work, wbytes);
  if (rc) return rc;
  C32State s = c32_carve(work, k);
  c32_init_kernel<<<(k + 127) / 128, 128, 0, as_stream(stream)>>>(k, s, max_steps);
  return check_launch("cg32_init");
}

extern "C" int lxgb_cg32_refresh(int32_t k, int64_t nx, int64_t ny, const double* b, double* x,
                                 float* xlo, float* r, double rtol, double atol,
                                 int64_t max_steps, void* work, int64_t wbytes, void* stream) {
  int rc = c32_check(k, nx, ny, work, wbytes);
  if (rc) return rc;
  LXGB_REQUIRE(b && x && xlo && r, "cg32: null pointer");
  cudaStream_t st = as_stream(stream);
  C32State s = c32_carve(work, k);
  int* codes = c32_codes(work, k);
  dim3 g((unsigned)((ny + kC32Threads - 1) / kC32Threads),
         (unsigned)((nx + kC32RowsPerCta - 1) / kC32RowsPerCta), (unsigned)k);
  const int P = c32_parts(nx, ny);
  c32_fold_kernel<<<dim3((unsigned)c32_vec_grid(nx * ny), (unsigned)k), kC32Threads, 0, st>>>(
      nx * ny, s, x, xlo);
  c32_refresh_kernel<<<g, kC32Threads, 0, st>>>(nx, ny, s, b, x, r, codes, rtol, atol);
  c32_refresh_final_kernel<<<k, 32, 0, st>>>(k, s, codes, P, max_steps);
  return check_launch("cg32_refresh");
}

extern "C" int lxgb_cg32_iterate(int32_t k, int64_t nx, int64_t ny, int32_t iters, float* p,
                                 float* ap, float* xlo, float* r, void* work, int64_t wbytes,
                                 void* stream) {
  int rc = c32_check(k, nx, ny, work, wbytes);
  if (rc) return rc;
  LXGB_REQUIRE(p && ap && xlo && r, "cg32: null pointer");
  cudaStream_t st = as_stream(stream);
  C32State s = c32_carve(work, k);
  const int64_t n = nx * ny;
  dim3 gs((unsigned)((ny + kC32Threads - 1) / kC32Threads),
          (unsigned)((nx + kC32RowsPerCta - 1) / kC32RowsPerCta), (unsigned)k);
  const int Ps = c32_parts(nx, ny);
  const int Pv = c32_vec_grid(n);
  dim3 gv((unsigned)Pv, (unsigned)k);
  for (int it = 0; it < iters; ++it) {
    c32_stencil_dot_kernel<<<gs, kC32Threads, 0, st>>>(nx, ny, s, p, ap);
    c32_alpha_kernel<<<k, 32, 0, st>>>(k, s, Ps);
    c32_update_kernel<<<gv, kC32Threads, 0, st>>>(n, s, p, ap, xlo, r, Pv);
    c32_beta_kernel<<<k, 32, 0, st>>>(k, s, Pv);
    c32_direction_kernel<<<gv, kC32Threads, 0, st>>>(n, s, r, p);
  }
  return check_launch("cg32_iterate");
}

// p = r (FP32) after the first refresh.
__global__ void c32_copy_kernel(int64_t total, const float* __restrict__ src,
                                float* __restrict__ dst) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total;
       i += (int64_t)gridDim.x * blockDim.x)
    dst[i] = src[i];
}

extern "C" int lxgb_cg32_start_direction(int32_t k, int64_t n, const float* r, float* p,
                                         void* stream) {
  LXGB_REQUIRE(k >= 1 && n >= 0 && r && p, "cg32: bad arguments");
  const int64_t total = n * k;
  c32_copy_kernel<<<(unsigned)(total / 256 + 1 < 8192 ? total / 256 + 1 : 8192), 256, 0,
                    as_stream(stream)>>>(total, r, p);
  return check_launch("cg32_start_direction");
}

extern "C" int lxgb_cg32_status(int32_t k, int32_t* out, void* work, int64_t wbytes,
                                void* stream) {
  LXGB_REQUIRE(k >= 1 && out && work, "cg32: bad arguments");
  if (wbytes < lxgb_cg32_workspace_size(k)) {
    set_last_error("cg32: workspace too small");
    return LXGB_WORKSPACE_TOO_SMALL;
  }
  C32State s = c32_carve(work, k);
  c32_status_kernel<<<(k + 127) / 128, 128, 0, as_stream(stream)>>>(k, s, out);
  return check_launch("cg32_status");
}
