// BiCGStab (lineax/_solver/bicgstab.py:78-205) on the device for k
// right-hand sides at once, FP64, right-preconditioned.
//
// Vectors of a k-RHS block are stored back to back (vector c at base + c*n).
// The loop body is a fixed sequence of launches; operator and preconditioner
// products are formed by the caller between them.  Each right-hand side
// carries its scalars (rho, alpha, omega) and a flag set from lineax's loop
// condition (bicgstab.py:128-133): no breakdown, the two-space stopping test
// not yet met, step < max_steps.  Every kernel leaves an inactive right-hand
// side untouched, so iterations past its stop change nothing and its result
// is the same as when it is solved alone.  Dot products are two-stage
// (per-CTA partials, then a fixed-order combination), so results do not
// depend on timing.
#include "krylov.cuh"

namespace lxgb {

// Per right-hand side state in the workspace.
struct BcgWork {
  double* rho;        // k   rho of the last completed iteration (1 at start)
  double* rho_new;    // k   <r0, r> of the current iteration
  double* alpha;      // k
  double* omega;      // k
  double* omega_new;  // k
  int* step;          // k
  int* act;           // k   the loop condition for the next iteration
  int* nc;            // k   the stopping test's "not converged" at the last check
  double* pa;         // k × parts partials
  double* pb;
  double* pn1;
  double* pn2;
  int parts;
};

static int64_t bcg_ws_bytes(int k, int64_t n) {
  const int P = kparts(n);
  return 256 + (int64_t)k * 5 * 8 + (int64_t)k * 3 * 4 + 256 + 4LL * k * P * 8 + 256;
}

static BcgWork bcg_carve(void* work, int k, int64_t n) {
  BcgWork w;
  char* p = reinterpret_cast<char*>(work) + 256;
  w.parts = kparts(n);
  w.rho = reinterpret_cast<double*>(p); p += (int64_t)k * 8;
  w.rho_new = reinterpret_cast<double*>(p); p += (int64_t)k * 8;
  w.alpha = reinterpret_cast<double*>(p); p += (int64_t)k * 8;
  w.omega = reinterpret_cast<double*>(p); p += (int64_t)k * 8;
  w.omega_new = reinterpret_cast<double*>(p); p += (int64_t)k * 8;
  w.step = reinterpret_cast<int*>(p); p += (int64_t)k * 4;
  w.act = reinterpret_cast<int*>(p); p += (int64_t)k * 4;
  w.nc = reinterpret_cast<int*>(p); p += (int64_t)k * 4;
  p = reinterpret_cast<char*>(((uintptr_t)p + 255) & ~(uintptr_t)255);
  const int64_t kp = (int64_t)k * w.parts;
  w.pa = reinterpret_cast<double*>(p); p += kp * 8;
  w.pb = reinterpret_cast<double*>(p); p += kp * 8;
  w.pn1 = reinterpret_cast<double*>(p); p += kp * 8;
  w.pn2 = reinterpret_cast<double*>(p);
  return w;
}

// r0 = r (the shadow residual), p = v = 0; alpha = omega = rho = 1; the first
// loop condition: no breakdown at (1, 1, 1), diff = +inf fails the stopping
// test when there is a scale (and n > 0), step 0 < max_steps.
__global__ void bcg_start_kernel(int64_t n, int k, BcgWork w, const double* __restrict__ r,
                                 double* __restrict__ r0, double* __restrict__ p,
                                 double* __restrict__ v, int64_t max_steps, int has_scale) {
  const int c = blockIdx.y;
  const int64_t o = (int64_t)c * n;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    r0[o + i] = r[o + i];
    p[o + i] = 0.0;
    v[o + i] = 0.0;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    w.rho[c] = 1.0;
    w.rho_new[c] = 1.0;
    w.alpha[c] = 1.0;
    w.omega[c] = 1.0;
    w.omega_new[c] = 1.0;
    w.step[c] = 0;
    const int nc = has_scale ? (n > 0) : 1;
    w.nc[c] = nc;
    w.act[c] = nc && (max_steps > 0);
  }
}

// Partial <x1, y1> (and <x2, y2> when x2 is given) per (part, vector) of the
// active right-hand sides.
__global__ void __launch_bounds__(kKThreads)
bcg_dot_partial_kernel(int64_t n, BcgWork w, const double* __restrict__ x1,
                       const double* __restrict__ y1, double* __restrict__ part1,
                       const double* __restrict__ x2, const double* __restrict__ y2,
                       double* __restrict__ part2) {
  __shared__ double sm[kKThreads / 32];
  const int c = blockIdx.y;
  if (!w.act[c]) return;  // uniform over the block
  const int64_t o = (int64_t)c * n;
  double a1 = 0.0, a2 = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    a1 = fma(x1[o + i], y1[o + i], a1);
    if (x2) a2 = fma(x2[o + i], y2[o + i], a2);
  }
  const double s1 = block_reduce<false>(a1, sm);
  if (threadIdx.x == 0) part1[(int64_t)c * gridDim.x + blockIdx.x] = s1;
  if (x2) {
    const double s2 = block_reduce<false>(a2, sm);
    if (threadIdx.x == 0) part2[(int64_t)c * gridDim.x + blockIdx.x] = s2;
  }
}

// rho' = <r0, r>, beta = (rho'/rho)(alpha/omega), p = r + beta (p - omega v)
// (bicgstab.py:138-140).  Every CTA combines the partials itself (the same
// fixed order, so the same value); CTA 0 records rho'.
__global__ void __launch_bounds__(kKThreads)
bcg_direction_kernel(int64_t n, BcgWork w, const double* __restrict__ r,
                     const double* __restrict__ v, double* __restrict__ p) {
  const int c = blockIdx.y;
  if (!w.act[c]) return;
  const double rho_new = combine(w.pa + (int64_t)c * w.parts, w.parts, false);
  const double om = w.omega[c];
  const double beta = (rho_new / w.rho[c]) * (w.alpha[c] / om);
  if (blockIdx.x == 0 && threadIdx.x == 0) w.rho_new[c] = rho_new;
  const int64_t o = (int64_t)c * n;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    p[o + i] = fma(beta, fma(-om, v[o + i], p[o + i]), r[o + i]);
}

// alpha = rho' / <r0, v>, s = r - alpha v (bicgstab.py:147-148).
__global__ void __launch_bounds__(kKThreads)
bcg_s_kernel(int64_t n, BcgWork w, const double* __restrict__ r, const double* __restrict__ v,
             double* __restrict__ s) {
  const int c = blockIdx.y;
  if (!w.act[c]) return;
  const double den = combine(w.pb + (int64_t)c * w.parts, w.parts, false);
  const double a = w.rho_new[c] / den;
  if (blockIdx.x == 0 && threadIdx.x == 0) w.alpha[c] = a;
  const int64_t o = (int64_t)c * n;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    s[o + i] = fma(-a, v[o + i], r[o + i]);
}

// omega = <s, t>/<t, t>, diff = alpha x + omega z, y += diff,
// r = s - omega t (bicgstab.py:153-157), with the partial maxima of the
// stopping test on the new r and diff (y_scale from the new y).
__global__ void __launch_bounds__(kKThreads)
bcg_update_kernel(int64_t n, BcgWork w, const double* __restrict__ x,
                  const double* __restrict__ z, const double* s, const double* __restrict__ t,
                  const double* __restrict__ b, double* __restrict__ y, double* r, double rtol,
                  double atol) {
  __shared__ double sm[kKThreads / 32];
  const int c = blockIdx.y;
  if (!w.act[c]) return;
  const double st = combine(w.pa + (int64_t)c * w.parts, w.parts, false);
  const double tt = combine(w.pb + (int64_t)c * w.parts, w.parts, false);
  const double om = st / tt;
  const double a = w.alpha[c];
  if (blockIdx.x == 0 && threadIdx.x == 0) w.omega_new[c] = om;
  const int64_t o = (int64_t)c * n;
  int code1 = 0, code2 = 0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const double d = fma(a, x[o + i], om * z[o + i]);
    const double yn = y[o + i] + d;
    y[o + i] = yn;
    const double rn = fma(-om, t[o + i], s[o + i]);
    r[o + i] = rn;
    code1 = max(code1, ratio_code(rn, fma(rtol, fabs(b[o + i]), atol)));
    code2 = max(code2, ratio_code(d, fma(rtol, fabs(yn), atol)));
  }
  const double m1 = block_reduce<true>(code_class(code1), sm);
  const double m2 = block_reduce<true>(code_class(code2), sm);
  if (threadIdx.x == 0) {
    w.pn1[(int64_t)c * gridDim.x + blockIdx.x] = m1;
    w.pn2[(int64_t)c * gridDim.x + blockIdx.x] = m2;
  }
}

// End of an iteration: rho, omega take the new values, step += 1, and the
// loop condition for the next one (bicgstab.py:107-133, FP64 breakdown test).
__global__ void bcg_finalize_kernel(int k, BcgWork w, int64_t max_steps, int has_scale) {
  const int c = blockIdx.x;
  if (!w.act[c]) return;
  const double n1 = combine(w.pn1 + (int64_t)c * w.parts, w.parts, true);
  const double n2 = combine(w.pn2 + (int64_t)c * w.parts, w.parts, true);
  if (threadIdx.x == 0) {
    const double rho = w.rho_new[c], om = w.omega_new[c], a = w.alpha[c];
    w.rho[c] = rho;
    w.omega[c] = om;
    const int st = w.step[c] + 1;
    w.step[c] = st;
    const int nc = has_scale ? ((n1 > 1.0) || (n2 > 1.0)) : 1;
    w.nc[c] = nc;
    const bool brk = (om == 0.0) || (a == 0.0) || (rho == 0.0);
    w.act[c] = !brk && nc && (st < max_steps);
  }
}

__global__ void bcg_status_kernel(int k, BcgWork w, int32_t* steps, int32_t* active,
                                  double* scal, int32_t* nc) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= k) return;
  if (steps) steps[c] = w.step[c];
  if (active) active[c] = w.act[c];
  if (scal) {
    scal[c] = w.rho[c];
    scal[k + c] = w.alpha[c];
    scal[2 * k + c] = w.omega[c];
  }
  if (nc) nc[c] = w.nc[c];
}

}  // namespace lxgb

using namespace lxgb;

// ------------------------------- C ABI --------------------------------------

extern "C" int64_t lxgb_bicgstab_workspace_size(int32_t nrhs, int64_t n) {
  return bcg_ws_bytes(nrhs > 0 ? nrhs : 1, n > 0 ? n : 1);
}

static int bcg_check(int32_t k, int64_t n, void* work, int64_t wbytes) {
  LXGB_REQUIRE(k >= 1 && k <= 65535 && n >= 0, "bicgstab: bad sizes");
  LXGB_REQUIRE(work && ((uintptr_t)work & 255) == 0,
               "bicgstab: workspace must be 256-byte aligned");
  if (wbytes < bcg_ws_bytes(k, n > 0 ? n : 1)) {
    set_last_error("bicgstab: workspace too small");
    return LXGB_WORKSPACE_TOO_SMALL;
  }
  return LXGB_SUCCESSFUL;
}

static dim3 bcg_grid(const BcgWork& w, int k) { return dim3((unsigned)w.parts, (unsigned)k); }

extern "C" int lxgb_bicgstab_start(int32_t k, int64_t n, const double* r, double* r0, double* p,
                                   double* v, int64_t max_steps, int32_t has_scale, void* work,
                                   int64_t wbytes, void* stream) {
  int rc = bcg_check(k, n, work, wbytes);
  if (rc) return rc;
  LXGB_REQUIRE(n == 0 || (r && r0 && p && v), "bicgstab: null pointer");
  BcgWork w = bcg_carve(work, k, n > 0 ? n : 1);
  bcg_start_kernel<<<bcg_grid(w, k), kKThreads, 0, as_stream(stream)>>>(n, k, w, r, r0, p, v,
                                                                      max_steps, has_scale);
  return check_launch("bicgstab_start");
}

extern "C" int lxgb_bicgstab_direction(int32_t k, int64_t n, const double* r0, const double* r,
                                       const double* v, double* p, void* work, int64_t wbytes,
                                       void* stream) {
  int rc = bcg_check(k, n, work, wbytes);
  if (rc) return rc;
  if (n == 0) return LXGB_SUCCESSFUL;
  LXGB_REQUIRE(r0 && r && v && p, "bicgstab: null pointer");
  cudaStream_t st = as_stream(stream);
  BcgWork w = bcg_carve(work, k, n);
  const dim3 g = bcg_grid(w, k);
  bcg_dot_partial_kernel<<<g, kKThreads, 0, st>>>(n, w, r0, r, w.pa, nullptr, nullptr, nullptr);
  bcg_direction_kernel<<<g, kKThreads, 0, st>>>(n, w, r, v, p);
  return check_launch("bicgstab_direction");
}

extern "C" int lxgb_bicgstab_s(int32_t k, int64_t n, const double* r0, const double* r,
                               const double* v, double* s, void* work, int64_t wbytes,
                               void* stream) {
  int rc = bcg_check(k, n, work, wbytes);
  if (rc) return rc;
  if (n == 0) return LXGB_SUCCESSFUL;
  LXGB_REQUIRE(r0 && r && v && s && s != r, "bicgstab: null or aliased pointer");
  cudaStream_t st = as_stream(stream);
  BcgWork w = bcg_carve(work, k, n);
  const dim3 g = bcg_grid(w, k);
  bcg_dot_partial_kernel<<<g, kKThreads, 0, st>>>(n, w, r0, v, w.pb, nullptr, nullptr, nullptr);
  bcg_s_kernel<<<g, kKThreads, 0, st>>>(n, w, r, v, s);
  return check_launch("bicgstab_s");
}

extern "C" int lxgb_bicgstab_update(int32_t k, int64_t n, const double* x, const double* z,
                                    const double* s, const double* t, const double* b, double* y,
                                    double* r, double rtol, double atol, int64_t max_steps,
                                    int32_t has_scale, void* work, int64_t wbytes, void* stream) {
  int rc = bcg_check(k, n, work, wbytes);
  if (rc) return rc;
  if (n == 0) return LXGB_SUCCESSFUL;
  LXGB_REQUIRE(x && z && s && t && b && y && r && r != s && r != t && r != z && r != x &&
                   y != x && y != z && y != s && y != t,
               "bicgstab: null or aliased pointer");
  cudaStream_t st = as_stream(stream);
  BcgWork w = bcg_carve(work, k, n);
  const dim3 g = bcg_grid(w, k);
  bcg_dot_partial_kernel<<<g, kKThreads, 0, st>>>(n, w, s, t, w.pa, t, t, w.pb);
  bcg_update_kernel<<<g, kKThreads, 0, st>>>(n, w, x, z, s, t, b, y, r, rtol, atol);
  bcg_finalize_kernel<<<k, 32, 0, st>>>(k, w, max_steps, has_scale);
  return check_launch("bicgstab_update");
}

extern "C" int lxgb_bicgstab_status(int32_t k, int64_t n, int32_t* steps, int32_t* active,
                                    double* scal, int32_t* nc, void* work, int64_t wbytes,
                                    void* stream) {
  int rc = bcg_check(k, n, work, wbytes);
  if (rc) return rc;
  BcgWork w = bcg_carve(work, k, n > 0 ? n : 1);
  bcg_status_kernel<<<(k + 127) / 128, 128, 0, as_stream(stream)>>>(k, w, steps, active, scal,
                                                                   nc);
  return check_launch("bicgstab_status");
}
