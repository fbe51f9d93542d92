// Device side of the Krylov solvers (CG, GMRES) for k right-hand sides at
// once, FP64, plus the 5-point Poisson stencil operator.
//
// Vectors of a k-RHS block are stored back to back: vector c of length n at
// base + c*n.  lineax runs its solvers as lax.while_loops whose per-iteration
// condition needs reductions; here the loop body is a fixed sequence of
// launches and every right-hand side carries device-side flags, so an
// iteration of a converged (inactive) right-hand side changes nothing — the
// host may run iterations past convergence and only checks the flags now and
// then.  Reductions are two-stage (per-CTA partials, then one CTA per vector
// combining them in index order), so results do not depend on timing.
#include <math.h>

#include <vector>

#include "common.cuh"
#include "krylov.cuh"

namespace lxgb {

// ---------------------------------------------------------------------------
// CG state (per right-hand side c, in the workspace):
//   gamma[2][k]  <z, r> of the current / next iteration (double-buffered)
//   alpha[k], beta[k]
//   step[k] (int), act[2][k] (int)
//   partials: pa[k][P] (dot), pn2[k][P] (max |diff/y_scale|),
//             pb[k][P] (dot), pn1[k][P] (max |r/b_scale|)
// ---------------------------------------------------------------------------
struct CgWork {
  double* gamma;  // 2k
  double* alpha;  // k
  double* beta;   // k
  int* step;      // k
  int* act;       // 2k
  double* pa;
  double* pn2;
  double* pb;
  double* pn1;
  int parts;
};

static int64_t cg_ws_bytes(int k, int64_t n) {
  const int P = kparts(n);
  return 256 + (int64_t)k * (2 + 1 + 1) * 8 + (int64_t)k * 3 * 4 + 256 +
         4LL * k * P * 8 + 256;
}

static CgWork cg_carve(void* work, int k, int64_t n) {
  CgWork w;
  char* p = reinterpret_cast<char*>(work) + 256;
  w.parts = kparts(n);
  w.gamma = reinterpret_cast<double*>(p); p += 2LL * k * 8;
  w.alpha = reinterpret_cast<double*>(p); p += (int64_t)k * 8;
  w.beta = reinterpret_cast<double*>(p); p += (int64_t)k * 8;
  w.step = reinterpret_cast<int*>(p); p += (int64_t)k * 4;
  w.act = reinterpret_cast<int*>(p); p += 2LL * k * 4;
  p = reinterpret_cast<char*>(((uintptr_t)p + 255) & ~(uintptr_t)255);
  const int64_t kp = (int64_t)k * w.parts;
  w.pa = reinterpret_cast<double*>(p); p += kp * 8;
  w.pn2 = reinterpret_cast<double*>(p); p += kp * 8;
  w.pb = reinterpret_cast<double*>(p); p += kp * 8;
  w.pn1 = reinterpret_cast<double*>(p);
  return w;
}

// partial <x, y> per (vector, part); when n1 is given also partial
// max |r / (atol + rtol |b|)| with r = y, b = bvec.
__global__ void __launch_bounds__(kKThreads)
cg_dot_partial_kernel(int64_t n, const double* __restrict__ x, const double* __restrict__ y,
                      double* __restrict__ part, const double* __restrict__ bvec, double rtol,
                      double atol, double* __restrict__ pn1) {
  __shared__ double sm[kKThreads / 32];
  const int c = blockIdx.y;
  const double* xc = x + (int64_t)c * n;
  const double* yc = y + (int64_t)c * n;
  double acc = 0.0;
  int code = 0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const double yi = yc[i];
    acc = fma(xc[i], yi, acc);
    if (pn1) code = max(code, ratio_code(yi, fma(rtol, fabs(bvec[(int64_t)c * n + i]), atol)));
  }
  const double mx = code_class(code);
  const double s = block_reduce<false>(acc, sm);
  if (threadIdx.x == 0) part[(int64_t)c * gridDim.x + blockIdx.x] = s;
  if (pn1) {
    const double m = block_reduce<true>(mx, sm);
    if (threadIdx.x == 0) pn1[(int64_t)c * gridDim.x + blockIdx.x] = m;
  }
}

// gamma0 = <z, r>; p = z handled by the caller; act0 = gamma0 > 0 &&
// max_steps > 0 (the initial two-space test holds: diff = inf).
__global__ void cg_start_finalize_kernel(int k, CgWork w, int64_t max_steps, int64_t n,
                                         int has_scale) {
  const int c = blockIdx.x;
  const double g = combine(w.pb + (int64_t)c * w.parts, w.parts, false);
  if (threadIdx.x == 0) {
    w.gamma[c] = g;  // parity 0
    w.step[c] = 0;
    const bool nc = has_scale ? (n > 0) : true;
    w.act[c] = (g > 0.0) && (max_steps > 0) && nc;
    w.act[k + c] = 0;
  }
}

// alpha = gamma / <A p, p>, NaN when |<A p, p>| <= 100 rcond |gamma|
// (lineax/_solver/cg.py:172-178).
__global__ void cg_alpha_kernel(int k, CgWork w, int cur, double rcond) {
  const int c = blockIdx.x;
  const double inner = combine(w.pa + (int64_t)c * w.parts, w.parts, false);
  if (threadIdx.x == 0) {
    const double g = w.gamma[cur * k + c];
    double a = g / inner;
    if (!(fabs(inner) > 100.0 * rcond * fabs(g))) a = NAN;
    w.alpha[c] = a;
  }
}

// y += alpha p; partial max |alpha p / (atol + rtol |y|)|; r -= alpha A p
// unless the residual is recomputed this step.
__global__ void __launch_bounds__(kKThreads)
cg_update_kernel(int64_t n, int k, CgWork w, int cur, const double* __restrict__ p,
                 const double* __restrict__ mat_p, double* __restrict__ y, double* __restrict__ r,
                 int cheap_r, double rtol, double atol) {
  __shared__ double sm[kKThreads / 32];
  const int c = blockIdx.y;
  const bool act = w.act[cur * k + c] != 0;
  int code = 0;
  if (act) {
    const double a = w.alpha[c];
    const int64_t o = (int64_t)c * n;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
      const double d = a * p[o + i];
      const double yn = y[o + i] + d;
      y[o + i] = yn;
      code = max(code, ratio_code(d, fma(rtol, fabs(yn), atol)));
      if (cheap_r) r[o + i] = fma(-a, mat_p[o + i], r[o + i]);
    }
  }
  const double mx = code_class(code);
  const double m = block_reduce<true>(mx, sm);
  if (threadIdx.x == 0) w.pn2[(int64_t)c * gridDim.x + blockIdx.x] = m;
}

// r = b - A y for active right-hand sides (the periodic true residual).
__global__ void cg_true_residual_kernel(int64_t n, int k, CgWork w, int cur,
                                        const double* __restrict__ b,
                                        const double* __restrict__ ay, double* __restrict__ r) {
  const int c = blockIdx.y;
  if (!w.act[cur * k + c]) return;
  const int64_t o = (int64_t)c * n;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    r[o + i] = b[o + i] - ay[o + i];
}

// gamma' = <z, r>, beta = gamma'/gamma, step += 1, next flag from the loop
// condition of lineax/_solver/cg.py:162-167.
__global__ void cg_beta_kernel(int k, CgWork w, int cur, int64_t max_steps, int has_scale) {
  const int c = blockIdx.x;
  const double g = combine(w.pb + (int64_t)c * w.parts, w.parts, false);
  const double n1 = combine(w.pn1 + (int64_t)c * w.parts, w.parts, true);
  const double n2 = combine(w.pn2 + (int64_t)c * w.parts, w.parts, true);
  if (threadIdx.x == 0) {
    const int nxt = cur ^ 1;
    if (w.act[cur * k + c]) {
      const double gp = w.gamma[cur * k + c];
      const int st = w.step[c] + 1;
      w.step[c] = st;
      w.beta[c] = g / gp;
      w.gamma[nxt * k + c] = g;
      const bool nc = has_scale ? ((n1 > 1.0) || (n2 > 1.0)) : true;
      w.act[nxt * k + c] = (g > 0.0) && (st < max_steps) && nc;
    } else {
      w.gamma[nxt * k + c] = w.gamma[cur * k + c];
      w.beta[c] = 0.0;
      w.act[nxt * k + c] = 0;
    }
  }
}

// p = z + beta p for right-hand sides active in this iteration.
__global__ void cg_p_kernel(int64_t n, int k, CgWork w, int cur, const double* __restrict__ z,
                            double* __restrict__ p) {
  const int c = blockIdx.y;
  if (!w.act[cur * k + c]) return;
  const double bt = w.beta[c];
  const int64_t o = (int64_t)c * n;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    p[o + i] = fma(bt, p[o + i], z[o + i]);
}

__global__ void copy_vec_kernel(int64_t total, const double* __restrict__ src,
                                double* __restrict__ dst) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total;
       i += (int64_t)gridDim.x * blockDim.x)
    dst[i] = src[i];
}

// 5-point negative Laplacian on an nx×ny interior grid with Dirichlet zero
// boundary: (A u)[i,j] = 4u[i,j] - u[i-1,j] - u[i+1,j] - u[i,j-1] - u[i,j+1],
// scaled by `scale`; k vectors back to back.  Evaluated as
// fma(4, u[i,j], -((u[i-1,j] + u[i+1,j]) + (u[i,j-1] + u[i,j+1]))).
__global__ void __launch_bounds__(256)
poisson5_kernel(int64_t nx, int64_t ny, int k, double scale, const double* __restrict__ u,
                double* __restrict__ out) {
  const int64_t n = nx * ny;
  const int c = blockIdx.z;
  const int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;  // column (fast)
  const int64_t i = blockIdx.y;                                        // row
  if (j >= ny) return;
  const double* uc = u + (int64_t)c * n;
  const int64_t o = i * ny + j;
  const double cen = uc[o];
  const double up = (i > 0) ? uc[o - ny] : 0.0;
  const double dn = (i + 1 < nx) ? uc[o + ny] : 0.0;
  const double lf = (j > 0) ? uc[o - 1] : 0.0;
  const double rt = (j + 1 < ny) ? uc[o + 1] : 0.0;
  // four FP64 operations (the FP64 pipe bounds this kernel on GB300)
  const double v = fma(4.0, cen, -((up + dn) + (lf + rt)));
  out[(int64_t)c * n + o] = (scale == 1.0) ? v : scale * v;
}

// ---------------------------------------------------------------------------
// Generic k-vector reductions for GMRES: op 0 dot, 1 max|x|, 2 sum x².
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kKThreads)
kreduce_partial_kernel(int op, int64_t n, const double* __restrict__ x, int64_t ldx,
                       const double* __restrict__ y, int64_t ldy, double* __restrict__ part) {
  __shared__ double sm[kKThreads / 32];
  const int c = blockIdx.y;
  const double* xc = x + (int64_t)c * ldx;
  const double* yc = y ? y + (int64_t)c * ldy : nullptr;
  double acc = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const double v = xc[i];
    if (op == 0) acc = fma(v, yc[i], acc);
    else if (op == 1) acc = nanmax2(acc, fabs(v));
    else acc = fma(v, v, acc);
  }
  const double s = (op == 1) ? block_reduce<true>(acc, sm) : block_reduce<false>(acc, sm);
  if (threadIdx.x == 0) part[(int64_t)c * gridDim.x + blockIdx.x] = s;
}

__global__ void kreduce_final_kernel(int op, int parts, const double* __restrict__ part,
                                     double* __restrict__ out) {
  const int c = blockIdx.x;
  const double v = combine(part + (int64_t)c * parts, parts, op == 1);
  if (threadIdx.x == 0) out[c] = v;
}

}  // namespace lxgb

using namespace lxgb;

// ------------------------------- C ABI --------------------------------------

extern "C" int64_t lxgb_cg_workspace_size(int32_t nrhs, int64_t n) {
  return cg_ws_bytes(nrhs > 0 ? nrhs : 1, n > 0 ? n : 1);
}

static int cg_check(int32_t k, int64_t n, void* work, int64_t wbytes) {
  LXGB_REQUIRE(k >= 1 && k <= 65535 && n >= 0, "cg: bad sizes");
  LXGB_REQUIRE(work && ((uintptr_t)work & 255) == 0, "cg: workspace must be 256-byte aligned");
  if (wbytes < cg_ws_bytes(k, n > 0 ? n : 1)) {
    set_last_error("cg: workspace too small");
    return LXGB_WORKSPACE_TOO_SMALL;
  }
  return LXGB_SUCCESSFUL;
}

extern "C" int lxgb_cg_start(int32_t k, int64_t n, const double* r, const double* z, double* p,
                             int64_t max_steps, int32_t has_scale, void* work, int64_t wbytes,
                             void* stream) {
  int rc = cg_check(k, n, work, wbytes);
  if (rc) return rc;
  LXGB_REQUIRE(n == 0 || (r && z && p), "cg: null pointer");
  cudaStream_t st = as_stream(stream);
  CgWork w = cg_carve(work, k, n > 0 ? n : 1);
  if (n > 0) {
    copy_vec_kernel<<<2 * sm_count(), 256, 0, st>>>(n * k, z, p);
    dim3 g(w.parts, k);
    cg_dot_partial_kernel<<<g, kKThreads, 0, st>>>(n, z, r, w.pb, nullptr, 0.0, 0.0, nullptr);
  } else {
    LXGB_CUDA_TRY(cudaMemsetAsync(w.pb, 0, (size_t)k * w.parts * 8, st), "cg: memset");
  }
  cg_start_finalize_kernel<<<k, 32, 0, st>>>(k, w, max_steps, n, has_scale);
  return check_launch("cg_start");
}

extern "C" int lxgb_cg_step_alpha(int32_t k, int64_t n, const double* mat_p, double* p, double* y,
                                  double* r, int32_t cheap_r, int32_t parity, double rtol,
                                  double atol, double rcond, void* work, int64_t wbytes,
                                  void* stream) {
  int rc = cg_check(k, n, work, wbytes);
  if (rc) return rc;
  if (n == 0) return LXGB_SUCCESSFUL;
  LXGB_REQUIRE(mat_p && p && y && r, "cg: null pointer");
  cudaStream_t st = as_stream(stream);
  CgWork w = cg_carve(work, k, n);
  dim3 g(w.parts, k);
  cg_dot_partial_kernel<<<g, kKThreads, 0, st>>>(n, mat_p, p, w.pa, nullptr, 0.0, 0.0, nullptr);
  cg_alpha_kernel<<<k, 32, 0, st>>>(k, w, parity & 1, rcond);
  cg_update_kernel<<<g, kKThreads, 0, st>>>(n, k, w, parity & 1, p, mat_p, y, r, cheap_r, rtol,
                                            atol);
  return check_launch("cg_step_alpha");
}

extern "C" int lxgb_cg_true_residual(int32_t k, int64_t n, const double* b, const double* ay,
                                     double* r, int32_t parity, void* work, int64_t wbytes,
                                     void* stream) {
  int rc = cg_check(k, n, work, wbytes);
  if (rc) return rc;
  if (n == 0) return LXGB_SUCCESSFUL;
  LXGB_REQUIRE(b && ay && r, "cg: null pointer");
  CgWork w = cg_carve(work, k, n);
  dim3 g(w.parts, k);
  cg_true_residual_kernel<<<g, kKThreads, 0, as_stream(stream)>>>(n, k, w, parity & 1, b, ay, r);
  return check_launch("cg_true_residual");
}

extern "C" int lxgb_cg_step_beta(int32_t k, int64_t n, const double* b, const double* r,
                                 const double* z, double* p, int32_t parity, int64_t max_steps,
                                 int32_t has_scale, double rtol, double atol, void* work,
                                 int64_t wbytes, void* stream) {
  int rc = cg_check(k, n, work, wbytes);
  if (rc) return rc;
  if (n == 0) return LXGB_SUCCESSFUL;
  LXGB_REQUIRE(b && r && z && p, "cg: null pointer");
  cudaStream_t st = as_stream(stream);
  CgWork w = cg_carve(work, k, n);
  dim3 g(w.parts, k);
  cg_dot_partial_kernel<<<g, kKThreads, 0, st>>>(n, z, r, w.pb, b, rtol, atol, w.pn1);
  cg_beta_kernel<<<k, 32, 0, st>>>(k, w, parity & 1, max_steps, has_scale);
  cg_p_kernel<<<g, kKThreads, 0, st>>>(n, k, w, parity & 1, z, p);
  return check_launch("cg_step_beta");
}

// Copies per-RHS step counts and the flags of the given parity to device
// arrays the caller reads.
__global__ void cg_status_kernel(int k, CgWork w, int cur, int32_t* steps, int32_t* active) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= k) return;
  steps[c] = w.step[c];
  active[c] = w.act[cur * k + c];
}

extern "C" int lxgb_cg_status(int32_t k, int64_t n, int32_t parity, int32_t* steps,
                              int32_t* active, void* work, int64_t wbytes, void* stream) {
  int rc = cg_check(k, n, work, wbytes);
  if (rc) return rc;
  LXGB_REQUIRE(steps && active, "cg: null pointer");
  CgWork w = cg_carve(work, k, n > 0 ? n : 1);
  cg_status_kernel<<<(k + 127) / 128, 128, 0, as_stream(stream)>>>(k, w, parity & 1, steps,
                                                                   active);
  return check_launch("cg_status");
}

extern "C" int lxgb_poisson5_f64(int64_t nx, int64_t ny, int32_t k, double scale, const double* u,
                                 double* out, void* stream) {
  LXGB_REQUIRE(nx >= 0 && ny >= 0 && k >= 0, "poisson5: negative size");
  if (nx == 0 || ny == 0 || k == 0) return LXGB_SUCCESSFUL;
  LXGB_REQUIRE(u && out && u != out, "poisson5: bad pointers");
  LXGB_REQUIRE(nx <= 65535 && k <= 65535, "poisson5: grid too large");
  dim3 g((unsigned)((ny + 255) / 256), (unsigned)nx, (unsigned)k);
  poisson5_kernel<<<g, 256, 0, as_stream(stream)>>>(nx, ny, k, scale, u, out);
  return check_launch("poisson5");
}

extern "C" int64_t lxgb_kreduce_workspace_size(int32_t k, int64_t n) {
  return (int64_t)(k > 0 ? k : 1) * kparts(n > 0 ? n : 1) * 8;
}

extern "C" int lxgb_kreduce_f64(int32_t op, int32_t k, int64_t n, const double* x, int64_t ldx,
                                const double* y, int64_t ldy, double* out, void* work,
                                int64_t wbytes, void* stream) {
  LXGB_REQUIRE(op >= 0 && op <= 2 && k >= 1 && k <= 65535 && n >= 0, "kreduce: bad arguments");
  LXGB_REQUIRE(out && work && (n == 0 || x) && (op != 0 || n == 0 || y), "kreduce: null pointer");
  if (wbytes < lxgb_kreduce_workspace_size(k, n)) {
    set_last_error("kreduce: workspace too small");
    return LXGB_WORKSPACE_TOO_SMALL;
  }
  cudaStream_t st = as_stream(stream);
  const int P = kparts(n > 0 ? n : 1);
  double* part = reinterpret_cast<double*>(work);
  if (n == 0) {
    LXGB_CUDA_TRY(cudaMemsetAsync(part, 0, (size_t)k * P * 8, st), "kreduce: memset");
  } else {
    kreduce_partial_kernel<<<dim3(P, k), kKThreads, 0, st>>>(op, n, x, ldx, y, ldy, part);
  }
  kreduce_final_kernel<<<k, 32, 0, st>>>(op, P, part, out);
  return check_launch("kreduce");
}

// ---------------------------------------------------------------------------
// GMRES (lineax/_solver/gmres.py:106-413) for k right-hand sides.
//
// Per right-hand side c the workspace holds:
//   V[c]     (R+1) basis vectors of length n (R = restart)
//   coeff[c] R×(R+1) rows of projections (lineax's coeff_mat)
//   z[c]     R least-squares coefficients
//   scalars  r_norm, step_norm, r_min, flags (act, bd, breakdown, deferred,
//            step, stag, not-converged-at-exit)
// and partial sums for the reductions.  Every kernel honours the flags, so
// the host may launch the fixed sequence for all right-hand sides.
// ---------------------------------------------------------------------------
constexpr int kGmMaxRestart = 128;

struct GmWork {
  double* V;       // k*(R+1)*n
  double* coeff;   // k*R*(R+1)
  double* z;       // k*R
  double* proj;    // k*(R+1)
  double* sc;      // k*8 scalars: 0 r_norm 1 step_norm 2 r_min 3 wnorm
  int* fl;         // k*8 ints: 0 act[0] 1 act[1] 2 bd 3 breakdown 4 deferred 5 step 6 stag 7 nc_exit
  double* part;    // k*P*(R+2)
  int parts;
  int R;
};

// Exactly the regions gm_carve takes, each rounded up to 256 bytes.
static int64_t gm_ws_bytes(int k, int64_t n, int R) {
  const int P = kparts(n);
  auto r256 = [](int64_t b) { return (b + 255) & ~(int64_t)255; };
  int64_t b = 256;
  b += r256((int64_t)k * (R + 1) * n * 8);
  b += r256((int64_t)k * R * (R + 1) * 8) + r256((int64_t)k * R * 8) +
       r256((int64_t)k * (R + 1) * 8);
  b += r256((int64_t)k * 8 * 8) + r256((int64_t)k * 8 * 4);
  b += r256((int64_t)k * P * (R + 2) * 8);
  return b;
}

static GmWork gm_carve(void* work, int k, int64_t n, int R) {
  GmWork w;
  w.R = R;
  w.parts = kparts(n);
  char* p = reinterpret_cast<char*>(work) + 256;
  auto take = [&](int64_t bytes) {
    char* q = p;
    p += (bytes + 255) & ~(int64_t)255;
    return q;
  };
  w.V = reinterpret_cast<double*>(take((int64_t)k * (R + 1) * n * 8));
  w.coeff = reinterpret_cast<double*>(take((int64_t)k * R * (R + 1) * 8));
  w.z = reinterpret_cast<double*>(take((int64_t)k * R * 8));
  w.proj = reinterpret_cast<double*>(take((int64_t)k * (R + 1) * 8));
  w.sc = reinterpret_cast<double*>(take((int64_t)k * 8 * 8));
  w.fl = reinterpret_cast<int*>(take((int64_t)k * 8 * 4));
  w.part = reinterpret_cast<double*>(take((int64_t)k * w.parts * (R + 2) * 8));
  return w;
}

__device__ __forceinline__ bool gm_live(const GmWork& w, int c, int cur) {
  return w.fl[c * 8 + cur] != 0;
}

__global__ void gm_init_kernel(int k, GmWork w) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= k) return;
  for (int q = 0; q < 8; ++q) w.fl[c * 8 + q] = 0;
  w.fl[c * 8 + 0] = 1;  // the first (dummy) pass always runs
  w.sc[c * 8 + 2] = INFINITY;  // r_min
}

// Start of a restart cycle: r_norm = ||r||_2, bd = r_norm < eps,
// V[0] = r / (bd ? inf : r_norm), V[1..R] = 0, coeff = eye(R, R+1)
// (gmres.py:256-268).  Two kernels: partial sums, then normalise+reset.
__global__ void __launch_bounds__(kKThreads)
gm_sumsq_partial_kernel(int64_t n, int k, GmWork w, int cur, const double* __restrict__ x,
                        int64_t ldx) {
  __shared__ double sm[kKThreads / 32];
  const int c = blockIdx.y;
  double acc = 0.0;
  if (gm_live(w, c, cur)) {
    const double* xc = x + (int64_t)c * ldx;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
      acc = fma(xc[i], xc[i], acc);
  }
  const double s = block_reduce<false>(acc, sm);
  if (threadIdx.x == 0) w.part[(int64_t)c * w.parts + blockIdx.x] = s;
}

__device__ __forceinline__ double two_norm_from(double sumsq, double only, int64_t n) {
  return n == 1 ? fabs(only) : sqrt(sumsq);
}

__global__ void gm_cycle_norm_kernel(int k, int64_t n, GmWork w, int cur, const double* r) {
  const int c = blockIdx.x;
  const double ss = combine(w.part + (int64_t)c * w.parts, w.parts, false);
  if (threadIdx.x == 0 && gm_live(w, c, cur)) {
    const double nrm = two_norm_from(ss, r[(int64_t)c * n], n);
    w.sc[c * 8 + 0] = nrm;
    const bool bd = nrm < 2.220446049250313e-16;  // finfo(float64).eps
    w.fl[c * 8 + 2] = bd;
  }
}

__global__ void gm_cycle_reset_kernel(int64_t n, int k, GmWork w, int cur,
                                      const double* __restrict__ r) {
  const int c = blockIdx.y;
  if (!gm_live(w, c, cur)) return;
  const int R = w.R;
  const double nrm = w.sc[c * 8 + 0];
  const double safe = w.fl[c * 8 + 2] ? INFINITY : nrm;
  double* V = w.V + (int64_t)c * (R + 1) * n;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    V[i] = r[(int64_t)c * n + i] / safe;
    for (int j = 1; j <= R; ++j) V[(int64_t)j * n + i] = 0.0;
  }
  if (blockIdx.x == 0) {
    double* cm = w.coeff + (int64_t)c * R * (R + 1);
    for (int e = threadIdx.x; e < R * (R + 1); e += blockDim.x)
      cm[e] = (e / (R + 1) == e % (R + 1)) ? 1.0 : 0.0;
  }
}

// Arnoldi step kk for right-hand sides live and not broken down:
//   partial dots proj[j] = <V[j], w>, j <= kk, and ||w||^2   (gmres.py:355-363)
__global__ void __launch_bounds__(kKThreads)
gm_proj_partial_kernel(int64_t n, int k, GmWork w, int cur, int kk,
                       const double* __restrict__ wv) {
  __shared__ double sm[kKThreads / 32];
  const int c = blockIdx.y;
  const int R = w.R;
  const bool on = gm_live(w, c, cur) && !w.fl[c * 8 + 2];
  const double* V = w.V + (int64_t)c * (R + 1) * n;
  const double* wc = wv + (int64_t)c * n;
  double* part = w.part + (int64_t)c * w.parts * (R + 2);
  for (int j = 0; j <= kk + 1; ++j) {
    double acc = 0.0;
    if (on) {
      for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
           i += (int64_t)gridDim.x * blockDim.x) {
        const double x = wc[i];
        acc = (j <= kk) ? fma(V[(int64_t)j * n + i], x, acc) : fma(x, x, acc);
      }
    }
    const double s = block_reduce<false>(acc, sm);
    if (threadIdx.x == 0) part[(int64_t)(j <= kk ? j : R + 1) * w.parts + blockIdx.x] = s;
  }
}

__global__ void gm_proj_final_kernel(int k, int64_t n, GmWork w, int cur, int kk,
                                     const double* __restrict__ wv) {
  const int c = blockIdx.x;
  const int R = w.R;
  if (!(gm_live(w, c, cur) && !w.fl[c * 8 + 2])) return;
  const double* part = w.part + (int64_t)c * w.parts * (R + 2);
  for (int j = 0; j <= R; ++j) {
    double v = 0.0;
    if (j <= kk) v = combine(part + (int64_t)j * w.parts, w.parts, false);
    if (threadIdx.x == 0) w.proj[c * (R + 1) + j] = v;
  }
  const double ss = combine(part + (int64_t)(R + 1) * w.parts, w.parts, false);
  if (threadIdx.x == 0) w.sc[c * 8 + 1] = two_norm_from(ss, wv[(int64_t)c * n], n);
}

// w -= sum_{j<=kk} proj[j] V[j]; partial ||w||^2 (gmres.py:364-366).
__global__ void __launch_bounds__(kKThreads)
gm_orth_kernel(int64_t n, int k, GmWork w, int cur, int kk, double* __restrict__ wv) {
  __shared__ double sm[kKThreads / 32];
  const int c = blockIdx.y;
  const int R = w.R;
  const bool on = gm_live(w, c, cur) && !w.fl[c * 8 + 2];
  double acc = 0.0;
  if (on) {
    const double* V = w.V + (int64_t)c * (R + 1) * n;
    const double* pj = w.proj + c * (R + 1);
    double* wc = wv + (int64_t)c * n;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
      double s = 0.0;
      for (int j = 0; j <= kk; ++j) s = fma(V[(int64_t)j * n + i], pj[j], s);
      const double x = wc[i] - s;
      wc[i] = x;
      acc = fma(x, x, acc);
    }
  }
  const double s = block_reduce<false>(acc, sm);
  if (threadIdx.x == 0) w.part[(int64_t)c * w.parts * (R + 2) + blockIdx.x] = s;
}

// ||w||, breakdown = ||w|| < ||w_before|| eps, coeff[kk, :] = proj with
// proj[kk+1] = ||w|| (gmres.py:367-398).
__global__ void gm_norm_final_kernel(int k, int64_t n, GmWork w, int cur, int kk,
                                     const double* __restrict__ wv) {
  const int c = blockIdx.x;
  const int R = w.R;
  if (!(gm_live(w, c, cur) && !w.fl[c * 8 + 2])) return;
  const double ss = combine(w.part + (int64_t)c * w.parts * (R + 2), w.parts, false);
  if (threadIdx.x == 0) {
    const double nrm = two_norm_from(ss, wv[(int64_t)c * n], n);
    const double eps = w.sc[c * 8 + 1] * 2.220446049250313e-16;
    w.sc[c * 8 + 3] = nrm;
    const bool bd = nrm < eps;
    double* row = w.coeff + (int64_t)c * R * (R + 1) + (int64_t)kk * (R + 1);
    for (int j = 0; j <= R; ++j) row[j] = (j == kk + 1) ? nrm : w.proj[c * (R + 1) + j];
    w.fl[c * 8 + 2] = bd;
    w.sc[c * 8 + 4] = bd ? INFINITY : nrm;  // divisor for the new basis vector
  }
}

__global__ void gm_store_basis_kernel(int64_t n, int k, GmWork w, int cur, int kk,
                                      const double* __restrict__ wv, const int* __restrict__ was_on) {
  const int c = blockIdx.y;
  if (!was_on[c]) return;
  const int R = w.R;
  const double d = w.sc[c * 8 + 4];
  double* V = w.V + (int64_t)c * (R + 1) * n + (int64_t)(kk + 1) * n;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    V[i] = wv[(int64_t)c * n + i] / d;
}

__global__ void gm_snapshot_kernel(int k, GmWork w, int cur, int* on) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c < k) on[c] = gm_live(w, c, cur) && !w.fl[c * 8 + 2];
}

// Least squares min ||H z - r_norm e1|| with H = coeffᵀ ((R+1)×R) by
// Householder QR in shared memory, one CTA per right-hand side (the
// linear_solve(..., QR()) of gmres.py:301-303).
__global__ void __launch_bounds__(64)
gm_lstsq_kernel(int k, GmWork w, int cur) {
  extern __shared__ double smem_h[];  // (R+1)×(R+1) matrix, then rhs
  __shared__ double s_tau, s_beta, s_scal;
  const int c = blockIdx.x;
  if (!gm_live(w, c, cur)) return;
  const int R = w.R, m = R + 1;
  const int ldh = R + 1;
  double* rhs = smem_h + (int64_t)ldh * m;
#define H(i, j) smem_h[(i) * ldh + (j)]
  const double* cm = w.coeff + (int64_t)c * R * (R + 1);
  for (int e = threadIdx.x; e < m * R; e += blockDim.x) {
    const int i = e / R, j = e % R;
    H(i, j) = cm[(int64_t)j * (R + 1) + i];  // H = coeffᵀ
  }
  for (int i = threadIdx.x; i < m; i += blockDim.x) rhs[i] = (i == 0) ? w.sc[c * 8 + 0] : 0.0;
  __syncthreads();
  for (int j = 0; j < R; ++j) {
    if (threadIdx.x == 0) {
      double ss = 0.0;
      for (int i = j + 1; i < m; ++i) ss = fma(H(i, j), H(i, j), ss);
      const double alpha = H(j, j);
      const double xn = sqrt(ss);
      if (xn == 0.0) {
        s_tau = 0.0;
        s_scal = 1.0;
        s_beta = alpha;
      } else {
        const double beta = -copysign(hypot(alpha, xn), alpha);
        s_tau = (beta - alpha) / beta;
        s_scal = 1.0 / (alpha - beta);
        s_beta = beta;
      }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      for (int i = j + 1; i < m; ++i) H(i, j) *= s_scal;
      H(j, j) = s_beta;
    }
    __syncthreads();
    const double tj = s_tau;
    // apply H_j to the columns > j and to rhs (column index R)
    for (int q = j + 1 + threadIdx.x; q <= R; q += blockDim.x) {
      double* col_rhs = (q == R) ? rhs : nullptr;
      double wq = (q == R) ? rhs[j] : H(j, q);
      for (int i = j + 1; i < m; ++i) wq = fma(H(i, j), col_rhs ? rhs[i] : H(i, q), wq);
      wq *= tj;
      if (col_rhs) {
        rhs[j] -= wq;
        for (int i = j + 1; i < m; ++i) rhs[i] = fma(-wq, H(i, j), rhs[i]);
      } else {
        H(j, q) -= wq;
        for (int i = j + 1; i < m; ++i) H(i, q) = fma(-wq, H(i, j), H(i, q));
      }
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    double* zc = w.z + (int64_t)c * R;
    for (int i = R - 1; i >= 0; --i) {
      double s = rhs[i];
      for (int j = i + 1; j < R; ++j) s = fma(-H(i, j), zc[j], s);
      zc[i] = s / H(i, i);
    }
  }
#undef H
}

// diff = V[:, :R] z, y += diff (gmres.py:304-310); first pass: diff = inf.
__global__ void gm_update_kernel(int64_t n, int k, GmWork w, int cur, int first,
                                 double* __restrict__ y, double* __restrict__ diff) {
  const int c = blockIdx.y;
  if (!gm_live(w, c, cur)) return;
  const int R = w.R;
  const double* V = w.V + (int64_t)c * (R + 1) * n;
  const double* zc = w.z + (int64_t)c * R;
  const int64_t o = (int64_t)c * n;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    if (first) {
      diff[o + i] = INFINITY;
    } else {
      double s = 0.0;
      for (int j = 0; j < R; ++j) s = fma(V[(int64_t)j * n + i], zc[j], s);
      diff[o + i] = s;
      y[o + i] += s;
    }
  }
}

// r = t for live right-hand sides (t = M(b - A y) formed by the caller).
__global__ void gm_set_r_kernel(int64_t n, int k, GmWork w, int cur, const double* __restrict__ t,
                                double* __restrict__ r) {
  const int c = blockIdx.y;
  if (!gm_live(w, c, cur)) return;
  const int64_t o = (int64_t)c * n;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    r[o + i] = t[o + i];
}

// partial max |r|, max |r / b_scale|, max |diff / y_scale| (gmres.py:130-141, 175)
__global__ void __launch_bounds__(kKThreads)
gm_outer_partial_kernel(int64_t n, int k, GmWork w, const double* __restrict__ b,
                        const double* __restrict__ r, const double* __restrict__ diff,
                        const double* __restrict__ y, double rtol, double atol) {
  __shared__ double sm[kKThreads / 32];
  const int c = blockIdx.y;
  const int64_t o = (int64_t)c * n;
  double m0 = 0.0, m1 = 0.0, m2 = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const double ri = r[o + i];
    m0 = nanmax2(m0, fabs(ri));
    m1 = nanmax2(m1, code_class(ratio_code(ri, fma(rtol, fabs(b[o + i]), atol))));
    m2 = nanmax2(m2, code_class(ratio_code(diff[o + i], fma(rtol, fabs(y[o + i]), atol))));
  }
  const int R = w.R;
  double* part = w.part + (int64_t)c * w.parts * (R + 2);
  double v = block_reduce<true>(m0, sm);
  if (threadIdx.x == 0) part[blockIdx.x] = v;
  v = block_reduce<true>(m1, sm);
  if (threadIdx.x == 0) part[w.parts + blockIdx.x] = v;
  v = block_reduce<true>(m2, sm);
  if (threadIdx.x == 0) part[2 * w.parts + blockIdx.x] = v;
}

// Stagnation counter, minimum residual, deferred breakdown, step count and
// the next loop condition (gmres.py:143-188).
__global__ void gm_outer_final_kernel(int k, GmWork w, int cur, int first, int64_t max_steps,
                                      int stagnation_iters, int has_scale) {
  const int c = blockIdx.x;
  const int R = w.R;
  const double* part = w.part + (int64_t)c * w.parts * (R + 2);
  const double rn = combine(part, w.parts, true);
  const double n1 = combine(part + w.parts, w.parts, true);
  const double n2 = combine(part + 2 * w.parts, w.parts, true);
  if (threadIdx.x != 0) return;
  int* f = w.fl + c * 8;
  const int nxt = cur ^ 1;
  if (!f[cur]) {
    f[nxt] = 0;
    return;
  }
  const bool nc = has_scale ? ((n1 > 1.0) || (n2 > 1.0)) : true;
  f[7] = nc;
  const double rmin = w.sc[c * 8 + 2];
  const bool decreased = (rn - rmin) < 0.0;
  f[6] = decreased ? 0 : f[6] + 1;
  w.sc[c * 8 + 2] = (rn != rn || rmin != rmin) ? NAN : fmin(rn, rmin);
  const int bd_now = first ? 0 : f[2];
  f[4] = f[3];    // deferred <- previous breakdown
  f[3] = bd_now;  // breakdown of this cycle
  f[5] = f[5] + 1;
  const bool go = (!f[4]) && (f[6] < stagnation_iters) && nc && (f[5] < max_steps);
  f[nxt] = go ? 1 : 0;
}

__global__ void gm_status_kernel(int k, GmWork w, int cur, int32_t* out) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= k) return;
  const int* f = w.fl + c * 8;
  out[c * 5 + 0] = f[cur];
  out[c * 5 + 1] = f[5];
  out[c * 5 + 2] = f[6];
  out[c * 5 + 3] = f[4];
  out[c * 5 + 4] = f[7];
}

static int gm_check(int32_t k, int64_t n, int32_t R, void* work, int64_t wbytes) {
  LXGB_REQUIRE(k >= 1 && k <= 65535 && n >= 1, "gmres: bad sizes");
  LXGB_REQUIRE(R >= 1 && R <= kGmMaxRestart, "gmres: restart must be in [1, 128]");
  LXGB_REQUIRE(work && ((uintptr_t)work & 255) == 0, "gmres: workspace must be 256-byte aligned");
  if (wbytes < gm_ws_bytes(k, n, R)) {
    set_last_error("gmres: workspace too small");
    return LXGB_WORKSPACE_TOO_SMALL;
  }
  return LXGB_SUCCESSFUL;
}

extern "C" int64_t lxgb_gmres_workspace_size(int32_t nrhs, int64_t n, int32_t restart) {
  return gm_ws_bytes(nrhs > 0 ? nrhs : 1, n > 0 ? n : 1, restart > 0 ? restart : 1);
}

extern "C" int lxgb_gmres_init(int32_t k, int64_t n, int32_t restart, void* work, int64_t wbytes,
                               void* stream) {
  int rc = gm_check(k, n, restart, work, wbytes);
  if (rc) return rc;
  GmWork w = gm_carve(work, k, n, restart);
  gm_init_kernel<<<(k + 127) / 128, 128, 0, as_stream(stream)>>>(k, w);
  return check_launch("gmres_init");
}

// Start of a restart cycle (normalise r into V[0], reset coeff).
extern "C" int lxgb_gmres_cycle_begin(int32_t k, int64_t n, int32_t restart, int32_t parity,
                                      const double* r, void* work, int64_t wbytes, void* stream) {
  int rc = gm_check(k, n, restart, work, wbytes);
  if (rc) return rc;
  LXGB_REQUIRE(r, "gmres: null pointer");
  cudaStream_t st = as_stream(stream);
  GmWork w = gm_carve(work, k, n, restart);
  const int cur = parity & 1;
  dim3 g(w.parts, k);
  gm_sumsq_partial_kernel<<<g, kKThreads, 0, st>>>(n, k, w, cur, r, n);
  gm_cycle_norm_kernel<<<k, 32, 0, st>>>(k, n, w, cur, r);
  gm_cycle_reset_kernel<<<g, kKThreads, 0, st>>>(n, k, w, cur, r);
  return check_launch("gmres_cycle_begin");
}

// Byte offset, from the start of the workspace, of basis vector kk of
// right-hand side 0; vector kk of right-hand side c follows at
// c * (restart + 1) * n doubles further.
extern "C" int64_t lxgb_gmres_basis_offset(int32_t k, int64_t n, int32_t restart, int32_t kk) {
  if (k < 1 || n < 1 || restart < 1 || restart > kGmMaxRestart || kk < 0 || kk > restart)
    return -1;
  char* base = reinterpret_cast<char*>(0x100000);  // any 256-aligned base: offsets only
  GmWork w = gm_carve(base, k, n, restart);
  return (reinterpret_cast<char*>(w.V + (int64_t)kk * n) - base);
}

// One Arnoldi step on w = M A V[kk] (formed by the caller, k vectors of
// length n back to back); `on` is k ints of device scratch.
extern "C" int lxgb_gmres_arnoldi(int32_t k, int64_t n, int32_t restart, int32_t parity, int32_t kk,
                                  double* wv, int32_t* on, void* work, int64_t wbytes,
                                  void* stream) {
  int rc = gm_check(k, n, restart, work, wbytes);
  if (rc) return rc;
  LXGB_REQUIRE(wv && on && kk >= 0 && kk < restart, "gmres: bad arguments");
  cudaStream_t st = as_stream(stream);
  GmWork w = gm_carve(work, k, n, restart);
  const int cur = parity & 1;
  dim3 g(w.parts, k);
  gm_snapshot_kernel<<<(k + 127) / 128, 128, 0, st>>>(k, w, cur, on);
  gm_proj_partial_kernel<<<g, kKThreads, 0, st>>>(n, k, w, cur, kk, wv);
  gm_proj_final_kernel<<<k, 32, 0, st>>>(k, n, w, cur, kk, wv);
  gm_orth_kernel<<<g, kKThreads, 0, st>>>(n, k, w, cur, kk, wv);
  gm_norm_final_kernel<<<k, 32, 0, st>>>(k, n, w, cur, kk, wv);
  gm_store_basis_kernel<<<g, kKThreads, 0, st>>>(n, k, w, cur, kk, wv, on);
  return check_launch("gmres_arnoldi");
}

// End of the Arnoldi loop: least squares, y += V z, diff (first pass: inf).
extern "C" int lxgb_gmres_cycle_end(int32_t k, int64_t n, int32_t restart, int32_t parity,
                                    int32_t first, double* y, double* diff, void* work,
                                    int64_t wbytes, void* stream) {
  int rc = gm_check(k, n, restart, work, wbytes);
  if (rc) return rc;
  LXGB_REQUIRE(y && diff, "gmres: null pointer");
  cudaStream_t st = as_stream(stream);
  GmWork w = gm_carve(work, k, n, restart);
  const int cur = parity & 1;
  if (!first) {
    const size_t smem = (size_t)(restart + 1) * (restart + 2) * sizeof(double);
    LXGB_CUDA_TRY(ensure_dynamic_smem(reinterpret_cast<const void*>(gm_lstsq_kernel), (int)smem),
                  "gmres: set smem");
    gm_lstsq_kernel<<<k, 64, smem, st>>>(k, w, cur);
  }
  dim3 g(w.parts, k);
  gm_update_kernel<<<g, kKThreads, 0, st>>>(n, k, w, cur, first, y, diff);
  return check_launch("gmres_cycle_end");
}

// After the caller formed t = M(b - A y): r = t, norms, stagnation and the
// next loop condition.
extern "C" int lxgb_gmres_outer(int32_t k, int64_t n, int32_t restart, int32_t parity,
                                int32_t first, const double* b, const double* t, double* r,
                                const double* diff, const double* y, double rtol, double atol,
                                int64_t max_steps, int32_t stagnation_iters, int32_t has_scale,
                                void* work, int64_t wbytes, void* stream) {
  int rc = gm_check(k, n, restart, work, wbytes);
  if (rc) return rc;
  LXGB_REQUIRE(b && t && r && diff && y, "gmres: null pointer");
  cudaStream_t st = as_stream(stream);
  GmWork w = gm_carve(work, k, n, restart);
  const int cur = parity & 1;
  dim3 g(w.parts, k);
  gm_set_r_kernel<<<g, kKThreads, 0, st>>>(n, k, w, cur, t, r);
  gm_outer_partial_kernel<<<g, kKThreads, 0, st>>>(n, k, w, b, r, diff, y, rtol, atol);
  gm_outer_final_kernel<<<k, 32, 0, st>>>(k, w, cur, first, max_steps, stagnation_iters,
                                          has_scale);
  return check_launch("gmres_outer");
}

// Per right-hand side: [active(next), step, stagnation, breakdown(deferred),
// not_converged] as 5 ints.
extern "C" int lxgb_gmres_status(int32_t k, int64_t n, int32_t restart, int32_t parity,
                                 int32_t* out, void* work, int64_t wbytes, void* stream) {
  int rc = gm_check(k, n, restart, work, wbytes);
  if (rc) return rc;
  LXGB_REQUIRE(out, "gmres: null pointer");
  GmWork w = gm_carve(work, k, n, restart);
  gm_status_kernel<<<(k + 127) / 128, 128, 0, as_stream(stream)>>>(k, w, parity & 1, out);
  return check_launch("gmres_status");
}

// ---------------------------------------------------------------------------
// Single-call CG and GMRES: the whole loop on the device.
//
// lineax runs both solvers as lax.while_loops (cg.py:209, gmres.py:215,292):
// one compiled program per solve whose loop condition is evaluated on the
// device.  The CUDA form of that is a graph with a conditional WHILE node:
// its body is a fixed run of iterations (the step sequences above, captured
// from a private stream) followed by a one-thread kernel that sets the loop
// condition from the per-right-hand-side flags — any right-hand side still
// active — and from a round counter that bounds the number of rounds by the
// step budget, so the loop ends even if a flag were never cleared.  The host
// builds, launches and releases the graph; it never waits for the device.
// ---------------------------------------------------------------------------
namespace lxgb {

__global__ void loop_cond_kernel(cudaGraphConditionalHandle h, const int* __restrict__ flags,
                                 int k, int stride, int* __restrict__ counter, int max_rounds,
                                 int reset) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  int any = 0;
  for (int c = 0; c < k; ++c) any |= flags[(int64_t)c * stride];
  const int rounds = reset ? 0 : *counter + 1;
  *counter = rounds;
  cudaGraphSetConditional(h, (any && rounds < max_rounds) ? 1u : 0u);
}

__global__ void sub_kernel(int64_t total, const double* __restrict__ b, double* __restrict__ x) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x)
    x[e] = b[e] - x[e];
}

__global__ void strided_copy_kernel(int64_t n, int k, const double* __restrict__ x, int64_t ldx,
                                    double* __restrict__ y) {
  const int c = blockIdx.y;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    y[(int64_t)c * n + i] = x[(int64_t)c * ldx + i];
}

// lineax's result codes from the step counts (cg.py:213-222, gmres.py:217-237).
__global__ void cg_result_kernel(int k, CgWork w, int64_t max_steps, int max_given,
                                 int has_scale, int32_t* __restrict__ steps,
                                 int32_t* __restrict__ results) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= k) return;
  const int s = w.step[c];
  int res = LXGB_SUCCESSFUL;
  if (!max_given)
    res = (s == max_steps) ? LXGB_SINGULAR : LXGB_SUCCESSFUL;
  else if (has_scale)
    res = (s == max_steps) ? LXGB_MAX_STEPS_REACHED : LXGB_SUCCESSFUL;
  steps[c] = s;
  results[c] = res;
}

__global__ void gm_result_kernel(int k, GmWork w, int64_t max_steps, int max_given,
                                 int has_scale, int stagnation_iters,
                                 int32_t* __restrict__ steps, int32_t* __restrict__ results) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= k) return;
  const int* f = w.fl + c * 8;
  const int s = f[5];
  int res = LXGB_SUCCESSFUL;
  if (!max_given)
    res = (s == max_steps) ? LXGB_SINGULAR : LXGB_SUCCESSFUL;
  else if (has_scale)
    res = (s == max_steps) ? LXGB_MAX_STEPS_REACHED : LXGB_SUCCESSFUL;
  if (f[6] >= stagnation_iters) res = LXGB_STAGNATION;
  if (f[4] && f[7]) res = LXGB_BREAKDOWN;
  steps[c] = s;
  results[c] = res;
}

static int64_t al256(int64_t b) { return (b + 255) & ~(int64_t)255; }

__global__ void scale_kernel(int64_t total, double s, double* __restrict__ y) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x)
    y[e] *= s;
}

// Scratch bytes apply_op needs for k vectors of length n: room for a
// contiguous copy of x, then the double-float products' own scratch.
static int64_t apply_scratch_bytes(int k, int64_t n) {
  const int64_t a = lxgb_gemv_df_workspace_size((int32_t)n, k);
  const int64_t b = lxgb_lu32_apply_workspace_size((int32_t)n, k);
  const int64_t c = lxgb_qr32_apply_workspace_size((int32_t)n, k);
  const int64_t m = a > b ? a : b;
  return al256((int64_t)k * n * 8) + al256(m > c ? m : c);
}

// y = op(x) for k vectors; x_c at x + c*ldx, y contiguous.  `tmp` holds
// apply_scratch_bytes(k, n).
static int apply_op(const lxgb_linear_operator& op, int k, int64_t n, const double* x,
                    int64_t ldx, double* y, double* tmp, cudaStream_t st) {
  if (op.kind == LXGB_OP_DENSE)
    return lxgb_gemv_f64(n, n, op.a, op.lda, 0, k, x, ldx, y, n, op.scale, 0.0, st);
  const int64_t vb = al256((int64_t)k * n * 8);
  void* scratch = reinterpret_cast<char*>(tmp) + vb;
  const int64_t sbytes = apply_scratch_bytes(k, n) - vb;
  int rc;
  if (op.kind == LXGB_OP_SPLIT_DF) {
    rc = lxgb_gemv_df((int32_t)n, (int32_t)n, op.hi, op.lo, op.lda, k, x, ldx, nullptr, y, n, 1,
                      scratch, sbytes, st);
  } else {
    if (ldx != n) {
      dim3 g((unsigned)((n + 255) / 256 < 1024 ? (n + 255) / 256 : 1024), (unsigned)k);
      strided_copy_kernel<<<g, 256, 0, st>>>(n, k, x, ldx, tmp);
      x = tmp;
    }
    if (op.kind == LXGB_OP_POISSON5) return lxgb_poisson5_f64(op.nx, op.ny, k, op.scale, x, y, st);
    if (op.kind == LXGB_OP_QR32)
      rc = lxgb_qr32_apply((int32_t)n, k, op.hi, op.lo, 1, x, y, scratch, sbytes, st);
    else
      rc = lxgb_lu32_apply((int32_t)n, k, op.hi, op.lo, op.perm, 1, x, y, scratch, sbytes, st);
  }
  if (!rc && op.scale != 1.0) {
    const int64_t total = (int64_t)k * n;
    scale_kernel<<<(unsigned)((total + 255) / 256 < 4096 ? (total + 255) / 256 : 4096), 256, 0,
                   st>>>(total, op.scale, y);
    rc = check_launch("krylov run: scale");
  }
  return rc;
}

static int check_op(const lxgb_linear_operator* op, int64_t n, const char* who) {
  if (!op) return invalid("krylov run: null operator");
  if (op->kind == LXGB_OP_DENSE) {
    if (!op->a || op->lda < n) {
      set_last_error("%s: dense operator needs a matrix with lda >= n", who);
      return LXGB_INVALID_ARG;
    }
    return LXGB_SUCCESSFUL;
  }
  if (op->kind == LXGB_OP_POISSON5) {
    if (op->nx < 1 || op->ny < 1 || op->nx * op->ny != n) {
      set_last_error("%s: stencil grid does not match n", who);
      return LXGB_INVALID_ARG;
    }
    return LXGB_SUCCESSFUL;
  }
  if (op->kind == LXGB_OP_SPLIT_DF || op->kind == LXGB_OP_LU32_INV ||
      op->kind == LXGB_OP_QR32) {
    const bool ok = op->hi && n < (1LL << 31) &&
                    (op->kind == LXGB_OP_SPLIT_DF ? op->lda >= n
                     : op->kind == LXGB_OP_QR32   ? op->lo != nullptr
                                                  : (op->lo && op->perm));
    if (!ok) {
      set_last_error("%s: FP32 operator needs its factor arrays (and lda >= n)", who);
      return LXGB_INVALID_ARG;
    }
    return LXGB_SUCCESSFUL;
  }
  set_last_error("%s: unknown operator kind %d", who, op->kind);
  return LXGB_INVALID_ARG;
}

// Graph building by stream capture.  A Capture records what is issued on its
// root stream into a new graph.  Conditional nodes (while, if/else) are
// appended to a stream's ongoing capture; each body is recorded from a fresh
// private stream, so loops nest the way lax.while_loop bodies do.  Every
// stream still capturing when the Capture is destroyed (after an error) has
// its capture ended, so no stream is left in capture mode.
struct Capture {
  cudaStream_t root = nullptr;
  std::vector<cudaStream_t> streams;
  std::vector<cudaStream_t> open;  // streams whose capture has not ended
  ~Capture() {
    for (cudaStream_t s : open) {
      cudaGraph_t g = nullptr;
      if (cudaStreamEndCapture(s, &g) == cudaSuccess && g) cudaGraphDestroy(g);
    }
    cudaGetLastError();  // clear an error left by an abandoned capture
    for (cudaStream_t s : streams) cudaStreamDestroy(s);
  }
  int new_stream(cudaStream_t* s, const char* who) {
    LXGB_CUDA_TRY(cudaStreamCreateWithFlags(s, cudaStreamNonBlocking), who);
    streams.push_back(*s);
    return LXGB_SUCCESSFUL;
  }
  int begin(const char* who) {
    int rc = new_stream(&root, who);
    if (rc) return rc;
    LXGB_CUDA_TRY(cudaStreamBeginCapture(root, cudaStreamCaptureModeThreadLocal), who);
    open.push_back(root);
    return LXGB_SUCCESSFUL;
  }
  int end(cudaStream_t s, cudaGraph_t* g, const char* who) {
    for (size_t i = 0; i < open.size(); ++i)
      if (open[i] == s) {
        open.erase(open.begin() + i);
        break;
      }
    LXGB_CUDA_TRY(cudaStreamEndCapture(s, g), who);
    return LXGB_SUCCESSFUL;
  }
  // A handle for a conditional node that will be appended to st's capture.
  int handle(cudaStream_t st, cudaGraphConditionalHandle* h, const char* who) {
    cudaStreamCaptureStatus status;
    cudaGraph_t g = nullptr;
    LXGB_CUDA_TRY(cudaStreamGetCaptureInfo(st, &status, nullptr, &g), who);
    if (status != cudaStreamCaptureStatusActive || !g) {
      set_last_error("%s: stream is not capturing", who);
      return LXGB_CUDA_ERROR;
    }
    LXGB_CUDA_TRY(cudaGraphConditionalHandleCreate(h, g, 0, 0), who);
    return LXGB_SUCCESSFUL;
  }
  // Appends a conditional node with `size` bodies after everything captured
  // on st so far; bodies[i] receive fresh streams capturing into the bodies.
  int cond(cudaStream_t st, cudaGraphConditionalHandle h, cudaGraphConditionalNodeType type,
           unsigned size, cudaStream_t* bodies, const char* who) {
    cudaStreamCaptureStatus status;
    cudaGraph_t g = nullptr;
    const cudaGraphNode_t* deps = nullptr;
    const cudaGraphEdgeData* edata = nullptr;
    size_t ndeps = 0;
    LXGB_CUDA_TRY(cudaStreamGetCaptureInfo(st, &status, nullptr, &g, &deps, &edata, &ndeps), who);
    cudaGraphNodeParams cp = {};
    cp.type = cudaGraphNodeTypeConditional;
    cp.conditional.handle = h;
    cp.conditional.type = type;
    cp.conditional.size = size;
    cudaGraphNode_t node;
    LXGB_CUDA_TRY(cudaGraphAddNode(&node, g, deps, edata, ndeps, &cp), who);
    LXGB_CUDA_TRY(cudaStreamUpdateCaptureDependencies(st, &node, nullptr, 1,
                                                      cudaStreamSetCaptureDependencies),
                  who);
    for (unsigned i = 0; i < size; ++i) {
      int rc = new_stream(&bodies[i], who);
      if (rc) return rc;
      LXGB_CUDA_TRY(cudaStreamBeginCaptureToGraph(bodies[i], cp.conditional.phGraph_out[i],
                                                  nullptr, nullptr, 0,
                                                  cudaStreamCaptureModeThreadLocal),
                    who);
      open.push_back(bodies[i]);
    }
    return LXGB_SUCCESSFUL;
  }
  int end_body(cudaStream_t s, const char* who) {
    cudaGraph_t g = nullptr;
    return end(s, &g, who);
  }
  // Ends the root capture, instantiates the graph and launches it on `user`
  // (the executable graph is released once it has run).
  int launch(cudaStream_t user, const char* who) {
    cudaGraph_t g = nullptr;
    int rc = end(root, &g, who);
    if (rc) return rc;
    cudaGraphExec_t exec = nullptr;
    const cudaError_t ie = cudaGraphInstantiate(&exec, g, 0);
    cudaGraphDestroy(g);
    LXGB_CUDA_TRY(ie, who);
    const cudaError_t le = cudaGraphLaunch(exec, user);
    cudaGraphExecDestroy(exec);
    LXGB_CUDA_TRY(le, who);
    return LXGB_SUCCESSFUL;
  }
};

struct CgRunLayout {
  int64_t cg, counter, r, p, matp, ay, z, tmp, total;
};

static CgRunLayout cg_run_layout(int k, int64_t n, bool pre) {
  CgRunLayout L;
  const int64_t v = al256((int64_t)k * n * 8);
  L.cg = 0;
  L.counter = al256(cg_ws_bytes(k, n));
  L.r = L.counter + 256;
  L.p = L.r + v;
  L.matp = L.p + v;
  L.ay = L.matp + v;
  L.tmp = L.ay + v;
  L.z = L.tmp + al256(apply_scratch_bytes(k, n));
  L.total = L.z + (pre ? v : 0);
  return L;
}

}  // namespace lxgb

extern "C" int64_t lxgb_cg_run_workspace_size(int32_t k, int64_t n, int32_t has_precond) {
  if (k < 1 || n < 1) return 256;
  return cg_run_layout(k, n, has_precond != 0).total;
}

extern "C" int lxgb_cg_run(int32_t k, int64_t n, const lxgb_linear_operator* op,
                           const lxgb_linear_operator* precond, const double* b, double* y,
                           int32_t y0_given, double rtol, double atol, int64_t max_steps,
                           int32_t stabilise_every, int32_t* steps, int32_t* results,
                           void* work, int64_t work_bytes, void* stream) {
  const char* who = "cg_run";
  LXGB_REQUIRE(k >= 1 && k <= 65535 && n >= 1, "cg_run: bad sizes");
  LXGB_REQUIRE(b && y && steps && results && work, "cg_run: null pointer");
  LXGB_REQUIRE(((uintptr_t)work & 255) == 0, "cg_run: workspace must be 256-byte aligned");
  LXGB_REQUIRE(stabilise_every >= 0 && stabilise_every <= 64,
               "cg_run: stabilise_every must be in [0, 64] (0: never)");
  int rc = check_op(op, n, who);
  if (rc) return rc;
  if (precond && (rc = check_op(precond, n, who))) return rc;
  const bool pre = precond != nullptr;
  const CgRunLayout L = cg_run_layout(k, n, pre);
  if (work_bytes < L.total) {
    set_last_error("cg_run: workspace too small");
    return LXGB_WORKSPACE_TOO_SMALL;
  }
  char* wb = reinterpret_cast<char*>(work);
  void* cgws = wb + L.cg;
  const int64_t cgb = cg_ws_bytes(k, n);
  int* counter = reinterpret_cast<int*>(wb + L.counter);
  double* r = reinterpret_cast<double*>(wb + L.r);
  double* p = reinterpret_cast<double*>(wb + L.p);
  double* matp = reinterpret_cast<double*>(wb + L.matp);
  double* ay = reinterpret_cast<double*>(wb + L.ay);
  double* tmp = reinterpret_cast<double*>(wb + L.tmp);
  double* z = pre ? reinterpret_cast<double*>(wb + L.z) : r;
  const int64_t total = (int64_t)k * n;
  const bool max_given = max_steps >= 0;
  const int64_t max_s = max_given ? max_steps : 10 * n;
  const int has_scale = !(atol == 0.0 && rtol == 0.0);
  const double rcond = 2.0 * 2.220446049250313e-16 * (double)n;
  const unsigned g = (unsigned)((total + 255) / 256 < 4096 ? (total + 255) / 256 : 4096);
  // iterations per round: a multiple of stabilise_every (the true-residual
  // steps fall on fixed positions) and of 2 (the flag parity returns to 0)
  int per = stabilise_every == 0 ? 8 : stabilise_every;
  if (per & 1) per *= 2;
  while (per < 8) per *= 2;
  const int64_t rounds64 = (max_s + per - 1) / per + 1;
  const int max_rounds = (int)(rounds64 < (1LL << 30) ? rounds64 : (1LL << 30));
  CgWork w = cg_carve(cgws, k, n);
  Capture cap;
  if ((rc = cap.begin(who))) return rc;
  cudaStream_t st = cap.root;
  // r = b - A y0 (or b), z = M r, p = z, gamma = <z, r>, flags (cg.py:114-131)
  if (y0_given) {
    if ((rc = apply_op(*op, k, n, y, n, r, tmp, st))) return rc;
    sub_kernel<<<g, 256, 0, st>>>(total, b, r);
  } else {
    LXGB_CUDA_TRY(cudaMemsetAsync(y, 0, (size_t)total * 8, st), who);
    LXGB_CUDA_TRY(cudaMemcpyAsync(r, b, (size_t)total * 8, cudaMemcpyDeviceToDevice, st), who);
  }
  if (pre && (rc = apply_op(*precond, k, n, r, n, z, tmp, st))) return rc;
  if ((rc = lxgb_cg_start(k, n, r, z, p, max_s, has_scale, cgws, cgb, st))) return rc;
  cudaGraphConditionalHandle h;
  if ((rc = cap.handle(st, &h, who))) return rc;
  loop_cond_kernel<<<1, 32, 0, st>>>(h, w.act, k, 1, counter, max_rounds, 1);
  cudaStream_t sb;
  if ((rc = cap.cond(st, h, cudaGraphCondTypeWhile, 1, &sb, who))) return rc;
  for (int j = 0; j < per; ++j) {
    const int par = j & 1;
    const bool stable = stabilise_every == 1 ||
                        (stabilise_every > 1 && (j + 1) % stabilise_every == 0);
    if ((rc = apply_op(*op, k, n, p, n, matp, tmp, sb))) return rc;
    if ((rc = lxgb_cg_step_alpha(k, n, matp, p, y, r, stable ? 0 : 1, par, rtol, atol, rcond,
                                 cgws, cgb, sb)))
      return rc;
    if (stable) {
      if ((rc = apply_op(*op, k, n, y, n, ay, tmp, sb))) return rc;
      if ((rc = lxgb_cg_true_residual(k, n, b, ay, r, par, cgws, cgb, sb))) return rc;
    }
    if (pre && (rc = apply_op(*precond, k, n, r, n, z, tmp, sb))) return rc;
    if ((rc = lxgb_cg_step_beta(k, n, b, r, z, p, par, max_s, has_scale, rtol, atol, cgws, cgb,
                                sb)))
      return rc;
  }
  loop_cond_kernel<<<1, 32, 0, sb>>>(h, w.act, k, 1, counter, max_rounds, 0);
  if ((rc = cap.end_body(sb, who))) return rc;
  cg_result_kernel<<<(k + 127) / 128, 128, 0, st>>>(k, w, max_s, max_given, has_scale, steps,
                                                     results);
  if ((rc = check_launch(who))) return rc;
  return cap.launch(as_stream(stream), who);
}

namespace lxgb {

struct GmRunLayout {
  int64_t gm, counter, on, r, diff, w, t, tmp, tmp2, total;
};

static GmRunLayout gm_run_layout(int k, int64_t n, int R) {
  GmRunLayout L;
  const int64_t v = al256((int64_t)k * n * 8);
  L.gm = 0;
  L.counter = al256(gm_ws_bytes(k, n, R));
  L.on = L.counter + 256;
  L.r = L.on + al256((int64_t)k * 4);
  L.diff = L.r + v;
  L.w = L.diff + v;
  L.t = L.w + v;
  L.tmp = L.t + v;
  L.tmp2 = L.tmp + v;
  L.total = L.tmp2 + al256(apply_scratch_bytes(k, n));
  return L;
}

// One restarted GMRES solve (lineax/_solver/gmres.py:106-413) enqueued on st,
// which must be capturing: the dummy first pass, then a while node whose body
// runs two outer iterations (flag parities 1 and 0) and re-evaluates the loop
// condition, then the result codes.  y is the start vector (zero it first for
// y0 = 0).
struct GmresCall {
  int k;
  int64_t n;
  int R;
  const lxgb_linear_operator* op;
  const lxgb_linear_operator* pre;
  const double* b;
  double* y;
  double rtol, atol;
  int64_t max_s;
  int max_given;
  int stagnation_iters;
  void* work;  // GmRunLayout
  int32_t* steps;
  int32_t* results;
};

static int gmres_enqueue(Capture& cap, cudaStream_t st, const GmresCall& c, const char* who) {
  const int k = c.k, R = c.R;
  const int64_t n = c.n;
  const GmRunLayout L = gm_run_layout(k, n, R);
  char* wb = reinterpret_cast<char*>(c.work);
  void* gmws = wb + L.gm;
  const int64_t gmb = gm_ws_bytes(k, n, R);
  int* counter = reinterpret_cast<int*>(wb + L.counter);
  int32_t* on = reinterpret_cast<int32_t*>(wb + L.on);
  double* r = reinterpret_cast<double*>(wb + L.r);
  double* diff = reinterpret_cast<double*>(wb + L.diff);
  double* wv = reinterpret_cast<double*>(wb + L.w);
  double* t = reinterpret_cast<double*>(wb + L.t);
  double* tmp = reinterpret_cast<double*>(wb + L.tmp);
  double* tmp2 = reinterpret_cast<double*>(wb + L.tmp2);
  const int64_t total = (int64_t)k * n;
  const int has_scale = !(c.atol == 0.0 && c.rtol == 0.0);
  const unsigned g = (unsigned)((total + 255) / 256 < 4096 ? (total + 255) / 256 : 4096);
  GmWork w = gm_carve(gmws, k, n, R);
  // t = M (b - A y)
  auto residual = [&](cudaStream_t s) -> int {
    int e = apply_op(*c.op, k, n, c.y, n, tmp, tmp2, s);
    if (e) return e;
    sub_kernel<<<g, 256, 0, s>>>(total, c.b, tmp);
    if (c.pre) return apply_op(*c.pre, k, n, tmp, n, t, tmp2, s);
    LXGB_CUDA_TRY(cudaMemcpyAsync(t, tmp, (size_t)total * 8, cudaMemcpyDeviceToDevice, s), who);
    return check_launch(who);
  };
  // one outer iteration of parity `par` (gmres.py:143-188, 240-300)
  auto outer = [&](int par, int first, cudaStream_t s) -> int {
    int e = 0;
    if (!first) {
      e = lxgb_gmres_cycle_begin(k, n, R, par, r, gmws, gmb, s);
      for (int kk = 0; kk < R && !e; ++kk) {
        const double* vk = w.V + (int64_t)kk * n;  // vector c at + c*(R+1)*n
        e = apply_op(*c.op, k, n, vk, (int64_t)(R + 1) * n, c.pre ? tmp : wv, tmp2, s);
        if (!e && c.pre) e = apply_op(*c.pre, k, n, tmp, n, wv, tmp2, s);
        if (!e) e = lxgb_gmres_arnoldi(k, n, R, par, kk, wv, on, gmws, gmb, s);
      }
    }
    if (!e) e = lxgb_gmres_cycle_end(k, n, R, par, first, c.y, diff, gmws, gmb, s);
    if (!e) e = residual(s);
    if (!e)
      e = lxgb_gmres_outer(k, n, R, par, first, c.b, t, r, diff, c.y, c.rtol, c.atol, c.max_s,
                           c.stagnation_iters, has_scale, gmws, gmb, s);
    return e;
  };
  // start (gmres.py:192-205): r = 0, the dummy first pass
  LXGB_CUDA_TRY(cudaMemsetAsync(r, 0, (size_t)total * 8, st), who);
  int rc = lxgb_gmres_init(k, n, R, gmws, gmb, st);
  if (!rc) rc = outer(0, 1, st);
  if (rc) return rc;
  // rounds of two outer iterations (parities 1, 0); the flags of parity 1
  // are the loop condition after each round
  const int64_t rounds64 = (c.max_s + 1) / 2 + 2;
  const int max_rounds = (int)(rounds64 < (1LL << 30) ? rounds64 : (1LL << 30));
  cudaGraphConditionalHandle h;
  if ((rc = cap.handle(st, &h, who))) return rc;
  loop_cond_kernel<<<1, 32, 0, st>>>(h, w.fl + 1, k, 8, counter, max_rounds, 1);
  cudaStream_t sb;
  if ((rc = cap.cond(st, h, cudaGraphCondTypeWhile, 1, &sb, who))) return rc;
  rc = outer(1, 0, sb);
  if (!rc) rc = outer(0, 0, sb);
  if (rc) return rc;
  loop_cond_kernel<<<1, 32, 0, sb>>>(h, w.fl + 1, k, 8, counter, max_rounds, 0);
  if ((rc = cap.end_body(sb, who))) return rc;
  gm_result_kernel<<<(k + 127) / 128, 128, 0, st>>>(k, w, c.max_s, c.max_given, has_scale,
                                                     c.stagnation_iters, c.steps, c.results);
  return check_launch(who);
}

static int gmres_prepare(int R, const char* who) {
  // the least-squares kernel's shared memory is raised outside any capture
  const size_t smem = (size_t)(R + 1) * (R + 2) * sizeof(double);
  LXGB_CUDA_TRY(ensure_dynamic_smem(reinterpret_cast<const void*>(gm_lstsq_kernel), (int)smem),
                who);
  return LXGB_SUCCESSFUL;
}

}  // namespace lxgb

extern "C" int64_t lxgb_gmres_run_workspace_size(int32_t k, int64_t n, int32_t restart) {
  if (k < 1 || n < 1 || restart < 1) return 256;
  const int R = (int)(restart < n ? restart : n);
  return gm_run_layout(k, n, R).total;
}

extern "C" int lxgb_gmres_run(int32_t k, int64_t n, const lxgb_linear_operator* op,
                              const lxgb_linear_operator* precond, const double* b, double* y,
                              int32_t y0_given, double rtol, double atol, int64_t max_steps,
                              int32_t restart, int32_t stagnation_iters, int32_t* steps,
                              int32_t* results, void* work, int64_t work_bytes, void* stream) {
  const char* who = "gmres_run";
  LXGB_REQUIRE(k >= 1 && k <= 65535 && n >= 1, "gmres_run: bad sizes");
  LXGB_REQUIRE(b && y && steps && results && work, "gmres_run: null pointer");
  LXGB_REQUIRE(((uintptr_t)work & 255) == 0, "gmres_run: workspace must be 256-byte aligned");
  const int R = (int)(restart < n ? restart : n);  // lineax: restart = min(restart, size)
  LXGB_REQUIRE(R >= 1 && R <= kGmMaxRestart, "gmres_run: restart must be in [1, 128]");
  int rc = check_op(op, n, who);
  if (rc) return rc;
  if (precond && (rc = check_op(precond, n, who))) return rc;
  if (work_bytes < gm_run_layout(k, n, R).total) {
    set_last_error("gmres_run: workspace too small");
    return LXGB_WORKSPACE_TOO_SMALL;
  }
  if ((rc = gmres_prepare(R, who))) return rc;
  const bool max_given = max_steps >= 0;
  GmresCall c{k, n, R, op, precond, b, y, rtol, atol, max_given ? max_steps : 10 * n,
              max_given ? 1 : 0, stagnation_iters, work, steps, results};
  Capture cap;
  if ((rc = cap.begin(who))) return rc;
  if (!y0_given) LXGB_CUDA_TRY(cudaMemsetAsync(y, 0, (size_t)k * n * 8, cap.root), who);
  if ((rc = gmres_enqueue(cap, cap.root, c, who))) return rc;
  return cap.launch(as_stream(stream), who);
}

// ---------------------------------------------------------------------------
// Single-call GMRES-IR: the refinement loop of the mixed-precision LU solve
// (FP32 factor, FP64-accurate residuals) on the device, around the GMRES
// solve above.  Per outer step: in the first tier plain refinement
// x += M r; from the first step that stalls on, GMRES on the scaled residual
// (r / max|r|), preconditioned by M, x += max|r| y.  Then r = b - A x and the
// normwise backward error of every right-hand side; the loop ends when all
// are <= tol, when refinement stalls in the GMRES tier, or after max_outer
// steps.  The tier choice is an if/else node, the GMRES loop a while node
// inside it, both inside the outer while node.
// ---------------------------------------------------------------------------
namespace lxgb {

struct IrState {
  int tier, done, stop, it, inner_ok, code;
  double prev;
};

__global__ void ir_init_kernel(IrState* s, double* ones, int k, cudaGraphConditionalHandle hl,
                               int max_outer) {
  for (int c = threadIdx.x; c < k; c += blockDim.x) ones[c] = 1.0;
  if (threadIdx.x == 0) {
    s->tier = 0;
    s->done = s->stop = s->it = 0;
    s->inner_ok = 1;
    s->code = 2;
    s->prev = INFINITY;
    cudaGraphSetConditional(hl, max_outer > 0 ? 1u : 0u);
  }
}

// The tier node's condition: 1 (GMRES) once refinement has stalled, else 0.
__global__ void set_tier_handle_kernel(const IrState* s, cudaGraphConditionalHandle ht) {
  if (threadIdx.x == 0) cudaGraphSetConditional(ht, s->tier ? 1u : 0u);
}

__global__ void ir_inner_ok_kernel(IrState* s, const int32_t* __restrict__ results, int k) {
  if (threadIdx.x != 0) return;
  int ok = 1;
  if (results)
    for (int c = 0; c < k; ++c) ok &= results[c] == LXGB_SUCCESSFUL;
  s->inner_ok = ok;
}

// Backward errors, the stall test and the next tier / loop condition
// (the host loop of gmres_ir in lineax_gb300/mixed.py).
__global__ void ir_step_kernel(IrState* s, const double* __restrict__ rn,
                               const double* __restrict__ xn, const double* __restrict__ bn,
                               const double* __restrict__ anorm, double tol, int k, int max_outer,
                               int stop_on_stall, double* __restrict__ berr,
                               int32_t* __restrict__ status, cudaGraphConditionalHandle hl) {
  if (threadIdx.x != 0) return;
  const double an = *anorm;
  int all = 1;
  double mx = -INFINITY;
  for (int c = 0; c < k; ++c) {
    // separate roundings (no FMA contraction): the same value the host forms
    const double den = __dadd_rn(__dmul_rn(an, xn[c]), bn[c]);
    const double e = den > 0.0 ? __ddiv_rn(rn[c], den) : 0.0;
    berr[c] = e;
    all &= e <= tol;
    mx = (e != e || mx != mx) ? NAN : fmax(mx, e);
  }
  s->it += 1;
  if (all) {
    s->done = 1;
    s->code = 0;
  } else {
    const bool stalled = !s->inner_ok || !(mx <= s->prev / 2);
    if (stalled) {
      if (s->tier == 0) {
        s->tier = 1;
      } else if (stop_on_stall) {
        s->stop = 1;
        s->code = 1;
      }
    }
  }
  s->prev = mx;
  const bool go = !s->done && !s->stop && s->it < max_outer;
  if (!s->done && !s->stop && !go) s->code = 2;
  status[0] = s->it;
  status[1] = s->tier;
  status[2] = s->code;
  cudaGraphSetConditional(hl, go ? 1u : 0u);
}

struct IrRunLayout {
  GmRunLayout gm;
  int64_t gmres, rr, rhat, yin, tvec, rn, xn, bn, ones, gsteps, gres, state, kred, total;
};

static IrRunLayout ir_run_layout(int k, int64_t n, int R) {
  IrRunLayout L;
  const int64_t v = al256((int64_t)k * n * 8);
  const int64_t kv = al256((int64_t)k * 8);
  L.gm = gm_run_layout(k, n, R);
  L.gmres = 0;
  L.rr = al256(L.gm.total);
  L.rhat = L.rr + v;
  L.yin = L.rhat + v;
  L.tvec = L.yin + v;
  L.rn = L.tvec + v;
  L.xn = L.rn + kv;
  L.bn = L.xn + kv;
  L.ones = L.bn + kv;
  L.gsteps = L.ones + kv;
  L.gres = L.gsteps + kv;
  L.state = L.gres + kv;
  L.kred = L.state + 256;
  L.total = L.kred + al256(lxgb_kreduce_workspace_size(k, n));
  return L;
}

}  // namespace lxgb

extern "C" int64_t lxgb_gmres_ir_run_workspace_size(int32_t k, int64_t n, int32_t restart) {
  if (k < 1 || n < 1 || restart < 1) return 256;
  const int R = (int)(restart < n ? restart : n);
  return ir_run_layout(k, n, R).total;
}

extern "C" int lxgb_gmres_ir_run(int32_t k, int64_t n, const lxgb_linear_operator* op,
                                 const lxgb_linear_operator* precond, const double* b, double* x,
                                 const double* anorm, double tol, double inner_rtol,
                                 int32_t max_outer, int32_t restart, int32_t inner_max_steps,
                                 int32_t stagnation_iters, int32_t stop_on_stall, double* berr,
                                 int32_t* status, void* work, int64_t work_bytes, void* stream) {
  const char* who = "gmres_ir_run";
  LXGB_REQUIRE(k >= 1 && k <= 65535 && n >= 1, "gmres_ir_run: bad sizes");
  LXGB_REQUIRE(b && x && anorm && berr && status && work, "gmres_ir_run: null pointer");
  LXGB_REQUIRE(precond != nullptr, "gmres_ir_run: the refinement needs a preconditioner");
  LXGB_REQUIRE(((uintptr_t)work & 255) == 0, "gmres_ir_run: workspace must be 256-byte aligned");
  LXGB_REQUIRE(max_outer >= 0 && inner_max_steps >= 1, "gmres_ir_run: bad step limits");
  const int R = (int)(restart < n ? restart : n);
  LXGB_REQUIRE(R >= 1 && R <= kGmMaxRestart, "gmres_ir_run: restart must be in [1, 128]");
  int rc = check_op(op, n, who);
  if (!rc) rc = check_op(precond, n, who);
  if (rc) return rc;
  const IrRunLayout L = ir_run_layout(k, n, R);
  if (work_bytes < L.total) {
    set_last_error("gmres_ir_run: workspace too small");
    return LXGB_WORKSPACE_TOO_SMALL;
  }
  if ((rc = gmres_prepare(R, who))) return rc;
  char* wb = reinterpret_cast<char*>(work);
  double* rr = reinterpret_cast<double*>(wb + L.rr);
  double* rhat = reinterpret_cast<double*>(wb + L.rhat);
  double* yin = reinterpret_cast<double*>(wb + L.yin);
  double* tvec = reinterpret_cast<double*>(wb + L.tvec);
  double* rn = reinterpret_cast<double*>(wb + L.rn);
  double* xn = reinterpret_cast<double*>(wb + L.xn);
  double* bn = reinterpret_cast<double*>(wb + L.bn);
  double* ones = reinterpret_cast<double*>(wb + L.ones);
  int32_t* gsteps = reinterpret_cast<int32_t*>(wb + L.gsteps);
  int32_t* gres = reinterpret_cast<int32_t*>(wb + L.gres);
  IrState* state = reinterpret_cast<IrState*>(wb + L.state);
  void* kred = wb + L.kred;
  const int64_t kredb = L.total - L.kred;
  double* tmp = reinterpret_cast<double*>(wb + L.gm.tmp2);  // apply scratch (free outside GMRES)
  const int64_t total = (int64_t)k * n;
  Capture cap;
  if ((rc = cap.begin(who))) return rc;
  cudaStream_t st = cap.root;
  LXGB_CUDA_TRY(cudaMemsetAsync(x, 0, (size_t)total * 8, st), who);
  LXGB_CUDA_TRY(cudaMemcpyAsync(rr, b, (size_t)total * 8, cudaMemcpyDeviceToDevice, st), who);
  if ((rc = lxgb_kreduce_f64(1, k, n, b, n, nullptr, 0, bn, kred, kredb, st))) return rc;
  cudaGraphConditionalHandle hl;
  if ((rc = cap.handle(st, &hl, who))) return rc;
  ir_init_kernel<<<1, 128, 0, st>>>(state, ones, k, hl, max_outer);
  cudaStream_t s1;
  if ((rc = cap.cond(st, hl, cudaGraphCondTypeWhile, 1, &s1, who))) return rc;
  // the tier node (its handle belongs to the outer loop's body graph): body
  // 0 when the tier is GMRES, body 1 for plain refinement
  cudaGraphConditionalHandle htier;
  if ((rc = cap.handle(s1, &htier, who))) return rc;
  set_tier_handle_kernel<<<1, 32, 0, s1>>>(state, htier);
  cudaStream_t sb[2];
  if ((rc = cap.cond(s1, htier, cudaGraphCondTypeIf, 2, sb, who))) return rc;
  {  // GMRES on the scaled residual
    cudaStream_t s = sb[0];
    if ((rc = lxgb_kreduce_f64(1, k, n, rr, n, nullptr, 0, rn, kred, kredb, s))) return rc;
    LXGB_CUDA_TRY(cudaMemcpyAsync(rhat, rr, (size_t)total * 8, cudaMemcpyDeviceToDevice, s), who);
    if ((rc = lxgb_rows_scale_f64(k, n, rn, 1, rhat, s))) return rc;
    LXGB_CUDA_TRY(cudaMemsetAsync(yin, 0, (size_t)total * 8, s), who);
    GmresCall c{k, n, R, op, precond, rhat, yin, inner_rtol, inner_rtol, inner_max_steps, 1,
                stagnation_iters, wb + L.gmres, gsteps, gres};
    if ((rc = gmres_enqueue(cap, s, c, who))) return rc;
    if ((rc = lxgb_rows_axpy_f64(k, n, rn, yin, x, s))) return rc;
    ir_inner_ok_kernel<<<1, 32, 0, s>>>(state, gres, k);
    if ((rc = cap.end_body(s, who))) return rc;
  }
  {  // plain refinement: x += M r
    cudaStream_t s = sb[1];
    if ((rc = apply_op(*precond, k, n, rr, n, tvec, tmp, s))) return rc;
    if ((rc = lxgb_rows_axpy_f64(k, n, ones, tvec, x, s))) return rc;
    ir_inner_ok_kernel<<<1, 32, 0, s>>>(state, nullptr, k);
    if ((rc = cap.end_body(s, who))) return rc;
  }
  // r = b - A x, max|r|, max|x|, backward errors and the next step
  if (op->kind == LXGB_OP_SPLIT_DF) {
    const int64_t vb = al256(total * 8);
    if ((rc = lxgb_gemv_df((int32_t)n, (int32_t)n, op->hi, op->lo, op->lda, k, x, n, b, rr, n, 1,
                           reinterpret_cast<char*>(tmp) + vb, apply_scratch_bytes(k, n) - vb,
                           s1)))
      return rc;
  } else {
    if ((rc = apply_op(*op, k, n, x, n, rr, tmp, s1))) return rc;
    sub_kernel<<<(unsigned)((total + 255) / 256 < 4096 ? (total + 255) / 256 : 4096), 256, 0, s1>>>(
        total, b, rr);
  }
  if ((rc = lxgb_kreduce_f64(1, k, n, rr, n, nullptr, 0, rn, kred, kredb, s1))) return rc;
  if ((rc = lxgb_kreduce_f64(1, k, n, x, n, nullptr, 0, xn, kred, kredb, s1))) return rc;
  ir_step_kernel<<<1, 32, 0, s1>>>(state, rn, xn, bn, anorm, tol, k, max_outer, stop_on_stall,
                                   berr, status, hl);
  if ((rc = check_launch(who))) return rc;
  if ((rc = cap.end_body(s1, who))) return rc;
  return cap.launch(as_stream(stream), who);
}
