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

static int64_t gm_ws_bytes(int k, int64_t n, int R) {
  const int P = kparts(n);
  int64_t b = 256;
  b += (int64_t)k * (R + 1) * n * 8;
  b += (int64_t)k * R * (R + 1) * 8 + (int64_t)k * R * 8 + (int64_t)k * (R + 1) * 8;
  b += (int64_t)k * 8 * 8 + (int64_t)k * 8 * 4;
  b += (int64_t)k * P * (R + 2) * 8 + 1024;
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
