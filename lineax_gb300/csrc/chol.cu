// Cholesky factorisation (upper, A = Uᵀ U) of ragged batches, the matching
// solve, and the mixed-precision solve (FP32 factor + FP64 refinement).
//
// One persistent launch covers a ragged batch: in the mixed path CTAs pull
// systems from an atomic work queue in index order, in the plain FP64 path
// they take them round-robin.  Each system is factored by one CTA with
// a right-looking blocked algorithm; the matrix is staged in shared memory
// when it fits and otherwise factored where it lies (FP64 path: in place in
// the caller's buffer; FP32 path: in a per-CTA slice of the workspace), where
// it stays L2-resident while the CTA works on it.
#include <float.h>

#include "common.cuh"
#include "tri.cuh"

namespace lxgb {

constexpr int kCholThreads = 256;
// Largest order factored in shared memory: FP64 160*161*8 B = 206 KB,
// FP32 224*225*4 B = 202 KB (+ the correction vectors of the mixed path).
constexpr int kCholSmemMaxF64 = 160;
constexpr int kCholSmemMaxF32 = 224;
constexpr int kMixedRhsChunk = 16;
constexpr int kQueueHeader = 256;  // bytes reserved for the work-queue counter
constexpr int kMixedMaxN = 2048;   // one CTA per system; correction vectors in shared memory

// Right-looking blocked upper Cholesky by the whole CTA.  a has row stride ld;
// only j >= i is read or written.  Each element receives its updates as an FMA
// chain over k ascending.  Returns 0 or k+1 for the first pivot that is not
// positive (NaN included).  Must be entered and left by all threads together.
template <typename T, int NB>
__device__ int cta_potrf_upper(T* a, int ld, int n) {
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int nw = blockDim.x >> 5;
  for (int kb = 0; kb < n; kb += NB) {
    const int ke = min(kb + NB, n);
    for (int k = kb; k < ke; ++k) {
      const T akk = a[k * ld + k];
      if (!(akk > T(0))) return k + 1;  // uniform: every thread read the same value
      const T d = sqrt(akk);
      const T r = T(1) / d;
      for (int j = k + 1 + tid; j < n; j += blockDim.x) a[k * ld + j] *= r;
      __syncthreads();
      if (tid == 0) a[k * ld + k] = d;
      for (int i = k + 1 + warp; i < ke; i += nw) {
        const T uki = a[k * ld + i];
        for (int j = i + lane; j < n; j += 32) a[i * ld + j] = fma(-uki, a[k * ld + j], a[i * ld + j]);
      }
      __syncthreads();
    }
    // Trailing update of rows/cols [ke, n), upper triangle, 64×64 tiles.
    const int m = n - ke;
    if (m > 0) {
      const int tiles = (m + 63) >> 6;
      const int tx = tid & 15, ty = tid >> 4;
      for (int t = 0; t < tiles * tiles; ++t) {
        const int ti = t / tiles, tj = t % tiles;
        if (tj < ti) continue;
        const int i0 = ke + (ti << 6), j0 = ke + (tj << 6);
        T acc[4][4];
#pragma unroll
        for (int r = 0; r < 4; ++r)
#pragma unroll
          for (int c = 0; c < 4; ++c) {
            const int i = i0 + ty + 16 * r, j = j0 + tx + 16 * c;
            acc[r][c] = (i < n && j < n && j >= i) ? a[i * ld + j] : T(0);
          }
        for (int k = kb; k < ke; ++k) {
          T ui[4], uj[4];
#pragma unroll
          for (int r = 0; r < 4; ++r) {
            const int i = i0 + ty + 16 * r;
            ui[r] = (i < n) ? a[k * ld + i] : T(0);
          }
#pragma unroll
          for (int c = 0; c < 4; ++c) {
            const int j = j0 + tx + 16 * c;
            uj[c] = (j < n) ? a[k * ld + j] : T(0);
          }
#pragma unroll
          for (int r = 0; r < 4; ++r)
#pragma unroll
            for (int c = 0; c < 4; ++c) acc[r][c] = fma(-ui[r], uj[c], acc[r][c]);
        }
#pragma unroll
        for (int r = 0; r < 4; ++r)
#pragma unroll
          for (int c = 0; c < 4; ++c) {
            const int i = i0 + ty + 16 * r, j = j0 + tx + 16 * c;
            if (i < n && j < n && j >= i) a[i * ld + j] = acc[r][c];
          }
      }
      __syncthreads();
    }
  }
  return 0;
}

__device__ __forceinline__ int next_system(int* queue, int* s_next) {
  __syncthreads();
  if (threadIdx.x == 0) *s_next = atomicAdd(queue, 1);
  __syncthreads();
  return *s_next;
}

// ---------------------------------------------------------------------------
// Plain FP64 ragged potrf.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kCholThreads)
potrf_ragged_f64_kernel(int64_t batch, int max_n, const int32_t* __restrict__ nvec,
                        const int64_t* __restrict__ a_off, double* __restrict__ a,
                        int32_t* __restrict__ info) {
  extern __shared__ double smem_chol[];
  // Static round-robin over systems: deterministic, and needs no scratch
  // counter (this entry point has no workspace argument).
  for (int64_t s = blockIdx.x; s < batch; s += gridDim.x) {
    __syncthreads();
    const int n = nvec[s];
    double* g = a + a_off[s];
    if (n > max_n || n < 0) {
      if (threadIdx.x == 0) info[s] = -2;
      continue;
    }
    int rc;
    if (n <= kCholSmemMaxF64) {
      const int ld = n | 1;
      for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
        const int i = e / n, j = e - i * n;
        smem_chol[i * ld + j] = g[e];
      }
      __syncthreads();
      rc = cta_potrf_upper<double, 16>(smem_chol, ld, n);
      __syncthreads();
      for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
        const int i = e / n, j = e - i * n;
        g[e] = (j >= i) ? smem_chol[i * ld + j] : 0.0;
      }
    } else {
      rc = cta_potrf_upper<double, 32>(g, n, n);
      __syncthreads();
      for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
        const int i = e / n, j = e - i * n;
        if (j < i) g[e] = 0.0;
      }
    }
    if (threadIdx.x == 0) info[s] = rc;
  }
}

// ---------------------------------------------------------------------------
// FP64 ragged potrs: one CTA per (system, rhs) pair is wasteful for ragged
// batches with few vectors each, so one CTA handles a system and loops over
// its vectors.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kCholThreads)
potrs_ragged_f64_kernel(int64_t batch, int max_n, const int32_t* __restrict__ nvec,
                        const int32_t* __restrict__ nrhs, const int64_t* __restrict__ a_off,
                        const double* __restrict__ u, const int64_t* __restrict__ b_off,
                        double* __restrict__ b) {
  extern __shared__ double smem_x[];
  __shared__ TrsvSmem<double> tsm;
  for (int64_t s = blockIdx.x; s < batch; s += gridDim.x) {
    const int n = nvec[s];
    if (n > max_n || n <= 0) continue;
    const double* U = u + a_off[s];
    for (int r = 0; r < nrhs[s]; ++r) {
      double* g = b + b_off[s] + (int64_t)r * n;
      for (int i = threadIdx.x; i < n; i += blockDim.x) smem_x[i] = g[i];
      __syncthreads();
      cta_trsv<double>(U, n, n, /*lower=*/false, /*trans=*/true, /*unit=*/false, smem_x, tsm);
      cta_trsv<double>(U, n, n, /*lower=*/false, /*trans=*/false, /*unit=*/false, smem_x, tsm);
      for (int i = threadIdx.x; i < n; i += blockDim.x) g[i] = smem_x[i];
      __syncthreads();
    }
  }
}

// ---------------------------------------------------------------------------
// Mixed precision: FP32 factor, FP64 refinement.
// ---------------------------------------------------------------------------
struct MixedSmem {
  TrsvSmem<float> tsm;
  double red[32][kMixedRhsChunk];  // per-warp partial maxima
  double anorm;
  double bnorm[kMixedRhsChunk];
  double berr[kMixedRhsChunk];
  int done[kMixedRhsChunk];
  int next;
  int all_done;
};

// r = b - A x for the vectors [r0, r0+nc) of one system, A FP64 read from
// global memory (one warp per row, lanes along the row).  Writes the FP32
// copy of r into d, and per-vector max|r| and max|x| into red (per warp).
__device__ void residual_f64(const double* __restrict__ A, int n, const double* __restrict__ B,
                             const double* __restrict__ X, int nc, float* d, int ldd,
                             MixedSmem& sm) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  double rmax[kMixedRhsChunk], xmax[kMixedRhsChunk];
#pragma unroll
  for (int c = 0; c < kMixedRhsChunk; ++c) { rmax[c] = 0.0; xmax[c] = 0.0; }
  for (int i = warp; i < n; i += nw) {
    double acc[kMixedRhsChunk];
#pragma unroll
    for (int c = 0; c < kMixedRhsChunk; ++c) acc[c] = 0.0;
    const double* row = A + (int64_t)i * n;
    for (int j = lane; j < n; j += 32) {
      const double aij = row[j];
#pragma unroll
      for (int c = 0; c < kMixedRhsChunk; ++c)
        if (c < nc) acc[c] = fma(aij, X[(int64_t)c * n + j], acc[c]);
    }
#pragma unroll
    for (int c = 0; c < kMixedRhsChunk; ++c) {
      if (c < nc) {
        const double ax = warp_sum(acc[c]);
        const double r = B[(int64_t)c * n + i] - ax;
        if (lane == 0) {
          d[c * ldd + i] = (float)r;
          rmax[c] = fmax(rmax[c], fabs(r));
          xmax[c] = fmax(xmax[c], fabs(X[(int64_t)c * n + i]));
        }
      }
    }
  }
  if (lane == 0) {
#pragma unroll
    for (int c = 0; c < kMixedRhsChunk; ++c) sm.red[warp][c] = rmax[c];
  }
  __syncthreads();
  // fold per-warp maxima: thread c < nc owns vector c.
  if (threadIdx.x < nc) {
    double rm = 0.0;
    for (int w = 0; w < nw; ++w) rm = fmax(rm, sm.red[w][threadIdx.x]);
    sm.berr[threadIdx.x] = rm;  // numerator for now
  }
  __syncthreads();
  if (lane == 0) {
#pragma unroll
    for (int c = 0; c < kMixedRhsChunk; ++c) sm.red[warp][c] = xmax[c];
  }
  __syncthreads();
  if (threadIdx.x < nc) {
    double xm = 0.0;
    for (int w = 0; w < nw; ++w) xm = fmax(xm, sm.red[w][threadIdx.x]);
    const double den = sm.anorm * xm + sm.bnorm[threadIdx.x];
    const double num = sm.berr[threadIdx.x];
    sm.berr[threadIdx.x] = (den > 0.0) ? num / den : (num > 0.0 ? INFINITY : 0.0);
  }
  __syncthreads();
}

__global__ void __launch_bounds__(kCholThreads)
posv_mixed_kernel(int64_t batch, int max_n, int max_nrhs, const int32_t* __restrict__ nvec,
                  const int32_t* __restrict__ nrhs_vec, const int64_t* __restrict__ a_off,
                  const double* __restrict__ a, const int64_t* __restrict__ b_off,
                  const double* __restrict__ b, double* __restrict__ x, double tol, int max_iter,
                  int32_t* __restrict__ info, int32_t* __restrict__ iters,
                  double* __restrict__ berr_out, int* queue, float* __restrict__ factor_ws) {
  extern __shared__ float smem_mixed[];
  __shared__ MixedSmem sm;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nw = blockDim.x >> 5;
  for (;;) {
    const int s = next_system(queue, &sm.next);
    if (s >= batch) break;
    const int n = nvec[s];
    const int nrhs = nrhs_vec[s];
    if (n > max_n || n < 0 || nrhs > max_nrhs || nrhs < 0) {
      if (tid == 0) { info[s] = -2; iters[s] = 0; berr_out[s] = NAN; }
      continue;
    }
    const double* A = a + a_off[s];
    const bool in_smem = n <= kCholSmemMaxF32;
    const int ld = in_smem ? (n | 1) : n;
    float* F = in_smem ? smem_mixed : factor_ws + (int64_t)blockIdx.x * max_n * max_n;
    float* d = in_smem ? smem_mixed + n * ld : smem_mixed;  // correction vectors
    const int ldd = n;
    // Load the upper triangle in FP32 and form ||A||_inf in FP64 from the
    // full stored matrix (the operator whose residual is refined).
    double rowmax = 0.0;
    for (int i = warp; i < n; i += nw) {
      double rs = 0.0;
      for (int j = lane; j < n; j += 32) {
        const double v = A[(int64_t)i * n + j];
        rs += fabs(v);
        if (j >= i) F[i * ld + j] = (float)v;
      }
      rs = warp_sum(rs);
      rowmax = fmax(rowmax, rs);
    }
    if (lane == 0) sm.red[warp][0] = rowmax;
    __syncthreads();
    if (tid == 0) {
      double m = 0.0;
      for (int w = 0; w < nw; ++w) m = fmax(m, sm.red[w][0]);
      sm.anorm = m;
    }
    __syncthreads();
    int rc = in_smem ? cta_potrf_upper<float, 16>(F, ld, n) : cta_potrf_upper<float, 32>(F, ld, n);
    __syncthreads();
    if (rc != 0) {
      for (int e = tid; e < n * nrhs; e += blockDim.x) x[b_off[s] + e] = NAN;
      if (tid == 0) { info[s] = rc; iters[s] = 0; berr_out[s] = NAN; }
      continue;
    }
    double sys_berr = 0.0;
    int sys_iters = 0;
    int sys_info = 0;
    for (int c0 = 0; c0 < nrhs; c0 += kMixedRhsChunk) {
      const int nc = min(kMixedRhsChunk, nrhs - c0);
      const double* B = b + b_off[s] + (int64_t)c0 * n;
      double* X = x + b_off[s] + (int64_t)c0 * n;
      // x = 0, d = (float) b, ||b||_inf
      if (tid < nc) { sm.done[tid] = 0; sm.bnorm[tid] = 0.0; }
      __syncthreads();
      for (int c = 0; c < nc; ++c) {
        double bm = 0.0;
        for (int i = tid; i < n; i += blockDim.x) {
          const double v = B[(int64_t)c * n + i];
          X[(int64_t)c * n + i] = 0.0;
          d[c * ldd + i] = (float)v;
          bm = fmax(bm, fabs(v));
        }
        bm = warp_max(bm);
        if (lane == 0) sm.red[warp][c] = bm;
      }
      __syncthreads();
      if (tid < nc) {
        double m = 0.0;
        for (int w = 0; w < nw; ++w) m = fmax(m, sm.red[w][tid]);
        sm.bnorm[tid] = m;
      }
      __syncthreads();
      int it = 0;
      for (;;) {
        // correction solves with the FP32 factor, for vectors not yet done
        for (int c = 0; c < nc; ++c) {
          if (sm.done[c]) continue;  // uniform: shared value read after a barrier
          cta_trsv<float>(F, ld, n, /*lower=*/false, /*trans=*/true, /*unit=*/false, d + c * ldd, sm.tsm);
          cta_trsv<float>(F, ld, n, /*lower=*/false, /*trans=*/false, /*unit=*/false, d + c * ldd, sm.tsm);
        }
        for (int c = 0; c < nc; ++c) {
          if (sm.done[c]) continue;
          for (int i = tid; i < n; i += blockDim.x) X[(int64_t)c * n + i] += (double)d[c * ldd + i];
        }
        ++it;
        __syncthreads();
        residual_f64(A, n, B, X, nc, d, ldd, sm);
        if (tid == 0) {
          int all = 1;
          for (int c = 0; c < nc; ++c) {
            if (!(sm.berr[c] <= tol) && !sm.done[c]) all = 0;
            if (sm.berr[c] <= tol) sm.done[c] = 1;
          }
          sm.all_done = all;
        }
        __syncthreads();
        if (sm.all_done || it >= max_iter) break;
      }
      if (!sm.all_done) sys_info = -1;
      for (int c = 0; c < nc; ++c) sys_berr = fmax(sys_berr, sm.berr[c]);
      sys_iters = max(sys_iters, it);
      __syncthreads();
    }
    if (tid == 0) { info[s] = sys_info; iters[s] = sys_iters; berr_out[s] = sys_berr; }
  }
}

__global__ void reset_queue_kernel(int* queue) { *queue = 0; }

static int mixed_grid(int64_t batch) {
  const int64_t g = sm_count();
  return (int)((batch < g) ? batch : g);
}

static size_t mixed_smem_bytes(int max_n, int max_nrhs) {
  const int nc = max_nrhs < kMixedRhsChunk ? max_nrhs : kMixedRhsChunk;
  const int ns = max_n < kCholSmemMaxF32 ? max_n : kCholSmemMaxF32;
  size_t small = (size_t)ns * (ns | 1) * sizeof(float) + (size_t)ns * nc * sizeof(float);
  size_t large = (size_t)max_n * nc * sizeof(float);
  return small > large ? small : large;
}

}  // namespace lxgb

using namespace lxgb;

extern "C" int lxgb_potrf_ragged_f64(int64_t batch, int32_t max_n, const int32_t* n,
                                     const int64_t* a_off, double* a, int32_t* info,
                                     void* stream) {
  LXGB_REQUIRE(batch >= 0 && max_n >= 0, "potrf: negative size");
  if (batch == 0) return LXGB_SUCCESSFUL;
  LXGB_REQUIRE(n && a_off && a && info, "potrf: null pointer");
  LXGB_REQUIRE(batch < (1LL << 31), "potrf: batch too large");
  cudaStream_t st = as_stream(stream);
  const int ns = max_n < kCholSmemMaxF64 ? max_n : kCholSmemMaxF64;
  const size_t smem = (size_t)ns * (ns | 1) * sizeof(double);
  LXGB_CUDA_TRY(cudaFuncSetAttribute(potrf_ragged_f64_kernel,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
                "potrf: set smem");
  const int64_t g = sm_count();
  potrf_ragged_f64_kernel<<<(unsigned)(batch < g ? batch : g), kCholThreads, smem, st>>>(
      batch, max_n, n, a_off, a, info);
  return check_launch("potrf ragged");
}

extern "C" int lxgb_potrs_ragged_f64(int64_t batch, int32_t max_n, const int32_t* n,
                                     const int32_t* nrhs, const int64_t* a_off, const double* u,
                                     const int64_t* b_off, double* b, void* stream) {
  LXGB_REQUIRE(batch >= 0 && max_n >= 0, "potrs: negative size");
  if (batch == 0 || max_n == 0) return LXGB_SUCCESSFUL;
  LXGB_REQUIRE(n && nrhs && a_off && u && b_off && b, "potrs: null pointer");
  const size_t smem = (size_t)max_n * sizeof(double);
  LXGB_REQUIRE(smem <= 160 * 1024, "potrs: max_n too large for the shared-memory vector");
  LXGB_CUDA_TRY(cudaFuncSetAttribute(potrs_ragged_f64_kernel,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
                "potrs: set smem");
  const int64_t g = 4 * (int64_t)sm_count();
  potrs_ragged_f64_kernel<<<(unsigned)(batch < g ? batch : g), kCholThreads, smem,
                            as_stream(stream)>>>(batch, max_n, n, nrhs, a_off, u, b_off, b);
  return check_launch("potrs ragged");
}

extern "C" int64_t lxgb_posv_ragged_mixed_workspace_size(int64_t batch, int32_t max_n,
                                                         int32_t max_nrhs) {
  (void)max_nrhs;
  if (batch <= 0 || max_n <= 0) return kQueueHeader;
  int64_t bytes = kQueueHeader;
  if (max_n > kCholSmemMaxF32)
    bytes += (int64_t)mixed_grid(batch) * max_n * max_n * (int64_t)sizeof(float);
  return bytes;
}

extern "C" int lxgb_posv_ragged_mixed(int64_t batch, int32_t max_n, int32_t max_nrhs,
                                      const int32_t* n, const int32_t* nrhs, const int64_t* a_off,
                                      const double* a, const int64_t* b_off, const double* b,
                                      double* x, double tol, int32_t max_iter, int32_t* info,
                                      int32_t* iters, double* berr, void* work,
                                      int64_t work_bytes, void* stream) {
  LXGB_REQUIRE(batch >= 0 && max_n >= 0 && max_nrhs >= 0, "posv_mixed: negative size");
  if (batch == 0) return LXGB_SUCCESSFUL;
  LXGB_REQUIRE(batch < (1LL << 31), "posv_mixed: batch too large");
  LXGB_REQUIRE(n && nrhs && a_off && a && b_off && b && x && info && iters && berr && work,
               "posv_mixed: null pointer");
  LXGB_REQUIRE(max_iter >= 1, "posv_mixed: max_iter must be >= 1");
  LXGB_REQUIRE(((uintptr_t)work & 255) == 0, "posv_mixed: workspace must be 256-byte aligned");
  if (work_bytes < lxgb_posv_ragged_mixed_workspace_size(batch, max_n, max_nrhs)) {
    set_last_error("posv_mixed: workspace too small");
    return LXGB_WORKSPACE_TOO_SMALL;
  }
  cudaStream_t st = as_stream(stream);
  int* queue = reinterpret_cast<int*>(work);
  float* factor_ws = reinterpret_cast<float*>(reinterpret_cast<char*>(work) + kQueueHeader);
  reset_queue_kernel<<<1, 1, 0, st>>>(queue);
  const size_t smem = mixed_smem_bytes(max_n, max_nrhs);
  LXGB_REQUIRE(max_n <= kMixedMaxN, "posv_mixed: max_n above 2048");
  LXGB_CUDA_TRY(cudaFuncSetAttribute(posv_mixed_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)smem),
                "posv_mixed: set smem");
  posv_mixed_kernel<<<(unsigned)mixed_grid(batch), kCholThreads, smem, st>>>(
      batch, max_n, max_nrhs, n, nrhs, a_off, a, b_off, b, x, tol, max_iter, info, iters, berr,
      queue, factor_ws);
  return check_launch("posv_mixed");
}

// ---------------------------------------------------------------------------
// Allocation-free variant of lxgb_posv_ragged_mixed.
//
// Some callers cannot allocate device memory at the moment they need a solve:
// an XLA/JAX FFI handler owns no allocator of its own (device memory belongs to
// XLA, and a cudaMalloc inside the handler can synchronise the device or break
// a CUDA-graph capture XLA is recording), and a serving loop or real-time
// controller may forbid allocation once it has started.  For them the scratch
// of the mixed solve (work-queue counter + FP32 factors of systems too large for
// shared memory) lives in the fixed array below, which every GPU that loads this
// library holds until the process exits.
// ---------------------------------------------------------------------------
#include <mutex>

namespace lxgb {

static __device__ __align__(256) unsigned char g_posv_noalloc_scratch[LXGB_POSV_NOALLOC_SCRATCH_BYTES];

constexpr int kNoallocMaxDevices = 64;
static void* g_noalloc_addr[kNoallocMaxDevices] = {nullptr};
static std::mutex g_noalloc_mu;

// Device address of the scratch array on the current device, looked up once
// per device (the host-side symbol is not a device address).
static int noalloc_scratch_address(void** out) {
  int dev = -1;
  LXGB_CUDA_TRY(cudaGetDevice(&dev), "posv_mixed_noalloc: cudaGetDevice");
  if (dev < 0 || dev >= kNoallocMaxDevices) {
    set_last_error("posv_mixed_noalloc: device ordinal %d out of range", dev);
    return LXGB_INVALID_ARG;
  }
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  if (g_noalloc_addr[dev] == nullptr) {
    void* p = nullptr;
    LXGB_CUDA_TRY(cudaGetSymbolAddress(&p, g_posv_noalloc_scratch),
                  "posv_mixed_noalloc: cudaGetSymbolAddress");
    g_noalloc_addr[dev] = p;
  }
  *out = g_noalloc_addr[dev];
  return LXGB_SUCCESSFUL;
}

}  // namespace lxgb

extern "C" int lxgb_posv_ragged_mixed_noalloc(int64_t batch, int32_t max_n, int32_t max_nrhs,
                                              const int32_t* n, const int32_t* nrhs,
                                              const int64_t* a_off, const double* a,
                                              const int64_t* b_off, const double* b, double* x,
                                              double tol, int32_t max_iter, int32_t* info,
                                              int32_t* iters, double* berr, void* stream) {
  LXGB_REQUIRE(batch >= 0 && max_n >= 0 && max_nrhs >= 0, "posv_mixed_noalloc: negative size");
  if (batch == 0) return LXGB_SUCCESSFUL;
  LXGB_REQUIRE(batch < (1LL << 31), "posv_mixed_noalloc: batch too large");
  LXGB_REQUIRE(n && nrhs && a_off && a && b_off && b && x && info && iters && berr,
               "posv_mixed_noalloc: null pointer");
  LXGB_REQUIRE(max_iter >= 1, "posv_mixed_noalloc: max_iter must be >= 1");
  LXGB_REQUIRE(max_n <= kMixedMaxN,
               "posv_mixed_noalloc: max_n above 2048 (its FP32 factor exceeds the fixed scratch)");
  // Grid: one FP32 factor slice per CTA for systems above the shared-memory
  // size, as many slices as the fixed scratch holds.
  int64_t grid = sm_count();
  if (batch < grid) grid = batch;
  if (max_n > kCholSmemMaxF32) {
    const int64_t slice = (int64_t)max_n * max_n * (int64_t)sizeof(float);
    const int64_t slices = (int64_t)(LXGB_POSV_NOALLOC_SCRATCH_BYTES - kQueueHeader) / slice;
    if (slices < 1) {
      set_last_error("posv_mixed_noalloc: max_n=%d needs %lld bytes of scratch, limit %lld", max_n,
                     (long long)(slice + kQueueHeader),
                     (long long)LXGB_POSV_NOALLOC_SCRATCH_BYTES);
      return LXGB_INVALID_ARG;
    }
    if (slices < grid) grid = slices;
  }
  void* scratch = nullptr;
  int rc = noalloc_scratch_address(&scratch);
  if (rc) return rc;
  cudaStream_t st = as_stream(stream);
  int* queue = reinterpret_cast<int*>(scratch);
  float* factor_ws = reinterpret_cast<float*>(reinterpret_cast<char*>(scratch) + kQueueHeader);
  reset_queue_kernel<<<1, 1, 0, st>>>(queue);  // the array keeps the previous call's counter
  const size_t smem = mixed_smem_bytes(max_n, max_nrhs);
  LXGB_CUDA_TRY(cudaFuncSetAttribute(posv_mixed_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)smem),
                "posv_mixed_noalloc: set smem");
  posv_mixed_kernel<<<(unsigned)grid, kCholThreads, smem, st>>>(
      batch, max_n, max_nrhs, n, nrhs, a_off, a, b_off, b, x, tol, max_iter, info, iters, berr,
      queue, factor_ws);
  return check_launch("posv_mixed_noalloc");
}
