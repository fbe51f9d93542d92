// General triangular solve op(T) X = B (lower/upper, trans, unit diagonal),
// FP64, one CTA per right-hand side with the vector staged in shared memory.
#include "common.cuh"
#include "tri.cuh"

namespace lxgb {

constexpr int kTrsmThreads = 256;

__global__ void __launch_bounds__(kTrsmThreads)
trsm_kernel(int n, const double* __restrict__ t, int64_t ldt, int lower, int trans, int unit,
            double* __restrict__ b, int in_smem) {
  extern __shared__ double smem_v[];
  __shared__ TrsvSmem<double> tsm;
  double* g = b + (int64_t)blockIdx.x * n;
  double* x = in_smem ? smem_v : g;
  if (in_smem) {
    for (int i = threadIdx.x; i < n; i += blockDim.x) x[i] = g[i];
    __syncthreads();
  }
  cta_trsv<double>(t, ldt, n, lower != 0, trans != 0, unit != 0, x, tsm);
  if (in_smem)
    for (int i = threadIdx.x; i < n; i += blockDim.x) g[i] = x[i];
}

}  // namespace lxgb

using namespace lxgb;

extern "C" int lxgb_trsm_f64(int32_t n, int32_t nrhs, const double* t, int64_t ldt, int32_t lower,
                             int32_t trans, int32_t unit_diag, double* b, void* stream) {
  LXGB_REQUIRE(n >= 0 && nrhs >= 0, "trsm: negative size");
  if (n == 0 || nrhs == 0) return LXGB_SUCCESSFUL;
  LXGB_REQUIRE(t && b, "trsm: null pointer");
  LXGB_REQUIRE(ldt >= n, "trsm: ldt < n");
  const size_t need = (size_t)n * sizeof(double);
  const int in_smem = need <= 160 * 1024;
  const size_t smem = in_smem ? need : 0;
  if (in_smem)
    LXGB_CUDA_TRY(ensure_dynamic_smem(reinterpret_cast<const void*>(trsm_kernel), (int)smem),
                  "trsm: set smem");
  trsm_kernel<<<(unsigned)nrhs, kTrsmThreads, smem, as_stream(stream)>>>(
      n, t, ldt, lower, trans, unit_diag, b, in_smem);
  return check_launch("trsm");
}
