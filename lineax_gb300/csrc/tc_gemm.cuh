// Host-side launcher of the tcgen05 TF32 GEMM (tc_gemm.cu) for other
// translation units: C = alpha * A Bᵀ + beta * C, A m×k, B n×k (K-major).
#pragma once

#include "common.cuh"

namespace lxgb {
int gemm_tf32_nt(int M, int N, int K, const float* A, int64_t lda, const float* B, int64_t ldb,
                 float* C, int64_t ldc, float alpha, float beta, int* err, cudaStream_t st);
// 3xTF32 when Al and Bl (the lo parts) are given, plain TF32 otherwise.
int gemm_tf32_nt_split(int M, int N, int K, const float* A, const float* Al, int64_t lda,
                       const float* B, const float* Bl, int64_t ldb, float* C, int64_t ldc,
                       float alpha, float beta, int* err, cudaStream_t st);
// C = alpha A Aᵀ + beta C on the tiles holding C's lower triangle (M×M),
// 3xTF32 when Al is given; the full product when tiles cannot be skipped.
int gemm_tf32_nt_split_lower(int M, int K, const float* A, const float* Al, int64_t lda, float* C,
                             int64_t ldc, float alpha, float beta, int* err, cudaStream_t st);
// X = L_jj^{-1} W on rows [j0, j0+nb) of w, columns [c_begin, c_end), L_jj
// the unit-lower 64-block of lu at (j0, j0) (row stride n; lu and w may be
// the same array when the columns are disjoint from the block).  X goes back
// into w and, transposed and zero padded to 64 entries per column, into xt
// (ir.cu).
int launch_inv_diag_lower(int n, int j0, int nb, const float* lu, float* w, int c_begin,
                          int c_end, float* xt, cudaStream_t st);
// Split-K products C_s = A[:, K_s] B[:, K_s]ᵀ (K_s: splits ranges of chunk
// elements, chunk % 32 == 0), C_s at C + s * M * ldc, in one launch.
int gemm_tf32_nt_splitk(int M, int N, int K, const float* A, int64_t lda, const float* B,
                        int64_t ldb, float* C, int64_t ldc, int chunk, int splits, int* err,
                        cudaStream_t st);
// BF16 operands (kind::f16, FP32 accumulation); A and B hold __nv_bfloat16.
int gemm_bf16_nt(int M, int N, int K, const void* A, int64_t lda, const void* B, int64_t ldb,
                 float* C, int64_t ldc, float alpha, float beta, int* err, cudaStream_t st);
// dst = src rounded to BF16 (rows × cols; row strides in elements).
int bf16_convert(int64_t rows, int64_t cols, const float* src, int64_t lds, void* dst, int64_t ldd,
                 cudaStream_t st);
// hi/lo split of a rows×cols block (row stride lds) into hi, lo (row stride ldd).
int tf32_split(int64_t rows, int64_t cols, const float* src, int64_t lds, float* hi, float* lo,
               int64_t ldd, cudaStream_t st);
}
