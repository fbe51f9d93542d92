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
// hi/lo split of a rows×cols block (row stride lds) into hi, lo (row stride ldd).
int tf32_split(int64_t rows, int64_t cols, const float* src, int64_t lds, float* hi, float* lo,
               int64_t ldd, cudaStream_t st);
}
