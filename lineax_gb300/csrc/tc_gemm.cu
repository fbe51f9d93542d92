// Tensor-core GEMM on the 5th-generation tensor cores (tcgen05), TF32 inputs,
// FP32 accumulation in tensor memory:  C = alpha * A Bᵀ + beta * C.
//
// A is M×K and B is N×K, both row-major with K contiguous (K-major operands);
// C is M×N row-major.  This is the trailing-matrix update of the blocked
// factorisations (A22 -= L21 U12 with B = U12ᵀ).
//
// One CTA of 128 threads computes a 128×128 tile of C:
//   * warp 0 / lane 0 streams 128×32 tiles of A and B into shared memory with
//     TMA (cp.async.bulk.tensor, 128-byte swizzle) through a kStages-deep ring
//     guarded by "full" / "empty" mbarriers;
//   * warp 1 / lane 0 issues tcgen05.mma (M=128, N=128, K=8 per instruction)
//     into a 128-column FP32 accumulator in tensor memory and returns each
//     stage to the producer with tcgen05.commit;
//   * all four warps read the accumulator back with tcgen05.ld (each warp owns
//     32 TMEM lanes = 32 rows) and update C.
// Every mbarrier wait is bounded: on timeout the kernel records an error code
// in *err, waits (bounded) for the MMAs it issued, frees its tensor memory and
// returns, so a broken pipeline cannot hang the GPU.
#include <cuda.h>
#include <cudaTypedefs.h>

#include "common.cuh"
#include "tcgen05.cuh"

#include <cuda_bf16.h>

namespace lxgb {

constexpr int kTcM = 128;
constexpr int kTcN = 128;
constexpr int kTcK = 32;        // K elements per stage (128 bytes of FP32 = one swizzle row)
constexpr int kTcStages = 4;       // TF32: 32 KB per stage
constexpr int kTcStagesSplit = 3;  // 3xTF32: 64 KB per stage (hi and lo tiles)
constexpr int kTcThreads = 128;
constexpr int kTcTileBytes = kTcM * kTcK * 4;  // 16 KB per operand tile

template <int S, bool SPLIT>
struct TcSmem {
  alignas(1024) float a[S][kTcM * kTcK];
  alignas(1024) float b[S][kTcN * kTcK];
  alignas(1024) float al[SPLIT ? S : 1][SPLIT ? kTcM * kTcK : 1];
  alignas(1024) float bl[SPLIT ? S : 1][SPLIT ? kTcN * kTcK : 1];
  alignas(8) unsigned long long full[S];
  alignas(8) unsigned long long empty[S];
  alignas(8) unsigned long long done;
  alignas(8) unsigned long long cfull;  // old C tile landed (TMA epilogue)
  unsigned tmem_base;
  int abort;
};

// The TMA epilogue stages the 128×128 FP32 C tile (64 KB) in the stage buffers.
static_assert(sizeof(TcSmem<kTcStages, false>::a) + sizeof(TcSmem<kTcStages, false>::b) >=
                  4 * kTcTileBytes, "C tile does not fit the TF32 stage buffers");
static_assert(sizeof(TcSmem<kTcStagesSplit, true>::a) + sizeof(TcSmem<kTcStagesSplit, true>::b) >=
                  4 * kTcTileBytes, "C tile does not fit the 3xTF32 stage buffers");

__device__ __forceinline__ void mbar_expect_tx(unsigned long long* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}

__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, int x, int y,
                                            unsigned long long* bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3}], [%4];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<unsigned long long>(map)), "r"(x), "r"(y), "r"(smem_u32(bar))
      : "memory");
}

__device__ __forceinline__ void tma_store_2d(const CUtensorMap* map, int x, int y, const void* src) {
  asm volatile("cp.async.bulk.tensor.2d.global.shared::cta.bulk_group [%0, {%1, %2}], [%3];" ::"l"(
                   reinterpret_cast<unsigned long long>(map)),
               "r"(x), "r"(y), "r"(smem_u32(src))
               : "memory");
}

// MODE 0: TF32 operands (FP32 in memory, read as TF32).
// MODE 1 (3xTF32): A = Ah + Al and B = Bh + Bl with TF32-exact hi parts;
// A Bᵀ ~= Ah Bhᵀ + Ah Blᵀ + Al Bhᵀ accumulated in the same tensor memory,
// which restores FP32-level accuracy.
// MODE 2: BF16 operands in memory (tcgen05.mma kind::f16, both operands
// BF16, FP32 accumulation): a 128-byte shared-memory row holds 64 of them,
// so a stage covers K = 64 with the same layout and 32-byte K steps.
template <int MODE>
__global__ void __launch_bounds__(kTcThreads, 1)
gemm_tf32_nt_kernel(const __grid_constant__ CUtensorMap map_a,
                    const __grid_constant__ CUtensorMap map_b,
                    const __grid_constant__ CUtensorMap map_al,
                    const __grid_constant__ CUtensorMap map_bl,
                    const __grid_constant__ CUtensorMap map_c, int use_tma_c, int M, int N, int K,
                    float* C, int64_t ldc, float alpha, float beta, int* err,
                    int k_split_tiles, int64_t c_split_stride) {
  constexpr bool SPLIT = MODE == 1;
  constexpr bool BF = MODE == 2;
  constexpr int kK = BF ? 2 * kTcK : kTcK;  // K elements per 128-byte stage row
  constexpr int kStages = SPLIT ? kTcStagesSplit : kTcStages;
  using Smem = TcSmem<kStages, SPLIT>;
  extern __shared__ unsigned char smem_raw[];
  Smem& sm = *reinterpret_cast<Smem*>(
      (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~static_cast<uintptr_t>(1023));
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int m0 = blockIdx.y * kTcM, n0 = blockIdx.x * kTcN;
  // split-K: CTA layer z takes k-tiles [z * k_split_tiles, ...) and writes its
  // own C block at C + z * c_split_stride
  int t_begin = 0;
  int ktiles = (K + kK - 1) / kK;
  if (k_split_tiles > 0) {
    t_begin = (int)blockIdx.z * k_split_tiles;
    ktiles = max(0, min(ktiles - t_begin, k_split_tiles));
    C += (int64_t)blockIdx.z * c_split_stride;
  }

  if (threadIdx.x == 0) {
    for (int s = 0; s < kStages; ++s) {
      mbar_init(&sm.full[s], 1);
      mbar_init(&sm.empty[s], 1);
    }
    mbar_init(&sm.done, 1);
    mbar_init(&sm.cfull, 1);
    sm.abort = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {  // 128 TMEM columns for the 128×128 FP32 accumulator
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 128;" ::"r"(
                     smem_u32(&sm.tmem_base))
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const unsigned tmem = sm.tmem_base;

  if (warp == 0 && lane == 0) {
    // TMA producer
    for (int t = 0; t < ktiles; ++t) {
      const int s = t % kStages, r = t / kStages;
      if (!mbar_wait(&sm.empty[s], (r & 1) ^ 1)) { atomicExch(&sm.abort, 1); break; }
      if (*reinterpret_cast<volatile int*>(&sm.abort)) break;
      mbar_expect_tx(&sm.full[s], (SPLIT ? 4 : 2) * kTcTileBytes);
      tma_load_2d(sm.a[s], &map_a, (t_begin + t) * kK, m0, &sm.full[s]);
      tma_load_2d(sm.b[s], &map_b, (t_begin + t) * kK, n0, &sm.full[s]);
      if constexpr (SPLIT) {
        tma_load_2d(sm.al[s], &map_al, (t_begin + t) * kTcK, m0, &sm.full[s]);
        tma_load_2d(sm.bl[s], &map_bl, (t_begin + t) * kTcK, n0, &sm.full[s]);
      }
    }
  } else if (warp == 1 && lane == 0) {
    // MMA issuer
    constexpr unsigned idesc = BF ? idesc_bf16(kTcM, kTcN) : idesc_tf32(kTcM, kTcN);
    int issued = 0;
    for (int t = 0; t < ktiles; ++t) {
      const int s = t % kStages, r = t / kStages;
      if (!mbar_wait(&sm.full[s], r & 1)) { atomicExch(&sm.abort, 1); break; }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
#pragma unroll
      for (int k = 0; k < kTcK / 8; ++k) {  // K = 8 TF32 (32 bytes) per instruction
        const unsigned long long ad = smem_desc_sw128(sm.a[s]) + ((k * 32) >> 4);
        const unsigned long long bd = smem_desc_sw128(sm.b[s]) + ((k * 32) >> 4);
        if constexpr (BF)
          mma_bf16(tmem, ad, bd, idesc, (t > 0 || k > 0) ? 1 : 0);
        else
          mma_tf32(tmem, ad, bd, idesc, (t > 0 || k > 0) ? 1 : 0);
        if constexpr (SPLIT) {
          const unsigned long long ald = smem_desc_sw128(sm.al[s]) + ((k * 32) >> 4);
          const unsigned long long bld = smem_desc_sw128(sm.bl[s]) + ((k * 32) >> 4);
          mma_tf32(tmem, ad, bld, idesc, 1);
          mma_tf32(tmem, ald, bd, idesc, 1);
        }
      }
      mma_commit(&sm.empty[s]);
      issued = 1;
    }
    if (issued) {
      mma_commit(&sm.done);
    } else {
      // nothing issued (K == 0 or abort before the first stage): release the epilogue
      asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(&sm.done)) : "memory");
    }
  }
  __syncwarp();
  const bool done_ok = mbar_wait(&sm.done, 0);
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  if (!done_ok || sm.abort) {
    if (threadIdx.x == 0) atomicExch(err, 1);
  } else if (use_tma_c) {
    // Epilogue through shared memory: the old C tile arrives by TMA into the
    // (now idle) stage buffers as four 128-row × 32-column boxes with the
    // 128-byte swizzle, each thread updates its row in place (16-byte granule
    // g of row r sits at g ^ (r & 7): conflict-free), and TMA stores the tile
    // (rows and columns past M, N are clipped by the tensor map).
    float* cbuf = &sm.a[0][0];  // 64 KB: a[] and, for 3 stages, b[0] follow contiguously
    const bool has_acc = ktiles > 0;
    bool c_ok = true;
    if (beta != 0.0f) {
      if (threadIdx.x == 0) {
        mbar_expect_tx(&sm.cfull, 4 * kTcTileBytes);
#pragma unroll
        for (int i = 0; i < 4; ++i) tma_load_2d(cbuf + i * kTcM * kTcK, &map_c, n0 + 32 * i, m0,
                                                &sm.cfull);
      }
      c_ok = mbar_wait(&sm.cfull, 0);
    }
    if (!c_ok) {
      if (threadIdx.x == 0) atomicExch(err, 1);
    } else {
      const int r = warp * 32 + lane;
#pragma unroll 1
      for (int i = 0; i < 4; ++i) {
        float v[32];
        if (has_acc) {
          tmem_ld32(tmem + ((unsigned)(warp * 32) << 16) + (unsigned)(32 * i), v);
        } else {
#pragma unroll
          for (int e = 0; e < 32; ++e) v[e] = 0.0f;
        }
        char* rowp = reinterpret_cast<char*>(cbuf + i * kTcM * kTcK) + r * 128;
#pragma unroll
        for (int g = 0; g < 8; ++g) {
          float4* q = reinterpret_cast<float4*>(rowp + ((g ^ (r & 7)) << 4));
          float4 o = (beta != 0.0f) ? *q : make_float4(0.f, 0.f, 0.f, 0.f);
          o.x = fmaf(alpha, v[4 * g + 0], beta == 0.0f ? 0.0f : beta * o.x);
          o.y = fmaf(alpha, v[4 * g + 1], beta == 0.0f ? 0.0f : beta * o.y);
          o.z = fmaf(alpha, v[4 * g + 2], beta == 0.0f ? 0.0f : beta * o.z);
          o.w = fmaf(alpha, v[4 * g + 3], beta == 0.0f ? 0.0f : beta * o.w);
          *q = o;
        }
      }
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    __syncthreads();
    if (c_ok && threadIdx.x == 0) {
#pragma unroll
      for (int i = 0; i < 4; ++i) tma_store_2d(&map_c, n0 + 32 * i, m0, cbuf + i * kTcM * kTcK);
      asm volatile("cp.async.bulk.commit_group;" ::: "memory");
      asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");
    }
  } else {    // Epilogue: warp w owns rows 32w..32w+31 (TMEM lanes), 32 columns per load.
    const int row = m0 + warp * 32 + lane;
    const bool has_acc = ktiles > 0;
#pragma unroll 1
    for (int c0 = 0; c0 < kTcN; c0 += 32) {
      float v[32];
      if (has_acc) {
        tmem_ld32(tmem + ((unsigned)(warp * 32) << 16) + (unsigned)c0, v);
      } else {
#pragma unroll
        for (int i = 0; i < 32; ++i) v[i] = 0.0f;
      }
      if (row < M) {
        float* crow = C + (int64_t)row * ldc + n0 + c0;
#pragma unroll
        for (int i = 0; i < 32; ++i) {
          if (n0 + c0 + i < N) {
            const float old = (beta == 0.0f) ? 0.0f : beta * crow[i];
            crow[i] = fmaf(alpha, v[i], old);
          }
        }
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 128;" ::"r"(tmem) : "memory");
  }
}

// ---------------------------------------------------------------------------
// Persistent, warp-specialised form: one CTA per SM walks the output tiles
// (BN = 256 columns for TF32 and BF16, 128 for 3xTF32) with two tensor-memory
// accumulators, so the epilogue of tile i overlaps the MMAs of tile i+1.
//   warp 0 lane 0   TMA producer: A and B stages into a kPS-deep ring;
//   warp 1          allocates tensor memory; lane 0 issues tcgen05.mma into
//                   accumulator (tile & 1) once the epilogue has emptied it;
//   warps 2..5      epilogue: warp w reads TMEM lanes 32 (w % 4) ..+31 (rows
//                   of the tile), 32 columns at a time; the old C chunk
//                   (32 × 32) arrives by TMA one chunk ahead into a private
//                   double buffer, is updated in place and leaves by TMA.
// Tile order: groups of 8 row blocks, column blocks inside a group, so the
// CTAs running at the same time share A rows and B columns in L2.
// ---------------------------------------------------------------------------
constexpr int kPThreads = 192;
constexpr int kPEpiChunk = 32 * 32 * 4;  // one 32-row × 32-column FP32 C chunk

template <int MODE, int S_, int CB_>
struct PCfg {
  static constexpr bool SPLIT = MODE == 1;
  static constexpr int BN = SPLIT ? 128 : 256;
  static constexpr int S = S_;                       // operand stages
  static constexpr int CB = CB_;                     // C staging buffers per epilogue warp
  static constexpr int A_BYTES = kTcM * 128;         // 128 rows of 128 bytes
  static constexpr int B_BYTES = BN * 128;
  static constexpr int STAGE_BYTES = (A_BYTES + B_BYTES) * (SPLIT ? 2 : 1);
  static constexpr int OFF_B = S * A_BYTES;
  static constexpr int OFF_AL = OFF_B + S * B_BYTES;
  static constexpr int OFF_BL = OFF_AL + (SPLIT ? S * A_BYTES : 0);
  static constexpr int OFF_C = OFF_BL + (SPLIT ? S * B_BYTES : 0);
  static constexpr int OFF_BAR = OFF_C + 4 * CB * kPEpiChunk;
  // full[S], empty[S], tfull[2], tempty[2], cbar[4][CB], done, then tmem base and abort
  static constexpr int BAR_COUNT = 2 * S + 4 + 4 * CB + 1;
  static constexpr int BYTES = OFF_BAR + BAR_COUNT * 8 + 16;
  static constexpr int SMEM = BYTES + 1024;          // slack to align the base to 1 KB
  static constexpr unsigned TMEM_COLS = 2 * BN;
};
// Long K: four operand stages keep the tensor pipe fed; short K (the rank-64
// updates of the factorisations, one or two stages per tile): two stages and
// six C buffers per warp, so that five chunks of old C (80 KB per SM) are in
// flight while the epilogue streams C through HBM.
using PCfgTf32 = PCfg<0, 4, 2>;
using PCfgTf32ShortK = PCfg<0, 2, 6>;
using PCfgSplit = PCfg<1, 3, 2>;
using PCfgBf16 = PCfg<2, 4, 2>;
using PCfgBf16ShortK = PCfg<2, 2, 6>;
static_assert(PCfgTf32::SMEM <= 232448 && PCfgTf32ShortK::SMEM <= 232448 &&
                  PCfgSplit::SMEM <= 232448 && PCfgBf16::SMEM <= 232448 &&
                  PCfgBf16ShortK::SMEM <= 232448,
              "persistent GEMM exceeds shared memory");

// Lower mode (C symmetric, only its lower triangle wanted): the tiles that
// hold a part of the lower triangle, row block by row block.
__device__ __forceinline__ int lower_tiles_in_row(int mb, int n_nblk, int bn) {
  return min(n_nblk, (mb * 128 + 127) / bn + 1);
}

__device__ __forceinline__ void tile_coords_lower(int tile, int n_mblk, int n_nblk, int bn,
                                                  int& mb, int& nb) {
  mb = 0;
  for (; mb < n_mblk - 1; ++mb) {
    const int c = lower_tiles_in_row(mb, n_nblk, bn);
    if (tile < c) break;
    tile -= c;
  }
  nb = tile;
}

__device__ __forceinline__ void tile_coords(int tile, int n_mblk, int n_nblk, int& mb, int& nb) {
  constexpr int G = 8;
  const int per_group = G * n_nblk;
  const int group = tile / per_group;
  const int first = group * G;
  const int gsize = min(n_mblk - first, G);
  const int in = tile - group * per_group;
  mb = first + in % gsize;
  nb = in / gsize;
}

template <int MODE, class Cfg>
__global__ void __launch_bounds__(kPThreads, 1)
gemm_nt_persistent_kernel(const __grid_constant__ CUtensorMap map_a,
                          const __grid_constant__ CUtensorMap map_b,
                          const __grid_constant__ CUtensorMap map_al,
                          const __grid_constant__ CUtensorMap map_bl,
                          const __grid_constant__ CUtensorMap map_c, int M, int N, int K,
                          float alpha, float beta, int* err, int lower) {
  constexpr bool SPLIT = Cfg::SPLIT;
  constexpr bool BF = MODE == 2;
  constexpr int BN = Cfg::BN, S = Cfg::S;
  constexpr int kK = BF ? 2 * kTcK : kTcK;
  extern __shared__ unsigned char smem_raw[];
  unsigned char* base = reinterpret_cast<unsigned char*>(
      (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~static_cast<uintptr_t>(1023));
  unsigned long long* bars = reinterpret_cast<unsigned long long*>(base + Cfg::OFF_BAR);
  unsigned long long* full = bars;
  unsigned long long* empty = bars + S;
  unsigned long long* tfull = bars + 2 * S;
  unsigned long long* tempty = bars + 2 * S + 2;
  constexpr int CB = Cfg::CB;
  unsigned long long* cbar = bars + 2 * S + 4;   // [4][CB]
  unsigned long long* done = bars + 2 * S + 4 + 4 * CB;
  unsigned* tmem_slot = reinterpret_cast<unsigned*>(bars + Cfg::BAR_COUNT);
  int* abort_flag = reinterpret_cast<int*>(tmem_slot + 1);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int n_mblk = (M + kTcM - 1) / kTcM, n_nblk = (N + BN - 1) / BN;
  int tiles = n_mblk * n_nblk;
  if (lower) {
    tiles = 0;
    for (int mb = 0; mb < n_mblk; ++mb) tiles += lower_tiles_in_row(mb, n_nblk, BN);
  }
  auto coords = [&](int tile, int& mb, int& nb) {
    if (lower)
      tile_coords_lower(tile, n_mblk, n_nblk, BN, mb, nb);
    else
      tile_coords(tile, n_mblk, n_nblk, mb, nb);
  };
  const int ktiles = (K + kK - 1) / kK;

  if (threadIdx.x == 0) {
    for (int i = 0; i < Cfg::BAR_COUNT; ++i) mbar_init(&bars[i], 1);
    mbar_init(&tempty[0], 4);
    mbar_init(&tempty[1], 4);
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(tmem_slot)), "r"(Cfg::TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const unsigned tmem = *tmem_slot;
  volatile int* vabort = abort_flag;

  if (warp == 0) {
    if (lane == 0) {
      // ---------------- TMA producer ----------------
      int it = 0;
      for (int tile = blockIdx.x; tile < tiles && !*vabort; tile += gridDim.x) {
        int mb, nb;
        coords(tile, mb, nb);
        for (int t = 0; t < ktiles; ++t, ++it) {
          const int s = it % S, r = it / S;
          if (!mbar_wait(&empty[s], (r & 1) ^ 1)) { atomicExch(abort_flag, 1); break; }
          if (*vabort) break;
          mbar_expect_tx(&full[s], Cfg::STAGE_BYTES);
          tma_load_2d(base + s * Cfg::A_BYTES, &map_a, t * kK, mb * kTcM, &full[s]);
          tma_load_2d(base + Cfg::OFF_B + s * Cfg::B_BYTES, &map_b, t * kK, nb * BN, &full[s]);
          if constexpr (SPLIT) {
            tma_load_2d(base + Cfg::OFF_AL + s * Cfg::A_BYTES, &map_al, t * kK, mb * kTcM,
                        &full[s]);
            tma_load_2d(base + Cfg::OFF_BL + s * Cfg::B_BYTES, &map_bl, t * kK, nb * BN,
                        &full[s]);
          }
        }
      }
      // the last S stages issued have landed before shared memory is released
      for (int j = (it > S ? it - S : 0); j < it; ++j)
        if (!mbar_wait(&full[j % S], (j / S) & 1)) atomicExch(abort_flag, 1);
    }
  } else if (warp == 1) {
    if (lane == 0) {
      // ---------------- MMA issuer ----------------
      constexpr unsigned idesc = BF ? idesc_bf16(kTcM, BN) : idesc_tf32(kTcM, BN);
      int it = 0, tc = 0;
      for (int tile = blockIdx.x; tile < tiles && !*vabort; tile += gridDim.x, ++tc) {
        const int buf = tc & 1, use = tc >> 1;
        if (!mbar_wait(&tempty[buf], (use & 1) ^ 1)) { atomicExch(abort_flag, 1); break; }
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const unsigned d = tmem + (unsigned)(buf * BN);
        bool ok = true;
        for (int t = 0; t < ktiles; ++t, ++it) {
          const int s = it % S, r = it / S;
          if (!mbar_wait(&full[s], r & 1)) { atomicExch(abort_flag, 1); ok = false; break; }
          asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
          const unsigned char* sa = base + s * Cfg::A_BYTES;
          const unsigned char* sb = base + Cfg::OFF_B + s * Cfg::B_BYTES;
#pragma unroll
          for (int k = 0; k < 4; ++k) {  // 32 bytes of K per instruction
            const unsigned long long ad = smem_desc_sw128(sa) + (unsigned long long)(2 * k);
            const unsigned long long bd = smem_desc_sw128(sb) + (unsigned long long)(2 * k);
            if constexpr (BF)
              mma_bf16(d, ad, bd, idesc, (t > 0 || k > 0) ? 1 : 0);
            else
              mma_tf32(d, ad, bd, idesc, (t > 0 || k > 0) ? 1 : 0);
            if constexpr (SPLIT) {
              const unsigned long long ald =
                  smem_desc_sw128(base + Cfg::OFF_AL + s * Cfg::A_BYTES) + (unsigned long long)(2 * k);
              const unsigned long long bld =
                  smem_desc_sw128(base + Cfg::OFF_BL + s * Cfg::B_BYTES) + (unsigned long long)(2 * k);
              mma_tf32(d, ad, bld, idesc, 1);
              mma_tf32(d, ald, bd, idesc, 1);
            }
          }
          mma_commit(&empty[s]);
        }
        if (!ok) break;
        mma_commit(&tfull[buf]);
      }
      // every MMA issued has completed before tensor memory is freed
      mma_commit(done);
      if (!mbar_wait(done, 0)) atomicExch(abort_flag, 1);
    }
  } else {
    // ---------------- epilogue (warps 2..5) ----------------
    const int ew = warp - 2, q = warp & 3;
    unsigned char* cst = base + Cfg::OFF_C + ew * CB * kPEpiChunk;
    unsigned long long* cb = cbar + CB * ew;
    constexpr int kChunks = BN / 32;
    static_assert(CB <= kChunks + 1, "prefetch reaches past the next tile");
    const bool load_c = beta != 0.0f;
    unsigned cphase[CB];   // next phase to wait for, per staging buffer
    bool pending[CB];      // lane 0: a load into the buffer is in flight
#pragma unroll
    for (int b2 = 0; b2 < CB; ++b2) { cphase[b2] = 0u; pending[b2] = false; }
    // chunk d places after (tile, c): at most one tile further
    auto chunk_at = [&](int tile, int c, int d, int& x, int& y) -> bool {
      c += d;
      if (c >= kChunks) { c -= kChunks; tile += gridDim.x; }
      if (tile >= tiles) return false;
      int mb, nb;
      coords(tile, mb, nb);
      x = nb * BN + 32 * c;
      y = mb * kTcM + 32 * q;
      return x < N && y < M;   // chunks wholly outside C are skipped
    };
    // The warp's chunks (tile, c) are numbered g = 0, 1, ...; chunk g uses
    // staging buffer g % CB, and chunk g + CB - 1's old C is requested before
    // chunk g is processed.
    if (load_c && blockIdx.x < tiles && lane == 0) {
      for (int d = 0; d < CB - 1; ++d) {
        int x, y;
        if (chunk_at(blockIdx.x, 0, d, x, y)) {
          mbar_expect_tx(&cb[d], kPEpiChunk);
          tma_load_2d(cst + d * kPEpiChunk, &map_c, x, y, &cb[d]);
          pending[d] = true;
        }
      }
    }
    bool ok = true;
    int g = 0, tc = 0, last_store_buf = -1;
    for (int tile = blockIdx.x; tile < tiles; tile += gridDim.x, ++tc) {
      const int buf = tc & 1, use = tc >> 1;
      ok = __all_sync(0xffffffffu, mbar_wait(&tfull[buf], use & 1));
      if (!ok) break;
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      for (int c = 0; c < kChunks; ++c, ++g) {
        const int sbuf = g % CB;
        unsigned char* cur = cst + sbuf * kPEpiChunk;
        int cx = 0, cy = 0;
        const bool live = chunk_at(tile, c, 0, cx, cy);
        if (load_c && lane == 0) {
          const int nbuf = (g + CB - 1) % CB;   // last used by chunk g - 1
          int x, y;
          if (chunk_at(tile, c, CB - 1, x, y)) {
            // every store issued so far has finished reading its buffer
            asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
            mbar_expect_tx(&cb[nbuf], kPEpiChunk);
            tma_load_2d(cst + nbuf * kPEpiChunk, &map_c, x, y, &cb[nbuf]);
            pending[nbuf] = true;
          }
        }
        if (!live) continue;
        if (load_c) {
          ok = __all_sync(0xffffffffu, mbar_wait(&cb[sbuf], cphase[sbuf]));
          if (ok) { cphase[sbuf] ^= 1u; pending[sbuf] = false; }
        } else if (lane == 0) {
          // the last store from this buffer has finished reading it: it is the
          // newest bulk group or an older one
          if (last_store_buf == sbuf)
            asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
          else
            asm volatile("cp.async.bulk.wait_group.read 1;" ::: "memory");
        }
        __syncwarp();
        float v[32];
        tmem_ld32(tmem + ((unsigned)(32 * q) << 16) + (unsigned)(buf * BN + 32 * c), v);
        if (!ok) break;
        char* rowp = reinterpret_cast<char*>(cur) + lane * 128;
#pragma unroll
        for (int gq = 0; gq < 8; ++gq) {
          float4* p4 = reinterpret_cast<float4*>(rowp + ((gq ^ (lane & 7)) << 4));
          float4 o = load_c ? *p4 : make_float4(0.f, 0.f, 0.f, 0.f);
          o.x = fmaf(alpha, v[4 * gq + 0], load_c ? beta * o.x : 0.0f);
          o.y = fmaf(alpha, v[4 * gq + 1], load_c ? beta * o.y : 0.0f);
          o.z = fmaf(alpha, v[4 * gq + 2], load_c ? beta * o.z : 0.0f);
          o.w = fmaf(alpha, v[4 * gq + 3], load_c ? beta * o.w : 0.0f);
          *p4 = o;
        }
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncwarp();
        if (lane == 0) {
          tma_store_2d(&map_c, cx, cy, cur);
          asm volatile("cp.async.bulk.commit_group;" ::: "memory");
          last_store_buf = sbuf;
        }
      }
      if (!ok) break;
      // this warp's reads of accumulator buf are complete (tcgen05.ld waited)
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      __syncwarp();
      if (lane == 0)
        asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(&tempty[buf]))
                     : "memory");
      if (__any_sync(0xffffffffu, *vabort != 0)) break;
    }
    if (!ok) atomicExch(abort_flag, 1);
    if (lane == 0) {
      asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");
      // a requested chunk that was never consumed lands before shared memory is released
#pragma unroll
      for (int b2 = 0; b2 < CB; ++b2)
        if (pending[b2]) mbar_wait(&cb[b2], cphase[b2]);
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (*vabort && threadIdx.x == 0) atomicExch(err, 1);
  if (warp == 1) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                 "r"(Cfg::TMEM_COLS)
                 : "memory");
  }
}

// cuTensorMapEncodeTiled through the runtime's driver entry point (no libcuda link).
static PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  if (!fn) {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                         &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  }
  return fn;
}

// 2-D map over rows×cols (row stride ld elements) with 128-byte rows per box:
// FP32 (box 32 × box_rows) or BF16 (box 64 × box_rows).
static int make_map(CUtensorMap* map, const void* base, int64_t rows, int64_t cols, int64_t ld,
                    bool bf16 = false, unsigned box_rows = 128) {
  auto fn = encode_fn();
  if (!fn) {
    set_last_error("gemm_tf32: cuTensorMapEncodeTiled unavailable");
    return LXGB_CUDA_ERROR;
  }
  cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
  cuuint64_t strides[1] = {(cuuint64_t)(ld * (bf16 ? 2 : 4))};
  cuuint32_t box[2] = {(cuuint32_t)(bf16 ? 2 * kTcK : kTcK), (cuuint32_t)box_rows};
  cuuint32_t estr[2] = {1u, 1u};
  CUresult r = fn(map, bf16 ? CU_TENSOR_MAP_DATA_TYPE_BFLOAT16 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32,
                  2, const_cast<void*>(base), dims, strides,
                  box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                  CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) {
    set_last_error("gemm_tf32: cuTensorMapEncodeTiled failed (%d)", (int)r);
    return LXGB_INVALID_ARG;
  }
  return LXGB_SUCCESSFUL;
}

__global__ void scale_c_kernel(int M, int N, float* C, int64_t ldc, float beta) {
  const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (e >= (int64_t)M * N) return;
  float* p = C + (e / N) * ldc + (e % N);
  *p = (beta == 0.0f) ? 0.0f : beta * *p;
}

// 1 (default): C = alpha A Bᵀ + beta C runs on the persistent kernel when C
// can be addressed by a tensor map; 0: one CTA per 128×128 tile.
static int g_gemm_persistent = 1;

// Persistent launch; returns -1 when C cannot be addressed by a tensor map
// (the caller then uses the one-tile-per-CTA kernel).
template <int MODE, class Cfg>
static int gemm_persistent_cfg(int M, int N, int K, const void* A, const void* Al, int64_t lda,
                               const void* B, const void* Bl, int64_t ldb, float* C, int64_t ldc,
                               float alpha, float beta, int* err, cudaStream_t st,
                               int lower = 0) {
  constexpr bool BF = MODE == 2;
  if (!g_gemm_persistent) return -1;
  if ((((uintptr_t)C) & 15) != 0 || (ldc % 4) != 0) return -1;
  CUtensorMap ma, mb, mal, mbl, mc;
  if (make_map(&mc, C, M, N, ldc, false, 32) != 0) {
    cudaGetLastError();
    return -1;
  }
  int rc = make_map(&ma, A, M, K, lda, BF, kTcM);
  if (rc) return rc;
  rc = make_map(&mb, B, N, K, ldb, BF, Cfg::BN);
  if (rc) return rc;
  mal = ma;
  mbl = mb;
  if (Cfg::SPLIT) {
    rc = make_map(&mal, Al, M, K, lda, false, kTcM);
    if (rc) return rc;
    rc = make_map(&mbl, Bl, N, K, ldb, false, Cfg::BN);
    if (rc) return rc;
  }
  const int64_t tiles = (int64_t)((M + kTcM - 1) / kTcM) * ((N + Cfg::BN - 1) / Cfg::BN);
  const int grid = (int)(tiles < sm_count() ? tiles : sm_count());
  auto kern = gemm_nt_persistent_kernel<MODE, Cfg>;
  LXGB_CUDA_TRY(ensure_dynamic_smem(reinterpret_cast<const void*>(kern), Cfg::SMEM),
                "gemm persistent: set smem");
  kern<<<grid, kPThreads, Cfg::SMEM, st>>>(ma, mb, mal, mbl, mc, M, N, K, alpha, beta, err,
                                           lower);
  return check_launch("gemm persistent");
}

// K of at most two stages (beta != 0): the short-K configuration.
template <int MODE>
static int gemm_persistent(int M, int N, int K, const void* A, const void* Al, int64_t lda,
                           const void* B, const void* Bl, int64_t ldb, float* C, int64_t ldc,
                           float alpha, float beta, int* err, cudaStream_t st) {
  const int kstage = MODE == 2 ? 2 * kTcK : kTcK;
  const bool short_k = beta != 0.0f && K <= 2 * kstage;
  if constexpr (MODE == 0) {
    if (short_k)
      return gemm_persistent_cfg<0, PCfgTf32ShortK>(M, N, K, A, Al, lda, B, Bl, ldb, C, ldc,
                                                    alpha, beta, err, st);
    return gemm_persistent_cfg<0, PCfgTf32>(M, N, K, A, Al, lda, B, Bl, ldb, C, ldc, alpha, beta,
                                            err, st);
  } else if constexpr (MODE == 2) {
    if (short_k)
      return gemm_persistent_cfg<2, PCfgBf16ShortK>(M, N, K, A, Al, lda, B, Bl, ldb, C, ldc,
                                                    alpha, beta, err, st);
    return gemm_persistent_cfg<2, PCfgBf16>(M, N, K, A, Al, lda, B, Bl, ldb, C, ldc, alpha, beta,
                                            err, st);
  } else {
    return gemm_persistent_cfg<1, PCfgSplit>(M, N, K, A, Al, lda, B, Bl, ldb, C, ldc, alpha, beta,
                                             err, st);
  }
}

int gemm_tf32_nt_split(int M, int N, int K, const float* A, const float* Al, int64_t lda,
                       const float* B, const float* Bl, int64_t ldb, float* C, int64_t ldc,
                       float alpha, float beta, int* err, cudaStream_t st) {
  if (M <= 0 || N <= 0) return LXGB_SUCCESSFUL;
  if (K == 0) {  // C = beta * C
    const int64_t total = (int64_t)M * N;
    scale_c_kernel<<<(unsigned)((total + 255) / 256), 256, 0, st>>>(M, N, C, ldc, beta);
    return check_launch("gemm_tf32 (k = 0)");
  }
  const bool split = (Al != nullptr) && (Bl != nullptr);
  {
    const int prc = split ? gemm_persistent<1>(M, N, K, A, Al, lda, B, Bl, ldb, C, ldc, alpha,
                                               beta, err, st)
                          : gemm_persistent<0>(M, N, K, A, nullptr, lda, B, nullptr, ldb, C, ldc,
                                               alpha, beta, err, st);
    if (prc >= 0) return prc;
  }
  CUtensorMap ma, mb, mal, mbl;
  int rc = make_map(&ma, A, M, K, lda);
  if (rc) return rc;
  rc = make_map(&mb, B, N, K, ldb);
  if (rc) return rc;
  mal = ma;
  mbl = mb;
  if (split) {
    rc = make_map(&mal, Al, M, K, lda);
    if (rc) return rc;
    rc = make_map(&mbl, Bl, N, K, ldb);
    if (rc) return rc;
  }
  // TMA epilogue when C meets the tensor-map rules (16-byte base and row stride)
  CUtensorMap mc = ma;
  int use_tma_c = 0;
  if ((((uintptr_t)C) & 15) == 0 && (ldc % 4) == 0 && make_map(&mc, C, M, N, ldc) == 0)
    use_tma_c = 1;
  else
    cudaGetLastError();
  dim3 grid((unsigned)((N + kTcN - 1) / kTcN), (unsigned)((M + kTcM - 1) / kTcM));
  if (split) {
    const size_t smem = sizeof(TcSmem<kTcStagesSplit, true>) + 1024;
    LXGB_CUDA_TRY(ensure_dynamic_smem(reinterpret_cast<const void*>(gemm_tf32_nt_kernel<1>), (int)smem),
                  "gemm_tf32: set smem");
    gemm_tf32_nt_kernel<1><<<grid, kTcThreads, smem, st>>>(ma, mb, mal, mbl, mc, use_tma_c, M,
                                                          N, K, C, ldc, alpha, beta, err, 0, 0);
  } else {
    const size_t smem = sizeof(TcSmem<kTcStages, false>) + 1024;
    LXGB_CUDA_TRY(ensure_dynamic_smem(reinterpret_cast<const void*>(gemm_tf32_nt_kernel<0>), (int)smem),
                  "gemm_tf32: set smem");
    gemm_tf32_nt_kernel<0><<<grid, kTcThreads, smem, st>>>(ma, mb, mal, mbl, mc, use_tma_c, M,
                                                          N, K, C, ldc, alpha, beta, err, 0, 0);
  }
  return check_launch("gemm_tf32");
}

// C = alpha A Aᵀ + beta C on the tiles that hold C's lower triangle (C is
// M×M and symmetric, A M×K; 3xTF32 when Al is given).  Tiles on the diagonal
// are computed whole, so C's upper triangle is left partly updated.  Falls
// back to the full product when the persistent kernel is off or C cannot be
// addressed by a tensor map.
int gemm_tf32_nt_split_lower(int M, int K, const float* A, const float* Al, int64_t lda, float* C,
                             int64_t ldc, float alpha, float beta, int* err, cudaStream_t st) {
  if (M <= 0) return LXGB_SUCCESSFUL;
  if (K > 0) {
    int prc;
    if (Al != nullptr)
      prc = gemm_persistent_cfg<1, PCfgSplit>(M, M, K, A, Al, lda, A, Al, lda, C, ldc, alpha,
                                              beta, err, st, 1);
    else if (beta != 0.0f && K <= 2 * kTcK)
      prc = gemm_persistent_cfg<0, PCfgTf32ShortK>(M, M, K, A, nullptr, lda, A, nullptr, lda, C,
                                                   ldc, alpha, beta, err, st, 1);
    else
      prc = gemm_persistent_cfg<0, PCfgTf32>(M, M, K, A, nullptr, lda, A, nullptr, lda, C, ldc,
                                             alpha, beta, err, st, 1);
    if (prc >= 0) return prc;
  }
  return gemm_tf32_nt_split(M, M, K, A, Al, lda, A, Al, lda, C, ldc, alpha, beta, err, st);
}

int gemm_tf32_nt(int M, int N, int K, const float* A, int64_t lda, const float* B, int64_t ldb,
                 float* C, int64_t ldc, float alpha, float beta, int* err, cudaStream_t st) {
  return gemm_tf32_nt_split(M, N, K, A, nullptr, lda, B, nullptr, ldb, C, ldc, alpha, beta, err,
                            st);
}

// Split-K: C_s = A[:, K_s] B[:, K_s]ᵀ for s < splits, K_s the s-th range of
// chunk elements (chunk a multiple of 32), C_s at C + s * M * ldc — one launch
// (blockIdx.z = s) instead of one per range.  Pointer epilogue (rows past M
// are not written).
int gemm_tf32_nt_splitk(int M, int N, int K, const float* A, int64_t lda, const float* B,
                        int64_t ldb, float* C, int64_t ldc, int chunk, int splits, int* err,
                        cudaStream_t st) {
  if (M <= 0 || N <= 0 || splits <= 0) return LXGB_SUCCESSFUL;
  if ((chunk % kTcK) != 0 || chunk <= 0) return invalid("gemm_tf32 split-K: chunk not a multiple of 32");
  CUtensorMap ma, mb;
  int rc = make_map(&ma, A, M, K, lda);
  if (rc) return rc;
  rc = make_map(&mb, B, N, K, ldb);
  if (rc) return rc;
  dim3 grid((unsigned)((N + kTcN - 1) / kTcN), (unsigned)((M + kTcM - 1) / kTcM), (unsigned)splits);
  const size_t smem = sizeof(TcSmem<kTcStages, false>) + 1024;
  LXGB_CUDA_TRY(ensure_dynamic_smem(reinterpret_cast<const void*>(gemm_tf32_nt_kernel<0>), (int)smem),
                "gemm_tf32: set smem");
  gemm_tf32_nt_kernel<0><<<grid, kTcThreads, smem, st>>>(ma, mb, ma, mb, ma, 0, M, N, K, C, ldc,
                                                        1.0f, 0.0f, err, chunk / kTcK,
                                                        (int64_t)M * ldc);
  return check_launch("gemm_tf32 split-K");
}

// C = alpha A Bᵀ + beta C with BF16 operands (A m×k, B n×k, K-major, row
// strides multiples of 8 elements, 16-byte aligned), FP32 C.
int gemm_bf16_nt(int M, int N, int K, const void* A, int64_t lda, const void* B, int64_t ldb,
                 float* C, int64_t ldc, float alpha, float beta, int* err, cudaStream_t st) {
  if (M <= 0 || N <= 0) return LXGB_SUCCESSFUL;
  if (K == 0) {
    const int64_t total = (int64_t)M * N;
    scale_c_kernel<<<(unsigned)((total + 255) / 256), 256, 0, st>>>(M, N, C, ldc, beta);
    return check_launch("gemm_bf16 (k = 0)");
  }
  {
    const int prc = gemm_persistent<2>(M, N, K, A, nullptr, lda, B, nullptr, ldb, C, ldc, alpha,
                                       beta, err, st);
    if (prc >= 0) return prc;
  }
  CUtensorMap ma, mb;
  int rc = make_map(&ma, A, M, K, lda, true);
  if (rc) return rc;
  rc = make_map(&mb, B, N, K, ldb, true);
  if (rc) return rc;
  CUtensorMap mc = ma;
  int use_tma_c = 0;
  if ((((uintptr_t)C) & 15) == 0 && (ldc % 4) == 0 && make_map(&mc, C, M, N, ldc) == 0)
    use_tma_c = 1;
  else
    cudaGetLastError();
  dim3 grid((unsigned)((N + kTcN - 1) / kTcN), (unsigned)((M + kTcM - 1) / kTcM));
  const size_t smem = sizeof(TcSmem<kTcStages, false>) + 1024;
  LXGB_CUDA_TRY(ensure_dynamic_smem(reinterpret_cast<const void*>(gemm_tf32_nt_kernel<2>), (int)smem),
                "gemm_bf16: set smem");
  gemm_tf32_nt_kernel<2><<<grid, kTcThreads, smem, st>>>(ma, mb, ma, mb, mc, use_tma_c, M, N, K,
                                                        C, ldc, alpha, beta, err, 0, 0);
  return check_launch("gemm_bf16");
}

// dst (rows × cols, row stride ldd) = src rounded to BF16 (nearest even).
__global__ void bf16_convert_kernel(int64_t rows, int64_t cols, const float* __restrict__ src,
                                    int64_t lds, __nv_bfloat16* __restrict__ dst, int64_t ldd) {
  const int64_t total = rows * cols;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = e / cols, c = e % cols;
    dst[r * ldd + c] = __float2bfloat16_rn(src[r * lds + c]);
  }
}

int bf16_convert(int64_t rows, int64_t cols, const float* src, int64_t lds, void* dst, int64_t ldd,
                 cudaStream_t st) {
  const int64_t total = rows * cols;
  if (total <= 0) return LXGB_SUCCESSFUL;
  const int64_t blocks = (total + 255) / 256 < 4096 ? (total + 255) / 256 : 4096;
  bf16_convert_kernel<<<(unsigned)blocks, 256, 0, st>>>(rows, cols, src, lds,
                                                        reinterpret_cast<__nv_bfloat16*>(dst), ldd);
  return check_launch("bf16_convert");
}

// hi = x with the low 13 mantissa bits cleared (TF32-exact), lo = x - hi
// (exact in FP32): the operand split of 3xTF32.
__global__ void tf32_split_kernel(int64_t rows, int64_t cols, const float* __restrict__ src,
                                  int64_t lds, float* __restrict__ hi, float* __restrict__ lo,
                                  int64_t ldd) {
  const int64_t total = rows * cols;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = e / cols, c = e % cols;
    const float x = src[r * lds + c];
    const float h = __uint_as_float(__float_as_uint(x) & 0xFFFFE000u);
    hi[r * ldd + c] = h;
    lo[r * ldd + c] = x - h;
  }
}

int tf32_split(int64_t rows, int64_t cols, const float* src, int64_t lds, float* hi, float* lo,
               int64_t ldd, cudaStream_t st) {
  const int64_t total = rows * cols;
  if (total <= 0) return LXGB_SUCCESSFUL;
  const int64_t blocks = (total + 255) / 256 < 4096 ? (total + 255) / 256 : 4096;
  tf32_split_kernel<<<(unsigned)blocks, 256, 0, st>>>(rows, cols, src, lds, hi, lo, ldd);
  return check_launch("tf32_split");
}

}  // namespace lxgb

using namespace lxgb;

extern "C" int lxgb_gemm_3xtf32_nt(int32_t m, int32_t n, int32_t k, const float* a,
                                   const float* a_lo, int64_t lda, const float* b,
                                   const float* b_lo, int64_t ldb, float* c, int64_t ldc,
                                   float alpha, float beta, int32_t* err, void* stream);

extern "C" int lxgb_gemm_tf32_nt(int32_t m, int32_t n, int32_t k, const float* a, int64_t lda,
                                 const float* b, int64_t ldb, float* c, int64_t ldc, float alpha,
                                 float beta, int32_t* err, void* stream) {
  return lxgb_gemm_3xtf32_nt(m, n, k, a, nullptr, lda, b, nullptr, ldb, c, ldc, alpha, beta, err,
                             stream);
}

extern "C" int lxgb_gemm_3xtf32_nt(int32_t m, int32_t n, int32_t k, const float* a,
                                   const float* a_lo, int64_t lda, const float* b,
                                   const float* b_lo, int64_t ldb, float* c, int64_t ldc,
                                   float alpha, float beta, int32_t* err, void* stream) {
  LXGB_REQUIRE(m >= 0 && n >= 0 && k >= 0, "gemm_tf32: negative size");
  if (m == 0 || n == 0) return LXGB_SUCCESSFUL;
  LXGB_REQUIRE(c && err && (k == 0 || (a && b)), "gemm_tf32: null pointer");
  LXGB_REQUIRE(ldc >= n, "gemm_tf32: ldc < n");
  if (k > 0) {
    LXGB_REQUIRE(lda >= k && ldb >= k, "gemm_tf32: leading dimension too small");
    LXGB_REQUIRE((lda % 4) == 0 && (ldb % 4) == 0, "gemm_tf32: lda and ldb must be multiples of 4");
    LXGB_REQUIRE((((uintptr_t)a) & 15) == 0 && (((uintptr_t)b) & 15) == 0,
                 "gemm_tf32: A and B must be 16-byte aligned");
  }
  LXGB_REQUIRE((a_lo == nullptr) == (b_lo == nullptr), "gemm_3xtf32: give both lo parts or none");
  LXGB_REQUIRE((((uintptr_t)a_lo) & 15) == 0 && (((uintptr_t)b_lo) & 15) == 0,
               "gemm_3xtf32: lo parts must be 16-byte aligned");
  return gemm_tf32_nt_split(m, n, k, a, a_lo, lda, b, b_lo, ldb, c, ldc, alpha, beta, err,
                            as_stream(stream));
}

extern "C" int lxgb_gemm_bf16_nt(int32_t m, int32_t n, int32_t k, const void* a, int64_t lda,
                                 const void* b, int64_t ldb, float* c, int64_t ldc, float alpha,
                                 float beta, int32_t* err, void* stream) {
  LXGB_REQUIRE(m >= 0 && n >= 0 && k >= 0, "gemm_bf16: negative size");
  if (m == 0 || n == 0) return LXGB_SUCCESSFUL;
  LXGB_REQUIRE(c && err && (k == 0 || (a && b)), "gemm_bf16: null pointer");
  LXGB_REQUIRE(ldc >= n, "gemm_bf16: ldc < n");
  if (k > 0) {
    LXGB_REQUIRE(lda >= k && ldb >= k, "gemm_bf16: leading dimension too small");
    LXGB_REQUIRE((lda % 8) == 0 && (ldb % 8) == 0, "gemm_bf16: lda and ldb must be multiples of 8");
    LXGB_REQUIRE((((uintptr_t)a) & 15) == 0 && (((uintptr_t)b) & 15) == 0,
                 "gemm_bf16: A and B must be 16-byte aligned");
  }
  return gemm_bf16_nt(m, n, k, a, lda, b, ldb, c, ldc, alpha, beta, err, as_stream(stream));
}

extern "C" int lxgb_gemm_set_persistent(int32_t on) {
  g_gemm_persistent = on ? 1 : 0;
  return LXGB_SUCCESSFUL;
}
