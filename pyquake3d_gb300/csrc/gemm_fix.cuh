// Tensor-core (tcgen05) operator product of the batched stepper with exact
// fixed-point slices ("BF16x14").  See gemm_fix.cu.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace pq3d {
namespace fx {

constexpr int kTileM = 128;        // operator rows per CTA (one tcgen05 M=128 tile)
constexpr int kBlockK = 32;        // operator columns per pipeline stage
constexpr int kKPieces = 4;        // operator slices (32 bits per row and chunk)
constexpr int kVPieces = 5;        // right-hand-side slices (40 bits per run and chunk)
constexpr int kChunk = 1024;       // columns that share one exponent (per operator row / per run)
constexpr int kBlocksPerChunk = kChunk / kBlockK;
constexpr int kAcc = 7;            // tensor-memory accumulators per run
constexpr int kMaxRuns = 64;       // 7 accumulators x 64 runs fill the 512 tensor-memory columns

__host__ __device__ inline int64_t m_tiles(int64_t N) { return (3 * N + kTileM - 1) / kTileM; }
__host__ __device__ inline int64_t k_blocks(int64_t N) { return (2 * N + kBlockK - 1) / kBlockK; }
__host__ __device__ inline int64_t k_chunks(int64_t N) { return (2 * N + kChunk - 1) / kChunk; }

// [m_tiles][k_blocks][4 slices][128 x 32 BF16 image]
inline size_t packed_operator_bytes(int64_t N)
{
    return (size_t)m_tiles(N) * (size_t)k_blocks(N) * kKPieces * kTileM * kBlockK * 2;
}
// [k_blocks][5 slices][Bp x 32 BF16 image]
inline size_t packed_rhs_bytes(int64_t N, int Bp) { return (size_t)k_blocks(N) * kVPieces * Bp * kBlockK * 2; }

// out[(s * Bp + n) * 3N + m] = float2 (hi, lo): K slice s of sum_k K[m][k] V[n][k]
// to ~2^-44 relative (hi + lo), from the packed fixed-point operator and
// right-hand side.  Returns a PQ3D status.
int gemm_bf16x14(const void *Kpacked, const void *Vpacked, int64_t N, int Bp, int nsplit, float2 *out,
                 void *workspace, size_t workspace_bytes, cudaStream_t stream);

// Fixed-point slices of v'_r (r < B; runs B..Bp-1 and the padding columns are
// zero) from the FP64 slip rates of the batched stepper: v'_r[2j + s] =
// slipv_s[r][j] - Vpl * (cos, sin)(rake0)[r][j], cell j = order[p] at column
// position 2p + s (order null: j = p).
int pack_rhs_from_state(const double *slipv1, const double *slipv2, const double *cos_rake0,
                        const double *sin_rake0, double Vpl, const int64_t *order, int64_t N, int B, void *Vpacked,
                        cudaStream_t stream);

}  // namespace fx
}  // namespace pq3d
