// Tensor-core (tcgen05) operator product of the batched stepper with exact
// fixed-point slices ("BF16x18").  See gemm_fix.cu.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace pq3d {
namespace fx {

constexpr int kTileM = 128;        // operator rows per CTA (one tcgen05 M=128 tile)
constexpr int kBlockK = 32;        // operator columns per pipeline stage
constexpr int kKPieces = 4;        // operator slices (32 bits per row and operator chunk)
constexpr int kVPieces = 6;        // right-hand-side slices (48 bits per run and span)
constexpr int kChunk = 1024;       // operator columns that share one exponent per row
constexpr int kBlocksPerChunk = kChunk / kBlockK;
constexpr int kSpan = 256;         // columns of one exact accumulation (one v' exponent per run)
constexpr int kBlocksPerSpan = kSpan / kBlockK;
constexpr int kLevels = 6;         // tensor-memory slots: one per level p + q = 0..5
constexpr int kMaxRuns = 64;

__host__ __device__ inline int64_t m_tiles(int64_t N) { return (3 * N + kTileM - 1) / kTileM; }
__host__ __device__ inline int64_t k_blocks(int64_t N) { return (2 * N + kBlockK - 1) / kBlockK; }
__host__ __device__ inline int64_t k_chunks(int64_t N) { return (2 * N + kChunk - 1) / kChunk; }
__host__ __device__ inline int64_t k_spans(int64_t N) { return (2 * N + kSpan - 1) / kSpan; }
// runs of the product: B rounded up to 32 (the slots of one level are Bq
// tensor-memory columns apart, 32-column aligned)
__host__ __device__ inline int fix_runs(int B) { return (B + 31) / 32 * 32; }

// [m_tiles][k_blocks][4 slices][128 x 32 BF16 image]
inline size_t packed_operator_bytes(int64_t N)
{
    return (size_t)m_tiles(N) * (size_t)k_blocks(N) * kKPieces * kTileM * kBlockK * 2;
}
// [k_blocks][6 slices][Bq x 32 BF16 image], Bq = fix_runs(B)
inline size_t packed_rhs_bytes(int64_t N, int B) { return (size_t)k_blocks(N) * kVPieces * fix_runs(B) * kBlockK * 2; }

// out[(s * Bo + n) * 3N + m] = float2 (hi, lo) for n < Bo = B rounded up to 16:
// K slice s of sum_k K[m][k] V[n][k] to ~2^-44 relative (hi + lo), from the
// packed fixed-point operator and right-hand side.  Returns a PQ3D status.
int gemm_bf16x18(const void *Kpacked, const void *Vpacked, int64_t N, int B, int nsplit, float2 *out,
                 void *workspace, size_t workspace_bytes, cudaStream_t stream);

// Fixed-point slices of v'_r (r < B; the padding runs and columns are zero)
// from the FP64 slip rates of the batched stepper: v'_r[2j + s] =
// slipv_s[r][j] - Vpl * (cos, sin)(rake0)[r][j], cell j = order[p] at column
// position 2p + s (order null: j = p).
int pack_rhs_from_state(const double *slipv1, const double *slipv2, const double *cos_rake0,
                        const double *sin_rake0, double Vpl, const int64_t *order, int64_t N, int B, void *Vpacked,
                        cudaStream_t stream);

}  // namespace fx
}  // namespace pq3d
