// Tensor-core (tcgen05) operator product of the batched stepper, BF16 split
// products.  See gemm_tc.cu.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace pq3d {
namespace tc {

constexpr int kTileM = 128;   // operator rows per CTA (one tcgen05 M=128 tile)
constexpr int kBlockK = 32;   // operator columns per pipeline stage
constexpr int kPieces = 3;    // BF16 pieces per operand

// Blocks of the packed operator / right-hand side.
inline int64_t m_tiles(int64_t N) { return (3 * N + kTileM - 1) / kTileM; }
inline int64_t k_blocks(int64_t N) { return (2 * N + kBlockK - 1) / kBlockK; }

// Bytes of the packed operator: [m_tiles][k_blocks][3 pieces][128 x 32 BF16 image].
inline size_t packed_operator_bytes(int64_t N)
{
    return (size_t)m_tiles(N) * (size_t)k_blocks(N) * kPieces * kTileM * kBlockK * 2;
}
// Bytes of the packed right-hand side: [k_blocks][3 pieces][Bp x 32 BF16 image].
inline size_t packed_rhs_bytes(int64_t N, int Bp) { return (size_t)k_blocks(N) * kPieces * Bp * kBlockK * 2; }

// Element offset of (row, col) inside one rows x 32 BF16 core-matrix image:
// 8-row x 8-column core matrices of 128 bytes, column groups 128 B apart,
// 8-row groups 512 B apart (K-major, no swizzle).
__host__ __device__ inline int image_offset(int row, int col)
{
    return (row >> 3) * 256 + (col >> 3) * 64 + (row & 7) * 8 + (col & 7);
}

size_t gemm_bf16x6_workspace_bytes(int64_t N, int Bp, int nsplit);

// out[(s * Bp + n) * 3N + m] = sum over the columns k of slice s of K[m][k] * V[n][k],
// from the packed operator and right-hand side; FP32 accumulation in tensor
// memory, FP32 output (the accumulator); ctas_per_sm (0 = 2, else 1..3) CTAs
// resident per SM, fewer where shared or tensor memory does not fit them (the
// launch shape only: the result does not depend on it).  Returns a PQ3D status.
int gemm_bf16x6(const void *Kpacked, const void *Vpacked, int64_t N, int Bp, int nsplit, int ctas_per_sm, float *out,
                void *workspace, size_t workspace_bytes, cudaStream_t stream);
// CTAs per SM and pipeline stages that gemm_bf16x6 launches with.
int plan_bf16x6(int Bp, int ctas_per_sm, int *ctas, int *stages);

}  // namespace tc
}  // namespace pq3d
