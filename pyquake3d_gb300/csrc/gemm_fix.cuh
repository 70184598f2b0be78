// Tensor-core (tcgen05) operator product of the batched stepper with exact
// fixed-point slices ("BF16x18").  See gemm_fix.cu.
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "gemm_tc.cuh"

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

#ifdef __CUDACC__
// balanced base-256 digits of an integer |X| <= 2^(8 n - 1): X = sum d_p 2^(8 (n-1-p)),
// |d_p| <= 128, the most significant first
template <int n>
__device__ __forceinline__ void digits(long long X, int d[n])
{
#pragma unroll
    for (int p = n - 1; p >= 1; --p) {
        const int t = (int)((X + 128) & 255) - 128;
        d[p] = t;
        X = (X - t) >> 8;
    }
    d[0] = (int)X;
}

// exponent e with |x| < 2^e for the largest magnitude m of a chunk (0 for m = 0)
__device__ __forceinline__ int chunk_exponent(double m) { return m > 0.0 ? ilogb(m) + 1 : 0; }

// A right-hand-side span's exponent from its cells' values by integer
// operations: the high word of |v| (sign cleared) orders the exponents, the
// span takes the largest word over its cells (rhs_word, then a 32-bit max),
// and e = exponent + 1 with |v| < 2^e for every cell; a span whose largest
// exponent field is 0 (all zero, or subnormal: below FP32's range, its slices
// are zero either way) gets e = 0.
__device__ __forceinline__ int rhs_word(double a, double b)
{
    return max(__double2hiint(a) & 0x7fffffff, __double2hiint(b) & 0x7fffffff);
}
__device__ __forceinline__ int rhs_span_exponent(int word)
{
    const int f = word >> 20;
    return f ? f - 1022 : 0;
}

// The six right-hand-side slices of one cell, (v'_1, v'_2) of run r at column
// positions 2p and 2p + 1, e the exponent of its span (rhs_span_exponent): the
// one writer of the packed right-hand side (the pack kernel and the batched
// stepper's update both call it).  Positions past the last 32-column block
// (KB blocks) write nothing.  The scaling by 2^(47 - e) is one product with a
// power of two built from its bits; a span below 2^-976 (its slices would be
// below FP32's range) is written as zeros.
__device__ __forceinline__ void write_rhs_cell(__nv_bfloat16 *out, int Bq, int64_t KB, int64_t p, int r, int e,
                                               double v1, double v2)
{
    const int64_t kb = p / (kBlockK / 2);
    if (kb >= KB) return;
    int d1[kVPieces] = {}, d2[kVPieces] = {};
    if (e >= -976) {
        const double sc = __hiloint2double((8 * kVPieces - 1 - e + 1023) << 20, 0);   // 2^(47 - e)
        digits<kVPieces>(__double2ll_rn(v1 * sc), d1);
        digits<kVPieces>(__double2ll_rn(v2 * sc), d2);
    }
    const int64_t img = (int64_t)Bq * kBlockK;
    __nv_bfloat16 *P = out + kb * kVPieces * img + tc::image_offset(r, (int)((2 * p) % kBlockK));
#pragma unroll
    for (int q = 0; q < kVPieces; ++q) {
        __nv_bfloat162 w;
        w.x = __float2bfloat16_rn(ldexpf((float)d1[q], e - 7 - 8 * q));
        w.y = __float2bfloat16_rn(ldexpf((float)d2[q], e - 7 - 8 * q));
        reinterpret_cast<__nv_bfloat162 *>(P + q * img)[0] = w;
    }
}
#endif

// out[(s * Bo + n) * 3N + m] = float2 (hi, lo) for n < Bo = B rounded up to 16:
// nsplit partial sums of sum_k K[m][k] V[n][k] (K slices, or the balanced
// grid's tile shares; see gemm_fix.cu) to ~2^-44 relative (hi + lo), from the
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
