// Batched traction product on the 5th-generation tensor cores (tcgen05) with
// exact fixed-point slices ("BF16x14"):
//
//   out[s][n][m] = sum_{k in slice s} K[m][k] * V[n][k]   (hi + lo, ~2^-44 relative)
//   K: (3N) x (2N) traction operator, V: B slip-rate deficits v' = V - Vpl.
//
// Why: the reference evaluates K.(V - Vpl) in FP64 (src/QDsim_gpu.py:948-957).
// A product that rounds v' or its own running sums to FP32 level (~2^-24) each
// step -- BF16x3, TF32 or the three-piece BF16x6 product -- perturbs the
// traction rate by a fresh ~1e-7 every step, and a nucleating rupture
// amplifies that past 1e-5 in slip within ~25 accepted steps.  A static
// rounding of the operator is amplified far less (the operator rounded once
// to FP32 stays within 1e-5 for ~130 steps).  So this product carries v' to 40
// bits, the operator to 32 bits, and accumulates without rounding.
//
// Representation (Ozaki-style fixed point, one exponent per chunk of 1024
// columns):
//   * operator row m, chunk c:  e = exponent of max |K[m][c*1024 ..]|, and
//     K[m][k] ~= sum_{p<4} d_p 2^(e - 7 - 8p), integer digits |d_p| <= 128
//     (balanced base 256 of round(K 2^(31-e))): 32 bits relative to the
//     chunk's largest entry.
//   * run n, chunk c: the same with 5 digits of v'_n (40 bits).
//   Each digit times its power of two is exact in BF16 (8 significant bits),
//   and the slices are stored with that scale, so the products are plain BF16
//   tensor-core products.
//   * A product of digits d_p e_q is an integer of at most 2^14 units of
//     2^(eK + eV - 14 - 8(p+q)).  Within one chunk (1024 columns) every
//     product of one level l = p + q lies on that grid, and the sum of one
//     (p, q) pair over the chunk is at most 1024 * 2^14 = 2^24 units: exact in
//     the FP32 tensor-memory accumulator.  Pairs of levels 0, 1 and 2 (6
//     pairs) therefore get one accumulator each and are exact; the pairs of
//     levels 3 and 4 (8 pairs, 2^-24 and 2^-32 of the leading term) share a
//     seventh accumulator, whose rounding is ~2^-48 of the result.  Levels
//     >= 5 are dropped (~2^-40).
//   * After each chunk the 7 accumulators are drained (tcgen05.ld) and added,
//     exactly up to the final rounding, into a float-float running sum held
//     in registers: 5 TwoSums, then one float-float addition.
//
// Data path (one CTA = one 128-row tile of K x one K slice, all runs; 1 CTA
// per SM since the 7 accumulators of 64 runs take the 512 tensor-memory
// columns):
//   * warp 0 lane 0: producer, two 1-D bulk copies per 32-column stage (the
//     four operator slice images, 32 KB, and the five right-hand-side slice
//     images), completion on the stage's mbarrier;
//   * warp 1 lane 0: 2 K-steps x 14 tcgen05.mma (M=128, N=Bp, K=16) per
//     stage, the stage freed by tcgen05.commit; at the end of a chunk a
//     commit tells the epilogue that the accumulators are complete, and before
//     the next chunk it waits until they are drained;
//   * warps 2-9: epilogue, two warps per 32-lane quarter of tensor memory
//     (the rows), each taking half of the runs.
//   Every mbarrier wait is bounded; a wait that gives up records an error word
//   in the workspace, the kernel waits (bounded) for its own tensor-core work,
//   frees its tensor memory and returns.  No cluster, no multicast.
#include <cuda_bf16.h>
#include <math.h>
#include <stdint.h>

#include "common.cuh"
#include "gemm_fix.cuh"
#include "gemm_tc.cuh"
#include "tc_ptx.cuh"

namespace pq3d {
namespace fx {

using tc::image_offset;

constexpr int kEpiWarps = 8;
constexpr int kThreads = 64 + 32 * kEpiWarps;
constexpr uint32_t kImageA = kTileM * kBlockK * 2;   // one operator slice image: 8 KB

__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e)
{
    s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

__global__ void __launch_bounds__(kThreads, 1)
gemm_fix_kernel(const uint8_t *__restrict__ Kp, const uint8_t *__restrict__ Vp, int64_t N, int Bp, int nsplit,
                float2 *__restrict__ out, int *__restrict__ err, int stages)
{
    extern __shared__ __align__(1024) uint8_t smem[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t mt = blockIdx.x;
    const int slice = blockIdx.y;
    const int64_t KB = (2 * N + kBlockK - 1) / kBlockK;
    const int64_t kb0 = KB * slice / nsplit, kb1 = KB * (slice + 1) / nsplit;
    const int nkb = (int)(kb1 - kb0);
    const int nch = nkb > 0 ? (int)((kb1 - 1) / kBlocksPerChunk - kb0 / kBlocksPerChunk + 1) : 0;
    const uint32_t a_bytes = kKPieces * kImageA;
    const uint32_t b_img = (uint32_t)Bp * kBlockK * 2;
    const uint32_t b_bytes = kVPieces * b_img;
    const uint32_t stage_bytes = a_bytes + b_bytes;
    uint8_t *bars = smem + (size_t)stages * stage_bytes;
    const uint32_t full0 = tc::smem_u32(bars), empty0 = full0 + 8 * stages;
    const uint32_t acc_full = full0 + 16 * stages, acc_empty = acc_full + 8, done = acc_full + 16;
    uint32_t *tmem_slot = (uint32_t *)(bars + 16 * stages + 24);
    const int astride = (Bp + 31) / 32 * 32;   // tensor-memory columns per accumulator
    const uint32_t ncols = tc::tmem_cols(kAcc * astride);

    if (threadIdx.x == 0) {
        for (int s = 0; s < stages; ++s) {
            tc::mbar_init(full0 + 8 * s, 1);
            tc::mbar_init(empty0 + 8 * s, 1);
        }
        tc::mbar_init(acc_full, 1);
        tc::mbar_init(acc_empty, kEpiWarps);
        tc::mbar_init(done, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(tc::smem_u32(tmem_slot)),
                     "r"(ncols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc::tc_fence_before();
    __syncthreads();
    tc::tc_fence_after();
    const uint32_t tmem = *(volatile uint32_t *)tmem_slot;

    if (warp == 0) {
        if (lane == 0) {
            // producer
            for (int it = 0; it < nkb; ++it) {
                const int st = it % stages, use = it / stages;
                if (!tc::mbar_wait(empty0 + 8 * st, (use & 1) ^ 1)) { atomicExch(err, 1); break; }
                const uint32_t sa = tc::smem_u32(smem + (size_t)st * stage_bytes);
                const int64_t kb = kb0 + it;
                tc::mbar_expect_tx(full0 + 8 * st, stage_bytes);
                tc::bulk_g2s(sa, Kp + (size_t)(mt * KB + kb) * a_bytes, a_bytes, full0 + 8 * st);
                tc::bulk_g2s(sa + a_bytes, Vp + (size_t)kb * b_bytes, b_bytes, full0 + 8 * st);
            }
        }
        __syncwarp();
    } else if (warp == 1) {
        if (lane == 0) {
            // tensor-core issuer
            const uint32_t idesc = tc::idesc_bf16(kTileM, Bp);
            int j = 0;   // local chunk
            for (int it = 0; it < nkb; ++it) {
                const int64_t kb = kb0 + it;
                const bool first = it == 0 || kb % kBlocksPerChunk == 0;
                const bool last = it == nkb - 1 || (kb + 1) % kBlocksPerChunk == 0;
                if (first && j > 0 && !tc::mbar_wait(acc_empty, (j - 1) & 1)) { atomicExch(err, 4); break; }
                const int st = it % stages, use = it / stages;
                if (!tc::mbar_wait(full0 + 8 * st, use & 1)) { atomicExch(err, 2); break; }
                tc::tc_fence_after();
                const uint32_t sa = tc::smem_u32(smem + (size_t)st * stage_bytes);
                const uint32_t sb = sa + a_bytes;
#pragma unroll
                for (int ks = 0; ks < 2; ++ks) {
                    const uint32_t acc_on = (first && ks == 0) ? 0u : 1u;
                    auto mma = [&](int p, int q, int acc, uint32_t accumulate) {
                        const uint64_t ad = tc::smem_desc(sa + p * kImageA + ks * 256, 128, 512);
                        const uint64_t bd = tc::smem_desc(sb + q * b_img + ks * 256, 128, 512);
                        tc::mma_bf16(tmem + (uint32_t)(acc * astride), ad, bd, idesc, accumulate);
                    };
                    // levels 0-2: one exact accumulator per (operator slice, rhs slice)
                    mma(0, 0, 0, acc_on);
                    mma(0, 1, 1, acc_on);
                    mma(1, 0, 2, acc_on);
                    mma(0, 2, 3, acc_on);
                    mma(1, 1, 4, acc_on);
                    mma(2, 0, 5, acc_on);
                    // levels 3 and 4 share accumulator 6
                    mma(0, 3, 6, acc_on);
                    mma(1, 2, 6, 1u);
                    mma(2, 1, 6, 1u);
                    mma(3, 0, 6, 1u);
                    mma(0, 4, 6, 1u);
                    mma(1, 3, 6, 1u);
                    mma(2, 2, 6, 1u);
                    mma(3, 1, 6, 1u);
                }
                tc::mma_commit(empty0 + 8 * st);
                if (last) {
                    tc::mma_commit(acc_full);
                    ++j;
                }
            }
            tc::mma_commit(done);
        }
        __syncwarp();
    } else {
        // epilogue: TMEM lane = tile row; this warp's runs [c0, c0 + half)
        const int e = warp - 2;
        const int quarter = warp & 3;
        const int half = Bp / 2;
        const int c0 = (e >> 2) * half;
        const uint32_t tbase = tmem + ((uint32_t)(32 * quarter) << 16) + (uint32_t)c0;
        float H[32], L[32];
#pragma unroll
        for (int c = 0; c < 32; ++c) H[c] = L[c] = 0.f;
        bool ok = true;
        for (int j = 0; j < nch; ++j) {
            ok = __all_sync(0xffffffffu, tc::mbar_wait(acc_full, j & 1) ? 1 : 0);
            if (!ok) {
                if (lane == 0) atomicExch(err, 3);
                break;
            }
            tc::tc_fence_after();
#pragma unroll
            for (int g = 0; g < 4; ++g) {
                if (g * 8 < half) {
                    uint32_t r[kAcc][8];
#pragma unroll
                    for (int a = 0; a < kAcc; ++a) tc::tmem_ld8_nowait(tbase + (uint32_t)(a * astride + g * 8), r[a]);
                    tc::tmem_wait_ld();
#pragma unroll
                    for (int x = 0; x < 8; ++x) {
                        float s, e0, e1, e2, e3, e4;
                        two_sum(__uint_as_float(r[0][x]), __uint_as_float(r[1][x]), s, e0);
                        two_sum(s, __uint_as_float(r[2][x]), s, e1);
                        two_sum(s, __uint_as_float(r[3][x]), s, e2);
                        two_sum(s, __uint_as_float(r[4][x]), s, e3);
                        two_sum(s, __uint_as_float(r[5][x]), s, e4);
                        const float t = __fadd_rn(
                            __fadd_rn(__fadd_rn(__fadd_rn(__fadd_rn(e0, e1), e2), e3), e4), __uint_as_float(r[6][x]));
                        // (H, L) += (s, t)
                        float S, E;
                        two_sum(H[g * 8 + x], s, S, E);
                        E = __fadd_rn(E, __fadd_rn(L[g * 8 + x], t));
                        const float Hn = __fadd_rn(S, E);
                        L[g * 8 + x] = __fsub_rn(E, __fsub_rn(Hn, S));
                        H[g * 8 + x] = Hn;
                    }
                }
            }
            tc::tc_fence_before();
            __syncwarp();
            if (lane == 0) tc::mbar_arrive(acc_empty);
        }
        const int64_t M = 3 * N;
        const int64_t m = mt * kTileM + 32 * quarter + lane;
        if (ok && m < M) {
#pragma unroll
            for (int c = 0; c < 32; ++c)
                if (c < half) out[((int64_t)slice * Bp + c0 + c) * M + m] = make_float2(H[c], L[c]);
        }
    }
    // free tensor memory once the tensor-core work of this CTA has completed
    if (warp == 0) {
        const bool fin = __all_sync(0xffffffffu, tc::mbar_wait(done, 0) ? 1 : 0);
        if (!fin && lane == 0) atomicExch(err, 5);
    }
    tc::tc_fence_before();
    __syncthreads();
    tc::tc_fence_after();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(ncols) : "memory");
}

// ---------------------------------------------------------------------------
// packing

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

// operator: one warp per row of the tile, 1024 columns of chunk blockIdx.x
__global__ void __launch_bounds__(256) pack_operator_fix_kernel(const double *__restrict__ K64, int64_t N,
                                                                 const int64_t *__restrict__ order,
                                                                 __nv_bfloat16 *__restrict__ out)
{
    const int64_t ch = blockIdx.x, mt = blockIdx.y;
    const int64_t M = 3 * N, Kd = 2 * N, KB = k_blocks(N);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int rr = warp; rr < kTileM; rr += 8) {
        const int64_t m = mt * kTileM + rr;
        const int64_t mrow = (m < M && order) ? 3 * order[m / 3] + m % 3 : m;   // operator row at position m
        double x[kBlocksPerChunk];
        double mx = 0.0;
#pragma unroll
        for (int t = 0; t < kBlocksPerChunk; ++t) {
            const int64_t col = ch * kChunk + t * kBlockK + lane;
            const int64_t kcol = (col < Kd && order) ? 2 * order[col / 2] + (col & 1) : col;
            x[t] = (m < M && col < Kd) ? K64[mrow * Kd + kcol] : 0.0;
            mx = fmax(mx, fabs(x[t]));
        }
        for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
        const int e = chunk_exponent(mx);
#pragma unroll
        for (int t = 0; t < kBlocksPerChunk; ++t) {
            const int64_t kb = ch * kBlocksPerChunk + t;
            if (kb >= KB) break;
            int d[kKPieces];
            digits<kKPieces>(__double2ll_rn(ldexp(x[t], 8 * kKPieces - 1 - e)), d);
            __nv_bfloat16 *base = out + (size_t)(mt * KB + kb) * kKPieces * kTileM * kBlockK;
            const int o = image_offset(rr, lane);
#pragma unroll
            for (int p = 0; p < kKPieces; ++p)
                base[(size_t)p * kTileM * kBlockK + o] = __float2bfloat16_rn(ldexpf((float)d[p], e - 7 - 8 * p));
        }
    }
}

// right-hand side: one block of 512 threads per (chunk, run), one cell per
// thread (a chunk is 512 cells = 1024 columns); v' from `v` ([B][2N] FP64) or
// from the stepper's slip rates
struct RhsSrc {
    const double *v;   // [B][2N] or null
    const double *slipv1, *slipv2, *cos_rake0, *sin_rake0;   // [B][N]
    double Vpl;
    const int64_t *order;   // position -> cell, or null (identity)
};

__global__ void __launch_bounds__(512) pack_rhs_fix_kernel(RhsSrc src, int64_t N, int B, int Bp,
                                                            __nv_bfloat16 *__restrict__ out)
{
    __shared__ double red[16];
    const int64_t ch = blockIdx.x;
    const int r = blockIdx.y;
    const int i = threadIdx.x;
    const int64_t pos = ch * (kChunk / 2) + i;
    const int64_t KB = k_blocks(N);
    double v1 = 0.0, v2 = 0.0;
    if (r < B && pos < N) {
        const int64_t cell = src.order ? src.order[pos] : pos;
        const int64_t idx = (int64_t)r * N + cell;
        if (src.v) {
            v1 = src.v[(int64_t)r * 2 * N + 2 * cell];
            v2 = src.v[(int64_t)r * 2 * N + 2 * cell + 1];
        } else {
            v1 = src.slipv1[idx] - src.Vpl * src.cos_rake0[idx];
            v2 = src.slipv2[idx] - src.Vpl * src.sin_rake0[idx];
        }
    }
    double mx = fmax(fabs(v1), fabs(v2));
    for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if ((i & 31) == 0) red[i >> 5] = mx;
    __syncthreads();
    if (i < 32) {
        double t = i < 16 ? red[i] : 0.0;
        for (int o = 8; o > 0; o >>= 1) t = fmax(t, __shfl_xor_sync(0xffffffffu, t, o));
        if (i == 0) red[0] = t;
    }
    __syncthreads();
    const int e = chunk_exponent(red[0]);
    const int64_t kb = ch * kBlocksPerChunk + i / 16;
    if (kb >= KB) return;
    int d1[kVPieces], d2[kVPieces];
    digits<kVPieces>(__double2ll_rn(ldexp(v1, 8 * kVPieces - 1 - e)), d1);
    digits<kVPieces>(__double2ll_rn(ldexp(v2, 8 * kVPieces - 1 - e)), d2);
    const int64_t img = (int64_t)Bp * kBlockK;
    __nv_bfloat16 *P = out + kb * kVPieces * img + image_offset(r, (2 * i) % kBlockK);
#pragma unroll
    for (int q = 0; q < kVPieces; ++q) {
        __nv_bfloat162 w;
        w.x = __float2bfloat16_rn(ldexpf((float)d1[q], e - 7 - 8 * q));
        w.y = __float2bfloat16_rn(ldexpf((float)d2[q], e - 7 - 8 * q));
        reinterpret_cast<__nv_bfloat162 *>(P + q * img)[0] = w;
    }
}

static int launch_pack_rhs(const RhsSrc &src, int64_t N, int B, int Bp, void *Vpacked, cudaStream_t stream)
{
    dim3 grid((unsigned)k_chunks(N), (unsigned)Bp);
    pack_rhs_fix_kernel<<<grid, kChunk / 2, 0, stream>>>(src, N, B, Bp, (__nv_bfloat16 *)Vpacked);
    PQ3D_CUDA_TRY(cudaGetLastError());
    return PQ3D_OK;
}

int pack_rhs_from_state(const double *slipv1, const double *slipv2, const double *cos_rake0, const double *sin_rake0,
                        double Vpl, const int64_t *order, int64_t N, int B, void *Vpacked, cudaStream_t stream)
{
    const RhsSrc src{nullptr, slipv1, slipv2, cos_rake0, sin_rake0, Vpl, order};
    return launch_pack_rhs(src, N, B, (B + 15) / 16 * 16, Vpacked, stream);
}

// ---------------------------------------------------------------------------
// launch

static int stages_for(int Bp, int *stages)
{
    int dev, maxs = 0;
    PQ3D_CUDA_TRY(cudaGetDevice(&dev));
    PQ3D_CUDA_TRY(cudaDeviceGetAttribute(&maxs, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    const size_t stage_bytes = (size_t)kKPieces * kImageA + (size_t)kVPieces * Bp * kBlockK * 2;
    int s = (int)((maxs - 1024 - 64) / (stage_bytes + 16));
    if (s > 6) s = 6;
    PQ3D_REQUIRE(s >= 2, "gemm_bf16x14: not enough shared memory for B=%d", Bp);
    static thread_local int cfg_dev = -1;
    if (cfg_dev != dev) {
        PQ3D_CUDA_TRY(cudaFuncSetAttribute(gemm_fix_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, maxs));
        cfg_dev = dev;
    }
    *stages = s;
    return PQ3D_OK;
}

int gemm_bf16x14(const void *Kpacked, const void *Vpacked, int64_t N, int Bp, int nsplit, float2 *out,
                 void *workspace, size_t workspace_bytes, cudaStream_t stream)
{
    PQ3D_REQUIRE(Kpacked && Vpacked && out && workspace, "gemm_bf16x14: null pointer");
    PQ3D_REQUIRE(N > 0, "gemm_bf16x14: N must be positive");
    PQ3D_REQUIRE(workspace_bytes >= 256 && aligned16(workspace), "gemm_bf16x14: workspace must be >= 256 bytes");
    PQ3D_REQUIRE(Bp >= 16 && Bp <= kMaxRuns && Bp % 16 == 0,
                 "gemm_bf16x14: padded run count must be 16..%d, multiple of 16", kMaxRuns);
    PQ3D_REQUIRE(aligned16(Kpacked) && aligned16(Vpacked) && aligned16(out),
                 "gemm_bf16x14: operands must be 16-byte aligned");
    const int64_t KB = k_blocks(N);
    PQ3D_REQUIRE(nsplit >= 1 && nsplit <= KB, "gemm_bf16x14: nsplit must be in [1, %lld]", (long long)KB);
    int stages;
    int rc = stages_for(Bp, &stages);
    if (rc) return rc;
    const size_t stage_bytes = (size_t)kKPieces * kImageA + (size_t)kVPieces * Bp * kBlockK * 2;
    const size_t smem = (size_t)stages * stage_bytes + 16 * (size_t)stages + 48;
    dim3 grid((unsigned)m_tiles(N), (unsigned)nsplit);
    gemm_fix_kernel<<<grid, kThreads, smem, stream>>>((const uint8_t *)Kpacked, (const uint8_t *)Vpacked, N, Bp,
                                                      nsplit, out, (int *)workspace, stages);
    PQ3D_CUDA_TRY(cudaGetLastError());
    return PQ3D_OK;
}

}  // namespace fx
}  // namespace pq3d

using namespace pq3d;

extern "C" size_t pq3d_batch_operator_fix_bytes(int64_t N) { return N > 0 ? fx::packed_operator_bytes(N) : 0; }

extern "C" size_t pq3d_batch_rhs_fix_bytes(int64_t N, int B)
{
    const int Bp = (B + 15) / 16 * 16;
    return N > 0 && B > 0 ? fx::packed_rhs_bytes(N, Bp) : 0;
}

extern "C" int pq3d_batch_pack_operator_fix(const double *K64, int64_t N, const int64_t *order, void *Kpacked,
                                            void *stream)
{
    clear_error();
    PQ3D_REQUIRE(K64 && Kpacked && N > 0, "pq3d_batch_pack_operator_fix: bad arguments");
    PQ3D_REQUIRE(aligned16(Kpacked), "pq3d_batch_pack_operator_fix: output must be 16-byte aligned");
    dim3 grid((unsigned)fx::k_chunks(N), (unsigned)fx::m_tiles(N));
    fx::pack_operator_fix_kernel<<<grid, 256, 0, (cudaStream_t)stream>>>(K64, N, order, (__nv_bfloat16 *)Kpacked);
    PQ3D_CUDA_TRY(cudaGetLastError());
    return PQ3D_OK;
}

extern "C" int pq3d_batch_pack_rhs_fix(const double *v, int64_t N, int B, const int64_t *order, void *Vpacked,
                                       void *stream)
{
    clear_error();
    PQ3D_REQUIRE(v && Vpacked && N > 0 && B >= 1 && B <= fx::kMaxRuns, "pq3d_batch_pack_rhs_fix: bad arguments");
    PQ3D_REQUIRE(aligned16(Vpacked), "pq3d_batch_pack_rhs_fix: output must be 16-byte aligned");
    const fx::RhsSrc src{v, nullptr, nullptr, nullptr, nullptr, 0.0, order};
    return fx::launch_pack_rhs(src, N, B, (B + 15) / 16 * 16, Vpacked, (cudaStream_t)stream);
}

extern "C" int pq3d_batch_gemm_bf16x14(const void *Kpacked, const void *Vpacked, int64_t N, int B, int nsplit,
                                       float *out, void *workspace, size_t workspace_bytes, void *stream)
{
    clear_error();
    PQ3D_REQUIRE(B >= 1 && B <= fx::kMaxRuns, "pq3d_batch_gemm_bf16x14: B must be 1..%d", fx::kMaxRuns);
    return fx::gemm_bf16x14(Kpacked, Vpacked, N, (B + 15) / 16 * 16, nsplit, (float2 *)out, workspace,
                            workspace_bytes, (cudaStream_t)stream);
}
