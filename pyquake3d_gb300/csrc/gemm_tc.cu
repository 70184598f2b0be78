// Batched traction product on the 5th-generation tensor cores (tcgen05).
//
//   out[s][n][m] = sum_{k in slice s} K[m][k] * V[n][k]
//   K: (3N) x (2N) traction operator, V: B slip-rate deficits (one per run).
//
// Precision ("BF16x6"): the FP64 operator and the FP64 right-hand side are
// split into three BF16 pieces each (x = x0 + x1 + x2, 24 significant bits);
// the six cross products x_i * y_j with i + j <= 2 are accumulated in FP32 in
// tensor memory.  Their sum carries the operands to ~2^-26 (the dropped
// products are x_1 y_2, x_2 y_1, x_2 y_2), while two-piece "BF16x3" carries
// them to ~2^-16.  The leading product x_0 y_0 and the five corrections go to
// two accumulators, added (round to nearest) when drained: the tensor-memory
// accumulation loses more than an FP32 FMA chain would when small terms are
// added to a large accumulator, and the corrections are 2^-8 of the leading
// product and less.  (On the N = 10,000 planar operator with a nucleation
// patch, one accumulator for all six products gave a 2.7e-6 normwise error,
// the leading product alone 7.4e-7, FP32 FMA 3.7e-7, the pieces' exact sum
// 1.6e-8.)  Slices of the reduction (split-K) are written as FP32 and added
// in float-float by the consumer.
//
// Data path (one CTA = one 128-row tile of K x one K slice, all runs):
//   * the operator pieces are packed once, after assembly, into ready-made
//     shared-memory images: for every (tile, 32-column block) three 128 x 32
//     BF16 images of 8-row x 16-byte core matrices (K-major, no swizzle); the
//     right-hand side pieces are written in the same image layout by the
//     stepper.  One pipeline stage is therefore two contiguous 1-D bulk
//     copies (cp.async.bulk, completion on an mbarrier), no tensor map.
//   * warp 0 lane 0 produces stages, warp 1 lane 0 issues 12 tcgen05.mma
//     (M=128, N=B, K=16; 6 products x 2 K-steps) per stage and frees the stage
//     with tcgen05.commit; all 4 warps drain the two FP32 accumulators from
//     tensor memory (tcgen05.ld 32x32b) and store their sum (FP32).
//   * every mbarrier wait is bounded; a wait that gives up records an error
//     word in the workspace, the kernel still waits (bounded) for its own
//     tensor-core work, frees its tensor memory and returns.
// No cluster, no multicast: each CTA reads its own tiles.
#include <cuda_bf16.h>
#include <stdint.h>
#include <stdlib.h>

#include "common.cuh"
#include "gemm_tc.cuh"
#include "tc_ptx.cuh"

namespace pq3d {
namespace tc {

constexpr uint32_t kImageA = kTileM * kBlockK * 2;   // bytes of one A piece image (8 KB)

// The 6 leading cross products of the 3-piece splits: (piece of K, piece of V).
__constant__ int kPairA[6] = {0, 0, 1, 0, 1, 2};
__constant__ int kPairB[6] = {0, 1, 0, 2, 1, 0};

__global__ void __launch_bounds__(128, 1)
gemm_bf16x6_kernel(const uint8_t *__restrict__ Kp, const uint8_t *__restrict__ Vp, int64_t N, int Bp, int nsplit,
                   float *__restrict__ out, int *__restrict__ err, int stages)
{
    extern __shared__ __align__(1024) uint8_t smem[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t mt = blockIdx.x;
    const int slice = blockIdx.y;
    const int64_t KB = (2 * N + kBlockK - 1) / kBlockK;
    const int64_t kb0 = KB * slice / nsplit, kb1 = KB * (slice + 1) / nsplit;
    const int nkb = (int)(kb1 - kb0);
    const uint32_t a_bytes = kPieces * kImageA;
    const uint32_t b_img = (uint32_t)Bp * kBlockK * 2;
    const uint32_t b_bytes = kPieces * b_img;
    const uint32_t stage_bytes = a_bytes + b_bytes;
    uint8_t *bars = smem + (size_t)stages * stage_bytes;
    const uint32_t full0 = smem_u32(bars), empty0 = full0 + 8 * stages, done = full0 + 16 * stages;
    uint32_t *tmem_slot = (uint32_t *)(bars + 16 * stages + 8);
    const uint32_t ncols = tmem_cols(Bp);   // per accumulator; two accumulators

    if (threadIdx.x == 0) {
        for (int s = 0; s < stages; ++s) {
            mbar_init(full0 + 8 * s, 1);
            mbar_init(empty0 + 8 * s, 1);
        }
        mbar_init(done, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                     "r"(2 * ncols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *(volatile uint32_t *)tmem_slot;

    if (warp == 0 && lane == 0) {
        // producer: two bulk copies per stage
        for (int it = 0; it < nkb; ++it) {
            const int st = it % stages, use = it / stages;
            if (!mbar_wait(empty0 + 8 * st, (use & 1) ^ 1)) { atomicExch(err, 1); break; }
            const uint32_t sa = smem_u32(smem + (size_t)st * stage_bytes);
            const int64_t kb = kb0 + it;
            mbar_expect_tx(full0 + 8 * st, stage_bytes);
            bulk_g2s(sa, Kp + (size_t)(mt * KB + kb) * a_bytes, a_bytes, full0 + 8 * st);
            bulk_g2s(sa + a_bytes, Vp + (size_t)kb * b_bytes, b_bytes, full0 + 8 * st);
        }
    } else if (warp == 1 && lane == 0) {
        // tensor-core issuer
        const uint32_t idesc = idesc_bf16(kTileM, Bp);
        for (int it = 0; it < nkb; ++it) {
            const int st = it % stages, use = it / stages;
            if (!mbar_wait(full0 + 8 * st, use & 1)) { atomicExch(err, 2); break; }
            tc_fence_after();
            const uint32_t sa = smem_u32(smem + (size_t)st * stage_bytes);
            const uint32_t sb = sa + a_bytes;
#pragma unroll
            for (int ks = 0; ks < 2; ++ks) {
#pragma unroll
                for (int p = 0; p < 6; ++p) {
                    const uint64_t ad = smem_desc(sa + kPairA[p] * kImageA + ks * 256, 128, 512);
                    const uint64_t bd = smem_desc(sb + kPairB[p] * b_img + ks * 256, 128, 512);
                    // leading product into the first accumulator, the five
                    // corrections (2^-8 of it and less) into the second
                    const uint32_t acc = it > 0 || ks > 0 || p > 1;
                    mma_bf16(p == 0 ? tmem : tmem + ncols, ad, bd, idesc, p == 0 ? (uint32_t)(it > 0 || ks > 0) : acc);
                }
            }
            mma_commit(empty0 + 8 * st);
        }
        mma_commit(done);
    }
    __syncwarp();

    // epilogue: TMEM lane = tile row, column = run
    const bool got = __all_sync(0xffffffffu, mbar_wait(done, 0) ? 1 : 0);
    tc_fence_after();
    const int64_t M = 3 * N;
    const int64_t m = mt * kTileM + 32 * warp + lane;
    if (got) {
        for (int c0 = 0; c0 < Bp; c0 += 16) {
            uint32_t r[16], q[16];
            tmem_ld16(tmem + ((uint32_t)(32 * warp) << 16) + (uint32_t)c0, r);
            tmem_ld16(tmem + ((uint32_t)(32 * warp) << 16) + ncols + (uint32_t)c0, q);
            if (m < M) {
#pragma unroll
                for (int j = 0; j < 16; ++j)
                    out[((int64_t)slice * Bp + c0 + j) * M + m] = __fadd_rn(__uint_as_float(r[j]), __uint_as_float(q[j]));
            }
        }
    } else if (lane == 0) {
        atomicExch(err, 3);
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(2 * ncols) : "memory");
}

// FP64 operator -> three BF16 pieces in the tile-image layout.
__global__ void pack_operator_kernel(const double *__restrict__ K64, int64_t N, __nv_bfloat16 *__restrict__ out)
{
    const int64_t mt = blockIdx.y, kb = blockIdx.x;
    const int64_t KB = gridDim.x;
    const int64_t M = 3 * N, Kd = 2 * N;
    __nv_bfloat16 *base = out + (size_t)(mt * KB + kb) * kPieces * kTileM * kBlockK;
    for (int e = threadIdx.x; e < kTileM * kBlockK; e += blockDim.x) {
        const int row = e / kBlockK, col = e % kBlockK;
        const int64_t m = mt * kTileM + row, k = kb * kBlockK + col;
        const double x = (m < M && k < Kd) ? K64[m * Kd + k] : 0.0;
        const __nv_bfloat16 p0 = __double2bfloat16(x);
        const double r1 = x - (double)__bfloat162float(p0);
        const __nv_bfloat16 p1 = __double2bfloat16(r1);
        const __nv_bfloat16 p2 = __double2bfloat16(r1 - (double)__bfloat162float(p1));
        const int o = image_offset(row, col);
        base[o] = p0;
        base[kTileM * kBlockK + o] = p1;
        base[2 * kTileM * kBlockK + o] = p2;
    }
}

size_t gemm_bf16x6_workspace_bytes(int64_t, int, int) { return 256; }

struct Cfg {
    int device = -1;
    int max_smem = 0;   // per block (opt-in)
    int sm_smem = 0;    // per SM
};
static thread_local Cfg g_cfg;

static int device_cfg()
{
    int dev;
    PQ3D_CUDA_TRY(cudaGetDevice(&dev));
    if (g_cfg.device != dev) {
        int maxs = 0, sms = 0;
        PQ3D_CUDA_TRY(cudaDeviceGetAttribute(&maxs, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
        PQ3D_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev));
        PQ3D_CUDA_TRY(cudaFuncSetAttribute(gemm_bf16x6_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, maxs));
        g_cfg.device = dev;
        g_cfg.max_smem = maxs;
        g_cfg.sm_smem = sms;
    }
    return PQ3D_OK;
}

// Launch plan for `ctas_per_sm` requested CTAs per SM (0 = 2): the most CTAs
// per SM, not above the request, for which each CTA still gets a pipeline of
// at least 2 stages and its tensor-memory columns, with up to 6 stages each.
// Several CTAs per SM let one stream the operator while another fills its
// pipeline or drains its accumulator, and make the last wave finer.
int plan_bf16x6(int Bp, int ctas_per_sm, int *ctas, int *stages)
{
    int rc = device_cfg();
    if (rc) return rc;
    const int want = ctas_per_sm == 0 ? 2 : ctas_per_sm;
    const size_t stage_bytes = (size_t)kPieces * (kImageA + (size_t)Bp * kBlockK * 2);
    *ctas = 0;
    *stages = 0;
    for (int c = want; c >= 1 && *stages == 0; --c) {
        int s = (int)((g_cfg.sm_smem / c - 1024 - 16) / (stage_bytes + 16));
        if (s > 6) s = 6;
        if (s > (int)((g_cfg.max_smem - 1024) / (stage_bytes + 16))) s = (int)((g_cfg.max_smem - 1024) / (stage_bytes + 16));
        if (s >= 2 && c * 2 * (int)tmem_cols(Bp) <= 512) {
            *stages = s;
            *ctas = c;
        }
    }
    PQ3D_REQUIRE(*stages >= 2, "gemm_bf16x6: not enough shared memory for B=%d", Bp);
    return PQ3D_OK;
}

int gemm_bf16x6(const void *Kpacked, const void *Vpacked, int64_t N, int Bp, int nsplit, int ctas_per_sm, float *out,
                void *workspace, size_t workspace_bytes, cudaStream_t stream)
{
    PQ3D_REQUIRE(Kpacked && Vpacked && out && workspace, "gemm_bf16x6: null pointer");
    PQ3D_REQUIRE(workspace_bytes >= 256 && aligned16(workspace), "gemm_bf16x6: workspace must be >= 256 bytes");
    PQ3D_REQUIRE(Bp >= 16 && Bp <= 256 && Bp % 16 == 0, "gemm_bf16x6: padded run count must be 16..256, multiple of 16");
    PQ3D_REQUIRE(aligned16(Kpacked) && aligned16(Vpacked), "gemm_bf16x6: operands must be 16-byte aligned");
    PQ3D_REQUIRE(ctas_per_sm >= 0 && ctas_per_sm <= 3, "gemm_bf16x6: ctas_per_sm must be 0 (default) or 1..3");
    const int64_t KB = k_blocks(N);
    PQ3D_REQUIRE(nsplit >= 1 && nsplit <= KB, "gemm_bf16x6: nsplit must be in [1, %lld]", (long long)KB);
    int ctas, stages;
    int rc = plan_bf16x6(Bp, ctas_per_sm, &ctas, &stages);
    if (rc) return rc;
    const size_t stage_bytes = (size_t)kPieces * (kImageA + (size_t)Bp * kBlockK * 2);
    const size_t smem = (size_t)stages * stage_bytes + 16 * (size_t)stages + 16;
    dim3 grid((unsigned)m_tiles(N), (unsigned)nsplit);
    gemm_bf16x6_kernel<<<grid, 128, smem, stream>>>((const uint8_t *)Kpacked, (const uint8_t *)Vpacked, N, Bp, nsplit,
                                                     out, (int *)workspace, stages);
    PQ3D_CUDA_TRY(cudaGetLastError());
    return PQ3D_OK;
}

}  // namespace tc
}  // namespace pq3d

using namespace pq3d;

extern "C" size_t pq3d_batch_operator_bytes(int64_t N) { return N > 0 ? tc::packed_operator_bytes(N) : 0; }

extern "C" size_t pq3d_batch_rhs_bytes(int64_t N, int B)
{
    const int Bp = (B + 15) / 16 * 16;
    return N > 0 && B > 0 ? tc::packed_rhs_bytes(N, Bp) : 0;
}

extern "C" int pq3d_batch_pack_operator(const double *K64, int64_t N, void *Kpacked, void *stream)
{
    clear_error();
    PQ3D_REQUIRE(K64 && Kpacked && N > 0, "pq3d_batch_pack_operator: bad arguments");
    PQ3D_REQUIRE(aligned16(Kpacked), "pq3d_batch_pack_operator: output must be 16-byte aligned");
    dim3 grid((unsigned)tc::k_blocks(N), (unsigned)tc::m_tiles(N));
    tc::pack_operator_kernel<<<grid, 256, 0, (cudaStream_t)stream>>>(K64, N, (__nv_bfloat16 *)Kpacked);
    PQ3D_CUDA_TRY(cudaGetLastError());
    return PQ3D_OK;
}

extern "C" int pq3d_batch_gemm_bf16x6(const void *Kpacked, const void *Vpacked, int64_t N, int B, int nsplit,
                                      int ctas_per_sm, float *out, void *workspace, size_t workspace_bytes,
                                      void *stream)
{
    clear_error();
    return tc::gemm_bf16x6(Kpacked, Vpacked, N, (B + 15) / 16 * 16, nsplit, ctas_per_sm, out, workspace,
                           workspace_bytes, (cudaStream_t)stream);
}

extern "C" int pq3d_batch_gemm_bf16x6_plan(int B, int ctas_per_sm, int32_t *plan)
{
    clear_error();
    PQ3D_REQUIRE(plan && B >= 1 && B <= 256, "pq3d_batch_gemm_bf16x6_plan: bad arguments");
    PQ3D_REQUIRE(ctas_per_sm >= 0 && ctas_per_sm <= 3, "pq3d_batch_gemm_bf16x6_plan: ctas_per_sm must be 0..3");
    int ctas, stages;
    int rc = tc::plan_bf16x6((B + 15) / 16 * 16, ctas_per_sm, &ctas, &stages);
    if (rc) return rc;
    plan[0] = ctas;
    plan[1] = stages;
    return PQ3D_OK;
}
