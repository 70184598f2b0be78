// Batched traction product on the 5th-generation tensor cores (tcgen05) with
// exact fixed-point slices ("BF16x18"):
//
//   sum_s out[s][n][m] = sum_k K[m][k] * V[n][k]   (hi + lo, ~2^-44 relative;
//   s: a K slice, or a share of the balanced grid below)
//   K: (3N) x (2N) traction operator, V: B slip-rate deficits v' = V - Vpl.
//
// Why: the reference evaluates K.(V - Vpl) in FP64 (src/QDsim_gpu.py:948-957).
// A product that rounds v' or its own running sums at FP32 level (~2^-24) each
// step -- BF16x3, TF32 or the three-piece BF16x6 product -- perturbs the
// traction rate by a fresh ~1e-7 every step, and a nucleating rupture
// amplifies that past 1e-5 in slip within ~25 accepted steps.  A static
// rounding of the operator is amplified far less (rounded once to FP32 it
// stays within 1e-5 for ~130 steps).  So this product carries the operator to
// 32 bits (static) and v' to 48 bits (dynamic), keeps every slice product down
// to 2^-40 of the leading one, and accumulates without rounding.
//
// Representation (Ozaki-style fixed point):
//   * operator row m, 1024-column chunk c: e = exponent of max |K[m][c..]|,
//     K[m][k] ~= sum_{p<4} d_p 2^(e - 7 - 8p), integer digits |d_p| <= 128
//     (balanced base 256 of round(K 2^(31-e))): 32 bits of the chunk's largest
//     entry;
//   * run n, 256-column span: the same with 6 digits of v'_n (48 bits of the
//     span's largest |v'|).
//   Each digit times its power of two is exact in BF16, and the slices are
//   stored with that scale, so the products are plain BF16 tensor-core
//   products.
//   * A digit product d_p e_q is an integer of at most 2^14 units of
//     2^(eK + eV - 14 - 8(p+q)): within one span every product of one level
//     l = p + q lies on that grid.  Level l collects min(l+1, 4) slice pairs
//     over 256 columns: at most 4 * 256 * 2^14 = 2^24 units, exact in the FP32
//     tensor-memory accumulator.  The 18 pairs with p + q <= 5 are kept (the
//     dropped ones are below 2^-40 of the leading product).
//   * Tensor-memory slot l (Bq columns, Bq = runs rounded up to 32) holds level
//     l.  With the right-hand-side slices stored one after another, the
//     products of operator slice p with slices q..q+w-1 are ONE tcgen05.mma of
//     N = w Bq whose accumulator starts at slot p + q: 6 instructions per
//     16-column step cover the 18 pairs (an instruction costs about the same
//     for N = 64 and 128, so wide instructions halve the time of 14 narrow
//     ones).
//   * After each span the 6 slots are drained (tcgen05.ld) and combined into
//     a float-float pair (s, t): levels 0-3 by three exact Fast2Sums, 4 and 5
//     into t.  The slots are then released, and (s, t) is added into the
//     running float-float sum in registers while the tensor cores already
//     fill the slots with the next span.  Packed f32x2 additions, two runs
//     per instruction.
//
// Data path (one CTA per SM: one 128-row tile of K x one K slice, or in the
// balanced grid an equal share of the tile-major 32-column blocks; all runs):
//   * warp 0 lane 0: producer, two 1-D bulk copies per 32-column stage (the
//     four operator slice images, 32 KB, and the six right-hand-side slice
//     images), completion on the stage's mbarrier;
//   * warp 1 lane 0: 2 K-steps x 6 tcgen05.mma per stage (descriptors
//     precomputed per stage), the stage freed by tcgen05.commit; at the end of
//     a span a commit hands the slots to the epilogue, and before the next
//     span it waits until they are drained;
//   * warps 2-9: epilogue, two warps per 32-lane quarter of tensor memory
//     (the rows), each taking half of the runs (16 epilogue warps measured
//     no faster: the drain is bound by FP32 issue, not by warps).
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

constexpr int kEpiWarps = 8;                         // a multiple of 4 (one group per TMEM lane quarter)
constexpr int kEpiRuns = kMaxRuns / (kEpiWarps / 4);   // runs per epilogue warp at most
constexpr int kThreads = 64 + 32 * kEpiWarps;
constexpr uint32_t kImageA = kTileM * kBlockK * 2;   // one operator slice image: 8 KB

// Two FP32 values in one 64-bit register and the packed (f32x2) additions of
// sm_100 and later: each lane adds two pairs per instruction, IEEE round to
// nearest, so the drain below rounds exactly as the scalar __fadd_rn would.
typedef uint64_t f32x2;
__device__ __forceinline__ f32x2 pack2(uint32_t a, uint32_t b)
{
    f32x2 r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "r"(a), "r"(b));
    return r;
}
__device__ __forceinline__ float2 unpack2(f32x2 a)
{
    float2 r;
    asm("mov.b64 {%0, %1}, %2;" : "=f"(r.x), "=f"(r.y) : "l"(a));
    return r;
}
__device__ __forceinline__ f32x2 add2(f32x2 a, f32x2 b)
{
    f32x2 r;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ f32x2 sub2(f32x2 a, f32x2 b)
{
    f32x2 r;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ void two_sum2(f32x2 a, f32x2 b, f32x2 &s, f32x2 &e)
{
    s = add2(a, b);
    const f32x2 bb = sub2(s, a);
    e = add2(sub2(a, sub2(s, bb)), sub2(b, bb));
}

// Fast2Sum (s + e = a + b exactly) for the level combination.  Levels lie on
// nested grids: level l is an integer I_l, |I_l| <= 2^24, in units u 2^(-8l).
// With a a multiple of 256 units of b's grid and b such an integer, s - a is
// representable (for ulp(s) = 2^k, k <= 8: a multiple of 2^k below 2^(24+k);
// k > 8: |a| >= 2^(22+k), so a and s - a are multiples of 2^(k-1) with a
// significand below 2^24), and the error a + b - s is an integer of at most
// 2^(k-1) <= 2^24 units while the running sum stays below 2^49 units of the
// finest level -- true for the four levels (2^24 * 2^24 + ...).  So the
// error is exact although |a| >= |b| need not hold, and equals what TwoSum
// (6 operations instead of 3) would return.
__device__ __forceinline__ void fast_two_sum2(f32x2 a, f32x2 b, f32x2 &s, f32x2 &e)
{
    s = add2(a, b);
    e = sub2(b, sub2(s, a));
}

// descriptor of the operand `bytes` further on in shared memory (the start
// address field, bits 0-13 in 16-byte units, does not overflow below 256 KB)
__device__ __forceinline__ uint64_t desc_at(uint64_t d, uint32_t bytes) { return d + (bytes >> 4); }

// The work of a CTA as segments: blocks [kb0, kb1) of one 128-row tile,
// summed into output slice `slice`.
//   * Slice grid (units == 0): CTA (tile blockIdx.x, K slice blockIdx.y), one
//     segment, the slice's blocks KB s / nsplit .. KB (s + 1) / nsplit.
//   * Balanced grid (units = tiles x KB): one CTA per SM; CTA c takes the
//     units [c W / G, (c + 1) W / G) of the tile-major list u = tile KB + kb,
//     so every CTA streams the same number of blocks and no partial last
//     wave is left.  Its segment of a tile writes slice c - c0, c0 the CTA
//     holding the tile's first block (the host launches this grid only when
//     no tile meets more than nsplit CTAs), and the segment that ends a tile
//     writes zeros to the slices above its own.
struct Seg {
    int64_t tile, kb0, kb1;
    int slice;
    bool tail;   // ends the tile in a balanced grid: zero the slices above
};

struct FixSched {
    int64_t KB, units;   // blocks per tile; units of the balanced grid (0: slice grid)
    int nsplit;
};

// CTA of a balanced grid of G CTAs over W units that holds unit x
__host__ __device__ inline int64_t bal_owner(int64_t x, int64_t W, int64_t G) { return ((x + 1) * G - 1) / W; }

// segment i of this CTA (false past the last)
__device__ __forceinline__ bool fix_segment(const FixSched &sc, int i, Seg &sg)
{
    if (sc.units == 0) {
        if (i > 0) return false;
        sg.tile = blockIdx.x;
        sg.slice = blockIdx.y;
        sg.kb0 = sc.KB * sg.slice / sc.nsplit;
        sg.kb1 = sc.KB * (sg.slice + 1) / sc.nsplit;
        sg.tail = false;
        return sg.kb1 > sg.kb0;
    }
    const int64_t G = gridDim.x, c = blockIdx.x;
    const int64_t u0 = c * sc.units / G, u1 = (c + 1) * sc.units / G;
    const int64_t t = u0 / sc.KB + i;
    const int64_t ub = i == 0 ? u0 : t * sc.KB;   // first unit of the segment
    if (ub >= u1) return false;
    sg.tile = t;
    sg.kb0 = ub - t * sc.KB;
    sg.kb1 = min(sc.KB, u1 - t * sc.KB);
    sg.slice = sg.kb0 == 0 ? 0 : (int)(c - bal_owner(t * sc.KB, sc.units, G));
    sg.tail = sg.kb1 == sc.KB;
    return true;
}

// Bq: runs of the product (32 or 64); Bo: runs written (<= Bq, multiple of 16)
__global__ void __launch_bounds__(kThreads, 1)
gemm_fix_kernel(const uint8_t *__restrict__ Kp, const uint8_t *__restrict__ Vp, int64_t N, int Bq, int Bo,
                FixSched sc, float2 *__restrict__ out, int *__restrict__ err, int stages)
{
    extern __shared__ __align__(1024) uint8_t smem[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t KB = sc.KB;
    const uint32_t a_bytes = kKPieces * kImageA;
    const uint32_t b_img = (uint32_t)Bq * kBlockK * 2;
    const uint32_t b_bytes = kVPieces * b_img;
    const uint32_t stage_bytes = a_bytes + b_bytes;
    uint8_t *bars = smem + (size_t)stages * stage_bytes;
    const uint32_t full0 = tc::smem_u32(bars), empty0 = full0 + 8 * stages;
    const uint32_t acc_full = full0 + 16 * stages, acc_empty = acc_full + 8, done = acc_full + 16;
    uint32_t *tmem_slot = (uint32_t *)(bars + 16 * stages + 24);
    const uint32_t ncols = tc::tmem_cols(kLevels * Bq);

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
            int it = 0;
            bool fail = false;
            Seg sg;
            for (int si = 0; !fail && fix_segment(sc, si, sg); ++si)
                for (int64_t kb = sg.kb0; kb < sg.kb1; ++kb, ++it) {
                    const int st = it % stages, use = it / stages;
                    if (!tc::mbar_wait(empty0 + 8 * st, (use & 1) ^ 1)) { atomicExch(err, 1); fail = true; break; }
                    const uint32_t sa = tc::smem_u32(smem + (size_t)st * stage_bytes);
                    tc::mbar_expect_tx(full0 + 8 * st, stage_bytes);
                    tc::bulk_g2s(sa, Kp + (size_t)(sg.tile * KB + kb) * a_bytes, a_bytes, full0 + 8 * st);
                    tc::bulk_g2s(sa + a_bytes, Vp + (size_t)kb * b_bytes, b_bytes, full0 + 8 * st);
                }
        }
        __syncwarp();
    } else if (warp == 1) {
        if (lane == 0) {
            // tensor-core issuer: instruction descriptors for N = Bq, 2Bq, 3Bq,
            // 4Bq and the slot addresses, computed once
            const uint32_t id1 = tc::idesc_bf16(kTileM, Bq), id2 = tc::idesc_bf16(kTileM, 2 * Bq);
            const uint32_t id3 = tc::idesc_bf16(kTileM, 3 * Bq), id4 = tc::idesc_bf16(kTileM, 4 * Bq);
            const uint32_t slot1 = tmem + (uint32_t)Bq, slot2 = tmem + 2u * Bq, slot3 = tmem + 3u * Bq;
            const uint32_t slot4 = tmem + 4u * Bq, slot5 = tmem + 5u * Bq;
            const uint32_t bq4 = 4u * b_img;
            int j = 0;    // span of this CTA
            int it = 0;   // block of this CTA
            bool fail = false;
            Seg sg;
            for (int si = 0; !fail && fix_segment(sc, si, sg); ++si)
                for (int64_t kb = sg.kb0; kb < sg.kb1; ++kb, ++it) {
                    const bool first = kb == sg.kb0 || kb % kBlocksPerSpan == 0;
                    const bool last = kb == sg.kb1 - 1 || (kb + 1) % kBlocksPerSpan == 0;
                    if (first && j > 0 && !tc::mbar_wait(acc_empty, (j - 1) & 1)) {
                        atomicExch(err, 4);
                        fail = true;
                        break;
                    }
                    const int st = it % stages, use = it / stages;
                    if (!tc::mbar_wait(full0 + 8 * st, use & 1)) { atomicExch(err, 2); fail = true; break; }
                    tc::tc_fence_after();
                    const uint32_t sa = tc::smem_u32(smem + (size_t)st * stage_bytes);
                    const uint64_t ad = tc::smem_desc(sa, 128, 512), bd = tc::smem_desc(sa + a_bytes, 128, 512);
#pragma unroll
                    for (int ks = 0; ks < 2; ++ks) {
                        const uint32_t f = (first && ks == 0) ? 0u : 1u;   // the first instruction of a slot overwrites it
                        const uint32_t k0 = ks * 256;
                        // operator slice 0 x rhs slices 0-3 -> slots 0-3, x slices 4-5 -> slots 4-5
                        tc::mma_bf16(tmem, desc_at(ad, k0), desc_at(bd, k0), id4, f);
                        tc::mma_bf16(slot4, desc_at(ad, k0), desc_at(bd, bq4 + k0), id2, f);
                        // slice 1 x 0-3 -> slots 1-4, x 4 -> slot 5
                        tc::mma_bf16(slot1, desc_at(ad, kImageA + k0), desc_at(bd, k0), id4, 1u);
                        tc::mma_bf16(slot5, desc_at(ad, kImageA + k0), desc_at(bd, bq4 + k0), id1, 1u);
                        // slice 2 x 0-3 -> slots 2-5; slice 3 x 0-2 -> slots 3-5
                        tc::mma_bf16(slot2, desc_at(ad, 2 * kImageA + k0), desc_at(bd, k0), id4, 1u);
                        tc::mma_bf16(slot3, desc_at(ad, 3 * kImageA + k0), desc_at(bd, k0), id3, 1u);
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
        // epilogue: TMEM lane = tile row; this warp's runs [c0, c0 + per)
        const int e = warp - 2;
        const int quarter = warp & 3;
        const int per = Bq / (kEpiWarps / 4);
        const int c0 = (e >> 2) * per;
        const uint32_t tbase = tmem + ((uint32_t)(32 * quarter) << 16) + (uint32_t)c0;
        f32x2 H[kEpiRuns / 2], L[kEpiRuns / 2];   // (hi, lo) of runs c0 + 2i, c0 + 2i + 1
        f32x2 Sp[kEpiRuns / 2], Tp[kEpiRuns / 2];  // the span's (s, t), added after the slots are freed
#pragma unroll
        for (int c = 0; c < kEpiRuns / 2; ++c) H[c] = L[c] = Sp[c] = Tp[c] = 0ull;
        bool ok = true;
        const int64_t M = 3 * N;
        int j = 0;   // span of this CTA
        Seg sg;
        for (int si = 0; ok && fix_segment(sc, si, sg); ++si) {
            const int nspan = (int)((sg.kb1 - 1) / kBlocksPerSpan - sg.kb0 / kBlocksPerSpan + 1);
            for (int js = 0; js < nspan; ++js, ++j) {
                ok = __all_sync(0xffffffffu, tc::mbar_wait(acc_full, j & 1) ? 1 : 0);
                if (!ok) {
                    if (lane == 0) atomicExch(err, 3);
                    break;
                }
                tc::tc_fence_after();
#pragma unroll
                for (int g = 0; g < kEpiRuns / 8; ++g) {
                    if (g * 8 < per) {
                        uint32_t r[kLevels][8];
#pragma unroll
                        for (int l = 0; l < kLevels; ++l) tc::tmem_ld8_nowait(tbase + (uint32_t)(l * Bq + g * 8), r[l]);
                        tc::tmem_wait_ld();
#pragma unroll
                        for (int x = 0; x < 8; x += 2) {
                            // levels 0-3 exactly (Fast2Sum on the nested grids), 4 and 5
                            // (2^-32, 2^-40) into the low part; two runs per instruction
                            f32x2 s, e0, e1, e2;
                            fast_two_sum2(pack2(r[0][x], r[0][x + 1]), pack2(r[1][x], r[1][x + 1]), s, e0);
                            fast_two_sum2(s, pack2(r[2][x], r[2][x + 1]), s, e1);
                            fast_two_sum2(s, pack2(r[3][x], r[3][x + 1]), s, e2);
                            Tp[(g * 8 + x) / 2] = add2(add2(add2(e0, e1), e2),
                                                       add2(pack2(r[4][x], r[4][x + 1]), pack2(r[5][x], r[5][x + 1])));
                            Sp[(g * 8 + x) / 2] = s;
                        }
                    }
                }
                tc::tc_fence_before();
                __syncwarp();
                if (lane == 0) tc::mbar_arrive(acc_empty);
                // (H, L) += (s, t) while the tensor cores fill the slots with the next span
#pragma unroll
                for (int c = 0; c < kEpiRuns / 2; ++c) {
                    if (2 * c < per) {
                        f32x2 S, E;
                        two_sum2(H[c], Sp[c], S, E);
                        E = add2(E, add2(L[c], Tp[c]));
                        const f32x2 Hn = add2(S, E);
                        L[c] = sub2(E, sub2(Hn, S));
                        H[c] = Hn;
                    }
                }
            }
            if (!ok) break;
            // the segment's sums: its slice; a balanced grid's tile end zeroes the slices above
            const int64_t m = sg.tile * kTileM + 32 * quarter + lane;
            if (m < M) {
#pragma unroll
                for (int c = 0; c < kEpiRuns; c += 2) {
                    const float2 h = unpack2(H[c / 2]), l = unpack2(L[c / 2]);
                    if (c < per && c0 + c < Bo) out[((int64_t)sg.slice * Bo + c0 + c) * M + m] = make_float2(h.x, l.x);
                    if (c + 1 < per && c0 + c + 1 < Bo)
                        out[((int64_t)sg.slice * Bo + c0 + c + 1) * M + m] = make_float2(h.y, l.y);
                }
                if (sg.tail)
                    for (int s2 = sg.slice + 1; s2 < sc.nsplit; ++s2)
                        for (int c = 0; c < per && c0 + c < Bo; ++c)
                            out[((int64_t)s2 * Bo + c0 + c) * M + m] = make_float2(0.f, 0.f);
            }
#pragma unroll
            for (int c = 0; c < kEpiRuns / 2; ++c) H[c] = L[c] = 0ull;
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

// right-hand side: one block of 128 threads per (256-column span, run), one
// cell per thread; v' from `v` ([B][2N] FP64) or from the stepper's slip rates
struct RhsSrc {
    const double *v;   // [B][2N] or null
    const double *slipv1, *slipv2, *cos_rake0, *sin_rake0;   // [B][N]
    double Vpl;
    const int64_t *order;   // position -> cell, or null (identity)
};

__global__ void __launch_bounds__(kSpan / 2) pack_rhs_fix_kernel(RhsSrc src, int64_t N, int B, int Bq,
                                                                  __nv_bfloat16 *__restrict__ out)
{
    __shared__ int red[kSpan / 64];
    const int64_t sp = blockIdx.x;
    const int r = blockIdx.y;
    const int i = threadIdx.x;
    const int64_t pos = sp * (kSpan / 2) + i;
    const int64_t KB = k_blocks(N);
    double v1 = 0.0, v2 = 0.0;
    if (r < B && pos < N) {
        const int64_t cell = src.order ? src.order[pos] : pos;
        const int64_t idx = (int64_t)r * N + cell;
        if (src.v) {
            v1 = src.v[(int64_t)r * 2 * N + 2 * cell];
            v2 = src.v[(int64_t)r * 2 * N + 2 * cell + 1];
        } else {
            v1 = fma(-src.Vpl, src.cos_rake0[idx], src.slipv1[idx]);
            v2 = fma(-src.Vpl, src.sin_rake0[idx], src.slipv2[idx]);
        }
    }
    int mx = rhs_word(v1, v2);
    for (int o = 16; o > 0; o >>= 1) mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if ((i & 31) == 0) red[i >> 5] = mx;
    __syncthreads();
    int m = red[0];
#pragma unroll
    for (int w = 1; w < kSpan / 64; ++w) m = max(m, red[w]);
    write_rhs_cell(out, Bq, KB, pos, r, rhs_span_exponent(m), v1, v2);
}

static int launch_pack_rhs(const RhsSrc &src, int64_t N, int B, void *Vpacked, cudaStream_t stream)
{
    const int Bq = fix_runs(B);
    dim3 grid((unsigned)k_spans(N), (unsigned)Bq);
    pack_rhs_fix_kernel<<<grid, kSpan / 2, 0, stream>>>(src, N, B, Bq, (__nv_bfloat16 *)Vpacked);
    PQ3D_CUDA_TRY(cudaGetLastError());
    return PQ3D_OK;
}

int pack_rhs_from_state(const double *slipv1, const double *slipv2, const double *cos_rake0, const double *sin_rake0,
                        double Vpl, const int64_t *order, int64_t N, int B, void *Vpacked, cudaStream_t stream)
{
    const RhsSrc src{nullptr, slipv1, slipv2, cos_rake0, sin_rake0, Vpl, order};
    return launch_pack_rhs(src, N, B, Vpacked, stream);
}

// ---------------------------------------------------------------------------
// launch

static size_t stage_bytes_for(int Bq) { return (size_t)kKPieces * kImageA + (size_t)kVPieces * Bq * kBlockK * 2; }

static int stages_for(int Bq, int *stages)
{
    int dev, maxs = 0;
    PQ3D_CUDA_TRY(cudaGetDevice(&dev));
    PQ3D_CUDA_TRY(cudaDeviceGetAttribute(&maxs, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    int s = (int)((maxs - 1024 - 64) / (stage_bytes_for(Bq) + 16));
    if (s > 6) s = 6;
    PQ3D_REQUIRE(s >= 2, "gemm_bf16x18: not enough shared memory for %d runs", Bq);
    static thread_local int cfg_dev = -1;
    if (cfg_dev != dev) {
        PQ3D_CUDA_TRY(cudaFuncSetAttribute(gemm_fix_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, maxs));
        cfg_dev = dev;
    }
    *stages = s;
    return PQ3D_OK;
}

int gemm_bf16x18(const void *Kpacked, const void *Vpacked, int64_t N, int B, int nsplit, float2 *out,
                 void *workspace, size_t workspace_bytes, cudaStream_t stream)
{
    PQ3D_REQUIRE(Kpacked && Vpacked && out && workspace, "gemm_bf16x18: null pointer");
    PQ3D_REQUIRE(N > 0, "gemm_bf16x18: N must be positive");
    PQ3D_REQUIRE(workspace_bytes >= 256 && aligned16(workspace), "gemm_bf16x18: workspace must be >= 256 bytes");
    PQ3D_REQUIRE(B >= 1 && B <= kMaxRuns, "gemm_bf16x18: B must be 1..%d", kMaxRuns);
    PQ3D_REQUIRE(aligned16(Kpacked) && aligned16(Vpacked) && aligned16(out),
                 "gemm_bf16x18: operands must be 16-byte aligned");
    const int64_t KB = k_blocks(N);
    PQ3D_REQUIRE(nsplit >= 1 && nsplit <= KB, "gemm_bf16x18: nsplit must be in [1, %lld]", (long long)KB);
    const int Bq = fix_runs(B), Bo = (B + 15) / 16 * 16;
    int stages;
    int rc = stages_for(Bq, &stages);
    if (rc) return rc;
    const size_t smem = (size_t)stages * stage_bytes_for(Bq) + 16 * (size_t)stages + 48;
    // the balanced grid (one CTA per SM, equal shares of the tile-major
    // blocks) when no tile meets more than nsplit CTAs' shares; else one CTA
    // per (tile, K slice)
    int dev, sms = 0;
    PQ3D_CUDA_TRY(cudaGetDevice(&dev));
    PQ3D_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const int64_t tiles = m_tiles(N), W = tiles * KB, G = sms;
    bool balanced = nsplit >= 2 && G >= 1 && W >= G;
    for (int64_t t = 0; balanced && t < tiles; ++t)
        balanced = bal_owner((t + 1) * KB - 1, W, G) - bal_owner(t * KB, W, G) + 1 <= nsplit;
    const FixSched sc{KB, balanced ? W : 0, nsplit};
    const dim3 grid = balanced ? dim3((unsigned)G) : dim3((unsigned)tiles, (unsigned)nsplit);
    gemm_fix_kernel<<<grid, kThreads, smem, stream>>>((const uint8_t *)Kpacked, (const uint8_t *)Vpacked, N, Bq, Bo,
                                                      sc, out, (int *)workspace, stages);
    PQ3D_CUDA_TRY(cudaGetLastError());
    return PQ3D_OK;
}

}  // namespace fx
}  // namespace pq3d

using namespace pq3d;

extern "C" size_t pq3d_batch_operator_fix_bytes(int64_t N) { return N > 0 ? fx::packed_operator_bytes(N) : 0; }

extern "C" size_t pq3d_batch_rhs_fix_bytes(int64_t N, int B)
{
    return N > 0 && B > 0 ? fx::packed_rhs_bytes(N, B) : 0;
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
    return fx::launch_pack_rhs(src, N, B, Vpacked, (cudaStream_t)stream);
}

extern "C" int pq3d_batch_gemm_bf16x18(const void *Kpacked, const void *Vpacked, int64_t N, int B, int nsplit,
                                       float *out, void *workspace, size_t workspace_bytes, void *stream)
{
    clear_error();
    return fx::gemm_bf16x18(Kpacked, Vpacked, N, B, nsplit, (float2 *)out, workspace, workspace_bytes,
                            (cudaStream_t)stream);
}
