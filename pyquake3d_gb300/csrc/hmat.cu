// H-matrix of the traction operator on the GPU: ACA compression of the
// admissible blocks, dense near-field blocks, and the product with B
// right-hand sides.
//
// Reference: src/Hmatrix.py -- partition 68-192 and 2077-2196 (restated on the
// host in pyquake3d_gb300/hmatrix.py), ACA 661-1344, product 1773-1866.
//
// Differences in method (stated):
//   * one ACA per block on the combined (3m x 2n) block of K (rows = receiver x
//     traction component, columns = source x slip direction), i.e. all six
//     reference operators at once, with partial pivoting and the relative
//     Frobenius stopping rule |u_k| |v_k| <= tol |S_k|_F (the reference runs one
//     ACA+ per slip direction, pivoting on the first component only, with an
//     absolute step tolerance and an unseeded random start);
//   * rows and columns are generated on the fly by the GF device math
//     (no host round trip per row), the first pivot row is row 0, ties in
//     argmax go to the smallest index -- deterministic;
//   * a block that has not converged at its rank cap is stored dense;
//   * factors and dense blocks are stored in FP32; products use FP32 FMAs
//     with the right-hand side split into FP32 hi + lo pieces (2 FMAs per
//     entry, FP32 sums over one block segment, FP64 beyond), accumulated per
//     output row in a fixed order (no atomics, the same result for a run alone
//     or in a batch).  The ACA tolerance (1e-4) dominates this rounding by
//     orders of magnitude.
//   * several right-hand sides run in one launch (one grid row per run); each
//     run streams the blocks itself (a single-pass multi-run product would
//     need a GEMM-style tiling of the near field; not done).
// Index space: elements are renumbered so that every cluster is a contiguous
// range (perm[p] = element at position p); a block is a pair of ranges.
#include <math.h>

#include "common.cuh"
#include "gf_device.cuh"
#include "hs_device.cuh"

namespace pq3d {
namespace hm {

using namespace ::pq3d::gf;

struct GSrc {   // source fields from the global structure-of-arrays table
    const double *base;
    int64_t stride;
    __device__ __forceinline__ double operator()(int f) const { return __ldg(base + f * stride); }
};

constexpr int kThreads = 256;

// The six tractions of pair (receiver record R, source element j): full
// space, or half space (image record and free-surface side table).
template <bool kHalf>
struct PairGen {
    const double *src, *img, *fsc;
    int64_t N;
    double nu, kf, two_mu, lam;
    __device__ __forceinline__ void operator()(int64_t j, const double *R, double ts[3], double td[3]) const
    {
        if (kHalf)
            pair_tractions_hs(GSrc{src + j, N}, GSrc{img + j, N}, GSrc{fsc + j, N}, R, nu, kf, two_mu, lam, ts, td);
        else
            pair_tractions(GSrc{src + j, N}, R, nu, kf, two_mu, lam, ts, td);
    }
};

__device__ __forceinline__ void block_argmax(double v, int idx, double *sv, int *si, double &best, int &bidx)
{
    // max |v| with the smallest index on ties; result broadcast to all threads
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const double ov = __shfl_xor_sync(0xffffffffu, v, o);
        const int oi = __shfl_xor_sync(0xffffffffu, idx, o);
        if (ov > v || (ov == v && oi < idx)) { v = ov; idx = oi; }
    }
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    __syncthreads();
    if (lane == 0) { sv[w] = v; si[w] = idx; }
    __syncthreads();
    best = sv[0];
    bidx = si[0];
    for (int q = 1; q < (int)(blockDim.x >> 5); ++q)
        if (sv[q] > best || (sv[q] == best && si[q] < bidx)) { best = sv[q]; bidx = si[q]; }
}

__device__ __forceinline__ double block_sum(double v, double *sv)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    __syncthreads();
    if (lane == 0) sv[w] = v;
    __syncthreads();
    double s = 0.0;
    for (int q = 0; q < (int)(blockDim.x >> 5); ++q) s += sv[q];
    return s;
}

// One CTA per admissible block.  U: kcap x M (row l = u_l), V: kcap x Nc.
// kAcaThreads per CTA (246 registers in full space: one CTA per SM).  Other
// shapes measured no better (N = 100,000, ACA launches: 1.28 s with 256
// threads; 128 and 64 threads with 2 and 4 CTAs per SM 1.55 s and 2.69 s --
// the residual updates, norms and pivot searches of an iteration scale with
// the CTA's threads; 256 threads capped at 128 registers for 2 CTAs per SM
// 1.34 s; 512 threads at 128 registers 1.26 s): the FP64 pipe, busy with the
// GF evaluations of the pivot rows and columns, sets the pace.
constexpr int kAcaThreads = 256;
constexpr int kAcaMinBlocks = 1;
template <bool kHalf>
__global__ void __launch_bounds__(kAcaThreads, kHalf ? 1 : kAcaMinBlocks)
aca_kernel(PairGen<kHalf> gen, const double *__restrict__ recv, const int64_t *__restrict__ perm,
           const int64_t *__restrict__ blk, const int32_t *__restrict__ kcap, double tol,
           double *__restrict__ UV, const int64_t *__restrict__ uv_off,
           uint8_t *__restrict__ used_ws, const int64_t *__restrict__ used_off, int32_t *__restrict__ rank_out,
           int32_t *__restrict__ status_out)
{
    __shared__ double sv[kAcaThreads / 32];
    __shared__ int si[kAcaThreads / 32];
    const int b = blockIdx.x;
    const int64_t r0 = blk[4 * b], r1 = blk[4 * b + 1], c0 = blk[4 * b + 2], c1 = blk[4 * b + 3];
    const int m = (int)(r1 - r0), n = (int)(c1 - c0);
    const int M = 3 * m, Nc = 2 * n;
    const int K = kcap[b];
    double *U = UV + uv_off[b];
    double *V = U + (int64_t)K * M;
    uint8_t *used = used_ws + used_off[b];
    const int t = threadIdx.x;
    double frob2 = 0.0;
    int k = 0, istar = 0, status = 1;
    int guard = 0;
    while (k < K && guard < M + K) {
        ++guard;
        // residual row istar (receiver p, component c) over all columns
        const int pr = istar / 3, cr = istar % 3;
        const double *R = recv + kRecvStride * perm[r0 + pr];
        double *v = V + (int64_t)k * Nc;
        for (int q = t; q < n; q += kAcaThreads) {
            double ts[3], td[3];
            gen(perm[c0 + q], R, ts, td);
            v[2 * q] = ts[cr];
            v[2 * q + 1] = td[cr];
        }
        __syncthreads();
        double best = 0.0;
        int jstar = 0;
        {
            double mv = -1.0;
            int mi = 0x7fffffff;
            for (int col = t; col < Nc; col += kAcaThreads) {
                double x = v[col];
                for (int l = 0; l < k; ++l) x -= U[(int64_t)l * M + istar] * V[(int64_t)l * Nc + col];
                v[col] = x;
                const double ax = fabs(x);
                if (ax > mv) { mv = ax; mi = col; }
            }
            block_argmax(mv, mi, sv, si, best, jstar);
        }
        if (t == 0) used[istar] = 1;
        __syncthreads();
        if (!(best > 0.0) || !isfinite(best)) {
            // row represented exactly (or not finite): next unused row, no new term
            if (!isfinite(best)) { status = 2; break; }
            int nxt = -1;
            for (int r = 0; r < M; ++r)
                if (!used[r]) { nxt = r; break; }
            if (nxt < 0) { status = 0; break; }
            istar = nxt;
            continue;
        }
        const double pivot = v[jstar];
        // residual column jstar (source q, slip s) over all rows, scaled by the pivot
        const int qc = jstar / 2, sc = jstar % 2;
        const int64_t jb = perm[c0 + qc];
        double *u = U + (int64_t)k * M;
        for (int p = t; p < m; p += kAcaThreads) {
            double ts[3], td[3];
            gen(jb, recv + kRecvStride * perm[r0 + p], ts, td);
            const double *tt = sc ? td : ts;
            u[3 * p] = tt[0];
            u[3 * p + 1] = tt[1];
            u[3 * p + 2] = tt[2];
        }
        __syncthreads();
        for (int row = t; row < M; row += kAcaThreads) {
            double x = u[row];
            for (int l = 0; l < k; ++l) x -= V[(int64_t)l * Nc + jstar] * U[(int64_t)l * M + row];
            u[row] = x / pivot;
        }
        __syncthreads();
        // norms: |S_k|^2 = |S_{k-1}|^2 + 2 sum_l (u.u_l)(v.v_l) + |u|^2 |v|^2
        double nu2 = 0.0, nv2 = 0.0;
        for (int row = t; row < M; row += kAcaThreads) nu2 += u[row] * u[row];
        for (int col = t; col < Nc; col += kAcaThreads) nv2 += v[col] * v[col];
        nu2 = block_sum(nu2, sv);
        nv2 = block_sum(nv2, sv);
        // the k cross products (u.u_l)(v.v_l): one warp per term l (warp
        // shuffles, no block barrier), then one block sum of the warps' parts
        double cross_w = 0.0;
        {
            const int w = t >> 5, lane = t & 31;
            for (int l = w; l < k; l += kAcaThreads / 32) {
                double du = 0.0, dv = 0.0;
                for (int row = lane; row < M; row += 32) du += u[row] * U[(int64_t)l * M + row];
                for (int col = lane; col < Nc; col += 32) dv += v[col] * V[(int64_t)l * Nc + col];
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) {
                    du += __shfl_xor_sync(0xffffffffu, du, o);
                    dv += __shfl_xor_sync(0xffffffffu, dv, o);
                }
                cross_w += du * dv;
            }
        }
        const double cross = block_sum((t & 31) == 0 ? cross_w : 0.0, sv);
        frob2 += 2.0 * cross + nu2 * nv2;
        ++k;
        if (sqrt(nu2 * nv2) <= tol * sqrt(fmax(frob2, 0.0))) { status = 0; break; }
        // next pivot row: largest |u| among unused rows
        double mv = -1.0;
        int mi = 0x7fffffff;
        for (int row = t; row < M; row += kAcaThreads) {
            const double ax = fabs(u[row]);
            if (!used[row] && ax > mv) { mv = ax; mi = row; }
        }
        double bv;
        int bi;
        block_argmax(mv, mi, sv, si, bv, bi);
        if (bv < 0.0) { status = 0; break; }   // every row used: exact
        istar = bi;
    }
    if (t == 0) {
        rank_out[b] = k;
        status_out[b] = status;
    }
}

// Storage of block b at data + off[b] (FP32, column-major so that the lanes
// of a warp read consecutive rows of one column):
//   dense:    D[col * M + row]                 (M = 3m rows, Nc = 2n columns)
//   low rank: U[l * M + row] for l < k, then V[l * Nc + col]   (K_b ~ U V)
// Rows are receiver x traction component (3p + c), columns source x slip
// direction (2q + s) in the block's local (renumbered) order.

// Dense blocks, one CTA per block; consecutive threads take consecutive
// receivers of one source.
template <bool kHalf>
__global__ void __launch_bounds__(kThreads)
dense_blocks_kernel(PairGen<kHalf> gen, const double *__restrict__ recv, const int64_t *__restrict__ perm,
                    const int64_t *__restrict__ blk, const int32_t *__restrict__ ids, float *__restrict__ D,
                    const int64_t *__restrict__ d_off)
{
    const int b = ids[blockIdx.x];
    const int64_t r0 = blk[4 * b], r1 = blk[4 * b + 1], c0 = blk[4 * b + 2], c1 = blk[4 * b + 3];
    const int m = (int)(r1 - r0), n = (int)(c1 - c0);
    const int64_t M = 3 * (int64_t)m;
    float *Db = D + d_off[b];
    for (int64_t e = threadIdx.x; e < (int64_t)m * n; e += kThreads) {
        const int q = (int)(e / m), p = (int)(e % m);
        double ts[3], td[3];
        gen(perm[c0 + q], recv + kRecvStride * perm[r0 + p], ts, td);
        float *col_s = Db + (int64_t)(2 * q) * M + 3 * p;
        float *col_d = col_s + M;
        for (int c = 0; c < 3; ++c) {
            col_s[c] = (float)ts[c];
            col_d[c] = (float)td[c];
        }
    }
}

// Copy the converged ACA factors (FP64, U as k rows of length M, then V as k
// rows of length Nc) to FP32 storage in the same order.
__global__ void pack_factors_kernel(const double *__restrict__ UV, const int64_t *__restrict__ uv_off,
                                    const int64_t *__restrict__ blk, const int32_t *__restrict__ kcap,
                                    const int32_t *__restrict__ rank, const int32_t *__restrict__ ids,
                                    float *__restrict__ out, const int64_t *__restrict__ out_off)
{
    const int b = ids[blockIdx.x];
    const int M = 3 * (int)(blk[4 * b + 1] - blk[4 * b]), Nc = 2 * (int)(blk[4 * b + 3] - blk[4 * b + 2]);
    const int k = rank[b], K = kcap[b];
    const double *U = UV + uv_off[b];
    const double *V = U + (int64_t)K * M;
    float *Uo = out + out_off[b];
    float *Vo = Uo + (int64_t)M * k;
    for (int64_t e = threadIdx.x; e < (int64_t)M * k; e += blockDim.x) Uo[e] = (float)U[e];
    for (int64_t e = threadIdx.x; e < (int64_t)k * Nc; e += blockDim.x) Vo[e] = (float)V[e];
}

// ---------------------------------------------------------------------------
// product  Y[r][3e + c] = sum over blocks of the H-matrix rows of element e
//
// Arithmetic: FP32 entries times the right-hand side split into FP32 hi + lo
// (2 FMAs per entry), FP32 partial sums over at most one block segment (or
// 1024 columns), then float-float (FF) sums; FP64 only for the final sum of a
// row's per-warp partials.

struct Acc2 {   // FP32 partial sum of one lane
    float s, c;
};

__device__ __forceinline__ void acc2_add(Acc2 &a, float k, float2 x)
{
    a.s = fmaf(k, x.x, a.s);
    a.c = fmaf(k, x.y, a.c);
}


// Float-float (unevaluated sum hi + lo) accumulation with FP32 operations
// only (Knuth's TwoSum), for the reductions of the low-rank product: GB300's
// FP64 rate is 1/64 of FP32, and an FP64 reduction per rank row made that
// kernel FP64-bound.
struct FF {
    float hi, lo;
};

__device__ __forceinline__ FF ff_add(FF a, FF b)
{
    const float s = __fadd_rn(a.hi, b.hi);
    const float bb = __fsub_rn(s, a.hi);
    const float e = __fadd_rn(__fsub_rn(a.hi, __fsub_rn(s, bb)), __fsub_rn(b.hi, bb));
    const float l = __fadd_rn(__fadd_rn(a.lo, b.lo), e);
    const float h = __fadd_rn(s, l);
    return FF{h, __fsub_rn(l, __fsub_rn(h, s))};
}

__device__ __forceinline__ FF warp_sum_ff(FF v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        FF w;
        w.hi = __shfl_xor_sync(0xffffffffu, v.hi, o);
        w.lo = __shfl_xor_sync(0xffffffffu, v.lo, o);
        v = ff_add(v, w);
    }
    return v;
}

__device__ __forceinline__ float2 split2(double x)
{
    const float h = (float)x;
    return make_float2(h, (float)(x - (double)h));
}

// X (FP64, [B][2N], element order) -> Xs ([B][2N] float (hi, lo) pairs, permuted order)
// run r takes part iff act == NULL or act[r * act_stride] != 0
__device__ __forceinline__ bool run_on(const int32_t *act, int act_stride, int r)
{
    return act == nullptr || act[(int64_t)r * act_stride] != 0;
}

__global__ void permute_split_kernel(const double *__restrict__ X, const int64_t *__restrict__ perm, int64_t N, int B,
                                     float2 *__restrict__ Xs, const int32_t *act, int act_stride)
{
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int r = blockIdx.y;
    if (i >= 2 * N || r >= B || !run_on(act, act_stride, r)) return;
    const int64_t q = i >> 1;
    Xs[(int64_t)r * 2 * N + i] = split2(X[(int64_t)r * 2 * N + 2 * perm[q] + (i & 1)]);
}

// T[w * B + r] = V_b[l] . x_r[cols of b] as an FP32 (hi, lo) pair for rank
// row w (row l of low-rank block b).  Two work lists, built by the host with
// the split at 8,192 columns.  The shorter rows come in groups of up to 4
// consecutive rows of one block (t_grp: one 16-byte record per group holding
// the first row's storage offset, first x column and length, the first rank
// row and the group size), kTGroupsPerWarp consecutive groups per warp: the
// warp loads the next group's record while it streams the current group, so
// no dependent descriptor load sits between two groups, and consecutive
// groups of one block find their x values in L1.  The longer rows (t_sched
// tail, t_info records) take one CTA each with the columns cut into kTWarps
// contiguous pieces (a warp streams only a few KB in flight, so a long row on
// one warp would be the tail) and the partial sums added in warp order.
// Runs are the fastest-varying part of the block index, so the B CTAs that
// read the same factor rows run together and share them in L2.
constexpr int kTWarps = 4;
constexpr int kTGroupsPerWarp = 2;

__device__ __forceinline__ FF t_row_part(const float *__restrict__ v, const float2 *__restrict__ x, int c_begin,
                                         int c_end, int lane)
{
    FF sum{0.f, 0.f};
    for (int c0k = c_begin; c0k < c_end; c0k += 1024) {
        const int cend = min(c_end, c0k + 1024);
        Acc2 a0{0.f, 0.f}, a1{0.f, 0.f};
        int col = c0k + lane;
        // 16 columns per lane in flight: an average rank row (~630 columns)
        // is one or two rounds
        for (; col + 480 < cend; col += 512) {
            float k[16];
            float2 xv[16];
#pragma unroll
            for (int u = 0; u < 16; ++u) {
                k[u] = __ldg(v + col + 32 * u);
                xv[u] = x[col + 32 * u];
            }
#pragma unroll
            for (int u = 0; u < 16; u += 2) {
                acc2_add(a0, k[u], xv[u]);
                acc2_add(a1, k[u + 1], xv[u + 1]);
            }
        }
        for (; col + 96 < cend; col += 128) {
            float k[4];
            float2 xv[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                k[u] = __ldg(v + col + 32 * u);
                xv[u] = x[col + 32 * u];
            }
            acc2_add(a0, k[0], xv[0]);
            acc2_add(a1, k[1], xv[1]);
            acc2_add(a0, k[2], xv[2]);
            acc2_add(a1, k[3], xv[3]);
        }
        for (; col < cend; col += 32) acc2_add(a0, __ldg(v + col), x[col]);
        // the hi and lo parts of the FP32 partial sums of this chunk
        sum = ff_add(sum, FF{a0.s, 0.f});
        sum = ff_add(sum, FF{a1.s, 0.f});
        sum = ff_add(sum, FF{__fadd_rn(a0.c, a1.c), 0.f});
    }
    return warp_sum_ff(sum);
}

// Up to 4 consecutive short rank rows of one block on one warp: the rows
// share their x values, so a lane loads x once per column for all of them and
// keeps 8 columns of every row in flight; a warp therefore moves ~4x the bytes
// per memory round trip of a one-row walk (the ~630-column rows were bound by
// their round trips).  Row j starts at v + j * nc.  Columns beyond the end
// are predicated off (zero terms); partial sums move to float-float every
// 1024 columns.
__device__ __forceinline__ void t_row_group(const float *__restrict__ v, int nc, int g, const float2 *__restrict__ x,
                                            int lane, FF (&out)[4])
{
    FF sum[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) sum[j] = FF{0.f, 0.f};
    for (int c0k = 0; c0k < nc; c0k += 1024) {
        Acc2 a[4];   // one FMA chain pair per row: the 4 rows give the pipeline its independent chains
#pragma unroll
        for (int j = 0; j < 4; ++j) a[j] = Acc2{0.f, 0.f};
        const int cend = min(nc, c0k + 1024);
        for (int col = c0k + lane; col - lane < cend; col += 256) {
            float2 xv[8];
            float k[4][8];
#pragma unroll
            for (int u = 0; u < 8; ++u) {
                const int c = col + 32 * u;
                const bool ok = c < cend;
                xv[u] = ok ? x[c] : make_float2(0.f, 0.f);
#pragma unroll
                for (int j = 0; j < 4; ++j) k[j][u] = (ok && j < g) ? __ldg(v + (int64_t)j * nc + c) : 0.f;
            }
#pragma unroll
            for (int u = 0; u < 8; ++u)
#pragma unroll
                for (int j = 0; j < 4; ++j) acc2_add(a[j], k[j][u], xv[u]);
        }
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            sum[j] = ff_add(sum[j], FF{a[j].s, 0.f});
            sum[j] = ff_add(sum[j], FF{a[j].c, 0.f});
        }
    }
#pragma unroll
    for (int j = 0; j < 4; ++j) out[j] = warp_sum_ff(sum[j]);
}

__global__ void __launch_bounds__(kTWarps * 32, 6)
lowrank_T_kernel(const float *__restrict__ data, const longlong2 *__restrict__ t_info,
                 const int32_t *__restrict__ t_sched, const longlong2 *__restrict__ t_grp, int64_t ngrp,
                 int64_t nshort, int64_t nlong, int64_t short_ctas,
                 const float2 *__restrict__ Xs, int64_t N, int B, float2 *__restrict__ T, const int32_t *act,
                 int act_stride)
{
    __shared__ FF part[kTWarps];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int r = (int)(blockIdx.x % (unsigned)B);
    const int64_t cta = blockIdx.x / (unsigned)B;
    if (!run_on(act, act_stride, r)) return;   // uniform per CTA
    const float2 *xr = Xs + (int64_t)r * 2 * N;
    if (cta < short_ctas) {
        const int64_t g0 = (cta * kTWarps + wid) * kTGroupsPerWarp;
        if (g0 >= ngrp) return;
        const int64_t g1 = min(ngrp, g0 + kTGroupsPerWarp);
        // record of group gi: .x = V offset | row length << 40 | size << 56,
        // .y = first x column | first rank row << 32
        longlong2 nrec = t_grp[g0];
        for (int64_t gi = g0; gi < g1; ++gi) {
            const longlong2 rec = nrec;
            if (gi + 1 < g1) nrec = t_grp[gi + 1];
            const int64_t off = rec.x & ((1ll << 40) - 1);
            const int nc = (int)((rec.x >> 40) & 0xffff), g = (int)(rec.x >> 56);
            const int64_t w0 = (int64_t)((uint64_t)rec.y >> 32);
            FF sg[4];
            t_row_group(data + off, nc, g, xr + (int32_t)(rec.y & 0xffffffffll), lane, sg);
            if (lane == 0)
                for (int j = 0; j < g; ++j) T[(w0 + j) * (int64_t)B + r] = make_float2(sg[j].hi, sg[j].lo);
        }
        return;
    }
    const int64_t q = cta - short_ctas;
    if (q >= nlong) return;   // uniform per CTA
    const int w = t_sched[nshort + q];
    const longlong2 info = t_info[w];
    const int Nc = (int)(info.y >> 32);
    const int piece = (Nc / kTWarps + 31) / 32 * 32;
    const int c_begin = min(Nc, wid * piece), c_end = min(Nc, (wid + 1) * piece);
    const FF s = t_row_part(data + info.x, xr + (int32_t)(info.y & 0xffffffffll), c_begin, c_end, lane);
    if (lane == 0) part[wid] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        FF t = part[0];
        for (int k = 1; k < kTWarps; ++k) t = ff_add(t, part[k]);
        T[w * (int64_t)B + r] = make_float2(t.hi, t.lo);
    }
}

// One CTA per (leaf row cluster, run), the run fastest in the block index so
// that the B CTAs of one leaf read its blocks together (L2 reuse).
//
// Lane j of every warp owns rows j, j + 32, ... of the leaf (up to kPassRows
// rows per pass).  The work of the leaf -- the columns of its dense blocks and
// the rank columns of its low-rank blocks, in list order -- is cut into 8
// contiguous ranges, one per warp; a warp walks its range column by column
// (a coalesced 128-byte load per 32 rows, the column's x value broadcast),
// and the 8 per-warp partial sums of a row are added in warp order through
// shared memory.  The result does not depend on B or on timing.
struct BlkDesc {
    int64_t off;    // storage offset (floats)
    int64_t x0;     // dense: first column in Xs (2 c0); low rank: first T row (t_off)
    int32_t row0;   // first local row of this leaf in the block
    int32_t M;      // rows of the block (column stride)
    int32_t w;      // work columns: Nc (dense) or k (low rank)
    int32_t dense;
};

constexpr int kMaxLeafBlocks = 160;
constexpr int kWarps = kThreads / 32;
constexpr int kMaxR = 6;
constexpr int kPassRows = 32 * kMaxR;

template <int R>
__device__ __forceinline__ void leaf_segment(const float *__restrict__ col0, int64_t M, const float2 *__restrict__ xp,
                                             int64_t xs, int ca, int cb, bool last_ok, FF (&acc)[kMaxR])
{
    constexpr int U = 4;   // columns in flight per warp
    Acc2 a[R];
#pragma unroll
    for (int i = 0; i < R; ++i) a[i] = Acc2{0.f, 0.f};
    int c = ca;
    for (; c + U <= cb; c += U) {
        float k[U][R];
        float2 x[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const float *p = col0 + (int64_t)(c + u) * M;
            x[u] = xp[(int64_t)(c + u) * xs];
#pragma unroll
            for (int i = 0; i < R; ++i) {
                const bool ok = (i < R - 1) || last_ok;
                k[u][i] = ok ? __ldg(p + 32 * i) : 0.f;
            }
        }
#pragma unroll
        for (int u = 0; u < U; ++u)
#pragma unroll
            for (int i = 0; i < R; ++i) acc2_add(a[i], k[u][i], x[u]);
    }
    for (; c < cb; ++c) {
        const float *p0 = col0 + (int64_t)c * M;
        const float2 x0 = xp[(int64_t)c * xs];
#pragma unroll
        for (int i = 0; i < R; ++i) {
            const bool ok = (i < R - 1) || last_ok;
            acc2_add(a[i], ok ? __ldg(p0 + 32 * i) : 0.f, x0);
        }
    }
#pragma unroll
    for (int i = 0; i < R; ++i) {
        acc[i] = ff_add(acc[i], FF{a[i].s, 0.f});
        acc[i] = ff_add(acc[i], FF{a[i].c, 0.f});
    }
}

template <int R>
__device__ __forceinline__ void leaf_range(const BlkDesc *desc, const int *wpre, int nq, int64_t lo, int64_t hi, int pr0, int prow,
                           const float *__restrict__ data, const float2 *__restrict__ xr,
                           const float2 *__restrict__ T, int B, int r, FF (&acc)[kMaxR])
{
    const int lane = threadIdx.x & 31;
    const bool last_ok = lane + 32 * (R - 1) < prow;
    // first descriptor whose range ends after lo
    int q = 0;
    while (q < nq && wpre[q + 1] <= lo) ++q;
    for (; q < nq && wpre[q] < hi; ++q) {
        const BlkDesc d = desc[q];
        const int ca = (int)max((int64_t)0, lo - wpre[q]);
        const int cb = (int)min((int64_t)d.w, hi - wpre[q]);
        if (ca >= cb) continue;
        const float *col0 = data + d.off + d.row0 + pr0 + lane;
        if (d.dense) leaf_segment<R>(col0, d.M, xr + d.x0, 1, ca, cb, last_ok, acc);
        else leaf_segment<R>(col0, d.M, T + d.x0 * B + r, B, ca, cb, last_ok, acc);
    }
}

__global__ void __launch_bounds__(kThreads, 3)
leaf_rows_kernel(const float *__restrict__ data, const int64_t *__restrict__ off, const int64_t *__restrict__ blk,
                 const int32_t *__restrict__ rank, const int64_t *__restrict__ leaf, const int64_t *__restrict__ leaf_ptr,
                 const int32_t *__restrict__ leaf_blocks, const int64_t *__restrict__ perm, const float2 *__restrict__ Xs,
                 const float2 *__restrict__ T, const int64_t *__restrict__ t_off, int64_t N, int B,
                 double *__restrict__ Y, const int32_t *act, int act_stride)
{
    __shared__ BlkDesc desc[kMaxLeafBlocks];
    __shared__ int wpre[kMaxLeafBlocks + 1];
    __shared__ double red[kWarps][kPassRows];
    const int L = (int)(blockIdx.x / (unsigned)B), r = (int)(blockIdx.x % (unsigned)B);
    if (!run_on(act, act_stride, r)) return;   // uniform per CTA: before any barrier
    const int64_t p0 = leaf[2 * L], p1 = leaf[2 * L + 1];
    const int rows = 3 * (int)(p1 - p0);
    const int64_t q0 = leaf_ptr[L], q1 = leaf_ptr[L + 1];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const float2 *xr = Xs + (int64_t)r * 2 * N;
    double *Yr = Y + (int64_t)r * 3 * N;
    for (int pr0 = 0; pr0 < rows; pr0 += kPassRows) {
        const int prow = min(kPassRows, rows - pr0);
        const int R = (prow + 31) / 32;
        FF acc[kMaxR];
#pragma unroll
        for (int i = 0; i < kMaxR; ++i) acc[i] = FF{0.f, 0.f};
        for (int64_t qs = q0; qs < q1; qs += kMaxLeafBlocks) {
            const int nq = (int)min((int64_t)kMaxLeafBlocks, q1 - qs);
            __syncthreads();
            for (int i = threadIdx.x; i < nq; i += kThreads) {
                const int bb = leaf_blocks[qs + i];
                const int64_t r0 = blk[4 * bb], c0 = blk[4 * bb + 2];
                const int k = rank[bb];
                BlkDesc d;
                d.off = off[bb];
                d.row0 = 3 * (int)(p0 - r0);
                d.M = 3 * (int)(blk[4 * bb + 1] - r0);
                d.dense = k < 0;
                d.w = k < 0 ? 2 * (int)(blk[4 * bb + 3] - c0) : k;
                d.x0 = k < 0 ? 2 * c0 : t_off[bb];
                desc[i] = d;
            }
            __syncthreads();
            if (threadIdx.x == 0) {
                int s = 0;
                for (int i = 0; i < nq; ++i) { wpre[i] = s; s += desc[i].w; }
                wpre[nq] = s;
            }
            __syncthreads();
            const int64_t W = wpre[nq];
            const int64_t lo = W * wid / kWarps, hi = W * (wid + 1) / kWarps;
            switch (R) {
                case 1: leaf_range<1>(desc, wpre, nq, lo, hi, pr0, prow, data, xr, T, B, r, acc); break;
                case 2: leaf_range<2>(desc, wpre, nq, lo, hi, pr0, prow, data, xr, T, B, r, acc); break;
                case 3: leaf_range<3>(desc, wpre, nq, lo, hi, pr0, prow, data, xr, T, B, r, acc); break;
                case 4: leaf_range<4>(desc, wpre, nq, lo, hi, pr0, prow, data, xr, T, B, r, acc); break;
                case 5: leaf_range<5>(desc, wpre, nq, lo, hi, pr0, prow, data, xr, T, B, r, acc); break;
                default: leaf_range<6>(desc, wpre, nq, lo, hi, pr0, prow, data, xr, T, B, r, acc); break;
            }
        }
        __syncthreads();
#pragma unroll
        for (int i = 0; i < kMaxR; ++i) red[wid][lane + 32 * i] = (double)acc[i].hi + (double)acc[i].lo;
        __syncthreads();
        for (int lr = threadIdx.x; lr < prow; lr += kThreads) {
            double s = 0.0;
#pragma unroll
            for (int w = 0; w < kWarps; ++w) s += red[w][lr];
            const int row = pr0 + lr;
            Yr[3 * perm[p0 + row / 3] + row % 3] = s;
        }
    }
}

}  // namespace hm
}  // namespace pq3d

using namespace pq3d;
using namespace pq3d::hm;

static inline double poisson_(double mu, double lam) { return 1.0 / (1.0 + lam / mu) / 2.0; }

// Table layout written by pq3d_gf_setup: source [kSrcStride][N], receiver
// [N][kRecvStride], image [kImgStride][N], side table [kFscStride][N].
template <bool kHalf>
static PairGen<kHalf> make_gen(const double *tables, int64_t N, double mu, double lambda_)
{
    const double nu = poisson_(mu, lambda_);
    const double *img = tables + (size_t)(kSrcStride + kRecvStride) * N;
    return PairGen<kHalf>{tables, img, img + (size_t)kImgStride * N, N, nu, 1.0 / (8.0 * kPi * (1.0 - nu)),
                          2.0 * mu, lambda_};
}

extern "C" int pq3d_hmat_aca(const double *tables, int64_t N, const int64_t *perm, int nblocks, const int64_t *blk,
                             const int32_t *kcap, double tol, double mu, double lambda_, int halfspace, double *UV,
                             const int64_t *uv_off, uint8_t *used, const int64_t *used_off, int32_t *rank,
                             int32_t *status, void *stream)
{
    clear_error();
    PQ3D_REQUIRE(tables && perm && blk && kcap && UV && uv_off && used && used_off && rank && status && N > 0,
                 "pq3d_hmat_aca: bad arguments");
    if (nblocks <= 0) return PQ3D_OK;
    const double *recv = tables + (size_t)kSrcStride * N;
    cudaStream_t st = (cudaStream_t)stream;
    if (halfspace)
        aca_kernel<true><<<nblocks, kAcaThreads, 0, st>>>(make_gen<true>(tables, N, mu, lambda_), recv, perm, blk, kcap,
                                                       tol, UV, uv_off, used, used_off, rank, status);
    else
        aca_kernel<false><<<nblocks, kAcaThreads, 0, st>>>(make_gen<false>(tables, N, mu, lambda_), recv, perm, blk,
                                                        kcap, tol, UV, uv_off, used, used_off, rank, status);
    PQ3D_CUDA_TRY(cudaGetLastError());
    return PQ3D_OK;
}

extern "C" int pq3d_hmat_dense_blocks(const double *tables, int64_t N, const int64_t *perm, const int64_t *blk,
                                      const int32_t *ids, int nids, double mu, double lambda_, int halfspace,
                                      float *D, const int64_t *d_off, void *stream)
{
    clear_error();
    PQ3D_REQUIRE(tables && perm && blk && ids && D && d_off && N > 0, "pq3d_hmat_dense_blocks: bad arguments");
    PQ3D_REQUIRE(((uintptr_t)D & 3u) == 0, "pq3d_hmat_dense_blocks: D must be 4-byte aligned");
    if (nids <= 0) return PQ3D_OK;
    const double *recv = tables + (size_t)kSrcStride * N;
    cudaStream_t st = (cudaStream_t)stream;
    if (halfspace)
        dense_blocks_kernel<true><<<nids, kThreads, 0, st>>>(make_gen<true>(tables, N, mu, lambda_), recv, perm, blk,
                                                             ids, D, d_off);
    else
        dense_blocks_kernel<false><<<nids, kThreads, 0, st>>>(make_gen<false>(tables, N, mu, lambda_), recv, perm,
                                                              blk, ids, D, d_off);
    PQ3D_CUDA_TRY(cudaGetLastError());
    return PQ3D_OK;
}

extern "C" int pq3d_hmat_pack_factors(const double *UV, const int64_t *uv_off, const int64_t *blk, const int32_t *kcap,
                                      const int32_t *rank, const int32_t *ids, int nids, float *out,
                                      const int64_t *out_off, void *stream)
{
    clear_error();
    if (nids <= 0) return PQ3D_OK;
    pack_factors_kernel<<<nids, 256, 0, (cudaStream_t)stream>>>(UV, uv_off, blk, kcap, rank, ids, out, out_off);
    PQ3D_CUDA_TRY(cudaGetLastError());
    return PQ3D_OK;
}

extern "C" int pq3d_hmat_apply_masked(const pq3d_hmat *H, const double *X, int B, double *Y,
                                      const int32_t *run_active, int active_stride, void *workspace,
                                      size_t workspace_bytes, void *stream)
{
    clear_error();
    PQ3D_REQUIRE(H && X && Y && workspace && B >= 1, "pq3d_hmat_apply: bad arguments");
    const int64_t N = H->N;
    const size_t need = (size_t)B * 2 * N * sizeof(float2) + (size_t)H->t_rows * B * sizeof(float2);
    PQ3D_REQUIRE(workspace_bytes >= need && aligned16(workspace), "pq3d_hmat_apply: workspace too small (%zu < %zu)",
                 workspace_bytes, need);
    cudaStream_t st = (cudaStream_t)stream;
    float2 *Xs = (float2 *)workspace;
    float2 *T = (float2 *)((char *)workspace + (size_t)B * 2 * N * sizeof(float2));
    dim3 g1((unsigned)((2 * N + 255) / 256), (unsigned)B);
    permute_split_kernel<<<g1, 256, 0, st>>>(X, H->perm, N, B, Xs, run_active, active_stride);
    // all runs in one launch, run fastest in the block index; a run's result
    // does not depend on B
    if (H->t_rows > 0) {
        const int64_t nshort = H->t_rows - H->t_nlong;
        const int64_t short_ctas = (H->t_ngrp + kTWarps * kTGroupsPerWarp - 1) / (kTWarps * kTGroupsPerWarp);
        const int64_t nT = (short_ctas + H->t_nlong) * B;
        PQ3D_REQUIRE(nT < (int64_t)INT32_MAX, "pq3d_hmat_apply: too many rank rows x runs");
        lowrank_T_kernel<<<(unsigned)nT, kTWarps * 32, 0, st>>>(H->data, (const longlong2 *)H->t_info, H->t_sched,
                                                               (const longlong2 *)H->t_grp,
                                                       H->t_ngrp, nshort,
                                                       H->t_nlong, short_ctas, Xs, N, B, T, run_active,
                                                       active_stride);
    }
    PQ3D_REQUIRE((int64_t)H->nleaves * B < (int64_t)INT32_MAX, "pq3d_hmat_apply: too many leaves x runs");
    const unsigned gL = (unsigned)(H->nleaves * B);
    leaf_rows_kernel<<<gL, kThreads, 0, st>>>(H->data, H->off, H->blk, H->rank, H->leaf, H->leaf_ptr, H->leaf_blocks,
                                              H->perm, Xs, T, H->t_off, N, B, Y, run_active, active_stride);
    PQ3D_CUDA_TRY(cudaGetLastError());
    return PQ3D_OK;
}

extern "C" int pq3d_hmat_apply(const pq3d_hmat *H, const double *X, int B, double *Y, void *workspace,
                               size_t workspace_bytes, void *stream)
{
    return pq3d_hmat_apply_masked(H, X, B, Y, nullptr, 0, workspace, workspace_bytes, stream);
}

extern "C" size_t pq3d_hmat_workspace_bytes(const pq3d_hmat *H, int B)
{
    if (!H || B < 1) return 0;
    return (size_t)B * 2 * H->N * sizeof(float2) + (size_t)H->t_rows * B * sizeof(float2);
}
