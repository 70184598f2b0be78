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
//     entry, per-lane FP32 sums, FP64 across lanes), accumulated per output
//     row in a fixed block order (no atomics, the same result for a run alone
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

namespace pq3d {
namespace hm {

using namespace ::pq3d::gf;

struct GSrc {   // source fields from the global structure-of-arrays table
    const double *base;
    int64_t stride;
    __device__ __forceinline__ double operator()(int f) const { return __ldg(base + f * stride); }
};

constexpr int kThreads = 256;

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
__global__ void __launch_bounds__(kThreads)
aca_kernel(const double *__restrict__ src, const double *__restrict__ recv, int64_t N, const int64_t *__restrict__ perm,
           const int64_t *__restrict__ blk, const int32_t *__restrict__ kcap, double tol, double nu, double kf,
           double two_mu, double lam, double *__restrict__ UV, const int64_t *__restrict__ uv_off,
           uint8_t *__restrict__ used_ws, const int64_t *__restrict__ used_off, int32_t *__restrict__ rank_out,
           int32_t *__restrict__ status_out)
{
    __shared__ double sv[kThreads / 32];
    __shared__ int si[kThreads / 32];
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
        for (int q = t; q < n; q += kThreads) {
            const int64_t j = perm[c0 + q];
            double ts[3], td[3];
            pair_tractions(GSrc{src + j, N}, R, nu, kf, two_mu, lam, ts, td);
            v[2 * q] = ts[cr];
            v[2 * q + 1] = td[cr];
        }
        __syncthreads();
        double best = 0.0;
        int jstar = 0;
        {
            double mv = -1.0;
            int mi = 0x7fffffff;
            for (int col = t; col < Nc; col += kThreads) {
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
        const double *Fb = src + perm[c0 + qc];
        double *u = U + (int64_t)k * M;
        for (int p = t; p < m; p += kThreads) {
            double ts[3], td[3];
            pair_tractions(GSrc{Fb, N}, recv + kRecvStride * perm[r0 + p], nu, kf, two_mu, lam, ts, td);
            const double *tt = sc ? td : ts;
            u[3 * p] = tt[0];
            u[3 * p + 1] = tt[1];
            u[3 * p + 2] = tt[2];
        }
        __syncthreads();
        for (int row = t; row < M; row += kThreads) {
            double x = u[row];
            for (int l = 0; l < k; ++l) x -= V[(int64_t)l * Nc + jstar] * U[(int64_t)l * M + row];
            u[row] = x / pivot;
        }
        __syncthreads();
        // norms: |S_k|^2 = |S_{k-1}|^2 + 2 sum_l (u.u_l)(v.v_l) + |u|^2 |v|^2
        double nu2 = 0.0, nv2 = 0.0;
        for (int row = t; row < M; row += kThreads) nu2 += u[row] * u[row];
        for (int col = t; col < Nc; col += kThreads) nv2 += v[col] * v[col];
        nu2 = block_sum(nu2, sv);
        nv2 = block_sum(nv2, sv);
        double cross = 0.0;
        for (int l = 0; l < k; ++l) {
            double du = 0.0, dv = 0.0;
            for (int row = t; row < M; row += kThreads) du += u[row] * U[(int64_t)l * M + row];
            for (int col = t; col < Nc; col += kThreads) dv += v[col] * V[(int64_t)l * Nc + col];
            du = block_sum(du, sv);
            dv = block_sum(dv, sv);
            cross += du * dv;
        }
        frob2 += 2.0 * cross + nu2 * nv2;
        ++k;
        if (sqrt(nu2 * nv2) <= tol * sqrt(fmax(frob2, 0.0))) { status = 0; break; }
        // next pivot row: largest |u| among unused rows
        double mv = -1.0;
        int mi = 0x7fffffff;
        for (int row = t; row < M; row += kThreads) {
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

// Dense blocks: block b stored row-major (3m x 2n) FP32 at d_off[b]; d_off[b]
// must be a multiple of 2 floats (float2 stores; the host pads to 4).
__global__ void __launch_bounds__(kThreads)
dense_blocks_kernel(const double *__restrict__ src, const double *__restrict__ recv, int64_t N,
                    const int64_t *__restrict__ perm, const int64_t *__restrict__ blk, const int32_t *__restrict__ ids,
                    double nu, double kf, double two_mu, double lam, float *__restrict__ D,
                    const int64_t *__restrict__ d_off)
{
    const int b = ids[blockIdx.x];
    const int64_t r0 = blk[4 * b], r1 = blk[4 * b + 1], c0 = blk[4 * b + 2], c1 = blk[4 * b + 3];
    const int m = (int)(r1 - r0), n = (int)(c1 - c0);
    float *Db = D + d_off[b];
    for (int64_t e = threadIdx.x; e < (int64_t)m * n; e += kThreads) {
        const int p = (int)(e / n), q = (int)(e % n);
        double ts[3], td[3];
        pair_tractions(GSrc{src + perm[c0 + q], N}, recv + kRecvStride * perm[r0 + p], nu, kf, two_mu, lam, ts, td);
        for (int c = 0; c < 3; ++c)
            *reinterpret_cast<float2 *>(Db + (int64_t)(3 * p + c) * 2 * n + 2 * q) = make_float2((float)ts[c], (float)td[c]);
    }
}

// Copy the converged ACA factors to FP32 storage: U_b (3m x k) row-major, V_b (k x 2n).
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
    for (int64_t e = threadIdx.x; e < (int64_t)M * k; e += blockDim.x) {
        const int row = (int)(e / k), l = (int)(e % k);
        Uo[e] = (float)U[(int64_t)l * M + row];
    }
    for (int64_t e = threadIdx.x; e < (int64_t)k * Nc; e += blockDim.x) Vo[e] = (float)V[e];
}

// ---------------------------------------------------------------------------
// product  Y[r][3e + c] = sum over blocks of the H-matrix rows of element e

struct Acc2 {   // FP32 partial sum of one lane
    float s, c;
};

__device__ __forceinline__ void acc2_add(Acc2 &a, float k, float vh, float vl)
{
    a.s = fmaf(k, vh, a.s);
    a.c = fmaf(k, vl, a.c);
}

__device__ __forceinline__ double warp_sum(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// X (FP64, [B][2N], element order) -> Xs ([B][2N] float (hi, lo) pairs, permuted order)
__global__ void permute_split_kernel(const double *__restrict__ X, const int64_t *__restrict__ perm, int64_t N, int B,
                                     float2 *__restrict__ Xs)
{
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int r = blockIdx.y;
    if (i >= 2 * N || r >= B) return;
    const int64_t q = i >> 1;
    const double x = X[(int64_t)r * 2 * N + 2 * perm[q] + (i & 1)];
    const float h = (float)x;
    Xs[(int64_t)r * 2 * N + i] = make_float2(h, (float)(x - (double)h));
}

// T[(t_off[b] + l) * B + r] = V_b[l] . x_r[cols of b]; one warp per (block,
// rank row).  Runs are the fastest-varying part of the block index, so the B
// CTAs that read the same factor rows run together and share them in L2.
__global__ void lowrank_T_kernel(const float *__restrict__ data, const int64_t *__restrict__ off,
                                 const int64_t *__restrict__ blk, const int32_t *__restrict__ rank,
                                 const int32_t *__restrict__ lr_ids, const int64_t *__restrict__ lr_row0, int nlr_rows,
                                 const float2 *__restrict__ Xs, int64_t N, int B, double *__restrict__ T,
                                 const int64_t *__restrict__ t_off)
{
    const int lane = threadIdx.x & 31;
    const int r = (int)(blockIdx.x % (unsigned)B);
    const int64_t w = ((blockIdx.x / (unsigned)B) * (int64_t)blockDim.x + threadIdx.x) >> 5;
    if (w >= nlr_rows) return;
    // locate (block, l): lr_row0 = [count, prefix sums of the ranks of the
    // low-rank blocks (count + 1 values)]; find the last block starting <= w
    const int nlr = (int)lr_row0[0];
    int lo = 0, hi = nlr;
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (lr_row0[1 + mid] <= w) lo = mid; else hi = mid;
    }
    const int b = lr_ids[lo];
    const int l = (int)(w - lr_row0[1 + lo]);
    const int k = rank[b];
    const int64_t c0 = blk[4 * b + 2];
    const int Nc = 2 * (int)(blk[4 * b + 3] - c0);
    const int M = 3 * (int)(blk[4 * b + 1] - blk[4 * b]);
    const float *v = data + off[b] + (int64_t)M * k + (int64_t)l * Nc;
    const float2 *x = Xs + (int64_t)r * 2 * N + 2 * c0;
    Acc2 a{0.f, 0.f};
    for (int col = lane; col < Nc; col += 32) {
        const float2 xv = x[col];
        acc2_add(a, __ldg(v + col), xv.x, xv.y);
    }
    const double sum = warp_sum((double)a.s + (double)a.c);
    if (lane == 0) T[(t_off[b] + l) * (int64_t)B + r] = sum;
}

// One CTA per (leaf row cluster, run), the run fastest in the block index so
// that the B CTAs of one leaf read its blocks together (L2 reuse).  The descriptors
// of the leaf's blocks are staged in shared memory; every warp owns groups of
// 4 consecutive output rows and adds the blocks of the leaf in list order.
struct BlkDesc {
    int64_t off, c0, row0;   // storage offset (floats), first column element, first local row of this leaf
    int64_t t0;              // first rank row in T
    int32_t Nc, k;           // columns (2n), rank (-1 dense)
};

constexpr int kMaxLeafBlocks = 160;
constexpr int kRowsPerWarp = 4;

__global__ void __launch_bounds__(kThreads)
leaf_rows_kernel(const float *__restrict__ data, const int64_t *__restrict__ off, const int64_t *__restrict__ blk,
                 const int32_t *__restrict__ rank, const int64_t *__restrict__ leaf, const int64_t *__restrict__ leaf_ptr,
                 const int32_t *__restrict__ leaf_blocks, const int64_t *__restrict__ perm, const float2 *__restrict__ Xs,
                 const double *__restrict__ T, const int64_t *__restrict__ t_off, int64_t N, int B,
                 double *__restrict__ Y)
{
    constexpr int R = kRowsPerWarp;
    __shared__ BlkDesc desc[kMaxLeafBlocks];
    const int L = (int)(blockIdx.x / (unsigned)B), r = (int)(blockIdx.x % (unsigned)B);
    const int64_t p0 = leaf[2 * L], p1 = leaf[2 * L + 1];
    const int rows = 3 * (int)(p1 - p0);
    const int64_t q0 = leaf_ptr[L], q1 = leaf_ptr[L + 1];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = kThreads / 32;
    const int ngroups = (rows + R - 1) / R;
    const float2 *xr = Xs + (int64_t)r * 2 * N;
    double *Yr = Y + (int64_t)r * 3 * N;
    for (int64_t qs = q0; qs < q1; qs += kMaxLeafBlocks) {
        const int nq = (int)min((int64_t)kMaxLeafBlocks, q1 - qs);
        __syncthreads();
        for (int i = threadIdx.x; i < nq; i += kThreads) {
            const int bb = leaf_blocks[qs + i];
            const int64_t r0 = blk[4 * bb], c0 = blk[4 * bb + 2];
            BlkDesc d;
            d.off = off[bb];
            d.c0 = c0;
            d.row0 = 3 * (p0 - r0);
            d.t0 = t_off[bb];
            d.Nc = 2 * (int)(blk[4 * bb + 3] - c0);
            d.k = rank[bb];
            desc[i] = d;
        }
        __syncthreads();
        for (int g = w; g < ngroups; g += nw) {
            const int lr0 = R * g;
            const int nr = min(R, rows - lr0);
            Acc2 a[R];
#pragma unroll
            for (int i = 0; i < R; ++i) a[i] = Acc2{0.f, 0.f};
            // carry the partial sums of the previous descriptor chunk
            if (qs > q0 && lane == 0) {
                for (int i = 0; i < nr; ++i) {
                    const int lr = lr0 + i;
                    const double prev = Yr[3 * perm[p0 + lr / 3] + lr % 3];
                    const float h = (float)prev;
                    a[i].s = h;
                    a[i].c = (float)(prev - (double)h);
                }
            }
            for (int q = 0; q < nq; ++q) {
                const BlkDesc d = desc[q];
                if (d.k < 0) {
                    const float *base = data + d.off + (d.row0 + lr0) * d.Nc;
                    const float2 *x = xr + 2 * d.c0;
                    for (int col = lane; col < d.Nc; col += 32) {
                        const float2 xv = x[col];
#pragma unroll
                        for (int i = 0; i < R; ++i)
                            if (i < nr) acc2_add(a[i], __ldg(base + (int64_t)i * d.Nc + col), xv.x, xv.y);
                    }
                } else if (d.k > 0) {
                    const float *base = data + d.off + (d.row0 + lr0) * d.k;
                    const double *tb = T + d.t0 * (int64_t)B;
                    for (int l = lane; l < d.k; l += 32) {
                        const double tv = tb[(int64_t)l * B + r];
                        const float th = (float)tv, tl = (float)(tv - (double)th);
#pragma unroll
                        for (int i = 0; i < R; ++i)
                            if (i < nr) acc2_add(a[i], __ldg(base + (int64_t)i * d.k + l), th, tl);
                    }
                }
            }
#pragma unroll
            for (int i = 0; i < R; ++i) {
                const double sum = warp_sum((double)a[i].s + (double)a[i].c);
                if (lane == 0 && i < nr) {
                    const int lr = lr0 + i;
                    Yr[3 * perm[p0 + lr / 3] + lr % 3] = sum;
                }
            }
        }
    }
}

}  // namespace hm
}  // namespace pq3d

using namespace pq3d;
using namespace pq3d::hm;

static inline double poisson_(double mu, double lam) { return 1.0 / (1.0 + lam / mu) / 2.0; }

extern "C" int pq3d_gf_setup(const double *nodes, const int64_t *tris, int64_t N, void *workspace,
                             size_t workspace_bytes, void *stream);

extern "C" int pq3d_hmat_aca(const double *tables, int64_t N, const int64_t *perm, int nblocks, const int64_t *blk,
                             const int32_t *kcap, double tol, double mu, double lambda_, double *UV,
                             const int64_t *uv_off, uint8_t *used, const int64_t *used_off, int32_t *rank,
                             int32_t *status, void *stream)
{
    clear_error();
    PQ3D_REQUIRE(tables && perm && blk && kcap && UV && uv_off && used && used_off && rank && status && N > 0,
                 "pq3d_hmat_aca: bad arguments");
    if (nblocks <= 0) return PQ3D_OK;
    const double nu = poisson_(mu, lambda_);
    const double kf = 1.0 / (8.0 * kPi * (1.0 - nu));
    aca_kernel<<<nblocks, kThreads, 0, (cudaStream_t)stream>>>(tables, tables + (size_t)kSrcStride * N, N, perm, blk,
                                                               kcap, tol, nu, kf, 2.0 * mu, lambda_, UV, uv_off, used,
                                                               used_off, rank, status);
    PQ3D_CUDA_TRY(cudaGetLastError());
    return PQ3D_OK;
}

extern "C" int pq3d_hmat_dense_blocks(const double *tables, int64_t N, const int64_t *perm, const int64_t *blk,
                                      const int32_t *ids, int nids, double mu, double lambda_, float *D,
                                      const int64_t *d_off, void *stream)
{
    clear_error();
    PQ3D_REQUIRE(tables && perm && blk && ids && D && d_off && N > 0, "pq3d_hmat_dense_blocks: bad arguments");
    PQ3D_REQUIRE(((uintptr_t)D & 7u) == 0, "pq3d_hmat_dense_blocks: D must be 8-byte aligned");
    if (nids <= 0) return PQ3D_OK;
    const double nu = poisson_(mu, lambda_);
    const double kf = 1.0 / (8.0 * kPi * (1.0 - nu));
    dense_blocks_kernel<<<nids, kThreads, 0, (cudaStream_t)stream>>>(tables, tables + (size_t)kSrcStride * N, N, perm,
                                                                     blk, ids, nu, kf, 2.0 * mu, lambda_, D, d_off);
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

extern "C" int pq3d_hmat_apply(const pq3d_hmat *H, const double *X, int B, double *Y, void *workspace,
                               size_t workspace_bytes, void *stream)
{
    clear_error();
    PQ3D_REQUIRE(H && X && Y && workspace && B >= 1, "pq3d_hmat_apply: bad arguments");
    const int64_t N = H->N;
    const size_t need = (size_t)B * 2 * N * sizeof(float2) + (size_t)H->t_rows * B * sizeof(double);
    PQ3D_REQUIRE(workspace_bytes >= need && aligned16(workspace), "pq3d_hmat_apply: workspace too small (%zu < %zu)",
                 workspace_bytes, need);
    cudaStream_t st = (cudaStream_t)stream;
    float2 *Xs = (float2 *)workspace;
    double *T = (double *)((char *)workspace + (size_t)B * 2 * N * sizeof(float2));
    dim3 g1((unsigned)((2 * N + 255) / 256), (unsigned)B);
    permute_split_kernel<<<g1, 256, 0, st>>>(X, H->perm, N, B, Xs);
    // all runs in one launch, run fastest in the block index; a run's result
    // does not depend on B
    if (H->t_rows > 0) {
        const int64_t nT = (H->t_rows * 32 + 255) / 256 * B;
        PQ3D_REQUIRE(nT < (int64_t)INT32_MAX, "pq3d_hmat_apply: too many rank rows x runs");
        const unsigned gT = (unsigned)nT;
        lowrank_T_kernel<<<gT, 256, 0, st>>>(H->data, H->off, H->blk, H->rank, H->lr_ids, H->lr_row0, (int)H->t_rows,
                                             Xs, N, B, T, H->t_off);
    }
    PQ3D_REQUIRE((int64_t)H->nleaves * B < (int64_t)INT32_MAX, "pq3d_hmat_apply: too many leaves x runs");
    const unsigned gL = (unsigned)(H->nleaves * B);
    leaf_rows_kernel<<<gL, kThreads, 0, st>>>(H->data, H->off, H->blk, H->rank, H->leaf, H->leaf_ptr, H->leaf_blocks,
                                              H->perm, Xs, T, H->t_off, N, B, Y);
    PQ3D_CUDA_TRY(cudaGetLastError());
    return PQ3D_OK;
}

extern "C" size_t pq3d_hmat_workspace_bytes(const pq3d_hmat *H, int B)
{
    if (!H || B < 1) return 0;
    return (size_t)B * 2 * H->N * sizeof(float2) + (size_t)H->t_rows * B * sizeof(double);
}
