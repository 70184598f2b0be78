// H-matrix partition on the device: the cluster tree over the element
// centroids and the block tree, level by level, without host recursion.
//
// Rules (src/Hmatrix.py:68-113, 153-192, 2077-2142):
//   * cluster tree: a node with more than min_size points bisects the longest
//     axis of its bounding box (the first one on ties) at its midpoint
//     (lo + hi) / 2; points <= midpoint go left, the others right, each side
//     in its previous order; a node is a leaf when it has <= min_size points
//     or when a side would be empty;
//   * block tree from (root, root): a pair is a leaf block when it is
//     admissible, min(diam_r, diam_c) <= eta * dist(box_r, box_c), or when
//     either cluster has <= mini_leaf points or no children; otherwise its
//     four child pairs (left/right x left/right, in that order) follow;
//   * a leaf block is low rank when both sides have more than mini_leaf points.
// Elements are renumbered in depth-first leaf order, so a cluster is a
// contiguous range; blocks come out in depth-first order.  Every comparison
// uses the reference's FP64 expressions in its order of operations (box
// extents, the midpoint, sqrt of ((0 + a) + b) + c sums), so the partition is
// the reference's bit for bit.
//
// Device work per cluster level: one CTA per node of the level computes the
// box, the split and a stable partition of its range (block-wide scans);
// one small kernel numbers the children.  Per block-tree level: one thread per
// pair decides, one small kernel numbers the child pairs.  Then the leaf
// counts go up the block tree and the depth-first offsets come down, and every
// leaf pair writes its block at its offset.  The host reads one count per
// level to size the next launch.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include <vector>

#include "common.cuh"

namespace pq3d {
namespace htree {

constexpr int kT = 256;   // threads of the per-node and scan kernels

struct Tree {
    int64_t *start, *end;   // [cap] cluster range
    double *lo, *hi;         // [cap][3] bounding box
    int32_t *left;           // [cap] first child (right = left + 1), -1 for a leaf
    int64_t *nleft;          // [cap] points of the left child
    int32_t *split;          // [cap] 1 if the node splits
};

// ---------------------------------------------------------------------------
// block-wide helpers

__device__ __forceinline__ double block_min(double v, double *red)
{
    for (int o = 16; o > 0; o >>= 1) v = fmin(v, __shfl_xor_sync(0xffffffffu, v, o));
    __syncthreads();
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    double r = red[0];
    for (int w = 1; w < (int)(blockDim.x >> 5); ++w) r = fmin(r, red[w]);
    return r;
}

__device__ __forceinline__ double block_max(double v, double *red)
{
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    __syncthreads();
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    double r = red[0];
    for (int w = 1; w < (int)(blockDim.x >> 5); ++w) r = fmax(r, red[w]);
    return r;
}

// exclusive scan of one int per thread over the block; returns the block total
__device__ __forceinline__ int64_t block_scan(int64_t v, int64_t &excl, int64_t *sm)
{
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    int64_t x = v;
    for (int o = 1; o < 32; o <<= 1) {
        const int64_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    __syncthreads();
    if (lane == 31) sm[w] = x;
    __syncthreads();
    int64_t base = 0, total = 0;
    for (int k = 0; k < nw; ++k) {
        if (k < w) base += sm[k];
        total += sm[k];
    }
    excl = base + x - v;
    return total;
}

// ---------------------------------------------------------------------------
// cluster tree: one CTA per node of the level [n0, n1)

__global__ void __launch_bounds__(kT) cluster_level_kernel(Tree T, const double *__restrict__ xg, int64_t n0,
                                                            const int64_t *__restrict__ pin, int64_t *__restrict__ pout,
                                                            int min_size)
{
    __shared__ double red[kT / 32];
    __shared__ int64_t sm[kT / 32];
    __shared__ int s_axis;
    __shared__ double s_g;
    const int64_t nd = n0 + blockIdx.x;
    const int64_t s = T.start[nd], e = T.end[nd];
    double lo[3], hi[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        double a = INFINITY, b = -INFINITY;
        for (int64_t p = s + threadIdx.x; p < e; p += blockDim.x) {
            const double x = xg[3 * pin[p] + d];
            a = fmin(a, x);
            b = fmax(b, x);
        }
        lo[d] = block_min(a, red);
        hi[d] = block_max(b, red);
    }
    if (threadIdx.x == 0) {
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            T.lo[3 * nd + d] = lo[d];
            T.hi[3 * nd + d] = hi[d];
        }
        // longest axis, first on ties (numpy argmax), and its midpoint
        int j = 0;
        double ext = __dsub_rn(hi[0], lo[0]);
        for (int d = 1; d < 3; ++d) {
            const double x = __dsub_rn(hi[d], lo[d]);
            if (x > ext) { ext = x; j = d; }
        }
        s_axis = j;
        s_g = __dmul_rn(__dadd_rn(lo[j], hi[j]), 0.5);
    }
    __syncthreads();
    const int j = s_axis;
    const double g = s_g;
    int64_t nl = 0;
    if (e - s > min_size) {
        int64_t c = 0;
        for (int64_t p = s + threadIdx.x; p < e; p += blockDim.x) c += xg[3 * pin[p] + j] <= g;
        int64_t ex;
        nl = block_scan(c, ex, sm);
    }
    const bool split = e - s > min_size && nl > 0 && nl < e - s;
    if (threadIdx.x == 0) {
        T.split[nd] = split ? 1 : 0;
        T.nleft[nd] = nl;
        T.left[nd] = -1;
    }
    if (!split) {
        for (int64_t p = s + threadIdx.x; p < e; p += blockDim.x) pout[p] = pin[p];
        return;
    }
    // stable partition: chunks of blockDim elements, running left/right counts
    int64_t lbase = 0;
    for (int64_t c0 = s; c0 < e; c0 += blockDim.x) {
        const int64_t p = c0 + threadIdx.x;
        const int64_t el = p < e ? pin[p] : 0;
        const int f = p < e && xg[3 * el + j] <= g ? 1 : 0;
        int64_t ex;
        const int64_t tot = block_scan(f, ex, sm);
        if (p < e) {
            const int64_t lpos = lbase + ex;                           // left elements before p
            const int64_t rpos = (p - s) - lpos;                       // right elements before p
            pout[f ? s + lpos : s + nl + rpos] = el;
        }
        lbase += tot;
    }
}

// children of the split nodes of level [n0, n1): ids from `next` on, in node order
__global__ void __launch_bounds__(kT) cluster_children_kernel(Tree T, int64_t n0, int64_t n1, int64_t next,
                                                               int64_t *count)
{
    __shared__ int64_t sm[kT / 32];
    int64_t base = 0;
    for (int64_t c0 = n0; c0 < n1; c0 += blockDim.x) {
        const int64_t nd = c0 + threadIdx.x;
        const int f = nd < n1 ? T.split[nd] : 0;
        int64_t ex;
        const int64_t tot = block_scan(f, ex, sm);
        if (f) {
            const int64_t id = next + 2 * (base + ex);
            const int64_t s = T.start[nd], e = T.end[nd], nl = T.nleft[nd];
            T.left[nd] = (int32_t)id;
            T.start[id] = s;
            T.end[id] = s + nl;
            T.start[id + 1] = s + nl;
            T.end[id + 1] = e;
        }
        base += tot;
    }
    if (threadIdx.x == 0) *count = 2 * base;
}

// ---------------------------------------------------------------------------
// block tree

struct Pairs {
    int32_t *r, *c;         // [cap] cluster nodes
    int32_t *child;         // [cap] first child pair (the four are contiguous), -1 for a leaf
    int32_t *flag;          // [cap] 1 if the pair splits
    int64_t *cnt;           // [cap] leaf blocks below the pair
    int64_t *off;           // [cap] depth-first position of the pair's first leaf block
};

__device__ __forceinline__ double diam(const Tree &T, int n)
{
    const double *l = T.lo + 3 * n, *h = T.hi + 3 * n;
    double s = 0.0;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        const double x = __dsub_rn(h[d], l[d]);
        s = __dadd_rn(s, __dmul_rn(x, x));
    }
    return __dsqrt_rn(s);
}

__device__ __forceinline__ double box_dist(const Tree &T, int a, int b)
{
    const double *al = T.lo + 3 * a, *ah = T.hi + 3 * a, *bl = T.lo + 3 * b, *bh = T.hi + 3 * b;
    double s = 0.0;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        const double u = fmax(0.0, __dsub_rn(bl[d], ah[d])), v = fmax(0.0, __dsub_rn(al[d], bh[d]));
        s = __dadd_rn(s, __dadd_rn(__dmul_rn(u, u), __dmul_rn(v, v)));
    }
    return __dsqrt_rn(s);
}

__global__ void pair_level_kernel(Tree T, Pairs P, int64_t p0, int64_t p1, int mini_leaf, double eta)
{
    const int64_t q = p0 + blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (q >= p1) return;
    const int r = P.r[q], c = P.c[q];
    const int64_t nr = T.end[r] - T.start[r], nc = T.end[c] - T.start[c];
    const bool adm = fmin(diam(T, r), diam(T, c)) <= __dmul_rn(eta, box_dist(T, r, c));
    const bool leaf = adm || nr <= mini_leaf || nc <= mini_leaf || T.left[r] < 0 || T.left[c] < 0;
    P.flag[q] = leaf ? 0 : 1;
    P.child[q] = -1;
    P.cnt[q] = leaf ? 1 : 0;
}

__global__ void __launch_bounds__(kT) pair_children_kernel(Tree T, Pairs P, int64_t p0, int64_t p1, int64_t next,
                                                            int64_t *count)
{
    __shared__ int64_t sm[kT / 32];
    int64_t base = 0;
    for (int64_t c0 = p0; c0 < p1; c0 += blockDim.x) {
        const int64_t q = c0 + threadIdx.x;
        const int f = q < p1 ? P.flag[q] : 0;
        int64_t ex;
        const int64_t tot = block_scan(f, ex, sm);
        if (f) {
            const int64_t id = next + 4 * (base + ex);
            const int r = P.r[q], c = P.c[q];
            const int rl = T.left[r], cl = T.left[c];
            P.child[q] = (int32_t)id;
            P.r[id] = rl;     P.c[id] = cl;
            P.r[id + 1] = rl; P.c[id + 1] = cl + 1;
            P.r[id + 2] = rl + 1; P.c[id + 2] = cl;
            P.r[id + 3] = rl + 1; P.c[id + 3] = cl + 1;
        }
        base += tot;
    }
    if (threadIdx.x == 0) *count = 4 * base;
}

// leaf blocks below each split pair of [p0, p1) (children already counted)
__global__ void pair_count_kernel(Pairs P, int64_t p0, int64_t p1)
{
    const int64_t q = p0 + blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (q >= p1 || P.flag[q] == 0) return;
    const int64_t ch = P.child[q];
    P.cnt[q] = P.cnt[ch] + P.cnt[ch + 1] + P.cnt[ch + 2] + P.cnt[ch + 3];
}

// depth-first offsets of the children of each split pair of [p0, p1)
__global__ void pair_offset_kernel(Pairs P, int64_t p0, int64_t p1)
{
    const int64_t q = p0 + blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (q >= p1 || P.flag[q] == 0) return;
    const int64_t ch = P.child[q];
    int64_t o = P.off[q];
    for (int k = 0; k < 4; ++k) {
        P.off[ch + k] = o;
        o += P.cnt[ch + k];
    }
}

__global__ void pair_emit_kernel(Tree T, Pairs P, int64_t npairs, int mini_leaf, int64_t *__restrict__ blocks)
{
    const int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (q >= npairs || P.flag[q] != 0) return;
    const int r = P.r[q], c = P.c[q];
    int64_t *b = blocks + 5 * P.off[q];
    b[0] = T.start[r];
    b[1] = T.end[r];
    b[2] = T.start[c];
    b[3] = T.end[c];
    b[4] = (T.end[r] - T.start[r] > mini_leaf && T.end[c] - T.start[c] > mini_leaf) ? 1 : 0;
}

// cluster leaves in order of their start: mark, then compact
__global__ void leaf_mark_kernel(Tree T, int64_t nnodes, int64_t *__restrict__ mark)
{
    const int64_t nd = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (nd >= nnodes || T.split[nd]) return;
    mark[T.start[nd]] = T.end[nd];
}

__global__ void __launch_bounds__(kT) leaf_compact_kernel(const int64_t *__restrict__ mark, int64_t N,
                                                           int64_t *__restrict__ leaves, int64_t *count)
{
    __shared__ int64_t sm[kT / 32];
    int64_t base = 0;
    for (int64_t c0 = 0; c0 < N; c0 += blockDim.x) {
        const int64_t p = c0 + threadIdx.x;
        const int f = p < N && mark[p] >= 0 ? 1 : 0;
        int64_t ex;
        const int64_t tot = block_scan(f, ex, sm);
        if (f) {
            leaves[2 * (base + ex)] = p;
            leaves[2 * (base + ex) + 1] = mark[p];
        }
        base += tot;
    }
    if (threadIdx.x == 0) *count = base;
}

__global__ void iota_kernel(int64_t *p, int64_t n)
{
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n) p[i] = i;
}

// ---------------------------------------------------------------------------
// host driver

struct DevBuf {
    void *p = nullptr;
    ~DevBuf() { if (p) cudaFree(p); }
};

static unsigned nblk(int64_t n, int t) { return (unsigned)((n + t - 1) / t); }

}  // namespace htree
}  // namespace pq3d

using namespace pq3d;
using namespace pq3d::htree;

#define HT_TRY(call)                                                                                             \
    do {                                                                                                         \
        cudaError_t e_ = (call);                                                                                 \
        if (e_ != cudaSuccess)                                                                                   \
            return set_error(PQ3D_ERR_CUDA, "pq3d_hmat_partition: %s: %s", #call, cudaGetErrorString(e_));      \
    } while (0)

static int partition(const double *xg, int64_t N, int min_size, int mini_leaf, double eta, int64_t *perm,
                     int64_t *leaves, int64_t *n_leaves, int64_t *blocks, int64_t cap_blocks, int64_t *n_blocks,
                     int32_t *depth, void *stream, bool tree_only);

extern "C" int pq3d_hmat_cluster_order(const double *xg, int64_t N, int min_size, int64_t *perm, int32_t *depth,
                                       void *stream)
{
    clear_error();
    PQ3D_REQUIRE(xg && perm && N > 0 && N < (1ll << 30) && min_size >= 1, "pq3d_hmat_cluster_order: bad arguments");
    return partition(xg, N, min_size, 1, 0.0, perm, nullptr, nullptr, nullptr, 0, nullptr, depth, stream, true);
}

extern "C" int pq3d_hmat_partition(const double *xg, int64_t N, int min_size, int mini_leaf, double eta,
                                   int64_t *perm, int64_t *leaves, int64_t *n_leaves, int64_t *blocks,
                                   int64_t cap_blocks, int64_t *n_blocks, int32_t *depth, void *stream)
{
    clear_error();
    PQ3D_REQUIRE(xg && perm && leaves && n_leaves && n_blocks && N > 0 && N < (1ll << 30),
                 "pq3d_hmat_partition: bad arguments");
    return partition(xg, N, min_size, mini_leaf, eta, perm, leaves, n_leaves, blocks, cap_blocks, n_blocks, depth,
                     stream, false);
}

static int partition(const double *xg, int64_t N, int min_size, int mini_leaf, double eta, int64_t *perm,
                     int64_t *leaves, int64_t *n_leaves, int64_t *blocks, int64_t cap_blocks, int64_t *n_blocks,
                     int32_t *depth, void *stream, bool tree_only)
{
    PQ3D_REQUIRE(min_size >= 1 && mini_leaf >= 1 && eta >= 0.0, "pq3d_hmat_partition: bad parameters");
    cudaStream_t st = (cudaStream_t)stream;
    // scratch: nodes (at most 2N - 1), the other perm buffer, a count word
    const int64_t ncap = 2 * N;
    DevBuf nodes_mem, cnt_mem;
    const size_t node_bytes = (size_t)ncap * (8 + 8 + 24 + 24 + 4 + 8 + 4) + (size_t)N * 8 * 2;
    HT_TRY(cudaMalloc(&nodes_mem.p, node_bytes));
    HT_TRY(cudaMalloc(&cnt_mem.p, 64));
    char *q = (char *)nodes_mem.p;
    Tree T;
    T.start = (int64_t *)q; q += ncap * 8;
    T.end = (int64_t *)q; q += ncap * 8;
    T.lo = (double *)q; q += ncap * 24;
    T.hi = (double *)q; q += ncap * 24;
    T.nleft = (int64_t *)q; q += ncap * 8;
    int64_t *pbuf = (int64_t *)q; q += (size_t)N * 8;
    int64_t *mark = (int64_t *)q; q += (size_t)N * 8;
    T.left = (int32_t *)q; q += ncap * 4;
    T.split = (int32_t *)q; q += ncap * 4;
    int64_t *dcount = (int64_t *)cnt_mem.p;

    // cluster tree
    iota_kernel<<<nblk(N, 256), 256, 0, st>>>(perm, N);
    const int64_t zero = 0;
    HT_TRY(cudaMemcpyAsync(T.start, &zero, 8, cudaMemcpyHostToDevice, st));
    HT_TRY(cudaMemcpyAsync(T.end, &N, 8, cudaMemcpyHostToDevice, st));
    int64_t n0 = 0, n1 = 1;
    int lev = 0;
    int64_t *pin = perm, *pout = pbuf;
    while (n1 > n0) {
        cluster_level_kernel<<<(unsigned)(n1 - n0), kT, 0, st>>>(T, xg, n0, pin, pout, min_size);
        cluster_children_kernel<<<1, kT, 0, st>>>(T, n0, n1, n1, dcount);
        HT_TRY(cudaGetLastError());
        int64_t nc = 0;
        HT_TRY(cudaMemcpyAsync(&nc, dcount, 8, cudaMemcpyDeviceToHost, st));
        HT_TRY(cudaStreamSynchronize(st));
        PQ3D_REQUIRE(n1 + nc <= ncap, "pq3d_hmat_partition: cluster tree exceeds %lld nodes", (long long)ncap);
        n0 = n1;
        n1 += nc;
        std::swap(pin, pout);
        ++lev;
    }
    const int64_t nnodes = n1;
    // both perm buffers hold every final range; make sure `perm` has them
    if (pin != perm) HT_TRY(cudaMemcpyAsync(perm, pin, (size_t)N * 8, cudaMemcpyDeviceToDevice, st));
    if (depth) *depth = lev;
    if (tree_only) {
        HT_TRY(cudaStreamSynchronize(st));
        return PQ3D_OK;
    }
    // cluster leaves in depth-first order
    HT_TRY(cudaMemsetAsync(mark, 0xff, (size_t)N * 8, st));
    leaf_mark_kernel<<<nblk(nnodes, 256), 256, 0, st>>>(T, nnodes, mark);
    leaf_compact_kernel<<<1, kT, 0, st>>>(mark, N, leaves, dcount);
    HT_TRY(cudaGetLastError());
    HT_TRY(cudaMemcpyAsync(n_leaves, dcount, 8, cudaMemcpyDeviceToHost, st));

    // block tree, level by level; pair arrays grow by the split count
    std::vector<int64_t> lv = {0, 1};
    int64_t pcap = 1 << 16;
    DevBuf pmem;
    auto alloc_pairs = [&](int64_t cap, Pairs &P) -> int {
        DevBuf nm;
        HT_TRY(cudaMalloc(&nm.p, (size_t)cap * (4 + 4 + 4 + 4 + 8 + 8)));
        Pairs Q;
        char *z = (char *)nm.p;
        Q.cnt = (int64_t *)z; z += cap * 8;
        Q.off = (int64_t *)z; z += cap * 8;
        Q.r = (int32_t *)z; z += cap * 4;
        Q.c = (int32_t *)z; z += cap * 4;
        Q.child = (int32_t *)z; z += cap * 4;
        Q.flag = (int32_t *)z; z += cap * 4;
        if (pmem.p) {   // keep the pairs made so far
            const int64_t used = lv.back();
            HT_TRY(cudaMemcpyAsync(Q.cnt, P.cnt, used * 8, cudaMemcpyDeviceToDevice, st));
            HT_TRY(cudaMemcpyAsync(Q.off, P.off, used * 8, cudaMemcpyDeviceToDevice, st));
            HT_TRY(cudaMemcpyAsync(Q.r, P.r, used * 4, cudaMemcpyDeviceToDevice, st));
            HT_TRY(cudaMemcpyAsync(Q.c, P.c, used * 4, cudaMemcpyDeviceToDevice, st));
            HT_TRY(cudaMemcpyAsync(Q.child, P.child, used * 4, cudaMemcpyDeviceToDevice, st));
            HT_TRY(cudaMemcpyAsync(Q.flag, P.flag, used * 4, cudaMemcpyDeviceToDevice, st));
            HT_TRY(cudaStreamSynchronize(st));
            cudaFree(pmem.p);
        }
        pmem.p = nm.p;
        nm.p = nullptr;
        P = Q;
        return PQ3D_OK;
    };
    Pairs P{};
    int rc = alloc_pairs(pcap, P);
    if (rc) return rc;
    const int32_t root = 0;
    HT_TRY(cudaMemcpyAsync(P.r, &root, 4, cudaMemcpyHostToDevice, st));
    HT_TRY(cudaMemcpyAsync(P.c, &root, 4, cudaMemcpyHostToDevice, st));
    HT_TRY(cudaMemcpyAsync(P.off, &zero, 8, cudaMemcpyHostToDevice, st));
    for (;;) {
        const int64_t p0 = lv[lv.size() - 2], p1 = lv.back();
        if (p1 == p0) break;
        pair_level_kernel<<<nblk(p1 - p0, 256), 256, 0, st>>>(T, P, p0, p1, mini_leaf, eta);
        HT_TRY(cudaGetLastError());
        // worst case: every pair splits
        if (p1 + 4 * (p1 - p0) > pcap) {
            while (p1 + 4 * (p1 - p0) > pcap) pcap *= 2;
            HT_TRY(cudaStreamSynchronize(st));
            rc = alloc_pairs(pcap, P);
            if (rc) return rc;
        }
        pair_children_kernel<<<1, kT, 0, st>>>(T, P, p0, p1, p1, dcount);
        HT_TRY(cudaGetLastError());
        int64_t nc = 0;
        HT_TRY(cudaMemcpyAsync(&nc, dcount, 8, cudaMemcpyDeviceToHost, st));
        HT_TRY(cudaStreamSynchronize(st));
        lv.push_back(p1 + nc);
    }
    const int64_t npairs = lv.back();
    // leaf counts up, offsets down
    for (size_t k = lv.size() - 1; k-- > 0;)
        if (lv[k + 1] > lv[k]) pair_count_kernel<<<nblk(lv[k + 1] - lv[k], 256), 256, 0, st>>>(P, lv[k], lv[k + 1]);
    for (size_t k = 0; k + 1 < lv.size(); ++k)
        if (lv[k + 1] > lv[k]) pair_offset_kernel<<<nblk(lv[k + 1] - lv[k], 256), 256, 0, st>>>(P, lv[k], lv[k + 1]);
    HT_TRY(cudaGetLastError());
    int64_t nb = 0;
    HT_TRY(cudaMemcpyAsync(&nb, P.cnt, 8, cudaMemcpyDeviceToHost, st));
    HT_TRY(cudaStreamSynchronize(st));
    *n_blocks = nb;
    if (!blocks || nb > cap_blocks)
        return set_error(PQ3D_ERR_ARG, "pq3d_hmat_partition: %lld blocks need a blocks array of that capacity "
                         "(given %lld)", (long long)nb, (long long)cap_blocks);
    pair_emit_kernel<<<nblk(npairs, 256), 256, 0, st>>>(T, P, npairs, mini_leaf, blocks);
    HT_TRY(cudaGetLastError());
    HT_TRY(cudaStreamSynchronize(st));
    return PQ3D_OK;
}
