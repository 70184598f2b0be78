// Green's-function kernels and the reference-compatible C-ABI.
//
//   setup_sources / setup_receivers   once per mesh: per-source record (frame,
//                                     angles, side vectors) and per-receiver
//                                     record (centroid, frame)
//   assemble_dense                    one (receiver, source) pair per thread,
//                                     both unit slips, 6 tractions -> FP64 K
//                                     (+ FP32 copy) with 16-byte stores
//   points_one_source / point_many_sources
//                                     the two host-pointer entry points of the
//                                     reference TDstressFS_C.so
//   half-space (jud_halfspace / halfspace != 0): per-source image record and
//   free-surface side table (setup_hs), the pair evaluated by
//   pair_tractions_hs / point_strain_hs (hs_device.cuh)
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <mutex>
#include <vector>

#include "common.cuh"
#include "gf_device.cuh"
#include "hs_device.cuh"

namespace pq3d {
namespace gf {

struct SoaSrc {   // field f of one source in a structure-of-arrays table
    const double *base;
    int stride;
    __device__ __forceinline__ double operator()(int f) const { return base[f * stride]; }
};

struct ValSrc {   // fields held in a small array
    const double *f;
    __device__ __forceinline__ double operator()(int i) const { return f[i]; }
};

struct SrcVal { double f[kSrcStride]; };
struct FscVal { double f[kFscStride]; };

__global__ void setup_sources_kernel(const double *__restrict__ nodes, const int64_t *__restrict__ tris, int64_t N,
                                     double *__restrict__ src)
{
    const int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (j >= N) return;
    const double *P1 = nodes + 3 * (tris[3 * j] - 1);
    const double *P2 = nodes + 3 * (tris[3 * j + 1] - 1);
    const double *P3 = nodes + 3 * (tris[3 * j + 2] - 1);
    double a[3] = {P1[0], P1[1], P1[2]}, b[3] = {P2[0], P2[1], P2[2]}, c[3] = {P3[0], P3[1], P3[2]};
    setup_source(a, b, c, src + j, (int)N);
}

__global__ void setup_receivers_kernel(const double *__restrict__ nodes, const int64_t *__restrict__ tris, int64_t N,
                                       double *__restrict__ recv)
{
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= N) return;
    const double *A = nodes + 3 * (tris[3 * i] - 1);
    const double *B = nodes + 3 * (tris[3 * i + 1] - 1);
    const double *C = nodes + 3 * (tris[3 * i + 2] - 1);
    double a[3] = {A[0], A[1], A[2]}, b[3] = {B[0], B[1], B[2]}, c[3] = {C[0], C[1], C[2]};
    setup_receiver(a, b, c, recv + kRecvStride * i);
}

// Half-space records of source j: the mirrored triangle's source record
// (img, stride N) and the free-surface side table (fsc, stride N).
__global__ void setup_hs_kernel(const double *__restrict__ nodes, const int64_t *__restrict__ tris, int64_t N,
                                double *__restrict__ img, double *__restrict__ fsc)
{
    const int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (j >= N) return;
    const double *P1 = nodes + 3 * (tris[3 * j] - 1);
    const double *P2 = nodes + 3 * (tris[3 * j + 1] - 1);
    const double *P3 = nodes + 3 * (tris[3 * j + 2] - 1);
    double a[3] = {P1[0], P1[1], P1[2]}, b[3] = {P2[0], P2[1], P2[2]}, c[3] = {P3[0], P3[1], P3[2]};
    double am[3] = {a[0], a[1], -a[2]}, bm[3] = {b[0], b[1], -b[2]}, cm[3] = {c[0], c[1], -c[2]};
    setup_source(am, bm, cm, img + j, (int)N);
    setup_fsc(a, b, c, fsc + j, (int)N);
}

constexpr int kTJ = 128;   // sources per block (one per thread)
constexpr int kTI = 32;    // receivers per block (looped by every thread)

// K64 / K32 point at row 3*row0; leading dimension 2N.
template <bool kWrite32>
__global__ void __launch_bounds__(kTJ)
assemble_dense_kernel(const double *__restrict__ src, const double *__restrict__ recv, int64_t N, int64_t row0,
                      int64_t row1, double nu, double k, double two_mu, double lam, double *__restrict__ K64,
                      float *__restrict__ K32)
{
    __shared__ double s_src[F_COUNT * kTJ];
    __shared__ double s_rcv[kTI * kRecvStride];
    const int t = threadIdx.x;
    const int64_t j0 = (int64_t)blockIdx.x * kTJ;
    const int64_t i0 = row0 + (int64_t)blockIdx.y * kTI;
    const int64_t j = j0 + t;
    for (int f = 0; f < F_COUNT; ++f) s_src[f * kTJ + t] = (j < N) ? src[f * N + j] : 0.0;
    const int nrec = (int)((row1 - i0) < kTI ? (row1 - i0) : kTI);
    // receiver records with e1 and e2 multiplied by the traction scale
    const double axis_scale = traction_axis_scale(k, two_mu);
    for (int q = t; q < nrec * kRecvStride; q += kTJ) {
        const int fq = q % kRecvStride;
        const double v = recv[i0 * kRecvStride + q];
        s_rcv[q] = (fq >= 3 && fq < 9) ? v * axis_scale : v;
    }
    __syncthreads();
    if (j >= N) return;
    const SoaSrc F{s_src + t, kTJ};
    const int64_t ld = 2 * N;
    for (int ii = 0; ii < nrec; ++ii) {
        double ts[3], td[3];
        pair_tractions<SoaSrc, true>(F, s_rcv + ii * kRecvStride, nu, k, two_mu, lam, ts, td);
        const int64_t r = 3 * (i0 + ii - row0);
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            *reinterpret_cast<double2 *>(K64 + (r + c) * ld + 2 * j) = make_double2(ts[c], td[c]);
            if (kWrite32)
                *reinterpret_cast<float2 *>(K32 + (r + c) * ld + 2 * j) = make_float2(d2f_rn_bits(ts[c]), d2f_rn_bits(td[c]));
        }
    }
}

// Half-space variant: main record in shared memory, image record and side
// table read from their structure-of-arrays tables (coalesced over sources).
template <bool kWrite32>
__global__ void __launch_bounds__(kTJ)
assemble_dense_hs_kernel(const double *__restrict__ src, const double *__restrict__ recv,
                         const double *__restrict__ img, const double *__restrict__ fsc, int64_t N, int64_t row0,
                         int64_t row1, double nu, double k, double two_mu, double lam, double *__restrict__ K64,
                         float *__restrict__ K32)
{
    __shared__ double s_src[F_COUNT * kTJ];
    __shared__ double s_rcv[kTI * kRecvStride];
    const int t = threadIdx.x;
    const int64_t j0 = (int64_t)blockIdx.x * kTJ;
    const int64_t i0 = row0 + (int64_t)blockIdx.y * kTI;
    const int64_t j = j0 + t;
    for (int f = 0; f < F_COUNT; ++f) s_src[f * kTJ + t] = (j < N) ? src[f * N + j] : 0.0;
    const int nrec = (int)((row1 - i0) < kTI ? (row1 - i0) : kTI);
    for (int q = t; q < nrec * kRecvStride; q += kTJ) s_rcv[q] = recv[i0 * kRecvStride + q];
    __syncthreads();
    if (j >= N) return;
    const SoaSrc F{s_src + t, kTJ};
    const SoaSrc Fi{img + j, (int)N};
    const SoaSrc G{fsc + j, (int)N};
    const int64_t ld = 2 * N;
    for (int ii = 0; ii < nrec; ++ii) {
        double ts[3], td[3];
        pair_tractions_hs(F, Fi, G, s_rcv + ii * kRecvStride, nu, k, two_mu, lam, ts, td);
        const int64_t r = 3 * (i0 + ii - row0);
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            *reinterpret_cast<double2 *>(K64 + (r + c) * ld + 2 * j) = make_double2(ts[c], td[c]);
            if (kWrite32)
                *reinterpret_cast<float2 *>(K32 + (r + c) * ld + 2 * j) = make_float2(d2f_rn_bits(ts[c]), d2f_rn_bits(td[c]));
        }
    }
}

__global__ void points_one_source_hs_kernel(SrcVal s, SrcVal si, FscVal g, const double *__restrict__ X,
                                            const double *__restrict__ Y, const double *__restrict__ Z, int64_t n,
                                            double bx, double by, double bz, double mu, double lam, double nu,
                                            double k, double *__restrict__ stress, double *__restrict__ strain)
{
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const ValSrc F{s.f}, Fi{si.f}, G{g.f};
    double e[6], sg[6];
    point_strain_hs(F, Fi, G, X[i], Y[i], Z[i], bx, by, bz, nu, k, e);
    hooke(e, mu, lam, sg);
    for (int c = 0; c < 6; ++c) { stress[6 * i + c] = sg[c]; strain[6 * i + c] = e[c]; }
}

__global__ void point_many_sources_hs_kernel(double X, double Y, double Z, const double *__restrict__ P1,
                                             const double *__restrict__ P2, const double *__restrict__ P3,
                                             int64_t ns, double bx, double by, double bz, double mu, double lam,
                                             double nu, double k, double *__restrict__ stress,
                                             double *__restrict__ strain)
{
    const int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (j >= ns) return;
    double f[kSrcStride], fi[kSrcStride], g[kFscStride];
    double a[3] = {P1[3 * j], P1[3 * j + 1], P1[3 * j + 2]};
    double b[3] = {P2[3 * j], P2[3 * j + 1], P2[3 * j + 2]};
    double c[3] = {P3[3 * j], P3[3 * j + 1], P3[3 * j + 2]};
    double am[3] = {a[0], a[1], -a[2]}, bm[3] = {b[0], b[1], -b[2]}, cm[3] = {c[0], c[1], -c[2]};
    setup_source(a, b, c, f, 1);
    setup_source(am, bm, cm, fi, 1);
    setup_fsc(a, b, c, g, 1);
    const ValSrc F{f}, Fi{fi}, G{g};
    double e[6], sg[6];
    point_strain_hs(F, Fi, G, X, Y, Z, bx, by, bz, nu, k, e);
    hooke(e, mu, lam, sg);
    for (int q = 0; q < 6; ++q) { stress[6 * j + q] = sg[q]; strain[6 * j + q] = e[q]; }
}

__global__ void points_one_source_kernel(SrcVal s, const double *__restrict__ X, const double *__restrict__ Y,
                                         const double *__restrict__ Z, int64_t n, double bx, double by, double bz,
                                         double mu, double lam, double nu, double k, double *__restrict__ stress,
                                         double *__restrict__ strain)
{
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const ValSrc F{s.f};
    double x, y, z, E[6], e[6], sg[6];
    tdcs_point(F, X[i], Y[i], Z[i], x, y, z);
    tdcs_strain_general(F, x, y, z, bx, by, bz, nu, k, E);
    tdcs_to_efcs(F, E, e);
    hooke(e, mu, lam, sg);
    for (int c = 0; c < 6; ++c) { stress[6 * i + c] = sg[c]; strain[6 * i + c] = e[c]; }
}

__global__ void point_many_sources_kernel(double X, double Y, double Z, const double *__restrict__ P1,
                                          const double *__restrict__ P2, const double *__restrict__ P3, int64_t ns,
                                          double bx, double by, double bz, double mu, double lam, double nu, double k,
                                          double *__restrict__ stress, double *__restrict__ strain)
{
    const int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (j >= ns) return;
    double f[kSrcStride];
    double a[3] = {P1[3 * j], P1[3 * j + 1], P1[3 * j + 2]};
    double b[3] = {P2[3 * j], P2[3 * j + 1], P2[3 * j + 2]};
    double c[3] = {P3[3 * j], P3[3 * j + 1], P3[3 * j + 2]};
    setup_source(a, b, c, f, 1);
    const ValSrc F{f};
    double x, y, z, E[6], e[6], sg[6];
    tdcs_point(F, X, Y, Z, x, y, z);
    tdcs_strain_general(F, x, y, z, bx, by, bz, nu, k, E);
    tdcs_to_efcs(F, E, e);
    hooke(e, mu, lam, sg);
    for (int q = 0; q < 6; ++q) { stress[6 * j + q] = sg[q]; strain[6 * j + q] = e[q]; }
}

static inline double poisson(double mu, double lam) { return 1.0 / (1.0 + lam / mu) / 2.0; }
static inline double kfac(double nu) { return 1.0 / (8.0 * kPi * (1.0 - nu)); }

// ---------------------------------------------------------------------------
// host-pointer context: one stream and one growing device buffer per host thread
struct HostCtx {
    int device = -1;
    cudaStream_t stream = nullptr;
    double *buf = nullptr;
    size_t cap = 0;   // doubles
};
static thread_local HostCtx g_ctx;

static int host_ctx(size_t need_doubles, HostCtx **out)
{
    int dev = 0;
    PQ3D_CUDA_TRY(cudaGetDevice(&dev));
    HostCtx &c = g_ctx;
    if (c.device != dev) {
        c = HostCtx();
        c.device = dev;
        PQ3D_CUDA_TRY(cudaStreamCreateWithFlags(&c.stream, cudaStreamNonBlocking));
    }
    if (c.cap < need_doubles) {
        if (c.buf) cudaFree(c.buf);
        c.buf = nullptr;
        size_t cap = std::max<size_t>(need_doubles, 1 << 16);
        PQ3D_CUDA_TRY(cudaMalloc(&c.buf, cap * sizeof(double)));
        c.cap = cap;
    }
    *out = &c;
    return PQ3D_OK;
}

static void nan_fill(double *p, size_t n)
{
    if (!p) return;
    for (size_t i = 0; i < n; ++i) p[i] = NAN;
}

// The reference prints this and carries on (src/TDstressFS_C.cpp:1949-1953).
static void warn_halfspace_z(const double *X, const double *Y, const double *Z, size_t n, const double *P1,
                             const double *P2, const double *P3)
{
    (void)X; (void)Y;
    bool bad = (P1 && P1[2] > 0.0) || (P2 && P2[2] > 0.0) || (P3 && P3[2] > 0.0);
    for (size_t i = 0; i < n && !bad; ++i) bad = Z[i] > 0.0;
    if (bad) fprintf(stdout, "Half-space solution: Z coordinates must be negative!\n");
}

static int points_one_source(const double *X, const double *Y, const double *Z, size_t n, const double *P1,
                             const double *P2, const double *P3, double Ss, double Ds, double Ts, double mu,
                             double lam, bool half, double *stress, double *strain)
{
    clear_error();
    if (n == 0) return PQ3D_OK;
    PQ3D_REQUIRE(X && Y && Z && P1 && P2 && P3 && stress && strain, "TDstressFS_C: null pointer");
    if (half) warn_halfspace_z(X, Y, Z, n, P1, P2, P3);
    HostCtx *c;
    int rc = host_ctx(15 * n, &c);
    if (rc) return rc;
    double *dX = c->buf, *dY = dX + n, *dZ = dY + n, *dS = dZ + n, *dE = dS + 6 * n;
    PQ3D_CUDA_TRY(cudaMemcpyAsync(dX, X, n * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    PQ3D_CUDA_TRY(cudaMemcpyAsync(dY, Y, n * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    PQ3D_CUDA_TRY(cudaMemcpyAsync(dZ, Z, n * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    SrcVal s;
    double a[3] = {P1[0], P1[1], P1[2]}, b[3] = {P2[0], P2[1], P2[2]}, cc[3] = {P3[0], P3[1], P3[2]};
    setup_source(a, b, cc, s.f, 1);
    const double nu = poisson(mu, lam);
    const int threads = 128;
    if (half) {
        SrcVal si;
        FscVal g;
        double am[3] = {a[0], a[1], -a[2]}, bm[3] = {b[0], b[1], -b[2]}, cm[3] = {cc[0], cc[1], -cc[2]};
        setup_source(am, bm, cm, si.f, 1);
        setup_fsc(a, b, cc, g.f, 1);
        points_one_source_hs_kernel<<<(unsigned)((n + threads - 1) / threads), threads, 0, c->stream>>>(
            s, si, g, dX, dY, dZ, (int64_t)n, Ts, Ss, Ds, mu, lam, nu, kfac(nu), dS, dE);
    } else {
        points_one_source_kernel<<<(unsigned)((n + threads - 1) / threads), threads, 0, c->stream>>>(
            s, dX, dY, dZ, (int64_t)n, Ts, Ss, Ds, mu, lam, nu, kfac(nu), dS, dE);
    }
    PQ3D_CUDA_TRY(cudaGetLastError());
    PQ3D_CUDA_TRY(cudaMemcpyAsync(stress, dS, 6 * n * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    PQ3D_CUDA_TRY(cudaMemcpyAsync(strain, dE, 6 * n * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    PQ3D_CUDA_TRY(cudaStreamSynchronize(c->stream));
    return PQ3D_OK;
}

static int point_many_sources(double x, double y, double z, const double *P1, const double *P2, const double *P3,
                              size_t ns, double Ss, double Ds, double Ts, double mu, double lam, bool half,
                              double *stress, double *strain)
{
    clear_error();
    if (ns == 0) return PQ3D_OK;
    PQ3D_REQUIRE(P1 && P2 && P3 && stress && strain, "TDstressEachSourceAtReceiver_C: null pointer");
    if (half) warn_halfspace_z(&x, &y, &z, 1, nullptr, nullptr, nullptr);
    HostCtx *c;
    int rc = host_ctx(21 * ns, &c);
    if (rc) return rc;
    double *d1 = c->buf, *d2 = d1 + 3 * ns, *d3 = d2 + 3 * ns, *dS = d3 + 3 * ns, *dE = dS + 6 * ns;
    PQ3D_CUDA_TRY(cudaMemcpyAsync(d1, P1, 3 * ns * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    PQ3D_CUDA_TRY(cudaMemcpyAsync(d2, P2, 3 * ns * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    PQ3D_CUDA_TRY(cudaMemcpyAsync(d3, P3, 3 * ns * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    const double nu = poisson(mu, lam);
    const int threads = 128;
    if (half)
        point_many_sources_hs_kernel<<<(unsigned)((ns + threads - 1) / threads), threads, 0, c->stream>>>(
            x, y, z, d1, d2, d3, (int64_t)ns, Ts, Ss, Ds, mu, lam, nu, kfac(nu), dS, dE);
    else
        point_many_sources_kernel<<<(unsigned)((ns + threads - 1) / threads), threads, 0, c->stream>>>(
            x, y, z, d1, d2, d3, (int64_t)ns, Ts, Ss, Ds, mu, lam, nu, kfac(nu), dS, dE);
    PQ3D_CUDA_TRY(cudaGetLastError());
    PQ3D_CUDA_TRY(cudaMemcpyAsync(stress, dS, 6 * ns * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    PQ3D_CUDA_TRY(cudaMemcpyAsync(strain, dE, 6 * ns * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    PQ3D_CUDA_TRY(cudaStreamSynchronize(c->stream));
    return PQ3D_OK;
}

// Workspace: source table [kSrcStride][N], receiver table [N][kRecvStride],
// then (half-space) image table [kImgStride][N] and side table [kFscStride][N].
static size_t ws_bytes(int64_t N, bool half)
{
    return (size_t)N * (kSrcStride + kRecvStride + (half ? kImgStride + kFscStride : 0)) * sizeof(double);
}

static int assemble_rows(const double *nodes, const int64_t *tris, int64_t N, int64_t row0, int64_t row1, double mu,
                         double lam, double *K64, float *K32, double *src, double *recv, bool do_setup,
                         cudaStream_t st, bool half = false)
{
    double *img = recv + (size_t)kRecvStride * N, *fsc = img + (size_t)kImgStride * N;
    if (do_setup) {
        const int th = 128;
        const unsigned nb = (unsigned)((N + th - 1) / th);
        setup_sources_kernel<<<nb, th, 0, st>>>(nodes, tris, N, src);
        setup_receivers_kernel<<<nb, th, 0, st>>>(nodes, tris, N, recv);
        if (half) setup_hs_kernel<<<nb, th, 0, st>>>(nodes, tris, N, img, fsc);
        PQ3D_CUDA_TRY(cudaGetLastError());
    }
    const double nu = poisson(mu, lam);
    dim3 grid((unsigned)((N + kTJ - 1) / kTJ), (unsigned)((row1 - row0 + kTI - 1) / kTI));
    if (half) {
        if (K32)
            assemble_dense_hs_kernel<true><<<grid, kTJ, 0, st>>>(src, recv, img, fsc, N, row0, row1, nu, kfac(nu),
                                                                2.0 * mu, lam, K64, K32);
        else
            assemble_dense_hs_kernel<false><<<grid, kTJ, 0, st>>>(src, recv, img, fsc, N, row0, row1, nu, kfac(nu),
                                                                 2.0 * mu, lam, K64, K32);
    } else if (K32)
        assemble_dense_kernel<true><<<grid, kTJ, 0, st>>>(src, recv, N, row0, row1, nu, kfac(nu), 2.0 * mu, lam,
                                                         K64, K32);
    else
        assemble_dense_kernel<false><<<grid, kTJ, 0, st>>>(src, recv, N, row0, row1, nu, kfac(nu), 2.0 * mu, lam,
                                                          K64, K32);
    PQ3D_CUDA_TRY(cudaGetLastError());
    return PQ3D_OK;
}

// ---------------------------------------------------------------------------
// Fixed scratch for pq3d_assemble_dense_noalloc: the source and receiver
// tables of one call (kSrcStride + kRecvStride doubles per element) for up to
// kNoAllocMaxN elements, 14.2 MB held by every GPU that loads this library.
constexpr int64_t kNoAllocMaxN = 32768;
static __device__ __align__(256) double g_noalloc_scratch[(size_t)(kSrcStride + kRecvStride) * kNoAllocMaxN];

// Device address of the fixed scratch on the current device, looked up with
// that device current on every call (cheap): a cached address would go stale
// if the device were reset or its primary context recreated between calls.
static int noalloc_scratch(double **out)
{
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p)
        return set_error(PQ3D_ERR_CUDA, "pq3d_assemble_dense_noalloc: cudaGetSymbolAddress failed: %s",
                         cudaGetErrorString(e));
    *out = (double *)p;
    return PQ3D_OK;
}

}  // namespace gf
}  // namespace pq3d

using namespace pq3d;
using namespace pq3d::gf;

extern "C" void TDstressFS_C(const double *X, const double *Y, const double *Z, size_t n, const double *P1,
                             const double *P2, const double *P3, double Ss, double Ds, double Ts, double mu,
                             double lambda_, bool jud_halfspace, double *stress, double *strain)
{
    int rc = points_one_source(X, Y, Z, n, P1, P2, P3, Ss, Ds, Ts, mu, lambda_, jud_halfspace, stress, strain);
    if (rc != PQ3D_OK) {
        fprintf(stderr, "pq3d: %s\n", pq3d_last_error());
        nan_fill(stress, 6 * n);
        nan_fill(strain, 6 * n);
    }
}

extern "C" void TDstressEachSourceAtReceiver_C(double x, double y, double z, const double *P1_flat,
                                               const double *P2_flat, const double *P3_flat, size_t n_sources,
                                               double Ss, double Ds, double Ts, double mu, double lambda_,
                                               bool jud_halfspace, double *stress_out, double *strain_out)
{
    int rc = point_many_sources(x, y, z, P1_flat, P2_flat, P3_flat, n_sources, Ss, Ds, Ts, mu, lambda_,
                                jud_halfspace, stress_out, strain_out);
    if (rc != PQ3D_OK) {
        fprintf(stderr, "pq3d: %s\n", pq3d_last_error());
        nan_fill(stress_out, 6 * n_sources);
        nan_fill(strain_out, 6 * n_sources);
    }
}

extern "C" void TDstressFS_C1(const double *X, const double *Y, const double *Z, size_t n, const double *P1,
                              const double *P2, const double *P3, double Ss, double Ds, double Ts, double mu,
                              double lambda_, double *Sxx, double *Syy, double *Szz, double *Sxy, double *Sxz,
                              double *Syz, double *Exx, double *Eyy, double *Ezz, double *Exy, double *Exz,
                              double *Eyz)
{
    std::vector<double> s(6 * n), e(6 * n);
    int rc = points_one_source(X, Y, Z, n, P1, P2, P3, Ss, Ds, Ts, mu, lambda_, false, s.data(), e.data());
    if (rc != PQ3D_OK) {
        fprintf(stderr, "pq3d: %s\n", pq3d_last_error());
        std::fill(s.begin(), s.end(), NAN);
        std::fill(e.begin(), e.end(), NAN);
    }
    double *S[6] = {Sxx, Syy, Szz, Sxy, Sxz, Syz}, *E[6] = {Exx, Eyy, Ezz, Exy, Exz, Eyz};
    for (size_t i = 0; i < n; ++i)
        for (int c = 0; c < 6; ++c) {
            S[c][i] = s[6 * i + c];
            E[c][i] = e[6 * i + c];
        }
}

// the size that serves both full- and half-space assemblies
extern "C" size_t pq3d_gf_workspace_bytes(int64_t N) { return N > 0 ? ws_bytes(N, true) : 0; }

extern "C" int pq3d_assemble_dense(const double *nodes, const int64_t *tris, int64_t N, int64_t row0, int64_t row1,
                                   double mu, double lambda_, int halfspace, double *K64, float *K32, void *workspace,
                                   size_t workspace_bytes, void *stream)
{
    clear_error();
    PQ3D_REQUIRE(N > 0 && row0 >= 0 && row1 <= N && row0 <= row1, "pq3d_assemble_dense: bad sizes");
    PQ3D_REQUIRE(nodes && tris && K64 && workspace, "pq3d_assemble_dense: null pointer");
    PQ3D_REQUIRE(aligned16(K64) && (!K32 || ((uintptr_t)K32 & 7u) == 0) && aligned16(workspace),
                 "pq3d_assemble_dense: K64/workspace must be 16-byte aligned, K32 8-byte aligned");
    PQ3D_REQUIRE(workspace_bytes >= ws_bytes(N, halfspace != 0), "pq3d_assemble_dense: workspace too small (%zu < %zu)",
                 workspace_bytes, ws_bytes(N, halfspace != 0));
    if (row0 == row1) return PQ3D_OK;
    double *src = (double *)workspace;
    double *recv = src + (size_t)kSrcStride * N;
    return assemble_rows(nodes, tris, N, row0, row1, mu, lambda_, K64, K32, src, recv, true, (cudaStream_t)stream,
                         halfspace != 0);
}

// Device address of page-locked host memory mapped into the device address
// space (cudaHostAlloc / cudaHostRegister under unified addressing), else NULL.
static void *mapped_device_ptr(void *host)
{
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, host) != cudaSuccess) {
        (void)cudaGetLastError();
        return nullptr;
    }
    return (a.type == cudaMemoryTypeHost) ? a.devicePointer : nullptr;
}

// Output already in mapped page-locked host memory: the assembly kernel
// stores straight into it (its output rate, ~40 GB/s at N = 20,000, is far
// below the host link's), one launch over all rows, no staging buffers and
// no separate copies.
static int assemble_host_direct(const double *nodes_host, int64_t n_nodes, const int64_t *tris_host, int64_t N,
                                double mu, double lambda_, bool half, double *dK64, float *dK32)
{
    double *d_nodes = nullptr, *d_ws = nullptr;
    int64_t *d_tris = nullptr;
    cudaStream_t st = nullptr;
    int rc = PQ3D_OK;
#define PQ3D_D_TRY(call)                                                                              \
    do {                                                                                              \
        cudaError_t e_ = (call);                                                                      \
        if (e_ != cudaSuccess) {                                                                      \
            rc = set_error(PQ3D_ERR_CUDA, "pq3d_assemble_dense_host: %s: %s", #call, cudaGetErrorString(e_)); \
            goto done;                                                                                \
        }                                                                                             \
    } while (0)
    PQ3D_D_TRY(cudaMalloc(&d_nodes, 3 * n_nodes * sizeof(double)));
    PQ3D_D_TRY(cudaMalloc(&d_tris, 3 * N * sizeof(int64_t)));
    PQ3D_D_TRY(cudaMalloc(&d_ws, ws_bytes(N, half)));
    PQ3D_D_TRY(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    PQ3D_D_TRY(cudaMemcpyAsync(d_nodes, nodes_host, 3 * n_nodes * sizeof(double), cudaMemcpyHostToDevice, st));
    PQ3D_D_TRY(cudaMemcpyAsync(d_tris, tris_host, 3 * N * sizeof(int64_t), cudaMemcpyHostToDevice, st));
    rc = assemble_rows(d_nodes, d_tris, N, 0, N, mu, lambda_, dK64, dK32, d_ws, d_ws + (size_t)kSrcStride * N, true,
                       st, half);
    if (rc) goto done;
    PQ3D_D_TRY(cudaStreamSynchronize(st));
done:
#undef PQ3D_D_TRY
    if (st) { cudaStreamSynchronize(st); cudaStreamDestroy(st); }
    cudaFree(d_nodes);
    cudaFree(d_tris);
    cudaFree(d_ws);
    return rc;
}

extern "C" int pq3d_assemble_dense_host(const double *nodes_host, int64_t n_nodes, const int64_t *tris_host,
                                        int64_t N, double mu, double lambda_, int halfspace, double *K64_host,
                                        float *K32_host)
{
    clear_error();
    PQ3D_REQUIRE(N > 0 && n_nodes > 0 && nodes_host && tris_host && K64_host, "pq3d_assemble_dense_host: bad args");
    const bool half = halfspace != 0;
    {
        double *dK64 = (double *)mapped_device_ptr(K64_host);
        float *dK32 = K32_host ? (float *)mapped_device_ptr(K32_host) : nullptr;
        if (dK64 && aligned16(dK64) && (!K32_host || (dK32 && ((uintptr_t)dK32 & 7u) == 0)))
            return assemble_host_direct(nodes_host, n_nodes, tris_host, N, mu, lambda_, half, dK64, dK32);
    }
    const size_t ld = 2 * (size_t)N;
    // rows per block: about 256 MB of FP64 output per block
    int64_t rb = std::max<int64_t>(kTI, ((int64_t)(256u << 20) / (int64_t)(3 * ld * sizeof(double))) / kTI * kTI);
    rb = std::min<int64_t>(rb, N);
    double *d_nodes = nullptr, *d_ws = nullptr, *d_K64[2] = {nullptr, nullptr};
    float *d_K32[2] = {nullptr, nullptr};
    int64_t *d_tris = nullptr;
    cudaStream_t st[2] = {nullptr, nullptr};
    cudaEvent_t setup_done = nullptr;
    int rc = PQ3D_OK;
#define PQ3D_H_TRY(call)                                                                              \
    do {                                                                                              \
        cudaError_t e_ = (call);                                                                      \
        if (e_ != cudaSuccess) {                                                                      \
            rc = set_error(PQ3D_ERR_CUDA, "pq3d_assemble_dense_host: %s: %s", #call, cudaGetErrorString(e_)); \
            goto done;                                                                                \
        }                                                                                             \
    } while (0)
    PQ3D_H_TRY(cudaMalloc(&d_nodes, 3 * n_nodes * sizeof(double)));
    PQ3D_H_TRY(cudaMalloc(&d_tris, 3 * N * sizeof(int64_t)));
    PQ3D_H_TRY(cudaMalloc(&d_ws, ws_bytes(N, half)));
    for (int b = 0; b < 2; ++b) {
        PQ3D_H_TRY(cudaMalloc(&d_K64[b], 3 * rb * ld * sizeof(double)));
        if (K32_host) PQ3D_H_TRY(cudaMalloc(&d_K32[b], 3 * rb * ld * sizeof(float)));
        PQ3D_H_TRY(cudaStreamCreateWithFlags(&st[b], cudaStreamNonBlocking));
    }
    PQ3D_H_TRY(cudaEventCreateWithFlags(&setup_done, cudaEventDisableTiming));
    PQ3D_H_TRY(cudaMemcpyAsync(d_nodes, nodes_host, 3 * n_nodes * sizeof(double), cudaMemcpyHostToDevice, st[0]));
    PQ3D_H_TRY(cudaMemcpyAsync(d_tris, tris_host, 3 * N * sizeof(int64_t), cudaMemcpyHostToDevice, st[0]));
    {
        double *src = d_ws, *recv = d_ws + (size_t)kSrcStride * N;
        const int th = 128;
        const unsigned nb = (unsigned)((N + th - 1) / th);
        setup_sources_kernel<<<nb, th, 0, st[0]>>>(d_nodes, d_tris, N, src);
        setup_receivers_kernel<<<nb, th, 0, st[0]>>>(d_nodes, d_tris, N, recv);
        if (half) {
            double *img = recv + (size_t)kRecvStride * N;
            setup_hs_kernel<<<nb, th, 0, st[0]>>>(d_nodes, d_tris, N, img, img + (size_t)kImgStride * N);
        }
        PQ3D_H_TRY(cudaGetLastError());
        PQ3D_H_TRY(cudaEventRecord(setup_done, st[0]));
        PQ3D_H_TRY(cudaStreamWaitEvent(st[1], setup_done, 0));
        int blk = 0;
        for (int64_t r0 = 0; r0 < N; r0 += rb, ++blk) {
            const int b = blk & 1;
            const int64_t r1 = std::min<int64_t>(N, r0 + rb);
            rc = assemble_rows(d_nodes, d_tris, N, r0, r1, mu, lambda_, d_K64[b], d_K32[b], src, recv, false, st[b],
                               half);
            if (rc) goto done;
            PQ3D_H_TRY(cudaMemcpyAsync(K64_host + 3 * r0 * ld, d_K64[b], 3 * (r1 - r0) * ld * sizeof(double),
                                       cudaMemcpyDeviceToHost, st[b]));
            if (K32_host)
                PQ3D_H_TRY(cudaMemcpyAsync(K32_host + 3 * r0 * ld, d_K32[b], 3 * (r1 - r0) * ld * sizeof(float),
                                           cudaMemcpyDeviceToHost, st[b]));
        }
        PQ3D_H_TRY(cudaStreamSynchronize(st[0]));
        PQ3D_H_TRY(cudaStreamSynchronize(st[1]));
    }
done:
#undef PQ3D_H_TRY
    for (int b = 0; b < 2; ++b) {
        if (st[b]) { cudaStreamSynchronize(st[b]); cudaStreamDestroy(st[b]); }
        cudaFree(d_K64[b]);
        cudaFree(d_K32[b]);
    }
    if (setup_done) cudaEventDestroy(setup_done);
    cudaFree(d_nodes);
    cudaFree(d_tris);
    cudaFree(d_ws);
    return rc;
}

extern "C" int pq3d_assemble_dense_noalloc(const double *nodes, const int64_t *tris, int64_t N, int64_t row0,
                                           int64_t row1, double mu, double lambda_, int halfspace, double *K64,
                                           float *K32, void *stream)
{
    clear_error();
    PQ3D_REQUIRE(N > 0 && row0 >= 0 && row1 <= N && row0 <= row1, "pq3d_assemble_dense_noalloc: bad sizes");
    PQ3D_REQUIRE(N <= kNoAllocMaxN, "pq3d_assemble_dense_noalloc: N = %lld exceeds the fixed scratch limit of %lld "
                 "elements (use pq3d_assemble_dense with a caller-provided workspace)", (long long)N,
                 (long long)kNoAllocMaxN);
    PQ3D_REQUIRE(nodes && tris && K64, "pq3d_assemble_dense_noalloc: null pointer");
    PQ3D_REQUIRE(aligned16(K64) && (!K32 || ((uintptr_t)K32 & 7u) == 0),
                 "pq3d_assemble_dense_noalloc: K64 must be 16-byte aligned, K32 8-byte aligned");
    if (halfspace)
        return set_error(PQ3D_ERR_UNSUPPORTED, "pq3d_assemble_dense_noalloc: the fixed scratch holds the full-space "
                         "tables only; use pq3d_assemble_dense for the half-space");
    double *scratch = nullptr;
    int rc = noalloc_scratch(&scratch);
    if (rc) return rc;
    if (row0 == row1) return PQ3D_OK;
    // every table entry the assembly reads is rewritten by this call's set-up
    // kernels, so nothing has to be cleared between calls
    return assemble_rows(nodes, tris, N, row0, row1, mu, lambda_, K64, K32, scratch, scratch + (size_t)kSrcStride * N,
                         true, (cudaStream_t)stream);
}

extern "C" int pq3d_gf_setup(const double *nodes, const int64_t *tris, int64_t N, int halfspace, void *workspace,
                             size_t workspace_bytes, void *stream)
{
    clear_error();
    PQ3D_REQUIRE(nodes && tris && workspace && N > 0, "pq3d_gf_setup: bad arguments");
    PQ3D_REQUIRE(workspace_bytes >= ws_bytes(N, halfspace != 0) && aligned16(workspace),
                 "pq3d_gf_setup: workspace too small");
    double *src = (double *)workspace;
    double *recv = src + (size_t)kSrcStride * N;
    const int th = 128;
    const unsigned nb = (unsigned)((N + th - 1) / th);
    setup_sources_kernel<<<nb, th, 0, (cudaStream_t)stream>>>(nodes, tris, N, src);
    setup_receivers_kernel<<<nb, th, 0, (cudaStream_t)stream>>>(nodes, tris, N, recv);
    if (halfspace) {
        double *img = recv + (size_t)kRecvStride * N;
        setup_hs_kernel<<<nb, th, 0, (cudaStream_t)stream>>>(nodes, tris, N, img, img + (size_t)kImgStride * N);
    }
    PQ3D_CUDA_TRY(cudaGetLastError());
    return PQ3D_OK;
}
