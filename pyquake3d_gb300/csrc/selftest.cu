// Self-tests of the bounded device waits: a wait whose partner never arrives
// must give up after its iteration limit, report through the status the host
// reads, and let every thread return with the context still usable.  They
// exercise the same primitives the steppers and the tensor-core products use
// (grid_barrier, tc::mbar_wait), with a lowered limit so that a test takes
// milliseconds.  Nothing here faults or waits without a bound.  Also: the
// integer FP64 <-> float-float conversions of the float-float attempt on
// host-chosen values (subnormal, infinite and NaN operands included), which
// the steppers reach only through rare states; and the assembly's
// configuration test (FP32 decisions with a division-based fallback) against
// the division-based test on host-chosen points.
#include <cuda_runtime.h>

#include "common.cuh"
#include "gf_device.cuh"
#include "rk_device.cuh"
#include "tc_ptx.cuh"

namespace pq3d {
namespace selftest {

// Every block but `skip` arrives at one grid barrier; the arriving blocks
// time out.  returned[b] once block b leaves: 1 = gave up, 2 = passed the
// barrier, 3 = the block that skipped it.
__global__ void barrier_kernel(unsigned *bar, int skip, unsigned limit, int *returned, int *status)
{
    const unsigned nb = gridDim.x;
    bool ok = true;
    if ((int)blockIdx.x != skip) {
        ok = grid_barrier(bar, bar + 1, nb, limit);
        if (!ok && threadIdx.x == 0) atomicExch(status, PQ3D_ERR_TIMEOUT);
    }
    if (threadIdx.x == 0) returned[blockIdx.x] = (int)blockIdx.x == skip ? 3 : (ok ? 2 : 1);
}

// An mbarrier (arrival count 1) that nobody arrives at: every thread waits
// with the bounded wait of the tensor-core kernels and records when it gave up.
__global__ void mbar_kernel(uint32_t limit, int *gave_up, int *err)
{
    __shared__ __align__(8) unsigned long long bar;
    const uint32_t b = tc::smem_u32(&bar);
    if (threadIdx.x == 0) {
        tc::mbar_init(b, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    const bool ok = tc::mbar_wait(b, 0, limit);
    if (!ok) {
        atomicAdd(gave_up, 1);
        if (threadIdx.x == 0) atomicExch(err, 2);
    }
}

// The conversions of the float-float attempt on n values: ff_split_fast(x),
// f2d_bits(f), and |(x, y)| by ff_hypot of the two splits, back to FP64.
__global__ void ffconv_kernel(const double *x, const float *f, const double *y, int n, float *ff, double *d,
                              double *h)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const rk::FF a = rk::ff_split_fast(x[i]);
    ff[2 * i] = a.hi;
    ff[2 * i + 1] = a.lo;
    d[i] = rk::f2d_bits(f[i]);
    h[i] = rk::ff_to_double_fast(rk::ff_hypot(a, rk::ff_split_fast(y[i])));
}

}  // namespace selftest
}  // namespace pq3d

using namespace pq3d;

extern "C" int pq3d_selftest_barrier_timeout(int nblocks, int skip_block, unsigned spin_limit, int *returned_host)
{
    clear_error();
    PQ3D_REQUIRE(nblocks >= 1 && nblocks <= 64 && returned_host, "pq3d_selftest_barrier_timeout: bad arguments");
    PQ3D_REQUIRE(spin_limit >= 1 && spin_limit <= (1u << 16), "pq3d_selftest_barrier_timeout: limit 1..65536");
    int dev, coop = 0, per_sm = 0, sms = 0;
    PQ3D_CUDA_TRY(cudaGetDevice(&dev));
    PQ3D_CUDA_TRY(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev));
    PQ3D_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    PQ3D_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, selftest::barrier_kernel, 32, 0));
    PQ3D_REQUIRE(coop && nblocks <= per_sm * sms, "pq3d_selftest_barrier_timeout: cooperative launch unavailable");
    void *mem = nullptr;
    PQ3D_CUDA_TRY(cudaMalloc(&mem, 256 + 4 * 64));
    unsigned *bar = (unsigned *)mem;
    int *status = (int *)((char *)mem + 8);
    int *returned = (int *)((char *)mem + 256);
    int rc = PQ3D_OK;
    cudaError_t e = cudaMemset(mem, 0, 256 + 4 * 64);
    if (e == cudaSuccess) {
        void *args[] = {&bar, &skip_block, &spin_limit, &returned, &status};
        e = cudaLaunchCooperativeKernel((const void *)selftest::barrier_kernel, dim3(nblocks), dim3(32), args, 0, 0);
    }
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    int st = 0;
    if (e == cudaSuccess) e = cudaMemcpy(&st, status, sizeof(int), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(returned_host, returned, sizeof(int) * nblocks, cudaMemcpyDeviceToHost);
    cudaFree(mem);
    if (e != cudaSuccess) return set_error(PQ3D_ERR_CUDA, "pq3d_selftest_barrier_timeout: %s", cudaGetErrorString(e));
    if (st) rc = set_error(st, "grid barrier gave up after %u iterations", spin_limit);
    return rc;
}

extern "C" int pq3d_selftest_mbar_timeout(unsigned wait_limit, int *gave_up_host)
{
    clear_error();
    PQ3D_REQUIRE(gave_up_host && wait_limit >= 1 && wait_limit <= (1u << 16), "pq3d_selftest_mbar_timeout: bad arguments");
    void *mem = nullptr;
    PQ3D_CUDA_TRY(cudaMalloc(&mem, 16));
    int *gave_up = (int *)mem, *err = gave_up + 1;
    cudaError_t e = cudaMemset(mem, 0, 16);
    if (e == cudaSuccess) {
        selftest::mbar_kernel<<<1, 128>>>(wait_limit, gave_up, err);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    int h[2] = {0, 0};
    if (e == cudaSuccess) e = cudaMemcpy(h, mem, sizeof(h), cudaMemcpyDeviceToHost);
    cudaFree(mem);
    if (e != cudaSuccess) return set_error(PQ3D_ERR_CUDA, "pq3d_selftest_mbar_timeout: %s", cudaGetErrorString(e));
    *gave_up_host = h[0];
    return h[1] ? set_error(PQ3D_ERR_TIMEOUT, "mbarrier wait gave up after %u tries (error word %d)", wait_limit, h[1])
                : PQ3D_OK;
}

extern "C" int pq3d_selftest_ff_conversions(const double *x_host, const float *f_host, const double *y_host, int n,
                                            float *ff_host, double *d_host, double *h_host)
{
    clear_error();
    PQ3D_REQUIRE(x_host && f_host && y_host && ff_host && d_host && h_host && n >= 1 && n <= (1 << 20),
                 "pq3d_selftest_ff_conversions: bad arguments");
    const size_t nd = (size_t)n * sizeof(double), nf = (size_t)n * sizeof(float);
    void *mem = nullptr;
    PQ3D_CUDA_TRY(cudaMalloc(&mem, 4 * nd + 3 * nf + 64));
    char *p = (char *)mem;
    double *x = (double *)p, *y = x + n, *d = y + n, *h = d + n;
    float *f = (float *)(h + n), *ff = f + n;
    cudaError_t e = cudaMemcpy(x, x_host, nd, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(y, y_host, nd, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(f, f_host, nf, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        selftest::ffconv_kernel<<<(n + 127) / 128, 128>>>(x, f, y, n, ff, d, h);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    if (e == cudaSuccess) e = cudaMemcpy(ff_host, ff, 2 * nf, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(d_host, d, nd, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(h_host, h, nd, cudaMemcpyDeviceToHost);
    cudaFree(mem);
    if (e != cudaSuccess) return set_error(PQ3D_ERR_CUDA, "pq3d_selftest_ff_conversions: %s", cudaGetErrorString(e));
    return PQ3D_OK;
}

namespace pq3d {
namespace selftest {

// pts[i] = (x, y, z, p1y, p1z, p3y, p3z, den): the assembly's configuration
// test (tri_mode_fast, reciprocal of den as the source record holds it) and
// the division-based one (tri_mode) on the same point.
__global__ void tri_mode_kernel(const double *pts, int n, int *fast, int *exact)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double *q = pts + 8 * (size_t)i;
    fast[i] = gf::tri_mode_fast(q[0], q[1], q[2], q[3], q[4], q[5], q[6], q[7], 1.0 / q[7]);
    exact[i] = gf::tri_mode<double>(q[0], q[1], q[2], q[3], q[4], q[5], q[6], q[7]);
}

}  // namespace selftest
}  // namespace pq3d

extern "C" int pq3d_selftest_tri_mode(const double *pts_host, int n, int *fast_host, int *exact_host)
{
    clear_error();
    PQ3D_REQUIRE(pts_host && fast_host && exact_host && n >= 1 && n <= (1 << 22),
                 "pq3d_selftest_tri_mode: bad arguments");
    const size_t np = (size_t)n * 8 * sizeof(double), ni = (size_t)n * sizeof(int);
    void *mem = nullptr;
    PQ3D_CUDA_TRY(cudaMalloc(&mem, np + 2 * ni));
    double *pts = (double *)mem;
    int *fast = (int *)((char *)mem + np), *exact = fast + n;
    cudaError_t e = cudaMemcpy(pts, pts_host, np, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        selftest::tri_mode_kernel<<<(n + 255) / 256, 256>>>(pts, n, fast, exact);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    if (e == cudaSuccess) e = cudaMemcpy(fast_host, fast, ni, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(exact_host, exact, ni, cudaMemcpyDeviceToHost);
    cudaFree(mem);
    if (e != cudaSuccess) return set_error(PQ3D_ERR_CUDA, "pq3d_selftest_tri_mode: %s", cudaGetErrorString(e));
    return PQ3D_OK;
}
