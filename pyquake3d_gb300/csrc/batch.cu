// Batched ensemble stepping: B simulations that share one mesh (one traction
// operator) and differ in friction, stress and nucleation, stepped together.
//
// One iteration (graph-capturable, no host synchronisation):
//   1. operator product for all runs at once:  rates[.][r] = K . v'_r
//      (a GEMM (3N x 2N) x (2N x B) instead of B matrix-vector products)
//   2. attempt: one Dormand-Prince 5(4) attempt per (run, cell) with the run's
//      own dt, per-run max error norms by one atomicMax per block
//   3. decide: per run accept/reject and the next dt (src/QDsim_gpu.py:959-985)
//   4. update: accepted runs advance (slip rate, slip, v'); rejected runs keep
//      their state and retry with the smaller dt at the next iteration
//      ("masked stage acceptance": every run keeps its own step sequence).
// Semantics per run are those of the single-simulation stepper (step.cu) and
// the reference CPU path (src/QDsim_gpu.py:1029-1122).
#include <cuda_bf16.h>
#include <math.h>

#include "common.cuh"
#include "gemm_fix.cuh"
#include "gemm_tc.cuh"
#include "rk_device.cuh"

namespace pq3d {
namespace batch {

using namespace ::pq3d::rk;


// padded run count of the operator right-hand side and of the rate partials
__host__ __device__ inline int padded_runs(int B) { return (B + 15) / 16 * 16; }

// cells of the whole mesh (a row shard holds N of them, from cell0)
__host__ __device__ inline int64_t total_cells(const pq3d_batch_sim &S) { return S.N_total > 0 ? S.N_total : S.N; }

// ---------------------------------------------------------------------------
// operator right-hand side v'_r = V_r - Vpl (cos, sin)(rake0), interleaved

__device__ __forceinline__ void vprime(const pq3d_batch_sim &S, int64_t idx, double &v1, double &v2)
{
    v1 = S.slipv1[idx] - S.Vpl * S.cos_rake0[idx];
    v2 = S.slipv2[idx] - S.Vpl * S.sin_rake0[idx];
}

// 3-piece BF16 split of an FP32 value: x = p0 + p1 + p2 exactly (each
// residual is exact in FP32 and has 8 fewer significant bits than the last)
// x = p0 + p1 + p2 to ~2^-26 relative (each piece rounds the remainder of the
// previous ones to BF16), the remainders formed exactly in FP64
__device__ __forceinline__ void split3(double x, __nv_bfloat16 &p0, __nv_bfloat16 &p1, __nv_bfloat16 &p2)
{
    p0 = __double2bfloat16(x);
    const double r1 = x - (double)__bfloat162float(p0);
    p1 = __double2bfloat16(r1);
    p2 = __double2bfloat16(r1 - (double)__bfloat162float(p1));
}

// the same for an FP32 value (exact: 24 bits in three 8-bit pieces), on the
// FP32 pipe
__device__ __forceinline__ void split3(float x, __nv_bfloat16 &p0, __nv_bfloat16 &p1, __nv_bfloat16 &p2)
{
    p0 = __float2bfloat16_rn(x);
    const float r1 = x - __bfloat162float(p0);
    p1 = __float2bfloat16_rn(r1);
    p2 = __float2bfloat16_rn(r1 - __bfloat162float(p1));
}

// i: local cell of the shard; v' goes to the mesh-wide position cell0 + i
// kExactV: v' carries an FP64 slip rate (the FP64 attempt and update) and is
// split from FP64; otherwise the slip rate is the mixed update's FP32 value,
// v' has its 24 bits at most and the split runs on the FP32 pipe.
template <bool kExactV>
__device__ __forceinline__ void write_vop(const pq3d_batch_sim &S, int r, int64_t i, double v1, double v2)
{
    if (S.precision == PQ3D_BATCH_BF16X18) return;   // packed per chunk after the update (fx::pack_rhs_from_state)
    const int Bp = padded_runs(S.B);
    const int64_t o = (int64_t)r * 2 * total_cells(S) + 2 * (S.cell0 + i);
    if (S.precision == PQ3D_BATCH_FP64 || S.precision == PQ3D_BATCH_HMAT) {
        reinterpret_cast<double2 *>((double *)S.vop + o)[0] = make_double2(v1, v2);
    } else if (S.precision == PQ3D_BATCH_FP32) {
        reinterpret_cast<float2 *>((float *)S.vop + o)[0] = make_float2((float)v1, (float)v2);
    } else {
        // packed images [k block][piece][Bp x 32] (see gemm_tc.cuh); never sharded
        const int64_t k = 2 * i;
        const int64_t img = (int64_t)Bp * tc::kBlockK;
        __nv_bfloat16 *P = (__nv_bfloat16 *)S.vop + (k / tc::kBlockK) * tc::kPieces * img +
                           tc::image_offset(r, (int)(k % tc::kBlockK));
        __nv_bfloat16 a0, a1, a2, b0, b1, b2;
        if (kExactV) {
            split3(v1, a0, a1, a2);   // v' to ~26 bits, like the operator's pieces
            split3(v2, b0, b1, b2);
        } else {
            split3((float)v1, a0, a1, a2);
            split3((float)v2, b0, b1, b2);
        }
        __nv_bfloat162 q;
        q.x = a0; q.y = b0; reinterpret_cast<__nv_bfloat162 *>(P)[0] = q;
        q.x = a1; q.y = b1; reinterpret_cast<__nv_bfloat162 *>(P + img)[0] = q;
        q.x = a2; q.y = b2; reinterpret_cast<__nv_bfloat162 *>(P + 2 * img)[0] = q;
    }
}

__device__ __forceinline__ double log_eta_v0(const pq3d_batch_sim &S) { return log(S.eta * S.V0); }

__global__ void prepare_kernel(pq3d_batch_sim S)
{
    const int r = blockIdx.y;
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= S.N) return;
    double v1 = 0.0, v2 = 0.0;
    if (r < S.B) {   // padding runs stay zero
        const int64_t idx = (int64_t)r * S.N + i;
        vprime(S, idx, v1, v2);
        if (S.base) {
            float *pb = S.base + idx;
            const int64_t stride = (int64_t)S.B * S.N;
            store_base_constants(pb, stride, S.a[idx], S.b[idx], S.dc[idx], S.f0[idx]);
            MixedBase m;
            store_base_state(pb, stride, S.Tno[idx], S.Tt1o[idx], S.Tt2o[idx], S.state[idx],
                             ff_split(log_eta_v0(S)), m);
            pb[19 * stride] = (float)S.slipv[idx];
        }
    }
    // the split the update of this precision writes, so that a prepare (a run
    // loaded into another slot) leaves the other runs' v' bit for bit as it was
    if (S.precision != PQ3D_BATCH_FP64 && !S.attempt64) write_vop<false>(S, r, i, v1, v2);
    else write_vop<true>(S, r, i, v1, v2);
}

// ---------------------------------------------------------------------------
// CUDA-core operator products (FP64 and FP32 arms)

// FP64: one warp per (run, receiver): rows 3i..3i+2 (N receivers of the
// shard) against v'_r (Nt sources of the mesh).
__global__ void __launch_bounds__(256) gemm_f64_kernel(const double2 *__restrict__ K, const double2 *__restrict__ V,
                                                       int64_t N, int64_t Nt, int B, double *__restrict__ out)
{
    const int lane = threadIdx.x & 31;
    const int64_t w = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    if (w >= N * B) return;
    const int r = (int)(w / N);
    const int64_t i = w - (int64_t)r * N;
    const double2 *v = V + (int64_t)r * Nt;
    const double2 *r0 = K + 3 * i * Nt, *r1 = r0 + Nt, *r2 = r1 + Nt;
    double a0 = 0, a1 = 0, a2 = 0;
    for (int64_t j = lane; j < Nt; j += 32) {
        const double2 x = v[j], k0 = r0[j], k1 = r1[j], k2 = r2[j];
        a0 = fma(k0.x, x.x, fma(k0.y, x.y, a0));
        a1 = fma(k1.x, x.x, fma(k1.y, x.y, a1));
        a2 = fma(k2.x, x.x, fma(k2.y, x.y, a2));
    }
    for (int o = 16; o > 0; o >>= 1) {
        a0 += __shfl_xor_sync(0xffffffffu, a0, o);
        a1 += __shfl_xor_sync(0xffffffffu, a1, o);
        a2 += __shfl_xor_sync(0xffffffffu, a2, o);
    }
    if (lane == 0) {
        double *o = out + (int64_t)r * 3 * N + 3 * i;
        o[0] = a0; o[1] = a1; o[2] = a2;
    }
}

// FP32: CTA tile 128 rows x 64 runs x one K slice (split-K over gridDim.z:
// the 3N x B outputs alone fill only part of the SMs), K chunks of 32 through
// shared memory (the next chunk is loaded into registers while the current
// one is used), FP32 FMAs with the partial sums moved to FP64 every 256
// columns; the FP64 sums live in dynamic shared memory (64 KB per CTA), which
// keeps the kernel at 2 CTAs per SM.  Each slice writes its FP64 sums; the
// attempt adds them in slice order.  N receivers of the shard (3N rows), Nt
// sources of the mesh (2 Nt columns).
constexpr int kF32Rows = 128, kF32Runs = 64, kF32K = 32;
constexpr int kF32Smem = 32 * 256 * (int)sizeof(double);

__global__ void __launch_bounds__(256, 2) gemm_f32_kernel(const float *__restrict__ K, const float *__restrict__ V,
                                                          int64_t N, int64_t Nt, int Bp, double *__restrict__ out)
{
    // K slice blockIdx.z of gridDim.z: 32-column chunks [c0, c1) of the 2 Nt
    // columns, its sums to out + z * Bp * 3N
    const int64_t nch = (2 * Nt + kF32K - 1) / kF32K;
    const int64_t kbeg = nch * blockIdx.z / gridDim.z * kF32K, kend = nch * (blockIdx.z + 1) / gridDim.z * kF32K;
    out += (int64_t)blockIdx.z * Bp * 3 * N;
    __shared__ float As[kF32K][kF32Rows + 4];
    __shared__ float Vs[kF32K][kF32Runs + 4];
    extern __shared__ double acc64s[];   // [32][256]: FP64 sum j of thread t at j * 256 + t
    const int t = threadIdx.x;
    const int tr = t & 31, tn = t >> 5;       // rows tr*4..+3, runs tn*8..+7
    const int64_t M = 3 * N, Kd = 2 * Nt;
    const int64_t m0 = (int64_t)blockIdx.x * kF32Rows;
    const int n0 = blockIdx.y * kF32Runs;
    float acc[4][8];
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 8; ++b) acc[a][b] = 0.f;
#pragma unroll
    for (int j = 0; j < 32; ++j) acc64s[j * 256 + t] = 0.0;
    // this thread's share of a chunk: K rows (t >> 5) + 8u and runs (t >> 5) + 8u, column t & 31
    const int kk = t & 31, g = t >> 5;
    float pk[16], pv[8];
    auto load = [&](int64_t k0) {
        const int64_t k = k0 + kk;
#pragma unroll
        for (int u = 0; u < 16; ++u) {
            const int64_t m = m0 + g + 8 * u;
            pk[u] = (m < M && k < Kd) ? K[m * Kd + k] : 0.f;
        }
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            const int n = n0 + g + 8 * u;
            pv[u] = (n < Bp && k < Kd) ? V[(int64_t)n * Kd + k] : 0.f;
        }
    };
    if (kbeg < kend) load(kbeg);
    int chunk = 0;
    for (int64_t k0 = kbeg; k0 < kend; k0 += kF32K, ++chunk) {
#pragma unroll
        for (int u = 0; u < 16; ++u) As[kk][g + 8 * u] = pk[u];
#pragma unroll
        for (int u = 0; u < 8; ++u) Vs[kk][g + 8 * u] = pv[u];
        __syncthreads();
        if (k0 + kF32K < kend) load(k0 + kF32K);
#pragma unroll 8
        for (int c = 0; c < kF32K; ++c) {
            float a[4], b[8];
#pragma unroll
            for (int x = 0; x < 4; ++x) a[x] = As[c][tr * 4 + x];
#pragma unroll
            for (int y = 0; y < 8; ++y) b[y] = Vs[c][tn * 8 + y];
#pragma unroll
            for (int x = 0; x < 4; ++x)
#pragma unroll
                for (int y = 0; y < 8; ++y) acc[x][y] = fmaf(a[x], b[y], acc[x][y]);
        }
        __syncthreads();
        if ((chunk & 7) == 7) {
#pragma unroll
            for (int x = 0; x < 4; ++x)
#pragma unroll
                for (int y = 0; y < 8; ++y) {
                    acc64s[(x * 8 + y) * 256 + t] += (double)acc[x][y];
                    acc[x][y] = 0.f;
                }
        }
    }
#pragma unroll
    for (int x = 0; x < 4; ++x) {
        const int64_t m = m0 + tr * 4 + x;
        if (m >= M) continue;
#pragma unroll
        for (int y = 0; y < 8; ++y) {
            const int n = n0 + tn * 8 + y;
            if (n < Bp) out[(int64_t)n * M + m] = acc64s[(x * 8 + y) * 256 + t] + (double)acc[x][y];
        }
    }
}

// Traction rates of cell i of run r as float-float values (FP32 pipes): the
// BF16X18 product leaves float-float partials per K slice, BF16X6 FP32
// partials per K slice (added here in float-float, slice order), the other
// mixed products FP64 sums (FP64 K-slice partials; one for H-matrix products).
__device__ __forceinline__ void ff_partials(const pq3d_batch_sim &S, int r, int64_t i, FF q[3])
{
    const int64_t N = S.N;
    const int Bp = padded_runs(S.B);
    if (S.precision == PQ3D_BATCH_BF16X18) {
        const int64_t pos = S.fix_pos ? S.fix_pos[i] : i;
        const float2 *pr = (const float2 *)S.rates + (int64_t)r * 3 * N + 3 * pos;
        const int64_t sstride = (int64_t)Bp * 3 * N;
#pragma unroll
        for (int c = 0; c < 3; ++c) q[c] = ff_norm(pr[c].x, pr[c].y);
        for (int sl = 1; sl < S.nsplit; ++sl)
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                const float2 t = pr[sl * sstride + c];
                q[c] = ff_add2(q[c], FF{t.x, t.y});
            }
    } else if (S.precision == PQ3D_BATCH_BF16X6) {
        const float *pr = (const float *)S.rates + (int64_t)r * 3 * N + 3 * i;
        const int64_t sstride = (int64_t)Bp * 3 * N;
#pragma unroll
        for (int c = 0; c < 3; ++c) q[c] = FF{pr[c], 0.f};
        for (int sl = 1; sl < S.nsplit; ++sl)
#pragma unroll
            for (int c = 0; c < 3; ++c) q[c] = ff_add(q[c], pr[sl * sstride + c]);
    } else {
        const double *pr = S.rates + (int64_t)r * 3 * N + 3 * i;
        const int64_t sstride = (int64_t)Bp * 3 * N;
        double t[3] = {pr[0], pr[1], pr[2]};
        for (int sl = 1; sl < S.nsplit; ++sl)
#pragma unroll
            for (int c = 0; c < 3; ++c) t[c] += pr[sl * sstride + c];
#pragma unroll
        for (int c = 0; c < 3; ++c) q[c] = ff_split(t[c]);
    }
}

// ---------------------------------------------------------------------------
// attempt / decide / update

// kFF: the float-float attempt (attempt64 = 2), with its own launch bounds
// (3 CTAs per SM: its float-float chains are latency bound, not register bound)
template <bool kMixed, bool kFF = false>
__global__ void __launch_bounds__(256, kMixed ? 4 : (kFF ? 3 : 2)) attempt_kernel(pq3d_batch_sim S)
{
    __shared__ unsigned long long red[32];
    __shared__ int act;
    __shared__ double hs;
    __shared__ float hsf, V0f;
    __shared__ double lnev;   // ln(eta V0 1e-6) of the float-float attempt
    __shared__ FF etab[64];
    const int r = blockIdx.y;
    pq3d_run_ctrl *C = S.ctrl + r;
    if (threadIdx.x == 0) {
        act = C->active;
        hs = C->h;
        if (kMixed) {
            hsf = (float)hs;
            V0f = (float)S.V0;
        } else if (kFF) {
            lnev = log(S.eta * S.V0 * 1e-6);
        }
    }
    if (kFF && threadIdx.x < 64) etab[threadIdx.x] = ffv(kExp2Tab.v[threadIdx.x]);
    __syncthreads();
    if (!act) return;
    const int64_t N = S.N;
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    double m1 = 0.0, m2 = 0.0;
    float f1 = 0.f, f2 = 0.f;
    if (i < N) {
        const int64_t idx = (int64_t)r * N + i;
        const int Bp = padded_runs(S.B);
        const double y[4] = {S.Tno[idx], S.Tt1o[idx], S.Tt2o[idx], S.state[idx]};
        double yo[4];
        if (kMixed) {
            FF q[3];
            ff_partials(S, r, i, q);
            MixedBase m = load_base(S.base + idx, (int64_t)S.B * N);
            const float shear = (float)S.shear_loading[idx];
            const float dsig = S.fix_Tn ? (float)S.normal_loading[idx]
                                        : (q[2].hi + (q[2].lo + (float)S.normal_loading[idx]));
            m.V0 = V0f;
            m.dsf = dsig;
            m.L[0] = (shear - q[0].hi) - q[0].lo;
            m.L[1] = (shear - q[1].hi) - q[1].lo;
            dp_attempt_mixed(m, dsig, hsf, y, yo, f1, f2);
        } else if (kFF) {
            // float-float attempt: the rates stay float-float (no FP64 sums)
            FF q[3];
            ff_partials(S, r, i, q);
            const FF nl = ff_split_fast(S.normal_loading[idx]);
            const FFRates fr{q[0], q[1], S.fix_Tn ? nl : ff_add2(q[2], nl)};
            const Cell c{S.a[idx], S.b[idx], S.dc[idx], S.f0[idx], S.shear_loading[idx], S.slipv[idx], 0.0, 0.0, 0.0,
                         0.0, 0.0};
            dp_attempt_ff(c, fr, S.V0, lnev, hs, y, yo, m1, m2, etab);
        } else {
            double q0 = 0.0, q1 = 0.0, q2 = 0.0;
            if (S.precision == PQ3D_BATCH_BF16X18) {   // float-float K-slice partials, added in FP64
                const int64_t pos = S.fix_pos ? S.fix_pos[i] : i;
                for (int s = 0; s < S.nsplit; ++s) {
                    const float2 *p = (const float2 *)S.rates + ((int64_t)s * Bp + r) * 3 * N + 3 * pos;
                    q0 += (double)p[0].x + (double)p[0].y;
                    q1 += (double)p[1].x + (double)p[1].y;
                    q2 += (double)p[2].x + (double)p[2].y;
                }
            } else if (S.precision == PQ3D_BATCH_BF16X6) {   // FP32 K-slice partials, added in FP64
                for (int s = 0; s < S.nsplit; ++s) {
                    const float *p = (const float *)S.rates + ((int64_t)s * Bp + r) * 3 * N + 3 * i;
                    q0 += (double)p[0]; q1 += (double)p[1]; q2 += (double)p[2];
                }
            } else {
                for (int s = 0; s < S.nsplit; ++s) {
                    const double *p = S.rates + ((int64_t)s * Bp + r) * 3 * N + 3 * i;
                    q0 += p[0]; q1 += p[1]; q2 += p[2];
                }
            }
            const double dsig = S.fix_Tn ? S.normal_loading[idx] : q2 + S.normal_loading[idx];
            const Cell c{S.a[idx], S.b[idx], S.dc[idx], S.f0[idx], S.shear_loading[idx], S.slipv[idx], q0, q1, dsig,
                         0.0, 0.0};
            // the FP64 precision keeps the reference formula (it is the arm the
            // others are compared with); the FP64 attempt of the mixed
            // products (attempt64 = 1) takes the reciprocal form, the
            // float-float attempt (attempt64 = 2) the w-form on the FP32 pipes
            if (S.precision == PQ3D_BATCH_FP64) dp_attempt<false>(c, S.V0, S.eta, hs, y, yo, m1, m2);
            else dp_attempt<true>(c, S.V0, S.eta, hs, y, yo, m1, m2);
        }
        reinterpret_cast<double4_16a *>(S.cand)[idx] = make_double4_16a(yo[0], yo[1], yo[2], yo[3]);
    }
    if (kMixed) {
        // float maxima, widened to FP64 once per block
        unsigned *red32 = reinterpret_cast<unsigned *>(red);
        const unsigned b1 = block_max_bits32(f1, red32);
        const unsigned b2 = block_max_bits32(f2, red32);
        if (threadIdx.x == 0) {
            atomicMax((unsigned long long *)&C->err1_bits, dbits((double)__uint_as_float(b1)));
            atomicMax((unsigned long long *)&C->err2_bits, dbits((double)__uint_as_float(b2)));
        }
    } else {
        const unsigned long long b1 = block_max_bits(dbits(m1), red);
        const unsigned long long b2 = block_max_bits(dbits(m2), red);
        if (threadIdx.x == 0) {
            atomicMax((unsigned long long *)&C->err1_bits, b1);
            atomicMax((unsigned long long *)&C->err2_bits, b2);
        }
    }
}

__global__ void decide_kernel(pq3d_run_ctrl *ctrl, int B)
{
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= B) return;
    pq3d_run_ctrl *C = ctrl + r;
    if (!C->active) { C->accepted = 0; return; }
    const double err1 = __longlong_as_double((long long)C->err1_bits) + 1e-10;
    const double err2 = __longlong_as_double((long long)C->err2_bits) + 1e-10;
    C->err1_bits = 0ull;
    C->err2_bits = 0ull;
    const double h = C->h;
    C->attempts += 1;
    const double c1 = err1 / kRelTol, c2 = err2 / kRelTol;
    const double hn1 = h * 0.9 * pow(kRelTol / err1, 0.2);
    const double hn2 = h * 0.9 * pow(kRelTol / err2, 0.2);
    if (fmax(c1, c2) < 1.0 && !(isnan(c1) || isnan(c2))) {
        C->accepted = 1;
        C->h_last = h;
        C->time = C->time + h;
        C->steps += 1;
        C->nrjct = 0;
        C->h = pymin(1.5 * h, pymin(hn1, hn2));
        if (C->steps >= C->max_steps || C->time >= C->t_end) C->active = 0;
    } else {
        C->accepted = 0;
        C->nrjct += 1;
        const double hn = pymax(0.5 * h, pymin(hn1, hn2));
        C->h = hn;
        if (hn < 1.e-15 || C->nrjct > 20) {
            C->status = PQ3D_ERR_STEP;
            C->active = 0;
        }
    }
}

// The update kernel packs the BF16x18 right-hand side itself when the packed
// columns follow the cells (no cell order, one shard): its 256-cell blocks are
// then two whole 256-column spans, and a rejected run keeps its packed v'.
__host__ __device__ inline bool fused_rhs_pack(const pq3d_batch_sim &S)
{
    return S.precision == PQ3D_BATCH_BF16X18 && S.fix_order == nullptr && S.cell0 == 0 &&
           (S.N_total == 0 || S.N_total == S.N);
}

// kMixed: the new state's start-of-step constants (in float-float from the
// FP64 state, once per accepted step for all the attempts of the next step)
// and from them the slip rate 2 V0 e^{-psi/a} sinh(tau / (sigma a)) (~2e-7
// relative, as the mixed right-hand side); FP64 for the slip accumulation.
// The FP64 arm keeps the reference formula (src/QDsim_gpu.py:994-1027).
template <bool kMixed>
__global__ void __launch_bounds__(256) update_kernel(pq3d_batch_sim S)
{
    __shared__ int acc;
    __shared__ double hs, lnv0;
    __shared__ float inv_eta, c0hi, c0lo;
    __shared__ FF etab[64];
    const int r = blockIdx.y;
    const pq3d_run_ctrl *C = S.ctrl + r;
    const bool ffu = !kMixed && S.attempt64 == 2 && S.precision != PQ3D_BATCH_FP64;
    if (threadIdx.x == 0) {
        acc = C->accepted;
        hs = C->h_last;
        if (kMixed) {
            const FF c0 = ff_split(log_eta_v0(S));
            c0hi = c0.hi;
            c0lo = c0.lo;
            inv_eta = (float)(1.0 / S.eta);
        } else if (ffu) {
            lnv0 = log(S.V0);
        }
    }
    if (ffu && threadIdx.x < 64) etab[threadIdx.x] = ffv(kExp2Tab.v[threadIdx.x]);
    __syncthreads();
    if (!acc) return;
    const int64_t N = S.N;
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const bool fuse = fused_rhs_pack(S);
    if (i >= N && !fuse) return;
    double p1 = 0.0, p2 = 0.0;   // the cell's v' (fused packing; zero past the last cell)
    if (i < N) {
        const int64_t idx = (int64_t)r * N + i;
        const double h = hs;
        const double4_16a y = reinterpret_cast<const double4_16a *>(S.cand)[idx];
        const double Tno = y.x, T1 = y.y, T2 = y.z, st = y.w;
        S.Tno[idx] = Tno; S.Tt1o[idx] = T1; S.Tt2o[idx] = T2; S.state[idx] = st;
        double v1, v2, v;
        if (kMixed) {
            float *pb = S.base + idx;
            const int64_t stride = (int64_t)S.B * N;
            MixedBase m;
            store_base_state(pb, stride, Tno, T1, T2, st, FF{c0hi, c0lo}, m);
            const float f1 = base_slip_rate(m, 0, inv_eta), f2 = base_slip_rate(m, 1, inv_eta);
            // |V| without under/overflow of the squares
            const float p = fmaxf(fabsf(f1), fabsf(f2)), q = fminf(fabsf(f1), fabsf(f2));
            const float t = p > 0.f ? q / p : 0.f;
            const float vf = fmaxf(p * sqrtf(fmaf(t, t, 1.f)), 1e-30f);
            pb[19 * stride] = vf;
            v1 = f1; v2 = f2; v = vf;
        } else if (ffu) {
            // the float-float arm: 2 V0 e^{-psi/a} sinh(x) = sign(x) V0 e^{-psi/a + |x|} (1 - e^{-2|x|}),
            // x = tau / (a sigma), the exponent argument in FP64 (reduced), the rest float-float
            const double a = S.a[idx];
            const double psia = st * rcp_d(a), iaT = rcp_d(a * Tno);
            const FF f1 = ff_slip_rate(lnv0, psia, T1 * iaT, etab), f2 = ff_slip_rate(lnv0, psia, T2 * iaT, etab);
            v1 = ff_to_double_fast(f1);
            v2 = ff_to_double_fast(f2);
            v = ff_to_double_fast(ff_hypot(f1, f2));   // |V| in float-float, like its components
        } else {
            const double a = S.a[idx];
            const double e = (2.0 * S.V0) * exp(-st / a);
            v1 = e * sinh(T1 / Tno / a);
            v2 = e * sinh(T2 / Tno / a);
            v = sqrt(v1 * v1 + v2 * v2);
        }
        if (v < 1e-30) v = 1e-30;
        S.slipv1[idx] = v1; S.slipv2[idx] = v2; S.slipv[idx] = v;
        S.slip1[idx] += v1 * h;
        S.slip2[idx] += v2 * h;
        write_vop<!kMixed>(S, r, i, v1 - S.Vpl * S.cos_rake0[idx], v2 - S.Vpl * S.sin_rake0[idx]);
        if (fuse) {
            p1 = fma(-S.Vpl, S.cos_rake0[idx], v1);
            p2 = fma(-S.Vpl, S.sin_rake0[idx], v2);
        }
    }
    if (fuse) {
        // the fixed-point slices of v': threads 0-127 and 128-255 are the
        // cells of two 256-column spans; each span's largest |v'| sets its
        // exponent (as the pack kernel does)
        __shared__ int smax[8];
        int mx = fx::rhs_word(p1, p2);
        for (int o = 16; o > 0; o >>= 1) mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, o));
        if ((threadIdx.x & 31) == 0) smax[threadIdx.x >> 5] = mx;
        __syncthreads();
        const int w0 = (threadIdx.x >> 7) * 4;
        const int m = max(max(smax[w0], smax[w0 + 1]), max(smax[w0 + 2], smax[w0 + 3]));
        fx::write_rhs_cell((__nv_bfloat16 *)S.vop, fx::fix_runs(S.B), fx::k_blocks(N), i, r,
                           fx::rhs_span_exponent(m), p1, p2);
    }
}

// The Dormand-Prince attempt and update in mixed precision (FP32 stages on the
// FP64 state), or in the reference FP64 arithmetic: always for the FP64
// product, on request (attempt64) for the others.
static bool mixed_attempt(const pq3d_batch_sim &S) { return S.precision != PQ3D_BATCH_FP64 && !S.attempt64; }

static int check_sim(const pq3d_batch_sim *S)
{
    PQ3D_REQUIRE(S && S->N > 0 && S->B > 0 && S->B <= 1024 && S->ctrl && S->K && S->vop && S->rates && S->cand,
                 "pq3d_batch: bad simulation structure");
    PQ3D_REQUIRE(S->precision >= PQ3D_BATCH_FP64 && S->precision <= PQ3D_BATCH_BF16X18, "pq3d_batch: bad precision");
    if (S->precision == PQ3D_BATCH_BF16X18) {
        PQ3D_REQUIRE(S->B <= fx::kMaxRuns, "pq3d_batch: the BF16X18 product takes at most %d runs", fx::kMaxRuns);
        PQ3D_REQUIRE((S->fix_order == nullptr) == (S->fix_pos == nullptr),
                     "pq3d_batch: fix_order and fix_pos are given together");
    }
    if (S->precision == PQ3D_BATCH_HMAT)
        PQ3D_REQUIRE(((const pq3d_hmat *)S->K)->N == S->N, "pq3d_batch: H-matrix size differs from N");
    PQ3D_REQUIRE(S->nsplit >= 1, "pq3d_batch: nsplit must be >= 1");
    PQ3D_REQUIRE(S->tc_ctas >= 0 && S->tc_ctas <= 3, "pq3d_batch: tc_ctas must be 0 (default) or 1..3");
    PQ3D_REQUIRE(aligned16(S->cand) && aligned16(S->vop) && aligned16(S->K), "pq3d_batch: buffers must be 16-byte aligned");
    if (S->precision == PQ3D_BATCH_FP64 || S->precision == PQ3D_BATCH_HMAT)
        PQ3D_REQUIRE(S->nsplit == 1, "pq3d_batch: the FP64 and H-matrix products use nsplit = 1");
    if (S->precision == PQ3D_BATCH_FP32)
        PQ3D_REQUIRE(S->nsplit <= 64, "pq3d_batch: the FP32 product takes at most 64 K slices");
    PQ3D_REQUIRE(S->attempt64 >= 0 && S->attempt64 <= 2, "pq3d_batch: attempt64 must be 0, 1 or 2");
    if (mixed_attempt(*S))
        PQ3D_REQUIRE(S->base != nullptr && aligned16(S->base), "pq3d_batch: mixed precisions need the base array");
    PQ3D_REQUIRE(S->N_total >= 0 && S->cell0 >= 0, "pq3d_batch: bad shard");
    if (S->N_total > 0 && (S->N_total != S->N || S->cell0 != 0)) {
        PQ3D_REQUIRE(S->precision == PQ3D_BATCH_FP64 || S->precision == PQ3D_BATCH_FP32,
                     "pq3d_batch: row shards need the FP64 or FP32 product");
        PQ3D_REQUIRE(S->cell0 + S->N <= S->N_total, "pq3d_batch: shard [%lld, %lld) outside the mesh of %lld cells",
                     (long long)S->cell0, (long long)(S->cell0 + S->N), (long long)S->N_total);
    }
    return PQ3D_OK;
}

}  // namespace batch
}  // namespace pq3d

using namespace pq3d;
using namespace pq3d::batch;

extern "C" size_t pq3d_batch_workspace_bytes(const pq3d_batch_sim *sim)
{
    if (sim && sim->precision == PQ3D_BATCH_HMAT)
        return pq3d_hmat_workspace_bytes((const pq3d_hmat *)sim->K, padded_runs(sim->B));
    if (sim && sim->precision == PQ3D_BATCH_BF16X18) return 256;
    if (!sim || sim->precision != PQ3D_BATCH_BF16X6) return 0;
    return pq3d::tc::gemm_bf16x6_workspace_bytes(sim->N, padded_runs(sim->B), sim->nsplit);
}

extern "C" int pq3d_batch_prepare(const pq3d_batch_sim *sim, void *stream)
{
    clear_error();
    int rc = check_sim(sim);
    if (rc) return rc;
    const int Bp = padded_runs(sim->B);
    dim3 grid((unsigned)((sim->N + 255) / 256), (unsigned)Bp);
    prepare_kernel<<<grid, 256, 0, (cudaStream_t)stream>>>(*sim);   // the shard's own slice of v'
    PQ3D_CUDA_TRY(cudaGetLastError());
    if (sim->precision == PQ3D_BATCH_BF16X18)
        return fx::pack_rhs_from_state(sim->slipv1, sim->slipv2, sim->cos_rake0, sim->sin_rake0, sim->Vpl,
                                       sim->fix_order, sim->N, sim->B, sim->vop, (cudaStream_t)stream);
    return PQ3D_OK;
}

extern "C" int pq3d_batch_iterate_begin(const pq3d_batch_sim *sim, void *workspace, size_t workspace_bytes,
                                        void *stream)
{
    clear_error();
    int rc = check_sim(sim);
    if (rc) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    const pq3d_batch_sim &S = *sim;
    const int Bp = padded_runs(S.B);
    const int64_t Nt = total_cells(S);
    // 1. operator product
    if (S.precision == PQ3D_BATCH_FP64) {
        const int64_t warps = S.N * Bp;
        gemm_f64_kernel<<<(unsigned)((warps * 32 + 255) / 256), 256, 0, st>>>(
            (const double2 *)S.K, (const double2 *)S.vop, S.N, Nt, Bp, S.rates);
    } else if (S.precision == PQ3D_BATCH_FP32) {
        dim3 grid((unsigned)((3 * S.N + kF32Rows - 1) / kF32Rows), (unsigned)((Bp + kF32Runs - 1) / kF32Runs),
                  (unsigned)S.nsplit);
        static thread_local int smem_dev = -1;
        int dev;
        PQ3D_CUDA_TRY(cudaGetDevice(&dev));
        if (smem_dev != dev) {
            PQ3D_CUDA_TRY(cudaFuncSetAttribute(gemm_f32_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kF32Smem));
            smem_dev = dev;
        }
        gemm_f32_kernel<<<grid, 256, kF32Smem, st>>>((const float *)S.K, (const float *)S.vop, S.N, Nt, Bp, S.rates);
    } else if (S.precision == PQ3D_BATCH_BF16X18) {
        rc = fx::gemm_bf16x18(S.K, S.vop, S.N, S.B, S.nsplit, (float2 *)S.rates, workspace, workspace_bytes, st);
        if (rc) return rc;
    } else if (S.precision == PQ3D_BATCH_BF16X6) {
        rc = pq3d::tc::gemm_bf16x6((const float *)S.K, (const void *)S.vop, S.N, Bp, S.nsplit, S.tc_ctas, (float *)S.rates,
                                   workspace, workspace_bytes, st);
        if (rc) return rc;
    } else {
        // the H-matrix product needs no padding runs: the first B rows only
        // inactive runs (free slots, finished runs) skip the product
        rc = pq3d_hmat_apply_masked((const pq3d_hmat *)S.K, (const double *)S.vop, S.B, S.rates, &S.ctrl[0].active,
                                    (int)(sizeof(pq3d_run_ctrl) / sizeof(int32_t)), workspace, workspace_bytes,
                                    stream);
        if (rc) return rc;
    }
    PQ3D_CUDA_TRY(cudaGetLastError());
    // 2. attempt (FP64 arm: the reference arithmetic; mixed arms: dp_attempt_mixed)
    dim3 grid((unsigned)((S.N + 255) / 256), (unsigned)S.B);
    if (mixed_attempt(S)) attempt_kernel<true><<<grid, 256, 0, st>>>(S);
    else if (S.attempt64 == 2 && S.precision != PQ3D_BATCH_FP64) attempt_kernel<false, true><<<grid, 256, 0, st>>>(S);
    else attempt_kernel<false><<<grid, 256, 0, st>>>(S);
    PQ3D_CUDA_TRY(cudaGetLastError());
    return PQ3D_OK;
}

extern "C" int pq3d_batch_iterate_end(const pq3d_batch_sim *sim, void *stream)
{
    clear_error();
    int rc = check_sim(sim);
    if (rc) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    const pq3d_batch_sim &S = *sim;
    // 3-4. decide, update
    decide_kernel<<<(S.B + 127) / 128, 128, 0, st>>>(S.ctrl, S.B);
    dim3 grid((unsigned)((S.N + 255) / 256), (unsigned)S.B);
    if (mixed_attempt(S)) update_kernel<true><<<grid, 256, 0, st>>>(S);
    else update_kernel<false><<<grid, 256, 0, st>>>(S);
    PQ3D_CUDA_TRY(cudaGetLastError());
    if (S.precision == PQ3D_BATCH_BF16X18 && !fused_rhs_pack(S))   // v' of every run from its slip rates
        return fx::pack_rhs_from_state(S.slipv1, S.slipv2, S.cos_rake0, S.sin_rake0, S.Vpl, S.fix_order, S.N, S.B,
                                       S.vop, st);
    return PQ3D_OK;
}

extern "C" int pq3d_batch_iterate(const pq3d_batch_sim *sim, void *workspace, size_t workspace_bytes, void *stream)
{
    const int rc = pq3d_batch_iterate_begin(sim, workspace, workspace_bytes, stream);
    return rc ? rc : pq3d_batch_iterate_end(sim, stream);
}
