// Dense quasi-dynamic stepping on the GPU (plain FP64 path, or the FP32
// operator copy).
//
// Reference behaviour (src/QDsim_gpu.py):
//   traction product K.(V - Vpl), once per accepted step        948-957
//   right-hand side (aging law, radiation damping)             830-891
//   Dormand-Prince 5(4) attempt, max-relative error norm      1128-1262
//   accept / reject and dt control                              959-985
//   closed-form slip rate, rake, slip integration              994-1027
//
// GPU design, per accepted step two launches queued back to back (no host
// synchronisation between steps): (1) the traction product, a warp per
// receiver streaming its three operator rows (16-byte loads) against the
// interleaved slip-rate deficit v', at the full occupancy of a small kernel;
// (2) one cooperative kernel: every thread runs the 7 right-hand-side
// evaluations of its cells in registers (the traction rates are frozen over
// the step, so the stages are cell-local), block-max + one atomicMax per block
// give the two error norms, one grid barrier, every thread takes the same
// accept/reject decision, retry until accepted; (3) the state update writes v'
// for the next step's product.  The step's control values (dt, time, attempt
// count) live in the control block between launches.  Grid barriers are
// bounded.  (The product inside one persistent kernel for all steps ran at
// the occupancy of the attempt code and took ~10 % longer: 4.93 against
// 4.50 ms per step at N = 20,000.)
#include <math.h>

#include "common.cuh"
#include "rk_device.cuh"

namespace pq3d {
namespace step {

using namespace ::pq3d::rk;

// ---------------------------------------------------------------------------
// traction product: rows 3i..3i+2 of K times v' (interleaved strike/dip)

__device__ __forceinline__ double warp_sum(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// One warp: out[3i+c] for c = 0..2.  K rows have N double2 (strike, dip).
__device__ __forceinline__ void rows3_f64(const double2 *__restrict__ K, const double2 *__restrict__ v, int64_t N,
                                          int64_t i, int lane, double acc[3])
{
    const double2 *r0 = K + (3 * i) * N, *r1 = r0 + N, *r2 = r1 + N;
    double a0 = 0.0, a1 = 0.0, a2 = 0.0, b0 = 0.0, b1 = 0.0, b2 = 0.0;
    int64_t j = lane;
    for (; j + 32 < N; j += 64) {
        const double2 x0 = __ldg(v + j), x1 = __ldg(v + j + 32);
        const double2 k00 = __ldcs(r0 + j), k10 = __ldcs(r1 + j), k20 = __ldcs(r2 + j);
        const double2 k01 = __ldcs(r0 + j + 32), k11 = __ldcs(r1 + j + 32), k21 = __ldcs(r2 + j + 32);
        a0 = fma(k00.x, x0.x, a0); a0 = fma(k00.y, x0.y, a0);
        a1 = fma(k10.x, x0.x, a1); a1 = fma(k10.y, x0.y, a1);
        a2 = fma(k20.x, x0.x, a2); a2 = fma(k20.y, x0.y, a2);
        b0 = fma(k01.x, x1.x, b0); b0 = fma(k01.y, x1.y, b0);
        b1 = fma(k11.x, x1.x, b1); b1 = fma(k11.y, x1.y, b1);
        b2 = fma(k21.x, x1.x, b2); b2 = fma(k21.y, x1.y, b2);
    }
    for (; j < N; j += 32) {
        const double2 x0 = __ldg(v + j);
        const double2 k00 = __ldcs(r0 + j), k10 = __ldcs(r1 + j), k20 = __ldcs(r2 + j);
        a0 = fma(k00.x, x0.x, a0); a0 = fma(k00.y, x0.y, a0);
        a1 = fma(k10.x, x0.x, a1); a1 = fma(k10.y, x0.y, a1);
        a2 = fma(k20.x, x0.x, a2); a2 = fma(k20.y, x0.y, a2);
    }
    acc[0] = warp_sum(a0 + b0);
    acc[1] = warp_sum(a1 + b1);
    acc[2] = warp_sum(a2 + b2);
}

// FP32 operator: rows of N float2.  The products and sums are compensated so
// that the result is the FP32-rounded operator applied exactly (to ~2^-44):
// v' is split into hi + lo floats, k * vhi is formed exactly as p + e
// (TwoProduct with an FMA), the running sum is carried as s + c (TwoSum).  The
// _rn intrinsics keep the compiler from contracting these sequences.  FP32
// operations are ~64x cheaper than FP64 ones on this part, so the ~11 FP32
// operations per entry stay below the HBM time of the 4-byte entry.
struct Acc2 {
    float s, c;
};

__device__ __forceinline__ void acc2_add(Acc2 &a, float k, float vh, float vl)
{
    const float p = __fmul_rn(k, vh);
    const float e = __fmaf_rn(k, vh, -p);
    const float t = __fadd_rn(a.s, p);
    const float bp = __fsub_rn(t, a.s);
    const float err = __fadd_rn(__fsub_rn(a.s, __fsub_rn(t, bp)), __fsub_rn(p, bp));
    a.s = t;
    a.c = __fmaf_rn(k, vl, __fadd_rn(a.c, __fadd_rn(err, e)));
}

// v' of one cell split into FP32 pieces: (hi1, hi2, lo1, lo2), v ~= hi + lo.
__device__ __forceinline__ float4 split_v(double v1, double v2)
{
    const float h1 = (float)v1, h2 = (float)v2;
    return make_float4(h1, h2, (float)(v1 - (double)h1), (float)(v2 - (double)h2));
}

__device__ __forceinline__ void rows3_f32(const float2 *__restrict__ K, const float4 *__restrict__ v, int64_t N,
                                          int64_t i, int lane, double acc[3])
{
    const float2 *r0 = K + (3 * i) * N, *r1 = r0 + N, *r2 = r1 + N;
    Acc2 a0{0.f, 0.f}, a1{0.f, 0.f}, a2{0.f, 0.f};
    int64_t j = lane;
    for (; j + 32 < N; j += 64) {
        const float4 x0 = __ldg(v + j), x1 = __ldg(v + j + 32);
        const float2 k00 = __ldcs(r0 + j), k10 = __ldcs(r1 + j), k20 = __ldcs(r2 + j);
        const float2 k01 = __ldcs(r0 + j + 32), k11 = __ldcs(r1 + j + 32), k21 = __ldcs(r2 + j + 32);
        acc2_add(a0, k00.x, x0.x, x0.z); acc2_add(a0, k00.y, x0.y, x0.w);
        acc2_add(a1, k10.x, x0.x, x0.z); acc2_add(a1, k10.y, x0.y, x0.w);
        acc2_add(a2, k20.x, x0.x, x0.z); acc2_add(a2, k20.y, x0.y, x0.w);
        acc2_add(a0, k01.x, x1.x, x1.z); acc2_add(a0, k01.y, x1.y, x1.w);
        acc2_add(a1, k11.x, x1.x, x1.z); acc2_add(a1, k11.y, x1.y, x1.w);
        acc2_add(a2, k21.x, x1.x, x1.z); acc2_add(a2, k21.y, x1.y, x1.w);
    }
    for (; j < N; j += 32) {
        const float4 x0 = __ldg(v + j);
        const float2 k00 = __ldcs(r0 + j), k10 = __ldcs(r1 + j), k20 = __ldcs(r2 + j);
        acc2_add(a0, k00.x, x0.x, x0.z); acc2_add(a0, k00.y, x0.y, x0.w);
        acc2_add(a1, k10.x, x0.x, x0.z); acc2_add(a1, k10.y, x0.y, x0.w);
        acc2_add(a2, k20.x, x0.x, x0.z); acc2_add(a2, k20.y, x0.y, x0.w);
    }
    acc[0] = warp_sum((double)a0.s + (double)a0.c);
    acc[1] = warp_sum((double)a1.s + (double)a1.c);
    acc[2] = warp_sum((double)a2.s + (double)a2.c);
}

template <bool kF32>
__global__ void __launch_bounds__(256) matvec_kernel(const void *__restrict__ K, const void *__restrict__ v,
                                                     int64_t N, double *__restrict__ out)
{
    const int lane = threadIdx.x & 31;
    const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t i = warp; i < N; i += nwarps) {
        double acc[3];
        if (kF32) rows3_f32((const float2 *)K, (const float4 *)v, N, i, lane, acc);
        else rows3_f64((const double2 *)K, (const double2 *)v, N, i, lane, acc);
        if (lane == 0) { out[3 * i] = acc[0]; out[3 * i + 1] = acc[1]; out[3 * i + 2] = acc[2]; }
    }
}

// ---------------------------------------------------------------------------
// pore-pressure dilatancy (src/QDsim_gpu.py:611-671)

constexpr int kMaxDepth = 64;   // tridiagonal unknowns per cell (the reference uses 59)

// table layout (pq3d_dilatancy_table): lower, diag, upper of the diffusion
// matrix (n each; M = dt * this + I), then the scalars below
enum DilaScalar { D_BC0, D_BCN, D_G, D_T1, D_T2, D_TG, D_DP, D_NSCAL };

// One implicit step for the cells [cell0, cell1) of this block (called by all
// threads of every block with the same h): the Thomas factorisation of M is formed once
// per block in shared memory (M is diagonally dominant by rows, so no
// pivoting is needed; the reference factorises with partial pivoting).
__device__ __noinline__ void dilatancy_step(const pq3d_dense_sim &S, double h, double *cp, double *inv, int64_t cell0,
                                            int64_t cell1)
{
    const int n = S.ndepth;
    const double *lo = S.dila, *di = lo + n, *up = di + n, *sc = up + n;
    __syncthreads();
    if (threadIdx.x == 0) {
        double prev = 0.0;
        for (int k = 0; k < n; ++k) {
            const double den = (1.0 + di[k] * h) - (k ? lo[k] * h * prev : 0.0);
            inv[k] = 1.0 / den;
            prev = (k + 1 < n) ? up[k] * h * inv[k] : 0.0;
            cp[k] = prev;
        }
    }
    __syncthreads();
    const int64_t N = S.N;
    for (int64_t i = cell0 + threadIdx.x; i < cell1; i += blockDim.x) {
        const double theta = S.dc[i] / S.V0 * exp((S.state[i] - S.f0[i]) / S.b[i]);
        const double dthetadt = 1.0 - S.slipv[i] * theta / S.dc[i];
        const double g = -sc[D_G] / theta * dthetadt;
        double *col = S.Parr + i;   // Parr[k * N + i]
        // forward sweep: d'_k into Parr
        double dprev = 0.0;
        for (int k = 0; k < n; ++k) {
            double b = col[k * N];
            if (k == 0) b -= sc[D_BC0] * g * h;
            if (k == n - 1) b += h * sc[D_BCN];
            const double d = (b - (k ? lo[k] * h * dprev : 0.0)) * inv[k];
            col[k * N] = d;
            dprev = d;
        }
        // back substitution
        double x = dprev;
        for (int k = n - 2; k >= 0; --k) {
            x = col[k * N] - cp[k] * x;
            col[k * N] = x;
        }
        const double x0 = col[0], x1 = col[N];
        const double term1 = -sc[D_T1] * (x0 - x1 + sc[D_TG] * g);
        const double term2 = sc[D_T2] * (x1 - x0);
        S.dPdt[i] = sc[D_DP] * (term1 + term2);
        S.P[i] = x0;
    }
}

// v' of every cell from its current slip rate (src/QDsim_gpu.py:948-949); the
// FP32 operator takes it as its hi/lo FP32 split
template <bool kF32>
__global__ void __launch_bounds__(256) vprime_kernel(pq3d_dense_sim S)
{
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= S.N) return;
    const double v1 = S.slipv1[i] - S.Vpl * cos(S.rake0[i]), v2 = S.slipv2[i] - S.Vpl * sin(S.rake0[i]);
    if (kF32) reinterpret_cast<float4 *>(S.vprime)[i] = split_v(v1, v2);
    else reinterpret_cast<double2 *>(S.vprime)[i] = make_double2(v1, v2);
}

// (1) traction rates of one step (src/QDsim_gpu.py:948-957): a warp per
// receiver, the normal component with the normal loading added (or the
// loading alone with fix_Tn)
template <bool kF32>
__global__ void __launch_bounds__(256) step_rates_kernel(pq3d_dense_sim S)
{
    const int lane = threadIdx.x & 31;
    const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const int64_t N = S.N;
    for (int64_t i = warp; i < N; i += nwarps) {
        double acc[3];
        if (kF32) rows3_f32((const float2 *)S.K32, (const float4 *)S.vprime, N, i, lane, acc);
        else rows3_f64((const double2 *)S.K64, (const double2 *)S.vprime, N, i, lane, acc);
        if (lane == 0) {
            S.rates[3 * i] = acc[0];
            S.rates[3 * i + 1] = acc[1];
            S.rates[3 * i + 2] = S.fix_Tn ? S.normal_loading[i] : acc[2] + S.normal_loading[i];
        }
    }
}

// (2)-(3) the rest of one accepted step, one cooperative launch: attempts
// until one is accepted (grid barrier per attempt for the error norms; every
// thread takes the same decision), the state update with v' for the next
// product, the dilatancy step.  `step` indexes h_hist / t_hist / h_force.
template <bool kF32>
__global__ void __launch_bounds__(256) dense_attempt_kernel(pq3d_dense_sim S, int step, double *h_hist, double *t_hist,
                                                            const double *h_force)
{
    __shared__ unsigned long long red[32];
    __shared__ double dil_cp[kMaxDepth], dil_inv[kMaxDepth];
    pq3d_step_ctrl *C = S.ctrl;
    // read before the first grid barrier (the lead changes them only after it)
    if (*(volatile int32_t *)&C->status != PQ3D_OK) return;   // same for every block
    const double dttry = *(volatile double *)&C->dttry, time = *(volatile double *)&C->time;
    int64_t attempt = *(volatile int64_t *)&C->attempts;      // rotates the error slots
    const int64_t N = S.N;
    const bool lead = (blockIdx.x == 0 && threadIdx.x == 0);
    unsigned *bc = &C->bar_count, *bg = &C->bar_gen;
    const unsigned nb = gridDim.x;
    double2 *vp = (double2 *)S.vprime;
    float4 *vs = (float4 *)S.vprime;
    // cells of this block: a contiguous share of N / gridDim, so that every SM
    // gets cells (N is often below the grid's thread count)
    const int64_t chunk = (N + nb - 1) / nb;
    const int64_t cell0 = (int64_t)blockIdx.x * chunk, cell1 = cell0 + chunk < N ? cell0 + chunk : N;
    if (lead) C->maxv_bits = 0ull;   // the update's atomicMax comes after at least one grid barrier

    // (2) attempts until one is accepted
    double h = h_force ? h_force[step] : dttry, dtnext = 0.0;
    int nrjct = 0;
    for (;;) {
        const int slot = (int)(attempt % 3);
        double m1 = 0.0, m2 = 0.0;
        for (int64_t i = cell0 + threadIdx.x; i < cell1; i += blockDim.x) {
            const Cell c{S.a[i], S.b[i], S.dc[i], S.f0[i], S.shear_loading[i], S.slipv[i],
                         S.rates[3 * i], S.rates[3 * i + 1], S.rates[3 * i + 2],
                         S.P ? S.P[i] : 0.0, S.dPdt ? S.dPdt[i] : 0.0};
            const double y[4] = {S.Tno[i], S.Tt1o[i], S.Tt2o[i], S.state[i]};
            double yo[4], e1, e2;
            dp_attempt(c, S.V0, S.eta, h, y, yo, e1, e2);
            reinterpret_cast<double4_16a *>(S.cand)[i] = make_double4_16a(yo[0], yo[1], yo[2], yo[3]);
            m1 = (isnan(m1) || isnan(e1)) ? NAN : fmax(m1, e1);
            m2 = (isnan(m2) || isnan(e2)) ? NAN : fmax(m2, e2);
        }
        const unsigned long long b1 = block_max_bits(dbits(m1), red);
        const unsigned long long b2 = block_max_bits(dbits(m2), red);
        if (threadIdx.x == 0) {
            atomicMax((unsigned long long *)&C->err_slot[2 * slot], b1);
            atomicMax((unsigned long long *)&C->err_slot[2 * slot + 1], b2);
        }
        if (!grid_barrier(bc, bg, nb)) { if (threadIdx.x == 0) C->status = PQ3D_ERR_TIMEOUT; return; }
        const double err1 = __longlong_as_double((long long)*((volatile unsigned long long *)&C->err_slot[2 * slot])) + 1e-10;
        const double err2 = __longlong_as_double((long long)*((volatile unsigned long long *)&C->err_slot[2 * slot + 1])) + 1e-10;
        if (lead) {
            // the slot of the attempt before this one: every thread has read it
            const int z = (int)((attempt + 2) % 3);
            C->err_slot[2 * z] = 0ull;
            C->err_slot[2 * z + 1] = 0ull;
            C->attempts += 1;
        }
        ++attempt;
        const double c1 = err1 / kRelTol, c2 = err2 / kRelTol;
        const double hn1 = h * 0.9 * pow(kRelTol / err1, 0.2);
        const double hn2 = h * 0.9 * pow(kRelTol / err2, 0.2);
        if (h_force || (fmax(c1, c2) < 1.0 && !(isnan(c1) || isnan(c2)))) {
            dtnext = pymin(1.5 * h, pymin(hn1, hn2));
            break;
        }
        ++nrjct;
        h = pymax(0.5 * h, pymin(hn1, hn2));
        if (h < 1.e-15 || nrjct > 20) {
            if (lead) { C->status = PQ3D_ERR_STEP; C->dttry = h; C->time = time; }
            return;
        }
    }

    // (3) state update (src/QDsim_gpu.py:994-1027)
    double vmax = 0.0;
    for (int64_t i = cell0 + threadIdx.x; i < cell1; i += blockDim.x) {
        const double4_16a y = reinterpret_cast<const double4_16a *>(S.cand)[i];
        const double Tno = y.x, T1 = y.y, T2 = y.z, st = y.w, a = S.a[i];
        S.Tno[i] = Tno; S.Tt1o[i] = T1; S.Tt2o[i] = T2; S.state[i] = st;
        S.Tt[i] = sqrt(T1 * T1 + T2 * T2);
        const double e = (2.0 * S.V0) * exp(-st / a);
        const double v1 = e * sinh(T1 / Tno / a);
        const double v2 = e * sinh(T2 / Tno / a);
        double v = sqrt(v1 * v1 + v2 * v2);
        S.slipv1[i] = v1; S.slipv2[i] = v2;
        S.rake[i] = atan2(v2, v1);
        if (v < 1e-30) v = 1e-30;
        S.slipv[i] = v;
        vmax = (isnan(vmax) || isnan(v)) ? NAN : fmax(vmax, v);
        const double s1 = S.slip1[i] + v1 * h, s2 = S.slip2[i] + v2 * h;
        S.slip1[i] = s1; S.slip2[i] = s2;
        S.slip[i] = sqrt(s1 * s1 + s2 * s2);
        S.fric[i] = S.P ? S.Tt[i] / (Tno - S.P[i] * 1e-6) : S.Tt[i] / Tno;   // pressure before its update
        const double w1 = v1 - S.Vpl * cos(S.rake0[i]), w2 = v2 - S.Vpl * sin(S.rake0[i]);
        if (kF32) vs[i] = split_v(w1, w2);
        else vp[i] = make_double2(w1, w2);
    }
    const unsigned long long bv = block_max_bits(dbits(vmax), red);
    if (threadIdx.x == 0) atomicMax((unsigned long long *)&C->maxv_bits, bv);
    // (3b) pore-pressure diffusion of every cell with the new state and
    // slip rate (src/QDsim_gpu.py:628-671, after the update 1119-1120)
    if (S.Parr) dilatancy_step(S, h, dil_cp, dil_inv, cell0, cell1);
    if (!grid_barrier(bc, bg, nb)) { if (threadIdx.x == 0) C->status = PQ3D_ERR_TIMEOUT; return; }
    if (lead) {
        if (h_hist) h_hist[step] = h;
        if (t_hist) t_hist[step] = time + h;
        C->steps_done += 1;
        C->dttry = dtnext;
        C->time = time + h;
        C->maxv = __longlong_as_double((long long)C->maxv_bits);
    }
}

}  // namespace step
}  // namespace pq3d

extern "C" size_t pq3d_dilatancy_table_len(int ndepth) { return ndepth > 0 ? (size_t)3 * ndepth + pq3d::step::D_NSCAL : 0; }

// The reference's matrix (src/QDsim_gpu.py:611-626) and right-hand-side
// constants (628-671) for depth nodes z[0..ndepth].
extern "C" int pq3d_dilatancy_table(const double *z, int ndepth, double c_hyd, double dilatancy, double thickness,
                                    double compressibility, double P0, double *out)
{
    using namespace pq3d;
    using namespace pq3d::step;
    clear_error();
    PQ3D_REQUIRE(z && out && ndepth >= 2 && ndepth <= kMaxDepth, "pq3d_dilatancy_table: bad arguments (ndepth %d)",
                 ndepth);
    const int n = ndepth;
    double *lo = out, *di = lo + n, *up = di + n, *sc = up + n;
    for (int i = 0; i < n; ++i) {
        const double dz = z[i + 1] - z[i];
        const double em = exp(-(2 * z[i] - dz / 2)), ep = exp(-(2 * z[i] + dz / 2));
        if (i == 0) {
            di[0] = c_hyd * (em + ep) / (dz * dz);
            up[0] = -c_hyd * (em + ep) / (dz * dz);
            lo[0] = 0.0;
        } else {
            di[i] = c_hyd * (em + ep) / (dz * dz);
            up[i] = (i + 1 < n) ? -c_hyd * ep / (dz * dz) : 0.0;
            lo[i] = -c_hyd * em / (dz * dz);
        }
    }
    const double dz0 = z[1] - z[0], dzl = z[n] - z[n - 1];
    sc[D_BC0] = 2.0 * c_hyd * exp(-(z[0] - dz0 / 2)) / dz0;
    sc[D_BCN] = 1.0 / (dzl * dzl) * c_hyd * exp(-(z[n - 1] - dzl / 2)) * P0;
    sc[D_G] = dilatancy * thickness / (2.0 * compressibility * c_hyd);
    sc[D_T1] = exp(-(z[0] - dz0 / 2));
    sc[D_T2] = exp(-(z[0] + dz0 / 2));
    sc[D_TG] = 2 * dz0 * exp(z[0]);
    sc[D_DP] = c_hyd * exp(-z[0]) / (dz0 * dz0);
    return PQ3D_OK;
}

namespace pq3d {
namespace step {

struct LaunchCfg {
    int device = -1;
    int grid64 = 0, grid32 = 0;
};
static thread_local LaunchCfg g_cfg;

static int coop_grid(bool f32, int *grid)
{
    int dev;
    PQ3D_CUDA_TRY(cudaGetDevice(&dev));
    if (g_cfg.device != dev) {
        int sms = 0, coop = 0, b64 = 0, b32 = 0;
        PQ3D_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        PQ3D_CUDA_TRY(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev));
        if (!coop) return set_error(PQ3D_ERR_UNSUPPORTED, "device has no cooperative launch");
        PQ3D_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b64, dense_attempt_kernel<false>, 256, 0));
        PQ3D_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b32, dense_attempt_kernel<true>, 256, 0));
        if (b64 < 1 || b32 < 1) return set_error(PQ3D_ERR_UNSUPPORTED, "stepper kernel does not fit on an SM");
        g_cfg.device = dev;
        g_cfg.grid64 = sms * b64;
        g_cfg.grid32 = sms * b32;
    }
    *grid = f32 ? g_cfg.grid32 : g_cfg.grid64;
    return PQ3D_OK;
}

}  // namespace step
}  // namespace pq3d

using namespace pq3d;
using namespace pq3d::step;

static int matvec(const void *K, int64_t N, const void *v, double *out, void *stream, bool f32)
{
    clear_error();
    PQ3D_REQUIRE(N > 0 && K && v && out, "pq3d_dense_matvec: bad arguments");
    PQ3D_REQUIRE(aligned16(v) && (f32 ? ((uintptr_t)K & 7u) == 0 : aligned16(K)),
                 "pq3d_dense_matvec: K and v must be aligned (16 bytes for FP64, 8 for FP32)");
    const int threads = 256;
    const int64_t warps = N;
    const unsigned blocks = (unsigned)((warps * 32 + threads - 1) / threads);
    if (f32) matvec_kernel<true><<<blocks, threads, 0, (cudaStream_t)stream>>>(K, v, N, out);
    else matvec_kernel<false><<<blocks, threads, 0, (cudaStream_t)stream>>>(K, v, N, out);
    PQ3D_CUDA_TRY(cudaGetLastError());
    return PQ3D_OK;
}

extern "C" int pq3d_dense_matvec_f64(const double *K64, int64_t N, const double *v, double *out, void *stream)
{
    return matvec(K64, N, v, out, stream, false);
}

extern "C" int pq3d_dense_matvec_f32(const float *K32, int64_t N, const float *vsplit, double *out, void *stream)
{
    return matvec(K32, N, vsplit, out, stream, true);
}

extern "C" int pq3d_dense_step(const pq3d_dense_sim *sim, int nsteps, double *h_hist, double *t_hist,
                               const double *h_force, void *stream)
{
    clear_error();
    PQ3D_REQUIRE(sim && sim->N > 0 && nsteps >= 0 && sim->ctrl, "pq3d_dense_step: bad arguments");
    PQ3D_REQUIRE((sim->K64 != nullptr) != (sim->K32 != nullptr), "pq3d_dense_step: exactly one of K64/K32");
    PQ3D_REQUIRE(aligned16(sim->vprime) && aligned16(sim->cand) && aligned16(sim->K64 ? (const void *)sim->K64
                                                                                      : (const void *)sim->K32),
                 "pq3d_dense_step: vprime, cand and K must be 16-byte aligned");
    if (sim->Parr)
        PQ3D_REQUIRE(sim->P && sim->dPdt && sim->dila && sim->ndepth >= 2 && sim->ndepth <= kMaxDepth,
                     "pq3d_dense_step: dilatancy needs P, dPdt, dila and 2 <= ndepth <= %d", kMaxDepth);
    if (nsteps == 0) return PQ3D_OK;
    const bool f32 = sim->K32 != nullptr;
    int grid = 0;
    int rc = coop_grid(f32, &grid);
    if (rc) return rc;
    // clear the reduction slots and the barrier counter of the control block
    cudaStream_t st = (cudaStream_t)stream;
    PQ3D_CUDA_TRY(cudaMemsetAsync(&sim->ctrl->err_slot[0], 0, sizeof(uint64_t) * 7 + sizeof(uint32_t), st));
    pq3d_dense_sim S = *sim;
    const unsigned cell_blocks = (unsigned)((sim->N + 255) / 256);
    const unsigned warp_blocks = (unsigned)((sim->N * 32 + 255) / 256);
    if (f32) vprime_kernel<true><<<cell_blocks, 256, 0, st>>>(S);
    else vprime_kernel<false><<<cell_blocks, 256, 0, st>>>(S);
    PQ3D_CUDA_TRY(cudaGetLastError());
    int step = 0;
    void *args[] = {(void *)&S, (void *)&step, (void *)&h_hist, (void *)&t_hist, (void *)&h_force};
    for (; step < nsteps; ++step) {
        if (f32) {
            step_rates_kernel<true><<<warp_blocks, 256, 0, st>>>(S);
            PQ3D_CUDA_TRY(cudaGetLastError());
            PQ3D_CUDA_TRY(cudaLaunchCooperativeKernel((const void *)dense_attempt_kernel<true>, grid, 256, args, 0, st));
        } else {
            step_rates_kernel<false><<<warp_blocks, 256, 0, st>>>(S);
            PQ3D_CUDA_TRY(cudaGetLastError());
            PQ3D_CUDA_TRY(cudaLaunchCooperativeKernel((const void *)dense_attempt_kernel<false>, grid, 256, args, 0, st));
        }
    }
    return PQ3D_OK;
}
