// Rate-and-state right-hand side and one Dormand-Prince 5(4) attempt of one
// cell, shared by the single-simulation and the batched steppers.
//
// Reference: src/QDsim_gpu.py:772-828 (derivative, with the pore pressure P
// and its rate dPdt of the dilatancy model; both zero when it is off),
// 830-891 (derivative_gpu), 1128-1262 (RungeKutte_solve_Dormand_Prince_gpu).
#pragma once

#include <math.h>

namespace pq3d {
namespace rk {

// Dormand-Prince tableau (src/QDsim_gpu.py:1129-1159)
constexpr double B21 = .2;
constexpr double B31 = 3. / 40, B32 = 9. / 40.;
constexpr double B41 = 44. / 45., B42 = -56. / 15, B43 = 32. / 9;
constexpr double B51 = 19372. / 6561., B52 = -25360 / 2187., B53 = 64448. / 6561., B54 = -212. / 729.;
constexpr double B61 = 9017. / 3168., B62 = -355. / 33., B63 = -46732. / 5247., B64 = 49. / 176.,
                 B65 = -5103. / 18656.;
constexpr double B71 = 35. / 384., B73 = 500. / 1113., B74 = 125. / 192., B75 = -2187. / 6784., B76 = 11. / 84.;
constexpr double B81 = 5179. / 57600., B83 = 7571. / 16695., B84 = 393. / 640., B85 = -92097. / 339200.,
                 B86 = 187. / 2100., B87 = 1. / 40.;
constexpr double kRelTol = 1e-4;

// ---------------------------------------------------------------------------
// right-hand side of one cell (src/QDsim_gpu.py:772-828)

struct Cell {
    double a, b, dc, f0, shear, slipv, AdotV1, AdotV2, dsig;
    double P, dPdt;   // pore pressure (Pa) and its rate (Pa/s); 0 without dilatancy
};

__device__ __forceinline__ double clip700(double x) { return fmin(fmax(x, -700.0), 700.0); }

__device__ __forceinline__ void rhs(const Cell &c, double V0, double eta, double Tno, double Tt1o, double Tt2o,
                                    double state, double &dstate, double &dsig, double &dtau1, double &dtau2)
{
    const double Tn = Tno * 1e6 - c.P, T1 = Tt1o * 1e6, T2 = Tt2o * 1e6;   // effective normal stress
    const double es = exp(clip700(-state / c.a));
    const double aTn = c.a * Tn;
    const double x1 = clip700(T1 / aTn), x2 = clip700(T2 / aTn);
    const double ep1 = exp(x1), em1 = exp(-x1), ep2 = exp(x2), em2 = exp(-x2);
    const double ch1 = (ep1 + em1) / 2, sh1 = (ep1 - em1) / 2;
    const double ch2 = (ep2 + em2) / 2, sh2 = (ep2 - em2) / 2;
    const double aTn2 = c.a * (Tn * Tn);
    const double dV1dtau = 2 * V0 / aTn * es * ch1;
    const double dV2dtau = 2 * V0 / aTn * es * ch2;
    const double dV1dsigma = -2 * V0 * T1 / aTn2 * es * ch1;
    const double dV2dsigma = -2 * V0 * T2 / aTn2 * es * ch2;
    const double dV1dstate = -2 * V0 / c.a * es * sh1;
    const double dV2dstate = -2 * V0 / c.a * es * sh2;
    dstate = c.b / c.dc * (V0 * exp(clip700((c.f0 - state) / c.b)) - c.slipv);
    const double ds = c.dsig - c.dPdt;
    const double t1 = (-c.AdotV1 + c.shear - eta * (dV1dsigma * ds + dV1dstate * dstate)) / (1.0 + eta * dV1dtau);
    const double t2 = (-c.AdotV2 + c.shear - eta * (dV2dsigma * ds + dV2dstate * dstate)) / (1.0 + eta * dV2dtau);
    dsig = c.dsig / 1e6;
    dtau1 = t1 / 1e6;
    dtau2 = t2 / 1e6;
}

// The same right-hand side in reciprocal form: the per-cell quotients 1/a,
// 1/b, b/dc and 2 V0/a once per attempt (`CellRecip`), one division 1/Tn per
// evaluation, e^{-x} as 1/e^{x}, the MPa scaling as a product: 5 divisions
// and 4 exponentials per evaluation against the reference formula's 15 and
// 6, with the same values to ~1e-15 relative.  GB300's FP64 pipe runs at
// 1/64 of the FP32 rate and a division or an exponential is a sequence of
// ~10-25 FP64 instructions, so this halves the FP64 attempt.
struct CellRecip {
    double ia, ib, bdc, v0ia2;   // 1/a, 1/b, b/dc, 2 V0 / a
};

__device__ __forceinline__ CellRecip cell_recip(const Cell &c, double V0)
{
    const double ia = 1.0 / c.a;
    return CellRecip{ia, 1.0 / c.b, c.b / c.dc, 2.0 * V0 * ia};
}

__device__ __forceinline__ void rhs_recip(const Cell &c, const CellRecip &k, double V0, double eta, double Tno,
                                          double Tt1o, double Tt2o, double state, double &dstate, double &dsig,
                                          double &dtau1, double &dtau2)
{
    const double Tn = Tno * 1e6 - c.P, T1 = Tt1o * 1e6, T2 = Tt2o * 1e6;
    const double iTn = 1.0 / Tn, iaTn = k.ia * iTn;
    const double es = exp(clip700(-state * k.ia));
    const double x1 = clip700(T1 * iaTn), x2 = clip700(T2 * iaTn);
    const double ep1 = exp(x1), em1 = 1.0 / ep1, ep2 = exp(x2), em2 = 1.0 / ep2;
    const double ch1 = (ep1 + em1) * 0.5, sh1 = (ep1 - em1) * 0.5;
    const double ch2 = (ep2 + em2) * 0.5, sh2 = (ep2 - em2) * 0.5;
    const double ct = 2.0 * V0 * iaTn * es;    // 2 V0 / (a Tn) e^{-psi/a}
    const double cs = k.v0ia2 * es;            // 2 V0 / a e^{-psi/a}
    const double dV1dtau = ct * ch1, dV2dtau = ct * ch2;
    const double dV1dsigma = -ct * (T1 * iTn) * ch1, dV2dsigma = -ct * (T2 * iTn) * ch2;
    const double dV1dstate = -cs * sh1, dV2dstate = -cs * sh2;
    dstate = k.bdc * (V0 * exp(clip700((c.f0 - state) * k.ib)) - c.slipv);
    const double ds = c.dsig - c.dPdt;
    const double t1 = (-c.AdotV1 + c.shear - eta * (dV1dsigma * ds + dV1dstate * dstate)) / (1.0 + eta * dV1dtau);
    const double t2 = (-c.AdotV2 + c.shear - eta * (dV2dsigma * ds + dV2dstate * dstate)) / (1.0 + eta * dV2dtau);
    dsig = c.dsig * 1e-6;
    dtau1 = t1 * 1e-6;
    dtau2 = t2 * 1e-6;
}


// ---------------------------------------------------------------------------
// Mixed-precision attempt (batched mixed modes).
//
// GB300 runs FP64 at 1/64 of the FP32 rate, so the seven right-hand sides of
// an attempt run in FP32; FP64 is kept for the state itself (start state and
// the accepted update).  Two reformulations keep FP32 both accurate and in
// range:
//
// (1) Increments.  A stage state is the attempt's start state y0 plus an
//     increment h * sum_l A_jl k_l that is formed in FP32 (relative error
//     ~1e-7 of the increment, not of the state).  The large exponent
//     arguments -psi/a and tau/(a sigma) (~200, nearly cancelling) are
//     evaluated once per step at y0, in float-float arithmetic from the
//     split FP64 state (MixedBase, stored per cell); at a stage only their
//     change is added, in FP32, to that float-float value, so the exponent
//     keeps ~1e-7 absolute accuracy.
//
// (2) Scale.  With u = -psi/a + |x|, x = tau/(a sigma), r = e^{-2|x|} and
//     W = eta V0 e^u the traction rate of the right-hand side (the
//     reference's dtau/dt, src/QDsim_gpu.py:772-828) is
//         dtau/dt = (L + W M) / (1 + W D),
//         D = (1 + r) / (a sigma),   M = D (tau/sigma) dsigma/dt
//                                      + sign(x) (1 - r)/a * dpsi/dt,
//     L = -K.v' + shear loading.  W spans e^{+-100} within one attempt
//     (an intermediate Dormand-Prince stage can overshoot by >100 in u;
//     FP64 stays finite there and may still accept the step), so the form
//     is evaluated with w = e^{-|ln W|} <= 1: (L + w M)/(1 + w D) when
//     W < 1, (L w + M)/(w + D) when W >= 1.  Nothing overflows.
//
// Derivatives then match the FP64 right-hand side to ~2e-7 relative and the
// error norms to ~1e-6.  A stage whose FP32 arithmetic still leaves the
// float range (psi itself running away, e^{(f0-psi)/b} > 1e38) gives an
// infinite error, i.e. a rejection with dt halved, which is what the FP64
// arithmetic decides for such a stage; a NaN in the inputs stays NaN.

struct FF {   // hi + lo, |lo| <= ulp(hi) / 2
    float hi, lo;
};

__device__ __forceinline__ FF ff_split(double x)
{
    const float h = (float)x;
    return FF{h, (float)(x - (double)h)};
}

// (b.hi + b.lo) + d as (s, lo); TwoSum with explicit rounding so that the
// compiler does not contract it
__device__ __forceinline__ FF ff_add(FF b, float d)
{
    const float s = __fadd_rn(b.hi, d);
    const float bp = __fsub_rn(s, b.hi);
    const float e = __fadd_rn(__fsub_rn(b.hi, __fsub_rn(s, bp)), __fsub_rn(d, bp));
    return FF{s, __fadd_rn(e, b.lo)};
}

// e^{-|v|} of v = hi + lo: e^{-|hi|} (1 -+ lo), |lo| ~ 1e-6 at most
__device__ __forceinline__ float ff_exp_neg_abs(FF v)
{
    const float e = expf(-fabsf(v.hi));
    return v.hi >= 0.f ? e * (1.f - v.lo) : e * (1.f + v.lo);
}

__device__ __forceinline__ float ff_exp(FF v) { return expf(v.hi) * (1.f + v.lo); }

// float-float arithmetic (Dekker / Knuth error-free transforms with FMA; ~2^-46
// relative), FP32 pipes only; the explicit rounding intrinsics keep the
// compiler from contracting the transforms
__device__ __forceinline__ FF ff_norm(float s, float e)
{
    const float h = __fadd_rn(s, e);
    return FF{h, __fsub_rn(e, __fsub_rn(h, s))};
}

__device__ __forceinline__ FF ff_add2(FF a, FF b)
{
    const float s = __fadd_rn(a.hi, b.hi);
    const float bp = __fsub_rn(s, a.hi);
    float e = __fadd_rn(__fsub_rn(a.hi, __fsub_rn(s, bp)), __fsub_rn(b.hi, bp));
    e = __fadd_rn(e, __fadd_rn(a.lo, b.lo));
    return ff_norm(s, e);
}

__device__ __forceinline__ FF ff_mul(FF a, FF b)
{
    const float p = __fmul_rn(a.hi, b.hi);
    float e = __fmaf_rn(a.hi, b.hi, -p);
    e = __fmaf_rn(a.hi, b.lo, e);
    e = __fmaf_rn(a.lo, b.hi, e);
    return ff_norm(p, e);
}

__device__ __forceinline__ FF ff_neg(FF a) { return FF{-a.hi, -a.lo}; }

// 1/d: the FP32 reciprocal r and one Newton step r + r (1 - d r), the
// residual 1 - d r formed exactly with FMAs
__device__ __forceinline__ FF ff_rcp(FF d)
{
    const float r = __frcp_rn(d.hi);
    float e = __fmaf_rn(-d.hi, r, 1.f);
    e = __fmaf_rn(-d.lo, r, e);
    return ff_norm(r, __fmul_rn(r, e));
}

// Constants of one cell at the start of a step (y0), shared by all the
// attempts of the step: computed once per accepted step, in float-float from
// the FP64 state (GB300's FP64 pipe, which also executes the FP64<->FP32
// conversions and the FP64 compares, is 1/64 of the FP32 rate), and stored as
// kBaseFields floats per cell.
struct MixedBase {
    float Tn0;          // effective normal stress at y0 (MPa)
    float q0[2];        // tau_k / sigma at y0
    float x0[2];        // tau_k / (a sigma) at y0 (FP32: sign and r only)
    FF Sp[2], Sm[2];    // -psi0/a + ln(eta V0) +- tau_k / (a sigma)
    FF g0;              // (f0 - psi0) / b
    float a, inv_a, inv_b, bdc;
    float slipv;        // slip rate at the start of the step
    // per attempt (not stored)
    float V0, dsf;      // V0; dsigma/dt - dP/dt (Pa/s)
    float L[2];         // -K.v' + shear loading (Pa/s)
};
// stored per cell: the 20 fields above, then the cell constants 1/a, 1/b and
// f0 as float-float lo parts / pairs (fields 20-23: 1/a lo, 1/b lo, f0 hi, f0 lo)
constexpr int kBaseFields = 24;

// The cell's constants, set once (FP64 quotients, split), fields 15-18, 20-23.
__device__ __forceinline__ void store_base_constants(float *p, int64_t stride, double a, double b, double dc,
                                                     double f0)
{
    const FF ia = ff_split(1.0 / a), ib = ff_split(1.0 / b), ff0 = ff_split(f0);
    p[15 * stride] = (float)a;
    p[16 * stride] = ia.hi;
    p[17 * stride] = ib.hi;
    p[18 * stride] = (float)b / (float)dc;
    p[20 * stride] = ia.lo;
    p[21 * stride] = ib.lo;
    p[22 * stride] = ff0.hi;
    p[23 * stride] = ff0.lo;
}

// The state-dependent constants (fields 0-14) of the state (Tn0, T1, T2, psi)
// (MPa, MPa, MPa, state), in float-float from the FP64 state: the FP64 work is
// the four splits.  c0 = ln(eta V0) as float-float.
__device__ __forceinline__ void store_base_state(float *p, int64_t stride, double Tn0, double T1, double T2,
                                                 double psi, FF c0, MixedBase &m)
{
    const float *q = p;
    const FF ia{q[16 * stride], q[20 * stride]}, ib{q[17 * stride], q[21 * stride]};
    const FF f0{q[22 * stride], q[23 * stride]};
    const FF tn = ff_split(Tn0), t1 = ff_split(T1), t2 = ff_split(T2), ps = ff_split(psi);
    const FF r0 = ff_rcp(tn);
    const FF q1 = ff_mul(t1, r0), q2 = ff_mul(t2, r0);
    const FF x1 = ff_mul(q1, ia), x2 = ff_mul(q2, ia);
    const FF sp = ff_add2(ff_neg(ff_mul(ps, ia)), c0);
    m.Tn0 = tn.hi;
    m.q0[0] = q1.hi; m.q0[1] = q2.hi;
    m.inv_a = ia.hi;
    m.x0[0] = m.q0[0] * m.inv_a; m.x0[1] = m.q0[1] * m.inv_a;
    m.Sp[0] = ff_add2(sp, x1); m.Sm[0] = ff_add2(sp, ff_neg(x1));
    m.Sp[1] = ff_add2(sp, x2); m.Sm[1] = ff_add2(sp, ff_neg(x2));
    m.g0 = ff_mul(ff_add2(f0, ff_neg(ps)), ib);
    const float v[15] = {m.Tn0, m.q0[0], m.q0[1], m.x0[0], m.x0[1], m.Sp[0].hi, m.Sp[0].lo, m.Sp[1].hi,
                         m.Sp[1].lo, m.Sm[0].hi, m.Sm[0].lo, m.Sm[1].hi, m.Sm[1].lo, m.g0.hi, m.g0.lo};
#pragma unroll
    for (int k = 0; k < 15; ++k) p[k * stride] = v[k];
}

__device__ __forceinline__ MixedBase load_base(const float *__restrict__ p, int64_t stride)
{
    float v[20];
#pragma unroll
    for (int k = 0; k < 20; ++k) v[k] = __ldg(p + k * stride);
    MixedBase m;
    m.Tn0 = v[0];
    m.q0[0] = v[1]; m.q0[1] = v[2];
    m.x0[0] = v[3]; m.x0[1] = v[4];
    m.Sp[0] = FF{v[5], v[6]}; m.Sp[1] = FF{v[7], v[8]};
    m.Sm[0] = FF{v[9], v[10]}; m.Sm[1] = FF{v[11], v[12]};
    m.g0 = FF{v[13], v[14]};
    m.a = v[15]; m.inv_a = v[16]; m.inv_b = v[17]; m.bdc = v[18]; m.slipv = v[19];
    return m;
}

// slip rate 2 V0 e^{-psi/a} sinh(x), x = tau/(a sigma), from the constants:
// V0 sign(x) e^{-psi/a + |x|} (1 - e^{-2|x|}) = sign(x) W (1 - r) / eta
__device__ __forceinline__ float base_slip_rate(const MixedBase &m, int k, float inv_eta)
{
    const float x = m.x0[k];
    const FF lw = x >= 0.f ? m.Sp[k] : m.Sm[k];
    const float v = ff_exp(lw) * inv_eta * -expm1f(-2.f * fabsf(x));
    return x < 0.f ? -v : v;
}

// Right-hand side at y0 + (dTn, dT1, dT2, dpsi) (MPa, MPa, MPa, state):
// dpsi/dt and dtau_k/dt (MPa/s).
__device__ __forceinline__ void mixed_rhs(const MixedBase &m, float dTn, float dT1, float dT2, float dpsi,
                                          float &dstate, float &dtau1, float &dtau2)
{
    const float rTn = __frcp_rn(m.Tn0 + dTn);
    const float iaTn = m.inv_a * rTn;                          // 1 / (a sigma), 1/MPa
    const float ed = ff_exp(ff_add(m.g0, -dpsi * m.inv_b));    // e^{(f0 - psi)/b}
    const float ds_dt = m.bdc * (m.V0 * ed - m.slipv);
    const float dpa = dpsi * m.inv_a;
    float out[2];
#pragma unroll
    for (int k = 0; k < 2; ++k) {
        const float dx = ((k ? dT2 : dT1) - m.q0[k] * dTn) * iaTn;   // change of tau/(a sigma)
        const float xs = m.x0[k] + dx;
        const bool pos = xs >= 0.f;
        const float em = expm1f(-2.f * fabsf(xs));                  // r - 1
        const FF lw = ff_add(pos ? m.Sp[k] : m.Sm[k], (pos ? dx : -dx) - dpa);   // ln W
        const float w = ff_exp_neg_abs(lw);
        const float q = m.q0[k] + m.a * dx;                         // tau / sigma
        const float D = (2.f + em) * iaTn * 1e-6f;                  // (1 + r) / (a sigma), 1/Pa
        const float M = D * q * m.dsf + m.inv_a * (pos ? -em : em) * ds_dt;
        const float L = m.L[k];
        out[k] = (lw.hi >= 0.f) ? __fdiv_rn(fmaf(L, w, M), w + D) : __fdiv_rn(fmaf(w, M, L), fmaf(w, D, 1.f));
    }
    dstate = ds_dt;
    dtau1 = out[0] * 1e-6f;
    dtau2 = out[1] * 1e-6f;
}

// |num| / |yo + num|: in FP32 where yo + num is in float range, else in FP64
__device__ __forceinline__ float rel_err(float num, double yo)
{
    const float ay = fabsf((float)yo + num);
    if (ay >= 1e-30f && ay <= 1e30f) return __fdiv_rn(fabsf(num), ay);
    return (float)(fabs((double)num) / fabs(yo + (double)num));
}

__device__ __forceinline__ bool finite_inputs(const MixedBase &m, const double y[4], float dsig)
{
    return isfinite(y[0]) && isfinite(y[1]) && isfinite(y[2]) && isfinite(y[3]) && isfinite(m.L[0]) &&
           isfinite(m.L[1]) && isfinite(dsig) && isfinite(m.slipv);
}

// One Dormand-Prince attempt of one cell in the mixed arithmetic above, from
// the cell's start-of-step constants m (with V0, dsf and L set) and its
// normal-stress rate dsig (Pa/s).  Writes the 5th-order solution to yo and
// returns the two relative errors (as the FP64 attempt below; as floats:
// they only decide accept / reject and the next dt).
__device__ __forceinline__ void dp_attempt_mixed(const MixedBase &m, float dsig, float hf, const double y[4],
                                                 double yo[4], float &e1, float &e2)
{
    const float dn = dsig * 1e-6f;   // d(Tno)/dt, MPa/s, constant over the step
    const float A[6][6] = {{(float)B21, 0, 0, 0, 0, 0},
                           {(float)B31, (float)B32, 0, 0, 0, 0},
                           {(float)B41, (float)B42, (float)B43, 0, 0, 0},
                           {(float)B51, (float)B52, (float)B53, (float)B54, 0, 0},
                           {(float)B61, (float)B62, (float)B63, (float)B64, (float)B65, 0},
                           {(float)B71, 0.f, (float)B73, (float)B74, (float)B75, (float)B76}};
    const float wsum[6] = {(float)B21, (float)(B31 + B32), (float)(B41 + B42 + B43), (float)(B51 + B52 + B53 + B54),
                           (float)(B61 + B62 + B63 + B64 + B65), (float)(B71 + B73 + B74 + B75 + B76)};
    float s[7], t[7], u[7];
    float inc[4] = {0.f, 0.f, 0.f, 0.f};
    mixed_rhs(m, 0.f, 0.f, 0.f, 0.f, s[0], t[0], u[0]);
#pragma unroll
    for (int j = 0; j < 6; ++j) {
        float ds = 0.f, dt1 = 0.f, dt2 = 0.f;
#pragma unroll
        for (int l = 0; l <= j; ++l) {
            ds = fmaf(A[j][l], s[l], ds);
            dt1 = fmaf(A[j][l], t[l], dt1);
            dt2 = fmaf(A[j][l], u[l], dt2);
        }
        const float dTn = hf * (wsum[j] * dn), dT1 = hf * dt1, dT2 = hf * dt2, dps = hf * ds;
        if (j == 5) { inc[0] = dTn; inc[1] = dT1; inc[2] = dT2; inc[3] = dps; }
        mixed_rhs(m, dTn, dT1, dT2, dps, s[j + 1], t[j + 1], u[j + 1]);
    }
    yo[0] = y[0] + (double)inc[0];
    yo[1] = y[1] + (double)inc[1];
    yo[2] = y[2] + (double)inc[2];
    yo[3] = y[3] + (double)inc[3];
    // 4th-order minus 5th-order solution: h * sum (B8i - B7i) k_i
    const float D[7] = {(float)(B81 - B71), 0.f, (float)(B83 - B73), (float)(B84 - B74), (float)(B85 - B75),
                        (float)(B86 - B76), (float)B87};
    float es = 0.f, e1t = 0.f, e2t = 0.f;
#pragma unroll
    for (int l = 0; l < 7; ++l) {
        es = fmaf(D[l], s[l], es);
        e1t = fmaf(D[l], t[l], e1t);
        e2t = fmaf(D[l], u[l], e2t);
    }
    es *= hf; e1t *= hf; e2t *= hf;
    // the normal stress: its rate is constant, the two orders differ by the
    // rounding of the weight sums
    const float wn = (float)((B81 + B83 + B84 + B85 + B86 + B87) - (B71 + B73 + B74 + B75 + B76));
    const float en = hf * (wn * dn);
    e1 = rel_err(es, yo[3]);
    const float ea = rel_err(e1t, yo[1]), eb = rel_err(e2t, yo[2]), ec = rel_err(en, yo[0]);
    e2 = (isnan(ea) || isnan(eb) || isnan(ec)) ? NAN : fmaxf(fmaxf(ea, eb), ec);
    if (!(isfinite(e1) && isfinite(e2)) && finite_inputs(m, y, dsig)) {
        if (!isfinite(e1)) e1 = INFINITY;
        if (!isfinite(e2)) e2 = INFINITY;
    }
}

// ---------------------------------------------------------------------------
// Float-float attempt (batched products with attempt64 = 2).
//
// The right-hand sides of the mixed attempt above, in float-float (hi + lo,
// ~2^-46 relative) instead of FP32, so that the attempt carries the FP64
// attempt's accuracy on the FP32 pipes.  What FP64 keeps is the work whose
// absolute accuracy matters: the large exponent arguments at the start
// state, ln(eta V0) - psi0/a +- tau_k/(a sigma) and (f0 - psi0)/b (each ~1e2
// and nearly cancelling), formed in FP64 once per attempt and carried as
// K ln 2 + r with an integer K and a float-float |r| <= ln 2 / 2 (Cody and
// Waite's reduction), so that their absolute error stays at the FP64 level
// (~1e-14) where a float-float value of ~1e2 would keep only ~1e-12.  At a
// stage only the change of each argument is added to r.  The exponentials
// are float-float; e^t - 1 (for 1 -+ e^{-2|x|} near x = 0) by reduction by a
// multiple of ln 2 and by 2^-5, the Taylor sum of e^s - 1 to s^7 (terms
// beyond s^3 in FP32, below 2^-48 of the sum), then five doublings
// p <- p (p + 2), which keep the relative accuracy of e^s - 1.
// The exponentials of the arguments carried as K ln 2 + r use a 64-entry
// table of 2^{j/64} and a Taylor sum to s^6 (|s| <= ln 2 / 128); e^{-2|x|} - 1
// near x = 0 keeps the doubling form.
// Units: stresses in MPa, so the right-hand side yields dtau/dt in MPa/s
// directly (the factors 1e-6 sit in the FP64 constants).  The float range
// bounds it like the mixed attempt: a stage with e^{(f0-psi)/b} > 1e38 gives
// an infinite error (a rejection, as FP64 decides for such a stage).

struct FFc {   // compile-time float-float constant
    float hi, lo;
};
__host__ __device__ constexpr FFc ffc(double x) { return FFc{(float)x, (float)(x - (double)(float)x)}; }
__device__ __forceinline__ FF ffv(FFc c) { return FF{c.hi, c.lo}; }

// FP64 <-> float-float with integer operations: GB300's FP64 pipe, which
// also executes the FP64 <-> FP32 conversions, runs at 1/64 of the FP32 rate.
// ff_split_fast: hi = x truncated to 24 significant bits, lo = the next 24
// (truncated: |x - hi - lo| < 2^-47 |x|), renormalised; |x| outside
// [2^-60, 2^127) (and infinities, NaN) takes the conversions of ff_split,
// out of line (a branch, not conversions predicated into every call),
// zero and FP64 subnormals give a signed zero.
static __device__ __noinline__ FF ff_split_rare(double x) { return ff_split(x); }
__device__ __forceinline__ FF ff_split_fast(double x)
{
    const unsigned hw = (unsigned)__double2hiint(x), lw = (unsigned)__double2loint(x);
    const int e = (int)((hw >> 20) & 0x7ffu);
    if (e == 0) return FF{__uint_as_float(hw & 0x80000000u), 0.f};
    if (e < 1023 - 60 || e > 1023 + 126) return ff_split_rare(x);
    const unsigned sign = hw & 0x80000000u;
    const float hi =
        __uint_as_float(sign | ((unsigned)(e - 1023 + 127) << 23) | ((hw & 0xfffffu) << 3) | (lw >> 29));
    const unsigned rem = lw & 0x1fffffffu;   // the 29 mantissa bits below hi's
    if (rem == 0) return FF{hi, 0.f};
    const int p = 31 - __clz((int)rem);       // rem = 2^p (1.m): p in 0..28
    const unsigned m = p <= 23 ? (rem << (23 - p)) : (rem >> (p - 23));
    const float lo = __uint_as_float(sign | ((unsigned)(p + e - 1075 + 127) << 23) | (m & 0x7fffffu));
    return ff_norm(hi, lo);
}

// float -> FP64 by the bit layout, integer operations only: normal floats
// re-biased; zero; subnormals normalised by the position of their leading
// bit (value = m 2^-149); infinities and NaN keep the all-ones exponent
__device__ __forceinline__ double f2d_bits(float f)
{
    const unsigned u = __float_as_uint(f);
    const unsigned sign = u & 0x80000000u, ef = (u >> 23) & 0xffu, mf = u & 0x7fffffu;
    unsigned hi, lo;
    if (ef == 0xffu) {
        hi = sign | 0x7ff00000u | (mf >> 3);
        lo = mf << 29;
    } else if (ef != 0) {
        hi = sign | ((ef - 127 + 1023) << 20) | (mf >> 3);
        lo = mf << 29;
    } else if (mf == 0) {
        hi = sign;
        lo = 0;
    } else {
        const int p = 31 - __clz((int)mf);   // leading bit: 0..22
        const unsigned long long m = (unsigned long long)(mf ^ (1u << p)) << (52 - p);
        hi = sign | ((unsigned)(p - 149 + 1023) << 20) | (unsigned)(m >> 32);
        lo = (unsigned)m;
    }
    return __hiloint2double((int)hi, (int)lo);
}

__device__ __forceinline__ double ff_to_double_fast(FF a) { return f2d_bits(a.hi) + f2d_bits(a.lo); }

constexpr double kLn2 = 0.69314718055994530941723212145818;
constexpr double kLn2Hi = kLn2;                                   // ln 2 rounded to FP64
constexpr double kLn2Lo = 2.3190468138462996154e-17;              // ln 2 - kLn2Hi
constexpr FFc kFFLn2 = ffc(kLn2);

__device__ __forceinline__ FF ff_sub(FF a, FF b) { return ff_add2(a, ff_neg(b)); }

__device__ __forceinline__ FF ff_mulf(FF a, float b)
{
    const float p = __fmul_rn(a.hi, b);
    float e = __fmaf_rn(a.hi, b, -p);
    e = __fmaf_rn(a.lo, b, e);
    return ff_norm(p, e);
}

// a / b: q1 = a.hi / b.hi, the remainder a - q1 b in float-float, one
// correction quotient
__device__ __forceinline__ FF ff_div(FF a, FF b)
{
    const float rb = __frcp_rn(b.hi);
    const float q1 = __fmul_rn(a.hi, rb);
    const FF rem = ff_sub(a, ff_mulf(b, q1));
    return ff_norm(q1, __fmul_rn(rem.hi, rb));
}

// a 2^k by two exact power-of-two products (FP32 pipe only; k clamped to
// +-252, beyond which every float result is 0 or infinite anyway)
__device__ __forceinline__ FF ff_ldexp(FF a, int k)
{
    k = min(252, max(-252, k));
    const int k1 = k >> 1, k2 = k - k1;
    const float s1 = __int_as_float((k1 + 127) << 23), s2 = __int_as_float((k2 + 127) << 23);
    return FF{__fmul_rn(__fmul_rn(a.hi, s1), s2), __fmul_rn(__fmul_rn(a.lo, s1), s2)};
}

// e^t = 2^k (1 + p) with |p| < 0.42, p returned.  k = rint(t / ln 2) by the
// 1.5 2^23 addition (the integer lands in the low mantissa bits; no
// float-to-integer conversion), t clamped to +-200 (e^{+-200} is out of the
// float-float range: the caller's scaling saturates to 0 or infinity)
__device__ __forceinline__ FF ff_expm1_red(FF t, int &k)
{
    if (!(fabsf(t.hi) <= 200.f)) t = FF{t.hi != t.hi ? t.hi : copysignf(200.f, t.hi), 0.f};
    const float sum = __fadd_rn(__fmul_rn(t.hi, 1.44269504f), 12582912.f);
    const float kf = __fsub_rn(sum, 12582912.f);
    k = __float_as_int(sum) - 0x4B400000;
    FF s = ff_add2(t, ff_mulf(ffv(kFFLn2), -kf));   // |s| <= ln 2 / 2 (+ rounding)
    s.hi *= 0.03125f;
    s.lo *= 0.03125f;
    const float x = s.hi;
    constexpr FFc c3 = ffc(1.0 / 6.0);
    const float T = fmaf(x, fmaf(x, fmaf(x, (float)(1.0 / 5040.0), (float)(1.0 / 720.0)), (float)(1.0 / 120.0)),
                         (float)(1.0 / 24.0));
    const FF u = ff_add2(ffv(c3), FF{__fmul_rn(x, T), 0.f});    // 1/6 + s/24 + ...
    const FF v = ff_add2(FF{0.5f, 0.f}, ff_mul(s, u));            // 1/2 + s u
    FF p = ff_add2(s, ff_mul(ff_mul(s, s), v));                    // s + s^2 v = e^s - 1
#pragma unroll
    for (int d = 0; d < 5; ++d) p = ff_mul(p, ff_add2(p, FF{2.f, 0.f}));
    return p;
}

// e^t - 1
__device__ __forceinline__ FF ff_expm1(FF t)
{
    int k;
    const FF p = ff_expm1_red(t, k);
    return k == 0 ? p : ff_add2(ff_ldexp(ff_add2(FF{1.f, 0.f}, p), k), FF{-1.f, 0.f});
}

// e^{-2x} - 1 for x >= 0 (a float-float |tau / (a sigma)|).  For x >= 8.5,
// r = e^{-2x} < 2^-24 is only the low part of -1 + r, so FP32 accuracy of r
// is float-float accuracy of the sum: r = expf(-2 hi) (1 - 2 lo) (the factor
// takes the low part of x to first order); below, the float-float e^t - 1.
__device__ __forceinline__ FF ff_em(FF x)
{
    return x.hi >= 8.5f ? FF{-1.f, expf(-2.f * x.hi) * (1.f - 2.f * x.lo)} : ff_expm1(FF{-2.f * x.hi, -2.f * x.lo});
}


// e^x by its Taylor series in FP64 (compile time, |x| < 0.7: 30 terms reach
// the FP64 rounding)
__host__ __device__ constexpr double exp_series(double x)
{
    double term = 1.0, sum = 1.0;
    for (int n = 1; n < 30; ++n) { term *= x / n; sum += term; }
    return sum;
}
// 2^{j/64}, j = 0..63, as float-float; each attempt block copies it to
// shared memory (lanes index it independently)
struct Exp2Table {
    FFc v[64];
    __host__ __device__ constexpr Exp2Table() : v()
    {
        for (int j = 0; j < 64; ++j) v[j] = ffc(exp_series(j * (kLn2 / 64.0)));
    }
};
static __constant__ Exp2Table kExp2Tab{};
constexpr FFc kFFLn2_64 = ffc(kLn2 / 64.0);

// e^{K ln 2 + t} = 2^{K + n/64} e^s, n = rint(64 t / ln 2), s = t - n ln 2 / 64
// (|s| <= ln 2 / 128: the Taylor sum to s^6, terms beyond s^3 in FP32), the
// factor 2^{(n mod 64)/64} from the table tab (shared memory)
__device__ __forceinline__ FF ff_exp2k_tab(int K, FF t, const FF *tab)
{
    if (!(fabsf(t.hi) <= 200.f)) t = FF{t.hi != t.hi ? t.hi : copysignf(200.f, t.hi), 0.f};
    const float sum = __fadd_rn(__fmul_rn(t.hi, 92.332482616893656f), 12582912.f);
    const float nf = __fsub_rn(sum, 12582912.f);
    const int n = __float_as_int(sum) - 0x4B400000;
    const FF s = ff_add2(t, ff_mulf(ffv(kFFLn2_64), -nf));
    const float x = s.hi;
    constexpr FFc c3 = ffc(1.0 / 6.0);
    const float T = fmaf(x, fmaf(x, (float)(1.0 / 720.0), (float)(1.0 / 120.0)), (float)(1.0 / 24.0));
    const FF u = ff_add2(ffv(c3), FF{__fmul_rn(x, T), 0.f});
    const FF v = ff_add2(FF{0.5f, 0.f}, ff_mul(s, u));
    const FF p = ff_add2(s, ff_mul(ff_mul(s, s), v));
    const FF tj = tab[n & 63];
    return ff_ldexp(ff_add2(tj, ff_mul(tj, p)), (n >> 6) + K);
}

// u = K ln 2 + r: K = rint(u / ln 2) by the 1.5 2^52 addition (the integer
// lands in the low word: no conversion instruction), r in FP64 to ~1e-16
// absolute, then split
__device__ __forceinline__ void reduce_ln2(double u, int &K, FF &r)
{
    // u clamped to [-1e4, 1e4] (NaN -> -1e4), tested on the high word:
    // 0x40C38800 is the high word of 1e4, so |u| >= 1e4, infinities and NaN
    // take the branch
    if ((__double2hiint(u) & 0x7fffffff) >= 0x40C38800) u = u != u ? -1.0e4 : copysign(1.0e4, u);
    const double t = fma(u, 1.4426950408889634, 6755399441055744.0);
    const double kd = t - 6755399441055744.0;
    K = __double2loint(t);
    r = ff_split_fast(fma(-kd, kLn2Lo, fma(-kd, kLn2Hi, u)));
}

// 1/a in FP64 from the float-float reciprocal and one Newton step (three
// FP64-pipe instructions where an FP64 division is a sequence of many)
__device__ __forceinline__ double rcp_d(double a)
{
    const double r0 = ff_to_double_fast(ff_rcp(ff_split_fast(a)));
    return fma(r0, fma(-a, r0, 1.0), r0);
}

// One cell at the attempt's start state y0 (float-float unless noted).
struct FFCell {
    FF sig0;          // effective normal stress (MPa)
    FF q0[2];         // tau_k / sigma
    FF x0[2];         // tau_k / (a sigma)
    int Ku[2][2];     // ln(eta V0 1e-6) - psi0/a + (x0_k, -x0_k) = Ku ln 2 + ru   ([k][0: +x, 1: -x])
    FF ru[2][2];
    int Kg;           // (f0 - psi0) / b = Kg ln 2 + rg
    FF rg;
    FF a, ia, ib, bdc, V0, slipv;
    FF dsf;           // dsigma/dt - dP/dt (MPa/s)
    FF L[2];          // -K.v'_k + shear loading (MPa/s)
};

// dpsi/dt (1/s) and dtau_k/dt (MPa/s) at y0 + (dTn, dT1, dT2, dpsi): the
// w-form of the mixed right-hand side, (L + w M)/(1 + w D) for W < 1 and
// (L w + M)/(w + D) for W >= 1, w = e^{-|ln W|} (W = eta V0 e^u in MPa).
// Not inlined: the seven call sites of an attempt share one copy of its code
// (inlined seven times the attempt overflowed the instruction cache).
static __device__ __noinline__ void ff_rhs(const FFCell &m, FF dTn, FF dT1, FF dT2, FF dpsi, FF &dstate, FF &dtau1,
                                    FF &dtau2, const FF *tab)
{
    const FF rs = ff_rcp(ff_add2(m.sig0, dTn));                   // 1 / sigma
    const FF iaS = ff_mul(m.ia, rs);                               // 1 / (a sigma)
    const FF ed = ff_exp2k_tab(m.Kg, ff_sub(m.rg, ff_mul(dpsi, m.ib)), tab);   // e^{(f0 - psi)/b}
    const FF ds_dt = ff_mul(m.bdc, ff_sub(ff_mul(m.V0, ed), m.slipv));
    const FF dpa = ff_mul(dpsi, m.ia);
    FF out[2];
#pragma unroll
    for (int k = 0; k < 2; ++k) {
        const FF dx = ff_mul(ff_sub(k ? dT2 : dT1, ff_mul(m.q0[k], dTn)), iaS);   // change of tau/(a sigma)
        const FF xs = ff_add2(m.x0[k], dx);
        const bool pos = xs.hi >= 0.f;
        const FF ax = pos ? xs : ff_neg(xs);
        // r - 1, r = e^{-2|x|} (ff_em)
        const FF em = ff_em(ax);
        const int K = m.Ku[k][pos ? 0 : 1];
        const FF res = ff_sub(ff_add2(m.ru[k][pos ? 0 : 1], pos ? dx : ff_neg(dx)), dpa);   // ln W - K ln 2
        // W >= 1; K as a float by the 1.5 2^23 bias (|K| < 2^22: no conversion instruction)
        const bool big = fmaf(__fsub_rn(__int_as_float(0x4B400000 + K), 12582912.f), 0.693147182f, res.hi) >= 0.f;
        const FF w = big ? ff_exp2k_tab(-K, ff_neg(res), tab) : ff_exp2k_tab(K, res, tab);                  // e^{-|ln W|}
        const FF q = ff_add2(m.q0[k], ff_mul(m.a, dx));                                    // tau / sigma
        const FF D = ff_mul(ff_add2(FF{2.f, 0.f}, em), iaS);                               // (1 + r)/(a sigma)
        const FF M = ff_add2(ff_mul(ff_mul(D, q), m.dsf), ff_mul(m.ia, ff_mul(pos ? ff_neg(em) : em, ds_dt)));
        out[k] = big ? ff_div(ff_add2(ff_mul(m.L[k], w), M), ff_add2(w, D))
                     : ff_div(ff_add2(m.L[k], ff_mul(w, M)), ff_add2(FF{1.f, 0.f}, ff_mul(w, D)));
    }
    dstate = ds_dt;
    dtau1 = out[0];
    dtau2 = out[1];
}

__device__ __forceinline__ double ff_to_double(FF a) { return (double)a.hi + (double)a.lo; }

__device__ __forceinline__ bool ff_finite(FF a) { return isfinite(a.hi) && isfinite(a.lo); }

// Rates of one cell for the float-float attempt, as float-float values from
// the product's partial sums (no FP64 arithmetic): K.v' strike and dip
// (Pa/s), the normal-stress rate dsigma/dt (Pa/s, loading included).
struct FFRates {
    FF A1, A2, dsig;
};

// One Dormand-Prince attempt of one cell in the float-float arithmetic above
// (the stage sums h sum_l A_jl k_l in float-float, the start state and the
// 5th-order solution in FP64).  c supplies the cell's friction parameters,
// shear loading, slip rate and pore pressure (its AdotV and dsig fields are
// not read: the rates come as float-float in q).  lnEV = ln(eta V0 1e-6).
// Writes the 5th-order solution to yo and returns the two relative errors.
__device__ __forceinline__ void dp_attempt_ff(const Cell &c, const FFRates &q, double V0, double lnEV, double h,
                                              const double y[4], double yo[4], double &e1, double &e2, const FF *tab)
{
    constexpr FFc kMicro = ffc(1e-6);
    FFCell m;
    {   // FP64 once per attempt
        const double Tn0 = y[0] - c.P * 1e-6;                    // MPa
        const double ia = rcp_d(c.a), iaT = rcp_d(c.a * Tn0);
        const double base = lnEV - y[3] * ia;                    // ln(eta V0 1e-6) - psi0/a
#pragma unroll
        for (int k = 0; k < 2; ++k) {
            const double x = y[1 + k] * iaT;
            m.x0[k] = ff_split_fast(x);
            m.q0[k] = ff_split_fast(x * c.a);
            reduce_ln2(base + x, m.Ku[k][0], m.ru[k][0]);
            reduce_ln2(base - x, m.Ku[k][1], m.ru[k][1]);
        }
        reduce_ln2((c.f0 - y[3]) * rcp_d(c.b), m.Kg, m.rg);
        m.sig0 = ff_split_fast(Tn0);
        m.ia = ff_split_fast(ia);
        m.a = ff_split_fast(c.a);
        const FF b = ff_split_fast(c.b);
        m.ib = ff_rcp(b);
        m.bdc = ff_mul(b, ff_rcp(ff_split_fast(c.dc)));
        m.V0 = ff_split_fast(V0);
        m.slipv = ff_split_fast(c.slipv);
        m.dsf = ff_mul(ff_sub(q.dsig, ff_split_fast(c.dPdt)), ffv(kMicro));
        const FF shear = ff_split_fast(c.shear);
        m.L[0] = ff_mul(ff_sub(shear, q.A1), ffv(kMicro));
        m.L[1] = ff_mul(ff_sub(shear, q.A2), ffv(kMicro));
    }
    constexpr FFc A[6][6] = {{ffc(B21), {0, 0}, {0, 0}, {0, 0}, {0, 0}, {0, 0}},
                             {ffc(B31), ffc(B32), {0, 0}, {0, 0}, {0, 0}, {0, 0}},
                             {ffc(B41), ffc(B42), ffc(B43), {0, 0}, {0, 0}, {0, 0}},
                             {ffc(B51), ffc(B52), ffc(B53), ffc(B54), {0, 0}, {0, 0}},
                             {ffc(B61), ffc(B62), ffc(B63), ffc(B64), ffc(B65), {0, 0}},
                             {ffc(B71), {0, 0}, ffc(B73), ffc(B74), ffc(B75), ffc(B76)}};
    constexpr FFc wsum[6] = {ffc(B21), ffc(B31 + B32), ffc(B41 + B42 + B43), ffc(B51 + B52 + B53 + B54),
                             ffc(B61 + B62 + B63 + B64 + B65), ffc(B71 + B73 + B74 + B75 + B76)};
    constexpr FFc Dw[7] = {ffc(B81 - B71), {0, 0}, ffc(B83 - B73), ffc(B84 - B74), ffc(B85 - B75), ffc(B86 - B76),
                           ffc(B87)};
    const FF hf = ff_split_fast(h);
    const FF dn = ff_mul(q.dsig, ffv(kMicro));   // d(Tno)/dt (MPa/s), constant over the step
    FF s[7], t[7], u[7];
    FF inc[4];
    const FF z{0.f, 0.f};
    ff_rhs(m, z, z, z, z, s[0], t[0], u[0], tab);
#pragma unroll
    for (int j = 0; j < 6; ++j) {
        FF ds = z, dt1 = z, dt2 = z;
#pragma unroll
        for (int l = 0; l <= j; ++l) {
            if (A[j][l].hi == 0.f) continue;
            ds = ff_add2(ds, ff_mul(ffv(A[j][l]), s[l]));
            dt1 = ff_add2(dt1, ff_mul(ffv(A[j][l]), t[l]));
            dt2 = ff_add2(dt2, ff_mul(ffv(A[j][l]), u[l]));
        }
        const FF dTn = ff_mul(hf, ff_mul(ffv(wsum[j]), dn)), dT1 = ff_mul(hf, dt1), dT2 = ff_mul(hf, dt2),
                 dps = ff_mul(hf, ds);
        if (j == 5) { inc[0] = dTn; inc[1] = dT1; inc[2] = dT2; inc[3] = dps; }
        ff_rhs(m, dTn, dT1, dT2, dps, s[j + 1], t[j + 1], u[j + 1], tab);
    }
#pragma unroll
    for (int q = 0; q < 4; ++q) yo[q] = y[q] + ff_to_double_fast(inc[q]);
    // 4th-order minus 5th-order solution: h sum (B8l - B7l) k_l
    FF es = z, e1t = z, e2t = z;
#pragma unroll
    for (int l = 0; l < 7; ++l) {
        if (Dw[l].hi == 0.f) continue;
        es = ff_add2(es, ff_mul(ffv(Dw[l]), s[l]));
        e1t = ff_add2(e1t, ff_mul(ffv(Dw[l]), t[l]));
        e2t = ff_add2(e2t, ff_mul(ffv(Dw[l]), u[l]));
    }
    es = ff_mul(hf, es);
    e1t = ff_mul(hf, e1t);
    e2t = ff_mul(hf, e2t);
    // the normal stress: its rate is constant, the two orders differ by the
    // rounding of the weight sums
    constexpr double wn = (B81 + B83 + B84 + B85 + B86 + B87) - (B71 + B73 + B74 + B75 + B76);
    const FF en = ff_mul(hf, ff_mulf(dn, (float)wn));
    // |y8 - yo| / |y8| with y8 = y0 + inc + (y8 - yo), in float-float (the
    // step-size control takes the 5th root of these: FP32 quotients alone
    // moved the step sizes, and after 40 steps the slips, by ~1e-9)
    auto rel = [&](FF num, int qi) {
        const FF y8 = ff_add2(ff_split_fast(y[qi]), ff_add2(inc[qi], num));
        const FF r = ff_div(num, y8);
        return r.hi < 0.f ? FF{-r.hi, -r.lo} : r;
    };
    const FF f1 = rel(es, 3), fa = rel(e1t, 1), fb = rel(e2t, 2), fc = rel(en, 0);
    auto ffmax = [](FF a, FF b) { return (a.hi > b.hi || (a.hi == b.hi && a.lo >= b.lo)) ? a : b; };
    const bool nan2 = isnan(fa.hi) || isnan(fb.hi) || isnan(fc.hi);
    const FF f2 = ffmax(ffmax(fa, fb), fc);
    e1 = ff_to_double_fast(f1);
    e2 = nan2 ? NAN : ff_to_double_fast(f2);
    if (!(isfinite(e1) && isfinite(e2))) {
        const bool fin = isfinite(y[0]) && isfinite(y[1]) && isfinite(y[2]) && isfinite(y[3]) &&
                         ff_finite(q.A1) && ff_finite(q.A2) && ff_finite(q.dsig) && isfinite(c.slipv);
        if (fin) {
            if (!isfinite(e1)) e1 = INFINITY;
            if (!isfinite(e2)) e2 = INFINITY;
        }
    }
}

// One slip-rate component of the float-float arm's update: 2 V0 e^{-psi/a}
// sinh(x) = sign(x) V0 e^{-psi/a + |x|} (1 - e^{-2|x|}), lnV0 = ln V0, psia =
// psi/a, x = tau/(a sigma) in FP64; the exponent argument reduced in FP64,
// the exponentials and the product in float-float, the result in FP64.
__device__ __forceinline__ FF ff_slip_rate(double lnV0, double psia, double x, const FF *tab)
{
    const double ax = fabs(x);
    int K;
    FF r;
    reduce_ln2(lnV0 - psia + ax, K, r);
    const FF e = ff_exp2k_tab(K, r, tab);
    const FF axf = ff_split_fast(ax);
    const FF em = ff_em(axf);
    const FF v = ff_mul(e, ff_neg(em));
    return __double2hiint(x) < 0 ? ff_neg(v) : v;   // the sign of x (its sign bit)
}

// sqrt(a) of a float-float a > 0: s = sqrtf(hi), one Newton correction
// (hi - s^2 by an exact FMA, plus lo) / 2s
__device__ __forceinline__ FF ff_sqrt(FF a)
{
    const float s = sqrtf(a.hi);
    const float d = __fadd_rn(__fmaf_rn(-s, s, a.hi), a.lo);
    return ff_norm(s, __fdiv_rn(d, __fadd_rn(s, s)));
}

// |(a, b)| of two float-float values without squaring them (no under- or
// overflow of the squares): p sqrt(1 + (q/p)^2), p = max, q = min magnitude
__device__ __forceinline__ FF ff_hypot(FF a, FF b)
{
    const FF x = a.hi < 0.f ? ff_neg(a) : a, y = b.hi < 0.f ? ff_neg(b) : b;
    const bool xl = x.hi > y.hi || (x.hi == y.hi && x.lo >= y.lo);
    const FF p = xl ? x : y, q = xl ? y : x;
    if (!(p.hi > 0.f)) return p;   // both zero (or NaN)
    const FF t = ff_div(q, p);
    return ff_mul(p, ff_sqrt(ff_add2(FF{1.f, 0.f}, ff_mul(t, t))));
}

// One Dormand-Prince attempt of one cell in FP64 (src/QDsim_gpu.py:1266-1397):
// kRecip = false evaluates the reference formula, true the reciprocal form
// (rhs_recip).  Writes the 5th-order solution to yo and returns the two
// relative errors.
template <bool kRecip = false>
__device__ __forceinline__ void dp_attempt(const Cell &c, double V0, double eta, double h, const double y[4],
                                           double yo[4], double &e1, double &e2)
{
    double s1, n1, t1, u1, s2, n2, t2, u2, s3, n3, t3, u3, s4, n4, t4, u4, s5, n5, t5, u5, s6, n6, t6, u6, s7, n7, t7,
        u7;
    const double Tno = y[0], Tt1o = y[1], Tt2o = y[2], st = y[3];
    const CellRecip kr = kRecip ? cell_recip(c, V0) : CellRecip{0.0, 0.0, 0.0, 0.0};
    auto rhs = [&](const Cell &cc, double V0_, double eta_, double a0, double a1, double a2, double a3, double &o0,
                   double &o1, double &o2, double &o3) {
        if (kRecip) rhs_recip(cc, kr, V0_, eta_, a0, a1, a2, a3, o0, o1, o2, o3);
        else ::pq3d::rk::rhs(cc, V0_, eta_, a0, a1, a2, a3, o0, o1, o2, o3);
    };
    rhs(c, V0, eta, Tno, Tt1o, Tt2o, st, s1, n1, t1, u1);
    rhs(c, V0, eta, Tno + h * B21 * n1, Tt1o + h * B21 * t1, Tt2o + h * B21 * u1, st + h * B21 * s1, s2, n2, t2, u2);
    rhs(c, V0, eta, Tno + h * (B31 * n1 + B32 * n2), Tt1o + h * (B31 * t1 + B32 * t2), Tt2o + h * (B31 * u1 + B32 * u2),
        st + h * (B31 * s1 + B32 * s2), s3, n3, t3, u3);
    rhs(c, V0, eta, Tno + h * (B41 * n1 + B42 * n2 + B43 * n3), Tt1o + h * (B41 * t1 + B42 * t2 + B43 * t3),
        Tt2o + h * (B41 * u1 + B42 * u2 + B43 * u3), st + h * (B41 * s1 + B42 * s2 + B43 * s3), s4, n4, t4, u4);
    rhs(c, V0, eta, Tno + h * (B51 * n1 + B52 * n2 + B53 * n3 + B54 * n4),
        Tt1o + h * (B51 * t1 + B52 * t2 + B53 * t3 + B54 * t4), Tt2o + h * (B51 * u1 + B52 * u2 + B53 * u3 + B54 * u4),
        st + h * (B51 * s1 + B52 * s2 + B53 * s3 + B54 * s4), s5, n5, t5, u5);
    rhs(c, V0, eta, Tno + h * (B61 * n1 + B62 * n2 + B63 * n3 + B64 * n4 + B65 * n5),
        Tt1o + h * (B61 * t1 + B62 * t2 + B63 * t3 + B64 * t4 + B65 * t5),
        Tt2o + h * (B61 * u1 + B62 * u2 + B63 * u3 + B64 * u4 + B65 * u5),
        st + h * (B61 * s1 + B62 * s2 + B63 * s3 + B64 * s4 + B65 * s5), s6, n6, t6, u6);
    yo[0] = Tno + h * (B71 * n1 + B73 * n3 + B74 * n4 + B75 * n5 + B76 * n6);
    yo[1] = Tt1o + h * (B71 * t1 + B73 * t3 + B74 * t4 + B75 * t5 + B76 * t6);
    yo[2] = Tt2o + h * (B71 * u1 + B73 * u3 + B74 * u4 + B75 * u5 + B76 * u6);
    yo[3] = st + h * (B71 * s1 + B73 * s3 + B74 * s4 + B75 * s5 + B76 * s6);
    rhs(c, V0, eta, yo[0], yo[1], yo[2], yo[3], s7, n7, t7, u7);
    const double Tn8 = Tno + h * (B81 * n1 + B83 * n3 + B84 * n4 + B85 * n5 + B86 * n6 + B87 * n7);
    const double T18 = Tt1o + h * (B81 * t1 + B83 * t3 + B84 * t4 + B85 * t5 + B86 * t6 + B87 * t7);
    const double T28 = Tt2o + h * (B81 * u1 + B83 * u3 + B84 * u4 + B85 * u5 + B86 * u6 + B87 * u7);
    const double st8 = st + h * (B81 * s1 + B83 * s3 + B84 * s4 + B85 * s5 + B86 * s6 + B87 * s7);
    e1 = fabs(fabs(st8 - yo[3]) / st8);
    const double ea = fabs(fabs(T18 - yo[1]) / T18);
    const double eb = fabs(fabs(T28 - yo[2]) / T28);
    const double ec = fabs(fabs(Tn8 - yo[0]) / Tn8);
    // max that propagates NaN, like numpy's max
    e2 = (isnan(ea) || isnan(eb) || isnan(ec)) ? NAN : fmax(fmax(ea, eb), ec);
}

// max over non-negative doubles (and NaN, which wins) through their bit
// patterns: for such values unsigned order is numeric order and a NaN's
// pattern lies above +inf's, so a NaN wins as in numpy's max
__device__ __forceinline__ unsigned long long dbits(double x) { return (unsigned long long)__double_as_longlong(fabs(x)); }

// block-wide max of such bit patterns (blockDim.x a multiple of 32, at most
// 1024; red[32] in shared memory); valid in thread 0
__device__ __forceinline__ unsigned long long block_max_bits(unsigned long long v, unsigned long long *red)
{
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long u = __shfl_xor_sync(0xffffffffu, v, o);
        v = u > v ? u : v;
    }
    __syncthreads();   // red may still be read by a previous call
    if (lane == 0) red[w] = v;
    __syncthreads();
    if (w == 0) {
        v = lane < (int)(blockDim.x >> 5) ? red[lane] : 0ull;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const unsigned long long u = __shfl_xor_sync(0xffffffffu, v, o);
            v = u > v ? u : v;
        }
    }
    return v;
}

// the same for non-negative floats (or NaN): 32-bit patterns, warp max in
// one reduction instruction
__device__ __forceinline__ unsigned block_max_bits32(float x, unsigned *red)
{
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    unsigned v = __reduce_max_sync(0xffffffffu, __float_as_uint(fabsf(x)));
    __syncthreads();
    if (lane == 0) red[w] = v;
    __syncthreads();
    if (w == 0) v = __reduce_max_sync(0xffffffffu, lane < (int)(blockDim.x >> 5) ? red[lane] : 0u);
    return v;
}

__device__ __forceinline__ double pymin(double a, double b) { return (b < a) ? b : a; }
__device__ __forceinline__ double pymax(double a, double b) { return (b > a) ? b : a; }


}  // namespace rk
}  // namespace pq3d
