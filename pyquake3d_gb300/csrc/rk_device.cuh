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
    double inv_a, inv_b, bdc;   // 1/a, 1/b, b/dc (used by the mixed-precision right-hand side)
    double P, dPdt;             // pore pressure (Pa) and its rate (Pa/s); 0 without dilatancy
    float L1, L2, dsf;          // mixed right-hand side: -AdotV1 + shear, -AdotV2 + shear, dsig - dPdt
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

// e^x for the mixed-precision right-hand side: x = (n + f) / log2(e) with n
// integer and |f| <= 1/2 (Cody-Waite range reduction); 2^f from the FP32
// exp2f, 2^n exact.  Relative error ~2.5e-7 (that of exp2f), 6 FP64
// operations instead of the ~20 of an FP64 exp.  The argument is clipped to
// +-700 like the reference's safe_exp.
__device__ __forceinline__ double fexp(double x)
{
    x = fmin(fmax(x, -700.0), 700.0);
    const double t = x * 1.4426950408889634;
    const double n = rint(t);
    const float f = (float)(t - n);
    const double scale = __longlong_as_double((long long)((int)n + 1023) << 52);
    return (double)exp2f(f) * scale;
}

// 1/d for the mixed right-hand side: the FP32 reciprocal refined by one
// Newton-Raphson step r <- r (2 - d r) in FP64 (the relative error squares:
// ~4e-15), two FMAs instead of a full FP64 division.  d > 0, in FP32 range.
__device__ __forceinline__ double rcp_nr(double d)
{
    const double r = (double)__frcp_rn((float)d);
    return fma(r, fma(-d, r, 1.0), r);
}

// e^x as FP32: the argument reduced in FP64 as in fexp, 2^f from exp2f and
// the exact power-of-two scaling in FP32 (ldexpf: underflow to 0 where the
// term is negligible).
__device__ __forceinline__ float fexpf(double x)
{
    x = fmin(fmax(x, -700.0), 700.0);
    const double t = x * 1.4426950408889634;
    const double n = rint(t);
    return ldexpf(exp2f((float)(t - n)), (int)fmax(fmin(n, 300.0), -300.0));
}

// Mixed-precision right-hand side (batched mixed modes).  Same equations as
// rhs().  What needs FP64 stays FP64: the state, the exponent arguments
// tau/(a sigma) and -psi/a (large and nearly cancelling: they are summed in
// FP64 before the exponential) and everything downstream of the right-hand
// side (stage sums, increments, error norm).  The factors e^{-psi/a} cosh(x),
// e^{-psi/a} sinh(x) are formed as (e^{x - psi/a} +- e^{-x - psi/a}) / 2 with
// fexpf, and the algebra after the exponentials (slip-rate derivatives,
// aging law, radiation-damping quotient; relative error ~1e-7, the level of
// the product's) runs in FP32 -- GB300's FP64 rate is 1/64 of FP32.
// Cell-constant loads (-AdotV + shear, sigma rate - P rate) come in as FP32.
__device__ __forceinline__ void rhs_mixed_f(const Cell &c, double V0, double eta, double Tno, double Tt1o,
                                            double Tt2o, double state, float &dstate, float &dtau1, float &dtau2)
{
    const double Tn = Tno * 1e6 - c.P, T1 = Tt1o * 1e6, T2 = Tt2o * 1e6;
    const double inv_aTn = rcp_nr(c.a * Tn);
    const double x1 = clip700(T1 * inv_aTn), x2 = clip700(T2 * inv_aTn);
    const double sp = clip700(-state * c.inv_a);
    const float e1p = fexpf(sp + x1), e1m = fexpf(sp - x1), e2p = fexpf(sp + x2), e2m = fexpf(sp - x2);
    const float ed = fexpf((c.f0 - state) * c.inv_b);
    const float V0f = (float)V0, iaT = (float)inv_aTn, inv_a = (float)c.inv_a, etaf = (float)eta;
    const float inv_Tn = (float)(c.a * inv_aTn);
    const float dV1dtau = V0f * iaT * (e1p + e1m);
    const float dV2dtau = V0f * iaT * (e2p + e2m);
    const float dV1dsigma = -dV1dtau * (float)T1 * inv_Tn;
    const float dV2dsigma = -dV2dtau * (float)T2 * inv_Tn;
    const float dV1dstate = -V0f * inv_a * (e1p - e1m);
    const float dV2dstate = -V0f * inv_a * (e2p - e2m);
    const float ds_dt = (float)c.bdc * (V0f * ed - (float)c.slipv);
    const float den1 = 1.0f + etaf * dV1dtau, den2 = 1.0f + etaf * dV2dtau;
    const float inv12 = 1.0f / (den1 * den2);
    const float t1 = (c.L1 - etaf * (dV1dsigma * c.dsf + dV1dstate * ds_dt)) * (den2 * inv12);
    const float t2 = (c.L2 - etaf * (dV2dsigma * c.dsf + dV2dstate * ds_dt)) * (den1 * inv12);
    dstate = ds_dt;
    dtau1 = t1 * 1e-6f;
    dtau2 = t2 * 1e-6f;
}

__device__ __forceinline__ void rhs_mixed(const Cell &c, double V0, double eta, double Tno, double Tt1o, double Tt2o,
                                          double state, double &dstate, double &dsig, double &dtau1, double &dtau2)
{
    float ds, t1, t2;
    rhs_mixed_f(c, V0, eta, Tno, Tt1o, Tt2o, state, ds, t1, t2);
    dstate = ds;
    dsig = c.dsig * 1e-6;
    dtau1 = t1;
    dtau2 = t2;
}

template <bool kMixed>
__device__ __forceinline__ void rhs_sel(const Cell &c, double V0, double eta, double Tno, double Tt1o, double Tt2o,
                                        double state, double &dstate, double &dsig, double &dtau1, double &dtau2)
{
    if (kMixed) rhs_mixed(c, V0, eta, Tno, Tt1o, Tt2o, state, dstate, dsig, dtau1, dtau2);
    else rhs(c, V0, eta, Tno, Tt1o, Tt2o, state, dstate, dsig, dtau1, dtau2);
}

// One Dormand-Prince attempt of one cell; y = (Tno, Tt1o, Tt2o, state).
// Writes the 5th-order solution to yo and returns the two relative errors.
// Mixed attempt: the stage derivatives come from rhs_mixed_f as FP32 and
// their weighted sums are formed in FP32 (they carry the derivatives' ~1e-7
// relative error already); each stage state is y + h * sum with one FP64
// multiply-add, and the 5th-minus-4th-order difference is summed directly
// (h * sum (b_i - b*_i) k_i) instead of subtracting two FP64 states.  The
// normal-stress rate is constant over the step.
__device__ __forceinline__ void dp_attempt_mixed(const Cell &c, double V0, double eta, double h, const double y[4],
                                                 double yo[4], double &e1, double &e2)
{
    float s[7], t[7], u[7];
    const double Tno = y[0], Tt1o = y[1], Tt2o = y[2], st = y[3];
    const double dn = c.dsig * 1e-6;   // d(Tno)/dt, MPa/s
    const float A[6][6] = {{(float)B21, 0, 0, 0, 0, 0},
                           {(float)B31, (float)B32, 0, 0, 0, 0},
                           {(float)B41, (float)B42, (float)B43, 0, 0, 0},
                           {(float)B51, (float)B52, (float)B53, (float)B54, 0, 0},
                           {(float)B61, (float)B62, (float)B63, (float)B64, (float)B65, 0},
                           {(float)B71, 0.f, (float)B73, (float)B74, (float)B75, (float)B76}};
    rhs_mixed_f(c, V0, eta, Tno, Tt1o, Tt2o, st, s[0], t[0], u[0]);
#pragma unroll
    for (int j = 0; j < 6; ++j) {
        float ds = 0.f, dt1 = 0.f, dt2 = 0.f;
#pragma unroll
        for (int l = 0; l <= j; ++l) {
            ds = fmaf(A[j][l], s[l], ds);
            dt1 = fmaf(A[j][l], t[l], dt1);
            dt2 = fmaf(A[j][l], u[l], dt2);
        }
        const double wsum[6] = {B21, B31 + B32, B41 + B42 + B43, B51 + B52 + B53 + B54, B61 + B62 + B63 + B64 + B65,
                                B71 + B73 + B74 + B75 + B76};
        const double Tn_j = Tno + h * (wsum[j] * dn);   // the normal-stress rate is constant
        const double T1_j = Tt1o + h * (double)dt1, T2_j = Tt2o + h * (double)dt2, st_j = st + h * (double)ds;
        if (j == 5) { yo[0] = Tn_j; yo[1] = T1_j; yo[2] = T2_j; yo[3] = st_j; }
        rhs_mixed_f(c, V0, eta, Tn_j, T1_j, T2_j, st_j, s[j + 1], t[j + 1], u[j + 1]);
    }
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
    const double wn = (B81 + B83 + B84 + B85 + B86 + B87) - (B71 + B73 + B74 + B75 + B76);
    const double st8 = yo[3] + h * (double)es;
    const double T18 = yo[1] + h * (double)e1t, T28 = yo[2] + h * (double)e2t, Tn8 = yo[0] + h * (wn * dn);
    e1 = fabs(fabs(h * (double)es) / st8);
    const double ea = fabs(fabs(h * (double)e1t) / T18);
    const double eb = fabs(fabs(h * (double)e2t) / T28);
    const double ec = fabs(fabs(h * (wn * dn)) / Tn8);
    e2 = (isnan(ea) || isnan(eb) || isnan(ec)) ? NAN : fmax(fmax(ea, eb), ec);
}

template <bool kMixed = false>
__device__ __forceinline__ void dp_attempt(const Cell &c, double V0, double eta, double h, const double y[4],
                                           double yo[4], double &e1, double &e2)
{
    if (kMixed) {
        dp_attempt_mixed(c, V0, eta, h, y, yo, e1, e2);
        return;
    }
    double s1, n1, t1, u1, s2, n2, t2, u2, s3, n3, t3, u3, s4, n4, t4, u4, s5, n5, t5, u5, s6, n6, t6, u6, s7, n7, t7,
        u7;
    const double Tno = y[0], Tt1o = y[1], Tt2o = y[2], st = y[3];
    rhs_sel<kMixed>(c, V0, eta, Tno, Tt1o, Tt2o, st, s1, n1, t1, u1);
    rhs_sel<kMixed>(c, V0, eta, Tno + h * B21 * n1, Tt1o + h * B21 * t1, Tt2o + h * B21 * u1, st + h * B21 * s1, s2, n2, t2, u2);
    rhs_sel<kMixed>(c, V0, eta, Tno + h * (B31 * n1 + B32 * n2), Tt1o + h * (B31 * t1 + B32 * t2), Tt2o + h * (B31 * u1 + B32 * u2),
        st + h * (B31 * s1 + B32 * s2), s3, n3, t3, u3);
    rhs_sel<kMixed>(c, V0, eta, Tno + h * (B41 * n1 + B42 * n2 + B43 * n3), Tt1o + h * (B41 * t1 + B42 * t2 + B43 * t3),
        Tt2o + h * (B41 * u1 + B42 * u2 + B43 * u3), st + h * (B41 * s1 + B42 * s2 + B43 * s3), s4, n4, t4, u4);
    rhs_sel<kMixed>(c, V0, eta, Tno + h * (B51 * n1 + B52 * n2 + B53 * n3 + B54 * n4),
        Tt1o + h * (B51 * t1 + B52 * t2 + B53 * t3 + B54 * t4), Tt2o + h * (B51 * u1 + B52 * u2 + B53 * u3 + B54 * u4),
        st + h * (B51 * s1 + B52 * s2 + B53 * s3 + B54 * s4), s5, n5, t5, u5);
    rhs_sel<kMixed>(c, V0, eta, Tno + h * (B61 * n1 + B62 * n2 + B63 * n3 + B64 * n4 + B65 * n5),
        Tt1o + h * (B61 * t1 + B62 * t2 + B63 * t3 + B64 * t4 + B65 * t5),
        Tt2o + h * (B61 * u1 + B62 * u2 + B63 * u3 + B64 * u4 + B65 * u5),
        st + h * (B61 * s1 + B62 * s2 + B63 * s3 + B64 * s4 + B65 * s5), s6, n6, t6, u6);
    yo[0] = Tno + h * (B71 * n1 + B73 * n3 + B74 * n4 + B75 * n5 + B76 * n6);
    yo[1] = Tt1o + h * (B71 * t1 + B73 * t3 + B74 * t4 + B75 * t5 + B76 * t6);
    yo[2] = Tt2o + h * (B71 * u1 + B73 * u3 + B74 * u4 + B75 * u5 + B76 * u6);
    yo[3] = st + h * (B71 * s1 + B73 * s3 + B74 * s4 + B75 * s5 + B76 * s6);
    rhs_sel<kMixed>(c, V0, eta, yo[0], yo[1], yo[2], yo[3], s7, n7, t7, u7);
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

// max over non-negative doubles (and NaN, which wins) through their bit patterns
__device__ __forceinline__ unsigned long long dbits(double x) { return (unsigned long long)__double_as_longlong(fabs(x)); }

__device__ __forceinline__ double block_max(double v, double *red)
{
    // NaN-propagating max across the block
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const double u = __shfl_xor_sync(0xffffffffu, v, o);
        v = (isnan(v) || isnan(u)) ? NAN : fmax(v, u);
    }
    __syncthreads();
    if (lane == 0) red[w] = v;
    __syncthreads();
    double m = 0.0;
    const int nw = blockDim.x >> 5;
    for (int q = 0; q < nw; ++q) m = (isnan(m) || isnan(red[q])) ? NAN : fmax(m, red[q]);
    return m;
}

__device__ __forceinline__ double pymin(double a, double b) { return (b < a) ? b : a; }
__device__ __forceinline__ double pymax(double a, double b) { return (b > a) ? b : a; }


}  // namespace rk
}  // namespace pq3d
