// Half-space terms of the triangular-dislocation Green's function: the image
// dislocation and the free-surface correction (FSC), per (receiver, source)
// pair, for unit strike and unit dip slip (assembly) or a general Burgers
// vector (point entry points).
//
// Reference behaviour reproduced (file:line in PyQuake3D):
//   total = main + FSC + image          src/TDstressFS_C.cpp:1934-2033 (TDstressHS)
//     image = full-space solution of the triangle mirrored in z = 0; when all
//     three vertices lie on the surface its xz and yz components change sign
//   FSC = sum over the sides           src/TDstressFS_C.cpp:1785-1931 (TDstress_HarFunc)
//   one side                           src/TDstressFS_C.cpp:1489-1782 (AngSetupFSC_S)
//     beta = angle of -side with e_Z; no contribution within 1e-4 of 0 or pi;
//     frame ey1 = horizontal side direction, ey3 = -e_Z, ey2 = ey3 x ey1;
//     configuration I (beta * yA_1 >= 0): evaluate at (-y1, -y2, y3) with
//     pi - beta and (-b1, -b2, b3), then flip the 13 and 23 strain components;
//     strain = (B end) - (A end), rotated to EFCS
//   harmonic displacement of one angular dislocation: the published formulas
//   (Nikkhoo & Walter 2015, after Comninou & Dundurs 1975), as stated in
//   src/DH_greenfunction.py:313-400 (AngDisDispFSC); an image point within
//   1e-12 m of the receiver contributes zero (src/TDstressFS_C.cpp:651-654).
//
// Method (stated): the reference differentiates the harmonic displacement by
// hand (AngDisStrainFSC, src/TDstressFS_C.cpp:613-1487, ~870 lines).  Here the
// displacement is evaluated once in forward-mode dual numbers (value and the
// three partial derivatives), which yields the exact Jacobian of the same
// function; strain = its symmetric part.  The displacement is linear in the
// Burgers vector, so the nine unit-Burgers components are formed once per end
// point and combined for every slip direction.  Divisions are replaced by a few
// reciprocals (1/rb, 1/(rb + y3b), 1/(rb + z3b), 1/cos beta).
#pragma once

#include "gf_device.cuh"

namespace pq3d {
namespace gf {

// ---------------------------------------------------------------------------
// forward-mode dual number: value and d/dy1, d/dy2, d/dy3

struct Dv {
    double v, x, y, z;
};

__host__ __device__ __forceinline__ Dv dconst(double a) { return Dv{a, 0.0, 0.0, 0.0}; }
__host__ __device__ __forceinline__ Dv operator+(Dv a, Dv b) { return Dv{a.v + b.v, a.x + b.x, a.y + b.y, a.z + b.z}; }
__host__ __device__ __forceinline__ Dv operator-(Dv a, Dv b) { return Dv{a.v - b.v, a.x - b.x, a.y - b.y, a.z - b.z}; }
__host__ __device__ __forceinline__ Dv operator-(Dv a) { return Dv{-a.v, -a.x, -a.y, -a.z}; }
__host__ __device__ __forceinline__ Dv operator+(Dv a, double s) { return Dv{a.v + s, a.x, a.y, a.z}; }
__host__ __device__ __forceinline__ Dv operator+(double s, Dv a) { return a + s; }
__host__ __device__ __forceinline__ Dv operator-(Dv a, double s) { return Dv{a.v - s, a.x, a.y, a.z}; }
__host__ __device__ __forceinline__ Dv operator-(double s, Dv a) { return Dv{s - a.v, -a.x, -a.y, -a.z}; }
__host__ __device__ __forceinline__ Dv operator*(Dv a, double s) { return Dv{a.v * s, a.x * s, a.y * s, a.z * s}; }
__host__ __device__ __forceinline__ Dv operator*(double s, Dv a) { return a * s; }
__host__ __device__ __forceinline__ Dv operator*(Dv a, Dv b)
{
    return Dv{a.v * b.v, a.v * b.x + b.v * a.x, a.v * b.y + b.v * a.y, a.v * b.z + b.v * a.z};
}
__host__ __device__ __forceinline__ Dv dinv(Dv a)
{
    const double r = 1.0 / a.v, m = -r * r;
    return Dv{r, m * a.x, m * a.y, m * a.z};
}
__host__ __device__ __forceinline__ Dv dsqrt(Dv a)
{
    const double r = sqrt(a.v), h = 0.5 / r;
    return Dv{r, h * a.x, h * a.y, h * a.z};
}
__host__ __device__ __forceinline__ Dv dlog(Dv a)
{
    const double r = 1.0 / a.v;
    return Dv{log(a.v), r * a.x, r * a.y, r * a.z};
}
// atan(u / w), principal value (as the reference's atan of the quotient)
__host__ __device__ __forceinline__ Dv datan_ratio(Dv u, Dv w)
{
    const double d = 1.0 / (u.v * u.v + w.v * w.v);
    return Dv{atan(u.v / w.v), (w.v * u.x - u.v * w.x) * d, (w.v * u.y - u.v * w.y) * d, (w.v * u.z - u.v * w.z) * d};
}

// ---------------------------------------------------------------------------
// per-source side table (three sides: P1->P2, P2->P3, P3->P1)

enum FscField {
    S_VALID,                       // 1: the side contributes
    S_PAX, S_PAY, S_PAZ, S_PBZ,    // start point, end-point depth
    S_C1, S_S1,                    // ey1 = (c1, s1, 0), ey2 = (s1, -c1, 0), ey3 = (0, 0, -1)
    S_YAB0, S_YAB1, S_YAB2,        // side vector in the side frame
    S_SIN2, S_COS2, S_COT2, S_CTH2,   // configuration II: sin, cos, cot of beta, cot(beta / 2)
    S_SIN1, S_COS1, S_COT1, S_CTH1,   // configuration I: the same for pi - beta
    S_BN0, S_BN1, S_BN2,           // unit tensile (normal) Burgers vector in the side frame
    S_BS0, S_BS1, S_BS2,           // unit strike
    S_BD0, S_BD1, S_BD2,           // unit dip
    S_COUNT
};
constexpr int kFscSurface = 3 * S_COUNT;   // 1 when all three vertices have z == 0
constexpr int kFscStride = 88;             // fields per source (>= 3 * S_COUNT + 1)
constexpr int kImgStride = kSrcStride;     // image-source record: setup_source of the mirrored triangle

__host__ __device__ inline void setup_fsc(const double P1[3], const double P2[3], const double P3[3], double *f,
                                          int fstride)
{
    // triangle frame (normal, strike, dip) as TDstress_HarFunc builds it
    double n[3] = {(P2[1] - P1[1]) * (P3[2] - P1[2]) - (P2[2] - P1[2]) * (P3[1] - P1[1]),
                   (P2[2] - P1[2]) * (P3[0] - P1[0]) - (P2[0] - P1[0]) * (P3[2] - P1[2]),
                   (P2[0] - P1[0]) * (P3[1] - P1[1]) - (P2[1] - P1[1]) * (P3[0] - P1[0])};
    const double nl = sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
    if (nl != 0.0) { n[0] /= nl; n[1] /= nl; n[2] /= nl; }
    double st[3] = {-n[1], n[0], 0.0};
    const double sl = sqrt(st[0] * st[0] + st[1] * st[1]);
    if (sl == 0.0) { st[0] = 0.0; st[1] = n[2]; }
    else { st[0] /= sl; st[1] /= sl; }
    const double dp[3] = {n[1] * st[2] - n[2] * st[1], n[2] * st[0] - n[0] * st[2], n[0] * st[1] - n[1] * st[0]};
    const double *P[4] = {P1, P2, P3, P1};
    for (int sd = 0; sd < 3; ++sd) {
        const double *PA = P[sd], *PB = P[sd + 1];
        double v[S_COUNT];
        for (int i = 0; i < S_COUNT; ++i) v[i] = 0.0;
        const double sv[3] = {PB[0] - PA[0], PB[1] - PA[1], PB[2] - PA[2]};
        const double len = sqrt(sv[0] * sv[0] + sv[1] * sv[1] + sv[2] * sv[2]);
        const double beta = acos(-sv[2] / len);
        if (!(fabs(beta) < 1e-4 || fabs(kPi - beta) < 1e-4)) {
            const double hl = sqrt(sv[0] * sv[0] + sv[1] * sv[1]);
            const double c1 = sv[0] / hl, s1 = sv[1] / hl;
            // ey1 = (c1, s1, 0), ey2 = (s1, -c1, 0), ey3 = (0, 0, -1)
            v[S_VALID] = 1.0;
            v[S_PAX] = PA[0]; v[S_PAY] = PA[1]; v[S_PAZ] = PA[2]; v[S_PBZ] = PB[2];
            v[S_C1] = c1; v[S_S1] = s1;
            v[S_YAB0] = sv[0] * c1 + sv[1] * s1;
            v[S_YAB1] = sv[0] * s1 - sv[1] * c1;
            v[S_YAB2] = -sv[2];
            v[S_SIN2] = sin(beta); v[S_COS2] = cos(beta); v[S_COT2] = 1.0 / tan(beta); v[S_CTH2] = 1.0 / tan(beta / 2.0);
            const double b1 = kPi - beta;
            v[S_SIN1] = sin(b1); v[S_COS1] = cos(b1); v[S_COT1] = 1.0 / tan(b1); v[S_CTH1] = 1.0 / tan(b1 / 2.0);
            const double *B[3] = {n, st, dp};
            for (int q = 0; q < 3; ++q) {
                v[S_BN0 + 3 * q] = B[q][0] * c1 + B[q][1] * s1;
                v[S_BN0 + 3 * q + 1] = B[q][0] * s1 - B[q][1] * c1;
                v[S_BN0 + 3 * q + 2] = -B[q][2];
            }
        }
        for (int i = 0; i < S_COUNT; ++i) f[(sd * S_COUNT + i) * fstride] = v[i];
    }
    f[kFscSurface * fstride] = (P1[2] == 0.0 && P2[2] == 0.0 && P3[2] == 0.0) ? 1.0 : 0.0;
}

// ---------------------------------------------------------------------------
// harmonic displacement of one angular dislocation, nine unit-Burgers parts:
// u[k][i] = component i of the displacement for b = e_k (without the common
// factor 1 / (4 pi (1 - nu)))
struct FscTrig {
    double s, c, ct, cth;
};

__device__ __forceinline__ void fsc_unit_disp(Dv y1, Dv y2, Dv y3, const FscTrig &T, double nu, double a,
                                              Dv u[3][3])
{
    const double s = T.s, c = T.c, ct = T.ct, ic = 1.0 / c;
    const double n1 = 1.0 - 2.0 * nu, n2 = 1.0 - nu;
    const double ct2 = ct * ct;
    const Dv y3b = y3 + 2.0 * a;
    const Dv z1b = y1 * c + y3b * s;
    const Dv z3b = y3b * c - y1 * s;
    const Dv rb = dsqrt(y1 * y1 + y2 * y2 + y3b * y3b);
    const Dv irb = dinv(rb);
    const Dv irb2 = irb * irb;
    const Dv P = rb + y3b, Q = rb + z3b;
    const Dv iP = dinv(P), iQ = dinv(Q);
    const Dv h = y3b - a;
    const Dv W = rb * c + y3b;
    const Dv ar = a * irb;
    const Dv Fib = 2.0 * datan_ratio(-y2, y1 - P * T.cth);
    const Dv lP = dlog(P), lQ = dlog(Q);
    const Dv y1s = y1 * y1, y2s = y2 * y2;
    // shared products (each formed once; the expressions below scale them)
    const Dv car = c + ar, nar = nu + ar, tar = 2.0 * nu + ar, ar1 = 1.0 + ar;
    const Dv hirb = h * irb;
    const Dv rsy = rb * s - y1;
    const Dv y1P = y1 * iP, y2P = y2 * iP, y2Q = y2 * iQ, z1Q = z1b * iQ;
    const Dv G = y2 * hirb, GP = G * iP, GQ = G * iQ;        // y2 h / rb, / P, / Q
    const Dv Y1h = y1 * hirb;                                // y1 h / rb
    const Dv HP = h * iP, HQ = h * iQ;
    const Dv WQ = W * iQ;
    const Dv airb2 = a * irb2;                              // a / rb^2
    const Dv ay3 = y3b * airb2;                             // a y3b / rb^2
    const Dv aic = (a * ic) * irb;                          // a / (rb cos)
    const Dv WQcar = WQ * car;
    const Dv y2Qcar = y2Q * car;
    // b1
    u[0][0] = (-2.0 * n2 * n1 * ct2) * Fib + n1 * (y2P * ((n1 - ar) * ct - y1P * nar)) + (n1 * c * ct) * y2Qcar
              + (a * ct) * (G * irb2)
              + GP * (-n1 * ct + y1P * tar + y1 * airb2)
              + GQ * ((c * ct) * (WQ * (n1 * c - ar)) + (2.0 * n2 * c * c) * (rsy * iQ) - (c * ct) * ay3);
    u[0][1] = n1 * ((2.0 * n2 * ct2 - nu) * lP - ((2.0 * n2 * ct2 + n1) * c) * lQ)
              - n1 * (iP * (ct * (y1 * (n1 - ar)) + nu * y3b - a + y2s * (iP * nar)))
              - (n1 * ct) * (z1Q * car) - (a * ct) * (Y1h * irb2)
              + HP * (-2.0 * nu + irb * ((n1 * ct) * y1 - a) + (y2s * irb) * (iP * tar) + y2s * (airb2 * irb))
              + HQ * (c * c - irb * ((n1 * ct) * z1b + a * c) + (a * ct) * (z1b * (y3b * (irb2 * irb)))
                      - (irb * iQ) * ((c * c) * y2s - (a * ct) * (z1b * (irb * W))));
    u[0][2] = (2.0 * n2) * ((n1 * ct) * Fib + y2P * tar - c * y2Qcar)
              + G * (2.0 * nu * iP + airb2)
              + c * (GQ * (n1 - WQcar - ay3));
    // b2
    u[1][0] = n1 * ((2.0 * n2 * ct2 + nu) * lP - ((2.0 * n2 * ct2 + 1.0) * c) * lQ)
              + n1 * (iP * (-(n1 * ct) * y1 + nu * y3b - a + (a * ct) * (y1 * irb) + y1s * (iP * nar)))
              - (n1 * ct) * (iQ * (c * z1b - rsy * aic)) - (a * ct) * (Y1h * irb2)
              + HP * (2.0 * nu + irb * ((n1 * ct) * y1 + a) - (y1s * irb) * (iP * tar) - y1s * (airb2 * irb))
              + ct * (HQ * (-c * s + ic * (y1 * (ay3 * irb)) + (rsy * irb) * ((2.0 * n2 * c) - WQ * (1.0 + aic))));
    u[1][1] = (2.0 * n2 * n1 * ct2) * Fib + n1 * (y2P * (-(n1 - ar) * ct + y1P * nar))
              - (n1 * ct) * (y2Q * (1.0 + aic)) - (a * ct) * (G * irb2)
              + GP * (n1 * ct - 2.0 * nu * y1P - (a * y1) * (irb * (irb + iP)))
              + ct * (GQ * (-2.0 * n2 * c + WQ * (1.0 + aic) + ic * ay3));
    u[1][2] = (-2.0 * n2 * n1 * ct) * (lP - c * lQ) - (2.0 * n2) * (y1P * tar)
              + (2.0 * n2) * (z1Q * car) + hirb * (n1 * ct - 2.0 * nu * y1P - y1 * airb2)
              - HQ * (c * s + ct * (W * irb) * (2.0 * n2 * c - WQ)
                      + ar * (s - z1b * (y3b * irb2) - z1b * (W * irb) * iQ));
    // b3
    u[2][0] = n1 * (y2P * ar1 - c * y2Qcar) - G * (airb2 + iP)
              + c * (GQ * (WQcar + ay3));
    u[2][1] = n1 * (-s * lQ - y1P * ar1 + z1Q * car) + Y1h * (airb2 + iP)
              - HQ * (s * (c - ar) + (z1b * irb) * (1.0 + ay3)
                      - (irb * iQ) * ((c * s) * y2s - a * (z1b * (irb * W))));
    u[2][2] = (2.0 * n2) * Fib + (2.0 * n2 * s) * y2Qcar
              + s * (GQ * (1.0 + WQcar + ay3));
}

// d/dy of the harmonic displacement at one end point for NB Burgers vectors b
// (side frame), accumulated with weight sgn into J[q][i][j] = d v_i / d y_j.
// Configuration I evaluates at (-y1, -y2, y3) with (-b1, -b2, b3) and maps
// the Jacobian back (rows and columns 1, 2 change sign).  A called function,
// not inlined: the dual-number intermediates of one end point then take the
// register file alone (inlined into the pair evaluation they spilled 1.6 KB
// per thread).
template <int NB>
__device__ PQ3D_NOINLINE void fsc_endpoint(const double y[3], bool confI, const FscTrig &T, double nu,
                                                      double a, const double b[NB][3], double sgn,
                                                      double J[NB][3][3])
{
    const double yb3 = y[2] + 2.0 * a;
    if (sqrt(y[0] * y[0] + y[1] * y[1] + yb3 * yb3) < 1e-12) return;
    const double r = confI ? -1.0 : 1.0;   // y1, y2 (and b1, b2, v1, v2) map by r
    const Dv y1{r * y[0], 1.0, 0.0, 0.0}, y2{r * y[1], 0.0, 1.0, 0.0}, y3{y[2], 0.0, 0.0, 1.0};
    Dv u[3][3];
    fsc_unit_disp(y1, y2, y3, T, nu, a, u);
    const double sg[3] = {r, r, 1.0};
#pragma unroll
    for (int q = 0; q < NB; ++q) {
        const double bb[3] = {r * b[q][0], r * b[q][1], b[q][2]};
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            // v_i = sg_i * sum_k bb_k u[k][i](y'),  y'_j = sg_j y_j
            const double wi = sgn * sg[i];
            const double gx = bb[0] * u[0][i].x + bb[1] * u[1][i].x + bb[2] * u[2][i].x;
            const double gy = bb[0] * u[0][i].y + bb[1] * u[1][i].y + bb[2] * u[2][i].y;
            const double gz = bb[0] * u[0][i].z + bb[1] * u[1][i].z + bb[2] * u[2][i].z;
            J[q][i][0] += wi * sg[0] * gx;
            J[q][i][1] += wi * sg[1] * gy;
            J[q][i][2] += wi * sg[2] * gz;
        }
    }
}

// FSC strain (EFCS, xx yy zz xy xz yz) of one side at (X, Y, Z) for NB
// Burgers vectors given in the side frame, added to E[q].
template <int NB, class Fs>
__device__ __forceinline__ void fsc_side(const Fs &G, int side, double X, double Y, double Z, double nu,
                                                  const double b[NB][3], double E[NB][6])
{
    const int o = side * S_COUNT;
    if (G(o + S_VALID) == 0.0) return;
    const double c1 = G(o + S_C1), s1 = G(o + S_S1);
    const double dx = X - G(o + S_PAX), dy = Y - G(o + S_PAY), dz = Z - G(o + S_PAZ);
    const double yA[3] = {dx * c1 + dy * s1, dx * s1 - dy * c1, -dz};
    const double yB[3] = {yA[0] - G(o + S_YAB0), yA[1] - G(o + S_YAB1), yA[2] - G(o + S_YAB2)};
    const bool confI = yA[0] >= 0.0;   // beta * yA_1 >= 0 with 0 < beta < pi
    FscTrig T;
    if (confI) { T.s = G(o + S_SIN1); T.c = G(o + S_COS1); T.ct = G(o + S_COT1); T.cth = G(o + S_CTH1); }
    else { T.s = G(o + S_SIN2); T.c = G(o + S_COS2); T.ct = G(o + S_COT2); T.cth = G(o + S_CTH2); }
    double J[NB][3][3];
#pragma unroll
    for (int q = 0; q < NB; ++q)
#pragma unroll
        for (int i = 0; i < 3; ++i) J[q][i][0] = J[q][i][1] = J[q][i][2] = 0.0;
    fsc_endpoint<NB>(yB, confI, T, nu, -G(o + S_PBZ), b, 1.0, J);
    fsc_endpoint<NB>(yA, confI, T, nu, -G(o + S_PAZ), b, -1.0, J);
    const double K = 1.0 / (4.0 * kPi * (1.0 - nu));
#pragma unroll
    for (int q = 0; q < NB; ++q) {
        // local strain, then EFCS: E = A e A^T with A = [[c1, s1, 0], [s1, -c1, 0], [0, 0, -1]]
        const double e11 = K * J[q][0][0], e22 = K * J[q][1][1], e33 = K * J[q][2][2];
        const double e12 = 0.5 * K * (J[q][0][1] + J[q][1][0]);
        const double e13 = 0.5 * K * (J[q][0][2] + J[q][2][0]);
        const double e23 = 0.5 * K * (J[q][1][2] + J[q][2][1]);
        const double cc = c1 * c1, ss = s1 * s1, cs = c1 * s1;
        E[q][0] += cc * e11 + 2.0 * cs * e12 + ss * e22;
        E[q][1] += ss * e11 - 2.0 * cs * e12 + cc * e22;
        E[q][2] += e33;
        E[q][3] += cs * (e11 - e22) + (ss - cc) * e12;
        E[q][4] += -(c1 * e13 + s1 * e23);
        E[q][5] += -(s1 * e13 - c1 * e23);
    }
}

// Tractions (e1, e2, n of the receiver record R) of an EFCS strain.
__device__ __forceinline__ void tractions_efcs(const double E[6], const double *R, double two_mu, double lam,
                                                        double out[3])
{
    const double *n = R + 9;
    const double u0 = E[0] * n[0] + E[3] * n[1] + E[4] * n[2];
    const double u1 = E[3] * n[0] + E[1] * n[1] + E[5] * n[2];
    const double u2 = E[4] * n[0] + E[5] * n[1] + E[2] * n[2];
    const double tr = E[0] + E[1] + E[2];
    out[0] = two_mu * (R[3] * u0 + R[4] * u1 + R[5] * u2);
    out[1] = two_mu * (R[6] * u0 + R[7] * u1 + R[8] * u2);
    out[2] = two_mu * (n[0] * u0 + n[1] * u1 + n[2] * u2) + lam * tr;
}

// Half-space tractions of one pair (unit strike ts, unit dip td): main
// dislocation F, image Fi (mirrored triangle), side table G.
template <class Src, class Fs>
__device__ __forceinline__ void pair_tractions_hs(const Src &F, const Src &Fi, const Fs &G, const double *R,
                                                  double nu, double k, double two_mu, double lam, double ts[3],
                                                  double td[3])
{
    pair_tractions(F, R, nu, k, two_mu, lam, ts, td);
    double is[3], id[3];
    if (G(kFscSurface) != 0.0) {
        // surface triangle: the image equals the main strain with xz, yz
        // negated, i.e. the main strain seen through receiver axes reflected in z
        double Rr[kRecvStride];
#pragma unroll
        for (int q = 0; q < kRecvStride; ++q) Rr[q] = R[q];
        Rr[5] = -R[5]; Rr[8] = -R[8]; Rr[11] = -R[11];
        pair_tractions(F, Rr, nu, k, two_mu, lam, is, id);
    } else {
        pair_tractions(Fi, R, nu, k, two_mu, lam, is, id);
    }
    double E[2][6];
#pragma unroll
    for (int q = 0; q < 2; ++q)
#pragma unroll
        for (int i = 0; i < 6; ++i) E[q][i] = 0.0;
    for (int sd = 0; sd < 3; ++sd) {
        const int o = sd * S_COUNT;
        const double b[2][3] = {{G(o + S_BS0), G(o + S_BS1), G(o + S_BS2)}, {G(o + S_BD0), G(o + S_BD1), G(o + S_BD2)}};
        fsc_side<2>(G, sd, R[0], R[1], R[2], nu, b, E);
    }
    double fs[3], fd[3];
    tractions_efcs(E[0], R, two_mu, lam, fs);
    tractions_efcs(E[1], R, two_mu, lam, fd);
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        ts[c] += fs[c] + is[c];
        td[c] += fd[c] + id[c];
    }
}

// Half-space strain (EFCS) at a point for the Burgers vector (bx, by, bz) =
// (tensile, strike, dip): the point entry points' counterpart.
template <class Src, class Fs>
__device__ __forceinline__ void point_strain_hs(const Src &F, const Src &Fi, const Fs &G, double X, double Y,
                                                double Z, double bx, double by, double bz, double nu, double k,
                                                double e[6])
{
    double x, y, z, E[6];
    tdcs_point(F, X, Y, Z, x, y, z);
    tdcs_strain_general(F, x, y, z, bx, by, bz, nu, k, E);
    tdcs_to_efcs(F, E, e);
    double ei[6];
    tdcs_point(Fi, X, Y, Z, x, y, z);
    tdcs_strain_general(Fi, x, y, z, bx, by, bz, nu, k, E);
    tdcs_to_efcs(Fi, E, ei);
    if (G(kFscSurface) != 0.0) { ei[4] = -ei[4]; ei[5] = -ei[5]; }
    double Ef[1][6] = {{0.0, 0.0, 0.0, 0.0, 0.0, 0.0}};
    for (int sd = 0; sd < 3; ++sd) {
        const int o = sd * S_COUNT;
        double b[1][3];
        for (int c = 0; c < 3; ++c)
            b[0][c] = bx * G(o + S_BN0 + c) + by * G(o + S_BS0 + c) + bz * G(o + S_BD0 + c);
        fsc_side<1>(G, sd, X, Y, Z, nu, b, Ef);
    }
    for (int i = 0; i < 6; ++i) e[i] += Ef[0][i] + ei[i];
}

}  // namespace gf
}  // namespace pq3d
