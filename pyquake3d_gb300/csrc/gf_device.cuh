// Device math of the triangular-dislocation Green's function (Nikkhoo &
// Walter 2015, full space), written for one (receiver, source) pair per
// thread.
//
// Reference behaviour reproduced (file:line in PyQuake3D):
//   angular-dislocation strain   src/TDstressFS_C.cpp:51-121
//   configuration test           src/TDstressFS_C.cpp:125-166
//   per-side rotation            src/TDstressFS_C.cpp:185-256
//   full-space entry point       src/TDstressFS_C.cpp:274-521
//   traction projection          src/QDsim_gpu.py:1400-1417
//   receiver frames              src/readmsh.py:75-134
//
// Formulation differences from the reference (same mathematics):
//   * each angular dislocation needs 1/r, 1/(r-z) and 1/W (W = zeta - r and
//     r - zeta = -W), so one square root and two reciprocals replace the ~30
//     divisions of the reference expression;
//   * the strain is linear in the Burgers vector, so the by- and bz-parts of
//     each angular dislocation are formed once and combined for unit strike
//     and unit dip slip (the reference evaluates the whole pair twice);
//   * the back-rotation of each angular dislocation's strain is done in
//     harmonic form (tdcs_strain_sd2k): rotation invariants summed, the
//     other parts turned by e^{-i th}, e^{-2i th}, e^{-3i th} and summed, strike
//     and dip read from the sums; the factor 1/(8 pi (1 - nu)) common to
//     every term is applied with the traction constants;
//   * rotation to the receiver frame, Hooke's law and the traction projection
//     are one contraction: with the receiver axes rotated into the source
//     system, t_c = 2 mu e_c^T E n + lambda tr(E) delta_{c,n} (tr and the
//     frame's orthonormality are rotation invariant).
//   * receivers on a side line in the triangle plane (mode 0) give zero, as
//     the C++ does; horizontal sources use e_Y*n_z as strike (published
//     algorithm; the reference C++ returns NaN there).
#pragma once

#include <math.h>

#ifndef __CUDACC__
// Host compilation (operation counting in oracle/count_gf_flops.cpp).
#include <cmath>
#define __host__
#define __device__
#define __forceinline__ inline
#define PQ3D_NOINLINE __attribute__((noinline))
#else
#define PQ3D_NOINLINE __noinline__
#endif

namespace pq3d {
namespace gf {

constexpr double kPi = 3.141592653589793;

// Per-source record (42 values, stored with stride kSrcStride).
enum SrcField {
    F_P2X, F_P2Y, F_P2Z,          // origin (vertex 2)
    F_NX, F_NY, F_NZ,             // triangle normal
    F_SX, F_SY, F_SZ,             // strike axis
    F_DX, F_DY, F_DZ,             // dip axis
    F_P1Y, F_P1Z, F_P3Y, F_P3Z,   // vertices 1, 3 in the triangle system (y, z)
    F_DEN,                        // barycentric denominator of the mode test
    F_E13Y, F_E13Z, F_E12Y, F_E12Z, F_E23Y, F_E23Z,   // unit side vectors (y, z)
    F_CA, F_SA, F_CB, F_SB, F_CC, F_SC,               // cos, sin of (angle - pi) per vertex
    // double angle (sz^2 - sy^2, 2 sy sz) of each vertex's side vector (sy,
    // sz) for the back-rotation (sign-free, so the same for both modes)
    F_C2A, F_S2A, F_C2B, F_S2B, F_C2C, F_S2C,
    // triple angle (Re, Im of (sz + i sy)^3) of each vertex's side vector as
    // stored (odd in the sign: negated with (sy, sz) for the other mode)
    F_C3A, F_S3A, F_C3B, F_S3B, F_C3C, F_S3C,
    F_IDEN,                       // 1 / F_DEN
    F_COUNT
};
constexpr int kSrcStride = 42;
constexpr int kRecvStride = 12;   // x, y, z, e1[3], e2[3], n[3]

__host__ __device__ inline void unit3(double v[3])
{
    const double l = sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    v[0] /= l; v[1] /= l; v[2] /= l;
}

// (sz + i sy)^3 of a side vector (sy, sz): the double angle times the angle.
__host__ __device__ inline double cube_re(double sy, double sz)
{
    return (sz * sz - sy * sy) * sz - 2.0 * (sy * sz) * sy;
}
__host__ __device__ inline double cube_im(double sy, double sz)
{
    return 2.0 * (sy * sz) * sz + (sz * sz - sy * sy) * sy;
}

// Source setup (src/TDstressFS_C.cpp:291-396).  f[i * fstride] receives field i.
__host__ __device__ inline void setup_source(const double P1[3], const double P2[3], const double P3[3],
                                             double *f, int fstride)
{
    double n[3] = {(P2[1] - P1[1]) * (P3[2] - P1[2]) - (P2[2] - P1[2]) * (P3[1] - P1[1]),
                   (P2[2] - P1[2]) * (P3[0] - P1[0]) - (P2[0] - P1[0]) * (P3[2] - P1[2]),
                   (P2[0] - P1[0]) * (P3[1] - P1[1]) - (P2[1] - P1[1]) * (P3[0] - P1[0])};
    unit3(n);
    double s[3] = {-n[1], n[0], 0.0};             // e_Z x n
    double ls = sqrt(s[0] * s[0] + s[1] * s[1]);
    if (ls == 0.0) { s[0] = 0.0; s[1] = n[2]; ls = fabs(n[2]); }
    s[0] /= ls; s[1] /= ls;
    const double d[3] = {n[1] * s[2] - n[2] * s[1], n[2] * s[0] - n[0] * s[2], n[0] * s[1] - n[1] * s[0]};
    const double q1[3] = {P1[0] - P2[0], P1[1] - P2[1], P1[2] - P2[2]};
    const double q3[3] = {P3[0] - P2[0], P3[1] - P2[1], P3[2] - P2[2]};
    double p1[3] = {n[0] * q1[0] + n[1] * q1[1] + n[2] * q1[2],
                    s[0] * q1[0] + s[1] * q1[1] + s[2] * q1[2],
                    d[0] * q1[0] + d[1] * q1[1] + d[2] * q1[2]};
    double p3[3] = {n[0] * q3[0] + n[1] * q3[1] + n[2] * q3[2],
                    s[0] * q3[0] + s[1] * q3[1] + s[2] * q3[2],
                    d[0] * q3[0] + d[1] * q3[1] + d[2] * q3[2]};
    double e12[3] = {-p1[0], -p1[1], -p1[2]};
    double e13[3] = {p3[0] - p1[0], p3[1] - p1[1], p3[2] - p1[2]};
    double e23[3] = {p3[0], p3[1], p3[2]};
    unit3(e12); unit3(e13); unit3(e23);
    const double A = acos(e12[0] * e13[0] + e12[1] * e13[1] + e12[2] * e13[2]);
    const double B = acos(-e12[0] * e23[0] - e12[1] * e23[1] - e12[2] * e23[2]);
    const double C = acos(e23[0] * e13[0] + e23[1] * e13[1] + e23[2] * e13[2]);
    const double Am = -kPi + A, Bm = -kPi + B, Cm = -kPi + C;
    const double vals[F_COUNT] = {
        P2[0], P2[1], P2[2], n[0], n[1], n[2], s[0], s[1], s[2], d[0], d[1], d[2],
        p1[1], p1[2], p3[1], p3[2],
        -p3[2] * (p1[1] - p3[1]) + p3[1] * (p1[2] - p3[2]),
        e13[1], e13[2], e12[1], e12[2], e23[1], e23[2],
        cos(Am), sin(Am), cos(Bm), sin(Bm), cos(Cm), sin(Cm),
        e13[2] * e13[2] - e13[1] * e13[1], 2.0 * (e13[1] * e13[2]),
        e12[2] * e12[2] - e12[1] * e12[1], 2.0 * (e12[1] * e12[2]),
        e23[2] * e23[2] - e23[1] * e23[1], 2.0 * (e23[1] * e23[2]),
        cube_re(e13[1], e13[2]), cube_im(e13[1], e13[2]),
        cube_re(e12[1], e12[2]), cube_im(e12[1], e12[2]),
        cube_re(e23[1], e23[2]), cube_im(e23[1], e23[2]),
        1.0 / (-p3[2] * (p1[1] - p3[1]) + p3[1] * (p1[2] - p3[2]))};
    for (int i = 0; i < F_COUNT; ++i) f[i * fstride] = vals[i];
}

// Receiver record (src/readmsh.py:75-134, node-order flag False).
__host__ __device__ inline void setup_receiver(const double a[3], const double b[3], const double c[3], double *r)
{
    for (int k = 0; k < 3; ++k) r[k] = ((a[k] + b[k]) + c[k]) / 3.0;
    const double ba[3] = {b[0] - a[0], b[1] - a[1], b[2] - a[2]};
    const double ca[3] = {c[0] - a[0], c[1] - a[1], c[2] - a[2]};
    double n[3] = {ba[1] * ca[2] - ba[2] * ca[1], ba[2] * ca[0] - ba[0] * ca[2], ba[0] * ca[1] - ba[1] * ca[0]};
    unit3(n);
    double e1[3];
    if (fabs(n[2]) < 1) {
        e1[0] = n[1]; e1[1] = -n[0]; e1[2] = 0.0;
        const double l = sqrt(e1[0] * e1[0] + e1[1] * e1[1]);
        e1[0] /= l; e1[1] /= l;
    } else {
        e1[0] = 1.0; e1[1] = 0.0; e1[2] = 0.0;
    }
    const double e2[3] = {n[1] * e1[2] - n[2] * e1[1], n[2] * e1[0] - n[0] * e1[2], n[0] * e1[1] - n[1] * e1[0]};
    r[3] = e1[0]; r[4] = e1[1]; r[5] = e1[2];
    r[6] = e2[0]; r[7] = e2[1]; r[8] = e2[2];
    r[9] = n[0];  r[10] = n[1]; r[11] = n[2];
}

// Configuration test: +1, -1, or 0 (side line in the plane).
template <class T>
__device__ __forceinline__ int tri_mode(T x, T y, T z, T p1y, T p1z, T p3y, T p3z, T den)
{
    const T a = ((y - p3y) * (0.0 - p3z) - (0.0 - p3y) * (z - p3z)) / den;
    const T b = ((p1y - p3y) * (z - p3z) - (y - p3y) * (p1z - p3z)) / den;
    const T c = 1.0 - a - b;
    int m = 1;
    if (a <= 0 && b > c && c > a) m = -1;
    else if (b <= 0 && c > a && a > b) m = -1;
    else if (c <= 0 && a > b && b > c) m = -1;
    else if (a == 0 && b >= 0 && c >= 0) m = 0;
    else if (a >= 0 && b == 0 && c >= 0) m = 0;
    else if (a >= 0 && b >= 0 && c == 0) m = 0;
    if (m == 0 && x != 0) m = 1;
    return m;
}

#ifdef __CUDACC__
// v truncated to FP32 by the bit layout for the configuration test's guard
// (relative error < 2^-23): |v| < 2^-126 gives 0, |v| >= 2^128, infinities
// and NaN give NaN (every comparison with it fails, so the guard falls back).
__device__ __forceinline__ float guard_f32(double v)
{
    const unsigned hw = (unsigned)__double2hiint(v), lw = (unsigned)__double2loint(v);
    const int e = (int)((hw >> 20) & 0x7ffu);
    if (e < 1023 - 126) return 0.f;
    if (e > 1023 + 127) return __uint_as_float(0x7fc00000u);
    return __uint_as_float((hw & 0x80000000u) | ((unsigned)(e - 896) << 23) | ((hw & 0xfffffu) << 3) | (lw >> 29));
}

// tri_mode with the barycentric coordinates from the reciprocal of the
// denominator and the decisions taken in FP32: where every coordinate and
// every difference of two is larger than 1e-5 of their scale, the FP64
// coordinates (a few ulps from tri_mode's quotients) and their FP32
// truncations order exactly as tri_mode's, and no coordinate is zero (so the
// result is +1 or -1); closer cases -- receivers near a side line or a
// boundary of the wedges -- are decided by tri_mode itself.  Keeps the two
// divisions and the FP64 compares off the FP64 pipe for almost every pair.
__device__ __forceinline__ int tri_mode_fast(double x, double y, double z, double p1y, double p1z, double p3y,
                                             double p3z, double den, double iden)
{
    const double ya = y - p3y, za = z - p3z;
    const double a = (ya * (0.0 - p3z) - (0.0 - p3y) * za) * iden;
    const double b = ((p1y - p3y) * za - ya * (p1z - p3z)) * iden;
    const double c = 1.0 - a - b;
    const float af = guard_f32(a), bf = guard_f32(b), cf = guard_f32(c);
    const float t = 1e-5f * fmaxf(1.f, fmaxf(fabsf(af), fabsf(bf)));
    const bool sep = fabsf(af) > t && fabsf(bf) > t && fabsf(cf) > t && fabsf(af - bf) > t &&
                     fabsf(bf - cf) > t && fabsf(cf - af) > t;
    if (!sep) return tri_mode<double>(x, y, z, p1y, p1z, p3y, p3z, den);
    if ((af < 0.f && bf > cf && cf > af) || (bf < 0.f && cf > af && af > bf) || (cf < 0.f && af > bf && bf > cf))
        return -1;
    return 1;
}
#endif
template <class T>
__host__ __device__ inline int tri_mode_fast(T x, T y, T z, T p1y, T p1z, T p3y, T p3z, T den, T)
{
    return tri_mode<T>(x, y, z, p1y, p1z, p3y, p3z, den);
}

#ifdef __CUDACC__
__device__ __forceinline__ bool isfinite_t(double v) { return isfinite(v); }
// v != 0 and finite, by integer tests of the bit pattern (GB300 runs FP64
// compares on its FP64 pipe, which the pair evaluation keeps busy)
__device__ __forceinline__ bool nonzero_finite_t(double v)
{
    const unsigned hw = (unsigned)__double2hiint(v), lw = (unsigned)__double2loint(v);
    return (hw & 0x7ff00000u) != 0x7ff00000u && ((hw & 0x7fffffffu) | lw) != 0u;
}
#else
inline bool isfinite_t(double v) { return std::isfinite(v); }
#ifndef PQ3D_OPCOUNT
inline bool isfinite_t(long double v) { return std::isfinite(v); }
#endif
#endif
template <class T>
__host__ __device__ inline bool nonzero_finite_t(T v) { return v != 0.0 && isfinite_t(v); }

// FP64 -> FP32, round to nearest even, by the bit layout: integer operations
// only where the result is a normal float; values that round to a subnormal
// float or to zero, overflow, infinities and NaN take the conversion
// instruction (a branch that the operator's entries do not take).
#ifdef __CUDACC__
__device__ __forceinline__ float d2f_rn_bits(double x)
{
    const unsigned hw = (unsigned)__double2hiint(x), lw = (unsigned)__double2loint(x);
    const int e = (int)((hw >> 20) & 0x7ffu);
    if (e < 1023 - 126 || e > 1023 + 127) return (float)x;
    unsigned f = (hw & 0x80000000u) | ((unsigned)(e - 1023 + 127) << 23) | ((hw & 0xfffffu) << 3) | (lw >> 29);
    const unsigned rem = lw & 0x1fffffffu;   // the 29 bits below the float's last
    // above half an ulp, or exactly half with an odd last bit: one ulp up (a
    // carry into the exponent is the next binade; past the largest float, inf)
    f += (rem > 0x10000000u || (rem == 0x10000000u && (f & 1u))) ? 1u : 0u;
    return __uint_as_float(f);
}
#endif

// Shared geometric terms of one angular dislocation at (x, y, z) of its own
// frame, opening angle with cos/sin (ca, sa).
template <class T>
struct AdGeom {
    T x, y, z, ca, sa;
    T eta, ycz, x2, y2, z2;
    T ir, ir3, iW2;
    T i_Wr, i_W2r2, i_Wr3, i_rz, i_r2z2, i_r3z, i_W2r;
    T C, S, gx, gy, gz, fx, fy, fz;
};

// qg scales the g-terms: 1/(4 pi) gives the strain's own terms; 2 (1 - nu)
// gives them divided by k = 1/(8 pi (1 - nu)), for a strain with k taken out.
template <class T>
__device__ __forceinline__ void ad_geom(T x, T y, T z, T ca, T sa, double nu, AdGeom<T> &g,
                                        double qg = 1.0 / (4.0 * kPi))
{
    g.x = x; g.y = y; g.z = z; g.ca = ca; g.sa = sa;
    g.eta = y * ca - z * sa;
    const T zeta = y * sa + z * ca;
    g.ycz = y * ca + z * sa;
    g.x2 = x * x; g.y2 = y * y; g.z2 = z * z;
    const T r2 = g.x2 + g.y2 + g.z2;
    const T r = sqrt(r2);
    const T rz = r - z, W = zeta - r;
    // the three reciprocals from one division (a division is ~9 FP64-pipe
    // instructions, a product one); the plain quotients where the product is
    // zero or not finite (singular lines of the dislocation)
    // 1/(r (r - z)) = W/p and 1/(W r) = (r - z)/p
    T ir, iW;
    const T rrz = r * rz, p = rrz * W;
    if (nonzero_finite_t(p)) {
        const T ip = 1.0 / p;
        g.i_rz = ip * W;
        g.i_Wr = ip * rz;
        iW = ip * rrz;
        ir = g.i_rz * rz;
    } else {
        ir = 1.0 / r;
        iW = 1.0 / W;
        g.i_rz = ir * (1.0 / rz);
        g.i_Wr = iW * ir;
    }
    const T ir2 = ir * ir;
    g.ir = ir;
    g.ir3 = ir2 * ir;
    g.iW2 = iW * iW;
    g.i_W2r2 = g.i_Wr * g.i_Wr;
    g.i_Wr3 = g.i_Wr * ir2;
    g.i_r2z2 = g.i_rz * g.i_rz;
    g.i_r3z = g.i_rz * ir2;
    g.i_W2r = iW * g.i_Wr;
    g.C = (r * ca - z) * g.i_Wr;
    g.S = (r * sa - y) * g.i_Wr;
    // with 1/(r - zeta) = -1/W:
    const double q = qg;
    g.gx = -q * (g.eta * g.i_Wr + y * g.i_rz);
    g.gy = (q * x) * (g.i_rz + ca * g.i_Wr);
    g.gz = -(q * x) * (sa * g.i_Wr);
    const double p2 = 2.0 * nu + 1.0;
    g.fx = p2 * g.i_Wr + g.x2 * (g.i_W2r2 - g.i_Wr3);
    g.fy = g.i_Wr + g.S * g.S - g.y2 * g.i_Wr3;
    g.fz = g.i_Wr + g.C * g.C - g.z2 * g.i_Wr3;
}

// Strain of unit by (Ey) and unit bz (Ez) Burgers components.  The
// published expressions share many products; they are grouped here (same
// mathematics, ~40 % fewer FP64 operations): with
//   A = 1/(r(r-z))^2 + 1/(r^3 (r-z)),  Q3 = S (nu + x^2/(W r)) + y x^2/(W r^3),
//   Q4 = C (nu + x^2/(W r)) + z x^2/(W r^3),
//   P = sa ca / W^2 - (y ca + z sa)/(W^2 r) + y z (1/(W r)^2 - 1/(W r^3)),
// the by-part uses Q3, Q4 and P scaled by cos(alpha) and the bz-part the same
// three scaled by sin(alpha).
template <class T>
__device__ __forceinline__ void ad_parts_yz(const AdGeom<T> &g, double nu, double k, T Ey[6], T Ez[6])
{
    const T x = g.x, y = g.y, z = g.z, ca = g.ca, sa = g.sa;
    const double p2 = 2.0 * nu + 1.0;
    const T xk = x * k, sak = sa * k, xsak = xk * sa;
    const T yz = y * z;
    const T A = g.i_r2z2 + g.i_r3z;
    const T x2i = g.x2 * g.i_Wr, x2w3 = g.x2 * g.i_Wr3;
    const T nux = nu + x2i;
    const T Q3 = g.S * nux + y * x2w3;
    const T Q4 = g.C * nux + z * x2w3;
    const T P = sa * ca * g.iW2 - g.ycz * g.i_W2r + yz * (g.i_W2r2 - g.i_Wr3);
    const T hgx = 0.5 * g.gx;
    Ey[0] = -xk * (g.fx * ca + p2 * g.i_rz - g.x2 * A);
    Ey[1] = g.gy - xk * (g.i_rz - g.y2 * A + g.fy * ca);
    Ey[2] = -xk * (g.fz * ca + z * g.ir3);
    Ey[3] = hgx + k * (g.x2 * y * A - nu * y * g.i_rz + ca * Q3);
    Ey[4] = k * (nu * g.ir - g.x2 * g.ir3 + ca * Q4);
    Ey[5] = 0.5 * g.gz - xk * (y * g.ir3 + ca * P);
    Ez[0] = xsak * g.fx;
    Ez[1] = xsak * g.fy;
    Ez[2] = g.gz + xsak * g.fz;
    Ez[3] = -sak * Q3;
    Ez[4] = hgx - sak * Q4;
    Ez[5] = 0.5 * g.gy + xsak * P;
}

// Strain of a unit bx (tensile) Burgers component.
__device__ __forceinline__ void ad_part_x(const AdGeom<double> &g, double nu, double k, double Ex[6])
{
    const double x = g.x, y = g.y, z = g.z, ca = g.ca, sa = g.sa, eta = g.eta;
    const double p2 = 2.0 * nu + 1.0;
    const double yz = y * z;
    Ex[0] = g.gx + k * (eta * g.i_Wr + eta * g.x2 * g.i_W2r2 - eta * g.x2 * g.i_Wr3 + y * g.i_rz
                        - g.x2 * y * g.i_r2z2 - g.x2 * y * g.i_r3z);
    Ex[1] = k * (g.fy * eta + p2 * y * g.i_rz - g.y2 * y * g.i_r2z2 - g.y2 * y * g.i_r3z - 2.0 * nu * ca * g.S);
    Ex[2] = k * (eta * g.i_Wr + eta * g.C * g.C - eta * g.z2 * g.i_Wr3 + yz * g.ir3 + 2.0 * nu * sa * g.C);
    Ex[3] = 0.5 * g.gy - k * (x * g.y2 * g.i_r2z2 - nu * x * g.i_rz + x * g.y2 * g.i_r3z - nu * x * ca * g.i_Wr
                              + eta * x * g.S * g.i_Wr + eta * x * y * g.i_Wr3);
    Ex[4] = 0.5 * g.gz - k * (-x * y * g.ir3 + nu * x * sa * g.i_Wr + eta * x * g.C * g.i_Wr + eta * x * z * g.i_Wr3);
    Ex[5] = k * (g.y2 * g.ir3 - nu * g.ir - nu * ca * g.C + nu * sa * g.S + eta * sa * ca * g.iW2
                 - eta * g.ycz * g.i_W2r + eta * yz * g.i_W2r2 - eta * yz * g.i_Wr3);
}

// acc += B^T T' B for the rotation B = [[1,0,0],[0,sz,-sy],[0,sy,sz]] about x
// (the back-rotation of src/TDstressFS_C.cpp:240-255), with the double angle
// (c2, s2) = (sz^2 - sy^2, 2 sy sz) of the unit vector (sy, sz): the yz-block
// is its mean, plus its half difference and off-diagonal term rotated by 2x.
template <class T>
__device__ __forceinline__ void add_rot_x(T acc[6], const T t[6], T sy, T sz, T c2, T s2)
{
    const T h = 0.5 * (t[1] + t[2]), d = 0.5 * (t[1] - t[2]);
    const T u = c2 * d + s2 * t[5];
    acc[0] += t[0];
    acc[1] += h + u;
    acc[2] += h - u;
    acc[3] += sz * t[3] + sy * t[4];
    acc[4] += sz * t[4] - sy * t[3];
    acc[5] += c2 * t[5] - s2 * d;
}

// Source fields through an accessor: F(i) returns field i.
template <class Src, class T>
__device__ __forceinline__ void tdcs_point(const Src &F, T X, T Y, T Z, T &x, T &y, T &z)
{
    const T dx = X - F(F_P2X), dy = Y - F(F_P2Y), dz = Z - F(F_P2Z);
    x = F(F_NX) * dx + F(F_NY) * dy + F(F_NZ) * dz;
    y = F(F_SX) * dx + F(F_SY) * dy + F(F_SZ) * dz;
    z = F(F_DX) * dx + F(F_DY) * dy + F(F_DZ) * dz;
}

// 2/k times the TDCS strain (triangle system) of unit strike (Es) and unit dip
// (Ed) slip, k = 1/(8 pi (1 - nu)).  Returns false for mode 0 (strain zero).
//
// The back-rotation of each angular dislocation (src/TDstressFS_C.cpp:185-256)
// in harmonic form.  With e^{i th} = sz + i sy the rotation about x from the
// triangle system to the dislocation's, a yz-vector v maps to e^{i th} v, so
// the Burgers vector b = by + i bz enters the dislocation as e^{i th} b and the
// strain returns with E_xx and E_yy + E_zz unchanged, w = E_xy + i E_xz
// multiplied by e^{-i th} and q = (E_yy - E_zz)/2 + i E_yz by e^{-2i th}.
// Writing the dislocation's real-linear response to b' as P b' + Q conj(b'):
//   w = P_w b + Q_w e^{-2i th} conj(b),   q = P_q e^{-i th} b + Q_q e^{-3i th} conj(b),
// so per dislocation only Q_w, P_q, Q_q are rotated (one complex product
// each, accumulated by fused multiply-adds), P_w is summed as it is, and
// strike (b = 1) and dip (b = i) are read from the same sums at the end.
// The responses are the grouped by- and bz-parts of ad_parts_yz divided by k
// (the g-terms scaled by 2 (1 - nu) instead of 1/(4 pi)).
template <class Src, class T>
__device__ __forceinline__ bool tdcs_strain_sd2k(const Src &F, T x, T y, T z, double nu, T Es[6], T Ed[6])
{
#pragma unroll
    for (int i = 0; i < 6; ++i) { Es[i] = 0.0; Ed[i] = 0.0; }
    const int m = tri_mode_fast(x, y, z, F(F_P1Y), F(F_P1Z), F(F_P3Y), F(F_P3Z), F(F_DEN), F(F_IDEN));
    if (m == 0) return false;
    const bool pm = (m == 1);   // the side vectors' signs by selection, not products
    const double p2 = 2.0 * nu + 1.0, qg = 2.0 * (1.0 - nu);
    T xs = 0.0, xd = 0.0;       // E_xx, strike and dip
    T Ss = 0.0, Sd = 0.0;       // E_yy + E_zz
    T Pr = 0.0, Pi = 0.0;       // 2 sum P_w
    T Rr = 0.0, Ri = 0.0;       // 2 sum Q_w e^{-2i th}
    T Ur = 0.0, Ui = 0.0;       // 4 sum P_q e^{-i th}
    T Vr = 0.0, Vi = 0.0;       // 4 sum Q_q e^{-3i th}
#pragma unroll
    for (int v = 0; v < 3; ++v) {
        T vy, vz, sy, sz, ca, sa, c2, s2, c3, s3;
        if (v == 0) {
            const T ey = F(F_E13Y), ez = F(F_E13Z), a3 = F(F_C3A), b3 = F(F_S3A);
            vy = F(F_P1Y); vz = F(F_P1Z); sy = pm ? -ey : ey; sz = pm ? -ez : ez; ca = F(F_CA); sa = F(F_SA);
            c2 = F(F_C2A); s2 = F(F_S2A); c3 = pm ? -a3 : a3; s3 = pm ? -b3 : b3;
        } else if (v == 1) {
            const T ey = F(F_E12Y), ez = F(F_E12Z), a3 = F(F_C3B), b3 = F(F_S3B);
            vy = 0.0; vz = 0.0; sy = pm ? ey : -ey; sz = pm ? ez : -ez; ca = F(F_CB); sa = F(F_SB);
            c2 = F(F_C2B); s2 = F(F_S2B); c3 = pm ? a3 : -a3; s3 = pm ? b3 : -b3;
        } else {
            const T ey = F(F_E23Y), ez = F(F_E23Z), a3 = F(F_C3C), b3 = F(F_S3C);
            vy = F(F_P3Y); vz = F(F_P3Z); sy = pm ? ey : -ey; sz = pm ? ez : -ez; ca = F(F_CC); sa = F(F_SC);
            c2 = F(F_C2C); s2 = F(F_S2C); c3 = pm ? a3 : -a3; s3 = pm ? b3 : -b3;
        }
        const T ty = y - vy, tz = z - vz;
        AdGeom<T> g;
        ad_geom<T>(x, sz * ty - sy * tz, sy * ty + sz * tz, ca, sa, nu, g, qg);
        const T ax = g.x, ay = g.y, az = g.z;
        const T xsa = ax * sa, yz = ay * az;
        const T A = g.i_r2z2 + g.i_r3z, x2A = g.x2 * A;
        const T x2i = g.x2 * g.i_Wr, x2w3 = g.x2 * g.i_Wr3;
        const T nux = nu + x2i;
        const T Q3 = g.S * nux + ay * x2w3;
        const T Q4 = g.C * nux + az * x2w3;
        const T Pq = sa * ca * g.iW2 - g.ycz * g.i_W2r + yz * (g.i_W2r2 - g.i_Wr3);
        // E_xx of by (ey) and bz (ez)
        const T e0y = -ax * ((g.fx * ca + p2 * g.i_rz) - x2A);
        const T e0z = xsa * g.fx;
        // E_yy, E_zz
        const T e1y = g.gy - ax * (g.i_rz - g.y2 * A + g.fy * ca);
        const T e2y = -ax * (g.fz * ca + az * g.ir3);
        const T e1z = xsa * g.fy;
        const T e2z = g.gz + xsa * g.fz;
        // 2 E_yz
        const T e5y = g.gz - (ax + ax) * (ay * g.ir3 + ca * Pq);
        const T e5z = g.gy + (xsa + xsa) * Pq;
        // 2 P_w and 2 Q_w from 2 (E_xy + i E_xz) of by and bz
        const T X3 = ay * (x2A - nu * g.i_rz) + ca * Q3;
        const T X4 = nu * g.ir - g.x2 * g.ir3 + ca * Q4;
        const T wPr = (X3 + g.gx) - sa * Q4, wPi = X4 + sa * Q3;
        const T wQr = X3 + sa * Q4, wQi = X4 - sa * Q3;
        // 4 P_q and 4 Q_q from (E_yy - E_zz) + 2i E_yz of by and bz
        const T Sy = e1y + e2y, Sz = e1z + e2z;
        const T Dy = e1y - e2y, Dz = e1z - e2z;
        const T ar = e5z + Dy, ai = e5y - Dz;
        const T br = Dy - e5z, bi = e5y + Dz;
        // invariants: strike b' = (sz, sy), dip b' = (-sy, sz); the rest rotated
        xs = sz * e0y + (sy * e0z + xs);
        xd = sz * e0z + (xd - sy * e0y);
        Ss = sz * Sy + (sy * Sz + Ss);
        Sd = sz * Sz + (Sd - sy * Sy);
        Pr = Pr + wPr;
        Pi = Pi + wPi;
        Rr = c2 * wQr + (s2 * wQi + Rr);
        Ri = c2 * wQi + (Ri - s2 * wQr);
        Ur = sz * ar + (sy * ai + Ur);
        Ui = sz * ai + (Ui - sy * ar);
        Vr = c3 * br + (s3 * bi + Vr);
        Vi = c3 * bi + (Vi - s3 * br);
    }
    // strike b = 1: 2w = P + R, 4q = U + V; dip b = i: 2w = i (P - R), 4q = i (U - V)
    const T uvr = Ur + Vr, uvi = Ui + Vi, umr = Ur - Vr, umi = Ui - Vi;
    Es[0] = 2.0 * xs; Es[1] = 0.5 * uvr + Ss; Es[2] = Ss - 0.5 * uvr;
    Es[3] = Pr + Rr; Es[4] = Pi + Ri; Es[5] = 0.5 * uvi;
    Ed[0] = 2.0 * xd; Ed[1] = Sd - 0.5 * umi; Ed[2] = 0.5 * umi + Sd;
    Ed[3] = Ri - Pi; Ed[4] = Pr - Rr; Ed[5] = 0.5 * umr;
    return true;
}

// General Burgers vector (bx = Ts, by = Ss, bz = Ds) strain in the triangle system.
template <class Src>
__device__ __forceinline__ void tdcs_strain_general(const Src &F, double x, double y, double z, double bx, double by,
                                                    double bz, double nu, double k, double E[6])
{
#pragma unroll
    for (int i = 0; i < 6; ++i) E[i] = 0.0;
    const int m = tri_mode<double>(x, y, z, F(F_P1Y), F(F_P1Z), F(F_P3Y), F(F_P3Z), F(F_DEN));
    if (m == 0) return;
    const double sg = (m == 1) ? 1.0 : -1.0;
    for (int v = 0; v < 3; ++v) {
        double vy, vz, sy, sz, ca, sa;
        if (v == 0) { vy = F(F_P1Y); vz = F(F_P1Z); sy = -sg * F(F_E13Y); sz = -sg * F(F_E13Z); ca = F(F_CA); sa = F(F_SA); }
        else if (v == 1) { vy = 0.0; vz = 0.0; sy = sg * F(F_E12Y); sz = sg * F(F_E12Z); ca = F(F_CB); sa = F(F_SB); }
        else { vy = F(F_P3Y); vz = F(F_P3Z); sy = sg * F(F_E23Y); sz = sg * F(F_E23Z); ca = F(F_CC); sa = F(F_SC); }
        const double ty = y - vy, tz = z - vz;
        AdGeom<double> g;
        ad_geom<double>(x, sz * ty - sy * tz, sy * ty + sz * tz, ca, sa, nu, g);
        double Ey[6], Ez[6], Ex[6];
        ad_parts_yz<double>(g, nu, k, Ey, Ez);
        const double by1 = sz * by - sy * bz, bz1 = sy * by + sz * bz;
        double t[6];
        if (bx != 0.0) {
            ad_part_x(g, nu, k, Ex);
            for (int i = 0; i < 6; ++i) t[i] = bx * Ex[i] + by1 * Ey[i] + bz1 * Ez[i];
        } else {
            for (int i = 0; i < 6; ++i) t[i] = by1 * Ey[i] + bz1 * Ez[i];
        }
        add_rot_x(E, t, sy, sz, sz * sz - sy * sy, 2.0 * (sy * sz));
    }
}

// T_EFCS = A^T T A with A rows (n, s, d) of the source system.
template <class Src>
__device__ __forceinline__ void tdcs_to_efcs(const Src &F, const double t[6], double e[6])
{
    const double A[3][3] = {{F(F_NX), F(F_NY), F(F_NZ)}, {F(F_SX), F(F_SY), F(F_SZ)}, {F(F_DX), F(F_DY), F(F_DZ)}};
    const double T[3][3] = {{t[0], t[3], t[4]}, {t[3], t[1], t[5]}, {t[4], t[5], t[2]}};
    double M[3][3];   // M = T A
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) M[i][j] = T[i][0] * A[0][j] + T[i][1] * A[1][j] + T[i][2] * A[2][j];
    e[0] = A[0][0] * M[0][0] + A[1][0] * M[1][0] + A[2][0] * M[2][0];
    e[1] = A[0][1] * M[0][1] + A[1][1] * M[1][1] + A[2][1] * M[2][1];
    e[2] = A[0][2] * M[0][2] + A[1][2] * M[1][2] + A[2][2] * M[2][2];
    e[3] = A[0][0] * M[0][1] + A[1][0] * M[1][1] + A[2][0] * M[2][1];
    e[4] = A[0][0] * M[0][2] + A[1][0] * M[1][2] + A[2][0] * M[2][2];
    e[5] = A[0][1] * M[0][2] + A[1][1] * M[1][2] + A[2][1] * M[2][2];
}

__device__ __forceinline__ void hooke(const double e[6], double mu, double lam, double s[6])
{
    const double tr = e[0] + e[1] + e[2];
    s[0] = 2.0 * mu * e[0] + lam * tr;
    s[1] = 2.0 * mu * e[1] + lam * tr;
    s[2] = 2.0 * mu * e[2] + lam * tr;
    s[3] = 2.0 * mu * e[3];
    s[4] = 2.0 * mu * e[4];
    s[5] = 2.0 * mu * e[5];
}

// Tractions (along e1, e2, n of the receiver) of a TDCS strain E, given the
// receiver axes already rotated into the source system (ue1, ue2, un).
template <class T>
__device__ __forceinline__ void tractions_tdcs(const T E[6], const T ue1[3], const T ue2[3], const T un[3],
                                               double two_mu, double lam, T out[3])
{
    const T u0 = E[0] * un[0] + E[3] * un[1] + E[4] * un[2];
    const T u1 = E[3] * un[0] + E[1] * un[1] + E[5] * un[2];
    const T u2 = E[4] * un[0] + E[5] * un[1] + E[2] * un[2];
    const T tr = E[0] + E[1] + E[2];
    out[0] = two_mu * (ue1[0] * u0 + ue1[1] * u1 + ue1[2] * u2);
    out[1] = two_mu * (ue2[0] * u0 + ue2[1] * u1 + ue2[2] * u2);
    out[2] = two_mu * (un[0] * u0 + un[1] * u1 + un[2] * u2) + lam * tr;
}

// tractions_tdcs with ue1, ue2 already multiplied by cmu (the traction
// scale): out_c = ue_c . (E un) for c = e1, e2, cmu un . (E un) + clam tr(E).
template <class T>
__device__ __forceinline__ void tractions_tdcs_scaled(const T E[6], const T ue1[3], const T ue2[3], const T un[3],
                                                      double cmu, double clam, T out[3])
{
    const T u0 = E[0] * un[0] + E[3] * un[1] + E[4] * un[2];
    const T u1 = E[3] * un[0] + E[1] * un[1] + E[5] * un[2];
    const T u2 = E[4] * un[0] + E[5] * un[1] + E[2] * un[2];
    const T tr = E[0] + E[1] + E[2];
    out[0] = ue1[0] * u0 + ue1[1] * u1 + ue1[2] * u2;
    out[1] = ue2[0] * u0 + ue2[1] * u1 + ue2[2] * u2;
    out[2] = cmu * (un[0] * u0 + un[1] * u1 + un[2] * u2) + clam * tr;
}

// The six tractions of one (receiver, source) pair: receiver record R
// (centroid, e1, e2, n), source fields F; ts = unit strike slip, td = unit dip
// slip, components (e1, e2, n).  kScaledAxes: R's e1 and e2 come multiplied
// by traction_axis_scale(k, two_mu) (the assembly kernel scales them once per
// receiver tile).
__host__ __device__ inline double traction_axis_scale(double k, double two_mu) { return (0.5 * k) * two_mu; }

template <class Src, bool kScaledAxes = false>
__device__ __forceinline__ void pair_tractions(const Src &F, const double *R, double nu, double k, double two_mu,
                                               double lam, double ts[3], double td[3])
{
    double x, y, z;
    tdcs_point(F, R[0], R[1], R[2], x, y, z);
    double Es[6], Ed[6];   // 2/k times the strains
    tdcs_strain_sd2k(F, x, y, z, nu, Es, Ed);
    double ue1[3], ue2[3], un[3];   // receiver axes in the source system
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const int fa = F_NX + 3 * a;
        ue1[a] = F(fa) * R[3] + F(fa + 1) * R[4] + F(fa + 2) * R[5];
        ue2[a] = F(fa) * R[6] + F(fa + 1) * R[7] + F(fa + 2) * R[8];
        un[a] = F(fa) * R[9] + F(fa + 1) * R[10] + F(fa + 2) * R[11];
    }
    const double hk = 0.5 * k;
    if (kScaledAxes) {
        tractions_tdcs_scaled(Es, ue1, ue2, un, traction_axis_scale(k, two_mu), hk * lam, ts);
        tractions_tdcs_scaled(Ed, ue1, ue2, un, traction_axis_scale(k, two_mu), hk * lam, td);
    } else {
        tractions_tdcs(Es, ue1, ue2, un, hk * two_mu, hk * lam, ts);
        tractions_tdcs(Ed, ue1, ue2, un, hk * two_mu, hk * lam, td);
    }
}

}  // namespace gf
}  // namespace pq3d
