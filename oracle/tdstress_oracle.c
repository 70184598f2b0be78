/*
 * CPU ORACLE -- test infrastructure only.
 *
 * Plain-C restatement of the triangular-dislocation (Nikkhoo & Walter 2015,
 * GJI 201:1119) stress/strain algorithm as PyQuake3D implements it, used by the
 * test-suite and by the CPU-baseline leg of bench.py as the checker.  Nothing in
 * the product path links or calls this file; the GPU library fails loudly when
 * its CUDA extension is missing instead of falling back here.
 *
 * Parity is pinned against the reference's own TDstressFS_C built from its
 * sources (oracle/Makefile target `ref`) through the fixtures under
 * tests/golden/ (see tests/golden/make_golden.py).
 *
 * Conventions followed (reference file:line):
 *   - angular-dislocation strain     src/TDstressFS_C.cpp:51-121  (AngDisStrain)
 *   - configuration test (+1/-1/0)    src/TDstressFS_C.cpp:125-166 (trimodefinder)
 *   - per-side frame rotation         src/TDstressFS_C.cpp:185-256 (TDSetupS)
 *   - tensor rotation T' = A^T T A    src/TDstressFS_C.cpp:21-49   (TensTrans)
 *   - full-space entry point          src/TDstressFS_C.cpp:274-521 (TDstressFS)
 *   - receivers exactly on a side line in the triangle plane (mode 0) keep zero
 *     strain, as the C++ does (src/TDstressFS_C.cpp:446-477); the NumPy twin
 *     writes NaN there instead (src/SH_greenfunction.py:297-302).
 *   - horizontal sources (e_Z x n = 0): the strike axis becomes e_Y * n_z, as in
 *     the published algorithm.  The reference C++ divides by the zero norm there
 *     (src/TDstressFS_C.cpp:317-325) and returns NaN; this is a documented
 *     deviation.
 *   - traction projection [t.e1, t.e2, t.n] with t = sigma.n
 *                                     src/QDsim_gpu.py:1400-1417 (GetTtstress)
 *   - receiver frames                 src/readmsh.py:75-134 (get_eleVec)
 *   - dense operator column j = source j, rows = receivers (centroids)
 *                                     src/QDsim_gpu.py:1745-1878
 */
#include <math.h>
#include <pthread.h>
#include <stdbool.h>
#include <stddef.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#define ORC_PI 3.141592653589793

/* strain order everywhere: xx, yy, zz, xy, xz, yz */

/* T' = A^T T A for a symmetric tensor T stored as 6 components. */
static void rotate_tensor(double t[6], const double A[3][3])
{
    double T[3][3] = {{t[0], t[3], t[4]}, {t[3], t[1], t[5]}, {t[4], t[5], t[2]}};
    double out[3][3];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            double s = 0.0;
            for (int k = 0; k < 3; ++k)
                for (int l = 0; l < 3; ++l) s += A[k][i] * T[k][l] * A[l][j];
            out[i][j] = s;
        }
    t[0] = out[0][0]; t[1] = out[1][1]; t[2] = out[2][2];
    t[3] = out[0][1]; t[4] = out[0][2]; t[5] = out[1][2];
}

/* Strain of an angular dislocation with Burgers vector (bx, by, bz) in its
 * own frame (src/TDstressFS_C.cpp:51-121). */
static void angdis_strain(double x, double y, double z, double alpha,
                          double bx, double by, double bz, double nu, double e[6])
{
    const double ca = cos(alpha), sa = sin(alpha);
    const double eta = y * ca - z * sa;
    const double zeta = y * sa + z * ca;
    const double xx = x * x, yy = y * y, zz = z * z;
    const double rr = xx + yy + zz;
    const double r = sqrt(rr);
    const double r3 = rr * r;
    const double rmz = r - z;
    const double rz = r * rmz;
    const double r2z2 = rr * rmz * rmz;
    const double r3z = r3 * rmz;
    const double W = zeta - r;
    const double W2 = W * W;
    const double Wr = W * r;
    const double W2r = W2 * r;
    const double Wr3 = W * r3;
    const double W2r2 = W2 * rr;
    const double C = (r * ca - z) / Wr;
    const double S = (r * sa - y) / Wr;
    const double k = 1.0 / (8.0 * ORC_PI * (1.0 - nu));
    const double q = 1.0 / (4.0 * ORC_PI);

    /* gradient of the Burgers function */
    const double gx = q * (eta / r / (r - zeta) - y / r / rmz);
    const double gy = q * (x / r / rmz - ca * x / r / (r - zeta));
    const double gz = q * (sa * x / r / (r - zeta));

    const double p2 = 2.0 * nu + 1.0;
    const double fx = p2 / Wr + xx / W2r2 - xx / Wr3;
    const double fy = 1.0 / Wr + S * S - yy / Wr3;
    const double fz = 1.0 / Wr + C * C - zz / Wr3;
    const double ycz = y * ca + z * sa;

    e[0] = bx * gx
         + bx * k * (eta / Wr + eta * xx / W2r2 - eta * xx / Wr3 + y / rz - xx * y / r2z2 - xx * y / r3z)
         - by * x * k * (fx * ca + p2 / rz - xx / r2z2 - xx / r3z)
         + bz * x * sa * k * fx;

    e[1] = by * gy
         + bx * k * (fy * eta + p2 * y / rz - yy * y / r2z2 - yy * y / r3z - 2.0 * nu * ca * S)
         - by * x * k * (1.0 / rz - yy / r2z2 - yy / r3z + fy * ca)
         + bz * x * sa * k * fy;

    e[2] = bz * gz
         + bx * k * (eta / W / r + eta * C * C - eta * zz / Wr3 + y * z / r3 + 2.0 * nu * sa * C)
         - by * x * k * (fz * ca + z / r3)
         + bz * x * sa * k * fz;

    e[3] = 0.5 * (bx * gy + by * gx)
         - bx * k * (x * yy / r2z2 - nu * x / rz + x * yy / r3z - nu * x * ca / Wr + eta * x * S / Wr + eta * x * y / Wr3)
         + by * k * (xx * y / r2z2 - nu * y / rz + xx * y / r3z + nu * ca * S + xx * y * ca / Wr3 + xx * ca * S / Wr)
         - bz * sa * k * (nu * S + xx * S / Wr + xx * y / Wr3);

    e[4] = 0.5 * (bx * gz + bz * gx)
         - bx * k * (-x * y / r3 + nu * x * sa / Wr + eta * x * C / Wr + eta * x * z / Wr3)
         + by * k * (-xx / r3 + nu / r + nu * ca * C + xx * z * ca / Wr3 + xx * ca * C / Wr)
         - bz * sa * k * (nu * C + xx * C / Wr + xx * z / Wr3);

    e[5] = 0.5 * (by * gz + bz * gy)
         + bx * k * (yy / r3 - nu / r - nu * ca * C + nu * sa * S + eta * sa * ca / W2 - eta * ycz / W2r + eta * y * z / W2r2 - eta * y * z / Wr3)
         - by * x * k * (y / r3 + sa * ca * ca / W2 - ca * ycz / W2r + y * z * ca / W2r2 - y * z * ca / Wr3)
         - bz * x * sa * k * (y * z / Wr3 - sa * ca / W2 + ycz / W2r - y * z / W2r2);
}

/* One angular dislocation at a triangle vertex, in the triangle's coordinate
 * system (src/TDstressFS_C.cpp:185-256).  side = (sy, sz) is the side
 * direction, vtx = (vy, vz) the vertex. */
static void side_strain(double x, double y, double z, double alpha, double bx, double by, double bz,
                        double nu, double vy, double vz, double sy, double sz, double e[6])
{
    const double dy = y - vy, dz = z - vz;
    const double y1 = sz * dy - sy * dz;
    const double z1 = sy * dy + sz * dz;
    const double by1 = sz * by - sy * bz;
    const double bz1 = sy * by + sz * bz;
    angdis_strain(x, y1, z1, alpha - ORC_PI, bx, by1, bz1, nu, e);
    const double B[3][3] = {{1.0, 0.0, 0.0}, {0.0, sz, -sy}, {0.0, sy, sz}};
    rotate_tensor(e, B);
}

typedef struct {
    double n[3], s[3], d[3];    /* triangle coordinate system axes */
    double P2[3];               /* origin */
    double p1[3], p3[3];        /* vertices 1 and 3 in the triangle system (vertex 2 = 0) */
    double e12[3], e13[3], e23[3];
    double A, B, C;             /* interior angles at vertices 1, 2, 3 */
} tri_setup;

static void unit(double v[3])
{
    double l = sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    v[0] /= l; v[1] /= l; v[2] /= l;
}

/* Per-source setup (src/TDstressFS_C.cpp:291-396). */
static void setup_triangle(const double P1[3], const double P2[3], const double P3[3], tri_setup *t)
{
    double n[3] = {(P2[1] - P1[1]) * (P3[2] - P1[2]) - (P2[2] - P1[2]) * (P3[1] - P1[1]),
                   (P2[2] - P1[2]) * (P3[0] - P1[0]) - (P2[0] - P1[0]) * (P3[2] - P1[2]),
                   (P2[0] - P1[0]) * (P3[1] - P1[1]) - (P2[1] - P1[1]) * (P3[0] - P1[0])};
    unit(n);
    /* strike = e_Z x n */
    double s[3] = {-n[1], n[0], 0.0};
    double ls = sqrt(s[0] * s[0] + s[1] * s[1] + s[2] * s[2]);
    if (ls == 0.0) {
        s[0] = 0.0; s[1] = n[2]; s[2] = 0.0;
        ls = fabs(n[2]);
    }
    s[0] /= ls; s[1] /= ls; s[2] /= ls;
    double d[3] = {n[1] * s[2] - n[2] * s[1], n[2] * s[0] - n[0] * s[2], n[0] * s[1] - n[1] * s[0]};
    memcpy(t->n, n, sizeof n); memcpy(t->s, s, sizeof s); memcpy(t->d, d, sizeof d);
    memcpy(t->P2, P2, 3 * sizeof(double));
    const double *ax[3] = {n, s, d};
    for (int i = 0; i < 3; ++i) {
        t->p1[i] = ax[i][0] * (P1[0] - P2[0]) + ax[i][1] * (P1[1] - P2[1]) + ax[i][2] * (P1[2] - P2[2]);
        t->p3[i] = ax[i][0] * (P3[0] - P2[0]) + ax[i][1] * (P3[1] - P2[1]) + ax[i][2] * (P3[2] - P2[2]);
    }
    for (int i = 0; i < 3; ++i) {
        t->e12[i] = -t->p1[i];
        t->e13[i] = t->p3[i] - t->p1[i];
        t->e23[i] = t->p3[i];
    }
    unit(t->e12); unit(t->e13); unit(t->e23);
    t->A = acos(t->e12[0] * t->e13[0] + t->e12[1] * t->e13[1] + t->e12[2] * t->e13[2]);
    t->B = acos(-t->e12[0] * t->e23[0] - t->e12[1] * t->e23[1] - t->e12[2] * t->e23[2]);
    t->C = acos(t->e23[0] * t->e13[0] + t->e23[1] * t->e13[1] + t->e23[2] * t->e13[2]);
}

/* Configuration of a receiver relative to the triangle
 * (src/TDstressFS_C.cpp:125-166): +1 first configuration, -1 second, 0 on a
 * side line inside the triangle plane. */
static int tri_mode(const tri_setup *t, double x, double y, double z)
{
    const double x1 = t->p1[1], y1 = t->p1[2];
    const double x2 = 0.0, y2 = 0.0;
    const double x3 = t->p3[1], y3 = t->p3[2];
    const double den = (x1 - x3) * (y2 - y3) - (x2 - x3) * (y1 - y3);
    const double a = ((y - x3) * (y2 - y3) - (x2 - x3) * (z - y3)) / den;
    const double b = ((x1 - x3) * (z - y3) - (y - x3) * (y1 - y3)) / den;
    const double c = 1.0 - a - b;
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

/* Full-space strain (EFCS) at one receiver from one triangle. */
static void fs_strain_point(const tri_setup *t, double X, double Y, double Z,
                            double bx, double by, double bz, double nu, double e[6])
{
    const double dx = X - t->P2[0], dy = Y - t->P2[1], dz = Z - t->P2[2];
    const double x = t->n[0] * dx + t->n[1] * dy + t->n[2] * dz;
    const double y = t->s[0] * dx + t->s[1] * dy + t->s[2] * dz;
    const double z = t->d[0] * dx + t->d[1] * dy + t->d[2] * dz;
    const int m = tri_mode(t, x, y, z);
    for (int i = 0; i < 6; ++i) e[i] = 0.0;
    if (m == 0) return;
    const double sg = (m == 1) ? 1.0 : -1.0; /* side vectors flip between configurations */
    double e1[6], e2[6], e3[6];
    side_strain(x, y, z, t->A, bx, by, bz, nu, t->p1[1], t->p1[2], -sg * t->e13[1], -sg * t->e13[2], e1);
    side_strain(x, y, z, t->B, bx, by, bz, nu, 0.0, 0.0, sg * t->e12[1], sg * t->e12[2], e2);
    side_strain(x, y, z, t->C, bx, by, bz, nu, t->p3[1], t->p3[2], sg * t->e23[1], sg * t->e23[2], e3);
    for (int i = 0; i < 6; ++i) e[i] = e1[i] + e2[i] + e3[i];
    const double A[3][3] = {{t->n[0], t->n[1], t->n[2]}, {t->s[0], t->s[1], t->s[2]}, {t->d[0], t->d[1], t->d[2]}};
    rotate_tensor(e, A);
}

static void hooke(const double e[6], double mu, double lam, double s[6])
{
    const double tr = e[0] + e[1] + e[2];
    s[0] = 2.0 * mu * e[0] + lam * tr;
    s[1] = 2.0 * mu * e[1] + lam * tr;
    s[2] = 2.0 * mu * e[2] + lam * tr;
    s[3] = 2.0 * mu * e[3];
    s[4] = 2.0 * mu * e[4];
    s[5] = 2.0 * mu * e[5];
}

#include "hs_oracle.inc"

static double poisson(double mu, double lam) { return 1.0 / (1.0 + lam / mu) / 2.0; }

/* Stress + strain at one receiver from one triangle, full- or half-space. */
static void td_point(const double P1[3], const double P2[3], const double P3[3], const tri_setup *t,
                     double X, double Y, double Z, double Ss, double Ds, double Ts,
                     double mu, double lam, bool half, double s[6], double e[6])
{
    const double nu = poisson(mu, lam);
    fs_strain_point(t, X, Y, Z, Ts, Ss, Ds, nu, e);
    if (half) hs_add_point(P1, P2, P3, X, Y, Z, Ss, Ds, Ts, mu, lam, nu, e);
    hooke(e, mu, lam, s);
}

/* ---- exported checker entry points (same meaning as the reference C-ABI) ---- */

/* src/TDstressFS_C.cpp:2095-2152 */
void oracle_TDstressFS_C(const double *X, const double *Y, const double *Z, size_t n,
                         const double *P1, const double *P2, const double *P3,
                         double Ss, double Ds, double Ts, double mu, double lam, bool half,
                         double *stress, double *strain)
{
    tri_setup t;
    setup_triangle(P1, P2, P3, &t);
    for (size_t i = 0; i < n; ++i)
        td_point(P1, P2, P3, &t, X[i], Y[i], Z[i], Ss, Ds, Ts, mu, lam, half, stress + 6 * i, strain + 6 * i);
}

/* src/TDstressFS_C.cpp:2155-2200 */
void oracle_TDstressEachSourceAtReceiver_C(double x, double y, double z,
                                           const double *P1, const double *P2, const double *P3, size_t ns,
                                           double Ss, double Ds, double Ts, double mu, double lam, bool half,
                                           double *stress, double *strain)
{
    for (size_t j = 0; j < ns; ++j) {
        tri_setup t;
        setup_triangle(P1 + 3 * j, P2 + 3 * j, P3 + 3 * j, &t);
        td_point(P1 + 3 * j, P2 + 3 * j, P3 + 3 * j, &t, x, y, z, Ss, Ds, Ts, mu, lam, half,
                 stress + 6 * j, strain + 6 * j);
    }
}

/* Receiver frames and centroids (src/readmsh.py:75-134, node order flag False). */
void oracle_element_frames(const double *nodes, const long long *tris, size_t N, double *frames, double *xg)
{
    for (size_t i = 0; i < N; ++i) {
        const double *a = nodes + 3 * (tris[3 * i] - 1);
        const double *b = nodes + 3 * (tris[3 * i + 1] - 1);
        const double *c = nodes + 3 * (tris[3 * i + 2] - 1);
        for (int k = 0; k < 3; ++k) xg[3 * i + k] = ((a[k] + b[k]) + c[k]) / 3.0;
        const double ba[3] = {b[0] - a[0], b[1] - a[1], b[2] - a[2]};
        const double ca[3] = {c[0] - a[0], c[1] - a[1], c[2] - a[2]};
        double n3[3] = {ba[1] * ca[2] - ba[2] * ca[1], ba[2] * ca[0] - ba[0] * ca[2], ba[0] * ca[1] - ba[1] * ca[0]};
        double rr = sqrt(n3[0] * n3[0] + n3[1] * n3[1] + n3[2] * n3[2]);
        n3[0] /= rr; n3[1] /= rr; n3[2] /= rr;
        double e1[3];
        if (fabs(n3[2]) < 1) {
            e1[0] = n3[1]; e1[1] = -n3[0]; e1[2] = 0.0;
            double r1 = sqrt(e1[0] * e1[0] + e1[1] * e1[1]);
            e1[0] /= r1; e1[1] /= r1;
        } else {
            e1[0] = 1.0; e1[1] = 0.0; e1[2] = 0.0;
        }
        const double e2[3] = {n3[1] * e1[2] - n3[2] * e1[1], n3[2] * e1[0] - n3[0] * e1[2], n3[0] * e1[1] - n3[1] * e1[0]};
        double *f = frames + 9 * i;
        f[0] = e1[0]; f[1] = e1[1]; f[2] = e1[2];
        f[3] = e2[0]; f[4] = e2[1]; f[5] = e2[2];
        f[6] = n3[0]; f[7] = n3[1]; f[8] = n3[2];
    }
}

/* [t.e1, t.e2, t.n] with t = sigma.n (src/QDsim_gpu.py:1400-1417). */
static void project(const double s[6], const double *f, double out[3])
{
    const double t0 = s[0] * f[6] + s[3] * f[7] + s[4] * f[8];
    const double t1 = s[3] * f[6] + s[1] * f[7] + s[5] * f[8];
    const double t2 = s[4] * f[6] + s[5] * f[7] + s[2] * f[8];
    out[0] = t0 * f[0] + t1 * f[1] + t2 * f[2];
    out[1] = t0 * f[3] + t1 * f[4] + t2 * f[5];
    out[2] = t0 * f[6] + t1 * f[7] + t2 * f[8];
}

typedef struct {
    const double *nodes;
    const long long *tris;
    const double *frames, *xg;
    size_t N, row0, row1;     /* receivers [row0, row1) */
    size_t col0, col1;        /* sources   [col0, col1) */
    double mu, lam;
    bool half;
    double *out;              /* 6 x N x N: A1s, A2s, Bs, A1d, A2d, Bd */
} asm_job;

static void *asm_worker(void *arg)
{
    asm_job *J = (asm_job *)arg;
    const size_t N = J->N;
    for (size_t j = J->col0; j < J->col1; ++j) {
        const double *P1 = J->nodes + 3 * (J->tris[3 * j] - 1);
        const double *P2 = J->nodes + 3 * (J->tris[3 * j + 1] - 1);
        const double *P3 = J->nodes + 3 * (J->tris[3 * j + 2] - 1);
        tri_setup t;
        setup_triangle(P1, P2, P3, &t);
        for (size_t i = J->row0; i < J->row1; ++i) {
            const double *x = J->xg + 3 * i;
            double s[6], e[6], tr[3];
            for (int dir = 0; dir < 2; ++dir) {
                const double Ss = dir == 0 ? 1.0 : 0.0, Ds = dir == 0 ? 0.0 : 1.0;
                td_point(P1, P2, P3, &t, x[0], x[1], x[2], Ss, Ds, 0.0, J->mu, J->lam, J->half, s, e);
                project(s, J->frames + 9 * i, tr);
                for (int c = 0; c < 3; ++c) J->out[(size_t)(dir * 3 + c) * N * N + i * N + j] = tr[c];
            }
        }
    }
    return NULL;
}

/* Dense traction operators (src/QDsim_gpu.py:1745-1878) for receivers at the
 * element centroids.  out: 6 x N x N doubles in the reference's order
 * (A1s, A2s, Bs, A1d, A2d, Bd); only columns [col0, col1) are written, so that
 * a bounded sample of the full assembly can be timed.  Sources are split
 * across `nthreads` POSIX threads. */
int oracle_assemble_dense(const double *nodes, const long long *tris, size_t N, double mu, double lam,
                          int half, size_t col0, size_t col1, int nthreads, double *out)
{
    double *frames = (double *)malloc(sizeof(double) * 9 * N);
    double *xg = (double *)malloc(sizeof(double) * 3 * N);
    if (!frames || !xg) { free(frames); free(xg); return 1; }
    oracle_element_frames(nodes, tris, N, frames, xg);
    if (nthreads < 1) nthreads = 1;
    pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * nthreads);
    asm_job *jobs = (asm_job *)malloc(sizeof(asm_job) * nthreads);
    size_t ncol = col1 - col0;
    for (int k = 0; k < nthreads; ++k) {
        asm_job J = {nodes, tris, frames, xg, N, 0, N,
                     col0 + ncol * k / nthreads, col0 + ncol * (k + 1) / nthreads, mu, lam, half != 0, out};
        jobs[k] = J;
        pthread_create(&th[k], NULL, asm_worker, &jobs[k]);
    }
    for (int k = 0; k < nthreads; ++k) pthread_join(th[k], NULL);
    free(th); free(jobs); free(frames); free(xg);
    return 0;
}
