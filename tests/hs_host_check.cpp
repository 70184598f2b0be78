// Host build of the half-space device math (pyquake3d_gb300/csrc/hs_device.cuh)
// for the CPU tests: reads cases from stdin and prints, per case, the EFCS
// strain for a general Burgers vector and the six unit-slip tractions of the
// (receiver, source) pair.  Test infrastructure only.
//
// stdin: "n" then n lines "P1(3) P2(3) P3(3) X Y Z Ss Ds Ts e1(3) e2(3) nv(3)"
// stdout: per case 18 numbers: half-space strain(6) ts(3) td(3), then the
// full-space ts(3) td(3) as the dense assembly kernel forms them (receiver
// axes e1, e2 pre-scaled, pair_tractions<..., true>)
#include <cmath>
#include <cstdio>

#include "../pyquake3d_gb300/csrc/hs_device.cuh"

using namespace pq3d::gf;

struct Arr {
    const double *f;
    double operator()(int i) const { return f[i]; }
};

int main()
{
    int n;
    if (scanf("%d", &n) != 1) return 1;
    const double mu = 32038120320.0, lam = mu;
    const double nu = 1.0 / (1.0 + lam / mu) / 2.0, k = 1.0 / (8.0 * kPi * (1.0 - nu));
    for (int c = 0; c < n; ++c) {
        double v[24];
        for (int i = 0; i < 24; ++i)
            if (scanf("%lf", &v[i]) != 1) return 1;
        const double *P1 = v, *P2 = v + 3, *P3 = v + 6;
        double f[kSrcStride], fi[kSrcStride], g[kFscStride];
        setup_source(P1, P2, P3, f, 1);
        const double Q1[3] = {P1[0], P1[1], -P1[2]}, Q2[3] = {P2[0], P2[1], -P2[2]}, Q3[3] = {P3[0], P3[1], -P3[2]};
        setup_source(Q1, Q2, Q3, fi, 1);
        setup_fsc(P1, P2, P3, g, 1);
        const Arr F{f}, Fi{fi}, G{g};
        double e[6];
        point_strain_hs(F, Fi, G, v[9], v[10], v[11], v[14], v[12], v[13], nu, k, e);
        double R[kRecvStride] = {v[9], v[10], v[11], v[15], v[16], v[17], v[18], v[19], v[20], v[21], v[22], v[23]};
        double ts[3], td[3];
        pair_tractions_hs(F, Fi, G, R, nu, k, 2.0 * mu, lam, ts, td);
        for (int i = 0; i < 6; ++i) printf("%.17g ", e[i]);
        for (int i = 0; i < 3; ++i) printf("%.17g ", ts[i]);
        for (int i = 0; i < 3; ++i) printf("%.17g ", td[i]);
        const double cmu = traction_axis_scale(k, 2.0 * mu);
        double Rs[kRecvStride];
        for (int i = 0; i < kRecvStride; ++i) Rs[i] = (i >= 3 && i < 9) ? R[i] * cmu : R[i];
        pair_tractions<Arr, true>(F, Rs, nu, k, 2.0 * mu, lam, ts, td);
        for (int i = 0; i < 3; ++i) printf("%.17g ", ts[i]);
        for (int i = 0; i < 3; ++i) printf("%.17g ", td[i]);
        printf("\n");
    }
    return 0;
}
