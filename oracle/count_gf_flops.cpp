// Operation count of the GPU assembly kernel's per-pair arithmetic -- test
// infrastructure.  Instantiates the device math of
// pyquake3d_gb300/csrc/gf_device.cuh with a counting scalar type and runs it
// over every (receiver, source) pair of a mesh read from stdin
// ("N" then N lines of 9 vertex coordinates), then prints the mean number of
// FP64 operations per pair as JSON.  Convention: add, sub, mul, div and sqrt
// count one each (a fused multiply-add is a mul and an add); comparisons and
// negations are free.  The kernel body's own lines (receiver axes rotated into
// the source system, 2 x traction contraction with e1, e2 pre-scaled) are restated here.
#include <cmath>
#include <cstdio>
#include <vector>

struct Ops { long long add = 0, mul = 0, div = 0, sqrt_ = 0; };
static Ops g_ops;

struct C {
    double v;
    C() : v(0) {}
    C(double x) : v(x) {}
};
inline C operator+(C a, C b) { ++g_ops.add; return C(a.v + b.v); }
inline C operator-(C a, C b) { ++g_ops.add; return C(a.v - b.v); }
inline C operator*(C a, C b) { ++g_ops.mul; return C(a.v * b.v); }
inline C operator/(C a, C b) { ++g_ops.div; return C(a.v / b.v); }
inline C operator-(C a) { return C(-a.v); }
inline C &operator+=(C &a, C b) { ++g_ops.add; a.v += b.v; return a; }
inline bool operator<=(C a, double b) { return a.v <= b; }
inline bool operator>=(C a, double b) { return a.v >= b; }
inline bool operator==(C a, double b) { return a.v == b; }
inline bool operator!=(C a, double b) { return a.v != b; }
inline bool operator>(C a, C b) { return a.v > b.v; }
inline C sqrt(C a) { ++g_ops.sqrt_; return C(std::sqrt(a.v)); }
inline bool isfinite_t(C a) { return std::isfinite(a.v); }

#include "../pyquake3d_gb300/csrc/gf_device.cuh"

using namespace pq3d::gf;

struct CntSrc {   // source fields read as counted scalars (loads are free)
    const double *f;
    C operator()(int i) const { return C(f[i]); }
};

int main()
{
    long long N;
    if (scanf("%lld", &N) != 1) return 1;
    std::vector<double> tri(9 * N);
    for (long long i = 0; i < 9 * N; ++i)
        if (scanf("%lf", &tri[i]) != 1) return 1;
    std::vector<double> src(kSrcStride * N), rcv(kRecvStride * N);
    for (long long j = 0; j < N; ++j) {
        setup_source(&tri[9 * j], &tri[9 * j + 3], &tri[9 * j + 6], &src[kSrcStride * j], 1);
        setup_receiver(&tri[9 * j], &tri[9 * j + 3], &tri[9 * j + 6], &rcv[kRecvStride * j]);
    }
    const double mu = 32038120320.0, lam = mu;
    const double nu = 1.0 / (1.0 + lam / mu) / 2.0, k = 1.0 / (8.0 * kPi * (1.0 - nu));
    long long pairs = 0, mode0 = 0;
    for (long long j = 0; j < N; ++j) {
        const CntSrc F{&src[kSrcStride * j]};
        for (long long i = 0; i < N; ++i) {
            const double *R = &rcv[kRecvStride * i];
            C x, y, z;
            tdcs_point(F, C(R[0]), C(R[1]), C(R[2]), x, y, z);
            C Es[6], Ed[6];   // 2/k times the strains
            if (!tdcs_strain_sd2k(F, x, y, z, nu, Es, Ed)) ++mode0;
            // e1, e2 multiplied by the traction scale once per receiver tile
            // in the kernel (not a per-pair operation)
            const double cmu = traction_axis_scale(k, 2.0 * mu);
            C ue1[3], ue2[3], un[3];
            for (int a = 0; a < 3; ++a) {
                const int fa = F_NX + 3 * a;
                ue1[a] = F(fa) * (cmu * R[3]) + F(fa + 1) * (cmu * R[4]) + F(fa + 2) * (cmu * R[5]);
                ue2[a] = F(fa) * (cmu * R[6]) + F(fa + 1) * (cmu * R[7]) + F(fa + 2) * (cmu * R[8]);
                un[a] = F(fa) * R[9] + F(fa + 1) * R[10] + F(fa + 2) * R[11];
            }
            C ts[3], td[3];
            tractions_tdcs_scaled<C>(Es, ue1, ue2, un, cmu, 0.5 * k * lam, ts);
            tractions_tdcs_scaled<C>(Ed, ue1, ue2, un, cmu, 0.5 * k * lam, td);
            ++pairs;
        }
    }
    const double p = (double)pairs;
    const double tot = (g_ops.add + g_ops.mul + g_ops.div + g_ops.sqrt_) / p;
    printf("{\"pairs\": %lld, \"mode0_pairs\": %lld, \"add\": %.3f, \"mul\": %.3f, \"div\": %.3f, \"sqrt\": %.3f, "
           "\"flops_per_pair\": %.3f}\n",
           pairs, mode0, g_ops.add / p, g_ops.mul / p, g_ops.div / p, g_ops.sqrt_ / p, tot);
    return 0;
}
