// Operation count of the GPU half-space assembly kernel's per-pair arithmetic
// -- test infrastructure.  Compiles the device math of
// pyquake3d_gb300/csrc/gf_device.cuh and hs_device.cuh with every `double`
// replaced by a counting scalar type and runs the kernel body
// (pair_tractions_hs: main dislocation, image dislocation, the free-surface
// correction of the three sides in forward-mode dual numbers, two traction
// contractions) over every (receiver, source) pair of a mesh read from stdin
// ("N" then N lines of 9 vertex coordinates; z <= 0).  Prints the mean number
// of FP64 operations per pair as JSON.  Convention as the full-space count:
// add, sub, mul, div and sqrt count one each (a fused multiply-add is a mul
// and an add); comparisons, negations and loads are free; each transcendental
// call (log, atan, sin, cos, tan, acos) counts one and is reported apart.
// (`double` becomes the counting type Q64 for the two headers.)  The per-source set-up (source records, side tables) is not counted: the
// kernel reads it from tables built once per source.
#include <cmath>
#include <cstdio>
#include <vector>

struct Ops { long long add = 0, mul = 0, div = 0, sqrt_ = 0, trans = 0; };
static Ops g_ops;

struct Q64 {
    double v;
    constexpr Q64() : v(0) {}
    constexpr Q64(double x) : v(x) {}
    explicit operator int() const { return (int)v; }
};
inline Q64 operator+(Q64 a, Q64 b) { ++g_ops.add; return Q64(a.v + b.v); }
inline Q64 operator-(Q64 a, Q64 b) { ++g_ops.add; return Q64(a.v - b.v); }
inline Q64 operator*(Q64 a, Q64 b) { ++g_ops.mul; return Q64(a.v * b.v); }
inline Q64 operator/(Q64 a, Q64 b) { ++g_ops.div; return Q64(a.v / b.v); }
inline Q64 operator-(Q64 a) { return Q64(-a.v); }
inline Q64 &operator+=(Q64 &a, Q64 b) { ++g_ops.add; a.v += b.v; return a; }
inline Q64 &operator-=(Q64 &a, Q64 b) { ++g_ops.add; a.v -= b.v; return a; }
inline Q64 &operator*=(Q64 &a, Q64 b) { ++g_ops.mul; a.v *= b.v; return a; }
inline Q64 &operator/=(Q64 &a, Q64 b) { ++g_ops.div; a.v /= b.v; return a; }
inline bool operator<(Q64 a, Q64 b) { return a.v < b.v; }
inline bool operator>(Q64 a, Q64 b) { return a.v > b.v; }
inline bool operator<=(Q64 a, Q64 b) { return a.v <= b.v; }
inline bool operator>=(Q64 a, Q64 b) { return a.v >= b.v; }
inline bool operator==(Q64 a, Q64 b) { return a.v == b.v; }
inline bool operator!=(Q64 a, Q64 b) { return a.v != b.v; }
inline Q64 sqrt(Q64 a) { ++g_ops.sqrt_; return Q64(std::sqrt(a.v)); }
inline Q64 fabs(Q64 a) { return Q64(std::fabs(a.v)); }
inline Q64 log(Q64 a) { ++g_ops.trans; return Q64(std::log(a.v)); }
inline Q64 atan(Q64 a) { ++g_ops.trans; return Q64(std::atan(a.v)); }
inline Q64 sin(Q64 a) { ++g_ops.trans; return Q64(std::sin(a.v)); }
inline Q64 cos(Q64 a) { ++g_ops.trans; return Q64(std::cos(a.v)); }
inline Q64 tan(Q64 a) { ++g_ops.trans; return Q64(std::tan(a.v)); }
inline Q64 acos(Q64 a) { ++g_ops.trans; return Q64(std::acos(a.v)); }
namespace std {
inline bool isfinite(Q64 a) { return std::isfinite(a.v); }
}

#define PQ3D_OPCOUNT
#define double Q64
#include "../pyquake3d_gb300/csrc/gf_device.cuh"
#include "../pyquake3d_gb300/csrc/hs_device.cuh"
#undef double

using namespace pq3d::gf;

struct Soa {   // field f of one source in a structure-of-arrays table (loads are free)
    const Q64 *base;
    int stride;
    Q64 operator()(int f) const { return base[f * stride]; }
};

int main()
{
    long long N;
    if (scanf("%lld", &N) != 1) return 1;
    std::vector<double> tri(9 * N);
    for (long long i = 0; i < 9 * N; ++i)
        if (scanf("%lf", &tri[i]) != 1) return 1;
    std::vector<Q64> src(kSrcStride * N), img(kSrcStride * N), fsc(kFscStride * N), rcv(kRecvStride * N);
    for (long long j = 0; j < N; ++j) {
        Q64 a[3], b[3], c[3], am[3], bm[3], cm[3];
        for (int q = 0; q < 3; ++q) {
            a[q] = tri[9 * j + q]; b[q] = tri[9 * j + 3 + q]; c[q] = tri[9 * j + 6 + q];
        }
        for (int q = 0; q < 3; ++q) { am[q] = a[q]; bm[q] = b[q]; cm[q] = c[q]; }
        am[2] = -a[2]; bm[2] = -b[2]; cm[2] = -c[2];
        setup_source(a, b, c, &src[j], (int)N);
        setup_source(am, bm, cm, &img[j], (int)N);
        setup_fsc(a, b, c, &fsc[j], (int)N);
        setup_receiver(a, b, c, &rcv[kRecvStride * j]);
    }
    const double mu = 32038120320.0, lam = mu;
    const double nu = 1.0 / (1.0 + lam / mu) / 2.0, k = 1.0 / (8.0 * 3.14159265358979323846 * (1.0 - nu));
    g_ops = Ops();
    long long pairs = 0;
    for (long long j = 0; j < N; ++j) {
        const Soa F{&src[j], (int)N}, Fi{&img[j], (int)N}, G{&fsc[j], (int)N};
        for (long long i = 0; i < N; ++i) {
            Q64 ts[3], td[3];
            pair_tractions_hs(F, Fi, G, &rcv[kRecvStride * i], Q64(nu), Q64(k), Q64(2.0 * mu), Q64(lam), ts, td);
            ++pairs;
        }
    }
    const double p = (double)pairs;
    printf("{\"pairs\": %lld, \"add\": %.3f, \"mul\": %.3f, \"div\": %.3f, \"sqrt\": %.3f, \"transcendental\": %.3f, "
           "\"flops_per_pair\": %.3f}\n",
           pairs, g_ops.add / p, g_ops.mul / p, g_ops.div / p, g_ops.sqrt_ / p, g_ops.trans / p,
           (g_ops.add + g_ops.mul + g_ops.div + g_ops.sqrt_) / p);
    return 0;
}
