// CPU check of the double-float helpers of quantumlab_gb300/csrc/df64.cuh
// (compiled by tests/test_df64.py with g++; no GPU).  Prints one line of
// measured bounds per check; the Python test compares them with the limits.
#include "df64.cuh"

#include <cmath>
#include <cstdio>
#include <random>

using namespace qg::df;

int main() {
    std::mt19937_64 rng(20261204);
    std::uniform_real_distribution<double> u(-1, 1);
    // double -> DF: relative error for |x| >= 2^-73, absolute below
    double inRel = 0, inAbsSmall = 0, outRel = 0;
    long loTooBig = 0;
    for (int i = 0; i < 2000000; ++i) {
        const double x = std::ldexp(u(rng), (int)(rng() % 240) - 120);
        const F2 f = fromDouble(x);
        const long double back = (long double)f.h + (long double)f.l;
        const double err = (double)std::fabs(back - (long double)x);
        if (std::fabs(x) >= std::ldexp(1.0, -73)) inRel = std::max(inRel, err / std::fabs(x));
        else inAbsSmall = std::max(inAbsSmall, err);
        if (!(std::fabs(f.l) <= std::ldexp(std::fabs(f.h), -23))) ++loTooBig;      // below one ulp of hi
        // DF -> double: the double nearest below |hi + lo| (truncation)
        const double y = toDouble(f);
        if (back != 0) outRel = std::max(outRel, (double)(std::fabs((long double)y - back) / std::fabs(back)));
    }
    printf("in_rel %.6e\nin_abs_small %.6e\nlo_not_below_ulp %ld\nout_rel %.6e\n", inRel, inAbsSmall, loTooBig, outRel);
    // DF results with |lo| <= half an ulp of hi, around powers of two and
    // with both signs of lo
    double pow2 = 0;
    for (int i = 0; i < 200000; ++i) {
        const float h = std::ldexp(1.0f, (int)(rng() % 100) - 50) * ((rng() & 1) ? -1.f : 1.f);
        const float l = (float)(u(rng) * std::ldexp((double)std::fabs(h), -25));
        const double want = (double)h + (double)l;                 // exact: 49 bits at most
        pow2 = std::max(pow2, std::fabs(toDouble(F2{h, l}) - want) / std::fabs(want));
    }
    printf("pow2_rel %.6e\n", pow2);
    // four-term dot products, with cancellation in every seventh case
    double dot = 0;
    for (int i = 0; i < 1000000; ++i) {
        double c[4], x[4];
        F2 cf[4], xf[4];
        for (int k = 0; k < 4; ++k) {
            c[k] = u(rng);
            x[k] = std::ldexp(u(rng), -(int)(rng() % 20));
        }
        if (i % 7 == 0) x[3] = -(c[0] * x[0] + c[1] * x[1] + c[2] * x[2]) / c[3];
        long double ref = 0, mx = 0;
        for (int k = 0; k < 4; ++k) {
            cf[k] = splitConst(c[k]);
            xf[k] = fromDouble(x[k]);
            ref += (long double)c[k] * x[k];
            mx = std::max(mx, std::fabs((long double)c[k] * x[k]));
        }
        const double got = toDouble(dot4(cf, xf));
        dot = std::max(dot, (double)(std::fabs((long double)got - ref) / mx));
    }
    printf("dot4_rel_to_largest_term %.6e\n", dot);
    // exact cases
    int exact = 1;
    const double sp[] = {0.0, -0.0, 1.0, -1.0, 0.5, 0.25, -3.0, 1.5, std::ldexp(1.0, -126)};
    for (double v : sp) exact &= (toDouble(fromDouble(v)) == v) && (std::signbit(toDouble(fromDouble(v))) == std::signbit(v));
    exact &= (toDouble(fromDouble(1e-40)) == 0.0);
    printf("exact_cases %d\n", exact);
    return 0;
}
