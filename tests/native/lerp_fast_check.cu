// Host check of smp::lerp_fast and smp::scale_exact (csrc/sampling.cuh):
// the integer-pipe shortcuts for the fractions 0, 1/2 and 1 must give the
// bits of the reference's lerp, (1 - f) * a + f * b, and the exponent add
// the bits of the FP64 product x * 2^k, for random values and random bit
// patterns (zeros of both signs, subnormals, values whose halves are
// subnormal, infinities, NaN, values near overflow). Built and run by
// tests/test_native.py with FP contraction off, like the reference.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <random>

#include "sampling.cuh"

using namespace jg::smp;

int main() {
    std::mt19937_64 g(7);
    long bad = 0, n = 0;
    auto bits = [](double x) {
        unsigned long long b;
        std::memcpy(&b, &x, 8);
        return b;
    };
    auto check = [&](double a, double b, double f) {
        volatile double va = a, vb = b, vf = f;
        const double r = lerp_ref(va, vb, vf);
        const double q = lerp_fast(a, b, f, bits(f));
        ++n;
        const bool same = bits(r) == bits(q) || (std::isnan(r) && std::isnan(q));
        if (!same) {
            if (bad < 10)
                std::printf("a=%.17g b=%.17g f=%.17g ref=%.17g fast=%.17g\n", a,
                            b, f, r, q);
            ++bad;
        }
    };
    const double special[] = {0.0, -0.0, 1e-310, -1e-310, 4.9e-324,
                              2.2250738585072014e-308, -2.2250738585072014e-308,
                              4.450147717014403e-308, 1.0, -1.0, 0.5, 1e308,
                              -1e308, 1.7976931348623157e308, INFINITY,
                              -INFINITY, NAN, 3.0, -7.25, 1e-300};
    const double fracs[] = {0.0, 0.5, 1.0, 0.25, 0.75, 1e-17, 0.4999999999999999};
    for (double a : special)
        for (double b : special)
            for (double f : fracs) check(a, b, f);
    std::uniform_real_distribution<double> U(-10, 10);
    for (int t = 0; t < 300000; ++t) {
        const double a = U(g), b = U(g);
        check(a, b, 0.0);
        check(a, b, 0.5);
        check(a, b, 1.0);
        check(a, b, std::fabs(U(g)) / 10.0);
    }
    for (int t = 0; t < 300000; ++t) {  // random bit patterns
        const unsigned long long x = g(), y = g();
        double a, b;
        std::memcpy(&a, &x, 8);
        std::memcpy(&b, &y, 8);
        check(a, b, 0.0);
        check(a, b, 0.5);
        check(a, b, 1.0);
    }
    for (int t = 0; t < 300000; ++t) {  // cancellation near the subnormal edge
        const double a = std::ldexp(1.0 + U(g) / 20.0, -1020 - (int)(g() % 4));
        const double b = -a * (1.0 + std::ldexp(U(g), -40));
        check(a, b, 0.5);
        check(b, a, 0.5);
    }
    // scale_exact(x, k, 2^k) against the FP64 product x * 2^k.
    auto check_scale = [&](double x, int k) {
        volatile double vx = x, vs = std::ldexp(1.0, k);
        const double r = vx * vs;
        const double q = scale_exact(x, k, std::ldexp(1.0, k));
        ++n;
        if (!(bits(r) == bits(q) || (std::isnan(r) && std::isnan(q)))) {
            if (bad < 10)
                std::printf("scale x=%.17g k=%d ref=%.17g fast=%.17g\n", x, k, r, q);
            ++bad;
        }
    };
    for (int k = -30; k <= 30; ++k) {
        for (double x : special) check_scale(x, k);
        for (int t = 0; t < 20000; ++t) {
            const unsigned long long y = g();
            double x;
            std::memcpy(&x, &y, 8);
            check_scale(x, k);
            check_scale(U(g), k);
            check_scale(std::ldexp(U(g), -1015 - (int)(g() % 12)), k);
        }
    }
    std::printf("checked %ld, mismatches %ld\n", n, bad);
    return bad != 0;
}
