// Host check of smp::bary_bits and smp::bary_bits2 (csrc/sampling.cuh): the
// integer-pipe barycentric split must give the same (index, fraction, and
// for bary_bits2 one minus the fraction) bits as the FP64
// form of getBarycentric (include/jet/detail/math_utils-inl.h:147-172) for
// random values, random bit patterns (negatives, NaN, infinities,
// subnormals), integers and their neighbours, and sample coordinates of the
// kind the transfers produce. Built and run by tests/test_native.py.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <random>

#include "sampling.cuh"

using namespace jg::smp;

// getBarycentric with an FP64 floor; an int conversion of NaN gives 0, as
// the GPU's does.
static void reference(double x, int iHigh, int* i, double* f) {
    const double s = std::floor(x);
    if (iHigh == 0) {
        *i = 0;
        *f = 0.0;
    } else if (s < 0.0) {
        *i = 0;
        *f = 0.0;
    } else if (s > (double)(iHigh - 1)) {
        *i = iHigh - 1;
        *f = 1.0;
    } else {
        *i = std::isnan(s) ? 0 : (int)s;
        *f = x - s;
    }
}

int main() {
    std::mt19937_64 g(1);
    long bad = 0, n = 0;
    auto check = [&](double x, int ih) {
        int i1, i2, i3;
        double f1, f2, f3, g3;
        reference(x, ih, &i1, &f1);
        bary_bits(x, ih, &i2, &f2);
        bary_bits2(x, ih, &i3, &f3, &g3);
        const double g1 = 1 - f1;
        auto same = [](double a, double b) {
            unsigned long long ba, bb;
            std::memcpy(&ba, &a, 8);
            std::memcpy(&bb, &b, 8);
            return ba == bb || (std::isnan(a) && std::isnan(b));
        };
        ++n;
        if (i1 != i2 || !same(f1, f2) || i1 != i3 || !same(f1, f3) ||
            !same(g1, g3)) {
            if (bad < 10)
                std::printf("x=%.17g iHigh=%d reference (%d, %.17g, %.17g) "
                            "bits (%d, %.17g) bits2 (%d, %.17g, %.17g)\n",
                            x, ih, i1, f1, g1, i2, f2, i3, f3, g3);
            ++bad;
        }
    };
    const int highs[] = {0, 1, 2, 3, 7, 16, 64, 255, 256, 257, 512, 1023,
                         4096, 100000, 1 << 30};
    std::uniform_real_distribution<double> U(-3, 600);
    for (int ih : highs) {
        for (int t = 0; t < 100000; ++t) check(U(g), ih);
        for (int t = 0; t < 50000; ++t) {
            const unsigned long long b = g();
            double x;
            std::memcpy(&x, &b, 8);
            check(x, ih);
        }
        for (int k = -3; k < 600; ++k) {
            const double x = k;
            check(x, ih);
            check(std::nextafter(x, 1e300), ih);
            check(std::nextafter(x, -1e300), ih);
            check(x + 0.5, ih);
            check(x * 0.999999999, ih);
        }
        const double special[] = {0.0, -0.0, 1e-310, -1e-310, NAN, -NAN,
                                  INFINITY, -INFINITY, 4.9e-324,
                                  2147483647.5, 1e300};
        for (double x : special) check(x, ih);
        for (int t = 0; t < 50000; ++t) {
            const double p = U(g) / 512.0;
            check((p - 0.5 / 256) * 256.0, ih);
        }
    }
    std::printf("checked %ld, mismatches %ld\n", n, bad);
    return bad != 0;
}
