// Host check of the double <-> double-float conversions of ig_arith.cuh (the
// same inline code the kernels run), compiled with g++ by test_arith_host.py.
// Prints one line per check: "<name> <max error> <limit>"; the test compares.
#include "../impulse_gb300/csrc/ig_arith.cuh"

#include <cmath>
#include <cstdio>
#include <initializer_list>
#include <random>

using namespace ig;

static long double lexp2(int e) { return std::ldexp(1.0L, e); }

int main()
{
    std::mt19937_64 g(7);
    std::uniform_real_distribution<double> U(-1, 1);
    // double -> df -> value, with line scales inside and outside the hoisted window,
    // inputs across the whole double range that the scale brings near 1 (subnormals included)
    for (int es : {-1020, -1003, -896, -500, 0, 500, 919, 920, 990, 1003, 1060}) {
        long double worst = 0;
        for (int t = 0; t < 20000; ++t) {
            const double x = U(g) * std::ldexp(1.0, -es + (int)(g() % 40) - 20);
            if (x == 0.0 || !std::isfinite(x)) continue;
            const df d = df_from_double(x, es);
            const long double back = ((long double)d.h + (long double)d.l) * lexp2(-es);
            const long double r = fabsl((back - x) / x);
            if (r > worst) worst = r;
        }
        std::printf("from_double_es%d %.3Le %.3e\n", es, worst, std::ldexp(1.0, -46));
    }
    // zeros stay zeros (signed) at every scale; infinities and NaN map through
    int bad = 0;
    for (int es : {-1100, -900, 0, 900, 990, 1100}) {
        const df z = df_from_double(0.0, es), nz = df_from_double(-0.0, es);
        bad += !(z.h == 0.0f && z.l == 0.0f && !std::signbit(z.h));
        bad += !(nz.h == 0.0f && nz.l == 0.0f && std::signbit(nz.h));
        bad += !std::isinf(df_from_double(INFINITY, es).h);
        bad += !std::isnan(df_from_double(NAN, es).h);
    }
    std::printf("specials %d 0\n", bad);
    // df -> double with scales: normal results to 1 ulp, subnormal results to half a subnormal step
    for (int es : {-1000, -896, 0, 896, 990, 1000, 1010}) {
        long double worst = 0;
        for (int t = 0; t < 20000; ++t) {
            const float h = (float)(U(g) * std::ldexp(1.0, (int)(g() % 12) - 6));
            const float l = (float)(U(g) * std::ldexp((double)std::fabs(h), -25));
            const df d{h, l};
            const long double exact = ((long double)d.h + (long double)d.l) * lexp2(-es);
            if (exact == 0) continue;
            const double got = df_to_double(d, es);
            const long double step = fabsl(exact) < lexp2(-1022) ? lexp2(-1074) : fabsl(exact) * lexp2(-52);
            const long double r = fabsl(got - exact) / step;
            if (r > worst) worst = r;
        }
        std::printf("to_double_es%d %.3Le %.3e\n", es, worst, 1.0);
    }
    // exact ties round to even, on the general path (scales outside the hoisted
    // window): a normal result and a subnormal one
    {
        int tbad = 0;
        // (1 + 2^-53) 2^-1000: halfway between 2^-1000 and its successor -> 2^-1000
        tbad += df_to_double(df{1.0f, std::ldexp(1.0f, -53)}, 1000) != std::ldexp(1.0, -1000);
        // (1 + 3 2^-53) 2^-1000: halfway, odd below -> rounds up to (1 + 2^-51) 2^-1000
        tbad += df_to_double(df{1.0f, 3.0f * std::ldexp(1.0f, -53)}, 1000) != std::ldexp(1.0 + std::ldexp(1.0, -51), -1000);
        // (1 + 2^-24) 2^-1051 = (2^23 + 1/2) 2^-1074: subnormal tie -> 2^23 2^-1074
        tbad += df_to_double(df{1.0f, std::ldexp(1.0f, -24)}, 1051) != std::ldexp(1.0, -1051);
        // (1 + 3 2^-24) 2^-1051 = (2^23 + 3/2) 2^-1074 -> (2^23 + 2) 2^-1074
        tbad += df_to_double(df{1.0f, 3.0f * std::ldexp(1.0f, -24)}, 1051) != std::ldexp(8388610.0, -1074);
        // negative subnormal tie
        tbad += df_to_double(df{-1.0f, -std::ldexp(1.0f, -24)}, 1051) != -std::ldexp(1.0, -1051);
        std::printf("ties_to_even %d 0\n", tbad);
    }
    return 0;
}
