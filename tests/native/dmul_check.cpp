// Checks bs2e::dmul_int against the IEEE 754 double multiply of the host:
// random significands over the whole exponent range the fast path takes,
// significands with few bits set (products that land exactly halfway between
// two doubles, where round-to-nearest-even decides), and inputs the fast path
// hands to the FP64 multiply (zero, subnormal, negative, overflow, underflow).
// Prints the number of mismatches and exits 1 if there is any.
#include <cstdio>
#include <cstring>
#include <random>

#include "../../b-spline-two-e_gb300/csrc/bs2e_dmul.h"

static uint64_t bits(double x) {
    uint64_t u;
    std::memcpy(&u, &x, 8);
    return u;
}
static double make(uint64_t e, uint64_t frac) {
    uint64_t u = (e << 52) | (frac & 0x000FFFFFFFFFFFFFull);
    double x;
    std::memcpy(&x, &u, 8);
    return x;
}

int main(int argc, char **argv) {
    long n = argc > 1 ? std::atol(argv[1]) : 20000000;
    std::mt19937_64 rng(12345);
    long bad = 0, checked = 0;
    auto check = [&](double x, double y) {
        volatile double a = x, b = y;
        const double want = a * b, got = bs2e::dmul_int(x, y);
        ++checked;
        if (bits(want) != bits(got) && !(want != want && got != got)) {
            if (bad < 10)
                std::printf("mismatch: %a * %a = %a, got %a\n", x, y, want, got);
            ++bad;
        }
    };
    for (long i = 0; i < n; ++i) {
        const uint64_t e1 = 1 + rng() % 2046, e2 = 1 + rng() % 2046;
        check(make(e1, rng()), make(e2, rng()));
        // exponents near 1023 (the range the R^k totals use) and few-bit significands
        const uint64_t f1 = rng() & (rng() | 0xFFF0000000000ull), f2 = 1ull << (rng() % 52);
        check(make(900 + rng() % 250, f1), make(900 + rng() % 250, f2 | (rng() & 0xF)));
    }
    // exact halfway products: (1 + 2^-52) * (1 + 2^-1), (1 + 3*2^-52) * 1.5, ...
    for (uint64_t a = 1; a < 4096; ++a)
        for (uint64_t b = 0; b < 52; ++b) {
            check(make(1023, a), make(1023, 1ull << b));
            check(make(1023, 0x000FFFFFFFFFFFFFull - a), make(1023, (1ull << b) | 1));
        }
    const double odd[] = {0.0, -1.5, 4.9e-324, 2.2250738585072014e-308, 1e308, 1e-308, 3.0,
                          -0.0, 1.0 / 0.0};
    for (double x : odd)
        for (double y : odd) check(x, y);
    // split_scaled against the FP64 conversions it replaces
    long sbad = 0, schecked = 0;
    auto fb = [](float f) {
        uint32_t u;
        std::memcpy(&u, &f, 4);
        return u;
    };
    auto check_split = [&](double v, int s) {
        volatile double vv = v;
        const double x = vv * make((uint64_t)(1023 + s), 0);
        const float hi_w = (float)x, lo_w = (float)(x - (double)hi_w);
        float hi, lo;
        bs2e::split_scaled(v, s, hi, lo);
        ++schecked;
        if (fb(hi) != fb(hi_w) || fb(lo) != fb(lo_w)) {
            if (sbad < 10)
                std::printf("split mismatch: v=%a s=%d want (%a, %a) got (%a, %a)\n", v, s,
                            (double)hi_w, (double)lo_w, (double)hi, (double)lo);
            ++sbad;
        }
    };
    for (long i = 0; i < n / 2; ++i) {
        const int s = (int)(rng() % 401) - 200;
        check_split(make(1023 + (int64_t)(rng() % 401) - 200, rng()), s);
        // few-bit significands: dropped parts exactly half, zero remainders
        check_split(make(1023 + (int64_t)(rng() % 301) - 150, rng() & (0xFFFFFull << (rng() % 33))), s);
        // far below the scale: hi and lo near or below the float normal range
        check_split(make(1023 - 120 - (int64_t)(rng() % 40), rng()), 0);
    }
    check_split(0.0, 17);
    check_split(1e-320, 50);
    std::printf("%ld products checked, %ld mismatches\n", checked, bad);
    std::printf("%ld splits checked, %ld mismatches\n", schecked, sbad);
    return (bad || sbad) ? 1 : 0;
}
