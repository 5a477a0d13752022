// Checks fgc::repeat_add (fauxgl_gb300/csrc/fgc_fpjump.cuh) against the plain
// loop t = t + a, k times, bit for bit, on seeded cases chosen to cross
// binades, hit round-to-nearest ties, cross zero, and use subnormals,
// infinities and NaN. Prints "ok <cases>" or the first mismatch.
// Build: g++ -O2 -ffp-contract=off -std=c++17 fpjump_check.cpp
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "../fauxgl_gb300/csrc/fgc_fpjump.cuh"

static uint64_t g_state = 0x9E3779B97F4A7C15ull;
static uint64_t next64() {  // splitmix64
    uint64_t z = (g_state += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
static double uni() { return (next64() >> 11) * (1.0 / 9007199254740992.0); }
static int irange(int lo, int hi) { return lo + (int)(next64() % (uint64_t)(hi - lo + 1)); }

static double serial(double s, double a, uint64_t k) {
    volatile double t = s;
    for (uint64_t i = 0; i < k; i++) t = t + a;
    return t;
}

static double pick_value(int scale_lo, int scale_hi) {
    switch (irange(0, 9)) {
    case 0: {  // few significant bits (ties)
        double m = (double)irange(1, 63);
        return (next64() & 1 ? -1 : 1) * std::ldexp(m, irange(scale_lo, scale_hi));
    }
    case 1:  // a power of two
        return (next64() & 1 ? -1 : 1) * std::ldexp(1.0, irange(scale_lo, scale_hi));
    case 2: {  // subnormal or tiny
        uint64_t b = next64() & 0x000fffffffffffffull;
        if (next64() & 1) b |= 0x8000000000000000ull;
        double x;
        memcpy(&x, &b, 8);
        return x;
    }
    default:
        return (next64() & 1 ? -1 : 1) * std::ldexp(0.5 + 0.5 * uni(), irange(scale_lo, scale_hi));
    }
}

int main(int argc, char** argv) {
    const long cases = argc > 1 ? atol(argv[1]) : 1000000;
    long n = 0;
    const double specials[] = {0.0, -0.0, INFINITY, -INFINITY, NAN, 1e308, -1e308, 4.9e-324, -4.9e-324,
                               2.2250738585072014e-308};
    for (long c = 0; c < cases; c++) {
        double s, a;
        uint64_t k;
        const int mode = irange(0, 9);
        if (mode == 0) {  // specials on either side
            s = next64() & 1 ? specials[irange(0, 9)] : pick_value(-20, 20);
            a = next64() & 1 ? specials[irange(0, 9)] : pick_value(-20, 20);
            k = irange(0, 50);
        } else if (mode == 1) {  // walk through zero from a multiple of a
            a = pick_value(-8, 4);
            s = -a * irange(1, 600) + (next64() & 1 ? 0.0 : pick_value(-30, -10));
            k = irange(0, 1500);
        } else if (mode == 2) {  // a tiny relative to s (fixed points, ties at u/2)
            s = pick_value(-5, 30);
            a = std::ldexp(s, -irange(40, 60)) * (next64() & 1 ? -1 : 1);
            if (next64() & 1) a = std::ldexp(1.0, std::ilogb(s) - 53) * (next64() & 1 ? -1 : 1);
            k = irange(0, 3000);
        } else if (mode == 3) {  // long runs, many binades
            s = pick_value(-30, 10);
            a = pick_value(-12, 2);
            k = irange(1000, 20000);
        } else {  // edge-function-like magnitudes
            s = pick_value(-4, 20);
            a = pick_value(-6, 6);
            k = irange(0, 2500);
        }
        const double want = serial(s, a, k);
        const double got = fgc::repeat_add(s, a, k);
        uint64_t wb, gb;
        memcpy(&wb, &want, 8);
        memcpy(&gb, &got, 8);
        const bool both_nan = std::isnan(want) && std::isnan(got);
        if (wb != gb && !both_nan) {
            printf("mismatch s=%a a=%a k=%llu want=%a got=%a\n", s, a, (unsigned long long)k, want, got);
            return 1;
        }
        n++;
    }
    printf("ok %ld\n", n);
    return 0;
}
