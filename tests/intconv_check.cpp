// Checks the integer-pipe conversions (fauxgl_gb300/csrc/fgc_intconv.cuh)
// against the C library's FP64 results on seeded values around every edge:
// zeros, subnormals, |f| < 1, halves, binade boundaries, 2^52/2^53, +-2^63,
// infinities and NaN. Prints "ok <cases>" or the first mismatch.
// Build: g++ -O2 -ffp-contract=off -std=c++17 intconv_check.cpp
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cfloat>
#include <cstring>
#include <initializer_list>

#include "../fauxgl_gb300/csrc/fgc_intconv.cuh"

static uint64_t g_state = 0xD1B54A32D192ED03ull;
static uint64_t next64() {
    uint64_t z = (g_state += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
static double from_bits(uint64_t b) {
    double d;
    memcpy(&d, &b, 8);
    return d;
}
static int64_t ref_f2i(double f) {  // Go's int(f) on amd64
    if (f >= -9223372036854775808.0 && f < 9223372036854775808.0) return (int64_t)f;
    return INT64_MIN;
}

static int check(double f, uint64_t* n) {
    (*n)++;
    if (fgc::go_f2i_i(f) != ref_f2i(f)) {
        printf("f2i %a: %lld vs %lld\n", f, (long long)fgc::go_f2i_i(f), (long long)ref_f2i(f));
        return 1;
    }
    if (fgc::go_floor_i(f) != ref_f2i(std::floor(f))) {
        printf("floor %a: %lld vs %lld\n", f, (long long)fgc::go_floor_i(f), (long long)ref_f2i(std::floor(f)));
        return 1;
    }
    if (fgc::go_ceil_i(f) != ref_f2i(std::ceil(f))) {
        printf("ceil %a: %lld vs %lld\n", f, (long long)fgc::go_ceil_i(f), (long long)ref_f2i(std::ceil(f)));
        return 1;
    }
    if (fgc::ic_lt0(f) != (f < 0) || fgc::ic_gt0(f) != (f > 0)) {
        printf("sign %a\n", f);
        return 1;
    }
    if (std::isfinite(f)) {  // f32_trunc_pos of |f|: toward zero, 0 below FLT_MIN, FLT_MAX above it
        const double a = std::fabs(f);
        float want;
        if (a < (double)FLT_MIN) want = 0.0f;
        else if (a >= (double)FLT_MAX) want = FLT_MAX;
        else {
            want = (float)a;
            if ((double)want > a) want = std::nextafter(want, 0.0f);
        }
        uint64_t ab;
        memcpy(&ab, &a, 8);
        const float got = fgc::f32_trunc_pos(ab);
        if (got != want) {
            printf("f32_trunc_pos %a: %a vs %a\n", a, (double)got, (double)want);
            return 1;
        }
    }
    if (std::isfinite(f) && std::fabs(f) < 9007199254740992.0 && f == std::trunc(f)) {
        const int64_t v = (int64_t)f;
        const double d = fgc::i2d_i(v);
        uint64_t a, b;
        const double r = (double)v;
        memcpy(&a, &d, 8);
        memcpy(&b, &r, 8);
        if (a != b) {
            printf("i2d %lld\n", (long long)v);
            return 1;
        }
    }
    return 0;
}

int main(int argc, char** argv) {
    const uint64_t cases = argc > 1 ? strtoull(argv[1], nullptr, 10) : 200000;
    uint64_t n = 0;
    const double special[] = {0.0, -0.0, 0.5, -0.5, 1.0, -1.0, 1.5, -1.5, 2.5, -2.5, 4503599627370495.5,
                              -4503599627370495.5, 4503599627370496.0, 9007199254740991.0, 9007199254740992.0,
                              9223372036854775808.0, -9223372036854775808.0, 9223372036854774784.0,
                              -9223372036854774784.0, 1e300, -1e300, INFINITY, -INFINITY, NAN, -NAN,
                              from_bits(1), from_bits(0x8000000000000001ull), from_bits(0x000fffffffffffffull),
                              0.9999999999999999, -0.9999999999999999, 1.0000000000000002};
    for (double f : special)
        if (check(f, &n)) return 1;
    for (int e = -1100; e <= 1100; e++)
        for (int k = -2; k <= 2; k++) {
            const double f = std::ldexp(1.0, e);
            for (double g : {f, -f, std::nextafter(f, 0.0), -std::nextafter(f, 0.0), std::nextafter(f, INFINITY)})
                if (check(g + k * 0.0, &n)) return 1;
        }
    for (uint64_t i = 0; i < cases; i++) {
        const uint64_t r = next64();
        double f;
        switch (r % 4) {
            case 0: f = from_bits(next64()); break;                                    // any pattern
            case 1: f = std::ldexp((double)(int64_t)(next64() >> 11) - 4.5e15, -(int)(r >> 8 & 63)); break;
            case 2: f = std::floor(((double)(next64() >> 11) - 4.5e15) / 1024.0) + ((r >> 9) & 1 ? 0.5 : 0.0); break;
            default: f = ((double)(int64_t)next64()) * 1.0; break;                     // near +-2^63
        }
        if (check(f, &n)) return 1;
    }
    printf("ok %llu\n", (unsigned long long)n);
    return 0;
}
