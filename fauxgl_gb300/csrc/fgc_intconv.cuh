// fgc_intconv.cuh -- Go's float64 -> int conversions, floor/ceil to int and
// small int -> float64 on the integer pipe.
//
// GB300 runs FP64 compares, conversions and rounding on the FP64 pipe at the
// FP64 rate; these bit-level versions return exactly what the FP64
// instructions would and leave that pipe to the arithmetic. Host and device
// share the code: tests/intconv_check.cpp compares it with the C library on
// the host.
#pragma once

#include "fgc_fpjump.cuh"  // FGC_HD, fj_bits, fj_double

namespace fgc {

FGC_HD bool ic_nan(uint64_t b) { return (b & 0x7fffffffffffffffull) > 0x7ff0000000000000ull; }
// x < 0 and x > 0 (NaN and signed zeros: false).
FGC_HD bool ic_lt0(double x) {
    const uint64_t b = fj_bits(x);
    return (b >> 63) != 0 && (b & 0x7fffffffffffffffull) != 0 && !ic_nan(b);
}
FGC_HD bool ic_gt0(double x) {
    const uint64_t b = fj_bits(x);
    return (b >> 63) == 0 && b != 0 && !ic_nan(b);
}

// int(f) on amd64 (CVTTSD2SQ): truncation toward zero; NaN and values outside
// [-2^63, 2^63) give INT64_MIN.
FGC_HD int64_t go_f2i_i(double f) {
    const uint64_t b = fj_bits(f);
    const int e = (int)((b >> 52) & 0x7ff);
    if (e < 1023) return 0;                 // |f| < 1
    if (e >= 1023 + 63) return INT64_MIN;   // |f| >= 2^63, Inf, NaN (-2^63 itself is INT64_MIN)
    const uint64_t m = (b & 0x000fffffffffffffull) | 0x0010000000000000ull;
    const int sh = e - 1075;
    const uint64_t mag = sh >= 0 ? (m << sh) : (m >> -sh);
    return (b >> 63) ? -(int64_t)mag : (int64_t)mag;
}

// Whether a finite f has a non-zero fractional part.
FGC_HD bool ic_frac(double f) {
    const uint64_t b = fj_bits(f);
    const int e = (int)((b >> 52) & 0x7ff);
    if (e < 1023) return (b & 0x7fffffffffffffffull) != 0;
    if (e >= 1075) return false;
    const uint64_t m = (b & 0x000fffffffffffffull) | 0x0010000000000000ull;
    return (m & ((1ull << (1075 - e)) - 1)) != 0;
}

// int(math.Floor(f)) and int(math.Ceil(f)), with int()'s out-of-range rule.
FGC_HD int64_t go_floor_i(double f) {
    const int64_t t = go_f2i_i(f);
    if (t == INT64_MIN) return t;
    return (ic_lt0(f) && ic_frac(f)) ? t - 1 : t;
}
FGC_HD int64_t go_ceil_i(double f) {
    const int64_t t = go_f2i_i(f);
    if (t == INT64_MIN) return t;
    return (ic_gt0(f) && ic_frac(f)) ? t + 1 : t;
}

// float32 of the bits b of a non-negative finite float64, rounded toward
// zero: 0 below the smallest normal float32, the largest float32 above it.
// An operand of estimates, not a conversion of record.
FGC_HD float f32_trunc_pos(uint64_t b) {
    const int e = (int)(b >> 52) - 1023 + 127;
    uint32_t f;
    if (e <= 0) f = 0u;
    else if (e >= 255) f = 0x7f7fffffu;
    else f = ((uint32_t)e << 23) | (uint32_t)((b >> 29) & 0x7fffffu);
#ifdef __CUDA_ARCH__
    return __uint_as_float(f);
#else
    float r;
    memcpy(&r, &f, 4);
    return r;
#endif
}

// float64(v), exact for |v| < 2^53.
FGC_HD double i2d_i(int64_t v) {
    if (v == 0) return 0.0;
    const uint64_t sgn = v < 0 ? 0x8000000000000000ull : 0ull;
    const uint64_t a = v < 0 ? (uint64_t)(-v) : (uint64_t)v;
#ifdef __CUDA_ARCH__
    const int lz = __clzll((long long)a);
#else
    const int lz = __builtin_clzll(a);
#endif
    const int e = 63 - lz;  // a in [2^e, 2^(e+1)), e <= 52
    const uint64_t frac = (a << (52 - e)) & 0x000fffffffffffffull;
    return fj_double(sgn | ((uint64_t)(1023 + e) << 52) | frac);
}

}  // namespace fgc
