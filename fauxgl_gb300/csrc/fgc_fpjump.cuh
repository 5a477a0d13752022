// fgc_fpjump.cuh -- the k-fold serial FP64 sum in O(binades) steps.
//
// rasterize (context.go:184-278) builds every edge value by repeated
// addition: w += a once per pixel along a row, w00 += b12 once per row. The
// result after k steps, t_k = RN(t_{k-1} + a), depends on every rounding on
// the way, so it is not s + k*a. It can still be computed without k steps:
// while t stays in one binade [2^E, 2^(E+1)) of width ulp u = 2^(E-52), t is
// a multiple of u and t + a = (m + q + f) u with integer m = t/u, q and
// fraction f of a/u fixed; round-to-nearest-even adds the same integer
// q + round(f) every step (a tie, |f| = 1/2, settles after one step on the
// even neighbour and then adds a constant too). So the sequence moves
// through a binade with one integer multiply-add, and real FP64 adds are
// only taken where it crosses into another binade (or near zero, or when
// |a| is not below the binade). repeat_add returns exactly the bits of the
// k-step loop, for every input including signed zeros, subnormals,
// infinities and NaN (the last three by plain steps).
//
// Host and device share this code: tests compare it with the plain loop.
#pragma once

#include <stdint.h>
#include <string.h>

#ifdef __CUDACC__
#define FGC_HD __host__ __device__ __forceinline__
#else
#define FGC_HD inline
#endif

namespace fgc {

// The bit pattern of x. On the device it passes through an opaque move:
// given a plain bit cast, the compiler turns masks, sign flips and compares of
// the bits back into FP64 abs, negate and NaN tests (DADD / DSETP), which
// issue on the FP64 pipe at the FP64 rate -- the pipe these helpers keep free.
FGC_HD uint64_t fj_bits(double x) {
#ifdef __CUDA_ARCH__
    unsigned long long b;
    asm("mov.b64 %0, %1;" : "=l"(b) : "d"(x));
    return (uint64_t)b;
#else
    uint64_t b;
    memcpy(&b, &x, 8);
    return b;
#endif
}

FGC_HD double fj_double(uint64_t b) {
#ifdef __CUDA_ARCH__
    double x;
    asm("mov.b64 %0, %1;" : "=d"(x) : "l"((unsigned long long)b));
    return x;
#else
    double x;
    memcpy(&x, &b, 8);
    return x;
#endif
}

FGC_HD double fj_add(double x, double y) {
#ifdef __CUDA_ARCH__
    return __dadd_rn(x, y);
#else
    volatile double r = x + y;  // one IEEE binary64 round-to-nearest add
    return r;
#endif
}

// Whether x * y <= z, without overflow.
FGC_HD bool fj_mul_fits(uint64_t x, uint64_t y, uint64_t z) {
#ifdef __CUDA_ARCH__
    return __umul64hi(x, y) == 0 && x * y <= z;
#else
    return (unsigned __int128)x * y <= z;
#endif
}

// t = s; repeat k times: t = RN(t + a). Returns t.
FGC_HD double repeat_add(double s, double a, uint64_t k) {
    const uint64_t kSign = 0x8000000000000000ull;
    const uint64_t kExp = 0x7ff0000000000000ull;
    const uint64_t kFrac = 0x000fffffffffffffull;
    const uint64_t kHidden = 0x0010000000000000ull;  // 2^52
    const uint64_t kTop = 0x0020000000000000ull;     // 2^53
    const uint64_t ab = fj_bits(a);
    if ((ab & kExp) == kExp || (ab << 1) == 0) {
        // a infinite, NaN or zero: one step reaches a fixed point
        return k ? fj_add(s, a) : s;
    }
    const int ea = (int)((ab >> 52) & 0x7ff);
    const uint64_t Ma = (ab & kFrac) | (ea ? kHidden : 0);
    while (k > 0) {
        s = fj_add(s, a);  // a real step: enters the binade the model then covers
        k--;
        if (k == 0) break;
        const uint64_t sb = fj_bits(s);
        if ((sb & kExp) == kExp) return s;  // infinite or NaN: fixed from here
        const int es = (int)((sb >> 52) & 0x7ff);
        if (es == 0) continue;              // zero or subnormal: plain steps
        if (ea >= es) continue;             // |a| not below the binade: plain steps
        // work on |t|: it grows when t and a have the same sign
        const bool grow = ((sb ^ ab) & kSign) == 0;
        uint64_t m = (sb & kFrac) | kHidden;  // |t| / u, in [2^52, 2^53)
        // shrinking from the binade's first value leaves it (finer spacing
        // below): plain steps
        if (!grow && m <= kHidden + 1) continue;
        const int sh = es - (ea ? ea : 1);  // a/u = Ma / 2^sh
        if (sh <= 0) continue;              // (smallest binade, subnormal a)
        if (sh >= 54) return s;             // |a| < u/2: t + a rounds back to t
        const uint64_t q = Ma >> sh;
        const uint64_t rem = Ma & ((1ull << sh) - 1);
        const uint64_t half = 1ull << (sh - 1);
        uint64_t d;                           // |t| changes by d (in units of u) per step
        if (rem != half) {
            d = q + (rem > half ? 1 : 0);
        } else {
            // tie: the even neighbour. m + q and m - q have the parity of
            // m + q; once m is even (after one tie step) d is constant.
            if ((m & 1) != 0) continue;
            d = q + (q & 1);
        }
        if (d == 0) return s;               // t + a rounds back to t from here on
        // steps that keep every exact sum (before rounding) inside the
        // binade, with one unit of margin at both ends
        uint64_t avail;  // n steps fit when (n - 1) * d <= avail
        if (grow) {
            const uint64_t lim = kTop - 2;  // m_i + q <= 2^53 - 2
            if (m + q > lim) continue;
            avail = lim - m - q;
        } else {
            const uint64_t lim = kHidden + 1;  // m_i - q >= 2^52 + 1
            if (m < q + lim) continue;
            avail = m - q - lim;
        }
        // all k remaining steps usually fit: only a jump that reaches the
        // binade's end needs the division
        const uint64_t n = fj_mul_fits(k - 1, d, avail) ? k : avail / d + 1;
        m = grow ? m + n * d : m - n * d;
        k -= n;
        s = fj_double((sb & kSign) | ((uint64_t)es << 52) | (m - kHidden));
    }
    return s;
}

}  // namespace fgc
