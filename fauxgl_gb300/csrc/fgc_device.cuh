// fgc_device.cuh -- device-side types and Go-semantics helpers shared by the
// kernels of libfauxglcuda.
//
// Every FP64 expression that feeds coverage, depth or (in the plain form)
// colour is written with explicit __dadd_rn / __dmul_rn / __dsub_rn in the
// reference's left-to-right order, and the library is compiled with
// --fmad=false, so no multiply-add is ever contracted: results are the
// reference's unfused IEEE binary64 results (Go on amd64 does not fuse).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/fauxglcuda.h"
#include "fgc_intconv.cuh"

namespace fgc {

// ---------------------------------------------------------------------------
// Launch-wide limits and status bits
// ---------------------------------------------------------------------------

// Device status word bits (a kernel that hits a bounded limit sets one and the
// host reports FGC_ERR_DEVICE_LIMIT or re-runs with larger buffers).
enum : uint32_t {
    ST_CLIP_OVERFLOW = 1u << 0,   // more clipped elements than the clip list holds
    ST_BIN_OVERFLOW = 1u << 1,    // more (prim, band) pairs than the bin array holds
    ST_LOOKBACK_TIMEOUT = 1u << 2,// a decoupled look-back wait gave up
    ST_POOL_OVERFLOW = 1u << 3,   // clip vertex pool too small
    ST_RASTER_INTERNAL = 1u << 4, // a raster invariant failed; the draw's output is not trusted
};

// Bounded spin: a look-back wait gives up after this many polls.
constexpr uint32_t kSpinLimit = 1u << 22;

// Element id flag for lines (winner ids): bit 31.
constexpr uint32_t kLineFlag = 0x80000000u;
// Vertex references: bit 31 set = index into the clip vertex pool.
constexpr uint32_t kPoolFlag = 0x80000000u;

// Vertex attributes a draw's shader reads (clipping interpolates only these).
enum : uint32_t { kAttrPos = 1, kAttrNrm = 2, kAttrTex = 4, kAttrCol = 8 };

// Primitive bounding boxes beyond these limits produce no fragments (the same
// rule as the oracle; the reference would loop ~2^63 times on them).
constexpr int64_t kMaxExtent = 67108864LL;  // 2^26

// ---------------------------------------------------------------------------
// Data layouts
// ---------------------------------------------------------------------------

// One raster primitive: a triangle handed to rasterize (context.go:151) after
// setup. Holds exactly the per-triangle values rasterize computes before its
// row loop, so the raster stage never recomputes them.
struct __align__(16) RPrim {
    double w0, w1, w2;     // w00, w01, w02: edge values at (x0+.5, y0+.5)
    double a0, a1, a2;     // a12, a20, a01: per-pixel increments
    double b0, b1, b2;     // b12, b20, b01: per-row increments
    double ra;             // 1 / edge(s0, s1, s2)
    double q0, q1, q2;     // ra12, ra20, ra01
    double z0, z1, z2;     // s0.Z, s1.Z, s2.Z
    double r0, r1, r2;     // 1 / Output.W of v0, v1, v2
    uint32_t v0, v1, v2;   // vertex attribute references
    uint32_t elem;         // element id (triangle index, or kLineFlag | line index)
};
static_assert(sizeof(RPrim) == 168 + 8, "RPrim layout");

// Integer bounding box of a primitive (empty: x0 > x1).
struct __align__(16) PBox {
    int32_t x0, x1, y0, y1;
};

// Per-unique-vertex results of the vertex stage.
struct __align__(16) VClip {   // Output (clip space)
    double x, y, z, w;
};
struct __align__(16) VScreen { // Screen.MulPosition(ndc) and 1/W
    double x, y, z, rw;
};

// Per-corner attributes, FP64 (plain form) and FP32 (mixed form).
struct __align__(16) APosNrm64 { double px, py, pz, nx, ny, nz; };
struct __align__(16) APosNrm32 { float px, py, pz, nx, ny, nz; };

// A vertex of the clip pool (an InterpolateVertexes result), and its FP32
// copy for the mixed form.
struct __align__(16) PoolVertex {
    double px, py, pz, nx, ny, nz, tu, tv, cr, cg, cb, ca;
};
struct __align__(16) PoolVertex32 {
    float px, py, pz, nx, ny, nz, tu, tv, cr, cg, cb, ca;
};

// Device view of a mesh.
struct MeshView {
    uint64_t ntri, nline;
    uint64_t nuniq;             // unique positions
    const double* upos_x;       // unique positions, SoA
    const double* upos_y;
    const double* upos_z;
    const uint32_t* corner_uniq;// corner -> unique position index (3*ntri + 2*nline)
    const APosNrm64* pn64;      // per corner
    const double* tex64;        // per corner, 2 values, or null
    const double* col64;        // per corner, 4 values, or null
    const APosNrm32* pn32;
    const float* tex32;
    const float* col32;
};

// Texture view: 16-bit premultiplied RGBA texels.
struct TexView {
    const ushort4* texels;
    const double* unit64;  // per texel the four channels as float64(c) / 0xffff (the FP64 shaders' texel colour)
    int32_t w, h;
};

// Shader parameters on the device.
struct ShaderView {
    int32_t kind;
    int32_t has_texture;
    int32_t object_is_discard;  // PhongShader: ObjectColor == Discard
    int32_t power_pos;          // SpecularPower > 0 (the Fragment's test, made once)
    int32_t gray_light;         // AmbientColor and DiffuseColor each have equal R, G, B (bit for bit)
    int32_t gray_spec;          // SpecularColor has equal R, G, B
    double m[16];
    double color[4];
    double light[3];
    double eye[3];
    double ambient[4], diffuse[4], specular[4];
    double power;
    uint64_t pow_yi;            // SpecularPower when it is an integer in [2, 2^63), else 0
    TexView tex;
    // the same parameters in FP32 for the mixed form (converted once on the
    // host: a conversion from FP64 runs on the FP64 pipe)
    float color32[4];
    float light32[3];
    float eye32[3];
    float ambient32[4], diffuse32[4], specular32[4];
    float power32;
};

struct StateView {
    int32_t read_depth, write_depth, write_color, alpha_blend, wireframe, front_face, cull, precision;
    double line_width, depth_bias;
};

// ---------------------------------------------------------------------------
// Go semantics
// ---------------------------------------------------------------------------

// int(f) on amd64 (CVTTSD2SQ): truncation; NaN / out of range -> INT64_MIN.
__device__ __forceinline__ int64_t go_f2i(double f) {
    if (f >= -9223372036854775808.0 && f < 9223372036854775808.0) return (int64_t)f;
    return INT64_MIN;
}

// NaN, infinity and finiteness from the bits (fj_bits: integer pipe).
__device__ __forceinline__ bool dnan(double x) { return (fj_bits(x) & 0x7fffffffffffffffull) > 0x7ff0000000000000ull; }
__device__ __forceinline__ bool dinf(double x) { return (fj_bits(x) & 0x7fffffffffffffffull) == 0x7ff0000000000000ull; }
__device__ __forceinline__ bool dfinite(double x) {
    return (fj_bits(x) & 0x7fffffffffffffffull) < 0x7ff0000000000000ull;
}

// math.Min / math.Max (explicit special cases: CUDA's fmin/fmax drop NaN).
__device__ __forceinline__ double go_min(double x, double y) {
    if ((dinf(x) && x < 0) || (dinf(y) && y < 0)) return __longlong_as_double(0xfff0000000000000LL);
    if (dnan(x) || dnan(y)) return __longlong_as_double(0x7ff8000000000000LL);
    if (x == 0 && x == y) return signbit(x) ? x : y;
    return x < y ? x : y;
}
__device__ __forceinline__ double go_max(double x, double y) {
    if ((dinf(x) && x > 0) || (dinf(y) && y > 0)) return __longlong_as_double(0x7ff0000000000000LL);
    if (dnan(x) || dnan(y)) return __longlong_as_double(0x7ff8000000000000LL);
    if (x == 0 && x == y) return signbit(x) ? y : x;
    return x > y ? x : y;
}

__device__ __forceinline__ double go_clamp(double x, double lo, double hi) {
    if (x < lo) return lo;
    if (x > hi) return hi;
    return x;
}

// ---------------------------------------------------------------------------
// Exact IEEE predicates on the integer pipe. GB300 issues FP64 adds at ~1/38
// of its integer rate, so comparisons that decide coverage and Go's Min/Max
// special cases are made on the bit patterns; each helper returns exactly
// what the FP64 comparison would.
// ---------------------------------------------------------------------------
constexpr unsigned long long kAbsMask = 0x7fffffffffffffffull;
constexpr unsigned long long kInfBits = 0x7ff0000000000000ull;

__device__ __forceinline__ unsigned long long dbits(double x) { return (unsigned long long)fj_bits(x); }
__device__ __forceinline__ bool bnan(unsigned long long b) { return (b & kAbsMask) > kInfBits; }
// Total order on non-NaN doubles as unsigned keys (-0 sorts below +0).
__device__ __forceinline__ unsigned long long okey(unsigned long long b) {
    return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}

// math.Min / math.Max from the bits: -Inf (+Inf) wins, then NaN, then the
// total order, which also gives Go's signed-zero results.
__device__ __forceinline__ double go_min_i(double x, double y) {
    const unsigned long long bx = dbits(x), by = dbits(y);
    if (bx == 0xfff0000000000000ull || by == 0xfff0000000000000ull) return __longlong_as_double(0xfff0000000000000LL);
    if (bnan(bx) || bnan(by)) return __longlong_as_double(0x7ff8000000000000LL);
    return okey(bx) <= okey(by) ? x : y;
}
__device__ __forceinline__ double go_max_i(double x, double y) {
    const unsigned long long bx = dbits(x), by = dbits(y);
    if (bx == kInfBits || by == kInfBits) return __longlong_as_double(0x7ff0000000000000LL);
    if (bnan(bx) || bnan(by)) return __longlong_as_double(0x7ff8000000000000LL);
    return okey(bx) >= okey(by) ? x : y;
}
// math.Max(x, 0): NaN stays NaN, positive values stay, everything else is +0.
__device__ __forceinline__ double go_max0(double x) {
    const unsigned long long b = dbits(x);
    if (bnan(b)) return x;
    return ((b >> 63) == 0 && b != 0) ? x : 0.0;
}
// math.Min(x, 1): NaN stays NaN, values below 1 stay, the rest is 1.
__device__ __forceinline__ double go_min1(double x) {
    const unsigned long long b = dbits(x);
    if (bnan(b)) return x;
    return ((b >> 63) || b < 0x3ff0000000000000ull) ? x : 1.0;
}
// x == 0 (either sign).
__device__ __forceinline__ bool dzero(double x) { return (dbits(x) & kAbsMask) == 0; }
// 0 + x: x itself except that -0 becomes +0 (a NaN stays a NaN).
__device__ __forceinline__ double zero_plus(double x) { return dbits(x) == 0x8000000000000000ull ? 0.0 : x; }
// 2 * x (exact): one more in the exponent of a normal x below the top binade.
__device__ __forceinline__ double twice(double x) {
    const unsigned long long b = dbits(x), e = (b >> 52) & 0x7ff;
    if (e >= 1 && e <= 2045) return __longlong_as_double((long long)(b + (1ull << 52)));
    return __dmul_rn(2.0, x);
}
// x < 1 (NaN: false).
__device__ __forceinline__ bool dlt1(double x) {
    const unsigned long long b = dbits(x);
    if (bnan(b)) return false;
    return (b >> 63) || b < 0x3ff0000000000000ull;
}
// x > 0 (NaN and -0: false).
__device__ __forceinline__ bool dgt0(double x) {
    const unsigned long long b = dbits(x);
    return (b >> 63) == 0 && b != 0 && !bnan(b);
}
// x < 0 (NaN and -0: false).
__device__ __forceinline__ bool dlt0(double x) { return ic_lt0(x); }

// x > y and x <= y exactly as IEEE compares (NaN: false; -0 == +0).
__device__ __forceinline__ unsigned long long okey0(unsigned long long b) {
    return okey((b & kAbsMask) ? b : 0ull);
}
__device__ __forceinline__ bool dgt_i(double x, double y) {
    const unsigned long long bx = dbits(x), by = dbits(y);
    if (bnan(bx) || bnan(by)) return false;
    return okey0(bx) > okey0(by);
}
__device__ __forceinline__ bool dle_i(double x, double y) {
    const unsigned long long bx = dbits(x), by = dbits(y);
    if (bnan(bx) || bnan(by)) return false;
    return okey0(bx) <= okey0(by);
}
// z + bias, skipping the add for a bias of +0: z + (+0) is z, or +0 for
// z = -0, and every use compares it, where -0 and +0 are equal.
__device__ __forceinline__ double add_bias(double z, double bias, bool bias_zero) {
    return bias_zero ? z : __dadd_rn(z, bias);
}

// uint8(Clamp(c, 0, 1) * 255) (color.go:56-63): the clamp and the truncation
// on the integer pipe, the one multiply in FP64. NaN gives 0.
__device__ __forceinline__ uint32_t go_u8_of_unit_i(double c) {
    const unsigned long long b = dbits(c);
    if (bnan(b)) return 0;
    if ((b >> 63) || b == 0) return 0;                // c <= 0 (or -0)
    if (b >= 0x3ff0000000000000ull) return 255;       // c >= 1
    const double v = __dmul_rn(c, 255.0);             // (0, 255)
    const unsigned long long vb = dbits(v);
    const int e = (int)((vb >> 52) & 0x7ff) - 1023;   // v < 255 so e <= 7
    if (e < 0) return 0;
    const unsigned long long m = (vb & 0x000fffffffffffffull) | 0x0010000000000000ull;
    return (uint32_t)(m >> (52 - e));
}
__device__ __forceinline__ uint32_t nrgba_pack_i(double r, double g, double b, double a) {
    return go_u8_of_unit_i(r) | (go_u8_of_unit_i(g) << 8) | (go_u8_of_unit_i(b) << 16) | (go_u8_of_unit_i(a) << 24);
}

// w * ra < 0, for the coverage test of rasterize (context.go:208-215). When
// ra is finite-or-infinite, nonzero and at least 2^-511 in magnitude and
// |w| >= 2^-511, the product is a nonzero non-NaN number whose sign is the
// XOR of the signs, so the bits decide; w = ±0 gives ±0 (or NaN), never
// negative. Anything else (tiny or NaN w, unusual ra) takes the FP64 product.
struct RaSign {
    unsigned long long sign;
    bool simple;
};
__device__ __forceinline__ RaSign ra_sign(double ra) {
    const unsigned long long b = dbits(ra), m = b & kAbsMask;
    return RaSign{b >> 63, m >= 0x2000000000000000ull && m <= kInfBits};
}
__device__ __forceinline__ bool neg_product(double w, double ra, RaSign rs) {
    const unsigned long long b = dbits(w), m = b & kAbsMask;
    if (rs.simple) {
        if (m >= 0x2000000000000000ull && m <= kInfBits) return (b >> 63) != rs.sign;
        if (m == 0) return false;
    }
    return __dmul_rn(w, ra) < 0;
}

// uint8(clamp(c, 0, 1) * 255) (color.go:56-63); NaN gives 0.
__device__ __forceinline__ uint32_t go_u8_of_unit(double c) {
    double v = __dmul_rn(go_clamp(c, 0.0, 1.0), 255.0);
    return (uint32_t)(go_f2i(v) & 0xff);
}

__device__ __forceinline__ uint32_t nrgba_pack(double r, double g, double b, double a) {
    return go_u8_of_unit(r) | (go_u8_of_unit(g) << 8) | (go_u8_of_unit(b) << 16) | (go_u8_of_unit(a) << 24);
}

// The alpha-blend write of rasterize (context.go:256-267): the source is
// NRGBA().RGBA() (16-bit premultiplied), blended in uint32 arithmetic.
__device__ __forceinline__ uint32_t blend_nrgba(uint32_t dst, uint32_t src_nrgba) {
    uint32_t ca = src_nrgba >> 24;
    uint32_t out = 0;
#pragma unroll
    for (int k = 0; k < 4; k++) {
        uint32_t s;
        if (k < 3) {
            s = (src_nrgba >> (8 * k)) & 0xff;
            s |= s << 8;
            s *= ca;
            s /= 0xff;
        } else {
            s = ca | (ca << 8);
        }
        uint32_t sa = ca | (ca << 8);
        uint32_t a = (0xffffu - sa) * 0x101u;
        uint32_t d = (dst >> (8 * k)) & 0xff;
        uint32_t r = (d * a / 0xffffu + s) >> 8;
        out |= (r & 0xff) << (8 * k);
    }
    return out;
}

__device__ __forceinline__ bool go_is_odd_int(double x) {
    if (fabs(x) >= 9007199254740992.0) return false;
    double xi;
    double xf = modf(x, &xi);
    return xf == 0 && ((((int64_t)xi) & 1) == 1);
}

// math.Pow (Go math/pow.go): special cases; x**yi by repeated squaring of the
// Frexp mantissa with exact power-of-two renormalisation; x**yf through
// exp(yf*log(x)) (CUDA's exp/log here, the only step not bit-identical to
// Go's; it runs only for a fractional SpecularPower).
__device__ inline double go_pow(double x, double y) {
    const double INF = __longlong_as_double(0x7ff0000000000000LL);
    const double NAN_ = __longlong_as_double(0x7ff8000000000000LL);
    // Pow(-Inf, y) is evaluated as Pow(1/x, -y) = Pow(-0, -y): at most one
    // extra pass through the special cases.
    for (int pass = 0; pass < 2; pass++) {
        if (y == 0 || x == 1) return 1;
        if (y == 1) return x;
        if (dnan(x) || dnan(y)) return NAN_;
        if (x == 0) {
            if (y < 0) return (signbit(x) && go_is_odd_int(y)) ? -INF : INF;
            if (y > 0) return (signbit(x) && go_is_odd_int(y)) ? x : 0.0;
        }
        if (dinf(y)) {
            if (x == -1) return 1;
            if ((fabs(x) < 1) == (y > 0)) return 0;
            return INF;
        }
        if (dinf(x)) {
            if (x < 0) {
                x = __ddiv_rn(1.0, x);
                y = -y;
                continue;
            }
            if (y < 0) return 0;
            if (y > 0) return INF;
        }
        break;
    }
    if (y == 0.5) return __dsqrt_rn(x);
    if (y == -0.5) return __ddiv_rn(1.0, __dsqrt_rn(x));

    double yi;
    double yf = modf(fabs(y), &yi);
    if (yf != 0 && x < 0) return NAN_;
    if (yi >= 9223372036854775808.0) {
        if (x == -1) return 1;
        if ((fabs(x) < 1) == (y > 0)) return 0;
        return INF;
    }
    double a1 = 1.0;
    int64_t ae = 0;
    if (yf != 0) {
        if (yf > 0.5) {
            yf = __dsub_rn(yf, 1.0);
            yi = __dadd_rn(yi, 1.0);
        }
        a1 = exp(__dmul_rn(yf, log(x)));
    }
    int xe_i;
    double x1 = frexp(x, &xe_i);
    int64_t xe = xe_i;
    for (int64_t i = (int64_t)yi; i != 0; i >>= 1) {
        if (xe < -(1 << 12) || (1 << 12) < xe) {
            ae += xe;
            break;
        }
        if ((i & 1) == 1) {
            a1 = __dmul_rn(a1, x1);
            ae += xe;
        }
        x1 = __dmul_rn(x1, x1);
        xe <<= 1;
        if (x1 < .5) {
            x1 = __dadd_rn(x1, x1);
            xe--;
        }
    }
    if (y < 0) {
        a1 = __ddiv_rn(1.0, a1);
        ae = -ae;
    }
    if (ae > 100000) ae = 100000;
    if (ae < -100000) ae = -100000;
    return ldexp(a1, (int)ae);
}

// Pow(x, SpecularPower) for the Fragment's specular term (x > 0). When the
// power is an integer yi in [2, 2^63) (classified on the host) and x is a
// normal number other than 1, math.Pow takes none of its special cases and
// forms x**yi by repeated squaring of Frexp(x); here Frexp, the "x1 < .5"
// renormalisation (an exact doubling) and the Ldexp of a normal result act on
// the exponent bits, and the multiplications are the reference's own. The
// reference squares once more after the last exponent bit; nothing reads that
// value, so it is skipped. Everything else goes through go_pow.
__device__ __forceinline__ double pow_specular(double x, double y, uint64_t yi) {
    const unsigned long long b = dbits(x);
    const unsigned long long ex = b >> 52;  // x > 0: no sign bit
    if (yi == 0 || ex == 0 || ex >= 2047 || b == 0x3ff0000000000000ull) return go_pow(x, y);
    unsigned long long x1 = (b & 0x000fffffffffffffull) | 0x3fe0000000000000ull;  // in [0.5, 1)
    int64_t xe = (int64_t)ex - 1022;
    unsigned long long a1 = 0x3ff0000000000000ull;  // 1.0
    bool one = true;
    int64_t ae = 0;
    for (uint64_t i = yi; i != 0; i >>= 1) {
        if (xe < -(1 << 12) || (1 << 12) < xe) {
            ae += xe;
            break;
        }
        if (i & 1) {  // a1 *= x1; 1 * x1 is x1 itself
            a1 = one ? x1 : dbits(__dmul_rn(__longlong_as_double((long long)a1), __longlong_as_double((long long)x1)));
            one = false;
            ae += xe;
        }
        if ((i >> 1) == 0) break;
        const double d1 = __longlong_as_double((long long)x1);
        x1 = dbits(__dmul_rn(d1, d1));  // in [0.25, 1)
        xe <<= 1;
        if (x1 < 0x3fe0000000000000ull) {  // x1 < .5: x1 += x1
            x1 += 1ull << 52;
            xe--;
        }
    }
    // Ldexp(a1, ae); a1 is a normal number in (0, 1]
    const int64_t e = (int64_t)(a1 >> 52) + ae;
    if (e >= 1 && e <= 2046) return __longlong_as_double((long long)(a1 + ((unsigned long long)ae << 52)));
    if (ae > 100000) ae = 100000;
    if (ae < -100000) ae = -100000;
    return ldexp(__longlong_as_double((long long)a1), (int)ae);
}

// ---------------------------------------------------------------------------
// FP64 vector helpers in the reference's operation order
// ---------------------------------------------------------------------------

struct D3 { double x, y, z; };
struct D4 { double x, y, z, w; };

__device__ __forceinline__ D3 d3(double x, double y, double z) { return D3{x, y, z}; }
__device__ __forceinline__ D3 add3(D3 a, D3 b) { return d3(__dadd_rn(a.x, b.x), __dadd_rn(a.y, b.y), __dadd_rn(a.z, b.z)); }
__device__ __forceinline__ D3 sub3(D3 a, D3 b) { return d3(__dsub_rn(a.x, b.x), __dsub_rn(a.y, b.y), __dsub_rn(a.z, b.z)); }
__device__ __forceinline__ D3 muls3(D3 a, double s) { return d3(__dmul_rn(a.x, s), __dmul_rn(a.y, s), __dmul_rn(a.z, s)); }
// Vector.Dot (vector.go:72-74): (x*x' + y*y') + z*z'.
__device__ __forceinline__ double dot3(D3 a, D3 b) {
    return __dadd_rn(__dadd_rn(__dmul_rn(a.x, b.x), __dmul_rn(a.y, b.y)), __dmul_rn(a.z, b.z));
}
__device__ __forceinline__ D3 cross3(D3 a, D3 b) {
    return d3(__dsub_rn(__dmul_rn(a.y, b.z), __dmul_rn(a.z, b.y)),
              __dsub_rn(__dmul_rn(a.z, b.x), __dmul_rn(a.x, b.z)),
              __dsub_rn(__dmul_rn(a.x, b.y), __dmul_rn(a.y, b.x)));
}
// Vector.Normalize (vector.go:83-86): multiply by 1/sqrt(x*x + y*y + z*z).
__device__ __forceinline__ D3 normalize3(D3 a) {
    double r = __drcp_rn(__dsqrt_rn(dot3(a, a)));  // 1 / sqrt(...), correctly rounded
    return muls3(a, r);
}

__device__ __forceinline__ D4 d4(double x, double y, double z, double w) { return D4{x, y, z, w}; }
__device__ __forceinline__ D4 add4(D4 a, D4 b) {
    return d4(__dadd_rn(a.x, b.x), __dadd_rn(a.y, b.y), __dadd_rn(a.z, b.z), __dadd_rn(a.w, b.w));
}
__device__ __forceinline__ D4 sub4(D4 a, D4 b) {
    return d4(__dsub_rn(a.x, b.x), __dsub_rn(a.y, b.y), __dsub_rn(a.z, b.z), __dsub_rn(a.w, b.w));
}
__device__ __forceinline__ D4 muls4(D4 a, double s) {
    return d4(__dmul_rn(a.x, s), __dmul_rn(a.y, s), __dmul_rn(a.z, s), __dmul_rn(a.w, s));
}
// VectorW.Dot (vector.go:217-219).
__device__ __forceinline__ double dot4(D4 a, D4 b) {
    return __dadd_rn(__dadd_rn(__dadd_rn(__dmul_rn(a.x, b.x), __dmul_rn(a.y, b.y)), __dmul_rn(a.z, b.z)),
                     __dmul_rn(a.w, b.w));
}
// VectorW.Outside (vector.go:212-215).
// VectorW.Outside (vector.go:212-215): x < -w || x > w || ... with IEEE
// comparisons (false for NaN, -0 == +0), evaluated on the integer pipe.
__device__ __forceinline__ bool outside4(D4 a) {
    const double nw = fj_double(dbits(a.w) ^ 0x8000000000000000ull);  // -w
    return dgt_i(nw, a.x) || dgt_i(a.x, a.w) || dgt_i(nw, a.y) || dgt_i(a.y, a.w) || dgt_i(nw, a.z) ||
           dgt_i(a.z, a.w);
}

// Matrix.MulPositionW (matrix.go:216-222).
__device__ __forceinline__ D4 mul_position_w(const double* m, double x, double y, double z) {
    return d4(__dadd_rn(__dadd_rn(__dadd_rn(__dmul_rn(m[0], x), __dmul_rn(m[1], y)), __dmul_rn(m[2], z)), m[3]),
              __dadd_rn(__dadd_rn(__dadd_rn(__dmul_rn(m[4], x), __dmul_rn(m[5], y)), __dmul_rn(m[6], z)), m[7]),
              __dadd_rn(__dadd_rn(__dadd_rn(__dmul_rn(m[8], x), __dmul_rn(m[9], y)), __dmul_rn(m[10], z)), m[11]),
              __dadd_rn(__dadd_rn(__dadd_rn(__dmul_rn(m[12], x), __dmul_rn(m[13], y)), __dmul_rn(m[14], z)), m[15]));
}

// Screen(w, h).MulPosition(ndc) (matrix.go:119-128, 209-214). For finite ndc
// the zero-coefficient terms contribute signed zeros that the final add of
// the nonzero translation absorbs, so the short form has the same bits; the
// literal form keeps NaN propagation (0 * Inf) for non-finite input.
__device__ __forceinline__ D3 screen_of_ndc(D3 n, double w2, double h2) {
    if (dfinite(n.x) && dfinite(n.y) && dfinite(n.z)) {
        return d3(__dadd_rn(__dmul_rn(w2, n.x), w2), __dadd_rn(__dmul_rn(-h2, n.y), h2),
                  __dadd_rn(__dmul_rn(0.5, n.z), 0.5));
    }
    double x = __dadd_rn(__dadd_rn(__dadd_rn(__dmul_rn(w2, n.x), __dmul_rn(0.0, n.y)), __dmul_rn(0.0, n.z)), w2);
    double y = __dadd_rn(__dadd_rn(__dadd_rn(__dmul_rn(0.0, n.x), __dmul_rn(-h2, n.y)), __dmul_rn(0.0, n.z)), h2);
    double z = __dadd_rn(__dadd_rn(__dadd_rn(__dmul_rn(0.0, n.x), __dmul_rn(0.0, n.y)), __dmul_rn(0.5, n.z)), 0.5);
    return d3(x, y, z);
}

// Output.DivScalar(W).Vector() (vector.go:233-235).
// x / w correctly rounded, given y = RN(1 / w). q0 = RN(x y) is within 1.5
// ulp of x / w; one FMA residual correction makes it a faithful rounding,
// whose residual x - w q1 is then exact, and the second correction
// RN(q1 + r1 y) is RN(x / w) by Markstein's theorem (P. Markstein,
// "Computation of elementary functions on the IBM RISC System/6000
// processor", IBM J. Res. Dev. 34(1), 1990). The argument assumes no
// underflow or overflow in any step, which |x| and |w| in [2^-400, 2^401)
// guarantee; other operands take the division itself.
// tests/divrcp_check.cu compares it with __ddiv_rn on the GPU.
__device__ __forceinline__ double div_by_rcp(double x, double w, double y) {
    const unsigned long long ex = (dbits(x) >> 52) & 0x7ff, ew = (dbits(w) >> 52) & 0x7ff;
    if (ex - 623ull > 800ull || ew - 623ull > 800ull) return __ddiv_rn(x, w);
    const double q0 = __dmul_rn(x, y);
    const double q1 = __fma_rn(__fma_rn(-w, q0, x), y, q0);
    return __fma_rn(__fma_rn(-w, q1, x), y, q1);
}

// Output.DivScalar(Output.W).Vector() (vector.go:233-235, context.go:318-320),
// with y = RN(1 / Output.W).
__device__ __forceinline__ D3 ndc_of_rcp(D4 o, double y) {
    return d3(div_by_rcp(o.x, o.w, y), div_by_rcp(o.y, o.w, y), div_by_rcp(o.z, o.w, y));
}
__device__ __forceinline__ D3 ndc_of(D4 o) { return ndc_of_rcp(o, __drcp_rn(o.w)); }

// Floor division for possibly negative numerators (b > 0).
__device__ __forceinline__ int64_t floordiv(int64_t a, int64_t b) {
    int64_t q = a / b;
    if ((a % b != 0) && (a < 0)) q--;
    return q;
}

}  // namespace fgc
