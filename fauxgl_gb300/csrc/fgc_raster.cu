// fgc_raster.cu -- band rasteriser: fragment generation, shading and ordered
// depth/colour resolve, one CTA per band, no framebuffer atomics.
//
// Reference: rasterize (context.go:151-281), InterpolateVertexes
// (vertex.go:18-47), the built-in Fragment shaders (shader.go:25-27, 44-46,
// 75-96), BilinearSample (texture.go:41-63), Color.NRGBA (color.go:56-63).
//
// Persistent CTAs take (draw, band) work from an atomic counter. A band's
// depth lives in shared memory and its colour in global memory (the band is
// the CTA's alone) while its bin (raster primitives in submission order) is
// processed in chunks of (primitive, row) units:
//   fragments every covered pixel of the band becomes a fragment (b0, b1,
//             b2, z) with exactly the edge values rasterize's serial row loop
//             gives it. Narrow primitives: one thread per unit runs that loop
//             (row start, skip-ahead d, per-pixel adds, inside test, break).
//             Wide ones: one thread per unit finds the row's covered interval
//             and its first edge values (exact jumps through the serial sums,
//             fgc_fpjump.cuh), then all threads walk windows of P.win pixels.
//             An early depth test against the band's current depth drops
//             fragments that cannot update (only when depth can only
//             decrease during the draw).
//   shade     one thread per fragment: perspective-correct weights,
//             interpolation and the built-in shader, in FP64 (plain) or FP32
//             (mixed).
//   resolve   fragments are applied per pixel in (primitive, row) order:
//             directly when no two fragments of the chunk share a pixel
//             bucket, otherwise one thread per bucket list applies its
//             fragments by increasing (pixel, unit) key. The depth test,
//             UpdatedPixels, depth write and the NRGBA / alpha-blend colour
//             write are exactly rasterize's (context.go:247-272).
#include "fgc_fpjump.cuh"
#include "fgc_internal.cuh"

namespace fgc {

constexpr int kRT = 256;  // threads per raster CTA
static_assert(kRasterHeads >= 2 * 1024 && (kRasterHeads & (kRasterHeads - 1)) == 0, "bucket count");
__device__ __forceinline__ uint32_t bucket_of(uint32_t pix) { return pix & (kRasterHeads - 1); }
constexpr uint8_t kFragDiscard = 1;
constexpr uint8_t kFragBlend = 2;

struct RasterSmem {
    double* depth;   // [L]
    double* fb0;     // [F] (reused as the u64 sort buffer)
    double* fb1;
    double* fb2;
    double* fz;
    uint32_t* fkey;  // [F] (pixel << 16) | unit
    uint32_t* fcol;  // [F] NRGBA
    double* uw0;     // [su] unit -> edge values at its first covered in-band pixel
    double* uw1;
    double* uw2;
    uint32_t* uslot; // [F] unit -> chunk slot
    int32_t* urow;   // [F] unit -> row y
    int32_t* ux;     // [su] unit -> first covered in-band x
    uint32_t* ucnt;  // [su] unit -> covered in-band pixels
    uint32_t* ufrag; // [su] unit -> first fragment offset in the chunk
    uint32_t* cprim; // [kChunkPrims] chunk slot -> primitive
    unsigned short* head;  // [kHeads] per pixel bucket: last fragment of its list (0xFFFF: none)
    unsigned short* nxt;   // [F] per fragment: the previous fragment in its bucket
    uint8_t* fflag;  // [F] discard / blend flags
    unsigned long long* scratch;
};

// The band being rasterised: rows [r0, rend) of its draw's frame, pixels
// [i0, i0 + npx) in linear index order.
struct BandCtx {
    int64_t i0;
    int32_t r0, rend;
    int32_t npx;
    uint32_t band;   // the band's index in its draw
    bool early;      // early depth rejection is valid
};

// ---------------------------------------------------------------------------
// Attribute fetch
// ---------------------------------------------------------------------------
__device__ __forceinline__ void fetch_pn64(const RasterParams& P, const MeshView& M, uint32_t v, D3& pos, D3& nrm) {
    if (v & kPoolFlag) {
        const PoolVertex& q = P.pool[v & ~kPoolFlag];
        pos = d3(q.px, q.py, q.pz);
        nrm = d3(q.nx, q.ny, q.nz);
    } else {
        APosNrm64 a = M.pn64[v];
        pos = d3(a.px, a.py, a.pz);
        nrm = d3(a.nx, a.ny, a.nz);
    }
}
__device__ __forceinline__ void fetch_tex64(const RasterParams& P, const MeshView& M, uint32_t v, double& u,
                                            double& w) {
    if (v & kPoolFlag) {
        const PoolVertex& q = P.pool[v & ~kPoolFlag];
        u = q.tu;
        w = q.tv;
    } else if (M.tex64) {
        u = M.tex64[2 * (uint64_t)v];
        w = M.tex64[2 * (uint64_t)v + 1];
    } else {
        u = 0.0;
        w = 0.0;
    }
}
__device__ __forceinline__ D4 fetch_col64(const RasterParams& P, const MeshView& M, uint32_t v) {
    if (v & kPoolFlag) {
        const PoolVertex& q = P.pool[v & ~kPoolFlag];
        return d4(q.cr, q.cg, q.cb, q.ca);
    }
    if (M.col64) {
        const double* c = M.col64 + 4 * (uint64_t)v;
        return d4(c[0], c[1], c[2], c[3]);
    }
    return d4(0, 0, 0, 0);
}

// ((0 + a*bX) + b*bY + c*bZ) * bW (vertex.go:57-79).
__device__ __forceinline__ double interp1(double a, double b, double c, D4 w) {
    double n = zero_plus(__dmul_rn(a, w.x));
    n = __dadd_rn(n, __dmul_rn(b, w.y));
    n = __dadd_rn(n, __dmul_rn(c, w.z));
    return __dmul_rn(n, w.w);
}

// ---------------------------------------------------------------------------
// FP64 shading (plain form)
// ---------------------------------------------------------------------------
__device__ __forceinline__ D4 tex_at64(const TexView& t, int64_t x, int64_t y) {
    if (x < 0 || y < 0 || x >= t.w || y >= t.h) return d4(0, 0, 0, 0);
    const double2* q = reinterpret_cast<const double2*>(t.unit64 + 4 * ((uint64_t)y * (uint64_t)t.w + (uint64_t)x));
    const double2 lo = q[0], hi = q[1];
    return d4(lo.x, lo.y, hi.x, hi.y);
}

__device__ D4 bilinear64(const TexView& t, double u, double v) {  // texture.go:41-63
    v = __dsub_rn(1.0, v);
    u = __dsub_rn(u, floor(u));
    v = __dsub_rn(v, floor(v));
    double x = __dmul_rn(u, (double)(t.w - 1));
    double y = __dmul_rn(v, (double)(t.h - 1));
    int64_t x0 = go_f2i_i(x), y0 = go_f2i_i(y);
    int64_t x1 = x0 + 1, y1 = y0 + 1;
    x = __dsub_rn(x, (double)x0);
    y = __dsub_rn(y, (double)y0);
    D4 c00 = tex_at64(t, x0, y0), c01 = tex_at64(t, x0, y1), c10 = tex_at64(t, x1, y0), c11 = tex_at64(t, x1, y1);
    double k00 = __dmul_rn(__dsub_rn(1.0, x), __dsub_rn(1.0, y));
    double k10 = __dmul_rn(x, __dsub_rn(1.0, y));
    double k01 = __dmul_rn(__dsub_rn(1.0, x), y);
    double k11 = __dmul_rn(x, y);
    D4 c = d4(0, 0, 0, 0);
    c = add4(c, muls4(c00, k00));
    c = add4(c, muls4(c10, k10));
    c = add4(c, muls4(c01, k01));
    c = add4(c, muls4(c11, k11));
    return c;
}

__device__ D4 shade64(const RasterParams& P, const ItemView& I, const RPrim& R, double b0, double b1, double b2) {
    const ShaderView& S = I.sh;
    const MeshView& M = I.mesh;
    if (S.kind == FGC_SHADER_SOLID_COLOR) return d4(S.color[0], S.color[1], S.color[2], S.color[3]);
    // perspective-correct barycentrics (context.go:236-237)
    D4 w = d4(__dmul_rn(b0, R.r0), __dmul_rn(b1, R.r1), __dmul_rn(b2, R.r2), 0.0);
    w.w = __drcp_rn(__dadd_rn(__dadd_rn(w.x, w.y), w.z));
    if (S.kind == FGC_SHADER_TEXTURE) {
        double u0, v0, u1, v1, u2, v2;
        fetch_tex64(P, M, R.v0, u0, v0);
        fetch_tex64(P, M, R.v1, u1, v1);
        fetch_tex64(P, M, R.v2, u2, v2);
        return bilinear64(S.tex, interp1(u0, u1, u2, w), interp1(v0, v1, v2, w));
    }
    // PhongShader.Fragment (shader.go:75-96)
    D3 p0, n0, p1, n1, p2, n2;
    fetch_pn64(P, M, R.v0, p0, n0);
    fetch_pn64(P, M, R.v1, p1, n1);
    fetch_pn64(P, M, R.v2, p2, n2);
    D3 nrm = normalize3(d3(interp1(n0.x, n1.x, n2.x, w), interp1(n0.y, n1.y, n2.y, w), interp1(n0.z, n1.z, n2.z, w)));
    D4 color;
    if (S.object_is_discard) {
        D4 c0 = fetch_col64(P, M, R.v0), c1 = fetch_col64(P, M, R.v1), c2 = fetch_col64(P, M, R.v2);
        color = d4(interp1(c0.x, c1.x, c2.x, w), interp1(c0.y, c1.y, c2.y, w), interp1(c0.z, c1.z, c2.z, w),
                   interp1(c0.w, c1.w, c2.w, w));
    } else {
        color = d4(S.color[0], S.color[1], S.color[2], S.color[3]);
    }
    if (S.has_texture) {
        double u0, v0, u1, v1, u2, v2;
        fetch_tex64(P, M, R.v0, u0, v0);
        fetch_tex64(P, M, R.v1, u1, v1);
        fetch_tex64(P, M, R.v2, u2, v2);
        color = bilinear64(S.tex, interp1(u0, u1, u2, w), interp1(v0, v1, v2, w));
    }
    D3 L = d3(S.light[0], S.light[1], S.light[2]);
    const double ndl = dot3(nrm, L);
    double diffuse = go_max0(ndl);
    // light = AmbientColor + DiffuseColor * diffuse (its alpha never reaches
    // the result); with equal R, G, B inputs the three channels are equal
    D3 light;
    light.x = __dadd_rn(S.ambient[0], __dmul_rn(S.diffuse[0], diffuse));
    if (S.gray_light) {
        light.y = light.z = light.x;
    } else {
        light.y = __dadd_rn(S.ambient[1], __dmul_rn(S.diffuse[1], diffuse));
        light.z = __dadd_rn(S.ambient[2], __dmul_rn(S.diffuse[2], diffuse));
    }
    if (dgt0(diffuse) && S.power_pos) {
        // the interpolated position is read only here
        const D3 pos = d3(interp1(p0.x, p1.x, p2.x, w), interp1(p0.y, p1.y, p2.y, w), interp1(p0.z, p1.z, p2.z, w));
        D3 camera = normalize3(sub3(d3(S.eye[0], S.eye[1], S.eye[2]), pos));
        D3 negl = d3(-L.x, -L.y, -L.z);
        // Reflect (vector.go:175-177) with n.Dot(-L) = -(n.Dot(L)): rounding is
        // symmetric, so the two differ at most in the sign of a zero, which
        // only flips zero signs in `reflected` where -L has a zero component;
        // those terms add nothing to a nonzero specular dot product and a zero
        // one fails the "> 0" test either way
        D3 reflected = sub3(negl, muls3(nrm, twice(-ndl)));
        double specular = go_max0(dot3(camera, reflected));
        if (dgt0(specular)) {
            specular = pow_specular(specular, S.power, S.pow_yi);
            const double s0 = __dmul_rn(S.specular[0], specular);
            if (S.gray_light && S.gray_spec) {
                light.x = __dadd_rn(light.x, s0);
                light.y = light.z = light.x;
            } else {
                const double s1 = S.gray_spec ? s0 : __dmul_rn(S.specular[1], specular);
                const double s2 = S.gray_spec ? s0 : __dmul_rn(S.specular[2], specular);
                light.x = __dadd_rn(light.x, s0);
                light.y = __dadd_rn(light.y, s1);
                light.z = __dadd_rn(light.z, s2);
            }
        }
    }
    return d4(go_min1(__dmul_rn(color.x, light.x)), go_min1(__dmul_rn(color.y, light.y)),
              go_min1(__dmul_rn(color.z, light.z)), color.w);
}

// ---------------------------------------------------------------------------
// FP32 shading (mixed form)
// ---------------------------------------------------------------------------
struct F3 { float x, y, z; };
__device__ __forceinline__ float dotf3(F3 a, F3 b) { return __fmaf_rn(a.z, b.z, __fmaf_rn(a.y, b.y, a.x * b.x)); }
__device__ __forceinline__ F3 normf3(F3 a) {
    float r = 1.0f / sqrtf(dotf3(a, a));
    return F3{a.x * r, a.y * r, a.z * r};
}
__device__ __forceinline__ float interpf(float a, float b, float c, float wx, float wy, float wz, float ww) {
    return __fmaf_rn(c, wz, __fmaf_rn(b, wy, a * wx)) * ww;
}

__device__ __forceinline__ void fetch_pn32(const RasterParams& P, const MeshView& M, uint32_t v, F3& pos, F3& nrm) {
    if (v & kPoolFlag) {
        const PoolVertex32& q = P.pool32[v & ~kPoolFlag];
        pos = F3{q.px, q.py, q.pz};
        nrm = F3{q.nx, q.ny, q.nz};
    } else {
        APosNrm32 a = M.pn32[v];
        pos = F3{a.px, a.py, a.pz};
        nrm = F3{a.nx, a.ny, a.nz};
    }
}

__device__ __forceinline__ float4 tex_at32(const TexView& t, int x, int y) {
    if (x < 0 || y < 0 || x >= t.w || y >= t.h) return make_float4(0, 0, 0, 0);
    ushort4 p = t.texels[(uint64_t)y * (uint64_t)t.w + (uint64_t)x];
    const float d = 1.0f / 65535.0f;
    return make_float4(p.x * d, p.y * d, p.z * d, p.w * d);
}

__device__ float4 bilinear32(const TexView& t, float u, float v) {
    v = 1.0f - v;
    u = u - floorf(u);
    v = v - floorf(v);
    float x = u * (float)(t.w - 1), y = v * (float)(t.h - 1);
    int x0 = (x == x && x < 2147483520.0f) ? (int)x : INT_MIN;
    int y0 = (y == y && y < 2147483520.0f) ? (int)y : INT_MIN;
    float fx = x - (float)x0, fy = y - (float)y0;
    float4 c00 = tex_at32(t, x0, y0), c01 = tex_at32(t, x0, y0 + 1), c10 = tex_at32(t, x0 + 1, y0),
           c11 = tex_at32(t, x0 + 1, y0 + 1);
    float k00 = (1 - fx) * (1 - fy), k10 = fx * (1 - fy), k01 = (1 - fx) * fy, k11 = fx * fy;
    return make_float4(c00.x * k00 + c10.x * k10 + c01.x * k01 + c11.x * k11,
                       c00.y * k00 + c10.y * k10 + c01.y * k01 + c11.y * k11,
                       c00.z * k00 + c10.z * k10 + c01.z * k01 + c11.z * k11,
                       c00.w * k00 + c10.w * k10 + c01.w * k01 + c11.w * k11);
}

__device__ float powf_int_or_general(float x, float p) {
    if (p == 32.0f) {  // the default SpecularPower: five squarings
        float y = x * x;
        y = y * y;
        y = y * y;
        y = y * y;
        return y * y;
    }
    return powf(x, p);
}

__device__ float4 shade32(const RasterParams& P, const ItemView& I, const RPrim& R, float4 rf, double b0, double b1,
                         double b2) {
    const ShaderView& S = I.sh;
    const MeshView& M = I.mesh;
    if (S.kind == FGC_SHADER_SOLID_COLOR) return make_float4(S.color32[0], S.color32[1], S.color32[2], S.color32[3]);
    float wx = (float)b0 * rf.x, wy = (float)b1 * rf.y, wz = (float)b2 * rf.z;
    float ww = 1.0f / (wx + wy + wz);
    float4 color;
    bool have_color = false;
    if (S.kind == FGC_SHADER_TEXTURE || S.has_texture) {
        float u[3], v[3];
        uint32_t vr[3] = {R.v0, R.v1, R.v2};
        for (int k = 0; k < 3; k++) {
            if (vr[k] & kPoolFlag) {
                const PoolVertex32& q = P.pool32[vr[k] & ~kPoolFlag];
                u[k] = q.tu;
                v[k] = q.tv;
            } else if (M.tex32) {
                u[k] = M.tex32[2 * (uint64_t)vr[k]];
                v[k] = M.tex32[2 * (uint64_t)vr[k] + 1];
            } else {
                u[k] = 0;
                v[k] = 0;
            }
        }
        color = bilinear32(S.tex, interpf(u[0], u[1], u[2], wx, wy, wz, ww), interpf(v[0], v[1], v[2], wx, wy, wz, ww));
        if (S.kind == FGC_SHADER_TEXTURE) return color;
        have_color = true;
    }
    F3 p0, n0, p1, n1, p2, n2;
    fetch_pn32(P, M, R.v0, p0, n0);
    fetch_pn32(P, M, R.v1, p1, n1);
    fetch_pn32(P, M, R.v2, p2, n2);
    F3 pos = F3{interpf(p0.x, p1.x, p2.x, wx, wy, wz, ww), interpf(p0.y, p1.y, p2.y, wx, wy, wz, ww),
                interpf(p0.z, p1.z, p2.z, wx, wy, wz, ww)};
    F3 nrm = normf3(F3{interpf(n0.x, n1.x, n2.x, wx, wy, wz, ww), interpf(n0.y, n1.y, n2.y, wx, wy, wz, ww),
                       interpf(n0.z, n1.z, n2.z, wx, wy, wz, ww)});
    if (!have_color) {
        if (S.object_is_discard) {
            uint32_t vr[3] = {R.v0, R.v1, R.v2};
            float c[3][4];
            for (int k = 0; k < 3; k++) {
                if (vr[k] & kPoolFlag) {
                    const PoolVertex32& q = P.pool32[vr[k] & ~kPoolFlag];
                    c[k][0] = q.cr; c[k][1] = q.cg; c[k][2] = q.cb; c[k][3] = q.ca;
                } else if (M.col32) {
                    for (int j = 0; j < 4; j++) c[k][j] = M.col32[4 * (uint64_t)vr[k] + j];
                } else {
                    for (int j = 0; j < 4; j++) c[k][j] = 0;
                }
            }
            color = make_float4(interpf(c[0][0], c[1][0], c[2][0], wx, wy, wz, ww),
                                interpf(c[0][1], c[1][1], c[2][1], wx, wy, wz, ww),
                                interpf(c[0][2], c[1][2], c[2][2], wx, wy, wz, ww),
                                interpf(c[0][3], c[1][3], c[2][3], wx, wy, wz, ww));
        } else {
            color = make_float4(S.color32[0], S.color32[1], S.color32[2], S.color32[3]);
        }
    }
    F3 L = F3{S.light32[0], S.light32[1], S.light32[2]};
    float lr = S.ambient32[0], lg = S.ambient32[1], lb = S.ambient32[2];
    float nl = dotf3(nrm, L);
    float diffuse = (nl > 0.0f) ? nl : ((nl != nl) ? nl : 0.0f);
    lr = __fmaf_rn(S.diffuse32[0], diffuse, lr);
    lg = __fmaf_rn(S.diffuse32[1], diffuse, lg);
    lb = __fmaf_rn(S.diffuse32[2], diffuse, lb);
    if (diffuse > 0 && S.power_pos) {
        F3 cam = normf3(F3{S.eye32[0] - pos.x, S.eye32[1] - pos.y, S.eye32[2] - pos.z});
        F3 negl = F3{-L.x, -L.y, -L.z};
        float k = 2.0f * dotf3(nrm, negl);
        F3 refl = F3{negl.x - nrm.x * k, negl.y - nrm.y * k, negl.z - nrm.z * k};
        float sp = dotf3(cam, refl);
        if (sp > 0) {
            sp = powf_int_or_general(sp, S.power32);
            lr = __fmaf_rn(S.specular32[0], sp, lr);
            lg = __fmaf_rn(S.specular32[1], sp, lg);
            lb = __fmaf_rn(S.specular32[2], sp, lb);
        }
    }
    return make_float4(fminf(color.x * lr, 1.0f), fminf(color.y * lg, 1.0f), fminf(color.z * lb, 1.0f), color.w);
}

__device__ __forceinline__ uint32_t u8_of_unit_f32(float c) {
    float v = fminf(fmaxf(c, 0.0f), 1.0f) * 255.0f;
    return (c == c) ? ((uint32_t)v & 0xff) : 0u;
}

// ---------------------------------------------------------------------------
// Rows (context.go:184-278)
// ---------------------------------------------------------------------------
// rasterize walks each row serially: w_k += a_k per pixel, w0k += b_k per
// row. Both sequences are monotone (round-to-nearest is monotone and a step
// never moves against the sign of its addend), and so is w*ra for a fixed
// ra; the coverage test "no b_k = w_k*ra is negative" is therefore true on
// exactly one interval of the row, and the walk's break after leaving the
// triangle never hides a later covered pixel. A row is handled as:
//   span     one thread finds the row's covered interval exactly (a plain
//            walk for short rows, the edges' sign changes located with exact
//            jumps for long ones) and the edge values at its first pixel in
//            the band;
//   windows  the chunk's covered pixels, numbered in unit order, are dealt
//            out P.win at a time; a window that starts inside a row starts
//            from an exact jump (repeat_add) and walks on from there.
// Every value is the one the serial walk would have had: the same adds in
// the same order, only not all of them executed one after the other.
constexpr int kNarrow = 32;      // boxes at most this wide are walked row by row
constexpr int kShortRow = 40;    // rows of at most this many steps are walked plainly

// The edge values w00, w01, w02 rasterize holds at row y of primitive pp
// (after y - y0 row increments): for a tall primitive its row start in this
// band (row_starts_kernel), for a short one its top row, advanced by the rows
// between that row and y -- a few plain adds, exact jumps beyond 64 rows.
__device__ __forceinline__ void row_start(const RasterParams& P, uint32_t pp, const RPrim& R, const PBox& bx,
                                          int32_t y, const ItemView& I, const BandCtx& B, double& w00, double& w01,
                                          double& w02) {
    int64_t first = bx.y0;
    if (I.row_table && uses_row_table(bx)) {
        const BandGeom G{I.W, I.H, I.R, I.nbands};
        uint32_t bl = 0, bh = 0;
        prim_bands(G, bx, bl, bh);  // the primitive is binned to this band: bl <= B.band
        const double* rs = P.rstart + 3 * ((uint64_t)P.prs[pp] + (B.band - bl));
        w00 = rs[0];
        w01 = rs[1];
        w02 = rs[2];
        first = (int64_t)B.r0 - floordiv_w(bx.x1, I.W);
        if (first < bx.y0) first = bx.y0;
    } else {
        w00 = R.w0;
        w01 = R.w1;
        w02 = R.w2;
    }
    const int64_t r = (int64_t)y - first;
    if (r > 64) {
        w00 = repeat_add(w00, R.b0, (uint64_t)r);
        w01 = repeat_add(w01, R.b1, (uint64_t)r);
        w02 = repeat_add(w02, R.b2, (uint64_t)r);
    } else {
        for (int64_t j = 0; j < r; j++) {
            w00 = __dadd_rn(w00, R.b0);
            w01 = __dadd_rn(w01, R.b1);
            w02 = __dadd_rn(w02, R.b2);
        }
    }
}

// Row state in 32-bit band-relative coordinates: the pixel at x of row y is
// band pixel rel + x, rel = (y - r0) * W. For a row that meets the band
// (rows_in_band) and a box within the setup limits (|coordinates| <= 2^30,
// extent <= 2^26), rel and rel + x stay far inside the int32 range.
struct Span {
    int32_t xa;        // first covered in-band x
    int32_t cnt;       // covered in-band pixels
    double w0, w1, w2; // edge values at xa
};

// +1: w*ra can only rise along the row (an edge the row enters), -1: only
// fall (an edge it leaves), 0: constant.
__device__ __forceinline__ int edge_dir(double a, double ra) {
    const unsigned long long ab = dbits(a), rb = dbits(ra);
    if ((ab & kAbsMask) == 0 || bnan(ab) || (rb & kAbsMask) == 0 || bnan(rb)) return 0;
    return ((ab ^ rb) >> 63) ? -1 : 1;
}

// Whether edge k's test "w*ra < 0", once true along a row, stays true for
// the rest of it: a and ra are not NaN and a is zero or of the opposite sign
// to ra (w*ra never rises). A row whose walk meets an outside pixel failing
// such an edge has no covered pixel after it, so the walk can end there.
__device__ __forceinline__ bool stays_out(double a, double ra) {
    const unsigned long long ab = dbits(a), rb = dbits(ra);
    if (bnan(ab) || bnan(rb)) return false;
    return (ab & kAbsMask) == 0 || ((ab ^ rb) >> 63) != 0;
}

// First step t in (lo, hi] at which edge k's test "w*ra < 0" becomes `want`,
// or hi + 1. The test is monotone in t and differs from `want` at lo. ws is
// the edge value at step 0, q = 1/a.
__device__ __noinline__ int64_t edge_flip(double ws, double a, double q, double ra, bool want, int64_t lo,
                                          int64_t hi) {
    const RaSign rs = ra_sign(ra);
    if (lo >= hi) return hi + 1;
    // the real-number crossing -ws/a is within a step or two of the exact one
    // (q = 1/a may be infinite for a subnormal a: the estimate then falls
    // outside (lo, hi] and the search starts at lo)
    const int64_t e = go_f2i_i(__dmul_rn(-ws, q));
    int64_t t = (e > lo + 2 && e - 2 <= hi) ? e - 2 : lo;
    double w;
    if (t > lo) {
        w = repeat_add(ws, a, (uint64_t)t);
        if (neg_product(w, ra, rs) == want) {
            hi = t - 1;  // at or before t: search (lo, t]
            int64_t L = lo, H = t;
            while (H - L > 1) {
                const int64_t mid = L + (H - L) / 2;
                if (neg_product(repeat_add(ws, a, (uint64_t)mid), ra, rs) == want) H = mid;
                else L = mid;
            }
            return H;
        }
        lo = t;
    } else {
        w = repeat_add(ws, a, (uint64_t)lo);
    }
    // a few plain steps from lo
    for (int i = 0; i < 8; i++) {
        if (lo >= hi) return hi + 1;
        w = __dadd_rn(w, a);
        lo++;
        if (neg_product(w, ra, rs) == want) return lo;
    }
    // then halving over (lo, hi]
    int64_t L = lo, H = hi + 1;
    while (H - L > 1) {
        const int64_t mid = L + (H - L) / 2;
        if (neg_product(repeat_add(ws, a, (uint64_t)mid), ra, rs) == want) H = mid;
        else L = mid;
    }
    return H;
}

// The covered in-band pixels of row y of a primitive whose row starts w00
// (after y - y0 row increments) are given: rasterize's skip-ahead d and the
// covered interval, clipped to the band. visited counts the pixel steps
// taken one by one.
__device__ __noinline__ Span row_span(const RPrim& R, const PBox& bx, int32_t y, double w00, double w01, double w02,
                                      int32_t r0, int32_t npx, int32_t W, uint64_t& visited) {
    Span sp;
    sp.xa = 0;
    sp.cnt = 0;
    sp.w0 = sp.w1 = sp.w2 = 0;
    double d = 0;
    double d0 = __dmul_rn(-w00, R.q0);
    double d1 = __dmul_rn(-w01, R.q1);
    double d2 = __dmul_rn(-w02, R.q2);
    if (dlt0(w00) && dgt_i(d0, d)) d = d0;
    if (dlt0(w01) && dgt_i(d1, d)) d = d1;
    if (dlt0(w02) && dgt_i(d2, d)) d = d2;
    int64_t di = go_f2i_i(d);  // d = float64(int(d)); if d < 0 { d = 0 }
    if (di < 0) di = 0;
    const int64_t T = (int64_t)bx.x1 - bx.x0 - di;  // steps after the first: x = x0 + d .. x1
    if (T < 0) return sp;
    d = i2d_i(di);
    const double ws0 = __dadd_rn(w00, __dmul_rn(R.a0, d));
    const double ws1 = __dadd_rn(w01, __dmul_rn(R.a1, d));
    const double ws2 = __dadd_rn(w02, __dmul_rn(R.a2, d));
    const int32_t xs = bx.x0 + (int32_t)di;
    const double ra = R.ra;
    const RaSign rs = ra_sign(ra);
    int64_t ta, tb;  // covered steps [ta, tb]
    double wa0, wa1, wa2;
    if (T < kShortRow) {
        // the plain walk, up to the break
        double w0 = ws0, w1 = ws1, w2 = ws2;
        ta = -1;
        tb = T;
        wa0 = wa1 = wa2 = 0;
        const bool s0 = stays_out(R.a0, ra), s1 = stays_out(R.a1, ra), s2 = stays_out(R.a2, ra);
        for (int64_t t = 0; t <= T; t++) {
            visited++;
            const bool o0 = neg_product(w0, ra, rs), o1 = neg_product(w1, ra, rs), o2 = neg_product(w2, ra, rs);
            if (o0 || o1 || o2) {
                if (ta >= 0) {
                    tb = t - 1;
                    break;
                }
                if ((o0 && s0) || (o1 && s1) || (o2 && s2)) break;  // nothing covered from here on
            } else if (ta < 0) {
                ta = t;
                wa0 = w0;
                wa1 = w1;
                wa2 = w2;
            }
            w0 = __dadd_rn(w0, R.a0);
            w1 = __dadd_rn(w1, R.a1);
            w2 = __dadd_rn(w2, R.a2);
        }
        if (ta < 0) return sp;
    } else {
        // each edge's test changes at most once along the row
        ta = 0;
        tb = T;
        const double ws[3] = {ws0, ws1, ws2};
        const double as[3] = {R.a0, R.a1, R.a2};
        const double qs[3] = {R.q0, R.q1, R.q2};
#pragma unroll 1
        for (int k = 0; k < 3; k++) {
            const int dir = edge_dir(as[k], ra);
            if (neg_product(ws[k], ra, rs)) {
                if (dir <= 0) return sp;  // outside for the whole row
                const int64_t e = edge_flip(ws[k], as[k], qs[k], ra, false, 0, T);
                if (e > T) return sp;
                if (e > ta) ta = e;
            } else if (dir < 0) {
                const int64_t e = edge_flip(ws[k], as[k], qs[k], ra, true, 0, T);
                if (e - 1 < tb) tb = e - 1;
            }
        }
        if (ta > tb) return sp;
        wa0 = repeat_add(ws0, R.a0, (uint64_t)ta);
        wa1 = repeat_add(ws1, R.a1, (uint64_t)ta);
        wa2 = repeat_add(ws2, R.a2, (uint64_t)ta);
        visited += 1;
    }
    // clip [xs + ta, xs + tb] to the band: pix = rel + x in [0, npx)
    const int32_t rel = (y - r0) * W;
    int64_t lo = (int64_t)xs + ta, hi = (int64_t)xs + tb;
    if (lo < -(int64_t)rel) lo = -(int64_t)rel;
    if (hi > (int64_t)npx - 1 - rel) hi = (int64_t)npx - 1 - rel;
    if (lo > hi) return sp;
    const uint64_t skip = (uint64_t)(lo - (xs + ta));
    sp.xa = (int32_t)lo;
    sp.cnt = (int32_t)(hi - lo + 1);
    sp.w0 = repeat_add(wa0, R.a0, skip);
    sp.w1 = repeat_add(wa1, R.a1, skip);
    sp.w2 = repeat_add(wa2, R.a2, skip);
    return sp;
}

// The fused walk for narrow primitives (rows of a few pixels, where finding
// the span first would only repeat the adds): rasterize's row loop for row
// y, recording every covered in-band pixel as a fragment. Returns the
// covered in-band pixels (TotalPixels). A fragment beyond the buffer sets bit
// 2 of *s_conflict: the chunk's size bound failed and the chunk is redone.
__device__ __forceinline__ uint32_t walk_row(uint32_t pp, const RPrim& R, const PBox& bx, int32_t y,
                                             const RasterParams& P, const ItemView& I, const BandCtx& B,
                                             RasterSmem& S, uint32_t unit, uint32_t* s_nfrag, uint32_t* s_conflict,
                                             uint64_t& visited) {
    double w00, w01, w02;
    row_start(P, pp, R, bx, y, I, B, w00, w01, w02);
    double d = 0;
    double d0 = __dmul_rn(-w00, R.q0);
    double d1 = __dmul_rn(-w01, R.q1);
    double d2 = __dmul_rn(-w02, R.q2);
    if (dlt0(w00) && dgt_i(d0, d)) d = d0;
    if (dlt0(w01) && dgt_i(d1, d)) d = d1;
    if (dlt0(w02) && dgt_i(d2, d)) d = d2;
    int64_t di = go_f2i_i(d);  // d = float64(int(d)); if d < 0 { d = 0 }
    if (di < 0) di = 0;
    if (di > (int64_t)bx.x1 - bx.x0) return 0;  // the row loop starts past x1
    d = i2d_i(di);
    double w0 = __dadd_rn(w00, __dmul_rn(R.a0, d));
    double w1 = __dadd_rn(w01, __dmul_rn(R.a1, d));
    double w2 = __dadd_rn(w02, __dmul_rn(R.a2, d));
    const int32_t rel = (y - B.r0) * I.W;
    const double bias = I.st.depth_bias;
    const bool bias_zero = dbits(bias) == 0;
    const double ra = R.ra;
    const RaSign rs = ra_sign(ra);
    const bool s0 = stays_out(R.a0, ra), s1 = stays_out(R.a1, ra), s2 = stays_out(R.a2, ra);
    uint32_t total = 0;
    bool was = false;
    for (int32_t x = bx.x0 + (int32_t)di; x <= bx.x1; x++) {
        const double c0 = w0, c1 = w1, c2 = w2;
        w0 = __dadd_rn(c0, R.a0);
        w1 = __dadd_rn(c1, R.a1);
        w2 = __dadd_rn(c2, R.a2);
        visited++;
        const bool o0 = neg_product(c0, ra, rs), o1 = neg_product(c1, ra, rs), o2 = neg_product(c2, ra, rs);
        if (o0 || o1 || o2) {
            // rasterize breaks after the covered run; before it, an edge the
            // row can only leave ends the row as well (nothing is covered later)
            if (was || (o0 && s0) || (o1 && s1) || (o2 && s2)) break;
            continue;
        }
        was = true;
        // i = y*W + x is skipped outside [0, W*H) (context.go:223-228); here
        // only this band's part of that range is drawn
        const int32_t pix = rel + x;
        if (pix >= B.npx) break;  // beyond this band: no later pixel of the row is in it
        if (pix < 0) continue;
        total++;
        const double b0 = __dmul_rn(c0, ra);
        const double b1 = __dmul_rn(c1, ra);
        const double b2 = __dmul_rn(c2, ra);
        const double z = __dadd_rn(__dadd_rn(__dmul_rn(b0, R.z0), __dmul_rn(b1, R.z1)), __dmul_rn(b2, R.z2));
        if (B.early && dgt_i(add_bias(z, bias, bias_zero), S.depth[pix])) continue;
        const uint32_t slot = atomicAdd(s_nfrag, 1u);
        if (slot >= (uint32_t)P.F) {
            atomicOr(s_conflict, 2u);
            continue;
        }
        S.fb0[slot] = b0;
        S.fb1[slot] = b1;
        S.fb2[slot] = b2;
        S.fz[slot] = z;
        S.fkey[slot] = ((uint32_t)pix << 16) | unit;
        unsigned short* hd = &S.head[bucket_of((uint32_t)pix)];
        unsigned short old = *hd, assumed;
        do {
            assumed = old;
            old = atomicCAS(hd, assumed, (unsigned short)slot);
        } while (old != assumed);
        S.nxt[slot] = old;
        if (old != 0xFFFFu) atomicOr(s_conflict, 1u);
    }
    return total;
}

// Applies one queued covered pixel of a warp: barycentrics b = w*ra and the
// depth with the owning lane's ra and vertex depths (fetched by shuffle:
// every lane of the warp calls this), then early depth rejection and the
// fragment record, as walk_row does for its own pixels.
__device__ __forceinline__ void flush_queued(uint32_t n, uint32_t q0, double ra, double z0, double z1, double z2,
                                             const RasterParams& P, const ItemView& I, const BandCtx& B,
                                             RasterSmem& S, uint32_t* s_nfrag, uint32_t* s_conflict) {
    const uint32_t lane = threadIdx.x & 31, e = q0 + lane;
    const int src = lane < n ? (int)S.ucnt[e] : (int)lane;
    const double rai = __shfl_sync(0xffffffffu, ra, src);
    const double z0i = __shfl_sync(0xffffffffu, z0, src);
    const double z1i = __shfl_sync(0xffffffffu, z1, src);
    const double z2i = __shfl_sync(0xffffffffu, z2, src);
    uint32_t key = 0, pix = 0;
    double b0 = 0, b1 = 0, b2 = 0, z = 0;
    bool keep = false;
    if (lane < n) {
        key = (uint32_t)S.ux[e];
        pix = key >> 16;
        b0 = __dmul_rn(S.uw0[e], rai);
        b1 = __dmul_rn(S.uw1[e], rai);
        b2 = __dmul_rn(S.uw2[e], rai);
        z = __dadd_rn(__dadd_rn(__dmul_rn(b0, z0i), __dmul_rn(b1, z1i)), __dmul_rn(b2, z2i));
        const double bias = I.st.depth_bias;
        keep = !(B.early && dgt_i(add_bias(z, bias, dbits(bias) == 0), S.depth[pix]));
    }
    // one fragment-slot allocation for the warp's kept pixels, in lane order
    const uint32_t km = __ballot_sync(0xffffffffu, keep);
    uint32_t base = 0;
    if (lane == 0 && km) base = atomicAdd(s_nfrag, (uint32_t)__popc(km));
    base = __shfl_sync(0xffffffffu, base, 0);
    if (!keep) return;
    const uint32_t slot = base + (uint32_t)__popc(km & ((1u << lane) - 1u));
    if (slot >= (uint32_t)P.F) {
        atomicOr(s_conflict, 2u);
        return;
    }
    S.fb0[slot] = b0;
    S.fb1[slot] = b1;
    S.fb2[slot] = b2;
    S.fz[slot] = z;
    S.fkey[slot] = key;
    unsigned short* hd = &S.head[bucket_of(pix)];
    unsigned short old = *hd, assumed;
    do {
        assumed = old;
        old = atomicCAS(hd, assumed, (unsigned short)slot);
    } while (old != assumed);
    S.nxt[slot] = old;
    if (old != 0xFFFFu) atomicOr(s_conflict, 1u);
}

// walk_row for a direct chunk with one unit per thread, every thread of the
// block taking part (has: the thread holds a unit). The row loops run in
// step across the warp; a covered in-band pixel is queued (edge values, band
// pixel, unit, owning lane) in the warp's 32 entries of the span arrays,
// which direct chunks do not use, and each full queue is applied with all
// 32 lanes busy, so the pixel's 8 FP64 operations cost one warp instruction
// per 32 pixels rather than one per step in which any lane is covered. A
// direct chunk's boxes are at most kNarrow wide, which bounds the loop.
__device__ __forceinline__ uint32_t walk_rows_queued(bool has, uint32_t pp, const RPrim& R, const PBox& bx,
                                                     int32_t y, const RasterParams& P, const ItemView& I,
                                                     const BandCtx& B, RasterSmem& S, uint32_t unit,
                                                     uint32_t* s_nfrag, uint32_t* s_conflict, uint64_t& visited) {
    const uint32_t lane = threadIdx.x & 31, q0 = threadIdx.x & ~31u;  // this warp's queue entries
    double w0 = 0, w1 = 0, w2 = 0, a0 = 0, a1 = 0, a2 = 0, ra = 0, z0 = 0, z1 = 0, z2 = 0;
    RaSign rs{0, false};
    bool active = false, was = false, s0 = false, s1 = false, s2 = false;
    int32_t x = 0, x1 = 0, rel = 0;
    if (has) {
        double w00, w01, w02;
        row_start(P, pp, R, bx, y, I, B, w00, w01, w02);
        double d = 0;
        const double d0 = __dmul_rn(-w00, R.q0);
        const double d1 = __dmul_rn(-w01, R.q1);
        const double d2 = __dmul_rn(-w02, R.q2);
        if (dlt0(w00) && dgt_i(d0, d)) d = d0;
        if (dlt0(w01) && dgt_i(d1, d)) d = d1;
        if (dlt0(w02) && dgt_i(d2, d)) d = d2;
        int64_t di = go_f2i_i(d);  // d = float64(int(d)); if d < 0 { d = 0 }
        if (di < 0) di = 0;
        if (di <= (int64_t)bx.x1 - bx.x0) {  // else the row loop starts past x1
            d = i2d_i(di);
            a0 = R.a0;
            a1 = R.a1;
            a2 = R.a2;
            w0 = __dadd_rn(w00, __dmul_rn(a0, d));
            w1 = __dadd_rn(w01, __dmul_rn(a1, d));
            w2 = __dadd_rn(w02, __dmul_rn(a2, d));
            ra = R.ra;
            rs = ra_sign(ra);
            s0 = stays_out(a0, ra);
            s1 = stays_out(a1, ra);
            s2 = stays_out(a2, ra);
            z0 = R.z0;
            z1 = R.z1;
            z2 = R.z2;
            x = bx.x0 + (int32_t)di;
            x1 = bx.x1;
            rel = (y - B.r0) * I.W;
            active = true;
        }
    }
    uint32_t total = 0, qn = 0;
    while (__any_sync(0xffffffffu, active)) {
        bool cov = false;
        double c0 = 0, c1 = 0, c2 = 0;
        int32_t pix = 0;
        if (active) {
            c0 = w0;
            c1 = w1;
            c2 = w2;
            w0 = __dadd_rn(c0, a0);
            w1 = __dadd_rn(c1, a1);
            w2 = __dadd_rn(c2, a2);
            visited++;
            const bool o0 = neg_product(c0, ra, rs), o1 = neg_product(c1, ra, rs), o2 = neg_product(c2, ra, rs);
            if (o0 || o1 || o2) {
                // rasterize breaks after the covered run; before it, an edge
                // the row can only leave ends the row as well
                if (was || (o0 && s0) || (o1 && s1) || (o2 && s2)) active = false;
            } else {
                was = true;
                // i = y*W + x is skipped outside [0, W*H) (context.go:223-228);
                // here only this band's part of that range is drawn
                pix = rel + x;
                if (pix >= B.npx) {
                    active = false;  // no later pixel of the row is in the band
                } else if (pix >= 0) {
                    total++;
                    cov = true;
                }
            }
            if (active && ++x > x1) active = false;
        }
        const uint32_t cm = __ballot_sync(0xffffffffu, cov);
        if (cm == 0) continue;
        const uint32_t pos = qn + (uint32_t)__popc(cm & ((1u << lane) - 1u));
        const uint32_t key = ((uint32_t)pix << 16) | unit;
        if (cov && pos < 32) {
            S.uw0[q0 + pos] = c0;
            S.uw1[q0 + pos] = c1;
            S.uw2[q0 + pos] = c2;
            S.ux[q0 + pos] = (int32_t)key;
            S.ucnt[q0 + pos] = lane;
        }
        qn += (uint32_t)__popc(cm);
        if (qn >= 32) {
            __syncwarp();
            flush_queued(32, q0, ra, z0, z1, z2, P, I, B, S, s_nfrag, s_conflict);
            __syncwarp();
            if (cov && pos >= 32) {
                S.uw0[q0 + pos - 32] = c0;
                S.uw1[q0 + pos - 32] = c1;
                S.uw2[q0 + pos - 32] = c2;
                S.ux[q0 + pos - 32] = (int32_t)key;
                S.ucnt[q0 + pos - 32] = lane;
            }
            qn -= 32;
        }
    }
    if (qn) {
        __syncwarp();
        flush_queued(qn, q0, ra, z0, z1, z2, P, I, B, S, s_nfrag, s_conflict);
    }
    return total;
}

// Fragments of one piece of a row: len covered in-band pixels from band pixel pix,
// edge values w at the first. Early depth rejection, fragment records, and
// the push onto the pixel bucket lists (a non-empty list is a possible
// conflict: same pixel or same bucket).
__device__ __forceinline__ void emit_segment(const RPrim& R, const ItemView& I, const BandCtx& B, RasterSmem& S,
                                             int32_t pix, int32_t len, double w0, double w1, double w2, uint32_t unit,
                                             uint32_t* s_nfrag, uint32_t* s_conflict) {
    const double bias = I.st.depth_bias;
    const bool bias_zero = dbits(bias) == 0;
    const double ra = R.ra;
    for (int32_t i = 0; i < len; i++, pix++) {
        const double b0 = __dmul_rn(w0, ra);
        const double b1 = __dmul_rn(w1, ra);
        const double b2 = __dmul_rn(w2, ra);
        if (i + 1 < len) {
            w0 = __dadd_rn(w0, R.a0);
            w1 = __dadd_rn(w1, R.a1);
            w2 = __dadd_rn(w2, R.a2);
        }
        const double z = __dadd_rn(__dadd_rn(__dmul_rn(b0, R.z0), __dmul_rn(b1, R.z1)), __dmul_rn(b2, R.z2));
        if (B.early && dgt_i(add_bias(z, bias, bias_zero), S.depth[pix])) continue;
        const uint32_t slot = atomicAdd(s_nfrag, 1u);  // below F: the round was sized for every pixel
        S.fb0[slot] = b0;
        S.fb1[slot] = b1;
        S.fb2[slot] = b2;
        S.fz[slot] = z;
        S.fkey[slot] = ((uint32_t)pix << 16) | unit;
        unsigned short* hd = &S.head[bucket_of((uint32_t)pix)];
        unsigned short old = *hd, assumed;
        do {
            assumed = old;
            old = atomicCAS(hd, assumed, (unsigned short)slot);
        } while (old != assumed);
        S.nxt[slot] = old;
        if (old != 0xFFFFu) atomicOr(s_conflict, 1u);
    }
}

// ---------------------------------------------------------------------------
// Resolve
// ---------------------------------------------------------------------------
// The colour of the pixel a resolve thread is applying fragments to, held in
// a register between fragments of the same pixel: one load (when a blend
// needs it) and one store per pixel instead of a global read-modify-write
// per fragment. One thread applies all of a pixel's fragments, in order.
struct ColorCache {
    uint32_t* p;  // the cached pixel's colour, or null
    uint32_t v;
    bool loaded, dirty;
};
__device__ __forceinline__ void cc_flush(ColorCache& cc) {
    if (cc.p && cc.dirty) *cc.p = cc.v;
    cc.p = nullptr;
    cc.dirty = false;
}

__device__ __forceinline__ void apply_fragment(const RasterParams& P, const ItemView& I, const BandCtx& B,
                                               RasterSmem& S, uint32_t f, uint64_t& updated, ColorCache& cc) {
    const uint8_t fl = S.fflag[f];
    if (fl & kFragDiscard) return;
    const uint32_t key = S.fkey[f];
    const int pix = (int)(key >> 16);
    const int unit = (int)(key & 0xffff);
    const double z = S.fz[f];
    const double bz = add_bias(z, I.st.depth_bias, dbits(I.st.depth_bias) == 0);
    if (!I.st.read_depth || dle_i(bz, S.depth[pix])) {
        updated++;
        if (I.st.write_depth) S.depth[pix] = z;
        if (I.st.write_color) {
            // The colour buffer stays in global memory: the band is this
            // CTA's alone and one thread applies all of a pixel's fragments.
            uint32_t* cp = I.color + B.i0 + pix;
            if (cc.p != cp) {
                cc_flush(cc);
                cc.p = cp;
                cc.loaded = false;
            }
            if (fl & kFragBlend) {
                if (!cc.loaded) {
                    cc.v = *cp;
                    cc.loaded = true;
                }
                cc.v = blend_nrgba(cc.v, S.fcol[f]);
                cc.dirty = true;
            } else {
                // SetNRGBA(x, y, c) ignores points outside the image rectangle:
                // x = i - y*W with i = r0*W + pix
                const int32_t x = pix - (S.urow[unit] - B.r0) * I.W;
                if (x >= 0 && x < I.W) {
                    cc.v = S.fcol[f];
                    cc.loaded = true;
                    cc.dirty = true;
                }
            }
        }
        if (I.winner) {
            const uint32_t p = S.cprim[S.uslot[unit]];
            I.winner[B.i0 + pix] = P.prims[p].elem;
        }
        if (I.shaded) {
            const double* src = P.dbg + ((uint64_t)blockIdx.x * P.F + f) * 4;
            double* dst = I.shaded + (uint64_t)(B.i0 + pix) * 4;
            dst[0] = src[0];
            dst[1] = src[1];
            dst[2] = src[2];
            dst[3] = src[3];
        }
    }
}

template <int PREC>
__device__ __forceinline__ void shade_fragment(const RasterParams& P, const ItemView& I, RasterSmem& S, uint32_t f) {
    const uint32_t unit = S.fkey[f] & 0xffff;
    const RPrim& R = P.prims[S.cprim[S.uslot[unit]]];
    const double b0 = S.fb0[f], b1 = S.fb1[f], b2 = S.fb2[f];
    uint8_t fl = 0;
    uint32_t packed;
    double c[4];
    if (PREC == FGC_PRECISION_PLAIN) {
        D4 col = shade64(P, I, R, b0, b1, b2);
        c[0] = col.x; c[1] = col.y; c[2] = col.z; c[3] = col.w;
        if (dzero(col.x) && dzero(col.y) && dzero(col.z) && dzero(col.w)) fl |= kFragDiscard;
        if (I.st.alpha_blend && dlt1(col.w)) fl |= kFragBlend;
        packed = nrgba_pack_i(col.x, col.y, col.z, col.w);
    } else {
        float4 col = shade32(P, I, R, P.rf[S.cprim[S.uslot[unit]]], b0, b1, b2);
        c[0] = col.x; c[1] = col.y; c[2] = col.z; c[3] = col.w;
        if (col.x == 0 && col.y == 0 && col.z == 0 && col.w == 0) fl |= kFragDiscard;
        if (I.st.alpha_blend && col.w < 1) fl |= kFragBlend;
        packed = u8_of_unit_f32(col.x) | (u8_of_unit_f32(col.y) << 8) | (u8_of_unit_f32(col.z) << 16) |
                 (u8_of_unit_f32(col.w) << 24);
    }
    S.fcol[f] = packed;
    S.fflag[f] = fl;
    if (P.dbg) {
        double* dst = P.dbg + ((uint64_t)blockIdx.x * P.F + f) * 4;
        dst[0] = c[0];
        dst[1] = c[1];
        dst[2] = c[2];
        dst[3] = c[3];
    }
}

// Apply the chunk's fragments per pixel in (primitive, row) order. Every
// fragment was pushed onto its pixel bucket's list when it was recorded
// (head / nxt). Without collisions each list has one entry and all apply in
// parallel. Otherwise every fragment counts, on its bucket's list, the
// fragments of its own pixel with a smaller key (pixel, then unit): that
// rank goes into the upper bits of its flags, and rounds r = 0, 1, ... apply
// the fragments of rank r in parallel (one per pixel per round). A pixel
// with more fragments in the chunk than the rank field holds sends the chunk
// to the serial form: the thread holding a list's head applies the bucket's
// fragments by increasing key, selecting the next key from the list each
// time. The lists are emptied for the next chunk afterwards.
constexpr int kRankShift = 2;
constexpr uint32_t kRankMax = 62;

__device__ void resolve_chunk(const RasterParams& P, const ItemView& I, const BandCtx& B, RasterSmem& S,
                              uint32_t nfrag, bool conflict, uint64_t& updated, uint32_t* s_rank) {
    ColorCache cc{nullptr, 0u, false, false};
    if (!conflict) {
        for (uint32_t f = threadIdx.x; f < nfrag; f += blockDim.x) {
            apply_fragment(P, I, B, S, f, updated, cc);
            cc_flush(cc);
            S.head[bucket_of(S.fkey[f] >> 16)] = 0xFFFFu;
        }
        return;
    }
    if (threadIdx.x == 0) *s_rank = 0;
    __syncthreads();
    uint32_t mymax = 0;
    for (uint32_t f = threadIdx.x; f < nfrag; f += blockDim.x) {
        const uint32_t key = S.fkey[f], pix = key >> 16;
        uint32_t r = 0, steps = 0;
        // A list holds at most nfrag entries; every traversal is capped at
        // that, and a list that does not end within it is reported instead
        // of followed.
        for (uint32_t g = S.head[bucket_of(pix)]; g != 0xFFFFu && g < nfrag; g = S.nxt[g]) {
            if (++steps > nfrag) {
                atomicOr(P.status, ST_RASTER_INTERNAL);
                break;
            }
            const uint32_t k = S.fkey[g];
            r += ((k >> 16) == pix && k < key) ? 1u : 0u;
        }
        if (r > kRankMax + 1) r = kRankMax + 1;
        S.fflag[f] = (uint8_t)((S.fflag[f] & ((1u << kRankShift) - 1u)) | (r << kRankShift));
        mymax = max(mymax, r);
    }
    for (int o = 16; o > 0; o >>= 1) mymax = max(mymax, __shfl_xor_sync(0xffffffffu, mymax, o));
    if ((threadIdx.x & 31) == 0 && mymax) atomicMax(s_rank, mymax);
    __syncthreads();
    const uint32_t maxr = *s_rank;
    if (maxr <= kRankMax) {
        for (uint32_t r = 0; r <= maxr; r++) {
            for (uint32_t f = threadIdx.x; f < nfrag; f += blockDim.x) {
                if ((uint32_t)(S.fflag[f] >> kRankShift) == r) {
                    apply_fragment(P, I, B, S, f, updated, cc);
                    cc_flush(cc);
                }
            }
            __syncthreads();
        }
        for (uint32_t f = threadIdx.x; f < nfrag; f += blockDim.x) S.head[bucket_of(S.fkey[f] >> 16)] = 0xFFFFu;
        return;
    }
    for (uint32_t f = threadIdx.x; f < nfrag; f += blockDim.x) {
        const uint32_t pix = bucket_of(S.fkey[f] >> 16);  // the bucket
        if (S.head[pix] != f) continue;  // not the list head
        uint32_t last = 0;               // keys in a bucket are distinct
        bool first = true;
        for (uint32_t picked = 0; picked < nfrag; picked++) {
            uint32_t best = 0xFFFFFFFFu, bestf = 0xFFFFu, steps = 0;
            for (uint32_t g = f; g != 0xFFFFu && g < nfrag; g = S.nxt[g]) {
                if (++steps > nfrag) {
                    atomicOr(P.status, ST_RASTER_INTERNAL);
                    break;
                }
                const uint32_t k = S.fkey[g];
                if ((first || k > last) && k < best) {
                    best = k;
                    bestf = g;
                }
            }
            if (bestf == 0xFFFFu) break;
            apply_fragment(P, I, B, S, bestf, updated, cc);
            last = best;
            first = false;
        }
        cc_flush(cc);
    }
    __syncthreads();  // every list walked before any head is cleared
    for (uint32_t f = threadIdx.x; f < nfrag; f += blockDim.x) S.head[bucket_of(S.fkey[f] >> 16)] = 0xFFFFu;
}

// ---------------------------------------------------------------------------
// Kernel
// ---------------------------------------------------------------------------
__device__ __forceinline__ void rows_in_band(const PBox& bx, int32_t W, const BandCtx& B, int32_t& ylo,
                                             int32_t& nrows) {
    // Rows y of the box whose index range [y*W + x0, y*W + x1] meets the
    // band's [r0*W, rend*W): y*W + x1 >= r0*W gives y >= r0 - floor(x1/W),
    // y*W + x0 < rend*W gives y <= rend - 1 - floor(x0/W).
    if (bx.x0 > bx.x1) {
        ylo = 0;
        nrows = 0;
        return;
    }
    int64_t a = (int64_t)B.r0 - floordiv_w(bx.x1, W);
    int64_t b = (int64_t)B.rend - 1 - floordiv_w(bx.x0, W);
    if (a < bx.y0) a = bx.y0;
    if (b > bx.y1) b = bx.y1;
    ylo = (int32_t)a;
    nrows = (b >= a) ? (int32_t)(b - a + 1) : 0;
}

// Add the CTA's counters of one draw to the draw's totals and reset them
// (all threads of the CTA call it together).
__device__ __forceinline__ void flush_counters(const RasterParams& P, uint32_t item, uint64_t& tot, uint64_t& upd,
                                               uint64_t& vis, uint64_t& shd) {
    for (int o = 16; o > 0; o >>= 1) {
        tot += __shfl_down_sync(0xffffffffu, tot, o);
        upd += __shfl_down_sync(0xffffffffu, upd, o);
        vis += __shfl_down_sync(0xffffffffu, vis, o);
        shd += __shfl_down_sync(0xffffffffu, shd, o);
    }
    if ((threadIdx.x & 31) == 0 && item < P.nitems) {
        unsigned long long* info = P.iout[item].info;
        if (tot) atomicAdd(&info[0], (unsigned long long)tot);
        if (upd) atomicAdd(&info[1], (unsigned long long)upd);
        if (vis) atomicAdd(&info[2], (unsigned long long)vis);
        if (shd) atomicAdd(&info[3], (unsigned long long)shd);
    }
    tot = upd = vis = shd = 0;
}

// One bin entry as the chunk builder sees it: the primitive, its rows in the
// band, a bound on its covered in-band pixels (rows x the widest chord, or x
// the box width) and whether its box is narrow enough for the direct walk.
struct ChunkEntry {
    uint32_t p;
    int32_t ylo, nrows;
    uint32_t bound;  // capped at 2^31 - 1
    bool narrow;
};

// A bin entry's primitive, box and widest chord, loaded ahead of its chunk.
struct EntryLoad {
    uint32_t p, span;
    PBox box;
};
__device__ __forceinline__ EntryLoad load_entry(const RasterParams& P, uint64_t at) {
    EntryLoad l;
    l.p = P.bins[at];
    l.box = P.pbox[l.p];
    l.span = P.pspan[l.p];
    return l;
}

__device__ __forceinline__ ChunkEntry chunk_entry(const ItemView& I, const BandCtx& B, const EntryLoad& l,
                                                  bool box_bound, uint32_t roff) {
    ChunkEntry c;
    c.p = l.p;
    const PBox bx = l.box;
    rows_in_band(bx, I.W, B, c.ylo, c.nrows);
    c.ylo += (int32_t)roff;  // rows an earlier chunk took
    c.nrows -= (int32_t)roff;
    int64_t wid = (int64_t)bx.x1 - bx.x0 + 1;
    c.narrow = wid <= kNarrow;
    if (!box_bound && (int64_t)l.span < wid) wid = l.span;
    if (wid > B.npx) wid = B.npx;
    if (wid < 0) wid = 0;
    const uint64_t bound = (uint64_t)c.nrows * (uint64_t)wid;
    c.bound = bound < 0x7FFFFFFFull ? (uint32_t)bound : 0x7FFFFFFFu;
    return c;
}

// Fragment estimates are the bound scaled by ratio / kRatioOne.
constexpr uint32_t kRatioOne = 256;
constexpr uint32_t kRatioMin = 16;

// The entry's share of a chunk's fragment budget F: its scaled bound in a
// direct chunk (F + 1 for a wide primitive, which ends the chunk before it),
// nothing in a span chunk (bounded by units instead).
__device__ __forceinline__ uint64_t chunk_key(const ChunkEntry& c, bool direct, uint32_t ratio, int F) {
    if (!direct) return 0;
    if (!c.narrow) return (uint64_t)F + 1;
    return ((uint64_t)c.bound * ratio + (kRatioOne - 1)) / kRatioOne;
}

// The ratio for the next chunk: twice the share of bounded pixels that
// became fragments in this one, not below half the previous ratio.
__device__ __forceinline__ uint32_t next_ratio(uint32_t prev, uint32_t nfrag, uint32_t bsum) {
    if (bsum == 0) return prev;
    uint64_t r = ((uint64_t)nfrag * 2 * kRatioOne + bsum - 1) / bsum;
    if (r < prev / 2) r = prev / 2;
    if (r < kRatioMin) r = kRatioMin;
    if (r > kRatioOne) r = kRatioOne;
    return (uint32_t)r;
}

template <int PREC>
__global__ void __launch_bounds__(kRT, 2) raster_kernel(RasterParams P) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int F = P.F;
    RasterSmem S;
    {
        unsigned char* q = smem_raw;
        S.depth = (double*)q; q += (size_t)P.Lmax * 8;
        S.fb0 = (double*)q; q += (size_t)F * 8;
        S.fb1 = (double*)q; q += (size_t)F * 8;
        S.fb2 = (double*)q; q += (size_t)F * 8;
        S.fz = (double*)q; q += (size_t)F * 8;
        S.uw0 = (double*)q; q += (size_t)P.su * 8;
        S.uw1 = (double*)q; q += (size_t)P.su * 8;
        S.uw2 = (double*)q; q += (size_t)P.su * 8;
        S.scratch = (unsigned long long*)q; q += 64 * 8;
        S.fkey = (uint32_t*)q; q += (size_t)F * 4;
        S.fcol = (uint32_t*)q; q += (size_t)F * 4;
        S.uslot = (uint32_t*)q; q += (size_t)F * 4;
        S.urow = (int32_t*)q; q += (size_t)F * 4;
        S.ux = (int32_t*)q; q += (size_t)P.su * 4;
        S.ucnt = (uint32_t*)q; q += (size_t)P.su * 4;
        S.ufrag = (uint32_t*)q; q += (size_t)P.su * 4;
        S.cprim = (uint32_t*)q; q += kChunkPrims * 4;
        S.head = (unsigned short*)q; q += (size_t)kRasterHeads * 2;
        S.nxt = (unsigned short*)q; q += (size_t)F * 2;
        S.fflag = (uint8_t*)q;
    }
    __shared__ uint32_t s_band, s_item, s_nfrag, s_conflict, s_nprim, s_nunit, s_ftotal, s_mode, s_bsum, s_ratio, s_split,
        s_rank;
    __shared__ uint64_t s_warp[kRT / 32 + 1];
    __shared__ ItemView s_iv;  // the draw of the current band
    const ItemView& I = s_iv;

    if (*P.status & (ST_CLIP_OVERFLOW | ST_BIN_OVERFLOW | ST_LOOKBACK_TIMEOUT | ST_POOL_OVERFLOW)) return;

    const uint64_t pair_total = *P.pair_total;
    uint64_t tot = 0, upd = 0, vis = 0, shd = 0;
    uint32_t cur = 0xFFFFFFFFu;  // the draw tot..shd count for

    for (;;) {
        // the next band of the pass: bands run draw by draw, band by band
        if (threadIdx.x == 0) {
            const uint32_t g = atomicAdd(P.band_counter, 1u);
            s_band = g;
            s_item = (g < P.nbands) ? find_item(P.starts.band, P.nitems, g) : 0xFFFFFFFFu;
        }
        __syncthreads();
        const uint32_t gband = s_band;
        const uint32_t item = s_item;
        if (gband >= P.nbands) break;
        if (item != cur) {
            flush_counters(P, cur, tot, upd, vis, shd);
            cur = item;
            const uint4* src = reinterpret_cast<const uint4*>(&P.items[item]);
            uint4* dst = reinterpret_cast<uint4*>(&s_iv);
            for (int j = threadIdx.x; j < (int)(sizeof(ItemView) / 16); j += blockDim.x) dst[j] = src[j];
            if (threadIdx.x == 0) s_ratio = kRatioOne;
        }
        __syncthreads();
        const uint32_t band = gband - I.band0;
        const uint64_t bstart = P.off[I.mat0 + (uint64_t)band * I.nblk];
        const uint64_t mend = I.mat0 + (uint64_t)(band + 1) * I.nblk;  // the next band's (or draw's) first entry
        const uint64_t bend = (mend < P.nmat) ? P.off[mend] : pair_total;
        const uint64_t bcount = bend - bstart;
        if (bcount == 0 && !I.clear_color_pending && !I.clear_depth_pending) continue;
        BandCtx B;
        B.r0 = (int32_t)band * I.R;
        B.rend = min(B.r0 + I.R, I.H);
        B.i0 = (int64_t)B.r0 * I.W;
        B.npx = (B.rend - B.r0) * I.W;
        B.band = band;
        B.early = I.st.read_depth && (!I.st.write_depth || I.st.depth_bias >= 0);
        const int npx = B.npx;
        for (int j = threadIdx.x; j < npx; j += blockDim.x) {
            S.depth[j] = I.clear_depth_pending ? I.clear_depth : I.depth[B.i0 + j];
            if (I.clear_color_pending) I.color[B.i0 + j] = I.clear_color;  // fused clear
        }
        for (int j = threadIdx.x; j < kRasterHeads; j += blockDim.x) S.head[j] = 0xFFFFu;
        __syncthreads();

        uint64_t k = 0;
        uint64_t pf_at = ~0ull;  // bin entry (band-relative) whose loads pf holds
        EntryLoad pf;
        uint32_t roff = 0;  // rows of the entry at k taken by earlier chunks
        int level = 0;      // 0: estimated fragments, 1: widest-chord bound, 2: box bound
        while (k < bcount) {
            // ---- chunk: a prefix of the remaining bin; thread t examines
            // entries k + kChunkPer*t + j. The first primitive picks how the
            // chunk is walked:
            //   direct  narrow primitives, each row walked and recorded by one
            //           thread as rasterize does, up to F units. The prefix
            //           keeps an estimate of its fragments within F: at level
            //           0 the bound (rows x widest chord) scaled by the share
            //           of bounded pixels that became fragments in earlier
            //           chunks (early depth rejection makes it small); a walk
            //           that outgrows F is redone at level 1 with the bound
            //           itself, then at level 2 with the box width
            //   spans   anything else, at most P.su units: spans, then
            //           windows of fragment offsets
            // An entry with more rows in the band than its chunk holds (rows
            // that wrap around the frame's sides) goes alone, its rows over
            // several chunks.
            const uint64_t e0 = k + (uint64_t)threadIdx.x * kChunkPer;
            ChunkEntry ce[kChunkPer];
#pragma unroll
            for (int j = 0; j < kChunkPer; j++) {
                if (e0 + j < bcount) {
                    const EntryLoad l = (j == 0 && pf_at == e0) ? pf : load_entry(P, bstart + e0 + j);
                    ce[j] = chunk_entry(I, B, l, level == 2, (e0 + j == k) ? roff : 0u);
                } else {
                    ce[j] = ChunkEntry{0, 0, 0, 0, true};
                }
            }
            if (threadIdx.x == 0) {
                const bool dm = ce[0].narrow && ce[0].bound <= (uint32_t)F;
                // a direct chunk holds at most one unit per thread: a second
                // pass over the units would double its first warps' walk
                const uint32_t cap0 = dm ? (uint32_t)min(F, kRT) : (uint32_t)P.su;
                s_mode = dm ? 1u : 0u;
                s_split = ((uint32_t)ce[0].nrows > cap0) ? cap0 : 0u;
                s_nprim = 0;
                s_nunit = 0;
                s_bsum = 0;
            }
            __syncthreads();
            const bool direct = s_mode != 0;
            const uint32_t split = s_split;  // rows of the entry at k this chunk takes, when it goes alone
            const uint32_t ratio = level == 0 ? s_ratio : kRatioOne;
            const uint64_t ucap = direct ? (uint64_t)min(F, kRT) : (uint64_t)P.su;
            const int jmax = split ? (threadIdx.x == 0 ? 1 : 0) : kChunkPer;
            if (split && threadIdx.x == 0) ce[0].nrows = (int32_t)split;
            // the fragment estimates and the units in one scan (estimates in
            // the high half, units in the low half). An entry whose estimate
            // is above F, or whose rows are more than the chunk's units, ends
            // the chunk wherever it stands, so each value is capped at one
            // above its limit: every comparison below is unchanged, and both
            // sums stay far below 2^32 (256 entries per chunk)
            uint64_t tkey = 0, tun = 0;
#pragma unroll
            for (int j = 0; j < kChunkPer; j++) {
                if (j >= jmax) break;
                tkey += min(chunk_key(ce[j], direct, ratio, F), (uint64_t)F + 1);
                tun += min((uint64_t)ce[j].nrows, ucap + 1);
            }
            uint64_t pagg;
            const uint64_t pr = block_exclusive_scan<kRT>((tkey << 32) | tun, s_warp, &pagg);
            uint64_t kr = pr >> 32, ur = pr & 0xffffffffull;
            // the entries inside the prefix (never empty: the first entry's
            // rows fit, and a direct chunk's first estimate is at most its
            // bound <= F)
            {
                const uint64_t ur0 = ur;
                uint32_t took = 0, bsum = 0;
#pragma unroll
                for (int j = 0; j < kChunkPer; j++) {
                    if (j >= jmax) break;
                    const uint64_t key = min(chunk_key(ce[j], direct, ratio, F), (uint64_t)F + 1);
                    if (e0 + j >= bcount || ur + (uint64_t)ce[j].nrows > ucap || kr + key > (uint64_t)F) break;
                    const uint32_t slot = threadIdx.x * kChunkPer + j;
                    S.cprim[slot] = ce[j].p;
                    for (int r = 0; r < ce[j].nrows; r++) {
                        S.uslot[ur + r] = slot;
                        S.urow[ur + r] = ce[j].ylo + r;
                    }
                    kr += key;
                    ur += (uint64_t)ce[j].nrows;
                    took++;
                    bsum += min(ce[j].bound, (uint32_t)F);
                }
                if (took) {
                    atomicAdd(&s_nprim, took);
                    atomicAdd(&s_nunit, (uint32_t)(ur - ur0));
                    atomicAdd(&s_bsum, bsum);
                }
            }
            __syncthreads();
            const uint32_t nprim = s_nprim, nunit = s_nunit;

            if (direct) {
                if (threadIdx.x == 0) {
                    s_nfrag = 0;
                    s_conflict = 0;
                }
                __syncthreads();
                uint64_t tchunk = 0;
                if (P.su >= kRT) {
                    // the span arrays hold a 32-entry queue per warp: every
                    // thread takes part, a unit each (nunit <= kRT here)
                    const uint32_t u = threadIdx.x;
                    const bool has = u < nunit;
                    const uint32_t pp = has ? S.cprim[S.uslot[u]] : 0u;
                    tchunk += walk_rows_queued(has, pp, P.prims[pp], P.pbox[pp], has ? S.urow[u] : 0, P, I, B, S, u,
                                               &s_nfrag, &s_conflict, vis);
                } else {
                    for (uint32_t u = threadIdx.x; u < nunit; u += blockDim.x) {
                        const uint32_t pp = S.cprim[S.uslot[u]];
                        tchunk += walk_row(pp, P.prims[pp], P.pbox[pp], S.urow[u], P, I, B, S, u, &s_nfrag,
                                           &s_conflict, vis);
                    }
                }
                {
                    // the next chunk's entries load during this one's shading
                    // and resolve (a redone chunk reloads)
                    const uint64_t nk = (split ? k : k + nprim) + threadIdx.x;
                    if (nk < bcount) {
                        pf = load_entry(P, bstart + nk);
                        pf_at = nk;
                    }
                }
                __syncthreads();
                const bool redo = (s_conflict & 2u) != 0;
                if (redo) {  // nothing was applied: empty the lists, redo with a safer bound
                    const uint32_t nrec = min(s_nfrag, (uint32_t)F);
                    for (uint32_t f = threadIdx.x; f < nrec; f += blockDim.x)
                        S.head[bucket_of(S.fkey[f] >> 16)] = 0xFFFFu;
                    if (threadIdx.x == 0) s_ratio = kRatioOne;
                } else {
                    tot += tchunk;
                    const uint32_t nfrag = s_nfrag;
                    if (threadIdx.x == 0) {
                        shd += nfrag;
                        s_ratio = next_ratio(s_ratio, nfrag, s_bsum);
                    }
                    for (uint32_t f = threadIdx.x; f < nfrag; f += blockDim.x) shade_fragment<PREC>(P, I, S, f);
                    __syncthreads();
                    resolve_chunk(P, I, B, S, nfrag, (s_conflict & 1u) != 0, upd, &s_rank);
                }
                __syncthreads();
                if (redo && level < 2) {
                    level++;
                    continue;
                }
                if (redo && threadIdx.x == 0) atomicOr(P.status, ST_RASTER_INTERNAL);
                level = 0;
                if (split) {
                    roff += split;
                } else {
                    k += nprim;
                    roff = 0;
                }
                continue;
            }
            level = 0;

            // ---- spans: each unit's covered in-band pixels
            for (uint32_t u = threadIdx.x; u < nunit; u += blockDim.x) {
                const uint32_t pp = S.cprim[S.uslot[u]];
                const RPrim& R = P.prims[pp];
                const PBox bx = P.pbox[pp];
                double w00, w01, w02;
                row_start(P, pp, R, bx, S.urow[u], I, B, w00, w01, w02);
                const Span sp = row_span(R, bx, S.urow[u], w00, w01, w02, B.r0, B.npx, I.W, vis);
                S.ux[u] = sp.xa;
                S.ucnt[u] = (uint32_t)sp.cnt;
                S.uw0[u] = sp.w0;
                S.uw1[u] = sp.w1;
                S.uw2[u] = sp.w2;
                tot += (uint64_t)sp.cnt;
            }
            {
                const uint64_t nk = (split ? k : k + nprim) + threadIdx.x;  // loads during the rounds
                if (nk < bcount) {
                    pf = load_entry(P, bstart + nk);
                    pf_at = nk;
                }
            }
            __syncthreads();
            // ---- fragment offsets of the units, in unit order
            {
                const uint32_t per = ((uint32_t)P.su + kRT - 1) / kRT;
                const uint32_t u0 = threadIdx.x * per;
                uint64_t local = 0;
                for (uint32_t j = 0; j < per; j++)
                    if (u0 + j < nunit) local += S.ucnt[u0 + j];
                uint64_t ftotal;
                uint64_t run = block_exclusive_scan<kRT>(local, s_warp, &ftotal);
                for (uint32_t j = 0; j < per; j++) {
                    if (u0 + j < nunit) {
                        S.ufrag[u0 + j] = (uint32_t)run;
                        run += S.ucnt[u0 + j];
                    }
                }
                if (threadIdx.x == 0) s_ftotal = (uint32_t)ftotal;
            }
            __syncthreads();
            const uint32_t ftotal = s_ftotal;

            // ---- rounds: fragment offsets [base, base + F), in unit order,
            // so that a pixel's fragments of earlier units are applied first
            for (uint32_t base = 0; base < ftotal; base += (uint32_t)F) {
                if (threadIdx.x == 0) {
                    s_nfrag = 0;
                    s_conflict = 0;
                }
                __syncthreads();
                const uint32_t rend = min(base + (uint32_t)F, ftotal);
                const uint32_t win = (uint32_t)P.win;  // fragment offsets one thread walks
                for (uint32_t w0 = base + threadIdx.x * win; w0 < rend; w0 += blockDim.x * win) {
                    const uint32_t w1 = min(w0 + win, rend);
                    // the unit holding offset w0: the last one starting at or before it
                    uint32_t lo = 0, hi = nunit - 1;
                    while (lo < hi) {
                        const uint32_t mid = (lo + hi + 1) >> 1;
                        if (S.ufrag[mid] <= w0) lo = mid;
                        else hi = mid - 1;
                    }
                    uint32_t u = lo, off = w0;
                    while (off < w1) {
                        const uint32_t fu = S.ufrag[u], cnt = S.ucnt[u];
                        const uint32_t o = off - fu;
                        const uint32_t len = min(w1 - off, fu + cnt - off);
                        const uint32_t pp = S.cprim[S.uslot[u]];
                        const RPrim& R = P.prims[pp];
                        double e0 = S.uw0[u], e1 = S.uw1[u], e2 = S.uw2[u];
                        if (o) {  // the edge values o steps further along the row
                            e0 = repeat_add(e0, R.a0, o);
                            e1 = repeat_add(e1, R.a1, o);
                            e2 = repeat_add(e2, R.a2, o);
                        }
                        const int32_t pix = (S.urow[u] - B.r0) * I.W + S.ux[u] + (int32_t)o;
                        emit_segment(R, I, B, S, pix, (int32_t)len, e0, e1, e2, u, &s_nfrag, &s_conflict);
                        vis += len;
                        off += len;
                        u++;
                    }
                }
                __syncthreads();
                const uint32_t nfrag = s_nfrag;
                if (threadIdx.x == 0) shd += nfrag;
                for (uint32_t f = threadIdx.x; f < nfrag; f += blockDim.x) shade_fragment<PREC>(P, I, S, f);
                __syncthreads();
                resolve_chunk(P, I, B, S, nfrag, (s_conflict & 1u) != 0, upd, &s_rank);
                __syncthreads();
            }
            if (split) {
                roff += split;
            } else {
                k += nprim;
                roff = 0;
            }
        }
        for (int j = threadIdx.x; j < npx; j += blockDim.x) I.depth[B.i0 + j] = S.depth[j];
        __syncthreads();
    }
    flush_counters(P, cur, tot, upd, vis, shd);
}

const void* raster_kernel_ptr(int precision) {
    return precision == FGC_PRECISION_MIXED ? (const void*)raster_kernel<FGC_PRECISION_MIXED>
                                            : (const void*)raster_kernel<FGC_PRECISION_PLAIN>;
}

cudaError_t launch_raster(int precision, int grid, int threads, size_t smem, cudaStream_t stream,
                          const RasterParams& P) {
    if (precision == FGC_PRECISION_MIXED)
        raster_kernel<FGC_PRECISION_MIXED><<<grid, threads, smem, stream>>>(P);
    else
        raster_kernel<FGC_PRECISION_PLAIN><<<grid, threads, smem, stream>>>(P);
    return cudaGetLastError();
}

}  // namespace fgc
