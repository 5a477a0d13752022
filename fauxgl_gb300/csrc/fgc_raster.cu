// fgc_raster.cu -- band rasteriser: fragment generation, shading and ordered
// depth/colour resolve, one CTA per band, no framebuffer atomics.
//
// Reference: rasterize (context.go:151-281), InterpolateVertexes
// (vertex.go:18-47), the built-in Fragment shaders (shader.go:25-27, 44-46,
// 75-96), BilinearSample (texture.go:41-63), Color.NRGBA (color.go:56-63).
//
// A persistent CTA takes bands from an atomic counter. A band's depth and
// colour live in shared memory while its bin (raster primitives in
// submission order) is processed in chunks:
//   A1 walk   one thread per (primitive, row) unit replays rasterize's row
//             loop exactly: the row's edge values are the serial sum of the
//             per-row increments, the skip-ahead d, then the serial per-pixel
//             adds with the inside test and the break after leaving the
//             triangle. Every covered pixel of the band becomes a fragment
//             (b0, b1, b2, z); an early depth test against the band's current
//             depth drops fragments that cannot update (only when depth can
//             only decrease during the draw).
//   A2 shade  one thread per fragment: perspective-correct weights,
//             interpolation and the built-in shader, in FP64 (plain) or FP32
//             (mixed).
//   resolve   fragments are applied per pixel in (primitive, row) order:
//             directly when no two fragments of the chunk share a pixel,
//             otherwise after a bitonic sort of (pixel, unit) keys, each
//             pixel's run applied by one thread in order. The depth test,
//             UpdatedPixels, depth write and the NRGBA / alpha-blend colour
//             write are exactly rasterize's (context.go:247-272).
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
    uint32_t* uslot; // [F] unit -> chunk slot, flags in bits 24..
    int32_t* urow;   // [F] unit -> row y
    uint32_t* cprim; // [kRT] chunk slot -> primitive
    int32_t* cylo;   // [kRT]
    int32_t* cnrow;  // [kRT]
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
    double n = __dadd_rn(0.0, __dmul_rn(a, w.x));
    n = __dadd_rn(n, __dmul_rn(b, w.y));
    n = __dadd_rn(n, __dmul_rn(c, w.z));
    return __dmul_rn(n, w.w);
}

// ---------------------------------------------------------------------------
// FP64 shading (plain form)
// ---------------------------------------------------------------------------
__device__ __forceinline__ D4 tex_at64(const TexView& t, int64_t x, int64_t y) {
    if (x < 0 || y < 0 || x >= t.w || y >= t.h) return d4(0, 0, 0, 0);
    ushort4 p = t.texels[(uint64_t)y * (uint64_t)t.w + (uint64_t)x];
    const double d = 65535.0;
    return d4(__ddiv_rn((double)p.x, d), __ddiv_rn((double)p.y, d), __ddiv_rn((double)p.z, d),
              __ddiv_rn((double)p.w, d));
}

__device__ D4 bilinear64(const TexView& t, double u, double v) {  // texture.go:41-63
    v = __dsub_rn(1.0, v);
    u = __dsub_rn(u, floor(u));
    v = __dsub_rn(v, floor(v));
    double x = __dmul_rn(u, (double)(t.w - 1));
    double y = __dmul_rn(v, (double)(t.h - 1));
    int64_t x0 = go_f2i(x), y0 = go_f2i(y);
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
    D3 pos = d3(interp1(p0.x, p1.x, p2.x, w), interp1(p0.y, p1.y, p2.y, w), interp1(p0.z, p1.z, p2.z, w));
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
    D4 light = d4(S.ambient[0], S.ambient[1], S.ambient[2], S.ambient[3]);
    double diffuse = go_max0(dot3(nrm, L));
    light = add4(light, muls4(d4(S.diffuse[0], S.diffuse[1], S.diffuse[2], S.diffuse[3]), diffuse));
    if (dgt0(diffuse) && S.power > 0) {
        D3 camera = normalize3(sub3(d3(S.eye[0], S.eye[1], S.eye[2]), pos));
        D3 negl = d3(-L.x, -L.y, -L.z);
        D3 reflected = sub3(negl, muls3(nrm, __dmul_rn(2.0, dot3(nrm, negl))));  // Reflect, vector.go:175-177
        double specular = go_max0(dot3(camera, reflected));
        if (dgt0(specular)) {
            specular = go_pow(specular, S.power);
            light = add4(light, muls4(d4(S.specular[0], S.specular[1], S.specular[2], S.specular[3]), specular));
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
        const PoolVertex& q = P.pool[v & ~kPoolFlag];
        pos = F3{(float)q.px, (float)q.py, (float)q.pz};
        nrm = F3{(float)q.nx, (float)q.ny, (float)q.nz};
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

__device__ float4 shade32(const RasterParams& P, const ItemView& I, const RPrim& R, double b0, double b1, double b2) {
    const ShaderView& S = I.sh;
    const MeshView& M = I.mesh;
    if (S.kind == FGC_SHADER_SOLID_COLOR)
        return make_float4((float)S.color[0], (float)S.color[1], (float)S.color[2], (float)S.color[3]);
    float wx = (float)b0 * (float)R.r0, wy = (float)b1 * (float)R.r1, wz = (float)b2 * (float)R.r2;
    float ww = 1.0f / (wx + wy + wz);
    float4 color;
    bool have_color = false;
    if (S.kind == FGC_SHADER_TEXTURE || S.has_texture) {
        float u[3], v[3];
        uint32_t vr[3] = {R.v0, R.v1, R.v2};
        for (int k = 0; k < 3; k++) {
            if (vr[k] & kPoolFlag) {
                const PoolVertex& q = P.pool[vr[k] & ~kPoolFlag];
                u[k] = (float)q.tu;
                v[k] = (float)q.tv;
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
                    const PoolVertex& q = P.pool[vr[k] & ~kPoolFlag];
                    c[k][0] = (float)q.cr; c[k][1] = (float)q.cg; c[k][2] = (float)q.cb; c[k][3] = (float)q.ca;
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
            color = make_float4((float)S.color[0], (float)S.color[1], (float)S.color[2], (float)S.color[3]);
        }
    }
    F3 L = F3{(float)S.light[0], (float)S.light[1], (float)S.light[2]};
    float lr = (float)S.ambient[0], lg = (float)S.ambient[1], lb = (float)S.ambient[2];
    float nl = dotf3(nrm, L);
    float diffuse = (nl > 0.0f) ? nl : ((nl != nl) ? nl : 0.0f);
    lr = __fmaf_rn((float)S.diffuse[0], diffuse, lr);
    lg = __fmaf_rn((float)S.diffuse[1], diffuse, lg);
    lb = __fmaf_rn((float)S.diffuse[2], diffuse, lb);
    if (diffuse > 0 && S.power > 0) {
        F3 cam = normf3(F3{(float)S.eye[0] - pos.x, (float)S.eye[1] - pos.y, (float)S.eye[2] - pos.z});
        F3 negl = F3{-L.x, -L.y, -L.z};
        float k = 2.0f * dotf3(nrm, negl);
        F3 refl = F3{negl.x - nrm.x * k, negl.y - nrm.y * k, negl.z - nrm.z * k};
        float sp = dotf3(cam, refl);
        if (sp > 0) {
            sp = powf_int_or_general(sp, (float)S.power);
            lr = __fmaf_rn((float)S.specular[0], sp, lr);
            lg = __fmaf_rn((float)S.specular[1], sp, lg);
            lb = __fmaf_rn((float)S.specular[2], sp, lb);
        }
    }
    return make_float4(fminf(color.x * lr, 1.0f), fminf(color.y * lg, 1.0f), fminf(color.z * lb, 1.0f), color.w);
}

__device__ __forceinline__ uint32_t u8_of_unit_f32(float c) {
    float v = fminf(fmaxf(c, 0.0f), 1.0f) * 255.0f;
    return (c == c) ? ((uint32_t)v & 0xff) : 0u;
}

// ---------------------------------------------------------------------------
// Row walk (context.go:184-278)
// ---------------------------------------------------------------------------
// A row walk in 32-bit band-relative coordinates: the pixel at x of the row
// is band pixel rel + x, rel = (y - r0) * W. For a row that meets the band
// (rows_in_band) and a box within the setup limits (|coordinates| <= 2^30,
// extent <= 2^26), rel and rel + x stay far inside the int32 range.
struct Walk {
    int32_t x, x1, rel;
    double w0, w1, w2;
    int32_t unit;
    bool was, done;
};

__device__ __forceinline__ void walk_init(Walk& s, const RPrim& R, const PBox& bx, int32_t y, const BandCtx& B,
                                          int32_t W, int32_t unit) {
    double w00 = R.w0, w01 = R.w1, w02 = R.w2;
    for (int32_t j = bx.y0; j < y; j++) {  // w00 += b12 at the end of each earlier row
        w00 = __dadd_rn(w00, R.b0);
        w01 = __dadd_rn(w01, R.b1);
        w02 = __dadd_rn(w02, R.b2);
    }
    double d = 0;
    double d0 = __dmul_rn(-w00, R.q0);
    double d1 = __dmul_rn(-w01, R.q1);
    double d2 = __dmul_rn(-w02, R.q2);
    if (w00 < 0 && d0 > d) d = d0;
    if (w01 < 0 && d1 > d) d = d1;
    if (w02 < 0 && d2 > d) d = d2;
    int64_t di = go_f2i(d);  // d = float64(int(d)); if d < 0 { d = 0 }
    if (di < 0) di = 0;
    s.unit = unit;
    s.was = false;
    s.x1 = bx.x1;
    s.rel = (y - B.r0) * W;
    if (di > (int64_t)bx.x1 - bx.x0) {  // the row loop starts past x1
        s.x = bx.x1 + 1;
        s.done = true;
        return;
    }
    d = (double)di;
    s.w0 = __dadd_rn(w00, __dmul_rn(R.a0, d));
    s.w1 = __dadd_rn(w01, __dmul_rn(R.a1, d));
    s.w2 = __dadd_rn(w02, __dmul_rn(R.a2, d));
    s.x = bx.x0 + (int32_t)di;
    s.done = false;
}

// Advance a walk, recording up to quota fragments. Returns the number of
// covered in-band pixels (TotalPixels).
__device__ __forceinline__ uint32_t walk_run(Walk& s, const RPrim& R, const RasterParams& P, const ItemView& I,
                                             const BandCtx& B, RasterSmem& S, uint32_t* s_nfrag,
                                             uint32_t* s_conflict, int quota, uint64_t& visited) {
    uint32_t total = 0;
    int rec = 0;
    const double bias = I.st.depth_bias;
    const double ra = R.ra;
    const RaSign rs = ra_sign(ra);
    while (s.x <= s.x1) {
        // b_k = w_k * ra is negative exactly when neg_product says so; the
        // products themselves are formed only for pixels that are used.
        const double w0 = s.w0, w1 = s.w1, w2 = s.w2;
        s.w0 = __dadd_rn(w0, R.a0);
        s.w1 = __dadd_rn(w1, R.a1);
        s.w2 = __dadd_rn(w2, R.a2);
        const int32_t x = s.x++;
        visited++;
        if (neg_product(w0, ra, rs) || neg_product(w1, ra, rs) || neg_product(w2, ra, rs)) {
            if (s.was) {
                s.done = true;
                return total;
            }
            continue;
        }
        s.was = true;
        // i = y*W + x is skipped outside [0, W*H) (context.go:223-228); here
        // only this band's part of that range is drawn
        const int32_t pix = s.rel + x;
        if (pix >= B.npx) {  // beyond this band (and possibly the frame): no later pixel of the row is in it
            s.done = true;
            return total;
        }
        if (pix < 0) continue;
        total++;
        const double b0 = __dmul_rn(w0, ra);
        const double b1 = __dmul_rn(w1, ra);
        const double b2 = __dmul_rn(w2, ra);
        double z = __dadd_rn(__dadd_rn(__dmul_rn(b0, R.z0), __dmul_rn(b1, R.z1)), __dmul_rn(b2, R.z2));
        if (B.early && __dadd_rn(z, bias) > S.depth[pix]) continue;
        uint32_t slot = atomicAdd(s_nfrag, 1u);
        if (slot >= (uint32_t)P.F) {  // the chunk's size bound did not hold: the chunk is redone
            atomicOr(s_conflict, 2u);
            continue;
        }
        S.fb0[slot] = b0;
        S.fb1[slot] = b1;
        S.fb2[slot] = b2;
        S.fz[slot] = z;
        S.fkey[slot] = ((uint32_t)pix << 16) | (uint32_t)s.unit;
        // push onto the pixel's bucket list; a non-empty list means a
        // possible conflict (same pixel or same bucket)
        unsigned short* hd = &S.head[bucket_of((uint32_t)pix)];
        unsigned short old = *hd, assumed;
        do {
            assumed = old;
            old = atomicCAS(hd, assumed, (unsigned short)slot);
        } while (old != assumed);
        S.nxt[slot] = old;
        if (old != 0xFFFFu) atomicOr(s_conflict, 1u);
        if (++rec == quota) return total;
    }
    s.done = true;
    return total;
}

// ---------------------------------------------------------------------------
// Resolve
// ---------------------------------------------------------------------------
__device__ __forceinline__ void apply_fragment(const RasterParams& P, const ItemView& I, const BandCtx& B,
                                               RasterSmem& S, uint32_t f, uint64_t& updated) {
    const uint8_t fl = S.fflag[f];
    if (fl & kFragDiscard) return;
    const uint32_t key = S.fkey[f];
    const int pix = (int)(key >> 16);
    const int unit = (int)(key & 0xffff);
    const double z = S.fz[f];
    const double bz = __dadd_rn(z, I.st.depth_bias);
    if (!I.st.read_depth || bz <= S.depth[pix]) {
        updated++;
        if (I.st.write_depth) S.depth[pix] = z;
        if (I.st.write_color) {
            // The colour buffer stays in global memory: the band is this
            // CTA's alone and one thread applies all of a pixel's fragments.
            uint32_t* cp = I.color + B.i0 + pix;
            if (fl & kFragBlend) {
                *cp = blend_nrgba(*cp, S.fcol[f]);
            } else {
                // SetNRGBA(x, y, c) ignores points outside the image rectangle:
                // x = i - y*W with i = r0*W + pix
                const int32_t x = pix - (S.urow[unit] - B.r0) * I.W;
                if (x >= 0 && x < I.W) *cp = S.fcol[f];
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
        float4 col = shade32(P, I, R, b0, b1, b2);
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
// fragment was pushed onto its pixel bucket's list in A1 (head / nxt).
// Without collisions each list has one entry and all apply in parallel;
// otherwise the thread holding a list's head applies the bucket's fragments
// by increasing key -- pixel, then unit -- selecting the next key from the
// short list each time. The lists are emptied for the next chunk as they are
// applied.
__device__ void resolve_chunk(const RasterParams& P, const ItemView& I, const BandCtx& B, RasterSmem& S,
                              uint32_t nfrag, bool conflict, uint64_t& updated) {
    if (!conflict) {
        for (uint32_t f = threadIdx.x; f < nfrag; f += blockDim.x) {
            apply_fragment(P, I, B, S, f, updated);
            S.head[bucket_of(S.fkey[f] >> 16)] = 0xFFFFu;
        }
        return;
    }
    for (uint32_t f = threadIdx.x; f < nfrag; f += blockDim.x) {
        const uint32_t pix = bucket_of(S.fkey[f] >> 16);  // the bucket
        if (S.head[pix] != f) continue;  // not the list head
        uint32_t last = 0;               // keys in a bucket are distinct
        bool first = true;
        // A list holds at most nfrag entries; every traversal is capped at
        // that, and a list that does not end within it is reported instead
        // of followed.
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
            apply_fragment(P, I, B, S, bestf, updated);
            last = best;
            first = false;
        }
        S.head[pix] = 0xFFFFu;
    }
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
        S.scratch = (unsigned long long*)q; q += 64 * 8;
        S.fkey = (uint32_t*)q; q += (size_t)F * 4;
        S.fcol = (uint32_t*)q; q += (size_t)F * 4;
        S.uslot = (uint32_t*)q; q += (size_t)F * 4;
        S.urow = (int32_t*)q; q += (size_t)F * 4;
        S.cprim = (uint32_t*)q; q += kRT * 4;
        S.cylo = (int32_t*)q; q += kRT * 4;
        S.cnrow = (int32_t*)q; q += kRT * 4;
        S.head = (unsigned short*)q; q += (size_t)kRasterHeads * 2;
        S.nxt = (unsigned short*)q; q += (size_t)F * 2;
        S.fflag = (uint8_t*)q;
    }
    __shared__ uint32_t s_band, s_item, s_nfrag, s_conflict, s_nprim, s_nunit, s_big;
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
        B.early = I.st.read_depth && (!I.st.write_depth || I.st.depth_bias >= 0);
        const int npx = B.npx;
        for (int j = threadIdx.x; j < npx; j += blockDim.x) {
            S.depth[j] = I.clear_depth_pending ? I.clear_depth : I.depth[B.i0 + j];
            if (I.clear_color_pending) I.color[B.i0 + j] = I.clear_color;  // fused clear
        }
        for (int j = threadIdx.x; j < kRasterHeads; j += blockDim.x) S.head[j] = 0xFFFFu;
        __syncthreads();

        uint64_t k = 0;
        bool box_bound = false;  // size the next chunk by bounding boxes only
        while (k < bcount) {
            // ---- chunk formation: a prefix of the remaining bin whose
            // fragment bound fits the buffer. A row of a primitive holds at
            // most pspan covered pixels (its widest chord, set up in
            // make_prim); box_bound falls back to the bounding-box width
            // after a chunk whose walk outgrew the buffer.
            uint32_t p = 0;
            PBox bx{1, 0, 1, 0};
            int32_t ylo = 0, nrows = 0;
            uint64_t bound = 0;
            const bool valid = (k + threadIdx.x) < bcount;
            if (valid) {
                p = P.bins[bstart + k + threadIdx.x];
                bx = P.pbox[p];
                rows_in_band(bx, I.W, B, ylo, nrows);
                int64_t wid = (int64_t)bx.x1 - bx.x0 + 1;
                if (!box_bound && (int64_t)P.pspan[p] < wid) wid = P.pspan[p];
                if (wid > npx) wid = npx;
                bound = (uint64_t)nrows * (uint64_t)wid;
            }
            uint64_t agg;
            uint64_t excl = block_exclusive_scan<kRT>(bound, s_warp, &agg);
            const bool take = valid && (excl + bound <= (uint64_t)F);
            // units of the taken primitives (the taken set is a prefix)
            uint64_t uagg;
            uint64_t ubase = block_exclusive_scan<kRT>(take ? (uint64_t)nrows : 0, s_warp, &uagg);
            if (threadIdx.x == 0) {
                s_nprim = 0;
                s_big = 0;
            }
            __syncthreads();
            if (take) {
                atomicAdd(&s_nprim, 1u);
                S.cprim[threadIdx.x] = p;
                S.cylo[threadIdx.x] = ylo;
                S.cnrow[threadIdx.x] = nrows;
                for (int r = 0; r < nrows; r++) {
                    S.uslot[ubase + r] = threadIdx.x;
                    S.urow[ubase + r] = ylo + r;
                }
            }
            __syncthreads();
            uint32_t nprim = s_nprim;
            uint32_t nunit = (uint32_t)uagg;
            bool big = false;
            if (nprim == 0) {
                // the next primitive alone exceeds the buffer: walk its rows in
                // rounds of at most F fragments
                big = true;
                nprim = 1;
                if (threadIdx.x == 0) {
                    S.cprim[0] = p;
                    S.cylo[0] = ylo;
                    S.cnrow[0] = nrows;
                }
                __syncthreads();
                nunit = (uint32_t)S.cnrow[0];
                for (uint32_t r = threadIdx.x; r < nunit; r += blockDim.x) {
                    S.uslot[r] = 0;
                    S.urow[r] = S.cylo[0] + (int32_t)r;
                }
            }
            __syncthreads();

            // ---- A1 / A2 / resolve, in rounds (one round unless big)
            Walk wk;
            wk.done = true;
            const int quota = big ? max(1, F / (int)max(nunit, 1u)) : 0x7fffffff;
            if (big && threadIdx.x < nunit) {
                const uint32_t pp = S.cprim[0];
                walk_init(wk, P.prims[pp], P.pbox[pp], S.urow[threadIdx.x], B, I.W, (int32_t)threadIdx.x);
            }
            for (;;) {
                if (threadIdx.x == 0) {
                    s_nfrag = 0;
                    s_conflict = 0;
                }
                __syncthreads();
                uint64_t tchunk = 0;
                if (big) {
                    if (threadIdx.x < nunit && !wk.done) {
                        const uint32_t pp = S.cprim[0];
                        tchunk += walk_run(wk, P.prims[pp], P, I, B, S, &s_nfrag, &s_conflict, quota, vis);
                    }
                } else {
                    for (uint32_t u = threadIdx.x; u < nunit; u += blockDim.x) {
                        const uint32_t pp = S.cprim[S.uslot[u]];
                        const RPrim& R = P.prims[pp];
                        Walk w2;
                        walk_init(w2, R, P.pbox[pp], S.urow[u], B, I.W, (int32_t)u);
                        tchunk += walk_run(w2, R, P, I, B, S, &s_nfrag, &s_conflict, 0x7fffffff, vis);
                    }
                }
                __syncthreads();
                if (s_conflict & 2u) {  // overflow: nothing was applied; empty the lists, redo with box bounds
                    const uint32_t nrec = min(s_nfrag, (uint32_t)F);
                    for (uint32_t f = threadIdx.x; f < nrec; f += blockDim.x)
                        S.head[bucket_of(S.fkey[f] >> 16)] = 0xFFFFu;
                    break;
                }
                tot += tchunk;
                const uint32_t nfrag = s_nfrag;
                if (threadIdx.x == 0) shd += nfrag;
                for (uint32_t f = threadIdx.x; f < nfrag; f += blockDim.x) shade_fragment<PREC>(P, I, S, f);
                __syncthreads();
                resolve_chunk(P, I, B, S, nfrag, (s_conflict & 1u) != 0, upd);
                __syncthreads();
                const int more = big ? __syncthreads_or(threadIdx.x < nunit && !wk.done) : 0;
                if (!more) break;
            }
            const bool redo = (s_conflict & 2u) != 0;
            __syncthreads();
            if (redo && !box_bound) {  // one redo per chunk, with bounds that cannot fail
                box_bound = true;
                continue;
            }
            if (redo && threadIdx.x == 0) atomicOr(P.status, ST_RASTER_INTERNAL);
            box_bound = false;
            k += nprim;
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
