/*
 * fauxgl_oracle.c -- TEST INFRASTRUCTURE ONLY (the checker and the timed CPU
 * baseline; never linked into the product).
 *
 * A CPU restatement of fogleman/fauxgl's triangle pipeline. Every function
 * cites the reference code it follows (file:line in fogleman/fauxgl). The
 * operation order of every FP64 expression is the reference's, evaluated left
 * to right without contraction (build with -ffp-contract=off).
 *
 * Parity unpinned: the reference has no tests or golden vectors for this path
 * and no Go toolchain exists on either machine; the restatement is pinned by
 * hand-derived known-answer tests instead.
 *
 * Deliberate divergence, shared with the GPU library: a primitive with a
 * non-finite screen coordinate, or a bounding box wider or taller than 2^26
 * pixels, produces no fragments. (In the reference such a primitive either
 * visits a single pixel at INT64_MIN or loops for ~2^63 iterations.)
 */
#include "fauxgl_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------------------ */
/* Go runtime semantics                                                      */
/* ------------------------------------------------------------------------ */

/* int(f) for float64 -> int on amd64 (CVTTSD2SQ): truncation toward zero;
 * NaN and out-of-range values give INT64_MIN. */
static int64_t go_f2i(double f) {
    if (f >= -9223372036854775808.0 && f < 9223372036854775808.0) return (int64_t)f;
    return INT64_MIN;
}

/* uint8(f): values in [0, 255] truncate; NaN gives 0. */
static uint8_t go_u8(double f) {
    return (uint8_t)(go_f2i(f) & 0xff);
}

/* math.Min (Go math/dim.go): -Inf wins, then NaN, then -0 < +0. */
static double go_min(double x, double y) {
    if ((isinf(x) && x < 0) || (isinf(y) && y < 0)) return -INFINITY;
    if (isnan(x) || isnan(y)) return NAN;
    if (x == 0 && x == y) return signbit(x) ? x : y;
    return x < y ? x : y;
}

/* math.Max: +Inf wins, then NaN, then +0 > -0. */
static double go_max(double x, double y) {
    if ((isinf(x) && x > 0) || (isinf(y) && y > 0)) return INFINITY;
    if (isnan(x) || isnan(y)) return NAN;
    if (x == 0 && x == y) return signbit(x) ? y : x;
    return x > y ? x : y;
}

static int go_is_odd_int(double x) {
    if (fabs(x) >= 9007199254740992.0) return 0;
    double xi;
    double xf = modf(x, &xi);
    return xf == 0 && (((int64_t)xi) & 1) == 1;
}

/* math.Pow (Go math/pow.go): special cases, then x**yi by repeated squaring
 * of the Frexp mantissa with exact power-of-two renormalisation, and x**yf
 * through Exp(yf*Log(x)) for a fractional exponent. The integer path (the
 * default SpecularPower 32) is exact to Go's; the fractional path uses the C
 * library's exp/log, which may differ from Go's by an ulp. */
double oracle_go_pow(double x, double y) {
    if (y == 0 || x == 1) return 1;
    if (y == 1) return x;
    if (isnan(x) || isnan(y)) return NAN;
    if (x == 0) {
        if (y < 0) return (signbit(x) && go_is_odd_int(y)) ? -INFINITY : INFINITY;
        if (y > 0) return (signbit(x) && go_is_odd_int(y)) ? x : 0.0;
    }
    if (isinf(y)) {
        if (x == -1) return 1;
        if ((fabs(x) < 1) == (y > 0)) return 0;
        return INFINITY;
    }
    if (isinf(x)) {
        if (x < 0) return oracle_go_pow(1 / x, -y);
        if (y < 0) return 0;
        if (y > 0) return INFINITY;
    }
    if (y == 0.5) return sqrt(x);
    if (y == -0.5) return 1 / sqrt(x);

    double yi;
    double yf = modf(fabs(y), &yi);
    if (yf != 0 && x < 0) return NAN;
    if (yi >= 9223372036854775808.0) {
        if (x == -1) return 1;
        if ((fabs(x) < 1) == (y > 0)) return 0;
        return INFINITY;
    }
    double a1 = 1.0;
    int64_t ae = 0;
    if (yf != 0) {
        if (yf > 0.5) {
            yf--;
            yi++;
        }
        a1 = exp(yf * log(x));
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
            a1 *= x1;
            ae += xe;
        }
        x1 *= x1;
        xe <<= 1;
        if (x1 < .5) {
            x1 += x1;
            xe--;
        }
    }
    if (y < 0) {
        a1 = 1 / a1;
        ae = -ae;
    }
    if (ae > 100000) ae = 100000;
    if (ae < -100000) ae = -100000;
    return ldexp(a1, (int)ae);
}

/* ------------------------------------------------------------------------ */
/* Value types (vector.go, color.go, vertex.go)                              */
/* ------------------------------------------------------------------------ */

typedef struct { double x, y, z; } V3;
typedef struct { double x, y, z, w; } V4;
typedef struct { double r, g, b, a; } C4;
typedef struct {
    V3 pos, nrm, tex;
    C4 col;
    V4 out;
} Vtx;

static V3 v3(double x, double y, double z) { V3 r = {x, y, z}; return r; }
static V3 v3_add(V3 a, V3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
static V3 v3_sub(V3 a, V3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
static V3 v3_muls(V3 a, double s) { return v3(a.x * s, a.y * s, a.z * s); }
static double v3_dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }     /* vector.go:72-74 */
static V3 v3_cross(V3 a, V3 b) {                                                  /* vector.go:76-81 */
    return v3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
static V3 v3_normalize(V3 a) {                                                    /* vector.go:83-86 */
    double r = 1 / sqrt(a.x * a.x + a.y * a.y + a.z * a.z);
    return v3(a.x * r, a.y * r, a.z * r);
}
static V3 v3_min(V3 a, V3 b) { return v3(go_min(a.x, b.x), go_min(a.y, b.y), go_min(a.z, b.z)); }
static V3 v3_max(V3 a, V3 b) { return v3(go_max(a.x, b.x), go_max(a.y, b.y), go_max(a.z, b.z)); }
static V3 v3_floor(V3 a) { return v3(floor(a.x), floor(a.y), floor(a.z)); }
static V3 v3_ceil(V3 a) { return v3(ceil(a.x), ceil(a.y), ceil(a.z)); }
/* Reflect (vector.go:175-177): i - n*(2*n.Dot(i)). */
static V3 v3_reflect(V3 i, V3 n) { return v3_sub(i, v3_muls(n, 2 * v3_dot(n, i))); }
/* Perpendicular (vector.go:179-187). */
static V3 v3_perpendicular(V3 a) {
    if (a.x == 0 && a.y == 0) {
        if (a.z == 0) return v3(0, 0, 0);
        return v3(0, 1, 0);
    }
    return v3_normalize(v3(-a.y, a.x, 0));
}

static V4 v4(double x, double y, double z, double w) { V4 r = {x, y, z, w}; return r; }
static V4 v4_add(V4 a, V4 b) { return v4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w); }
static V4 v4_sub(V4 a, V4 b) { return v4(a.x - b.x, a.y - b.y, a.z - b.z, a.w - b.w); }
static V4 v4_muls(V4 a, double s) { return v4(a.x * s, a.y * s, a.z * s, a.w * s); }
static double v4_dot(V4 a, V4 b) { return a.x * b.x + a.y * b.y + a.z * b.z + a.w * b.w; }  /* vector.go:217-219 */
/* VectorW.Outside (vector.go:212-215). */
static int v4_outside(V4 a) {
    return a.x < -a.w || a.x > a.w || a.y < -a.w || a.y > a.w || a.z < -a.w || a.z > a.w;
}

static C4 c4(double r, double g, double b, double a) { C4 c = {r, g, b, a}; return c; }
static C4 c4_add(C4 a, C4 b) { return c4(a.r + b.r, a.g + b.g, a.b + b.b, a.a + b.a); }
static C4 c4_muls(C4 a, double s) { return c4(a.r * s, a.g * s, a.b * s, a.a * s); }
static int c4_is_discard(C4 c) { return c.r == 0 && c.g == 0 && c.b == 0 && c.a == 0; }

/* Clamp (util.go:74-82). */
static double go_clamp(double x, double lo, double hi) {
    if (x < lo) return lo;
    if (x > hi) return hi;
    return x;
}

/* Color.NRGBA (color.go:56-63): clamp to [0,1], scale by 255, truncate. */
static void nrgba(C4 c, uint8_t out[4]) {
    const double d = 0xff;
    out[0] = go_u8(go_clamp(c.r, 0, 1) * d);
    out[1] = go_u8(go_clamp(c.g, 0, 1) * d);
    out[2] = go_u8(go_clamp(c.b, 0, 1) * d);
    out[3] = go_u8(go_clamp(c.a, 0, 1) * d);
}

void oracle_nrgba(const double c[4], uint8_t out[4]) { nrgba(c4(c[0], c[1], c[2], c[3]), out); }

/* The alpha-blend write of rasterize (context.go:256-267): the source is
 * color.NRGBA().RGBA() (image/color NRGBA.RGBA: 16-bit, alpha-premultiplied,
 * r = (R | R<<8) * A / 0xff), blended with uint32 arithmetic. */
static void blend_px(uint8_t* dst, C4 c) {
    uint8_t n[4];
    nrgba(c, n);
    uint32_t ca = n[3];
    uint32_t sr = n[0]; sr |= sr << 8; sr *= ca; sr /= 0xff;
    uint32_t sg = n[1]; sg |= sg << 8; sg *= ca; sg /= 0xff;
    uint32_t sb = n[2]; sb |= sb << 8; sb *= ca; sb /= 0xff;
    uint32_t sa = ca; sa |= sa << 8;
    uint32_t a = (0xffff - sa) * 0x101;
    dst[0] = (uint8_t)((((uint32_t)dst[0]) * a / 0xffff + sr) >> 8);
    dst[1] = (uint8_t)((((uint32_t)dst[1]) * a / 0xffff + sg) >> 8);
    dst[2] = (uint8_t)((((uint32_t)dst[2]) * a / 0xffff + sb) >> 8);
    dst[3] = (uint8_t)((((uint32_t)dst[3]) * a / 0xffff + sa) >> 8);
}

void oracle_blend(uint8_t dst[4], const double src[4]) { blend_px(dst, c4(src[0], src[1], src[2], src[3])); }

/* ------------------------------------------------------------------------ */
/* Matrix (matrix.go)                                                        */
/* ------------------------------------------------------------------------ */

/* MulPositionW (matrix.go:216-222). */
static V4 mul_position_w(const double* m, V3 b) {
    return v4(m[0] * b.x + m[1] * b.y + m[2] * b.z + m[3],
              m[4] * b.x + m[5] * b.y + m[6] * b.z + m[7],
              m[8] * b.x + m[9] * b.y + m[10] * b.z + m[11],
              m[12] * b.x + m[13] * b.y + m[14] * b.z + m[15]);
}

/* MulPosition (matrix.go:209-214). */
static V3 mul_position(const double* m, V3 b) {
    return v3(m[0] * b.x + m[1] * b.y + m[2] * b.z + m[3],
              m[4] * b.x + m[5] * b.y + m[6] * b.z + m[7],
              m[8] * b.x + m[9] * b.y + m[10] * b.z + m[11]);
}

/* Screen(w, h) (matrix.go:119-128). */
static void screen_matrix(int32_t w, int32_t h, double* m) {
    double w2 = (double)w / 2;
    double h2 = (double)h / 2;
    double s[16] = {w2, 0, 0, w2, 0, -h2, 0, h2, 0, 0, 0.5, 0.5, 0, 0, 0, 1};
    memcpy(m, s, sizeof(s));
}

/* ------------------------------------------------------------------------ */
/* Vertex interpolation (vertex.go)                                          */
/* ------------------------------------------------------------------------ */

/* InterpolateVectors (vertex.go:65-71): ((0 + v1*bX) + v2*bY + v3*bZ) * bW. */
static V3 interp_v3(V3 a, V3 b, V3 c, V4 w) {
    V3 n = v3(0, 0, 0);
    n = v3_add(n, v3_muls(a, w.x));
    n = v3_add(n, v3_muls(b, w.y));
    n = v3_add(n, v3_muls(c, w.z));
    return v3_muls(n, w.w);
}
static C4 interp_c4(C4 a, C4 b, C4 c, V4 w) {                                    /* vertex.go:57-63 */
    C4 n = c4(0, 0, 0, 0);
    n = c4_add(n, c4_muls(a, w.x));
    n = c4_add(n, c4_muls(b, w.y));
    n = c4_add(n, c4_muls(c, w.z));
    return c4_muls(n, w.w);
}
static V4 interp_v4(V4 a, V4 b, V4 c, V4 w) {                                    /* vertex.go:73-79 */
    V4 n = v4(0, 0, 0, 0);
    n = v4_add(n, v4_muls(a, w.x));
    n = v4_add(n, v4_muls(b, w.y));
    n = v4_add(n, v4_muls(c, w.z));
    return v4_muls(n, w.w);
}

/* InterpolateVertexes (vertex.go:18-47). */
static Vtx interp_vertex(const Vtx* v1, const Vtx* v2, const Vtx* v3_, V4 b) {
    Vtx v;
    v.pos = interp_v3(v1->pos, v2->pos, v3_->pos, b);
    v.nrm = v3_normalize(interp_v3(v1->nrm, v2->nrm, v3_->nrm, b));
    v.tex = interp_v3(v1->tex, v2->tex, v3_->tex, b);
    v.col = interp_c4(v1->col, v2->col, v3_->col, b);
    v.out = interp_v4(v1->out, v2->out, v3_->out, b);
    return v;
}

/* Barycentric (vertex.go:81-95). */
static V4 barycentric(V3 p1, V3 p2, V3 p3, V3 p) {
    V3 v0 = v3_sub(p2, p1);
    V3 v1 = v3_sub(p3, p1);
    V3 v2 = v3_sub(p, p1);
    double d00 = v3_dot(v0, v0);
    double d01 = v3_dot(v0, v1);
    double d11 = v3_dot(v1, v1);
    double d20 = v3_dot(v2, v0);
    double d21 = v3_dot(v2, v1);
    double d = d00 * d11 - d01 * d01;
    double v = (d11 * d20 - d01 * d21) / d;
    double w = (d00 * d21 - d01 * d20) / d;
    double u = 1 - v - w;
    return v4(u, v, w, 1);
}

/* Triangle.FixNormals (triangle.go:46-58) with Triangle.Normal (triangle.go:33-37). */
static void fix_normals(Vtx* a, Vtx* b, Vtx* c) {
    V3 e1 = v3_sub(b->pos, a->pos);
    V3 e2 = v3_sub(c->pos, a->pos);
    V3 n = v3_normalize(v3_cross(e1, e2));
    if (a->nrm.x == 0 && a->nrm.y == 0 && a->nrm.z == 0) a->nrm = n;
    if (b->nrm.x == 0 && b->nrm.y == 0 && b->nrm.z == 0) b->nrm = n;
    if (c->nrm.x == 0 && c->nrm.y == 0 && c->nrm.z == 0) c->nrm = n;
}

/* ------------------------------------------------------------------------ */
/* Clipping (clipping.go)                                                    */
/* ------------------------------------------------------------------------ */

/* clipPlanes (clipping.go:3-10): {P, N} for +x, -x, +y, -y, +z, -z. */
static const V4 CLIP_P[6] = {{1, 0, 0, 1}, {-1, 0, 0, 1}, {0, 1, 0, 1},
                             {0, -1, 0, 1}, {0, 0, 1, 1}, {0, 0, -1, 1}};
static const V4 CLIP_N[6] = {{-1, 0, 0, 1}, {1, 0, 0, 1}, {0, -1, 0, 1},
                             {0, 1, 0, 1}, {0, 0, -1, 1}, {0, 0, 1, 1}};

static int point_in_front(int k, V4 v) { return v4_dot(v4_sub(v, CLIP_P[k]), CLIP_N[k]) > 0; }  /* :16-18 */

static V4 intersect_segment(int k, V4 v0, V4 v1) {                                              /* :20-26 */
    V4 u = v4_sub(v1, v0);
    V4 w = v4_sub(v0, CLIP_P[k]);
    double d = v4_dot(CLIP_N[k], u);
    double n = -v4_dot(CLIP_N[k], w);
    return v4_add(v0, v4_muls(u, n / d));
}

/* sutherlandHodgman (clipping.go:28-52); at most 9 output points. */
static int sutherland_hodgman(const V4* points, int npoints, V4* out) {
    V4 buf_a[16], buf_b[16];
    const V4* input;
    V4* output = buf_a;
    int nout = npoints;
    memcpy(buf_a, points, sizeof(V4) * (size_t)npoints);
    for (int k = 0; k < 6; k++) {
        input = output;
        int nin = nout;
        output = (input == buf_a) ? buf_b : buf_a;
        nout = 0;
        if (nin == 0) return 0;
        V4 s = input[nin - 1];
        for (int j = 0; j < nin; j++) {
            V4 e = input[j];
            /* the buffers hold 16 points (a convex polygon has at most 9);
             * points beyond are dropped, as on the GPU */
            if (point_in_front(k, e)) {
                if (!point_in_front(k, s) && nout < 16) output[nout++] = intersect_segment(k, s, e);
                if (nout < 16) output[nout++] = e;
            } else if (point_in_front(k, s)) {
                if (nout < 16) output[nout++] = intersect_segment(k, s, e);
            }
            s = e;
        }
    }
    memcpy(out, output, sizeof(V4) * (size_t)nout);
    return nout;
}

/* ClipTriangle (clipping.go:54-74): fan (0, i-1, i) of interpolated vertices,
 * each sub-triangle through NewTriangle -> FixNormals. Returns the count. */
static int clip_triangle(const Vtx* t1, const Vtx* t2, const Vtx* t3, Vtx out[7][3]) {
    V3 p1 = v3(t1->out.x, t1->out.y, t1->out.z);
    V3 p2 = v3(t2->out.x, t2->out.y, t2->out.z);
    V3 p3 = v3(t3->out.x, t3->out.y, t3->out.z);
    V4 pts[3] = {t1->out, t2->out, t3->out};
    V4 np[16];
    int n = sutherland_hodgman(pts, 3, np);
    int cnt = 0;
    for (int i = 2; i < n && cnt < 7; i++) {  /* the GPU reserves 7 pieces per clipped triangle */
        V4 b1 = barycentric(p1, p2, p3, v3(np[0].x, np[0].y, np[0].z));
        V4 b2 = barycentric(p1, p2, p3, v3(np[i - 1].x, np[i - 1].y, np[i - 1].z));
        V4 b3 = barycentric(p1, p2, p3, v3(np[i].x, np[i].y, np[i].z));
        out[cnt][0] = interp_vertex(t1, t2, t3, b1);
        out[cnt][1] = interp_vertex(t1, t2, t3, b2);
        out[cnt][2] = interp_vertex(t1, t2, t3, b3);
        fix_normals(&out[cnt][0], &out[cnt][1], &out[cnt][2]);
        cnt++;
    }
    return cnt;
}

int oracle_clip_triangle(const double clip[12], double out_clip[7 * 3 * 4]) {
    Vtx t[3];
    memset(t, 0, sizeof(t));
    for (int c = 0; c < 3; c++) t[c].out = v4(clip[4 * c], clip[4 * c + 1], clip[4 * c + 2], clip[4 * c + 3]);
    Vtx o[7][3];
    int n = clip_triangle(&t[0], &t[1], &t[2], o);
    for (int i = 0; i < n; i++)
        for (int c = 0; c < 3; c++) {
            double* d = out_clip + (i * 3 + c) * 4;
            d[0] = o[i][c].out.x; d[1] = o[i][c].out.y; d[2] = o[i][c].out.z; d[3] = o[i][c].out.w;
        }
    return n;
}

/* ClipLine (clipping.go:76-98): only Output moves; returns 0 when culled. */
static int clip_line(Vtx* v1, Vtx* v2) {
    V4 w1 = v1->out, w2 = v2->out;
    for (int k = 0; k < 6; k++) {
        int f1 = point_in_front(k, w1);
        int f2 = point_in_front(k, w2);
        if (f1 && f2) continue;
        else if (f1) w2 = intersect_segment(k, w1, w2);
        else if (f2) w1 = intersect_segment(k, w2, w1);
        else return 0;
    }
    v1->out = w1;
    v2->out = w2;
    return 1;
}

/* ------------------------------------------------------------------------ */
/* Shaders (shader.go, texture.go)                                           */
/* ------------------------------------------------------------------------ */

typedef struct {
    const uint16_t* texels;
    int32_t w, h;
} Tex;

/* MakeColor(image.At(x, y)) (color.go:25-29); out-of-bounds At is zero. */
static C4 tex_at(const Tex* t, int64_t x, int64_t y) {
    if (x < 0 || y < 0 || x >= t->w || y >= t->h) return c4(0, 0, 0, 0);
    const uint16_t* p = t->texels + ((size_t)y * (size_t)t->w + (size_t)x) * 4;
    const double d = 0xffff;
    return c4((double)p[0] / d, (double)p[1] / d, (double)p[2] / d, (double)p[3] / d);
}

/* ImageTexture.BilinearSample (texture.go:41-63). */
static C4 bilinear_sample(const Tex* t, double u, double v) {
    v = 1 - v;
    u -= floor(u);
    v -= floor(v);
    double x = u * (double)(t->w - 1);
    double y = v * (double)(t->h - 1);
    int64_t x0 = go_f2i(x);
    int64_t y0 = go_f2i(y);
    int64_t x1 = x0 + 1;
    int64_t y1 = y0 + 1;
    x -= (double)x0;
    y -= (double)y0;
    C4 c00 = tex_at(t, x0, y0);
    C4 c01 = tex_at(t, x0, y1);
    C4 c10 = tex_at(t, x1, y0);
    C4 c11 = tex_at(t, x1, y1);
    C4 c = c4(0, 0, 0, 0);
    c = c4_add(c, c4_muls(c00, (1 - x) * (1 - y)));
    c = c4_add(c, c4_muls(c10, x * (1 - y)));
    c = c4_add(c, c4_muls(c01, (1 - x) * y));
    c = c4_add(c, c4_muls(c11, x * y));
    return c;
}

/* Fragment of the three built-ins (shader.go:25-27, 44-46, 75-96). */
static C4 fragment(const fgc_shader* sh, const Tex* tex, const Vtx* v) {
    if (sh->kind == FGC_SHADER_SOLID_COLOR)
        return c4(sh->color[0], sh->color[1], sh->color[2], sh->color[3]);
    if (sh->kind == FGC_SHADER_TEXTURE) return bilinear_sample(tex, v->tex.x, v->tex.y);
    /* PhongShader.Fragment */
    C4 light = c4(sh->ambient_color[0], sh->ambient_color[1], sh->ambient_color[2], sh->ambient_color[3]);
    C4 color = v->col;
    C4 obj = c4(sh->color[0], sh->color[1], sh->color[2], sh->color[3]);
    if (!c4_is_discard(obj)) color = obj;
    if (tex) color = bilinear_sample(tex, v->tex.x, v->tex.y);
    V3 L = v3(sh->light_direction[0], sh->light_direction[1], sh->light_direction[2]);
    double diffuse = go_max(v3_dot(v->nrm, L), 0);
    C4 dc = c4(sh->diffuse_color[0], sh->diffuse_color[1], sh->diffuse_color[2], sh->diffuse_color[3]);
    light = c4_add(light, c4_muls(dc, diffuse));
    if (diffuse > 0 && sh->specular_power > 0) {
        V3 E = v3(sh->camera_position[0], sh->camera_position[1], sh->camera_position[2]);
        V3 camera = v3_normalize(v3_sub(E, v->pos));
        V3 reflected = v3_reflect(v3(-L.x, -L.y, -L.z), v->nrm);
        double specular = go_max(v3_dot(camera, reflected), 0);
        if (specular > 0) {
            specular = oracle_go_pow(specular, sh->specular_power);
            C4 sc = c4(sh->specular_color[0], sh->specular_color[1], sh->specular_color[2], sh->specular_color[3]);
            light = c4_add(light, c4_muls(sc, specular));
        }
    }
    /* color.Mul(light).Min(White).Alpha(color.A) */
    return c4(go_min(color.r * light.r, 1), go_min(color.g * light.g, 1), go_min(color.b * light.b, 1), color.a);
}

/* ------------------------------------------------------------------------ */
/* Context (context.go)                                                      */
/* ------------------------------------------------------------------------ */

struct oracle_ctx {
    int32_t w, h;
    uint8_t* color;
    double* depth;
    uint32_t* winner;
    double* shaded;
    double screen[16];
    pthread_mutex_t locks[256];
};

oracle_ctx* oracle_create(int32_t width, int32_t height) {
    oracle_ctx* c = (oracle_ctx*)calloc(1, sizeof(oracle_ctx));
    size_t n = (size_t)width * (size_t)height;
    c->w = width;
    c->h = height;
    c->color = (uint8_t*)calloc(n * 4 + 1, 1);
    c->depth = (double*)malloc(n * sizeof(double) + 8);
    c->winner = (uint32_t*)malloc(n * sizeof(uint32_t) + 4);
    c->shaded = (double*)calloc(n * 4 + 1, sizeof(double));
    for (size_t i = 0; i < n; i++) {
        c->depth[i] = 1.7976931348623157e308; /* ClearDepthBuffer: math.MaxFloat64 */
        c->winner[i] = 0xFFFFFFFFu;
    }
    screen_matrix(width, height, c->screen);
    for (int i = 0; i < 256; i++) pthread_mutex_init(&c->locks[i], NULL);
    return c;
}

void oracle_destroy(oracle_ctx* c) {
    if (!c) return;
    for (int i = 0; i < 256; i++) pthread_mutex_destroy(&c->locks[i]);
    free(c->color);
    free(c->depth);
    free(c->winner);
    free(c->shaded);
    free(c);
}

/* ClearColorBufferWith (context.go:119-131). */
void oracle_clear_color(oracle_ctx* c, const double rgba[4]) {
    uint8_t n[4];
    nrgba(c4(rgba[0], rgba[1], rgba[2], rgba[3]), n);
    size_t np = (size_t)c->w * (size_t)c->h;
    for (size_t i = 0; i < np; i++) memcpy(c->color + 4 * i, n, 4);
}

/* ClearDepthBufferWith (context.go:137-141). */
void oracle_clear_depth(oracle_ctx* c, double value) {
    size_t np = (size_t)c->w * (size_t)c->h;
    for (size_t i = 0; i < np; i++) c->depth[i] = value;
}

uint8_t* oracle_color(oracle_ctx* c) { return c->color; }
double* oracle_depth(oracle_ctx* c) { return c->depth; }
uint32_t* oracle_winner(oracle_ctx* c) { return c->winner; }
double* oracle_shaded(oracle_ctx* c) { return c->shaded; }

typedef struct {
    oracle_ctx* ctx;
    const fgc_state* st;
    const fgc_shader* sh;
    const Tex* tex;
    int locked; /* 1 = the reference's concurrent form (striped locks) */
} Draw;

typedef struct {
    uint64_t total, updated;
} Acc;

/* edge (context.go:147-149). */
static double edge(V3 a, V3 b, V3 c) { return (b.x - c.x) * (a.y - c.y) - (b.y - c.y) * (a.x - c.x); }

static int finite3(V3 a) { return isfinite(a.x) && isfinite(a.y) && isfinite(a.z); }

#define MAX_EXTENT 67108864LL /* 2^26 */

/* rasterize (context.go:151-281). */
static void rasterize(const Draw* D, Acc* acc, const Vtx* v0, const Vtx* v1, const Vtx* v2, V3 s0, V3 s1,
                      V3 s2, uint32_t elem) {
    oracle_ctx* ctx = D->ctx;
    const fgc_state* st = D->st;
    if (!finite3(s0) || !finite3(s1) || !finite3(s2)) return; /* see header note */

    /* integer bounding box */
    V3 mn = v3_floor(v3_min(s0, v3_min(s1, s2)));
    V3 mx = v3_ceil(v3_max(s0, v3_max(s1, s2)));
    int64_t x0 = go_f2i(mn.x);
    int64_t x1 = go_f2i(mx.x);
    int64_t y0 = go_f2i(mn.y);
    int64_t y1 = go_f2i(mx.y);
    if (x1 - x0 > MAX_EXTENT || y1 - y0 > MAX_EXTENT) return; /* see header note */

    /* forward differencing variables */
    V3 p = v3((double)x0 + 0.5, (double)y0 + 0.5, 0);
    double w00 = edge(s1, s2, p);
    double w01 = edge(s2, s0, p);
    double w02 = edge(s0, s1, p);
    double a01 = s1.y - s0.y;
    double b01 = s0.x - s1.x;
    double a12 = s2.y - s1.y;
    double b12 = s1.x - s2.x;
    double a20 = s0.y - s2.y;
    double b20 = s2.x - s0.x;

    /* reciprocals */
    double ra = 1 / edge(s0, s1, s2);
    double r0 = 1 / v0->out.w;
    double r1 = 1 / v1->out.w;
    double r2 = 1 / v2->out.w;
    double ra12 = 1 / a12;
    double ra20 = 1 / a20;
    double ra01 = 1 / a01;

    const int64_t W = ctx->w;
    const int64_t N = (int64_t)ctx->w * (int64_t)ctx->h;
    for (int64_t y = y0; y <= y1; y++) {
        /* A row whose index range misses [0, N) can update nothing; its x
         * walk is skipped (the row-end increments below still run). */
        if (!(y * W + x1 < 0 || y * W + x0 >= N)) {
            double d = 0;
            double d0 = -w00 * ra12;
            double d1 = -w01 * ra20;
            double d2 = -w02 * ra01;
            if (w00 < 0 && d0 > d) d = d0;
            if (w01 < 0 && d1 > d) d = d1;
            if (w02 < 0 && d2 > d) d = d2;
            d = (double)go_f2i(d);
            if (d < 0) d = 0; /* occurs in pathological cases */
            double w0 = w00 + a12 * d;
            double w1 = w01 + a20 * d;
            double w2 = w02 + a01 * d;
            int was_inside = 0;
            for (int64_t x = x0 + go_f2i(d); x <= x1; x++) {
                double b0 = w0 * ra;
                double b1 = w1 * ra;
                double b2 = w2 * ra;
                w0 += a12;
                w1 += a20;
                w2 += a01;
                if (b0 < 0 || b1 < 0 || b2 < 0) {
                    if (was_inside) break;
                    continue;
                }
                was_inside = 1;
                int64_t i = y * W + x;
                if (i < 0 || i >= N) continue;
                acc->total++;
                double z = b0 * s0.z + b1 * s1.z + b2 * s2.z;
                double bz = z + st->depth_bias;
                if (st->read_depth && bz > ctx->depth[i]) continue;
                V4 b = v4(b0 * r0, b1 * r1, b2 * r2, 0);
                b.w = 1 / (b.x + b.y + b.z);
                Vtx v = interp_vertex(v0, v1, v2, b);
                C4 color = fragment(D->sh, D->tex, &v);
                if (c4_is_discard(color)) continue;
                pthread_mutex_t* lock = &ctx->locks[(x + y) & 255];
                if (D->locked) pthread_mutex_lock(lock);
                if (bz <= ctx->depth[i] || !st->read_depth) {
                    acc->updated++;
                    ctx->winner[i] = elem;
                    ctx->shaded[4 * i + 0] = color.r;
                    ctx->shaded[4 * i + 1] = color.g;
                    ctx->shaded[4 * i + 2] = color.b;
                    ctx->shaded[4 * i + 3] = color.a;
                    if (st->write_depth) ctx->depth[i] = z;
                    if (st->write_color) {
                        if (st->alpha_blend && color.a < 1) {
                            blend_px(ctx->color + 4 * i, color);
                        } else if (x >= 0 && y >= 0 && x < W && y < ctx->h) {
                            /* SetNRGBA(x, y, ...) ignores points outside the rectangle */
                            nrgba(color, ctx->color + 4 * i);
                        }
                    }
                }
                if (D->locked) pthread_mutex_unlock(lock);
            }
        }
        w00 += b12;
        w01 += b20;
        w02 += b01;
    }
}

/* line (context.go:283-294). */
static void line(const Draw* D, Acc* acc, const Vtx* v0, const Vtx* v1, V3 s0, V3 s1, uint32_t elem) {
    double lw2 = D->st->line_width / 2;
    V3 n = v3_muls(v3_perpendicular(v3_sub(s1, s0)), lw2);
    s0 = v3_add(s0, v3_muls(v3_normalize(v3_sub(s0, s1)), lw2));
    s1 = v3_add(s1, v3_muls(v3_normalize(v3_sub(s1, s0)), lw2));
    V3 s00 = v3_add(s0, n);
    V3 s01 = v3_sub(s0, n);
    V3 s10 = v3_add(s1, n);
    V3 s11 = v3_sub(s1, n);
    rasterize(D, acc, v1, v0, v0, s11, s01, s00, elem);
    rasterize(D, acc, v1, v1, v0, s10, s11, s00, elem);
}

/* wireframe (context.go:296-301). */
static void wireframe(const Draw* D, Acc* acc, const Vtx* v0, const Vtx* v1, const Vtx* v2, V3 s0, V3 s1,
                      V3 s2, uint32_t elem) {
    line(D, acc, v0, v1, s0, s1, elem);
    line(D, acc, v1, v2, s1, s2, elem);
    line(D, acc, v2, v0, s2, s0, elem);
}

static V3 ndc_of(V4 o) { return v3(o.x / o.w, o.y / o.w, o.z / o.w); }  /* DivScalar(W).Vector() */

/* drawClippedLine (context.go:303-314). */
static void draw_clipped_line(const Draw* D, Acc* acc, const Vtx* v0, const Vtx* v1, uint32_t elem) {
    V3 s0 = mul_position(D->ctx->screen, ndc_of(v0->out));
    V3 s1 = mul_position(D->ctx->screen, ndc_of(v1->out));
    line(D, acc, v0, v1, s0, s1, elem);
}

/* drawClippedTriangle (context.go:316-349). */
static void draw_clipped_triangle(const Draw* D, Acc* acc, const Vtx* v0, const Vtx* v1, const Vtx* v2,
                                  uint32_t elem) {
    const fgc_state* st = D->st;
    V3 ndc0 = ndc_of(v0->out);
    V3 ndc1 = ndc_of(v1->out);
    V3 ndc2 = ndc_of(v2->out);
    double a = (ndc1.x - ndc0.x) * (ndc2.y - ndc0.y) - (ndc2.x - ndc0.x) * (ndc1.y - ndc0.y);
    if (a < 0) {
        const Vtx* tv = v0; v0 = v2; v2 = tv;
        V3 tn = ndc0; ndc0 = ndc2; ndc2 = tn;
    }
    if (st->cull == FGC_CULL_FRONT) a = -a;
    if (st->front_face == FGC_FACE_CW) a = -a;
    if (st->cull != FGC_CULL_NONE && a <= 0) return;
    V3 s0 = mul_position(D->ctx->screen, ndc0);
    V3 s1 = mul_position(D->ctx->screen, ndc1);
    V3 s2 = mul_position(D->ctx->screen, ndc2);
    if (st->wireframe) wireframe(D, acc, v0, v1, v2, s0, s1, s2, elem);
    else rasterize(D, acc, v0, v1, v2, s0, s1, s2, elem);
}

typedef struct {
    const double *pos, *nrm, *tex, *col;
} Arrays;

static void load_vertex(const Arrays* A, int64_t v, Vtx* out) {
    memset(out, 0, sizeof(Vtx));
    out->pos = v3(A->pos[3 * v], A->pos[3 * v + 1], A->pos[3 * v + 2]);
    if (A->nrm) out->nrm = v3(A->nrm[3 * v], A->nrm[3 * v + 1], A->nrm[3 * v + 2]);
    if (A->tex) out->tex = v3(A->tex[2 * v], A->tex[2 * v + 1], 0);
    if (A->col) out->col = c4(A->col[4 * v], A->col[4 * v + 1], A->col[4 * v + 2], A->col[4 * v + 3]);
}

/* Shader.Vertex of the built-ins (shader.go:20-23, 39-42, 70-73). */
static void vertex_shader(const fgc_shader* sh, Vtx* v) { v->out = mul_position_w(sh->matrix, v->pos); }

/* DrawTriangle (context.go:370-389). */
static void draw_triangle(const Draw* D, Acc* acc, const Arrays* A, int64_t t) {
    Vtx v1, v2, v3_;
    load_vertex(A, 3 * t + 0, &v1);
    load_vertex(A, 3 * t + 1, &v2);
    load_vertex(A, 3 * t + 2, &v3_);
    vertex_shader(D->sh, &v1);
    vertex_shader(D->sh, &v2);
    vertex_shader(D->sh, &v3_);
    uint32_t elem = (uint32_t)t;
    if (v4_outside(v1.out) || v4_outside(v2.out) || v4_outside(v3_.out)) {
        /* ClipTriangle(NewTriangle(v1, v2, v3)): NewTriangle fixes zero normals first */
        fix_normals(&v1, &v2, &v3_);
        Vtx tris[7][3];
        int n = clip_triangle(&v1, &v2, &v3_, tris);
        for (int k = 0; k < n; k++) draw_clipped_triangle(D, acc, &tris[k][0], &tris[k][1], &tris[k][2], elem);
    } else {
        draw_clipped_triangle(D, acc, &v1, &v2, &v3_, elem);
    }
}

/* DrawLine (context.go:351-368). */
static void draw_line(const Draw* D, Acc* acc, const Arrays* A, int64_t l) {
    Vtx v1, v2;
    load_vertex(A, 2 * l + 0, &v1);
    load_vertex(A, 2 * l + 1, &v2);
    vertex_shader(D->sh, &v1);
    vertex_shader(D->sh, &v2);
    uint32_t elem = 0x80000000u | (uint32_t)l;
    if (v4_outside(v1.out) || v4_outside(v2.out)) {
        if (clip_line(&v1, &v2)) draw_clipped_line(D, acc, &v1, &v2, elem);
    } else {
        draw_clipped_line(D, acc, &v1, &v2, elem);
    }
}

typedef struct {
    const Draw* D;
    const Arrays* A;
    int64_t first, count;
    int is_line;
    int wi, wn;
    Acc acc;
} Worker;

static void* worker_main(void* arg) {
    Worker* w = (Worker*)arg;
    for (int64_t i = 0; i < w->count; i++) {
        if (i % w->wn != w->wi) continue;
        if (w->is_line) draw_line(w->D, &w->acc, w->A, w->first + i);
        else draw_triangle(w->D, &w->acc, w->A, w->first + i);
    }
    return NULL;
}

/* DrawTriangles / DrawLines (context.go:391-433), either sequential (the
 * oracle) or with the reference's worker split (the CPU baseline). */
static void draw_list(const Draw* D, const Arrays* A, int64_t first, int64_t count, int is_line, int nthreads,
                      Acc* acc) {
    if (nthreads <= 0) {
        for (int64_t i = 0; i < count; i++) {
            if (is_line) draw_line(D, acc, A, first + i);
            else draw_triangle(D, acc, A, first + i);
        }
        return;
    }
    Worker* ws = (Worker*)calloc((size_t)nthreads, sizeof(Worker));
    pthread_t* th = (pthread_t*)calloc((size_t)nthreads, sizeof(pthread_t));
    for (int i = 0; i < nthreads; i++) {
        ws[i].D = D; ws[i].A = A; ws[i].first = first; ws[i].count = count; ws[i].is_line = is_line;
        ws[i].wi = i; ws[i].wn = nthreads;
        pthread_create(&th[i], NULL, worker_main, &ws[i]);
    }
    for (int i = 0; i < nthreads; i++) {
        pthread_join(th[i], NULL);
        acc->total += ws[i].acc.total;
        acc->updated += ws[i].acc.updated;
    }
    free(ws);
    free(th);
}

int oracle_draw(oracle_ctx* ctx, const fgc_state* st, const fgc_shader* sh, const uint16_t* texture,
                int32_t tex_w, int32_t tex_h, const double* tri_pos, const double* tri_nrm,
                const double* tri_tex, const double* tri_col, int64_t tri_first, int64_t tri_count,
                const double* line_pos, const double* line_nrm, const double* line_tex,
                const double* line_col, int64_t line_first, int64_t line_count, int32_t what,
                int32_t nthreads, fgc_rasterize_info* info) {
    if (sh->kind < FGC_SHADER_SOLID_COLOR || sh->kind > FGC_SHADER_PHONG) return FGC_ERR_UNSUPPORTED_SHADER;
    Tex tex = {texture, tex_w, tex_h};
    if (sh->kind == FGC_SHADER_TEXTURE && !texture) return FGC_ERR_INVALID_ARGUMENT;
    Draw D = {ctx, st, sh, texture ? &tex : NULL, nthreads > 0};
    Acc acc = {0, 0};
    if ((what & 1) && tri_count > 0) {
        Arrays A = {tri_pos, tri_nrm, tri_tex, tri_col};
        draw_list(&D, &A, tri_first, tri_count, 0, nthreads, &acc);
    }
    if ((what & 2) && line_count > 0) {
        Arrays A = {line_pos, line_nrm, line_tex, line_col};
        draw_list(&D, &A, line_first, line_count, 1, nthreads, &acc);
    }
    info->total_pixels = acc.total;
    info->updated_pixels = acc.updated;
    return FGC_OK;
}

/* Box downsample: each output channel is (sum + n/2) / n over the scale*scale
 * block (the project's definition; the reference examples use a third-party
 * bilinear resize instead). */
void oracle_downsample(const uint8_t* src, int32_t width, int32_t height, int32_t scale, uint8_t* dst) {
    int32_t ow = width / scale, oh = height / scale;
    uint32_t n = (uint32_t)scale * (uint32_t)scale;
    for (int32_t y = 0; y < oh; y++)
        for (int32_t x = 0; x < ow; x++)
            for (int ch = 0; ch < 4; ch++) {
                uint32_t s = 0;
                for (int32_t dy = 0; dy < scale; dy++)
                    for (int32_t dx = 0; dx < scale; dx++)
                        s += src[(((size_t)(y * scale + dy)) * (size_t)width + (size_t)(x * scale + dx)) * 4 + ch];
                dst[((size_t)y * (size_t)ow + (size_t)x) * 4 + ch] = (uint8_t)((s + n / 2) / n);
            }
}

/* DepthImage (context.go:87-117). */
void oracle_depth_image(oracle_ctx* ctx, uint16_t* gray16) {
    const double maxf = 1.7976931348623157e308;
    double lo = maxf, hi = -maxf;
    size_t n = (size_t)ctx->w * (size_t)ctx->h;
    for (size_t i = 0; i < n; i++) {
        double d = ctx->depth[i];
        if (d == maxf) continue;
        if (d < lo) lo = d;
        if (d > hi) hi = d;
    }
    for (size_t i = 0; i < n; i++) {
        double d = ctx->depth[i];
        double t = (d - lo) / (hi - lo);
        if (d == maxf) t = 1;
        /* uint16(t * 0xffff): truncation; NaN and out-of-range give the low
         * 16 bits of INT64_MIN, i.e. 0 */
        gray16[i] = (uint16_t)(go_f2i(t * 0xffff) & 0xffff);
    }
}
