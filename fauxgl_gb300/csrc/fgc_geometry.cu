// fgc_geometry.cu -- vertex stage, triangle/line setup and view-volume
// clipping.
//
// Pipeline position: mesh (device-resident, positions welded to unique
// vertices) -> [vertex_kernel] per unique vertex: Output, Outside, NDC,
// screen position, 1/W -> [setup kernels] per element: culling, screen-space
// edge setup, ordered compaction of raster primitives (RPrim) -> [clip
// kernels] for the elements that needed ClipTriangle / ClipLine.
//
// Reference: context.go:283-389 (line, wireframe, drawClippedLine,
// drawClippedTriangle, DrawLine, DrawTriangle), clipping.go (ClipTriangle,
// ClipLine), vertex.go:14-95, triangle.go:33-58, shader.go:20-23 (Vertex).
#include "fgc_internal.cuh"

namespace fgc {

// ---------------------------------------------------------------------------
// Vertex stage: one thread per unique position of each draw (a draw's
// positions are transformed by its own matrix), tiles of kVertexTile
// positions strided over the grid.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kVertexTile) vertex_kernel(VertexParams P) {
    for (uint32_t t = blockIdx.x; t < P.ntiles; t += gridDim.x) {
        const uint32_t it = find_item(P.starts.vtile, P.nitems, t);
        const ItemView& I = P.items[it];
        const uint64_t u = (uint64_t)(t - I.vtile0) * kVertexTile + threadIdx.x;
        if (u >= I.mesh.nuniq) continue;
        D4 c = mul_position_w(I.sh.m, I.mesh.upos_x[u], I.mesh.upos_y[u], I.mesh.upos_z[u]);  // Shader.Vertex
        const uint64_t o = I.vbase + u;
        P.vclip[o] = VClip{c.x, c.y, c.z, c.w};
        P.vout[o] = outside4(c) ? 1 : 0;
        const double rw = __drcp_rn(c.w);
        D3 n = ndc_of_rcp(c, rw);
        P.vndc[o] = make_double2(n.x, n.y);
        D3 s = screen_of_ndc(n, I.w2, I.h2);
        P.vscr[o] = VScreen{s.x, s.y, s.z, rw};
    }
}

// ---------------------------------------------------------------------------
// Raster primitive construction: rasterize's per-triangle prologue
// (context.go:151-181).
// ---------------------------------------------------------------------------
__device__ __forceinline__ double edge_fn(D3 a, D3 b, D3 c) {  // context.go:147-149
    return __dsub_rn(__dmul_rn(__dsub_rn(b.x, c.x), __dsub_rn(a.y, c.y)),
                     __dmul_rn(__dsub_rn(b.y, c.y), __dsub_rn(a.x, c.x)));
}

__device__ void write_dead(const GeomParams& P, uint64_t slot) {
    if (slot >= P.prim_cap) {
        atomicOr(P.status, ST_CLIP_OVERFLOW);
        return;
    }
    P.pbox[slot] = PBox{1, 0, 1, 0};
}

__device__ void make_prim(const GeomParams& P, uint64_t slot, D3 s0, D3 s1, D3 s2, double r0, double r1,
                          double r2, uint32_t v0, uint32_t v1, uint32_t v2, uint32_t elem) {
    if (slot >= P.prim_cap) {  // slots reserved past an overflowing clip list
        atomicOr(P.status, ST_CLIP_OVERFLOW);
        return;
    }
    if (!(dfinite(s0.x) && dfinite(s0.y) && dfinite(s0.z) && dfinite(s1.x) && dfinite(s1.y) && dfinite(s1.z) &&
          dfinite(s2.x) && dfinite(s2.y) && dfinite(s2.z))) {
        write_dead(P, slot);
        return;
    }
    // integer bounding box (Min/Max, Floor/Ceil, int())
    const int64_t x0 = go_floor_i(go_min_i(s0.x, go_min_i(s1.x, s2.x)));
    const int64_t y0 = go_floor_i(go_min_i(s0.y, go_min_i(s1.y, s2.y)));
    const int64_t x1 = go_ceil_i(go_max_i(s0.x, go_max_i(s1.x, s2.x)));
    const int64_t y1 = go_ceil_i(go_max_i(s0.y, go_max_i(s1.y, s2.y)));
    const int64_t lim = 1LL << 30;
    if (x1 - x0 > kMaxExtent || y1 - y0 > kMaxExtent || x0 < -lim || x1 > lim || y0 < -lim || y1 > lim) {
        write_dead(P, slot);
        return;
    }
    D3 p = d3(__dadd_rn(i2d_i(x0), 0.5), __dadd_rn(i2d_i(y0), 0.5), 0.0);  // |x0|, |y0| <= 2^30 here
    RPrim R;
    // edge(a, b, p) = (b.X - p.X)(a.Y - p.Y) - (b.Y - p.Y)(a.X - p.X)
    // (context.go:147-149): the six differences to p are shared by the three
    // edges
    const double dx0 = __dsub_rn(s0.x, p.x), dx1 = __dsub_rn(s1.x, p.x), dx2 = __dsub_rn(s2.x, p.x);
    const double dy0 = __dsub_rn(s0.y, p.y), dy1 = __dsub_rn(s1.y, p.y), dy2 = __dsub_rn(s2.y, p.y);
    R.w0 = __dsub_rn(__dmul_rn(dx2, dy1), __dmul_rn(dy2, dx1));  // edge(s1, s2, p)
    R.w1 = __dsub_rn(__dmul_rn(dx0, dy2), __dmul_rn(dy0, dx2));  // edge(s2, s0, p)
    R.w2 = __dsub_rn(__dmul_rn(dx1, dy0), __dmul_rn(dy1, dx0));  // edge(s0, s1, p)
    double a01 = __dsub_rn(s1.y, s0.y);
    double b01 = __dsub_rn(s0.x, s1.x);
    double a12 = __dsub_rn(s2.y, s1.y);
    double b12 = __dsub_rn(s1.x, s2.x);
    double a20 = __dsub_rn(s0.y, s2.y);
    double b20 = __dsub_rn(s2.x, s0.x);
    R.a0 = a12; R.a1 = a20; R.a2 = a01;
    R.b0 = b12; R.b1 = b20; R.b2 = b01;
    // edge(s0, s1, s2) = (s1.X - s2.X)(s0.Y - s2.Y) - (s1.Y - s2.Y)(s0.X - s2.X):
    // its factors are b12, a20, -a12 and -b20 (a rounded difference changes
    // only its sign when the operands swap), and (-a12)(-b20) = a12 b20
    const double area2 = __dsub_rn(__dmul_rn(b12, a20), __dmul_rn(a12, b20));
    // Rows and columns of the box that hold no covered pixel centre.
    // rasterize walks rows y0 = floor(min y) .. y1 = ceil(max y) and columns
    // up to x1 = ceil(max x) (context.go:155-160, 184-207), so its last row
    // and column (and often the first row) lie wholly beyond the triangle.
    // The walk's edge values differ from the exact edge functions of the
    // FP64 screen positions by at most delta = 2^-53 (8 + 6n) (D + 2)^2,
    // n = D + 4 serial adds, D = box width + height >= the longest edge: the
    // first value's products and differences, then one rounding per add and
    // the increments' own rounding. A point whose computed tests all pass
    // thus has barycentrics >= -delta / |2A| and lies within
    // 3 delta D / |2A| of the triangle (area A). When 6 delta D <= eps |2A|,
    // a pixel centre more than eps above min y, below max y or right of max x
    // is outside in the reference's arithmetic as well, and its row or column
    // can be left out: the first row moves down when frac(min y) > 1/2 + eps
    // (the edge values step to it by the reference's own row adds), the last
    // row is the last centre at or above max y + eps, the last column the
    // last centre at or left of max x + eps. Outputs are unchanged; the walk
    // visits fewer rows and pixels. Boxes beyond the bound keep every row.
    int64_t ry0 = y0, ry1 = y1, rx1 = x1;
    {
        constexpr double kEps = 0.00390625;            // 2^-8 pixel
        constexpr double kHalfEps = 0.5 + kEps;
        const float D = (float)((x1 - x0) + (y1 - y0));
        const float n = D + 4.0f;
        const float lhs = 6.0f * 1.1102230246251565e-16f * (8.0f + 6.0f * n) * (D + 2.0f) * (D + 2.0f) * D;
        const float rhs = (float)kEps * f32_trunc_pos(dbits(area2) & kAbsMask);  // <= eps |2A|
        if (dfinite(area2) && rhs > 0.0f && lhs * 1.01f <= rhs) {
            const double ymin = go_min_i(s0.y, go_min_i(s1.y, s2.y));
            const double ymax = go_max_i(s0.y, go_max_i(s1.y, s2.y));
            const double xmax = go_max_i(s0.x, go_max_i(s1.x, s2.x));
            if (dgt_i(__dsub_rn(ymin, i2d_i(y0)), kHalfEps)) ry0 = y0 + 1;
            ry1 = y1 - 1 - (dgt_i(__dsub_rn(i2d_i(y1), ymax), kHalfEps) ? 1 : 0);
            rx1 = x1 - 1 - (dgt_i(__dsub_rn(i2d_i(x1), xmax), kHalfEps) ? 1 : 0);
            if (ry0 > ry1 || rx1 < x0) {
                write_dead(P, slot);  // no pixel centre can be covered
                return;
            }
            if (ry0 > y0) {  // w00 += b12 etc. (context.go:275-277) for the row left out
                R.w0 = __dadd_rn(R.w0, b12);
                R.w1 = __dadd_rn(R.w1, b20);
                R.w2 = __dadd_rn(R.w2, b01);
            }
        }
    }
    R.ra = __drcp_rn(area2);  // 1 / x, correctly rounded
    R.q0 = __drcp_rn(a12);
    R.q1 = __drcp_rn(a20);
    R.q2 = __drcp_rn(a01);
    R.z0 = s0.z; R.z1 = s1.z; R.z2 = s2.z;
    R.r0 = r0; R.r1 = r1; R.r2 = r2;
    R.v0 = v0; R.v1 = v1; R.v2 = v2;
    R.elem = elem;
    P.prims[slot] = R;
    P.pbox[slot] = PBox{(int32_t)x0, (int32_t)rx1, (int32_t)ry0, (int32_t)ry1};
    P.rf[slot] = make_float4((float)r0, (float)r1, (float)r2, 0.0f);
    // A row's covered pixel centres lie on one horizontal chord of the
    // triangle, so a row holds at most (widest chord) + 1 of them; +3 more
    // cover rounding at both ends and in this estimate. The widest chord runs
    // through the middle vertex and is |2 area| / height, with 2 area =
    // edge(s0, s1, s2) and height the largest |y difference| (FP32 from
    // truncated operands, with a relative margin far above their error). The
    // raster stage sizes its fragment chunks with this bound and redoes a
    // chunk the bound does not hold for, so it affects speed only.
    const unsigned long long h01 = dbits(a01) & kAbsMask, h12 = dbits(a12) & kAbsMask, h20 = dbits(a20) & kAbsMask;
    const unsigned long long hb = h01 > h12 ? (h01 > h20 ? h01 : h20) : (h12 > h20 ? h12 : h20);
    const uint32_t bw = (uint32_t)(rx1 - x0 + 1);
    uint32_t span = bw;
    if (hb != 0) {
        const float chord = f32_trunc_pos(dbits(area2) & kAbsMask) / f32_trunc_pos(hb);
        const float s = ceilf(chord * (1.0f + 1.0f / 1024.0f)) + 4.0f;
        if (s < (float)bw) span = (uint32_t)s;
    }
    P.pspan[slot] = span;
}

// line (context.go:283-294): a screen-space quad of width LineWidth as two
// raster primitives, (v1,v0,v0; s11,s01,s00) and (v1,v1,v0; s10,s11,s00).
__device__ void make_line_prims(const GeomParams& P, double line_width, uint64_t slot, D3 s0, D3 s1, double r0,
                                double r1, uint32_t v0, uint32_t v1, uint32_t elem) {
    double lw2 = __ddiv_rn(line_width, 2.0);
    D3 d = sub3(s1, s0);
    D3 perp;  // Perpendicular (vector.go:179-187)
    if (d.x == 0 && d.y == 0) {
        perp = (d.z == 0) ? d3(0, 0, 0) : d3(0, 1, 0);
    } else {
        perp = normalize3(d3(-d.y, d.x, 0.0));
    }
    D3 n = muls3(perp, lw2);
    s0 = add3(s0, muls3(normalize3(sub3(s0, s1)), lw2));
    s1 = add3(s1, muls3(normalize3(sub3(s1, s0)), lw2));
    D3 s00 = add3(s0, n);
    D3 s01 = sub3(s0, n);
    D3 s10 = add3(s1, n);
    D3 s11 = sub3(s1, n);
    make_prim(P, slot, s11, s01, s00, r1, r0, r0, v1, v0, v0, elem);
    make_prim(P, slot + 1, s10, s11, s00, r1, r1, r0, v1, v1, v0, elem);
}

// clipPlanes (clipping.go:3-10): {P, N} of +x, -x, +y, -y, +z, -z.
__device__ __forceinline__ void clip_plane(int k, D4& p, D4& n) {
    double s = (k & 1) ? -1.0 : 1.0;
    int axis = k >> 1;
    p = d4(axis == 0 ? s : 0.0, axis == 1 ? s : 0.0, axis == 2 ? s : 0.0, 1.0);
    n = d4(axis == 0 ? -s : 0.0, axis == 1 ? -s : 0.0, axis == 2 ? -s : 0.0, 1.0);
}

__device__ __forceinline__ bool finite4(D4 v) { return dfinite(v.x) && dfinite(v.y) && dfinite(v.z) && dfinite(v.w); }
__device__ __forceinline__ double axis_of(int k, D4 v) { return (k >> 1) == 0 ? v.x : (k >> 1) == 1 ? v.y : v.z; }

// The planes' P and N are zero except on their axis (+-1) and on w (1), so in
// a dot product with N in the reference's order ((x + y) + z) + w, the terms
// of the two other axes are signed zeros when their factors are finite.
// Adding a signed zero to a nonzero partial sum leaves it unchanged, so the
// dot product equals RN(N_axis * a + b) for the axis and w terms a, b, except
// possibly in the sign of a zero result. n_dot returns that short form.
__device__ __forceinline__ double n_dot(int k, double a, double b) {
    return __dadd_rn((k & 1) ? a : -a, b);  // N_axis = -1 for even k, +1 for odd k (exact products)
}

// pointInFront (clipping.go:16-18): (v - P).Dot(N) > 0. The sign of a zero
// does not change "> 0", so finite points take the short form.
__device__ __forceinline__ bool point_in_front(int k, D4 v) {
    if (finite4(v)) {
        const double s = (k & 1) ? -1.0 : 1.0;
        return dgt0(n_dot(k, __dsub_rn(axis_of(k, v), s), __dsub_rn(v.w, 1.0)));
    }
    D4 p, n;
    clip_plane(k, p, n);
    return dot4(sub4(v, p), n) > 0;
}

// Whether sutherlandHodgman (clipping.go:28-52) leaves anything of a
// triangle: planes the three vertices are all in front of pass the polygon
// through unchanged, so at the first plane they are not all in front of,
// no vertex in front means an empty result and some means real clipping.
__device__ __forceinline__ bool clip_leaves_something(D4 a, D4 b, D4 c) {
    for (int k = 0; k < 6; k++) {
        const int in = (int)point_in_front(k, a) + (int)point_in_front(k, b) + (int)point_in_front(k, c);
        if (in == 3) continue;
        return in > 0;
    }
    return true;  // in front of every plane: ClipTriangle returns the triangle itself
}

// drawClippedTriangle's cull decision (context.go:322-336) on NDC x/y.
// Returns +1 to draw in order (v0,v1,v2), -1 to draw swapped (v2,v1,v0),
// 0 when culled.
__device__ __forceinline__ int cull_decision(const StateView& st, double n0x, double n0y, double n1x, double n1y,
                                             double n2x, double n2y) {
    const double a = __dsub_rn(__dmul_rn(__dsub_rn(n1x, n0x), __dsub_rn(n2y, n0y)),
                               __dmul_rn(__dsub_rn(n2x, n0x), __dsub_rn(n1y, n0y)));
    const int order = ic_lt0(a) ? -1 : 1;  // a < 0
    // a = -a for a front-face cull and again for clockwise front faces (each
    // flips the sign bit), then a <= 0: zero or negative, not NaN
    const unsigned long long flip =
        ((st.cull == FGC_CULL_FRONT) != (st.front_face == FGC_FACE_CW)) ? 0x8000000000000000ull : 0ull;
    const unsigned long long b = dbits(a) ^ flip;
    const bool le0 = !bnan(b) && ((b & kAbsMask) == 0 || (b >> 63) != 0);
    if (st.cull != FGC_CULL_NONE && le0) return 0;
    return order;
}

// Emit the primitives of a triangle that survived culling: one, or six for
// wireframe (context.go:296-301, 344-348).
__device__ void emit_triangle(const GeomParams& P, const StateView& st, uint64_t slot, D3 s0, D3 s1, D3 s2,
                              double r0, double r1, double r2, uint32_t v0, uint32_t v1, uint32_t v2, uint32_t elem) {
    if (st.wireframe) {
        make_line_prims(P, st.line_width, slot + 0, s0, s1, r0, r1, v0, v1, elem);
        make_line_prims(P, st.line_width, slot + 2, s1, s2, r1, r2, v1, v2, elem);
        make_line_prims(P, st.line_width, slot + 4, s2, s0, r2, r0, v2, v0, elem);
    } else {
        make_prim(P, slot, s0, s1, s2, r0, r1, r2, v0, v1, v2, elem);
    }
}

// ---------------------------------------------------------------------------
// Setup: one thread per element. The pass's setup tiles run draw by draw,
// each draw's triangle tiles before its line tiles (DrawMesh draws lines after
// triangles, context.go:435-439), and the ordered allocation runs across all
// of them, so every draw's primitives are one contiguous, ordered range.
// Triangles take one slot (six in wireframe), or 7x that when they need
// clipping; lines always take two slots (dead when clipped away). The count
// kernel decides culling and clipping (and lists the clipped triangles),
// setup_kernel allocates; the surviving work items go to a list that
// setup_emit_kernel turns into raster primitives, while the clip kernels (on
// another stream) handle the clip entries.
// ---------------------------------------------------------------------------

// One piece of a triangle that survived culling: the whole triangle, or in
// wireframe its edge `piece` (two primitives at slot + 2*piece).
__device__ void emit_triangle_piece(const GeomParams& P, const ItemView& I, uint64_t t, uint64_t slot, int order,
                                    uint32_t u0, uint32_t u1, uint32_t u2, uint32_t piece) {
    uint32_t c0 = (uint32_t)(3 * t), c1 = c0 + 1, c2 = c0 + 2;
    if (order < 0) {  // swap v0 <-> v2
        uint32_t tu = u0; u0 = u2; u2 = tu;
        uint32_t tc = c0; c0 = c2; c2 = tc;
    }
    const VScreen* vscr = P.vscr + I.vbase;
    if (!I.st.wireframe) {
        const VScreen a = vscr[u0], b = vscr[u1], c = vscr[u2];
        make_prim(P, slot, d3(a.x, a.y, a.z), d3(b.x, b.y, b.z), d3(c.x, c.y, c.z), a.rw, b.rw, c.rw, c0, c1, c2,
                  (uint32_t)t);
        return;
    }
    // wireframe: line(v0, v1), line(v1, v2), line(v2, v0) (context.go:296-301)
    const uint32_t ua = piece == 0 ? u0 : piece == 1 ? u1 : u2;
    const uint32_t ub = piece == 0 ? u1 : piece == 1 ? u2 : u0;
    const uint32_t ca = piece == 0 ? c0 : piece == 1 ? c1 : c2;
    const uint32_t cb = piece == 0 ? c1 : piece == 1 ? c2 : c0;
    const VScreen a = vscr[ua], b = vscr[ub];
    make_line_prims(P, I.st.line_width, slot + 2 * piece, d3(a.x, a.y, a.z), d3(b.x, b.y, b.z), a.rw, b.rw, ca, cb,
                    (uint32_t)t);
}

// One element's setup decision: its primitive slots (count), the
// primitive-emitting pieces it hands to the emit kernel (work: a triangle,
// each edge of a wireframe triangle, or a line), or a clip entry instead.
struct SetupElem {
    uint32_t count, work, u0, u1, u2;
    int order;
    bool clip;
};
__device__ __forceinline__ SetupElem classify(const GeomParams& P, const ItemView& I, bool tri, uint64_t k,
                                              const uint8_t* vout) {
    SetupElem e{0, 0, 0, 0, 0, 0, false};
    if (tri) {
        if (k >= I.tri_count) return e;
        const int per = I.st.wireframe ? 6 : 1;
        const uint64_t t = I.tri_first + k;
        e.u0 = I.mesh.corner_uniq[3 * t + 0];
        e.u1 = I.mesh.corner_uniq[3 * t + 1];
        e.u2 = I.mesh.corner_uniq[3 * t + 2];
        e.clip = (vout[e.u0] | vout[e.u1] | vout[e.u2]) != 0;
        if (e.clip) {
            // a triangle the clipper empties needs no clip entry or slots
            const VClip* vc = P.vclip + I.vbase;
            const VClip a = vc[e.u0], b = vc[e.u1], c = vc[e.u2];
            if (!clip_leaves_something(d4(a.x, a.y, a.z, a.w), d4(b.x, b.y, b.z, b.w), d4(c.x, c.y, c.z, c.w)))
                e.clip = false;  // order stays 0: no primitives
        } else {
            const double2* vndc = P.vndc + I.vbase;
            const double2 n0 = vndc[e.u0], n1 = vndc[e.u1], n2 = vndc[e.u2];
            e.order = cull_decision(I.st, n0.x, n0.y, n1.x, n1.y, n2.x, n2.y);
        }
        e.count = e.clip ? (uint32_t)(7 * per) : (e.order != 0 ? (uint32_t)per : 0u);
        if (e.count != 0 && !e.clip) e.work = I.st.wireframe ? 3 : 1;
    } else {
        if (k >= I.line_count) return e;
        e.count = 2;
        const uint64_t cb = 3 * I.mesh.ntri + 2 * (I.line_first + k);
        e.u0 = I.mesh.corner_uniq[cb];
        e.u1 = I.mesh.corner_uniq[cb + 1];
        e.clip = (vout[e.u0] | vout[e.u1]) != 0;
        if (!e.clip) e.work = 1;
    }
    return e;
}

// The setup decision of an element in 16 bits: primitive slots (6 bits: 0,
// 1, 2, 6, 7 or 42), work items (2 bits), cull order + 1 (2 bits), clip.
__device__ __forceinline__ uint16_t pack_meta(const SetupElem& e) {
    return (uint16_t)(e.count | (e.work << 6) | ((uint32_t)(e.order + 1) << 8) | ((e.clip ? 1u : 0u) << 10));
}

// A setup tile: its draw, its index within the draw and its first element
// for this thread (kSetupPer consecutive elements per thread, so that the
// slots and work items of a thread's elements follow one another).
struct SetupTileOf {
    uint32_t item, lt;
    bool tri;
    uint64_t k0;
};
__device__ __forceinline__ SetupTileOf setup_tile_of(const GeomParams& P, uint32_t tile) {
    SetupTileOf T;
    T.item = find_item(P.starts.stile, P.nitems, tile);
    const ItemView& I = P.items[T.item];
    T.lt = tile - I.stile0;
    T.tri = T.lt < I.ntri_tiles;
    T.k0 = (uint64_t)(T.tri ? T.lt : T.lt - I.ntri_tiles) * (kSetupTile * kSetupPer) + (uint64_t)kSetupPer * threadIdx.x;
    return T;
}

// Setup in three launches, none of which waits on another block: the count
// kernel decides every element (culling, clipping, slots, work items) and
// sums each tile; one block scans the tile sums; the list kernel gives every
// element its slots and work-list positions from its tile's prefix and the
// block scan of the decisions.
__global__ void __launch_bounds__(kSetupTile) setup_count_kernel(GeomParams P) {
    __shared__ uint64_t s_warp[kSetupTile / 32 + 1];
    const uint32_t tile = blockIdx.x;
    const SetupTileOf T = setup_tile_of(P, tile);
    const ItemView& I = P.items[T.item];
    const uint8_t* vout = P.vout + I.vbase;
    const uint64_t e0 = (uint64_t)tile * (kSetupTile * kSetupPer) + (uint64_t)kSetupPer * threadIdx.x;
    uint32_t count = 0, work = 0;
#pragma unroll
    for (int j = 0; j < kSetupPer; j++) {
        const SetupElem e = classify(P, I, T.tri, T.k0 + j, vout);
        P.smeta[e0 + j] = pack_meta(e);
        count += e.count;
        work += e.work;
        if (T.tri && e.clip) {
            // a clip entry now (its slot follows from the scan: the list
            // writer fills it in), so that clipping starts before the scan
            const uint32_t idx = atomicAdd(P.clip_count, 1u);
            if (idx < P.clip_cap) P.clip_list[idx] = ClipEntry{~0ull, (uint32_t)(I.tri_first + T.k0 + j), T.item};
            else atomicOr(P.status, ST_CLIP_OVERFLOW);
            P.cidx[e0 + j] = idx;
        }
    }
    uint64_t agg;
    block_exclusive_scan<kSetupTile>(((uint64_t)count << 31) | work, s_warp, &agg);
    if (threadIdx.x == 0) P.tsum[tile] = agg;
}

// Exclusive scan of the tile sums in place, one block; the slot and work
// totals of the pass. Both fields of the packed sums stay below 2^31 (the
// host keeps a pass's slots and work items below it), so they add without
// carries into each other.
constexpr int kSetupScanThreads = 1024;
__global__ void __launch_bounds__(kSetupScanThreads) setup_scan_kernel(GeomParams P) {
    __shared__ uint64_t s_warp[kSetupScanThreads / 32 + 1];
    __shared__ uint64_t s_carry;
    constexpr int kPer = 4;
    if (threadIdx.x == 0) s_carry = 0;
    __syncthreads();
    for (uint64_t base = 0; base < P.ntiles; base += (uint64_t)kSetupScanThreads * kPer) {
        const uint64_t i0 = base + (uint64_t)threadIdx.x * kPer;
        uint64_t v[kPer], sum = 0;
#pragma unroll
        for (int j = 0; j < kPer; j++) {
            v[j] = (i0 + j < P.ntiles) ? P.tsum[i0 + j] : 0ull;
            sum += v[j];
        }
        uint64_t agg;
        uint64_t run = block_exclusive_scan<kSetupScanThreads>(sum, s_warp, &agg) + s_carry;
#pragma unroll
        for (int j = 0; j < kPer; j++) {
            if (i0 + j < P.ntiles) P.tsum[i0 + j] = run;
            run += v[j];
        }
        __syncthreads();
        if (threadIdx.x == 0) s_carry += agg;
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        *P.prim_total = s_carry >> 31;
        *P.work_total = s_carry & kLow31;
    }
}

__global__ void __launch_bounds__(kSetupTile) setup_kernel(GeomParams P) {
    __shared__ uint64_t s_warp[kSetupTile / 32 + 1];
    const uint32_t tile = blockIdx.x;
    const SetupTileOf T = setup_tile_of(P, tile);
    const ItemView& I = P.items[T.item];
    const bool tri = T.tri;
    const uint16_t* meta = P.smeta + (uint64_t)tile * (kSetupTile * kSetupPer) + (uint64_t)kSetupPer * threadIdx.x;
    uint16_t m[kSetupPer];
    uint32_t count = 0, work = 0;
#pragma unroll
    for (int j = 0; j < kSetupPer; j++) {
        m[j] = meta[j];
        count += m[j] & 63u;
        work += (m[j] >> 6) & 3u;
    }
    uint64_t agg;
    const uint64_t local = block_exclusive_scan<kSetupTile>(((uint64_t)count << 31) | work, s_warp, &agg);
    const uint64_t base = P.tsum[tile];
    uint64_t slot = (base >> 31) + (local >> 31);
    uint64_t wpos = (base & kLow31) + (local & kLow31);
    if (T.lt == 0 && threadIdx.x == 0) P.iout[T.item].prim_start = slot;  // thread 0's local prefix is 0
#pragma unroll
    for (int j = 0; j < kSetupPer; j++) {
        const uint32_t ecount = m[j] & 63u, ework = (m[j] >> 6) & 3u;
        const bool eclip = (m[j] >> 10) & 1u;
        const uint64_t k = T.k0 + j;
        if (ecount != 0 && eclip) {
            if (tri) {
                const uint32_t idx = P.cidx[(uint64_t)tile * (kSetupTile * kSetupPer) + (uint64_t)kSetupPer * threadIdx.x + j];
                if (idx < P.clip_cap) P.clip_list[idx].slot = slot;  // the count kernel listed it
            } else {
                uint32_t idx = atomicAdd(P.lclip_count, 1u);
                P.lclip_list[idx] = ClipEntry{slot, (uint32_t)(I.line_first + k), T.item};  // holds every line of the pass
            }
        }
        if (ework) {
            const uint32_t elem = (uint32_t)((tri ? I.tri_first : I.line_first) + k);
            const uint32_t meta8 = ((m[j] >> 8) & 3u) << 8 | (tri ? 0u : kWorkLine);
            uint32_t u0, u1, u2 = 0;
            if (tri) {
                u0 = I.mesh.corner_uniq[3 * (uint64_t)elem + 0];
                u1 = I.mesh.corner_uniq[3 * (uint64_t)elem + 1];
                u2 = I.mesh.corner_uniq[3 * (uint64_t)elem + 2];
            } else {
                const uint64_t cb = 3 * I.mesh.ntri + 2 * (uint64_t)elem;
                u0 = I.mesh.corner_uniq[cb];
                u1 = I.mesh.corner_uniq[cb + 1];
            }
            for (uint32_t w = 0; w < ework; w++) {
                if (wpos + w >= P.work_cap) {  // sized for every element: not reached
                    atomicOr(P.status, ST_RASTER_INTERNAL);
                    break;
                }
                P.work[wpos + w] = SetupWork{slot, elem, T.item, u0, u1, u2, meta8 | w};
            }
        }
        slot += ecount;
        wpos += ework;
    }
}

// The FP64 half of setup: one thread per work item, every lane busy (the
// work list holds only what survived culling), no barriers.
__global__ void __launch_bounds__(256, 3) setup_emit_kernel(GeomParams P) {
    // a look-back wait that gave up (a scan of an earlier pass) leaves the
    // pass to be reported as failed: emit nothing
    if (*P.status & ST_LOOKBACK_TIMEOUT) return;
    if (blockIdx.x == 0)  // each draw's primitive range: setup_kernel wrote the starts and the total
        for (uint32_t i = threadIdx.x; i < P.nitems; i += blockDim.x)
            P.iout[i].prim_end = (i + 1 < P.nitems) ? P.iout[i + 1].prim_start : *P.prim_total;
    const uint64_t n = min((uint64_t)*P.work_total, P.work_cap);
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const SetupWork w = P.work[i];
        const ItemView& I = P.items[w.item];
        const uint32_t piece = w.meta & 0xFFu;
        if (w.meta & kWorkLine) {
            const uint64_t cb = 3 * I.mesh.ntri + 2 * (uint64_t)w.elem;
            const VScreen* vscr = P.vscr + I.vbase;
            const VScreen a = vscr[w.u0], b = vscr[w.u1];
            make_line_prims(P, I.st.line_width, w.slot, d3(a.x, a.y, a.z), d3(b.x, b.y, b.z), a.rw, b.rw,
                            (uint32_t)cb, (uint32_t)(cb + 1), kLineFlag | w.elem);
        } else {
            const int order = (int)((w.meta >> 8) & 0xFFu) - 1;
            emit_triangle_piece(P, I, w.elem, w.slot, order, w.u0, w.u1, w.u2, piece);
        }
    }
}

// ---------------------------------------------------------------------------
// Clipping (clipping.go)
// ---------------------------------------------------------------------------

__device__ __forceinline__ D4 intersect_segment(int k, D4 v0, D4 v1) {  // clipping.go:20-26
    const D4 u = sub4(v1, v0);
    double d = 0, nn = 0;
    bool full = !(finite4(u) && finite4(v0));
    if (!full) {
        // the short form of both dot products (u and w = v0 - P finite); a
        // zero result takes the full form, where its sign matters
        const double s = (k & 1) ? -1.0 : 1.0;
        d = n_dot(k, axis_of(k, u), u.w);
        nn = -n_dot(k, __dsub_rn(axis_of(k, v0), s), __dsub_rn(v0.w, 1.0));
        full = (dbits(d) & kAbsMask) == 0 || (dbits(nn) & kAbsMask) == 0;
    }
    if (full) {
        D4 p, n;
        clip_plane(k, p, n);
        d = dot4(n, u);
        nn = -dot4(n, sub4(v0, p));
    }
    return add4(v0, muls4(u, __ddiv_rn(nn, d)));
}

// Barycentric (vertex.go:81-95).
__device__ D4 barycentric(D3 p1, D3 p2, D3 p3, D3 p) {
    D3 v0 = sub3(p2, p1), v1 = sub3(p3, p1), v2 = sub3(p, p1);
    double d00 = dot3(v0, v0), d01 = dot3(v0, v1), d11 = dot3(v1, v1);
    double d20 = dot3(v2, v0), d21 = dot3(v2, v1);
    double d = __dsub_rn(__dmul_rn(d00, d11), __dmul_rn(d01, d01));
    double v = __ddiv_rn(__dsub_rn(__dmul_rn(d11, d20), __dmul_rn(d01, d21)), d);
    double w = __ddiv_rn(__dsub_rn(__dmul_rn(d00, d21), __dmul_rn(d01, d20)), d);
    double u = __dsub_rn(__dsub_rn(1.0, v), w);
    return d4(u, v, w, 1.0);
}

struct FullVertex {
    D3 pos, nrm;
    double tu, tv, tz;
    D4 col;
    D4 out;
};

// ((0 + a*bX) + b*bY + c*bZ) * bW for one component (vertex.go:49-79).
__device__ __forceinline__ double interp1(double a, double b, double c, D4 w) {
    double n = zero_plus(__dmul_rn(a, w.x));
    n = __dadd_rn(n, __dmul_rn(b, w.y));
    n = __dadd_rn(n, __dmul_rn(c, w.z));
    return __dmul_rn(n, w.w);
}

// InterpolateVertexes (vertex.go:18-47), split so that the clip-space
// Output (which decides culling) is formed first and the other attributes
// only when the piece survives and the shader reads them: an attribute no
// shader reads never reaches an output, so skipping it changes nothing.
__device__ __forceinline__ D4 interp_out(const FullVertex& a, const FullVertex& b, const FullVertex& c, D4 w) {
    return d4(interp1(a.out.x, b.out.x, c.out.x, w), interp1(a.out.y, b.out.y, c.out.y, w),
              interp1(a.out.z, b.out.z, c.out.z, w), interp1(a.out.w, b.out.w, c.out.w, w));
}

__device__ void interp_attrs(FullVertex& v, const FullVertex& a, const FullVertex& b, const FullVertex& c, D4 w,
                             uint32_t mask) {
    if (mask & kAttrPos)
        v.pos = d3(interp1(a.pos.x, b.pos.x, c.pos.x, w), interp1(a.pos.y, b.pos.y, c.pos.y, w),
                   interp1(a.pos.z, b.pos.z, c.pos.z, w));
    else
        v.pos = d3(0, 0, 0);
    if (mask & kAttrNrm)
        v.nrm = normalize3(d3(interp1(a.nrm.x, b.nrm.x, c.nrm.x, w), interp1(a.nrm.y, b.nrm.y, c.nrm.y, w),
                              interp1(a.nrm.z, b.nrm.z, c.nrm.z, w)));
    else
        v.nrm = d3(0, 0, 0);
    if (mask & kAttrTex) {
        v.tu = interp1(a.tu, b.tu, c.tu, w);
        v.tv = interp1(a.tv, b.tv, c.tv, w);
    } else {
        v.tu = v.tv = 0.0;
    }
    v.tz = 0.0;
    if (mask & kAttrCol)
        v.col = d4(interp1(a.col.x, b.col.x, c.col.x, w), interp1(a.col.y, b.col.y, c.col.y, w),
                   interp1(a.col.z, b.col.z, c.col.z, w), interp1(a.col.w, b.col.w, c.col.w, w));
    else
        v.col = d4(0, 0, 0, 0);
}

// FixNormals (triangle.go:46-58).
// The face normal is formed only when a vertex normal is zero (== 0 as IEEE
// compares, either sign): otherwise nothing reads it.
__device__ __forceinline__ bool zero3(D3 v) { return dzero(v.x) && dzero(v.y) && dzero(v.z); }
__device__ void fix_normals(FullVertex& a, FullVertex& b, FullVertex& c) {
    const bool za = zero3(a.nrm), zb = zero3(b.nrm), zc = zero3(c.nrm);
    if (!(za || zb || zc)) return;
    const D3 n = normalize3(cross3(sub3(b.pos, a.pos), sub3(c.pos, a.pos)));
    if (za) a.nrm = n;
    if (zb) b.nrm = n;
    if (zc) c.nrm = n;
}

__device__ FullVertex load_corner(const GeomParams& P, const ItemView& I, uint64_t corner) {
    FullVertex v;
    const MeshView& M = I.mesh;
    APosNrm64 pn = M.pn64[corner];
    v.pos = d3(pn.px, pn.py, pn.pz);
    v.nrm = d3(pn.nx, pn.ny, pn.nz);
    v.tu = M.tex64 ? M.tex64[2 * corner] : 0.0;
    v.tv = M.tex64 ? M.tex64[2 * corner + 1] : 0.0;
    v.tz = 0.0;
    if (M.col64) {
        v.col = d4(M.col64[4 * corner], M.col64[4 * corner + 1], M.col64[4 * corner + 2], M.col64[4 * corner + 3]);
    } else {
        v.col = d4(0, 0, 0, 0);
    }
    VClip o = P.vclip[I.vbase + M.corner_uniq[corner]];
    v.out = d4(o.x, o.y, o.z, o.w);
    return v;
}

// ClipTriangle (clipping.go:54-74) + drawClippedTriangle for each piece, in
// three steps. Entry e owns primitive slots [base, base + 7*per) and pool
// vertices [21e, 21e + 21).
//   clip_poly_kernel    one thread per entry: sutherlandHodgman on the
//                       corners' Output (clipping.go:28-52)
//   clip_vert_kernel    one thread per polygon vertex: Barycentric weights of
//                       its clip-space point w.r.t. the original triangle,
//                       InterpolateVertexes of Output and of the attributes
//                       the shader reads (clipping.go:61-65), its NDC position
//   clip_piece_kernel   one thread per fan piece (0, i-1, i): the cull
//                       decision, FixNormals of the piece's own copies and
//                       the raster primitive (context.go:316-349)
// The results are those of one thread doing all three in turn: each polygon
// vertex is still built once and shared by the pieces that use it. The
// kernels run on a side stream: the first two beside the scan and the list
// writer, the third (it needs the slots the list writer assigns) beside the
// emission.
__device__ __forceinline__ FullVertex clip_vertex(const FullVertex* tv, D3 p1, D3 p2, D3 p3, D4 q, uint32_t mask) {
    const D4 bw = barycentric(p1, p2, p3, d3(q.x, q.y, q.z));
    FullVertex v;
    v.out = interp_out(tv[0], tv[1], tv[2], bw);
    interp_attrs(v, tv[0], tv[1], tv[2], bw, mask);
    return v;
}

__global__ void __launch_bounds__(32) clip_poly_kernel(GeomParams P) {
    const uint32_t n = min(*P.clip_count, P.clip_cap);
    for (uint32_t e = blockIdx.x * blockDim.x + threadIdx.x; e < n; e += gridDim.x * blockDim.x) {
        const ClipEntry ent = P.clip_list[e];
        const ItemView& I = P.items[ent.item];
        const uint64_t t = ent.elem;
        const VClip* vc = P.vclip + I.vbase;
        // sutherlandHodgman (clipping.go:28-52). Each plane adds at most one
        // vertex to a convex polygon (9 after six planes); the buffers hold 16
        // and drop vertices beyond that, which only a polygon made non-convex
        // by rounding at several planes could reach. A vertex's side of the
        // plane is computed once and reused as the next edge's start.
        constexpr int kPolyMax = 16;
        D4 bufa[kPolyMax], bufb[kPolyMax];
        for (int c = 0; c < 3; c++) {
            const VClip o = vc[I.mesh.corner_uniq[3 * t + c]];
            bufa[c] = d4(o.x, o.y, o.z, o.w);
        }
        int nin = 3;
        D4* in = bufa;
        D4* out = bufb;
        for (int k = 0; k < 6 && nin > 0; k++) {
            int no = 0;
            D4 s = in[nin - 1];
            bool sf = point_in_front(k, s);
            for (int j = 0; j < nin; j++) {
                const D4 ev = in[j];
                const bool ef = point_in_front(k, ev);
                // an edge that crosses the plane adds its intersection, then
                // its end if that is in front
                if (ef != sf && no < kPolyMax) out[no++] = intersect_segment(k, s, ev);
                if (ef && no < kPolyMax) out[no++] = ev;
                s = ev;
                sf = ef;
            }
            D4* tmp = in; in = out; out = tmp;
            nin = no;
        }
        ClipPoly& cp = P.cpoly[e];
        cp.n = (uint32_t)nin;
        for (int j = 0; j < nin && j < kClipPoly; j++) cp.v[j] = in[j];
    }
}

__global__ void __launch_bounds__(64) clip_vert_kernel(GeomParams P) {
    const uint64_t n = (uint64_t)min(*P.clip_count, P.clip_cap) * kClipPoly;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t e = (uint32_t)(i / kClipPoly), j = (uint32_t)(i % kClipPoly);
        const uint32_t np = P.cpoly[e].n;
        if (np < 3 || j >= np) continue;  // no fan, or a vertex the fan does not read
        const ClipEntry ent = P.clip_list[e];
        const ItemView& I = P.items[ent.item];
        const uint32_t mask = I.attr_mask;
        FullVertex tv[3];
        for (int c = 0; c < 3; c++) tv[c] = load_corner(P, I, 3 * (uint64_t)ent.elem + c);
        if (mask & kAttrNrm) fix_normals(tv[0], tv[1], tv[2]);  // NewTriangle(v1, v2, v3)
        const D3 p1 = d3(tv[0].out.x, tv[0].out.y, tv[0].out.z);
        const D3 p2 = d3(tv[1].out.x, tv[1].out.y, tv[1].out.z);
        const D3 p3 = d3(tv[2].out.x, tv[2].out.y, tv[2].out.z);
        const FullVertex v = clip_vertex(tv, p1, p2, p3, P.cpoly[e].v[j], mask);
        const D3 nd = ndc_of(v.out);
        P.cvert[i] = ClipVert{v.pos.x, v.pos.y, v.pos.z, v.nrm.x, v.nrm.y, v.nrm.z, v.tu, v.tv,
                              v.col.x, v.col.y, v.col.z, v.col.w, v.out.x, v.out.y, v.out.z, v.out.w,
                              nd.x, nd.y, nd.z};
    }
}

__device__ __forceinline__ FullVertex clip_vert_load(const ClipVert& c, D3& nd) {
    FullVertex v;
    v.pos = d3(c.px, c.py, c.pz);
    v.nrm = d3(c.nx, c.ny, c.nz);
    v.tu = c.tu;
    v.tv = c.tv;
    v.tz = 0.0;
    v.col = d4(c.cr, c.cg, c.cb, c.ca);
    v.out = d4(c.ox, c.oy, c.oz, c.ow);
    nd = d3(c.sx, c.sy, c.sz);
    return v;
}

__global__ void __launch_bounds__(64) clip_piece_kernel(GeomParams P) {
    const uint64_t n = (uint64_t)min(*P.clip_count, P.clip_cap) * 7;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t e = (uint32_t)(i / 7), sub = (uint32_t)(i % 7);
        const ClipEntry ent = P.clip_list[e];
        const ItemView& I = P.items[ent.item];
        const int per = I.st.wireframe ? 6 : 1;
        const uint64_t slot = ent.slot + (uint64_t)sub * per;
        const uint32_t np = P.cpoly[e].n;
        if (np < 3 || sub + 2 >= np) {  // the fan (0, i-1, i), i = 2 .. np-1, has no piece here
            for (int q = 0; q < per; q++) write_dead(P, slot + q);
            continue;
        }
        const uint32_t mask = I.attr_mask;
        const ClipVert* cv = P.cvert + (uint64_t)e * kClipPoly;
        D3 nn[3];
        FullVertex v[3] = {clip_vert_load(cv[0], nn[0]), clip_vert_load(cv[sub + 1], nn[1]),
                           clip_vert_load(cv[sub + 2], nn[2])};
        // drawClippedTriangle (context.go:316-349)
        const int order = cull_decision(I.st, nn[0].x, nn[0].y, nn[1].x, nn[1].y, nn[2].x, nn[2].y);
        if (order == 0) {
            for (int q = 0; q < per; q++) write_dead(P, slot + q);
            continue;
        }
        if (mask & kAttrNrm) fix_normals(v[0], v[1], v[2]);  // NewTriangle
        uint32_t pref[3];
        for (int c = 0; c < 3; c++) {
            const uint32_t pi = e * 21 + sub * 3 + c;
            if (mask) {
                P.pool[pi] = PoolVertex{v[c].pos.x, v[c].pos.y, v[c].pos.z, v[c].nrm.x, v[c].nrm.y, v[c].nrm.z,
                                        v[c].tu, v[c].tv, v[c].col.x, v[c].col.y, v[c].col.z, v[c].col.w};
                if (I.st.precision == FGC_PRECISION_MIXED)
                    P.pool32[pi] = PoolVertex32{(float)v[c].pos.x, (float)v[c].pos.y, (float)v[c].pos.z,
                                                (float)v[c].nrm.x, (float)v[c].nrm.y, (float)v[c].nrm.z,
                                                (float)v[c].tu, (float)v[c].tv, (float)v[c].col.x,
                                                (float)v[c].col.y, (float)v[c].col.z, (float)v[c].col.w};
            }
            pref[c] = kPoolFlag | pi;
        }
        int i0 = 0, i2 = 2;
        if (order < 0) { i0 = 2; i2 = 0; }
        const D3 s0 = screen_of_ndc(nn[i0], I.w2, I.h2);
        const D3 s1 = screen_of_ndc(nn[1], I.w2, I.h2);
        const D3 s2 = screen_of_ndc(nn[i2], I.w2, I.h2);
        emit_triangle(P, I.st, slot, s0, s1, s2, __drcp_rn(v[i0].out.w), __drcp_rn(v[1].out.w),
                      __drcp_rn(v[i2].out.w), pref[i0], pref[1], pref[i2], (uint32_t)ent.elem);
    }
}

// ClipLine (clipping.go:76-98) + drawClippedLine (context.go:303-314): only
// Output moves, the attributes stay the line's own.
__global__ void __launch_bounds__(128) clip_lines_kernel(GeomParams P) {
    uint32_t n = *P.lclip_count;
    for (uint32_t e = blockIdx.x * blockDim.x + threadIdx.x; e < n; e += gridDim.x * blockDim.x) {
        const ClipEntry ent = P.lclip_list[e];
        const ItemView& I = P.items[ent.item];
        const uint64_t l = ent.elem, slot = ent.slot;
        uint64_t cb = 3 * I.mesh.ntri + 2 * l;
        const VClip* vclip = P.vclip + I.vbase;
        VClip a = vclip[I.mesh.corner_uniq[cb]], b = vclip[I.mesh.corner_uniq[cb + 1]];
        D4 w1 = d4(a.x, a.y, a.z, a.w), w2 = d4(b.x, b.y, b.z, b.w);
        bool culled = false;
        for (int k = 0; k < 6; k++) {
            bool f1 = point_in_front(k, w1), f2 = point_in_front(k, w2);
            if (f1 && f2) continue;
            else if (f1) w2 = intersect_segment(k, w1, w2);
            else if (f2) w1 = intersect_segment(k, w2, w1);
            else { culled = true; break; }
        }
        if (culled) {
            write_dead(P, slot);
            write_dead(P, slot + 1);
            continue;
        }
        D3 s0 = screen_of_ndc(ndc_of(w1), I.w2, I.h2);
        D3 s1 = screen_of_ndc(ndc_of(w2), I.w2, I.h2);
        make_line_prims(P, I.st.line_width, slot, s0, s1, __ddiv_rn(1.0, w1.w), __ddiv_rn(1.0, w2.w), (uint32_t)cb,
                        (uint32_t)(cb + 1), kLineFlag | (uint32_t)l);
    }
}

// Each draw's primitive range ends where the next draw's begins (the last
// ends at the pass total). One thread per draw.
}  // namespace fgc
