/* TEST INFRASTRUCTURE ONLY: C restatement of the reference's mesh preparation
 * around the draw path -- the checker for the device versions in
 * fauxgl_gb300/csrc/fgc_meshops.cu. Never linked into the product.
 *
 *   oracle_stl_parse                 LoadSTL (stl.go:23-57), loadSTLA (stl.go:59-80),
 *                                    makeFloat (stl.go:82-84), loadSTLB (stl.go:86-154),
 *                                    Triangle.Normal (triangle.go:33-37)
 *   oracle_smooth_normals_threshold  smoothNormalsThreshold / SmoothNormalsThreshold
 *                                    (mesh.go:80-103)
 *   oracle_smooth_normals            SmoothNormals (mesh.go:105-120)
 *   oracle_sharp_edges               SharpEdges (mesh.go:258-292)
 *   oracle_silhouette                silhouette (silhouette.go:3-53), Mesh.Silhouette
 *                                    (mesh.go:207-209)
 *
 * Go's map[Vector] compares keys with == on float64: -0 and +0 are one key and
 * a key holding NaN never matches, so every insertion of it is a new entry and
 * every lookup of it finds nothing. The restatement groups corners the same
 * way (sorting by position, NaN positions ungrouped) and keeps each group in
 * corner order, the order of the reference's appends.
 *
 * Vector arithmetic follows vector.go literally (left to right, no fused
 * multiply-add: built with -ffp-contract=off).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "fauxgl_oracle.h"

typedef struct {
    double x, y, z;
} V3;

static V3 v3(double x, double y, double z) {
    V3 r = {x, y, z};
    return r;
}
static V3 vsub(V3 a, V3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
static V3 vadd(V3 a, V3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
static V3 vmuls(V3 a, double s) { return v3(a.x * s, a.y * s, a.z * s); }
static double vdot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static V3 vcross(V3 a, V3 b) {  /* vector.go:76-81 */
    return v3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
static V3 vnormalize(V3 a) {  /* vector.go:83-86 */
    double r = 1 / sqrt(a.x * a.x + a.y * a.y + a.z * a.z);
    return v3(a.x * r, a.y * r, a.z * r);
}
static int vless(V3 a, V3 b) {  /* vector.go:42-50 */
    if (a.x != b.x) return a.x < b.x;
    if (a.y != b.y) return a.y < b.y;
    return a.z < b.z;
}
static int vhas_nan(V3 a) { return a.x != a.x || a.y != a.y || a.z != a.z; }
static V3 corner(const double* p, uint64_t c) { return v3(p[3 * c], p[3 * c + 1], p[3 * c + 2]); }

/* Triangle.Normal (triangle.go:33-37) */
static V3 face_normal(V3 p1, V3 p2, V3 p3) { return vnormalize(vcross(vsub(p2, p1), vsub(p3, p1))); }

/* ---------------------------------------------------------------------- */
/* STL                                                                     */
/* ---------------------------------------------------------------------- */
static double le_float(const uint8_t* b) { /* makeFloat: float64(Float32frombits(LE)) */
    uint32_t u = (uint32_t)b[0] | ((uint32_t)b[1] << 8) | ((uint32_t)b[2] << 16) | ((uint32_t)b[3] << 24);
    float f;
    memcpy(&f, &u, 4);
    return (double)f;
}

/* A field of a "vertex x y z" line: strconv.ParseFloat with the error
 * ignored -- the value, or 0 when the field is not a number as a whole. */
static double parse_field(const char* s, size_t n) {
    char buf[128];
    if (n >= sizeof(buf)) return 0;
    memcpy(buf, s, n);
    buf[n] = 0;
    char* end = NULL;
    double v = strtod(buf, &end);
    if (end != buf + n) return 0;
    return v;
}

/* Returns the triangle count (positions and face normals written when the
 * arrays hold cap triangles), -1 for data too short for a header, -2 for an
 * ASCII vertex count that is not a multiple of three. */
int64_t oracle_stl_parse(const uint8_t* data, uint64_t n, double* tri_pos, double* tri_nrm, uint64_t cap) {
    if (n < 84) return -1;
    uint32_t count = (uint32_t)data[80] | ((uint32_t)data[81] << 8) | ((uint32_t)data[82] << 16) |
                     ((uint32_t)data[83] << 24);
    if ((uint64_t)count * 50 + 84 == n) {
        for (uint64_t i = 0; i < count && i < cap; i++) {
            const uint8_t* r = data + 84 + 50 * i;
            V3 p[3];
            for (int k = 0; k < 3; k++) p[k] = v3(le_float(r + 12 + 12 * k), le_float(r + 16 + 12 * k), le_float(r + 20 + 12 * k));
            V3 nn = face_normal(p[0], p[1], p[2]);
            for (int k = 0; k < 3; k++) {
                double* q = tri_pos + 9 * i + 3 * k;
                q[0] = p[k].x; q[1] = p[k].y; q[2] = p[k].z;
                double* m = tri_nrm + 9 * i + 3 * k;
                m[0] = nn.x; m[1] = nn.y; m[2] = nn.z;
            }
        }
        return count;
    }
    /* ASCII: every line whose whitespace-separated fields are exactly
     * "vertex x y z"; consecutive triples are triangles (FixNormals sets the
     * zero normals to the face normal) */
    uint64_t nv = 0;
    uint64_t i = 0;
    while (i < n) {
        uint64_t e = i;
        while (e < n && data[e] != '\n') e++;
        const char* f[5];
        size_t fl[5];
        int nf = 0;
        uint64_t j = i;
        while (j < e) {
            while (j < e && (data[j] == ' ' || data[j] == '\t' || data[j] == '\r' || data[j] == '\v' || data[j] == '\f')) j++;
            if (j >= e) break;
            uint64_t s = j;
            while (j < e && !(data[j] == ' ' || data[j] == '\t' || data[j] == '\r' || data[j] == '\v' || data[j] == '\f')) j++;
            if (nf < 5) {
                f[nf] = (const char*)data + s;
                fl[nf] = (size_t)(j - s);
            }
            nf++;
        }
        if (nf == 4 && fl[0] == 6 && memcmp(f[0], "vertex", 6) == 0) {
            if (nv / 3 < cap) {
                double* q = tri_pos + 3 * nv;
                q[0] = parse_field(f[1], fl[1]);
                q[1] = parse_field(f[2], fl[2]);
                q[2] = parse_field(f[3], fl[3]);
            }
            nv++;
        }
        i = e + 1;
    }
    if (nv % 3) return -2;
    for (uint64_t t = 0; t < nv / 3 && t < cap; t++) {
        V3 nn = face_normal(corner(tri_pos, 3 * t), corner(tri_pos, 3 * t + 1), corner(tri_pos, 3 * t + 2));
        for (int k = 0; k < 3; k++) {
            double* m = tri_nrm + 9 * t + 3 * k;
            m[0] = nn.x; m[1] = nn.y; m[2] = nn.z;
        }
    }
    return (int64_t)(nv / 3);
}

/* ---------------------------------------------------------------------- */
/* Position groups (map[Vector] keys)                                      */
/* ---------------------------------------------------------------------- */
static const double* g_pos;

static int cmp_corner(const void* pa, const void* pb) {
    uint64_t a = *(const uint64_t*)pa, b = *(const uint64_t*)pb;
    V3 u = corner(g_pos, a), v = corner(g_pos, b);
    int na = vhas_nan(u), nb = vhas_nan(v);
    if (na != nb) return na - nb;  /* NaN keys last */
    if (!na) {
        if (u.x != v.x) return u.x < v.x ? -1 : 1;
        if (u.y != v.y) return u.y < v.y ? -1 : 1;
        if (u.z != v.z) return u.z < v.z ? -1 : 1;
    }
    return a < b ? -1 : (a > b ? 1 : 0);  /* corner order inside a key */
}

static int same_key(V3 u, V3 v) { return u.x == v.x && u.y == v.y && u.z == v.z; }

/* order: corners sorted by key then corner; gstart[c] / gcount[c]: the range
 * of c's group in order (count 0 for NaN keys, which find nothing). */
static void position_groups(const double* pos, uint64_t nc, uint64_t* order, uint64_t* gstart, uint64_t* gcount) {
    for (uint64_t c = 0; c < nc; c++) order[c] = c;
    g_pos = pos;
    qsort(order, nc, sizeof(uint64_t), cmp_corner);
    uint64_t i = 0;
    while (i < nc) {
        V3 u = corner(pos, order[i]);
        if (vhas_nan(u)) {
            gstart[order[i]] = i;
            gcount[order[i]] = 0;
            i++;
            continue;
        }
        uint64_t j = i + 1;
        while (j < nc && same_key(u, corner(pos, order[j]))) j++;
        for (uint64_t k = i; k < j; k++) {
            gstart[order[k]] = i;
            gcount[order[k]] = j - i;
        }
        i = j;
    }
}

void oracle_smooth_normals_threshold(const double* tri_pos, double* tri_nrm, uint64_t ntri, double threshold) {
    const uint64_t nc = 3 * ntri;
    uint64_t* order = malloc(nc * sizeof(uint64_t) + 1);
    uint64_t* gs = malloc(nc * sizeof(uint64_t) + 1);
    uint64_t* gc = malloc(nc * sizeof(uint64_t) + 1);
    double* out = malloc(nc * 3 * sizeof(double) + 1);
    position_groups(tri_pos, nc, order, gs, gc);
    for (uint64_t c = 0; c < nc; c++) {
        V3 normal = corner(tri_nrm, c);
        V3 result = v3(0, 0, 0);
        for (uint64_t k = 0; k < gc[c]; k++) {
            V3 x = corner(tri_nrm, order[gs[c] + k]);
            if (vdot(x, normal) >= threshold) result = vadd(result, x);
        }
        V3 r = vnormalize(result);
        out[3 * c] = r.x; out[3 * c + 1] = r.y; out[3 * c + 2] = r.z;
    }
    memcpy(tri_nrm, out, nc * 3 * sizeof(double));
    free(order); free(gs); free(gc); free(out);
}

void oracle_smooth_normals(const double* tri_pos, double* tri_nrm, uint64_t ntri) {
    const uint64_t nc = 3 * ntri;
    uint64_t* order = malloc(nc * sizeof(uint64_t) + 1);
    uint64_t* gs = malloc(nc * sizeof(uint64_t) + 1);
    uint64_t* gc = malloc(nc * sizeof(uint64_t) + 1);
    double* out = malloc(nc * 3 * sizeof(double) + 1);
    position_groups(tri_pos, nc, order, gs, gc);
    for (uint64_t c = 0; c < nc; c++) {
        V3 r = v3(0, 0, 0);  /* a NaN key is never found: the zero Vector */
        if (gc[c]) {
            V3 sum = v3(0, 0, 0);
            for (uint64_t k = 0; k < gc[c]; k++) sum = vadd(sum, corner(tri_nrm, order[gs[c] + k]));
            r = vnormalize(sum);
        }
        out[3 * c] = r.x; out[3 * c + 1] = r.y; out[3 * c + 2] = r.z;
    }
    memcpy(tri_nrm, out, nc * 3 * sizeof(double));
    free(order); free(gs); free(gc); free(out);
}

/* ---------------------------------------------------------------------- */
/* SharpEdges                                                              */
/* ---------------------------------------------------------------------- */
typedef struct {
    V3 a, b;      /* makeEdge: ordered by Less */
    uint64_t occ; /* 3 * triangle + edge */
} EdgeOcc;

static int edge_nan(const EdgeOcc* e) { return vhas_nan(e->a) || vhas_nan(e->b); }

static int cmp_edge(const void* pa, const void* pb) {
    const EdgeOcc* a = pa;
    const EdgeOcc* b = pb;
    int na = edge_nan(a), nb = edge_nan(b);
    if (na != nb) return na - nb;
    if (!na) {
        const double ka[6] = {a->a.x, a->a.y, a->a.z, a->b.x, a->b.y, a->b.z};
        const double kb[6] = {b->a.x, b->a.y, b->a.z, b->b.x, b->b.y, b->b.z};
        for (int i = 0; i < 6; i++)
            if (ka[i] != kb[i]) return ka[i] < kb[i] ? -1 : 1;
    }
    return a->occ < b->occ ? -1 : (a->occ > b->occ ? 1 : 0);
}

static int same_edge(const EdgeOcc* a, const EdgeOcc* b) {
    return !edge_nan(a) && !edge_nan(b) && same_key(a->a, b->a) && same_key(a->b, b->b);
}

static EdgeOcc make_edge(V3 a, V3 b, uint64_t occ) {
    EdgeOcc e;
    if (vless(a, b)) { e.a = a; e.b = b; } else { e.a = b; e.b = a; }
    e.occ = occ;
    return e;
}

/* Lines (6 doubles: A then B) in the reference's emission order; returns
 * their count (written up to cap). */
int64_t oracle_sharp_edges(const double* tri_pos, uint64_t ntri, double angle_threshold, double* out, uint64_t cap) {
    const uint64_t ne = 3 * ntri;
    EdgeOcc* e = malloc(ne * sizeof(EdgeOcc) + 1);
    for (uint64_t t = 0; t < ntri; t++) {
        V3 p1 = corner(tri_pos, 3 * t), p2 = corner(tri_pos, 3 * t + 1), p3 = corner(tri_pos, 3 * t + 2);
        e[3 * t] = make_edge(p1, p2, 3 * t);
        e[3 * t + 1] = make_edge(p2, p3, 3 * t + 1);
        e[3 * t + 2] = make_edge(p3, p1, 3 * t + 2);
    }
    /* other[e] before triangle t: the last earlier triangle holding an equal
     * edge (any of its three), found from the occurrences sorted by key */
    EdgeOcc* s = malloc(ne * sizeof(EdgeOcc) + 1);
    memcpy(s, e, ne * sizeof(EdgeOcc));
    qsort(s, ne, sizeof(EdgeOcc), cmp_edge);
    int64_t* prev = malloc(ne * sizeof(int64_t) + 1);  /* previous triangle per occurrence, or -1 */
    for (uint64_t i = 0; i < ne; i++) {
        int64_t p = -1;
        const uint64_t t = s[i].occ / 3;
        for (uint64_t j = i; j-- > 0;) {
            if (!same_edge(&s[j], &s[i])) break;
            if (s[j].occ / 3 < t) {
                p = (int64_t)(s[j].occ / 3);
                break;
            }
        }
        prev[s[i].occ] = p;
    }
    int64_t nl = 0;
    for (uint64_t t = 0; t < ntri; t++) {
        V3 nt = face_normal(corner(tri_pos, 3 * t), corner(tri_pos, 3 * t + 1), corner(tri_pos, 3 * t + 2));
        for (int k = 0; k < 3; k++) {
            const int64_t u = prev[3 * t + k];
            if (u < 0) continue;
            V3 nu = face_normal(corner(tri_pos, 3 * u), corner(tri_pos, 3 * u + 1), corner(tri_pos, 3 * u + 2));
            double a = acos(vdot(nt, nu));
            if (a > angle_threshold) {
                if ((uint64_t)nl < cap) {
                    const EdgeOcc* q = &e[3 * t + k];
                    double* o = out + 6 * nl;
                    o[0] = q->a.x; o[1] = q->a.y; o[2] = q->a.z;
                    o[3] = q->b.x; o[4] = q->b.y; o[5] = q->b.z;
                }
                nl++;
            }
        }
    }
    free(e); free(s); free(prev);
    return nl;
}

/* ---------------------------------------------------------------------- */
/* silhouette                                                              */
/* ---------------------------------------------------------------------- */
static V3 lerp_g(V3 p1, V3 p2, double w1, double w2) {  /* silhouette.go:6-9, vector.go:64-66 */
    double t = -w1 / (w2 - w1);
    return vadd(p1, vmuls(vsub(p2, p1), t));
}

int64_t oracle_silhouette(const double* tri_pos, const double* tri_nrm, uint64_t ntri, const double eye_in[3],
                          double offset, double* out, uint64_t cap) {
    const uint64_t nc = 3 * ntri;
    double* nrm = malloc(nc * 3 * sizeof(double) + 1);
    memcpy(nrm, tri_nrm, nc * 3 * sizeof(double));
    oracle_smooth_normals(tri_pos, nrm, ntri);  /* on the copy */
    const V3 eye = v3(eye_in[0], eye_in[1], eye_in[2]);
    int64_t nl = 0;
    for (uint64_t t = 0; t < ntri; t++) {
        V3 p1 = corner(tri_pos, 3 * t), p2 = corner(tri_pos, 3 * t + 1), p3 = corner(tri_pos, 3 * t + 2);
        V3 n1 = corner(nrm, 3 * t), n2 = corner(nrm, 3 * t + 1), n3 = corner(nrm, 3 * t + 2);
        double g1 = vdot(n1, vsub(p1, eye));
        double g2 = vdot(n2, vsub(p2, eye));
        double g3 = vdot(n3, vsub(p3, eye));
        int b1 = g1 > 0, b2 = g2 > 0, b3 = g3 > 0;
        if (b1 == b2 && b2 == b3) continue;
        V3 v1, v2, vn1, vn2;
        if (b1 == b2) {
            v1 = lerp_g(p1, p3, g1, g3); vn1 = lerp_g(n1, n3, g1, g3);
            v2 = lerp_g(p2, p3, g2, g3); vn2 = lerp_g(n2, n3, g2, g3);
        } else if (b1 == b3) {
            v1 = lerp_g(p1, p2, g1, g2); vn1 = lerp_g(n1, n2, g1, g2);
            v2 = lerp_g(p3, p2, g3, g2); vn2 = lerp_g(n3, n2, g3, g2);
        } else {
            v1 = lerp_g(p2, p1, g2, g1); vn1 = lerp_g(n2, n1, g2, g1);
            v2 = lerp_g(p3, p1, g3, g1); vn2 = lerp_g(n3, n1, g3, g1);
        }
        v1 = vadd(v1, vmuls(vn1, offset));
        v2 = vadd(v2, vmuls(vn2, offset));
        if ((uint64_t)nl < cap) {
            double* o = out + 6 * nl;
            o[0] = v1.x; o[1] = v1.y; o[2] = v1.z;
            o[3] = v2.x; o[4] = v2.y; o[5] = v2.z;
        }
        nl++;
    }
    free(nrm);
    return nl;
}
