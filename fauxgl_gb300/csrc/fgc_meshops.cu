// fgc_meshops.cu -- mesh preparation on the device: STL decoding with face
// normals, SmoothNormalsThreshold / SmoothNormals, SharpEdges, the silhouette
// line mesh, and reading a mesh back.
//
// Reference: LoadSTL (stl.go:23-57), loadSTLA (stl.go:59-80), makeFloat
// (stl.go:82-84), loadSTLB (stl.go:86-154), Triangle.Normal
// (triangle.go:33-37), smoothNormalsThreshold / SmoothNormalsThreshold /
// SmoothNormals (mesh.go:80-120), SharpEdges (mesh.go:258-292), silhouette
// (silhouette.go:3-53) behind Mesh.Silhouette (mesh.go:207-209).
//
// Position groups. The reference keys its maps by Vector with Go's ==, so -0
// and +0 are one key and a position holding NaN is never found (each insert
// makes a new entry, each lookup finds nothing). On the device, triangle
// corners are grouped by the bit pattern of position + 0.0 through the weld's
// hash table; NaN positions get no group. A group lists its corners in corner
// order -- the order of the reference's appends -- so every sum below adds in
// the reference's order and gives its bits. Vector arithmetic follows
// vector.go left to right (the library is built without contraction).
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "fgc_host.cuh"
#include "fgc_internal.cuh"

using namespace fgc;

namespace {

struct V3d {
    double x, y, z;
};
__device__ __forceinline__ V3d mv(double x, double y, double z) { return V3d{x, y, z}; }
__device__ __forceinline__ V3d vsub(V3d a, V3d b) { return mv(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ V3d vadd(V3d a, V3d b) { return mv(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ V3d vmuls(V3d a, double s) { return mv(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ double vdot(V3d a, V3d b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ V3d vcross(V3d a, V3d b) {  // vector.go:76-81
    return mv(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
__device__ __forceinline__ V3d vnormalize(V3d a) {  // vector.go:83-86
    const double r = 1.0 / sqrt(a.x * a.x + a.y * a.y + a.z * a.z);
    return mv(a.x * r, a.y * r, a.z * r);
}
__device__ __forceinline__ bool vless(V3d a, V3d b) {  // vector.go:42-50
    if (a.x != b.x) return a.x < b.x;
    if (a.y != b.y) return a.y < b.y;
    return a.z < b.z;
}
__device__ __forceinline__ V3d face_normal(V3d p1, V3d p2, V3d p3) {  // triangle.go:33-37
    return vnormalize(vcross(vsub(p2, p1), vsub(p3, p1)));
}
__device__ __forceinline__ V3d pos_of(const APosNrm64* pn, uint64_t c) {
    const APosNrm64 a = pn[c];
    return mv(a.px, a.py, a.pz);
}
__device__ __forceinline__ V3d nrm_of(const APosNrm64* pn, uint64_t c) {
    const APosNrm64 a = pn[c];
    return mv(a.nx, a.ny, a.nz);
}
__device__ __forceinline__ void put3(double* p, uint64_t i, V3d v) {
    p[3 * i] = v.x;
    p[3 * i + 1] = v.y;
    p[3 * i + 2] = v.z;
}
__device__ __forceinline__ V3d get3(const double* p, uint64_t i) { return mv(p[3 * i], p[3 * i + 1], p[3 * i + 2]); }

#define GRID_LOOP(i, n) \
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < (n); i += (uint64_t)gridDim.x * blockDim.x)

constexpr uint32_t kNoGroup = 0xFFFFFFFFu;

// ---------------------------------------------------------------------------
// STL
// ---------------------------------------------------------------------------
__device__ __forceinline__ double le_float(const uint8_t* b) {  // makeFloat
    const uint32_t u = (uint32_t)b[0] | ((uint32_t)b[1] << 8) | ((uint32_t)b[2] << 16) | ((uint32_t)b[3] << 24);
    return (double)__uint_as_float(u);
}

// Binary records (50 bytes: normal, three vertices as little-endian float32,
// attribute count): positions widened to FP64, every corner's normal the
// triangle's Normal() (loadSTLB ignores the stored normal).
__global__ void stl_decode_kernel(const uint8_t* rec, uint64_t T, double* cp, double* nrm) {
    GRID_LOOP(t, T) {
        const uint8_t* r = rec + 50 * t;
        V3d p[3];
        for (int k = 0; k < 3; k++)
            p[k] = mv(le_float(r + 12 + 12 * k), le_float(r + 16 + 12 * k), le_float(r + 20 + 12 * k));
        const V3d n = face_normal(p[0], p[1], p[2]);
        for (int k = 0; k < 3; k++) {
            put3(cp, 3 * t + k, p[k]);
            put3(nrm, 3 * t + k, n);
        }
    }
}

// ASCII triangles: zero normals become the face normal (FixNormals,
// triangle.go:46-58, called by loadSTLA).
__global__ void face_normals_kernel(const double* cp, uint64_t T, double* nrm) {
    GRID_LOOP(t, T) {
        const V3d n = face_normal(get3(cp, 3 * t), get3(cp, 3 * t + 1), get3(cp, 3 * t + 2));
        for (int k = 0; k < 3; k++) put3(nrm, 3 * t + k, n);
    }
}

// ---------------------------------------------------------------------------
// Position groups
// ---------------------------------------------------------------------------
__global__ void group_keys_kernel(const APosNrm64* pn, uint64_t V, double* key, uint8_t* nanf) {
    GRID_LOOP(c, V) {
        const V3d p = pos_of(pn, c);
        put3(key, c, mv(p.x + 0.0, p.y + 0.0, p.z + 0.0));  // -0 -> +0
        nanf[c] = (p.x != p.x || p.y != p.y || p.z != p.z) ? 1 : 0;
    }
}

__global__ void group_ids_kernel(const uint32_t* slot_of, const uint32_t* minc, const uint32_t* uid,
                                 const uint8_t* nanf, uint64_t V, uint32_t* gid, uint32_t* count) {
    GRID_LOOP(c, V) {
        const uint32_t g = nanf[c] ? kNoGroup : uid[minc[slot_of[c]]];
        gid[c] = g;
        if (g != kNoGroup) atomicAdd(&count[g], 1u);
    }
}

__global__ void group_fill_kernel(const uint32_t* gid, const uint32_t* start, uint32_t* cursor, uint64_t V,
                                  uint32_t* member) {
    GRID_LOOP(c, V) {
        const uint32_t g = gid[c];
        if (g != kNoGroup) member[start[g] + atomicAdd(&cursor[g], 1u)] = (uint32_t)c;
    }
}

// Each group's corners into corner order (groups are small: the corners
// meeting at one position).
__global__ void group_sort_kernel(const uint32_t* start, const uint32_t* count, uint64_t G, uint32_t* member) {
    GRID_LOOP(g, G) {
        const uint32_t n = count[g];
        if (n < 2) continue;
        uint32_t* m = member + start[g];
        for (uint32_t i = 1; i < n; i++) {
            const uint32_t v = m[i];
            uint32_t j = i;
            while (j > 0 && m[j - 1] > v) {
                m[j] = m[j - 1];
                j--;
            }
            m[j] = v;
        }
    }
}

// ---------------------------------------------------------------------------
// Normal smoothing
// ---------------------------------------------------------------------------
// smoothNormalsThreshold (mesh.go:80-88) for every corner: the normalised sum,
// in corner order, of the group's normals whose dot product with the
// corner's own is at least the threshold. A NaN position finds no group: the
// sum is the zero vector and normalises to NaN.
__global__ void smooth_threshold_kernel(const APosNrm64* pn, const uint32_t* gid, const uint32_t* start,
                                        const uint32_t* count, const uint32_t* member, uint64_t V, double threshold,
                                        double* out) {
    GRID_LOOP(c, V) {
        const V3d normal = nrm_of(pn, c);
        V3d result = mv(0, 0, 0);
        const uint32_t g = gid[c];
        if (g != kNoGroup) {
            const uint32_t* m = member + start[g];
            for (uint32_t k = 0; k < count[g]; k++) {
                const V3d x = nrm_of(pn, m[k]);
                if (vdot(x, normal) >= threshold) result = vadd(result, x);
            }
        }
        put3(out, c, vnormalize(result));
    }
}

// SmoothNormals (mesh.go:105-120): per group the normalised sum of all its
// normals in corner order.
__global__ void smooth_sum_kernel(const APosNrm64* pn, const uint32_t* start, const uint32_t* count,
                                  const uint32_t* member, uint64_t G, double* gsum) {
    GRID_LOOP(g, G) {
        const uint32_t n = count[g];
        if (n == 0) continue;
        V3d s = mv(0, 0, 0);
        const uint32_t* m = member + start[g];
        for (uint32_t k = 0; k < n; k++) s = vadd(s, nrm_of(pn, m[k]));
        put3(gsum, g, vnormalize(s));
    }
}

// A NaN position's lookup finds nothing: the zero Vector.
__global__ void smooth_assign_kernel(const uint32_t* gid, const double* gsum, uint64_t V, double* out) {
    GRID_LOOP(c, V) {
        const uint32_t g = gid[c];
        put3(out, c, g == kNoGroup ? mv(0, 0, 0) : get3(gsum, g));
    }
}

__global__ void set_normals_kernel(const double* nrm, uint64_t V, APosNrm64* pn64, APosNrm32* pn32) {
    GRID_LOOP(c, V) {
        const V3d n = get3(nrm, c);
        pn64[c].nx = n.x;
        pn64[c].ny = n.y;
        pn64[c].nz = n.z;
        pn32[c].nx = (float)n.x;
        pn32[c].ny = (float)n.y;
        pn32[c].nz = (float)n.z;
    }
}

// ---------------------------------------------------------------------------
// SharpEdges
// ---------------------------------------------------------------------------
// Edge k of triangle t runs from corner k to corner (k+1)%3 (e1, e2, e3 of
// mesh.go:271-273). other[e] when t is reached is the last earlier triangle
// holding an equal edge: found among the corners of the edge's first
// position, latest first.
__device__ __forceinline__ bool has_edge(const uint32_t* gid, uint64_t t, uint32_t ga, uint32_t gb) {
    const uint32_t g0 = gid[3 * t], g1 = gid[3 * t + 1], g2 = gid[3 * t + 2];
    return (g0 == ga && g1 == gb) || (g0 == gb && g1 == ga) || (g1 == ga && g2 == gb) || (g1 == gb && g2 == ga) ||
           (g2 == ga && g0 == gb) || (g2 == gb && g0 == ga);
}

__global__ void sharp_flag_kernel(const APosNrm64* pn, const uint32_t* gid, const uint32_t* start,
                                  const uint32_t* count, const uint32_t* member, uint64_t T, double angle,
                                  uint32_t* flag) {
    GRID_LOOP(o, 3 * T) {
        const uint64_t t = o / 3;
        const uint32_t k = (uint32_t)(o % 3);
        const uint32_t ga = gid[3 * t + k], gb = gid[3 * t + (k + 1) % 3];
        uint32_t f = 0;
        if (ga != kNoGroup && gb != kNoGroup) {
            const uint32_t* m = member + start[ga];
            int64_t u = -1;
            for (uint32_t j = count[ga]; j-- > 0;) {
                const uint64_t tu = m[j] / 3;
                if (tu >= t) continue;
                if (has_edge(gid, tu, ga, gb)) {
                    u = (int64_t)tu;
                    break;
                }
            }
            if (u >= 0) {
                const V3d nt = face_normal(pos_of(pn, 3 * t), pos_of(pn, 3 * t + 1), pos_of(pn, 3 * t + 2));
                const V3d nu = face_normal(pos_of(pn, 3 * u), pos_of(pn, 3 * u + 1), pos_of(pn, 3 * u + 2));
                if (acos(vdot(nt, nu)) > angle) f = 1;
            }
        }
        flag[o] = f;
    }
}

// NewLineForPoints(e.A, e.B) with e = makeEdge of the current triangle's
// positions (ordered by Less).
__global__ void sharp_emit_kernel(const APosNrm64* pn, const uint32_t* flag, const uint32_t* pos, uint64_t T,
                                  double* lines) {
    GRID_LOOP(o, 3 * T) {
        if (!flag[o]) continue;
        const uint64_t t = o / 3;
        const uint32_t k = (uint32_t)(o % 3);
        V3d a = pos_of(pn, 3 * t + k), b = pos_of(pn, 3 * t + (k + 1) % 3);
        if (!vless(a, b)) {
            const V3d x = a;
            a = b;
            b = x;
        }
        put3(lines, 2 * (uint64_t)pos[o], a);
        put3(lines, 2 * (uint64_t)pos[o] + 1, b);
    }
}

// ---------------------------------------------------------------------------
// silhouette
// ---------------------------------------------------------------------------
__device__ __forceinline__ V3d lerp_g(V3d p1, V3d p2, double w1, double w2) {  // silhouette.go:6-9
    const double t = -w1 / (w2 - w1);
    return vadd(p1, vmuls(vsub(p2, p1), t));  // Lerp, vector.go:64-66
}

__global__ void silhouette_kernel(const APosNrm64* pn, const double* nrm, uint64_t T, double ex, double ey,
                                  double ez, double offset, uint32_t* flag, double* seg) {
    GRID_LOOP(t, T) {
        const V3d eye = mv(ex, ey, ez);
        const V3d p1 = pos_of(pn, 3 * t), p2 = pos_of(pn, 3 * t + 1), p3 = pos_of(pn, 3 * t + 2);
        const V3d n1 = get3(nrm, 3 * t), n2 = get3(nrm, 3 * t + 1), n3 = get3(nrm, 3 * t + 2);
        const double g1 = vdot(n1, vsub(p1, eye));
        const double g2 = vdot(n2, vsub(p2, eye));
        const double g3 = vdot(n3, vsub(p3, eye));
        const bool b1 = g1 > 0, b2 = g2 > 0, b3 = g3 > 0;
        if (b1 == b2 && b2 == b3) {
            flag[t] = 0;
            continue;
        }
        V3d v1, v2, vn1, vn2;
        if (b1 == b2) {
            v1 = lerp_g(p1, p3, g1, g3);
            vn1 = lerp_g(n1, n3, g1, g3);
            v2 = lerp_g(p2, p3, g2, g3);
            vn2 = lerp_g(n2, n3, g2, g3);
        } else if (b1 == b3) {
            v1 = lerp_g(p1, p2, g1, g2);
            vn1 = lerp_g(n1, n2, g1, g2);
            v2 = lerp_g(p3, p2, g3, g2);
            vn2 = lerp_g(n3, n2, g3, g2);
        } else {
            v1 = lerp_g(p2, p1, g2, g1);
            vn1 = lerp_g(n2, n1, g2, g1);
            v2 = lerp_g(p3, p1, g3, g1);
            vn2 = lerp_g(n3, n1, g3, g1);
        }
        put3(seg, 2 * t, vadd(v1, vmuls(vn1, offset)));
        put3(seg, 2 * t + 1, vadd(v2, vmuls(vn2, offset)));
        flag[t] = 1;
    }
}

__global__ void compact_lines_kernel(const uint32_t* flag, const uint32_t* pos, const double* seg, uint64_t n,
                                     double* lines) {
    GRID_LOOP(i, n) {
        if (!flag[i]) continue;
        put3(lines, 2 * (uint64_t)pos[i], get3(seg, 2 * i));
        put3(lines, 2 * (uint64_t)pos[i] + 1, get3(seg, 2 * i + 1));
    }
}

__global__ void download_kernel(const APosNrm64* pn, uint64_t V, double* pos, double* nrm) {
    GRID_LOOP(c, V) {
        const APosNrm64 a = pn[c];
        pos[3 * c] = a.px;
        pos[3 * c + 1] = a.py;
        pos[3 * c + 2] = a.pz;
        nrm[3 * c] = a.nx;
        nrm[3 * c + 1] = a.ny;
        nrm[3 * c + 2] = a.nz;
    }
}

#undef GRID_LOOP

// ---------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------
struct Work {
    int dev = 0, sms = 1;
    cudaStream_t s = nullptr;
    int rc = FGC_OK;
    Work(int device) : dev(device) {
        cudaSetDevice(dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaError_t e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
        if (e != cudaSuccess) rc = fail(FGC_ERR_CUDA, std::string("cudaStreamCreate: ") + cudaGetErrorString(e));
    }
    ~Work() {
        if (s) {
            cudaStreamSynchronize(s);
            cudaStreamDestroy(s);
        }
    }
    bool ok(cudaError_t e, const char* what) {
        if (e != cudaSuccess && rc == FGC_OK) rc = fail(FGC_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
        return rc == FGC_OK;
    }
    int grid(uint64_t n) const { return grid_for(n, 256, sms * 16); }
};

// Exclusive scan of n u32 on the device; *total receives the sum.
bool scan_u32(Work& W, const uint32_t* in, uint32_t* out, uint64_t n, uint64_t* total) {
    DevBuf<unsigned long long> tiles;
    DevBuf<unsigned int> words;  // ticket, status
    const uint64_t nt = (n + 2047) / 2048;
    if (!W.ok(tiles.ensure(nt + 2), "alloc scan") || !W.ok(words.ensure(2), "alloc scan")) return false;
    if (!W.ok(cudaMemsetAsync(tiles.p, 0, (nt + 2) * 8, W.s), "zero scan") ||
        !W.ok(cudaMemsetAsync(words.p, 0, 8, W.s), "zero scan"))
        return false;
    if (n == 0) {
        *total = 0;
        return true;
    }
    ScanParams sp;
    sp.n_dev = nullptr;
    sp.in = in;
    sp.out = out;
    sp.n = n;
    sp.lb = Lookback{tiles.p + 1, words.p, words.p + 1, tiles.p};
    scan_u32_kernel<<<(unsigned)nt, 256, 0, W.s>>>(sp);
    unsigned long long h[2] = {0, 0};
    if (!W.ok(cudaGetLastError(), "scan") ||
        !W.ok(cudaMemcpyAsync(&h[0], tiles.p, 8, cudaMemcpyDeviceToHost, W.s), "read scan total") ||
        !W.ok(cudaMemcpyAsync(&h[1], words.p + 1, 4, cudaMemcpyDeviceToHost, W.s), "read scan status") ||
        !W.ok(cudaStreamSynchronize(W.s), "scan"))
        return false;
    if ((unsigned int)h[1] != 0) {
        W.rc = fail(FGC_ERR_DEVICE_LIMIT, "a look-back wait in a scan timed out");
        return false;
    }
    *total = h[0];
    return true;
}

// Groups of the first V corners of a mesh by position (Go map keys).
struct Groups {
    DevBuf<uint32_t> gid, start, count, member;
    uint64_t G = 0;  // group slots (some may be empty)
};

bool build_groups(Work& W, const fgc_mesh* m, uint64_t V, Groups& Gr) {
    DevBuf<double> key;
    DevBuf<uint8_t> nanf;
    DevBuf<uint32_t> table, slot_of, minc, flag, uid, cursor;
    DevBuf<unsigned int> st;
    uint64_t tsize = 1;
    while (tsize < 2 * V) tsize <<= 1;
    if (!W.ok(key.ensure(3 * V), "alloc keys") || !W.ok(nanf.ensure(V), "alloc keys") ||
        !W.ok(table.ensure(tsize), "alloc table") || !W.ok(minc.ensure(tsize), "alloc table") ||
        !W.ok(slot_of.ensure(V), "alloc groups") || !W.ok(flag.ensure(V), "alloc groups") ||
        !W.ok(uid.ensure(V), "alloc groups") || !W.ok(cursor.ensure(V), "alloc groups") ||
        !W.ok(Gr.gid.ensure(V), "alloc groups") || !W.ok(Gr.start.ensure(V), "alloc groups") ||
        !W.ok(Gr.count.ensure(V), "alloc groups") || !W.ok(Gr.member.ensure(V), "alloc groups") ||
        !W.ok(st.ensure(1), "alloc status"))
        return false;
    const int grid = W.grid(V);
    if (!W.ok(cudaMemsetAsync(table.p, 0xFF, tsize * 4, W.s), "init table") ||
        !W.ok(cudaMemsetAsync(minc.p, 0xFF, tsize * 4, W.s), "init table") ||
        !W.ok(cudaMemsetAsync(st.p, 0, 4, W.s), "zero status") ||
        !W.ok(cudaMemsetAsync(Gr.count.p, 0, V * 4, W.s), "zero counts") ||
        !W.ok(cudaMemsetAsync(cursor.p, 0, V * 4, W.s), "zero cursors"))
        return false;
    group_keys_kernel<<<grid, 256, 0, W.s>>>(m->pn64.p, V, key.p, nanf.p);
    weld_insert_kernel<<<grid, 256, 0, W.s>>>(key.p, V, table.p, tsize - 1, slot_of.p, minc.p, st.p);
    weld_flag_kernel<<<grid, 256, 0, W.s>>>(slot_of.p, minc.p, V, flag.p);
    if (!W.ok(cudaGetLastError(), "group kernels")) return false;
    uint64_t nrep = 0;
    if (!scan_u32(W, flag.p, uid.p, V, &nrep)) return false;
    unsigned int hst = 0;
    if (!W.ok(cudaMemcpyAsync(&hst, st.p, 4, cudaMemcpyDeviceToHost, W.s), "read status") ||
        !W.ok(cudaStreamSynchronize(W.s), "groups"))
        return false;
    if (hst != 0) {
        W.rc = fail(FGC_ERR_DEVICE_LIMIT, "position grouping failed");
        return false;
    }
    Gr.G = nrep;
    group_ids_kernel<<<grid, 256, 0, W.s>>>(slot_of.p, minc.p, uid.p, nanf.p, V, Gr.gid.p, Gr.count.p);
    uint64_t total = 0;
    if (!W.ok(cudaGetLastError(), "group kernels") || !scan_u32(W, Gr.count.p, Gr.start.p, Gr.G, &total)) return false;
    group_fill_kernel<<<grid, 256, 0, W.s>>>(Gr.gid.p, Gr.start.p, cursor.p, V, Gr.member.p);
    group_sort_kernel<<<W.grid(Gr.G), 256, 0, W.s>>>(Gr.start.p, Gr.count.p, Gr.G, Gr.member.p);
    return W.ok(cudaGetLastError(), "group kernels");
}

// SmoothNormals of the mesh's triangle corners into out (3 doubles each).
bool smooth_normals_into(Work& W, const fgc_mesh* m, double* out) {
    const uint64_t V = 3 * m->ntri;
    Groups Gr;
    if (!build_groups(W, m, V, Gr)) return false;
    DevBuf<double> gsum;
    if (!W.ok(gsum.ensure(3 * std::max<uint64_t>(Gr.G, 1)), "alloc sums")) return false;
    smooth_sum_kernel<<<W.grid(Gr.G), 256, 0, W.s>>>(m->pn64.p, Gr.start.p, Gr.count.p, Gr.member.p, Gr.G, gsum.p);
    smooth_assign_kernel<<<W.grid(V), 256, 0, W.s>>>(Gr.gid.p, gsum.p, V, out);
    return W.ok(cudaGetLastError(), "smoothing kernels");
}

// A line mesh built from n lines (2 corners each) at device address lines.
int line_mesh(Work& W, const double* lines, uint64_t n, fgc_mesh** out) {
    fgc_mesh* m = new (std::nothrow) fgc_mesh();
    if (!m) return fail(FGC_ERR_OUT_OF_MEMORY, "host allocation failed");
    m->device = W.dev;
    m->ntri = 0;
    m->nline = n;
    int rc = n ? mesh_weld_attrs(m, W.s, W.sms, lines, nullptr, 2 * n) : FGC_OK;
    if (rc != FGC_OK) {
        delete m;
        return rc;
    }
    *out = m;
    return FGC_OK;
}

// loadSTLA's parse: every line whose whitespace-separated fields are exactly
// "vertex x y z" adds a vertex (strconv.ParseFloat with its error ignored: a
// field that is not a number as a whole reads as 0).
bool is_space(char ch) { return ch == ' ' || ch == '\t' || ch == '\r' || ch == '\v' || ch == '\f'; }

double parse_number(const char* s, size_t n) {
    if (n == 0 || n > 255) return 0;
    char buf[256];
    std::memcpy(buf, s, n);
    buf[n] = 0;
    char* end = nullptr;
    const double v = std::strtod(buf, &end);
    return end == buf + n ? v : 0;
}

void parse_ascii_stl(const char* d, uint64_t n, std::vector<double>& pos) {
    uint64_t i = 0;
    while (i < n) {
        uint64_t e = i;
        while (e < n && d[e] != '\n') e++;
        const char* f[4] = {nullptr, nullptr, nullptr, nullptr};
        size_t fl[4] = {0, 0, 0, 0};
        int nf = 0;
        uint64_t j = i;
        while (j < e) {
            while (j < e && is_space(d[j])) j++;
            if (j >= e) break;
            const uint64_t s0 = j;
            while (j < e && !is_space(d[j])) j++;
            if (nf < 4) {
                f[nf] = d + s0;
                fl[nf] = (size_t)(j - s0);
            }
            nf++;
        }
        if (nf == 4 && fl[0] == 6 && std::memcmp(f[0], "vertex", 6) == 0) {
            pos.push_back(parse_number(f[1], fl[1]));
            pos.push_back(parse_number(f[2], fl[2]));
            pos.push_back(parse_number(f[3], fl[3]));
        }
        i = e + 1;
    }
}

int check_mesh(const fgc_mesh* m) {
    if (!m) return fail(FGC_ERR_INVALID_ARGUMENT, "null mesh");
    return FGC_OK;
}

}  // namespace

extern "C" {

int fgc_mesh_load_stl(const void* data, uint64_t nbytes, fgc_mesh** out) {
    if (!out || (!data && nbytes)) return fail(FGC_ERR_INVALID_ARGUMENT, "null argument");
    *out = nullptr;
    if (nbytes < 84) return fail(FGC_ERR_INVALID_ARGUMENT, "STL data shorter than its 84-byte header");
    const uint8_t* b = static_cast<const uint8_t*>(data);
    const uint64_t count = (uint64_t)b[80] | ((uint64_t)b[81] << 8) | ((uint64_t)b[82] << 16) | ((uint64_t)b[83] << 24);
    int dev = 0;
    cudaGetDevice(&dev);
    Work W(dev);
    if (W.rc) return W.rc;
    DevBuf<double> cp, nrm;
    DevBuf<uint8_t> rec;
    uint64_t T = 0;
    if (count * 50 + 84 == nbytes) {  // binary (LoadSTL's size test)
        T = count;
        if (3 * T >= 0x7FFFFFFFull) return fail(FGC_ERR_UNSUPPORTED, "mesh has too many corners (2^31 limit)");
        if (T) {
            if (!W.ok(rec.ensure(50 * T), "alloc records") || !W.ok(cp.ensure(9 * T), "alloc positions") ||
                !W.ok(nrm.ensure(9 * T), "alloc normals") ||
                !W.ok(cudaMemcpyAsync(rec.p, b + 84, 50 * T, cudaMemcpyHostToDevice, W.s), "copy records"))
                return W.rc;
            stl_decode_kernel<<<W.grid(T), 256, 0, W.s>>>(rec.p, T, cp.p, nrm.p);
            if (!W.ok(cudaGetLastError(), "decode kernel")) return W.rc;
        }
    } else {
        std::vector<double> pos;
        parse_ascii_stl(reinterpret_cast<const char*>(b), nbytes, pos);
        const uint64_t nv = pos.size() / 3;
        if (nv % 3) return fail(FGC_ERR_INVALID_ARGUMENT, "ASCII STL vertex count is not a multiple of three");
        T = nv / 3;
        if (3 * T >= 0x7FFFFFFFull) return fail(FGC_ERR_UNSUPPORTED, "mesh has too many corners (2^31 limit)");
        if (T) {
            if (!W.ok(cp.ensure(9 * T), "alloc positions") || !W.ok(nrm.ensure(9 * T), "alloc normals") ||
                !W.ok(cudaMemcpyAsync(cp.p, pos.data(), 9 * T * 8, cudaMemcpyHostToDevice, W.s), "copy positions"))
                return W.rc;
            face_normals_kernel<<<W.grid(T), 256, 0, W.s>>>(cp.p, T, nrm.p);
            if (!W.ok(cudaGetLastError(), "normal kernel") || !W.ok(cudaStreamSynchronize(W.s), "copy positions"))
                return W.rc;
        }
    }
    fgc_mesh* m = new (std::nothrow) fgc_mesh();
    if (!m) return fail(FGC_ERR_OUT_OF_MEMORY, "host allocation failed");
    m->device = dev;
    m->ntri = T;
    m->nline = 0;
    const int rc = T ? mesh_weld_attrs(m, W.s, W.sms, cp.p, nrm.p, 3 * T) : FGC_OK;
    if (rc != FGC_OK) {
        delete m;
        return rc;
    }
    *out = m;
    return FGC_OK;
}

int fgc_mesh_smooth_normals_threshold(fgc_mesh* m, double radians) {
    if (int rc = check_mesh(m)) return rc;
    const uint64_t V = 3 * m->ntri;
    if (V == 0) return FGC_OK;
    Work W(m->device);
    if (W.rc) return W.rc;
    const double threshold = std::cos(radians);
    Groups Gr;
    DevBuf<double> out;
    if (!build_groups(W, m, V, Gr) || !W.ok(out.ensure(3 * V), "alloc normals")) return W.rc;
    smooth_threshold_kernel<<<W.grid(V), 256, 0, W.s>>>(m->pn64.p, Gr.gid.p, Gr.start.p, Gr.count.p, Gr.member.p, V,
                                                         threshold, out.p);
    set_normals_kernel<<<W.grid(V), 256, 0, W.s>>>(out.p, V, m->pn64.p, m->pn32.p);
    W.ok(cudaGetLastError(), "smoothing kernels");
    W.ok(cudaStreamSynchronize(W.s), "smoothing");
    return W.rc;
}

int fgc_mesh_smooth_normals(fgc_mesh* m) {
    if (int rc = check_mesh(m)) return rc;
    const uint64_t V = 3 * m->ntri;
    if (V == 0) return FGC_OK;
    Work W(m->device);
    if (W.rc) return W.rc;
    DevBuf<double> out;
    if (!W.ok(out.ensure(3 * V), "alloc normals") || !smooth_normals_into(W, m, out.p)) return W.rc;
    set_normals_kernel<<<W.grid(V), 256, 0, W.s>>>(out.p, V, m->pn64.p, m->pn32.p);
    W.ok(cudaGetLastError(), "smoothing kernels");
    W.ok(cudaStreamSynchronize(W.s), "smoothing");
    return W.rc;
}

int fgc_mesh_sharp_edges(const fgc_mesh* m, double angle_threshold, fgc_mesh** out) {
    if (!out) return fail(FGC_ERR_INVALID_ARGUMENT, "out is null");
    *out = nullptr;
    if (int rc = check_mesh(m)) return rc;
    Work W(m->device);
    if (W.rc) return W.rc;
    const uint64_t T = m->ntri, E = 3 * T;
    if (T == 0) return line_mesh(W, nullptr, 0, out);
    Groups Gr;
    DevBuf<uint32_t> flag, pos;
    DevBuf<double> lines;
    if (!build_groups(W, m, 3 * T, Gr) || !W.ok(flag.ensure(E), "alloc flags") || !W.ok(pos.ensure(E), "alloc flags"))
        return W.rc;
    sharp_flag_kernel<<<W.grid(E), 256, 0, W.s>>>(m->pn64.p, Gr.gid.p, Gr.start.p, Gr.count.p, Gr.member.p, T,
                                                   angle_threshold, flag.p);
    uint64_t n = 0;
    if (!W.ok(cudaGetLastError(), "edge kernel") || !scan_u32(W, flag.p, pos.p, E, &n)) return W.rc;
    if (!W.ok(lines.ensure(6 * std::max<uint64_t>(n, 1)), "alloc lines")) return W.rc;
    sharp_emit_kernel<<<W.grid(E), 256, 0, W.s>>>(m->pn64.p, flag.p, pos.p, T, lines.p);
    if (!W.ok(cudaGetLastError(), "edge kernel")) return W.rc;
    return line_mesh(W, lines.p, n, out);
}

int fgc_mesh_silhouette(const fgc_mesh* m, const double eye[3], double offset, fgc_mesh** out) {
    if (!out || !eye) return fail(FGC_ERR_INVALID_ARGUMENT, "null argument");
    *out = nullptr;
    if (int rc = check_mesh(m)) return rc;
    Work W(m->device);
    if (W.rc) return W.rc;
    const uint64_t T = m->ntri;
    if (T == 0) return line_mesh(W, nullptr, 0, out);
    DevBuf<double> nrm, seg, lines;
    DevBuf<uint32_t> flag, pos;
    if (!W.ok(nrm.ensure(9 * T), "alloc normals") || !W.ok(seg.ensure(6 * T), "alloc lines") ||
        !W.ok(flag.ensure(T), "alloc flags") || !W.ok(pos.ensure(T), "alloc flags"))
        return W.rc;
    if (!smooth_normals_into(W, m, nrm.p)) return W.rc;  // mesh.Copy(); SmoothNormals()
    silhouette_kernel<<<W.grid(T), 256, 0, W.s>>>(m->pn64.p, nrm.p, T, eye[0], eye[1], eye[2], offset, flag.p, seg.p);
    uint64_t n = 0;
    if (!W.ok(cudaGetLastError(), "silhouette kernel") || !scan_u32(W, flag.p, pos.p, T, &n)) return W.rc;
    if (!W.ok(lines.ensure(6 * std::max<uint64_t>(n, 1)), "alloc lines")) return W.rc;
    compact_lines_kernel<<<W.grid(T), 256, 0, W.s>>>(flag.p, pos.p, seg.p, T, lines.p);
    if (!W.ok(cudaGetLastError(), "silhouette kernel")) return W.rc;
    return line_mesh(W, lines.p, n, out);
}

int fgc_mesh_download(const fgc_mesh* m, double* tri_pos, double* tri_nrm, double* line_pos, double* line_nrm) {
    if (int rc = check_mesh(m)) return rc;
    const uint64_t V = 3 * m->ntri + 2 * m->nline;
    if (V == 0) return FGC_OK;
    Work W(m->device);
    if (W.rc) return W.rc;
    DevBuf<double> pos, nrm;
    std::vector<double> hp(3 * V), hn(3 * V);
    if (!W.ok(pos.ensure(3 * V), "alloc") || !W.ok(nrm.ensure(3 * V), "alloc")) return W.rc;
    download_kernel<<<W.grid(V), 256, 0, W.s>>>(m->pn64.p, V, pos.p, nrm.p);
    if (!W.ok(cudaGetLastError(), "download kernel") ||
        !W.ok(cudaMemcpyAsync(hp.data(), pos.p, 3 * V * 8, cudaMemcpyDeviceToHost, W.s), "read positions") ||
        !W.ok(cudaMemcpyAsync(hn.data(), nrm.p, 3 * V * 8, cudaMemcpyDeviceToHost, W.s), "read normals") ||
        !W.ok(cudaStreamSynchronize(W.s), "download"))
        return W.rc;
    const uint64_t nt = 9 * m->ntri, nl = 6 * m->nline;
    if (tri_pos) std::memcpy(tri_pos, hp.data(), nt * 8);
    if (tri_nrm) std::memcpy(tri_nrm, hn.data(), nt * 8);
    if (line_pos) std::memcpy(line_pos, hp.data() + nt, nl * 8);
    if (line_nrm) std::memcpy(line_nrm, hn.data() + nt, nl * 8);
    return FGC_OK;
}

}  // extern "C"
