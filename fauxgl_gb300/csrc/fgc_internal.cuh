// fgc_internal.cuh -- kernel parameter blocks and kernel declarations of
// libfauxglcuda (shared by the kernel translation units and the host runtime).
#pragma once

#include "fgc_device.cuh"
#include "fgc_scan.cuh"

namespace fgc {

// One draw of a pass: a mesh range, state, shader and target framebuffer,
// with its place in the pass-wide arrays. A pass renders any number of
// independent draws (views) with one launch per stage; a plain DrawMesh call
// is a pass of one draw. The table lives in device memory; the lookup arrays
// of ItemStarts map a global tile, block or band to its draw.
struct __align__(16) ItemView {
    MeshView mesh;
    StateView st;
    ShaderView sh;
    uint64_t tri_first, tri_count, line_first, line_count;
    double w2, h2;              // W/2, H/2 of the target (Screen matrix)
    int32_t W, H;
    int64_t N;                  // W*H
    int32_t R;                  // rows per band
    int32_t L;                  // pixels per band (R*W)
    uint32_t nbands;            // bands of this draw
    uint32_t band0;             // first pass-wide band
    uint32_t nblk;              // binning blocks of this draw
    uint32_t blk0;              // first pass-wide binning block
    uint64_t mat0;              // first bin-matrix entry ([nbands][nblk])
    uint64_t vbase;             // first vertex-stage record
    uint32_t vtile0;            // first vertex tile
    uint32_t stile0;            // first setup tile: triangle tiles, then line tiles
    uint32_t ntri_tiles, nline_tiles;
    uint32_t attr_mask;         // kAttr* bits the shader reads
    int32_t row_table;          // tall primitives take their row starts from the row-start table
    int32_t clear_color_pending, clear_depth_pending;
    uint32_t clear_color;
    double clear_depth;
    uint32_t* color;            // NRGBA, W*H
    double* depth;              // W*H
    uint32_t* winner;           // debug, or null
    double* shaded;             // debug, or null
};
static_assert(sizeof(ItemView) % 16 == 0, "ItemView is copied in 16-byte words");

// Per-draw results written by the device.
struct ItemOut {
    unsigned long long prim_start, prim_end;  // raster primitive slots [start, end)
    unsigned long long info[4];               // total, updated, visited pixels, shaded fragments
};

// Starts of each draw's tiles / blocks / bands in the pass-wide numbering;
// nitems + 1 entries each (the last is the total).
struct ItemStarts {
    const uint32_t* vtile;
    const uint32_t* stile;
    const uint32_t* blk;
    const uint32_t* band;
};

// Index of the draw whose range [start[i], start[i+1]) holds key.
__device__ __forceinline__ uint32_t find_item(const uint32_t* start, uint32_t nitems, uint32_t key) {
    uint32_t lo = 0, hi = nitems - 1;
    while (lo < hi) {
        const uint32_t mid = (lo + hi + 1) >> 1;
        if (start[mid] <= key) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// floor(x / W) for W > 0 in 32-bit arithmetic; most boxes lie inside the
// frame, where it is 0 without a division.
__device__ __forceinline__ int32_t floordiv_w(int32_t x, int32_t W) {
    if ((uint32_t)x < (uint32_t)W) return 0;
    int32_t q = x / W;
    if (q * W != x && x < 0) q--;
    return q;
}

// A clipped element: its primitive slots and draw.
// One primitive-emitting work item of the setup stage: a triangle (slot of
// its first primitive), one edge of a wireframe triangle, or a line.
struct __align__(16) SetupWork {
    uint64_t slot;
    uint32_t elem;              // triangle or line index in the mesh
    uint32_t item;              // draw of the pass
    uint32_t u0, u1, u2;        // unique-vertex indices (u2 unused for lines)
    uint32_t meta;              // piece | (cull order + 1) << 8 | kWorkLine
};
constexpr uint32_t kWorkLine = 1u << 16;

struct __align__(16) ClipEntry {
    unsigned long long slot;    // first primitive slot
    uint32_t elem;              // triangle (or line) index within the mesh
    uint32_t item;
};

// Clipped triangles pass through three kernels: the polygon of each after
// the six planes (clip space), then each polygon vertex with its
// interpolated attributes and NDC position.
constexpr int kClipPoly = 9;  // polygon vertices the fan reads (7 pieces)
struct __align__(16) ClipPoly {
    D4 v[kClipPoly];
    uint32_t n;                 // vertices of the clipped polygon (the fan reads the first kClipPoly)
};
struct __align__(16) ClipVert {
    double px, py, pz, nx, ny, nz, tu, tv, cr, cg, cb, ca;  // attributes, as a clip pool vertex
    double ox, oy, oz, ow;      // Output (clip space)
    double sx, sy, sz;          // NDC
};

struct VertexParams {
    const ItemView* items;
    ItemStarts starts;
    uint32_t nitems;
    uint32_t ntiles;            // vertex tiles of the pass (kVertexTile positions each)
    VClip* vclip;
    double2* vndc;
    VScreen* vscr;
    uint8_t* vout;
};
constexpr int kVertexTile = 256;

struct GeomParams {
    const ItemView* items;
    ItemStarts starts;
    uint32_t nitems;
    uint32_t ntiles;            // setup tiles of the pass
    ItemOut* iout;
    const VClip* vclip;
    const double2* vndc;
    const VScreen* vscr;
    const uint8_t* vout;
    RPrim* prims;
    PBox* pbox;
    float4* rf;                 // per primitive: 1/W of its vertices in FP32 (mixed-form shading)
    uint32_t* pspan;            // per primitive: bound on covered pixels in one row
    uint64_t prim_cap;          // slots available in prims / pbox
    ClipEntry* clip_list;       // clipped triangles
    uint32_t clip_cap;
    uint32_t* clip_count;
    ClipEntry* lclip_list;      // clipped lines (capacity: all lines of the pass)
    uint32_t* lclip_count;
    PoolVertex* pool;           // 21 per clip_list entry
    PoolVertex32* pool32;       // FP32 copies (draws in the mixed form)
    ClipPoly* cpoly;            // per clip_list entry
    ClipVert* cvert;            // kClipPoly per clip_list entry
    unsigned long long* prim_total;
    Lookback lb;
    unsigned int* status;
    SetupWork* work;            // the primitive-emitting work items, in slot order
    uint64_t work_cap;
    unsigned long long* work_total;
    uint16_t* smeta;            // per element of a setup tile: its setup decision (setup_count -> setup_kernel)
    uint32_t* cidx;             // per element of a setup tile: its clip_list entry, for a clipped triangle
    unsigned long long* tsum;   // per setup tile: slots << 31 | work items, then their exclusive prefix
};
constexpr int kSetupTile = 256;  // threads of a setup tile
constexpr int kSetupPer = 2;     // consecutive elements per thread

struct BinParams {
    const ItemView* items;
    ItemStarts starts;
    uint32_t nitems;
    const ItemOut* iout;
    const PBox* pbox;
    uint32_t* mat;              // per draw [nbands][nblk] counts, draws in order
    uint32_t* off;              // exclusive offsets of mat
    const unsigned long long* pair_total;
    uint32_t* bins;
    uint64_t bin_cap;
    unsigned int* status;
    uint32_t* pnb;              // per primitive: bands it is binned to (bin_count writes it)
};

// The draw's band geometry, as the binning blocks use it.
struct BandGeom {
    int32_t W, H, R;
    uint32_t nbands;
};

// Bands [bl, bh] that the box's linear index range [y0*W + x0, y1*W + x1],
// clipped to [0, W*H), meets. Index y*W + x lies in row y + floor(x/W), and
// band b holds rows [b*R, b*R + R).
__device__ __forceinline__ bool prim_bands(const BandGeom& G, const PBox& b, uint32_t& bl, uint32_t& bh) {
    if (b.x0 > b.x1) return false;
    int64_t rlo = (int64_t)b.y0 + floordiv_w(b.x0, G.W);
    int64_t rhi = (int64_t)b.y1 + floordiv_w(b.x1, G.W);
    if (rhi < 0 || rlo > G.H - 1) return false;
    if (rlo < 0) rlo = 0;
    if (rhi > G.H - 1) rhi = G.H - 1;
    bl = (uint32_t)rlo / (uint32_t)G.R;
    bh = (uint32_t)rhi / (uint32_t)G.R;
    return true;
}

// Row starts: for every (primitive, band) bin pair, the three edge values
// w00, w01, w02 rasterize holds at the primitive's first row in the band,
// built by stepping each primitive's rows serially (the reference's own
// w0k += b per row), so the raster stage starts a row a few steps from its
// band's first row instead of from the primitive's top.
struct RowStartParams {
    const ItemOut* iout;
    const ItemView* items;
    uint32_t nitems;
    const RPrim* prims;
    const PBox* pbox;
    const uint32_t* pnb;
    const uint32_t* prs;        // exclusive scan of pnb
    const unsigned long long* prim_total;
    uint64_t cap;               // row-start slots (the bin capacity)
    double* rstart;             // [slot][3]
    unsigned int* status;
};

struct ScanParams {
    const uint32_t* in;
    uint32_t* out;
    uint64_t n;
    Lookback lb;
    const unsigned long long* n_dev;  // when set, only the first min(n, *n_dev) values are scanned
};

// Primitives with boxes at most this many rows tall catch up their rows from
// the top themselves; taller ones have row starts per band.
constexpr int32_t kRowTableMinRows = 5;
__device__ __forceinline__ bool uses_row_table(const PBox& b) { return b.y1 - b.y0 + 1 >= kRowTableMinRows; }

struct RasterParams {
    const ItemView* items;
    ItemStarts starts;
    uint32_t nitems;
    uint32_t nbands;            // bands of the pass
    ItemOut* iout;
    const RPrim* prims;
    const PBox* pbox;
    const uint32_t* pspan;
    const uint32_t* bins;
    const uint32_t* off;        // bin offsets
    uint64_t nmat;              // entries of off
    const unsigned long long* pair_total;
    int32_t F;                  // fragment buffer capacity
    int32_t Lmax;               // largest band of the pass (depth staging)
    int32_t win;                // fragment offsets a thread walks per round (wide primitives)
    int32_t su;                 // units a chunk of wide primitives holds
    const PoolVertex* pool;
    const PoolVertex32* pool32;
    const float4* rf;
    const uint32_t* prs;        // first row-start slot of each primitive
    const double* rstart;       // row starts per (primitive, band)
    unsigned int* band_counter;
    unsigned int* status;
    double* dbg;                // debug scratch: gridDim * F * 4 doubles, or null
};

// Kernels (grid shapes chosen by the host runtime).
__global__ void vertex_kernel(VertexParams P);
__global__ void setup_count_kernel(GeomParams P);
__global__ void setup_scan_kernel(GeomParams P);
__global__ void setup_kernel(GeomParams P);
__global__ void setup_emit_kernel(GeomParams P);
__global__ void clip_poly_kernel(GeomParams P);
__global__ void clip_vert_kernel(GeomParams P);
__global__ void clip_piece_kernel(GeomParams P);
__global__ void clip_lines_kernel(GeomParams P);

__global__ void bin_count_kernel(BinParams P);
__global__ void scan_u32_kernel(ScanParams P);
__global__ void bin_scatter_kernel(BinParams P, int warps);
__global__ void row_starts_kernel(RowStartParams P);

// Raster kernel entry points (defined with the kernel in fgc_raster.cu).
const void* raster_kernel_ptr(int precision);
cudaError_t launch_raster(int precision, int grid, int threads, size_t smem, cudaStream_t stream,
                          const RasterParams& P);

// Helpers of fgc_misc.cu.
__global__ void fill_u32_kernel(uint32_t* p, uint64_t n, uint32_t v);
__global__ void texel_unit_kernel(const ushort4* src, uint64_t n, double* dst);
__global__ void fill_f64_kernel(double* p, uint64_t n, double v);
__global__ void downsample_kernel(const uint32_t* src, int32_t w, int32_t h, int32_t scale, uint32_t* dst);
__global__ void depth_minmax_kernel(const double* d, uint64_t n, unsigned long long* lohi);
__global__ void depth_image_kernel(const double* d, uint64_t n, const unsigned long long* lohi, uint16_t* out);
__global__ void weld_insert_kernel(const double* cp, uint64_t n, uint32_t* table, uint64_t tmask,
                                   uint32_t* slot_of, uint32_t* minc, unsigned int* status);
__global__ void weld_flag_kernel(const uint32_t* slot_of, const uint32_t* minc, uint64_t n, uint32_t* flag);
__global__ void weld_emit_kernel(const double* cp, const uint32_t* slot_of, const uint32_t* minc,
                                 const uint32_t* uid, uint64_t n, double* ux, double* uy, double* uz,
                                 uint32_t* corner_uniq);
__global__ void attrs_kernel(const double* cp, const double* nrm, uint64_t n, APosNrm64* pn64, APosNrm32* pn32);
__global__ void f64_to_f32_kernel(const double* in, uint64_t n, float* out);
__global__ void fp64_rate_kernel(double* out, double a, double b, int iters);

// Pixel buckets of the raster kernel's per-chunk fragment lists.
constexpr int kRasterHeads = 2048;

// Rows of a band at most.
constexpr int kBandRowsMax = 128;

// (primitive, row) units a chunk of wide primitives holds: kSpanUnitsMax
// (the span arrays then also hold the narrow walk's warp queues) unless
// shared memory cannot hold it, else kSpanUnitsMin. A primitive with more rows in a band than a chunk holds
// (wrap-around rows of a box beyond the frame's sides) is split over chunks.
constexpr int kSpanUnitsMin = 128;
constexpr int kSpanUnitsMax = 256;

// Bin entries a raster thread examines per chunk, and the chunk's primitive
// capacity (a chunk of narrow primitives may hold several units per thread).
constexpr int kChunkPer = 1;
constexpr int kChunkPrims = 256 * kChunkPer;

// Dynamic shared memory of the raster kernel (layout in fgc_raster.cu), for
// a fragment buffer of F and su span units: depth[L] f64, fragment
// b0/b1/b2/z[F] f64, span edge values[su] 3 x f64, scratch 64 u64, fragment
// key/colour[F] u32, unit slot/row[F] u32, span x/count/offset[su] u32, chunk
// primitives[kChunkPrims] u32, bucket list heads[kRasterHeads] u16, list
// links[F] u16, flags[F] u8. The colour buffer is not staged: the band's
// pixels are read and written in global memory by the CTA that owns them.
__host__ __device__ inline size_t raster_smem_bytes(int64_t L, int F, int threads, int su) {
    size_t b = 0;
    b += (size_t)L * 8;
    b += (size_t)F * 8 * 4;
    b += (size_t)su * 8 * 3;
    b += 64 * 8;
    b += (size_t)F * 4 * 4;
    b += (size_t)su * 4 * 3;
    b += (size_t)(threads > kChunkPrims ? threads : kChunkPrims) * 4;
    b += (size_t)kRasterHeads * 2;
    b += (size_t)F * 2;
    b += (size_t)F;
    return (b + 15) & ~(size_t)15;
}

}  // namespace fgc
