// fgc_internal.cuh -- kernel parameter blocks and kernel declarations of
// libfauxglcuda (shared by the kernel translation units and the host runtime).
#pragma once

#include "fgc_device.cuh"
#include "fgc_scan.cuh"

namespace fgc {

struct VertexParams {
    const double* ux;
    const double* uy;
    const double* uz;
    uint64_t n;
    double m[16];
    double w2, h2;
    VClip* vclip;
    double2* vndc;
    VScreen* vscr;
    uint8_t* vout;
};

struct GeomParams {
    MeshView mesh;
    StateView st;
    double w2, h2;
    uint64_t tri_first, tri_count, line_first, line_count;
    const VClip* vclip;
    const double2* vndc;
    const VScreen* vscr;
    const uint8_t* vout;
    RPrim* prims;
    PBox* pbox;
    uint32_t* pspan;            // per primitive: bound on covered pixels in one row
    uint64_t prim_cap;          // slots available in prims / pbox
    ulonglong2* clip_list;      // (triangle, first slot)
    uint32_t clip_cap;
    uint32_t* clip_count;
    ulonglong2* lclip_list;     // (line, first slot), line_count entries
    uint32_t* lclip_count;
    PoolVertex* pool;           // 21 per clip_list entry
    uint32_t attr_mask;         // kAttr* bits the shader reads
    unsigned long long* tri_slots;
    unsigned long long* line_slots;
    unsigned long long* prim_total;
    Lookback lb_tri, lb_line;
    unsigned int* status;
};

struct BinParams {
    const PBox* pbox;
    const unsigned long long* nprim;
    int32_t W;
    int64_t N;
    int64_t L;                  // pixels per band (R rows * W)
    uint32_t nbands;
    uint32_t nblk;              // blocks of the count/scatter grids
    uint32_t* mat;              // [nbands][nblk] counts
    uint32_t* off;              // [nbands][nblk] exclusive offsets
    const unsigned long long* pair_total;
    uint32_t* bins;
    uint64_t bin_cap;
    unsigned int* status;
};

struct ScanParams {
    const uint32_t* in;
    uint32_t* out;
    uint64_t n;
    Lookback lb;
};

struct RasterParams {
    const RPrim* prims;
    const PBox* pbox;
    const uint32_t* pspan;
    const uint32_t* bins;
    const uint32_t* off;        // bin offsets: band b starts at off[b * nblk]
    const unsigned long long* pair_total;
    uint32_t nblk;
    uint32_t nbands;
    int32_t W, H;
    int64_t N, L;
    int32_t F;                  // fragment buffer capacity
    uint32_t* color;
    double* depth;
    int32_t clear_color_pending, clear_depth_pending;
    uint32_t clear_color;
    double clear_depth;
    StateView st;
    ShaderView sh;
    MeshView mesh;
    const PoolVertex* pool;
    unsigned int* band_counter;
    unsigned int* status;
    unsigned long long* info;   // total, updated, visited pixels, shaded fragments
    uint32_t* winner;           // debug, or null
    double* shaded;             // debug, or null
    double* dbg;                // debug scratch: gridDim * F * 4 doubles
};

// Kernels (grid shapes chosen by the host runtime).
__global__ void vertex_kernel(VertexParams P);
__global__ void setup_triangles_kernel(GeomParams P);
__global__ void setup_lines_kernel(GeomParams P);
__global__ void clip_triangles_kernel(GeomParams P);
__global__ void clip_lines_kernel(GeomParams P);
__global__ void prim_total_kernel(GeomParams P);

__global__ void bin_count_kernel(BinParams P);
__global__ void scan_u32_kernel(ScanParams P);
__global__ void bin_scatter_kernel(BinParams P, int warps);

// Raster kernel entry points (defined with the kernel in fgc_raster.cu).
const void* raster_kernel_ptr(int precision);
cudaError_t launch_raster(int precision, int grid, int threads, size_t smem, cudaStream_t stream,
                          const RasterParams& P);

// Helpers of fgc_misc.cu.
__global__ void fill_u32_kernel(uint32_t* p, uint64_t n, uint32_t v);
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

// Dynamic shared memory of the raster kernel (layout in fgc_raster.cu):
// depth[L] f64, b0/b1/b2/z[F] f64, scratch 64 u64,
// key/colour/unit-slot/unit-row[F] u32, chunk tables 3*threads u32,
// bucket list heads[kRasterHeads] u16, list links[F] u16, flags[F] u8.
// The colour buffer is not staged: the band's pixels are read and written in
// global memory by the CTA that owns them.
__host__ __device__ inline size_t raster_smem_bytes(int64_t L, int F, int threads) {
    size_t b = 0;
    b += (size_t)L * 8;
    b += (size_t)F * 8 * 4;
    b += 64 * 8;
    b += (size_t)F * 4 * 4;
    b += (size_t)threads * 4 * 3;
    b += (size_t)kRasterHeads * 2;
    b += (size_t)F * 2;
    b += (size_t)F;
    return (b + 15) & ~(size_t)15;
}

}  // namespace fgc
