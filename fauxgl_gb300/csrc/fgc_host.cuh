// fgc_host.cuh -- host-side objects of libfauxglcuda shared by the C ABI
// (fgc_api.cu) and the pass engine (fgc_pass.cu): device buffers, the
// mesh / texture / context handles, and the pass interface.
//
// A pass renders any number of draws (a mesh range, state, shader and
// target context each) with one launch per pipeline stage. DrawMesh /
// DrawTriangles / DrawLines run a pass of one draw and wait for it, because
// the reference returns RasterizeInfo by value (context.go:391-439); the
// batch interface runs passes of many draws asynchronously.
#pragma once

#include <atomic>

#include <cuda_runtime.h>

#include <algorithm>
#include <cstddef>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "fgc_internal.cuh"

namespace fgc {

// Record msg as the calling thread's last error and return code.
int fail(int code, const std::string& msg);

#define FGC_CUDA(call)                                                                                             \
    do {                                                                                                           \
        cudaError_t e_ = (call);                                                                                   \
        if (e_ != cudaSuccess) return ::fgc::fail(FGC_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

template <typename T>
struct DevBuf {
    T* p = nullptr;
    size_t cap = 0;
    DevBuf() = default;
    DevBuf(const DevBuf&) = delete;
    DevBuf& operator=(const DevBuf&) = delete;
    ~DevBuf() { release(); }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        cap = 0;
    }
    // Make room for n elements (contents not preserved when it grows).
    cudaError_t ensure(size_t n) {
        if (n <= cap && p) return cudaSuccess;
        release();
        size_t want = std::max<size_t>(n + n / 4, 64);
        cudaError_t e = cudaMalloc((void**)&p, want * sizeof(T));
        if (e != cudaSuccess) {
            p = nullptr;
            return e;
        }
        cap = want;
        return cudaSuccess;
    }
};

// Page-locked host staging (the table upload and the results of a pass).
struct PinnedBuf {
    unsigned char* p = nullptr;
    size_t cap = 0;
    PinnedBuf() = default;
    PinnedBuf(const PinnedBuf&) = delete;
    PinnedBuf& operator=(const PinnedBuf&) = delete;
    ~PinnedBuf() { release(); }
    void release() {
        if (p) cudaFreeHost(p);
        p = nullptr;
        cap = 0;
    }
    cudaError_t ensure(size_t n) {
        if (n <= cap && p) return cudaSuccess;
        release();
        size_t want = std::max<size_t>(n + n / 4, 4096);
        cudaError_t e = cudaMallocHost((void**)&p, want);
        if (e != cudaSuccess) {
            p = nullptr;
            return e;
        }
        cap = want;
        return cudaSuccess;
    }
};

constexpr int kRasterThreads = 256;

// The look-back of the draw pipeline's ordered allocations and scans: the
// limit on polls of an unpublished predecessor (kSpinLimit) and no withheld
// block, unless fgc_debug_lookback set a test configuration.
extern std::atomic<uint32_t> g_lookback_spin_limit;
extern std::atomic<uint32_t> g_lookback_withhold;
inline Lookback draw_lookback(unsigned long long* tiles, unsigned int* ticket, unsigned int* status,
                              unsigned long long* total) {
    Lookback L{tiles, ticket, status, total};
    L.spin_limit = g_lookback_spin_limit.load(std::memory_order_relaxed);
    L.withhold = g_lookback_withhold.load(std::memory_order_relaxed);
    return L;
}
constexpr int kMaxBands = 24576;

uint32_t pack_nrgba_host(const double c[4]);
int grid_for(uint64_t n, int block, int cap);

// Shared-memory limits of a device and the raster kernels' static usage,
// read once per device.
struct DevLimits {
    int device = -1;
    int sms = 1;
    int smem_per_sm = 0;
    int smem_per_block_optin = 0;
    int smem_reserved_per_block = 0;
    int raster_static[2] = {0, 0};  // plain, mixed
};
int dev_limits(int device, const DevLimits** out);

}  // namespace fgc

struct fgc_texture {
    int device = 0;
    int32_t w = 0, h = 0;
    fgc::DevBuf<ushort4> texels;
    fgc::DevBuf<double> unit64;  // 4 per texel: the channels as float64(c) / 0xffff
};

struct fgc_mesh {
    int device = 0;
    uint64_t ntri = 0, nline = 0, nuniq = 0;
    fgc::DevBuf<double> ux, uy, uz;
    fgc::DevBuf<uint32_t> corner_uniq;
    fgc::DevBuf<fgc::APosNrm64> pn64;
    fgc::DevBuf<fgc::APosNrm32> pn32;
    fgc::DevBuf<double> tex64, col64;
    fgc::DevBuf<float> tex32, col32;
    bool has_tex = false, has_col = false;

    fgc::MeshView view() const {
        fgc::MeshView v;
        v.ntri = ntri;
        v.nline = nline;
        v.nuniq = nuniq;
        v.upos_x = ux.p;
        v.upos_y = uy.p;
        v.upos_z = uz.p;
        v.corner_uniq = corner_uniq.p;
        v.pn64 = pn64.p;
        v.tex64 = has_tex ? tex64.p : nullptr;
        v.col64 = has_col ? col64.p : nullptr;
        v.pn32 = pn32.p;
        v.tex32 = has_tex ? tex32.p : nullptr;
        v.col32 = has_col ? col32.p : nullptr;
        return v;
    }
};

// Weld device corner positions cp (3 doubles per corner) into m and fill its
// position/normal records from nrm (device, or null for zero normals).
int mesh_weld_attrs(fgc_mesh* m, cudaStream_t s, int sms, const double* cp, const double* nrm, uint64_t V);

namespace fgc {

// Pass-wide device counters (one block per pass; the status word is shared by
// all passes of one submission so that a later pass skips its raster stage
// once an earlier one has overflowed).
struct PassCounters {
    unsigned int clip_count;
    unsigned int lclip_count;
    unsigned int band_counter;
    unsigned int tick_setup;
    unsigned int tick_scan;
    unsigned int tick_rscan;
    unsigned long long prim_total;
    unsigned long long pair_total;
    unsigned long long reserved;
    unsigned long long work_total;  // setup work items of the pass
    unsigned long long pad1;
};

// Tunable shapes of a pass; results do not depend on them.
struct PassTuning {
    int64_t band_pixels = 4096;         // pixels per band, rounded to whole rows
    int64_t prims_per_bin_block = 4096; // raster primitives per binning block
    int frag_cap = 1024;                // upper bound of the raster fragment buffer
    int window = 8;                     // raster fragment offsets per thread and round (wide primitives)
};

// One draw of a pass, as the host describes it.
struct PassItem {
    fgc_context* ctx = nullptr;
    const fgc_mesh* mesh = nullptr;
    uint64_t tf = 0, tc = 0, lf = 0, lc = 0;
    StateView sv;
    ShaderView shv;
    bool clear_color = false, clear_depth = false;
    uint32_t clear_color_value = 0;
    double clear_depth_value = 0;
};

// Scratch of the pass pipeline (buffers grow on demand and are reused by the
// passes issued on one stream).
struct PassScratch {
    DevBuf<VClip> vclip;
    DevBuf<double2> vndc;
    DevBuf<VScreen> vscr;
    DevBuf<uint8_t> vout;
    DevBuf<RPrim> prims;
    DevBuf<PBox> pbox;
    DevBuf<float4> rf;
    DevBuf<uint32_t> pspan;
    DevBuf<ClipEntry> clip_list, lclip_list;
    DevBuf<PoolVertex> pool;
    DevBuf<PoolVertex32> pool32;
    DevBuf<ClipPoly> cpoly;        // per clip_list entry: its clipped polygon
    DevBuf<ClipVert> cvert;        // per clip_list entry: the polygon's vertices
    DevBuf<uint32_t> mat, off, bins;
    DevBuf<uint32_t> pnb, prs;     // per primitive: bands it is binned to, first row-start slot
    DevBuf<double> rstart;         // per (primitive, band): edge values at its first row in the band
    DevBuf<unsigned long long> tiles;
    DevBuf<unsigned char> table;   // item views + lookup starts + per-draw results + counters + status
    DevBuf<double> dbg;
    DevBuf<SetupWork> work;        // setup work items (triangles, wireframe edges, lines)
    DevBuf<uint16_t> smeta;        // per element of a setup tile: its setup decision
    DevBuf<uint32_t> cidx;         // per element of a setup tile: its clip_list entry (clipped triangles)
    DevBuf<unsigned long long> tsum;  // per setup tile: its sums, then their exclusive prefix
    PinnedBuf host_in, host_out;
    uint32_t clip_cap = 1024;
    uint64_t bin_cap = 0;
    // the clip kernels run on a second stream beside the setup scan, list
    // writer and emission
    int side_device = -1;
    cudaStream_t side = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_clip = nullptr, ev_join = nullptr;
    PassScratch() = default;
    PassScratch(const PassScratch&) = delete;
    PassScratch& operator=(const PassScratch&) = delete;
    ~PassScratch() {
        if (ev_fork) cudaEventDestroy(ev_fork);
        if (ev_join) cudaEventDestroy(ev_join);
        if (side) cudaStreamDestroy(side);
    }
};

// The host's record of one issued pass (for reading its results).
struct PassRecord {
    std::vector<uint32_t> items;  // indices into the submission's item list
    size_t in_off = 0;            // offset of its staging in host_in
    size_t out_off = 0;           // offset of its results in host_out
    uint32_t nbands = 0;
    int32_t band_rows = 0;
    uint64_t launches = 0;
};

// A submission: the passes that render a list of draws in order. Draws that
// share a target context or differ in precision go to separate passes.
struct Submission {
    std::vector<PassItem> items;
    std::vector<PassRecord> passes;
    std::vector<fgc_rasterize_info> infos;
    std::vector<std::vector<cudaEvent_t>> events;  // stage boundaries per pass, when timing
    fgc_stats stats = {};
    bool timing = false;
    Submission() = default;
    Submission(const Submission&) = delete;
    Submission& operator=(const Submission&) = delete;
    ~Submission();
    void reset();  // before the first issue: clears results, passes and events
};

// Plan the submission's passes and grow the scratch for them (no stream
// work): after it, issue_submission allocates nothing, so it may be captured
// into a CUDA graph.
int prepare_submission(PassScratch& S, const DevLimits& D, const PassTuning& T, const Submission& sub);
// Split items into passes and issue passes [first_pass, end) on stream (no
// host wait), each followed by the copy of its results. The submission's
// status word is zeroed first.
int issue_submission(PassScratch& S, cudaStream_t stream, const DevLimits& D, const PassTuning& T,
                     Submission& sub, size_t first_pass);
// After the stream has drained: read the results of passes [from, end).
// Sets *retry_from = passes.size() when they all succeeded; otherwise grows
// the scratch limits and sets *retry_from to the first pass to re-issue.
int collect_submission(PassScratch& S, Submission& sub, size_t from, size_t* retry_from);
// Wait for passes [from, end) and re-issue failed ones until all succeed.
int finish_submission(PassScratch& S, cudaStream_t stream, const DevLimits& D, const PassTuning& T, Submission& sub,
                      size_t from);
// reset + issue + finish.
int run_submission(PassScratch& S, cudaStream_t stream, const DevLimits& D, const PassTuning& T, Submission& sub);

// Validate a state / shader pair and convert it to device views.
int fill_views(const fgc_state* st, const fgc_shader* sh, StateView& sv, ShaderView& shv);
const char* last_error();

}  // namespace fgc

namespace fgc {
// FGC_ERR_BUSY while a batch has unfinished draws on the context (call with
// the context's mutex held).
int context_ready(const fgc_context* c);
// Allocate the debug buffers the context's flags ask for.
int ensure_debug(fgc_context* c);
}  // namespace fgc

struct fgc_context {
    int device = 0;
    int sms = 1;
    cudaStream_t stream = nullptr;      // the stream work is issued on
    cudaStream_t own_stream = nullptr;  // the context's own stream
    int32_t W = 0, H = 0;
    int64_t N = 0;
    fgc::DevBuf<uint32_t> color;
    fgc::DevBuf<double> depth;
    bool clear_color_pending = false, clear_depth_pending = false;
    uint32_t clear_color = 0;
    double clear_depth = 1.7976931348623157e308;
    int debug = 0;
    fgc::DevBuf<uint32_t> winner;
    fgc::DevBuf<double> shaded;
    fgc::PassScratch scratch;           // the context's own draws
    fgc::DevBuf<unsigned long long> lohi;
    fgc::DevBuf<uint32_t> ds;
    fgc::DevBuf<uint16_t> gray;
    bool timing = false;
    fgc_stats stats = {};
    const void* busy = nullptr;         // the batch that has unfinished work on this context
    std::mutex mu;
};
