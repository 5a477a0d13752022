// fgc_api.cu -- host runtime of libfauxglcuda: the C ABI of
// include/fauxglcuda.h (contexts, meshes, textures, draws, read-back).
//
// DrawMesh / DrawTriangles / DrawLines run a pass of one draw through the
// pass engine (fgc_pass.cu) on the context's stream and wait for it: the
// reference returns RasterizeInfo by value (context.go:391-439). The batch
// interface (fgc_batch.cu) runs passes of many draws.
#include "fgc_host.cuh"

#include <cmath>
#include <new>

using namespace fgc;

namespace fgc {

namespace {
thread_local std::string g_err = "";
}  // namespace

int fail(int code, const std::string& msg) {
    g_err = msg;
    return code;
}

const char* last_error() { return g_err.c_str(); }

int grid_for(uint64_t n, int block, int cap) {
    uint64_t g = (n + block - 1) / block;
    if (g < 1) g = 1;
    if (g > (uint64_t)cap) g = cap;
    return (int)g;
}

uint32_t pack_nrgba_host(const double c[4]) {
    uint32_t out = 0;
    for (int k = 0; k < 4; k++) {
        double v = c[k];
        if (v < 0) v = 0;
        if (v > 1) v = 1;
        double s = v * 255.0;
        uint32_t b = (s == s) ? (uint32_t)(int64_t)s : 0u;  // truncation, NaN -> 0
        out |= (b & 0xff) << (8 * k);
    }
    return out;
}

int fill_views(const fgc_state* st, const fgc_shader* sh, StateView& sv, ShaderView& shv) {
    if (sh->kind != FGC_SHADER_SOLID_COLOR && sh->kind != FGC_SHADER_TEXTURE && sh->kind != FGC_SHADER_PHONG)
        return fail(FGC_ERR_UNSUPPORTED_SHADER, "shader kind is not a built-in shader");
    if (st->cull < FGC_CULL_NONE || st->cull > FGC_CULL_BACK)
        return fail(FGC_ERR_INVALID_ARGUMENT, "cull must be FGC_CULL_NONE, FGC_CULL_FRONT or FGC_CULL_BACK");
    if (st->front_face != FGC_FACE_CW && st->front_face != FGC_FACE_CCW)
        return fail(FGC_ERR_INVALID_ARGUMENT, "front_face must be FGC_FACE_CW or FGC_FACE_CCW");
    if (st->precision != FGC_PRECISION_PLAIN && st->precision != FGC_PRECISION_MIXED)
        return fail(FGC_ERR_INVALID_ARGUMENT, "precision must be FGC_PRECISION_PLAIN or FGC_PRECISION_MIXED");
    if (sh->kind == FGC_SHADER_TEXTURE && !sh->texture)
        return fail(FGC_ERR_INVALID_ARGUMENT, "TextureShader needs a texture");
    sv.read_depth = st->read_depth != 0;
    sv.write_depth = st->write_depth != 0;
    sv.write_color = st->write_color != 0;
    sv.alpha_blend = st->alpha_blend != 0;
    sv.wireframe = st->wireframe != 0;
    sv.front_face = st->front_face;
    sv.cull = st->cull;
    sv.precision = st->precision;
    sv.line_width = st->line_width;
    sv.depth_bias = st->depth_bias;
    memset(&shv, 0, sizeof(shv));
    shv.kind = sh->kind;
    memcpy(shv.m, sh->matrix, sizeof(shv.m));
    memcpy(shv.color, sh->color, sizeof(shv.color));
    memcpy(shv.light, sh->light_direction, sizeof(shv.light));
    memcpy(shv.eye, sh->camera_position, sizeof(shv.eye));
    memcpy(shv.ambient, sh->ambient_color, sizeof(shv.ambient));
    memcpy(shv.diffuse, sh->diffuse_color, sizeof(shv.diffuse));
    memcpy(shv.specular, sh->specular_color, sizeof(shv.specular));
    shv.power = sh->specular_power;
    for (int k = 0; k < 4; k++) {
        shv.color32[k] = (float)shv.color[k];
        shv.ambient32[k] = (float)shv.ambient[k];
        shv.diffuse32[k] = (float)shv.diffuse[k];
        shv.specular32[k] = (float)shv.specular[k];
    }
    for (int k = 0; k < 3; k++) {
        shv.light32[k] = (float)shv.light[k];
        shv.eye32[k] = (float)shv.eye[k];
    }
    shv.power32 = (float)shv.power;
    shv.power_pos = shv.power > 0 ? 1 : 0;
    shv.pow_yi = 0;
    if (shv.power >= 2 && shv.power < 9223372036854775808.0 && shv.power == std::trunc(shv.power))
        shv.pow_yi = (uint64_t)shv.power;
    shv.object_is_discard = (sh->color[0] == 0 && sh->color[1] == 0 && sh->color[2] == 0 && sh->color[3] == 0);
    // equal channels give equal light channels: the shader then computes one
    auto same3 = [](const double* c) { return memcmp(&c[0], &c[1], 8) == 0 && memcmp(&c[0], &c[2], 8) == 0; };
    shv.gray_light = same3(shv.ambient) && same3(shv.diffuse) ? 1 : 0;
    shv.gray_spec = same3(shv.specular) ? 1 : 0;
    if (sh->texture) {
        shv.has_texture = 1;
        shv.tex.texels = sh->texture->texels.p;
        shv.tex.unit64 = sh->texture->unit64.p;
        shv.tex.w = sh->texture->w;
        shv.tex.h = sh->texture->h;
    }
    return FGC_OK;
}

int ensure_debug(fgc_context* c) {
    if (!(c->debug & (FGC_DEBUG_WINNER | FGC_DEBUG_SHADED_COLOR))) return FGC_OK;
    int grid = grid_for((uint64_t)c->N, 256, c->sms * 8);
    if ((c->debug & FGC_DEBUG_WINNER) && !c->winner.p) {
        FGC_CUDA(c->winner.ensure((size_t)c->N));
        fill_u32_kernel<<<grid, 256, 0, c->stream>>>(c->winner.p, (uint64_t)c->N, 0xFFFFFFFFu);
        FGC_CUDA(cudaGetLastError());
    }
    if ((c->debug & FGC_DEBUG_SHADED_COLOR) && !c->shaded.p) {
        FGC_CUDA(c->shaded.ensure((size_t)c->N * 4));
        FGC_CUDA(cudaMemsetAsync(c->shaded.p, 0, (size_t)c->N * 4 * sizeof(double), c->stream));
    }
    return FGC_OK;
}

int context_ready(const fgc_context* c) {
    if (c->busy) return fail(FGC_ERR_BUSY, "the context has draws in an unfinished batch");
    return FGC_OK;
}

}  // namespace fgc

namespace {

int apply_pending_clears(fgc_context* c) {
    int grid = grid_for((uint64_t)c->N, 256, c->sms * 8);
    if (c->clear_color_pending) {
        fill_u32_kernel<<<grid, 256, 0, c->stream>>>(c->color.p, (uint64_t)c->N, c->clear_color);
        FGC_CUDA(cudaGetLastError());
        c->clear_color_pending = false;
    }
    if (c->clear_depth_pending) {
        fill_f64_kernel<<<grid, 256, 0, c->stream>>>(c->depth.p, (uint64_t)c->N, c->clear_depth);
        FGC_CUDA(cudaGetLastError());
        c->clear_depth_pending = false;
    }
    return FGC_OK;
}

int draw(fgc_context* c, const fgc_mesh* m, uint64_t tf, uint64_t tc, uint64_t lf, uint64_t lc,
         const fgc_state* st, const fgc_shader* sh, fgc_rasterize_info* info) {
    if (!c || !m || !st || !sh) return fail(FGC_ERR_INVALID_ARGUMENT, "null argument");
    if (m->device != c->device) return fail(FGC_ERR_INVALID_ARGUMENT, "mesh and context are on different devices");
    if (tf > m->ntri || tc > m->ntri - tf) return fail(FGC_ERR_INVALID_ARGUMENT, "triangle range out of bounds");
    if (lf > m->nline || lc > m->nline - lf) return fail(FGC_ERR_INVALID_ARGUMENT, "line range out of bounds");
    if (sh->texture && sh->texture->device != c->device)
        return fail(FGC_ERR_INVALID_ARGUMENT, "texture is on another device");
    Submission sub;
    sub.items.resize(1);
    PassItem& it = sub.items[0];
    int rc = fill_views(st, sh, it.sv, it.shv);
    if (rc) return rc;
    std::lock_guard<std::mutex> lock(c->mu);
    rc = context_ready(c);
    if (rc) return rc;
    FGC_CUDA(cudaSetDevice(c->device));
    const DevLimits* D = nullptr;
    rc = dev_limits(c->device, &D);
    if (rc) return rc;
    rc = ensure_debug(c);
    if (rc) return rc;
    it.ctx = c;
    it.mesh = m;
    it.tf = tf;
    it.tc = tc;
    it.lf = lf;
    it.lc = lc;
    it.clear_color = c->clear_color_pending;
    it.clear_depth = c->clear_depth_pending;
    it.clear_color_value = c->clear_color;
    it.clear_depth_value = c->clear_depth;
    sub.timing = c->timing;
    static const PassTuning kDefaultTuning;
    rc = run_submission(c->scratch, c->stream, *D, kDefaultTuning, sub);
    c->stats = sub.stats;
    c->stats.elements = tc + lc;
    c->stats.unique_vertices = (tc > 0 || lc > 0) ? m->nuniq : 0;
    if (rc) return rc;
    // the pass applied the pending clears (fused into its raster stage)
    c->clear_color_pending = false;
    c->clear_depth_pending = false;
    if (info) *info = sub.infos[0];
    return FGC_OK;
}

}  // namespace

// ===========================================================================
// C ABI
// ===========================================================================
// Weld the corner positions cp (device, 3 per corner) and fill the mesh's
// unique-position arrays, corner index and position/normal records (nrm may
// be null: zero normals). Runs on stream s and waits for it.
int mesh_weld_attrs(fgc_mesh* m, cudaStream_t s, int sms, const double* cp, const double* nrm, uint64_t V) {
    int rc = FGC_OK;
    DevBuf<uint32_t> table, slot_of, minc, flag, uid;
    DevBuf<unsigned long long> tiles;
    DevBuf<unsigned int> st, tick;
    unsigned long long* h_tot = nullptr;
    auto step = [&](cudaError_t err, const char* what) {
        if (err != cudaSuccess && rc == FGC_OK) rc = fail(FGC_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(err));
        return rc == FGC_OK;
    };
    const int grid = grid_for(V, 256, sms * 16);
    do {
        // weld positions
        uint64_t tsize = 1;
        while (tsize < 2 * V) tsize <<= 1;
        if (!step(table.ensure(tsize), "alloc weld table")) break;
        if (!step(minc.ensure(tsize), "alloc weld table")) break;
        if (!step(slot_of.ensure(V), "alloc weld") || !step(flag.ensure(V), "alloc weld") || !step(uid.ensure(V), "alloc weld")) break;
        if (!step(st.ensure(1), "alloc status") || !step(cudaMemsetAsync(st.p, 0, 4, s), "zero status")) break;
        if (!step(cudaMemsetAsync(table.p, 0xFF, tsize * 4, s), "init table")) break;
        if (!step(cudaMemsetAsync(minc.p, 0xFF, tsize * 4, s), "init table")) break;
        weld_insert_kernel<<<grid, 256, 0, s>>>(cp, V, table.p, tsize - 1, slot_of.p, minc.p, st.p);
        weld_flag_kernel<<<grid, 256, 0, s>>>(slot_of.p, minc.p, V, flag.p);
        const uint64_t scan_tiles = (V + 2047) / 2048;
        if (!step(tiles.ensure(scan_tiles + 2), "alloc scan") || !step(cudaMemsetAsync(tiles.p, 0, (scan_tiles + 2) * 8, s), "zero scan")) break;
        ScanParams sp;
        sp.n_dev = nullptr;
        sp.in = flag.p;
        sp.out = uid.p;
        sp.n = V;
        sp.lb = Lookback{tiles.p + 1, (unsigned int*)(st.p), st.p, tiles.p};
        // the scan's ticket counter and status share the zeroed status word's
        // neighbour: use a dedicated zeroed word instead
        if (!step(tick.ensure(1), "alloc ticket") || !step(cudaMemsetAsync(tick.p, 0, 4, s), "zero ticket")) break;
        sp.lb.ticket = tick.p;
        scan_u32_kernel<<<(unsigned)scan_tiles, 256, 0, s>>>(sp);
        if (!step(cudaGetLastError(), "weld kernels")) break;
        if (!step(cudaMallocHost((void**)&h_tot, 16), "alloc pinned")) break;
        if (!step(cudaMemcpyAsync(h_tot, tiles.p, 8, cudaMemcpyDeviceToHost, s), "read unique count")) break;
        if (!step(cudaMemcpyAsync(h_tot + 1, st.p, 4, cudaMemcpyDeviceToHost, s), "read status")) break;
        if (!step(cudaStreamSynchronize(s), "weld")) break;
        if (((unsigned int*)(h_tot + 1))[0] != 0) {
            rc = fail(FGC_ERR_DEVICE_LIMIT, "mesh weld failed");
            break;
        }
        m->nuniq = h_tot[0];
        if (!step(m->ux.ensure(m->nuniq + 1), "alloc unique") || !step(m->uy.ensure(m->nuniq + 1), "alloc unique") ||
            !step(m->uz.ensure(m->nuniq + 1), "alloc unique") || !step(m->corner_uniq.ensure(V), "alloc index"))
            break;
        weld_emit_kernel<<<grid, 256, 0, s>>>(cp, slot_of.p, minc.p, uid.p, V, m->ux.p, m->uy.p, m->uz.p,
                                              m->corner_uniq.p);
        if (!step(m->pn64.ensure(V), "alloc attributes") || !step(m->pn32.ensure(V), "alloc attributes")) break;
        attrs_kernel<<<grid, 256, 0, s>>>(cp, nrm, V, m->pn64.p, m->pn32.p);
        if (!step(cudaGetLastError(), "attribute kernels")) break;
    } while (0);
    cudaStreamSynchronize(s);
    if (h_tot) cudaFreeHost(h_tot);
    return rc;
}

extern "C" {

int32_t fgc_abi_version(void) { return FGC_ABI_VERSION; }

const char* fgc_last_error(void) { return fgc::last_error(); }

void fgc_state_default(fgc_state* st) {
    if (!st) return;
    st->read_depth = 1;
    st->write_depth = 1;
    st->write_color = 1;
    st->alpha_blend = 1;
    st->wireframe = 0;
    st->front_face = FGC_FACE_CCW;
    st->cull = FGC_CULL_BACK;
    st->precision = FGC_PRECISION_PLAIN;
    st->line_width = 2;
    st->depth_bias = 0;
}

static void shader_common(fgc_shader* sh, int kind, const double matrix[16]) {
    memset(sh, 0, sizeof(*sh));
    sh->kind = kind;
    if (matrix) memcpy(sh->matrix, matrix, sizeof(sh->matrix));
}

void fgc_shader_solid_color(fgc_shader* sh, const double matrix[16], const double rgba[4]) {
    if (!sh) return;
    shader_common(sh, FGC_SHADER_SOLID_COLOR, matrix);
    if (rgba) memcpy(sh->color, rgba, sizeof(sh->color));
}

void fgc_shader_texture(fgc_shader* sh, const double matrix[16], const fgc_texture* tex) {
    if (!sh) return;
    shader_common(sh, FGC_SHADER_TEXTURE, matrix);
    sh->texture = tex;
}

void fgc_shader_phong(fgc_shader* sh, const double matrix[16], const double light_direction[3],
                      const double camera_position[3]) {
    if (!sh) return;
    shader_common(sh, FGC_SHADER_PHONG, matrix);
    if (light_direction) memcpy(sh->light_direction, light_direction, sizeof(sh->light_direction));
    if (camera_position) memcpy(sh->camera_position, camera_position, sizeof(sh->camera_position));
    const double amb[4] = {0.2, 0.2, 0.2, 1}, dif[4] = {0.8, 0.8, 0.8, 1}, spe[4] = {1, 1, 1, 1};
    memcpy(sh->ambient_color, amb, sizeof(amb));
    memcpy(sh->diffuse_color, dif, sizeof(dif));
    memcpy(sh->specular_color, spe, sizeof(spe));
    sh->specular_power = 32;
}

namespace {
int noalloc_prepare(int device);
}

int fgc_context_create(int32_t width, int32_t height, fgc_context** out) {
    if (!out) return fail(FGC_ERR_INVALID_ARGUMENT, "out is null");
    *out = nullptr;
    if (width < 1 || height < 1) return fail(FGC_ERR_INVALID_ARGUMENT, "width and height must be positive");
    if ((int64_t)width * height > (int64_t)1 << 34) return fail(FGC_ERR_INVALID_ARGUMENT, "frame too large");
    if (height > (1 << 30)) return fail(FGC_ERR_UNSUPPORTED, "frame height above 2^30 rows is not supported");
    fgc_context* c = new (std::nothrow) fgc_context();
    if (!c) return fail(FGC_ERR_OUT_OF_MEMORY, "host allocation failed");
    auto bail = [&](int rc) {
        delete c;
        return rc;
    };
    cudaError_t e = cudaGetDevice(&c->device);
    if (e != cudaSuccess) return bail(fail(FGC_ERR_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e)));
    cudaDeviceGetAttribute(&c->sms, cudaDevAttrMultiProcessorCount, c->device);
    e = cudaStreamCreateWithFlags(&c->own_stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) return bail(fail(FGC_ERR_CUDA, std::string("cudaStreamCreate: ") + cudaGetErrorString(e)));
    c->stream = c->own_stream;
    c->W = width;
    c->H = height;
    c->N = (int64_t)width * height;
    if (c->color.ensure((size_t)c->N) != cudaSuccess || c->depth.ensure((size_t)c->N) != cudaSuccess)
        return bail(fail(FGC_ERR_OUT_OF_MEMORY, "framebuffer allocation failed"));
    // NewContext: transparent colour buffer, depth cleared to MaxFloat64
    // (context.go:64-79); applied lazily by the first kernel that needs it.
    c->clear_color = 0;
    c->clear_color_pending = true;
    c->clear_depth = 1.7976931348623157e308;
    c->clear_depth_pending = true;
    // fgc_depth_image_noalloc's static scratch and kernels are made resident
    // here, so that the entry point itself never makes the driver allocate
    int rc = noalloc_prepare(c->device);
    if (rc) return bail(rc);
    *out = c;
    return FGC_OK;
}

int fgc_context_destroy(fgc_context* c) {
    if (!c) return FGC_OK;
    {
        std::lock_guard<std::mutex> lock(c->mu);
        int rc = context_ready(c);
        if (rc) return rc;
    }
    cudaSetDevice(c->device);
    cudaStreamSynchronize(c->stream);
    if (c->own_stream) cudaStreamDestroy(c->own_stream);
    delete c;
    return FGC_OK;
}

int fgc_context_size(const fgc_context* c, int32_t* w, int32_t* h) {
    if (!c) return fail(FGC_ERR_INVALID_ARGUMENT, "null context");
    if (w) *w = c->W;
    if (h) *h = c->H;
    return FGC_OK;
}

int fgc_context_set_debug(fgc_context* c, int32_t flags) {
    if (!c) return fail(FGC_ERR_INVALID_ARGUMENT, "null context");
    std::lock_guard<std::mutex> lock(c->mu);
    if (int rc_ = context_ready(c)) return rc_;
    FGC_CUDA(cudaSetDevice(c->device));
    c->debug = flags;
    int rc = ensure_debug(c);
    if (rc) return rc;
    FGC_CUDA(cudaStreamSynchronize(c->stream));
    return FGC_OK;
}

int fgc_context_set_timing(fgc_context* c, int32_t enable) {
    if (!c) return fail(FGC_ERR_INVALID_ARGUMENT, "null context");
    std::lock_guard<std::mutex> lock(c->mu);
    if (int rc_ = context_ready(c)) return rc_;
    c->timing = enable != 0;
    return FGC_OK;
}

int fgc_context_last_stats(const fgc_context* c, fgc_stats* out) {
    if (!c || !out) return fail(FGC_ERR_INVALID_ARGUMENT, "null argument");
    *out = c->stats;
    return FGC_OK;
}

int fgc_context_set_stream(fgc_context* c, void* cuda_stream) {
    if (!c) return fail(FGC_ERR_INVALID_ARGUMENT, "null context");
    std::lock_guard<std::mutex> lock(c->mu);
    if (int rc_ = context_ready(c)) return rc_;
    FGC_CUDA(cudaSetDevice(c->device));
    FGC_CUDA(cudaStreamSynchronize(c->stream));
    c->stream = cuda_stream ? (cudaStream_t)cuda_stream : c->own_stream;
    return FGC_OK;
}

int fgc_debug_lookback(uint32_t spin_limit, uint32_t withhold_block) {
    g_lookback_spin_limit.store(spin_limit ? spin_limit : kSpinLimit, std::memory_order_relaxed);
    g_lookback_withhold.store(withhold_block, std::memory_order_relaxed);
    return FGC_OK;
}

int fgc_measure_fp64_rate(double* gops_per_s) {
    if (!gops_per_s) return fail(FGC_ERR_INVALID_ARGUMENT, "null argument");
    int dev = 0, sms = 1;
    FGC_CUDA(cudaGetDevice(&dev));
    FGC_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const int blocks = sms * 8, threads = 256, iters = 4096;
    DevBuf<double> out;
    FGC_CUDA(out.ensure((size_t)blocks * threads));
    cudaStream_t s;
    FGC_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    float best = 1e30f;
    for (int r = 0; r < 4; r++) {
        cudaEventRecord(e0, s);
        fp64_rate_kernel<<<blocks, threads, 0, s>>>(out.p, 1e-9, 2e-9, iters);
        cudaEventRecord(e1, s);
        cudaError_t e = cudaEventSynchronize(e1);
        if (e != cudaSuccess) {
            cudaEventDestroy(e0);
            cudaEventDestroy(e1);
            cudaStreamDestroy(s);
            return fail(FGC_ERR_CUDA, std::string("fp64 probe: ") + cudaGetErrorString(e));
        }
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        if (r > 0 && ms < best) best = ms;  // the first run warms up
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaStreamDestroy(s);
    *gops_per_s = (double)blocks * threads * iters * 8 / (best * 1e-3) / 1e9;
    return FGC_OK;
}

int fgc_clear_color(fgc_context* c, const double rgba[4]) {
    if (!c || !rgba) return fail(FGC_ERR_INVALID_ARGUMENT, "null argument");
    std::lock_guard<std::mutex> lock(c->mu);
    if (int rc_ = context_ready(c)) return rc_;
    c->clear_color = pack_nrgba_host(rgba);
    c->clear_color_pending = true;
    return FGC_OK;
}

int fgc_clear_depth(fgc_context* c, double value) {
    if (!c) return fail(FGC_ERR_INVALID_ARGUMENT, "null context");
    std::lock_guard<std::mutex> lock(c->mu);
    if (int rc_ = context_ready(c)) return rc_;
    c->clear_depth = value;
    c->clear_depth_pending = true;
    return FGC_OK;
}

int fgc_mesh_upload(const double* tri_pos, const double* tri_nrm, const double* tri_tex, const double* tri_col,
                    uint64_t ntri, const double* line_pos, const double* line_nrm, const double* line_tex,
                    const double* line_col, uint64_t nline, fgc_mesh** out) {
    if (!out) return fail(FGC_ERR_INVALID_ARGUMENT, "out is null");
    *out = nullptr;
    if ((ntri && !tri_pos) || (nline && !line_pos)) return fail(FGC_ERR_INVALID_ARGUMENT, "positions are required");
    const uint64_t V = 3 * ntri + 2 * nline;
    if (V >= 0x7FFFFFFFull) return fail(FGC_ERR_UNSUPPORTED, "mesh has too many corners (2^31 limit)");
    fgc_mesh* m = new (std::nothrow) fgc_mesh();
    if (!m) return fail(FGC_ERR_OUT_OF_MEMORY, "host allocation failed");
    int dev = 0;
    cudaGetDevice(&dev);
    m->device = dev;
    m->ntri = ntri;
    m->nline = nline;
    int sms = 1;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaStream_t s;
    cudaError_t e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        delete m;
        return fail(FGC_ERR_CUDA, std::string("cudaStreamCreate: ") + cudaGetErrorString(e));
    }
    int rc = FGC_OK;
    DevBuf<double> cp, nrm;
    auto step = [&](cudaError_t err, const char* what) {
        if (err != cudaSuccess && rc == FGC_OK) rc = fail(FGC_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(err));
        return rc == FGC_OK;
    };
    const int grid = grid_for(V, 256, sms * 16);
    do {
        if (V == 0) break;
        if (!step(cp.ensure(V * 3), "alloc positions")) break;
        if (ntri && !step(cudaMemcpyAsync(cp.p, tri_pos, ntri * 9 * 8, cudaMemcpyHostToDevice, s), "copy positions")) break;
        if (nline && !step(cudaMemcpyAsync(cp.p + ntri * 9, line_pos, nline * 6 * 8, cudaMemcpyHostToDevice, s), "copy positions")) break;
        const bool have_nrm = tri_nrm || line_nrm;
        if (have_nrm) {
            if (!step(nrm.ensure(V * 3), "alloc normals")) break;
            if (!step(cudaMemsetAsync(nrm.p, 0, V * 3 * 8, s), "zero normals")) break;
            if (tri_nrm && !step(cudaMemcpyAsync(nrm.p, tri_nrm, ntri * 9 * 8, cudaMemcpyHostToDevice, s), "copy normals")) break;
            if (line_nrm && !step(cudaMemcpyAsync(nrm.p + ntri * 9, line_nrm, nline * 6 * 8, cudaMemcpyHostToDevice, s), "copy normals")) break;
        }
        rc = mesh_weld_attrs(m, s, sms, cp.p, have_nrm ? nrm.p : nullptr, V);
        if (rc != FGC_OK) break;
        if (tri_tex || line_tex) {
            m->has_tex = true;
            if (!step(m->tex64.ensure(V * 2), "alloc texcoords") || !step(m->tex32.ensure(V * 2), "alloc texcoords")) break;
            if (!step(cudaMemsetAsync(m->tex64.p, 0, V * 2 * 8, s), "zero texcoords")) break;
            if (tri_tex && !step(cudaMemcpyAsync(m->tex64.p, tri_tex, ntri * 6 * 8, cudaMemcpyHostToDevice, s), "copy texcoords")) break;
            if (line_tex && !step(cudaMemcpyAsync(m->tex64.p + ntri * 6, line_tex, nline * 4 * 8, cudaMemcpyHostToDevice, s), "copy texcoords")) break;
            f64_to_f32_kernel<<<grid, 256, 0, s>>>(m->tex64.p, V * 2, m->tex32.p);
        }
        if (tri_col || line_col) {
            m->has_col = true;
            if (!step(m->col64.ensure(V * 4), "alloc colours") || !step(m->col32.ensure(V * 4), "alloc colours")) break;
            if (!step(cudaMemsetAsync(m->col64.p, 0, V * 4 * 8, s), "zero colours")) break;
            if (tri_col && !step(cudaMemcpyAsync(m->col64.p, tri_col, ntri * 12 * 8, cudaMemcpyHostToDevice, s), "copy colours")) break;
            if (line_col && !step(cudaMemcpyAsync(m->col64.p + ntri * 12, line_col, nline * 8 * 8, cudaMemcpyHostToDevice, s), "copy colours")) break;
            f64_to_f32_kernel<<<grid, 256, 0, s>>>(m->col64.p, V * 4, m->col32.p);
        }
        if (!step(cudaGetLastError(), "attribute kernels")) break;
        step(cudaStreamSynchronize(s), "mesh upload");
    } while (0);
    cudaStreamSynchronize(s);
    cudaStreamDestroy(s);
    if (rc != FGC_OK) {
        delete m;
        return rc;
    }
    *out = m;
    return FGC_OK;
}

int fgc_mesh_release(fgc_mesh* m) {
    if (!m) return FGC_OK;
    cudaSetDevice(m->device);
    cudaDeviceSynchronize();
    delete m;
    return FGC_OK;
}

int fgc_mesh_counts(const fgc_mesh* m, uint64_t* ntri, uint64_t* nline) {
    if (!m) return fail(FGC_ERR_INVALID_ARGUMENT, "null mesh");
    if (ntri) *ntri = m->ntri;
    if (nline) *nline = m->nline;
    return FGC_OK;
}

int fgc_texture_upload(const uint16_t* rgba16, int32_t width, int32_t height, fgc_texture** out) {
    if (!out || !rgba16) return fail(FGC_ERR_INVALID_ARGUMENT, "null argument");
    *out = nullptr;
    if (width < 1 || height < 1) return fail(FGC_ERR_INVALID_ARGUMENT, "texture size must be positive");
    fgc_texture* t = new (std::nothrow) fgc_texture();
    if (!t) return fail(FGC_ERR_OUT_OF_MEMORY, "host allocation failed");
    cudaGetDevice(&t->device);
    t->w = width;
    t->h = height;
    size_t n = (size_t)width * height;
    cudaError_t e = t->texels.ensure(n);
    if (e == cudaSuccess) e = t->unit64.ensure(4 * n);
    if (e == cudaSuccess) e = cudaMemcpy(t->texels.p, rgba16, n * sizeof(ushort4), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        fgc::texel_unit_kernel<<<fgc::grid_for(n, 256, 4096), 256>>>(t->texels.p, n, t->unit64.p);
        e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaDeviceSynchronize();
    }
    if (e != cudaSuccess) {
        delete t;
        return fail(FGC_ERR_CUDA, std::string("texture upload: ") + cudaGetErrorString(e));
    }
    *out = t;
    return FGC_OK;
}

int fgc_texture_release(fgc_texture* t) {
    if (!t) return FGC_OK;
    cudaSetDevice(t->device);
    cudaDeviceSynchronize();
    delete t;
    return FGC_OK;
}

int fgc_draw_mesh(fgc_context* c, const fgc_mesh* m, const fgc_state* st, const fgc_shader* sh,
                  fgc_rasterize_info* info) {
    if (!m) return fail(FGC_ERR_INVALID_ARGUMENT, "null mesh");
    return draw(c, m, 0, m->ntri, 0, m->nline, st, sh, info);
}

int fgc_draw_triangles(fgc_context* c, const fgc_mesh* m, uint64_t first, uint64_t count, const fgc_state* st,
                       const fgc_shader* sh, fgc_rasterize_info* info) {
    return draw(c, m, first, count, 0, 0, st, sh, info);
}

int fgc_draw_lines(fgc_context* c, const fgc_mesh* m, uint64_t first, uint64_t count, const fgc_state* st,
                   const fgc_shader* sh, fgc_rasterize_info* info) {
    return draw(c, m, 0, 0, first, count, st, sh, info);
}

int fgc_read_color(fgc_context* c, uint8_t* nrgba) {
    if (!c || !nrgba) return fail(FGC_ERR_INVALID_ARGUMENT, "null argument");
    std::lock_guard<std::mutex> lock(c->mu);
    if (int rc_ = context_ready(c)) return rc_;
    FGC_CUDA(cudaSetDevice(c->device));
    int rc = apply_pending_clears(c);
    if (rc) return rc;
    FGC_CUDA(cudaMemcpyAsync(nrgba, c->color.p, (size_t)c->N * 4, cudaMemcpyDeviceToHost, c->stream));
    FGC_CUDA(cudaStreamSynchronize(c->stream));
    return FGC_OK;
}

int fgc_read_depth(fgc_context* c, double* depth) {
    if (!c || !depth) return fail(FGC_ERR_INVALID_ARGUMENT, "null argument");
    std::lock_guard<std::mutex> lock(c->mu);
    if (int rc_ = context_ready(c)) return rc_;
    FGC_CUDA(cudaSetDevice(c->device));
    int rc = apply_pending_clears(c);
    if (rc) return rc;
    FGC_CUDA(cudaMemcpyAsync(depth, c->depth.p, (size_t)c->N * 8, cudaMemcpyDeviceToHost, c->stream));
    FGC_CUDA(cudaStreamSynchronize(c->stream));
    return FGC_OK;
}

int fgc_write_color(fgc_context* c, const uint8_t* nrgba) {
    if (!c || !nrgba) return fail(FGC_ERR_INVALID_ARGUMENT, "null argument");
    std::lock_guard<std::mutex> lock(c->mu);
    if (int rc_ = context_ready(c)) return rc_;
    FGC_CUDA(cudaSetDevice(c->device));
    c->clear_color_pending = false;
    FGC_CUDA(cudaMemcpyAsync(c->color.p, nrgba, (size_t)c->N * 4, cudaMemcpyHostToDevice, c->stream));
    FGC_CUDA(cudaStreamSynchronize(c->stream));
    return FGC_OK;
}

int fgc_write_depth(fgc_context* c, const double* depth) {
    if (!c || !depth) return fail(FGC_ERR_INVALID_ARGUMENT, "null argument");
    std::lock_guard<std::mutex> lock(c->mu);
    if (int rc_ = context_ready(c)) return rc_;
    FGC_CUDA(cudaSetDevice(c->device));
    c->clear_depth_pending = false;
    FGC_CUDA(cudaMemcpyAsync(c->depth.p, depth, (size_t)c->N * 8, cudaMemcpyHostToDevice, c->stream));
    FGC_CUDA(cudaStreamSynchronize(c->stream));
    return FGC_OK;
}

int fgc_depth_image(fgc_context* c, uint16_t* gray16) {
    if (!c || !gray16) return fail(FGC_ERR_INVALID_ARGUMENT, "null argument");
    std::lock_guard<std::mutex> lock(c->mu);
    if (int rc_ = context_ready(c)) return rc_;
    FGC_CUDA(cudaSetDevice(c->device));
    int rc = apply_pending_clears(c);
    if (rc) return rc;
    FGC_CUDA(c->lohi.ensure(2));
    FGC_CUDA(c->gray.ensure((size_t)c->N));
    unsigned long long init[2] = {~0ull, 0ull};
    FGC_CUDA(cudaMemcpyAsync(c->lohi.p, init, sizeof(init), cudaMemcpyHostToDevice, c->stream));
    FGC_CUDA(cudaStreamSynchronize(c->stream));
    int grid = grid_for((uint64_t)c->N, 256, c->sms * 8);
    depth_minmax_kernel<<<grid, 256, 0, c->stream>>>(c->depth.p, (uint64_t)c->N, c->lohi.p);
    depth_image_kernel<<<grid, 256, 0, c->stream>>>(c->depth.p, (uint64_t)c->N, c->lohi.p, c->gray.p);
    FGC_CUDA(cudaGetLastError());
    FGC_CUDA(cudaMemcpyAsync(gray16, c->gray.p, (size_t)c->N * 2, cudaMemcpyDeviceToHost, c->stream));
    FGC_CUDA(cudaStreamSynchronize(c->stream));
    return FGC_OK;
}

int fgc_downsample(fgc_context* c, int32_t scale, uint8_t* out) {
    if (!c || !out) return fail(FGC_ERR_INVALID_ARGUMENT, "null argument");
    if (scale < 1 || c->W % scale != 0 || c->H % scale != 0)
        return fail(FGC_ERR_INVALID_ARGUMENT, "scale must divide width and height");
    std::lock_guard<std::mutex> lock(c->mu);
    if (int rc_ = context_ready(c)) return rc_;
    FGC_CUDA(cudaSetDevice(c->device));
    int rc = apply_pending_clears(c);
    if (rc) return rc;
    const uint64_t n = (uint64_t)(c->W / scale) * (uint64_t)(c->H / scale);
    FGC_CUDA(c->ds.ensure(n));
    downsample_kernel<<<grid_for(n, 256, c->sms * 8), 256, 0, c->stream>>>(c->color.p, c->W, c->H, scale, c->ds.p);
    FGC_CUDA(cudaGetLastError());
    FGC_CUDA(cudaMemcpyAsync(out, c->ds.p, n * 4, cudaMemcpyDeviceToHost, c->stream));
    FGC_CUDA(cudaStreamSynchronize(c->stream));
    return FGC_OK;
}

int fgc_read_winner(fgc_context* c, uint32_t* winner) {
    if (!c || !winner) return fail(FGC_ERR_INVALID_ARGUMENT, "null argument");
    if (!(c->debug & FGC_DEBUG_WINNER) || !c->winner.p) return fail(FGC_ERR_INVALID_ARGUMENT, "winner ids are off");
    std::lock_guard<std::mutex> lock(c->mu);
    if (int rc_ = context_ready(c)) return rc_;
    FGC_CUDA(cudaSetDevice(c->device));
    FGC_CUDA(cudaMemcpyAsync(winner, c->winner.p, (size_t)c->N * 4, cudaMemcpyDeviceToHost, c->stream));
    FGC_CUDA(cudaStreamSynchronize(c->stream));
    return FGC_OK;
}

int fgc_read_shaded_color(fgc_context* c, double* rgba) {
    if (!c || !rgba) return fail(FGC_ERR_INVALID_ARGUMENT, "null argument");
    if (!(c->debug & FGC_DEBUG_SHADED_COLOR) || !c->shaded.p)
        return fail(FGC_ERR_INVALID_ARGUMENT, "shaded colours are off");
    std::lock_guard<std::mutex> lock(c->mu);
    if (int rc_ = context_ready(c)) return rc_;
    FGC_CUDA(cudaSetDevice(c->device));
    FGC_CUDA(cudaMemcpyAsync(rgba, c->shaded.p, (size_t)c->N * 32, cudaMemcpyDeviceToHost, c->stream));
    FGC_CUDA(cudaStreamSynchronize(c->stream));
    return FGC_OK;
}

}  // extern "C"

// ===========================================================================
// DepthImage without device allocation.
//
// fgc_depth_image above grows c->lohi and c->gray with cudaMalloc the first
// time it runs. Callers that may not let the library allocate device memory
// once they are running (a service that reserves all its buffers before it
// admits work, a host application that owns the GPU memory of its plugins)
// use fgc_depth_image_noalloc instead: the same two kernels, with the
// min/max pair and the Gray16 staging image placed in the static array
// below. The array is reserved on a GPU when the first context on it is
// created and stays until the process exits, which is why it is kept to
// 16 MiB: frames up to FGC_DEPTH_IMAGE_NOALLOC_MAX_PIXELS (2^23) pixels.
//
// Host code cannot use the array's name as a device address. When the first
// context on a device is created (fgc_context_create, with that device
// current) the address is looked up with cudaGetSymbolAddress and kept, and
// the two kernels are loaded: with CUDA's lazy module loading both steps
// make the driver reserve device memory, so they happen at start-up and not
// inside the entry point. Every call re-initialises the min/max pair it
// needs, and every call uses the same array, so calls that overlap on the GPU
// race.
// ===========================================================================
namespace {

constexpr size_t kNoAllocPixels = FGC_DEPTH_IMAGE_NOALLOC_MAX_PIXELS;
constexpr size_t kNoAllocBytes = 256 + kNoAllocPixels * sizeof(uint16_t);

static __device__ __align__(256) unsigned char g_depth_image_scratch[kNoAllocBytes];

std::mutex g_noalloc_mu;
void* g_noalloc_ptr[256] = {};

// Once per device, with the device current: the scratch address and the
// kernels the entry point launches (cudaFuncGetAttributes loads a lazily
// loaded kernel).
int noalloc_prepare(int device) {
    if (device < 0 || device >= 256) return fail(FGC_ERR_UNSUPPORTED, "device ordinal out of range");
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (g_noalloc_ptr[device]) return FGC_OK;
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_depth_image_scratch);
    if (e != cudaSuccess || !p)
        return fail(FGC_ERR_CUDA, std::string("cudaGetSymbolAddress(depth image scratch): ") + cudaGetErrorString(e));
    cudaFuncAttributes fa;
    e = cudaFuncGetAttributes(&fa, depth_minmax_kernel);
    if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, depth_image_kernel);
    if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, fill_u32_kernel);  // pending clears
    if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, fill_f64_kernel);
    if (e != cudaSuccess)
        return fail(FGC_ERR_CUDA, std::string("loading the depth image kernels: ") + cudaGetErrorString(e));
    g_noalloc_ptr[device] = p;
    return FGC_OK;
}

// The scratch of a device prepared by fgc_context_create.
int noalloc_scratch(int device, unsigned char** out) {
    if (device < 0 || device >= 256) return fail(FGC_ERR_UNSUPPORTED, "device ordinal out of range");
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (!g_noalloc_ptr[device]) return fail(FGC_ERR_INVALID_ARGUMENT, "no context was created on this device");
    *out = (unsigned char*)g_noalloc_ptr[device];
    return FGC_OK;
}

}  // namespace

extern "C" int fgc_depth_image_noalloc(fgc_context* c, uint16_t* gray16) {
    if (!c || !gray16) return fail(FGC_ERR_INVALID_ARGUMENT, "null argument");
    if ((uint64_t)c->N > kNoAllocPixels)
        return fail(FGC_ERR_INVALID_ARGUMENT,
                    "fgc_depth_image_noalloc handles at most 8388608 pixels (its static scratch is 16 MiB); "
                    "use fgc_depth_image for larger frames");
    std::lock_guard<std::mutex> lock(c->mu);
    if (int rc_ = context_ready(c)) return rc_;
    FGC_CUDA(cudaSetDevice(c->device));
    unsigned char* base = nullptr;
    int rc = noalloc_scratch(c->device, &base);
    if (rc) return rc;
    rc = apply_pending_clears(c);
    if (rc) return rc;
    unsigned long long* lohi = (unsigned long long*)base;
    uint16_t* gray = (uint16_t*)(base + 256);
    // lo starts at the largest key, hi at the smallest (atomicMin / atomicMax)
    FGC_CUDA(cudaMemsetAsync(lohi, 0xFF, sizeof(unsigned long long), c->stream));
    FGC_CUDA(cudaMemsetAsync(lohi + 1, 0x00, sizeof(unsigned long long), c->stream));
    int grid = grid_for((uint64_t)c->N, 256, c->sms * 8);
    depth_minmax_kernel<<<grid, 256, 0, c->stream>>>(c->depth.p, (uint64_t)c->N, lohi);
    depth_image_kernel<<<grid, 256, 0, c->stream>>>(c->depth.p, (uint64_t)c->N, lohi, gray);
    FGC_CUDA(cudaGetLastError());
    FGC_CUDA(cudaMemcpyAsync(gray16, gray, (size_t)c->N * 2, cudaMemcpyDeviceToHost, c->stream));
    FGC_CUDA(cudaStreamSynchronize(c->stream));
    return FGC_OK;
}
