// fgc_pass.cu -- the pass engine of libfauxglcuda: plans and issues passes
// (any number of draws rendered with one launch per pipeline stage) and
// reads their results back.
//
// A pass, no host wait inside:
//   table upload              item views + lookup starts (pinned -> device)
//   vertex_kernel             per draw, per unique position
//   setup_count_kernel        draw by draw, triangles then lines: culling and
//                             clipping decisions, per-tile sums; lists the
//                             clipped triangles
//   setup_scan_kernel         one block: the tile prefix, the pass totals
//   setup_kernel              the ordered allocation across the pass (slots
//                             and work items), clipped lines listed
//   setup_emit_kernel         the work items' raster primitives and each draw's
//                             primitive range
//   on a second stream: clip_poly / clip_vert_kernel (from the count kernel
//   on), clip_piece / clip_lines_kernel (from the list writer on), joined
//   before binning
//   bin_count / scan_u32 / bin_scatter   per-draw band bins, one scan
//   scan_u32 / row_starts_kernel         (draws with tall primitives)
//   raster_kernel             persistent CTAs over the pass's (draw, band)
//                             queue
//   result copy               status, counters, per-draw RasterizeInfo
// A kernel that finds a buffer too small sets a status bit; the raster stage
// then leaves every framebuffer of the pass untouched, later passes of the
// same submission skip theirs, and the host re-issues from the first failed
// pass with the sizes the device measured.
#include "fgc_host.cuh"

namespace fgc {

std::atomic<uint32_t> g_lookback_spin_limit{kSpinLimit};
std::atomic<uint32_t> g_lookback_withhold{0xFFFFFFFFu};

namespace {

constexpr size_t kHeaderBytes = 80;

struct PassHeader {
    unsigned int status;  // submission-wide status word
    unsigned int pad[3];
    PassCounters c;
};
static_assert(sizeof(PassHeader) == kHeaderBytes, "pass header layout");

size_t align16(size_t x) { return (x + 15) & ~(size_t)15; }

// Device table of a submission (sized for its largest pass):
//   [header][ItemOut x nmax][ItemView x nmax][4 lookup arrays of nmax + 1]
struct TableLayout {
    uint32_t nmax = 0;
    size_t iout = 0, views = 0, starts = 0, total = 0;
    size_t in_bytes() const { return total - views; }        // uploaded per pass
    size_t out_bytes(uint32_t n) const { return iout + (size_t)n * sizeof(ItemOut); }
};

TableLayout table_layout(uint32_t nmax) {
    TableLayout t;
    t.nmax = nmax;
    t.iout = kHeaderBytes;
    t.views = align16(t.iout + (size_t)nmax * sizeof(ItemOut));
    t.starts = t.views + (size_t)nmax * sizeof(ItemView);
    t.total = align16(t.starts + 4 * sizeof(uint32_t) * ((size_t)nmax + 1));
    return t;
}

struct PassPlan {
    std::vector<uint32_t> items;  // indices into the submission
    std::vector<ItemView> views;
    std::vector<uint32_t> vtile, stile, blk, band;
    uint32_t vtiles = 0, stiles = 0, nblk = 0, nbands = 0, max_nbands = 0;
    uint64_t nmat = 0, nvert = 0, nlines = 0, prim_base = 0;
    int per_max = 1;
    bool any_tri = false, any_line = false, debug_shaded = false;
    int32_t Lmax = 1, band_rows = 1, Rmax = 1;
    int precision = FGC_PRECISION_PLAIN;
    int F = 0;
    int su = kSpanUnitsMin;
    size_t smem = 0;
    int bin_warps = 1;
    uint32_t scan_tiles = 1;
    bool row_table = false;      // some draw uses the row-start table
    uint64_t work_items = 0;     // setup work items at most (emitting triangles, wireframe edges, lines)
};

constexpr double kRowTablePixelsPerElement = 8.0;

uint64_t ceil_div(uint64_t a, uint64_t b) { return (a + b - 1) / b; }

// Draws go to the current pass until one repeats a target context (its
// draws must run in order) or changes precision (one raster variant per
// launch).
std::vector<std::vector<uint32_t>> split_passes(const std::vector<PassItem>& items) {
    std::vector<std::vector<uint32_t>> out;
    std::vector<const fgc_context*> seen;
    int prec = -1;
    for (uint32_t i = 0; i < (uint32_t)items.size(); i++) {
        const PassItem& it = items[i];
        bool fresh = out.empty() || it.sv.precision != prec ||
                     std::find(seen.begin(), seen.end(), it.ctx) != seen.end();
        if (fresh) {
            out.emplace_back();
            seen.clear();
            prec = it.sv.precision;
        }
        out.back().push_back(i);
        seen.push_back(it.ctx);
    }
    return out;
}

int fit_fragments(const DevLimits& D, const PassTuning& T, int precision, int32_t Lmax, int& F, int& su,
                  size_t& smem) {
    const int stat = D.raster_static[precision == FGC_PRECISION_MIXED ? 1 : 0];
    const long two_cta = (long)D.smem_per_sm / 2 - D.smem_reserved_per_block - stat;
    const long one_cta = (long)D.smem_per_block_optin - stat;
    F = std::max(256, std::min(T.frag_cap, 4096));
    // the larger span arrays first: they also hold the warp queues of the
    // narrow walk, which needs one 32-entry queue per warp (kSpanUnitsMax =
    // the CTA's threads) and is worth more than a larger fragment buffer
    su = kSpanUnitsMax;
    smem = raster_smem_bytes(Lmax, F, kRasterThreads, su);
    // two CTAs per SM (the register budget allows two) when a smaller
    // fragment buffer makes them fit
    while ((long)smem > two_cta && F > 512) {
        F -= 128;
        smem = raster_smem_bytes(Lmax, F, kRasterThreads, su);
    }
    while ((long)smem > one_cta && F > 256) {
        F /= 2;
        smem = raster_smem_bytes(Lmax, F, kRasterThreads, su);
    }
    if ((long)smem > one_cta) {
        // the smaller span arrays (narrow rows then walk thread by thread)
        su = kSpanUnitsMin;
        smem = raster_smem_bytes(Lmax, F, kRasterThreads, su);
    }
    if ((long)smem > one_cta) return fail(FGC_ERR_UNSUPPORTED, "frame too wide for the band rasteriser");
    return FGC_OK;
}

int plan_pass(const Submission& sub, const std::vector<uint32_t>& idx, const DevLimits& D, const PassTuning& T,
              PassPlan& P) {
    const uint32_t n = (uint32_t)idx.size();
    P.items = idx;
    P.views.resize(n);
    P.vtile.assign(n + 1, 0);
    P.stile.assign(n + 1, 0);
    P.blk.assign(n + 1, 0);
    P.band.assign(n + 1, 0);
    P.precision = sub.items[idx[0]].sv.precision;
    for (uint32_t j = 0; j < n; j++) {
        const PassItem& it = sub.items[idx[j]];
        const fgc_context* c = it.ctx;
        ItemView& v = P.views[j];
        memset(&v, 0, sizeof(v));
        v.mesh = it.mesh->view();
        v.st = it.sv;
        v.sh = it.shv;
        v.tri_first = it.tf;
        v.tri_count = it.tc;
        v.line_first = it.lf;
        v.line_count = it.lc;
        v.w2 = (double)c->W / 2;
        v.h2 = (double)c->H / 2;
        v.W = c->W;
        v.H = c->H;
        v.N = c->N;
        int64_t R = std::max<int64_t>(1, T.band_pixels / c->W);
        R = std::min<int64_t>(R, kBandRowsMax);
        R = std::min<int64_t>(R, c->H);
        if (R * c->W > 65535) return fail(FGC_ERR_UNSUPPORTED, "frame width above 65535 pixels is not supported");
        v.R = (int32_t)R;
        v.L = (int32_t)(R * c->W);
        v.nbands = (uint32_t)ceil_div((uint64_t)c->H, (uint64_t)R);
        if (v.nbands > (uint32_t)kMaxBands) return fail(FGC_ERR_UNSUPPORTED, "frame has too many bands");
        const int per = it.sv.wireframe ? 6 : 1;
        const uint64_t prims = it.tc * per + it.lc * 2;
        v.nblk = (uint32_t)std::min<uint64_t>(std::max<uint64_t>(1, ceil_div(prims, T.prims_per_bin_block)),
                                              (uint64_t)2 * D.sms);
        const bool draws = it.tc > 0 || it.lc > 0;
        const uint32_t vt = draws ? (uint32_t)ceil_div(it.mesh->nuniq, kVertexTile) : 0;
        v.ntri_tiles = (uint32_t)ceil_div(it.tc, kSetupTile * kSetupPer);
        v.nline_tiles = (uint32_t)ceil_div(it.lc, kSetupTile * kSetupPer);
        const uint32_t st = std::max<uint32_t>(1, v.ntri_tiles + v.nline_tiles);
        v.vtile0 = P.vtiles;
        v.stile0 = P.stiles;
        v.blk0 = P.nblk;
        v.band0 = P.nbands;
        v.mat0 = P.nmat;
        v.vbase = P.nvert;
        P.vtile[j] = P.vtiles;
        P.stile[j] = P.stiles;
        P.blk[j] = P.nblk;
        P.band[j] = P.nbands;
        P.vtiles += vt;
        P.stiles += st;
        P.nblk += v.nblk;
        P.nbands += v.nbands;
        P.nmat += (uint64_t)v.nbands * v.nblk;
        P.nvert += draws ? it.mesh->nuniq : 0;
        P.nlines += it.lc;
        P.prim_base += prims;
        P.work_items += it.tc * (it.sv.wireframe ? 3 : 1) + it.lc;
        P.max_nbands = std::max(P.max_nbands, v.nbands);
        P.per_max = std::max(P.per_max, per);
        P.any_tri = P.any_tri || it.tc > 0;
        P.any_line = P.any_line || it.lc > 0;
        P.Lmax = std::max(P.Lmax, v.L);
        P.Rmax = std::max(P.Rmax, v.R);
        if (j == 0) P.band_rows = v.R;
        v.attr_mask = 0;
        if (it.shv.kind == FGC_SHADER_PHONG) {
            v.attr_mask |= kAttrPos | kAttrNrm;
            if (it.shv.object_is_discard) v.attr_mask |= kAttrCol;
        }
        if (it.shv.has_texture || it.shv.kind == FGC_SHADER_TEXTURE) v.attr_mask |= kAttrTex;
        // the row-start table pays where primitives are a few rows tall or
        // more: frames with at least kRowTablePixelsPerElement pixels per
        // drawn element (1080p of a 1.3 M-triangle mesh is below it)
        v.row_table = ((double)c->W * c->H >= kRowTablePixelsPerElement * (double)std::max<uint64_t>(it.tc + it.lc, 1))
                          ? 1 : 0;
        P.row_table = P.row_table || v.row_table;
        v.clear_color_pending = it.clear_color;
        v.clear_depth_pending = it.clear_depth;
        v.clear_color = it.clear_color_value;
        v.clear_depth = it.clear_depth_value;
        v.color = c->color.p;
        v.depth = c->depth.p;
        v.winner = (c->debug & FGC_DEBUG_WINNER) ? c->winner.p : nullptr;
        v.shaded = (c->debug & FGC_DEBUG_SHADED_COLOR) ? c->shaded.p : nullptr;
        if (v.shaded) P.debug_shaded = true;
    }
    P.vtile[n] = P.vtiles;
    P.stile[n] = P.stiles;
    P.blk[n] = P.nblk;
    P.band[n] = P.nbands;
    if (P.nmat >= 0xFFFFFFFFull) return fail(FGC_ERR_UNSUPPORTED, "pass too large for its bin matrix");
    P.scan_tiles = (uint32_t)ceil_div(P.nmat, 2048);
    int rc = fit_fragments(D, T, P.precision, P.Lmax, P.F, P.su, P.smem);
    if (rc) return rc;
    const int warps = (int)std::min<int64_t>(8, (96 * 1024) / ((int64_t)P.max_nbands * 4));
    if (warps < 1) return fail(FGC_ERR_UNSUPPORTED, "frame has too many bands for binning");
    P.bin_warps = warps;
    return FGC_OK;
}

uint64_t prim_capacity(const PassPlan& P, uint32_t clip_cap) {
    return P.prim_base + (uint64_t)clip_cap * (uint64_t)(6 * P.per_max) + 1;
}

void mark(std::vector<cudaEvent_t>* evs, cudaStream_t stream) {
    if (!evs) return;
    cudaEvent_t e = nullptr;
    if (cudaEventCreate(&e) != cudaSuccess) return;
    cudaEventRecord(e, stream);
    evs->push_back(e);
}

void destroy_events(std::vector<cudaEvent_t>& evs) {
    for (cudaEvent_t e : evs) cudaEventDestroy(e);
    evs.clear();
}

}  // namespace

void Submission::reset() {
    infos.assign(items.size(), fgc_rasterize_info{0, 0});
    stats = fgc_stats{};
    passes.clear();
    for (auto& v : events) destroy_events(v);
    events.clear();
}

Submission::~Submission() {
    for (auto& v : events) destroy_events(v);
}

namespace {

// Plan every pass of a submission and grow the scratch to the largest.
// Buffers change size only here, before any pass of the submission is
// issued (passes issued earlier on the stream may still be using them).
int plan_submission(PassScratch& S, const DevLimits& D, const PassTuning& T, const Submission& sub,
                    std::vector<std::vector<uint32_t>>& groups, std::vector<PassPlan>& plans, uint32_t& nmax,
                    uint32_t& need_grid) {
    groups = split_passes(sub.items);
    plans.assign(groups.size(), PassPlan{});
    nmax = 1;
    for (size_t g = 0; g < groups.size(); g++) {
        int rc = plan_pass(sub, groups[g], D, T, plans[g]);
        if (rc) return rc;
        nmax = std::max<uint32_t>(nmax, (uint32_t)groups[g].size());
    }
    const TableLayout TL = table_layout(nmax);
    uint64_t need_prims = 0, need_vert = 1, need_lines = 1, need_mat = 1, need_tiles = 4, need_work = 1;
    bool need_dbg = false;
    need_grid = 1;
    for (const PassPlan& P : plans) {
        need_prims = std::max(need_prims, prim_capacity(P, S.clip_cap));
        need_vert = std::max(need_vert, P.nvert + 1);
        need_lines = std::max(need_lines, P.nlines + 1);
        need_mat = std::max(need_mat, P.nmat);
        need_tiles = std::max<uint64_t>(need_tiles, (uint64_t)P.stiles + P.scan_tiles + 4 +
                                                        ceil_div(prim_capacity(P, S.clip_cap), 2048) + 2);
        need_dbg = need_dbg || P.debug_shaded;
        need_grid = std::max<uint32_t>(need_grid, std::min<uint32_t>(2 * D.sms, P.nbands));
        need_work = std::max<uint64_t>(need_work, P.work_items);
    }
    // setup's ordered allocation carries the slot and work prefixes in 31
    // bits each
    if (need_prims >= (1ull << 31) || need_work >= (1ull << 31))
        return fail(FGC_ERR_UNSUPPORTED, "more than 2^31 primitives in one pass");
    if (S.bin_cap == 0) S.bin_cap = std::max<uint64_t>(2 * need_prims, 1 << 16);
    FGC_CUDA(S.vclip.ensure(need_vert));
    FGC_CUDA(S.vndc.ensure(need_vert));
    FGC_CUDA(S.vscr.ensure(need_vert));
    FGC_CUDA(S.vout.ensure(need_vert));
    FGC_CUDA(S.prims.ensure(need_prims));
    FGC_CUDA(S.pbox.ensure(need_prims));
    FGC_CUDA(S.rf.ensure(need_prims));
    FGC_CUDA(S.pspan.ensure(need_prims));
    FGC_CUDA(S.clip_list.ensure(S.clip_cap));
    FGC_CUDA(S.pool.ensure((size_t)S.clip_cap * 21));
    FGC_CUDA(S.pool32.ensure((size_t)S.clip_cap * 21));
    FGC_CUDA(S.cpoly.ensure(S.clip_cap));
    FGC_CUDA(S.cvert.ensure((size_t)S.clip_cap * kClipPoly));
    FGC_CUDA(S.lclip_list.ensure(need_lines));
    FGC_CUDA(S.mat.ensure(need_mat));
    FGC_CUDA(S.off.ensure(need_mat));
    FGC_CUDA(S.bins.ensure(S.bin_cap));
    FGC_CUDA(S.pnb.ensure(need_prims));
    FGC_CUDA(S.prs.ensure(need_prims));
    FGC_CUDA(S.rstart.ensure(3 * S.bin_cap));
    FGC_CUDA(S.tiles.ensure(need_tiles));
    FGC_CUDA(S.work.ensure(need_work));
    uint64_t need_stiles = 1;
    for (const PassPlan& P : plans) need_stiles = std::max<uint64_t>(need_stiles, P.stiles);
    FGC_CUDA(S.smeta.ensure(need_stiles * kSetupTile * kSetupPer));
    FGC_CUDA(S.cidx.ensure(need_stiles * kSetupTile * kSetupPer));
    FGC_CUDA(S.tsum.ensure(need_stiles));
    FGC_CUDA(S.table.ensure(TL.total));
    int dev = 0;
    FGC_CUDA(cudaGetDevice(&dev));
    if (!S.side || S.side_device != dev) {
        if (S.ev_fork) cudaEventDestroy(S.ev_fork);
        if (S.ev_clip) cudaEventDestroy(S.ev_clip);
        if (S.ev_join) cudaEventDestroy(S.ev_join);
        if (S.side) cudaStreamDestroy(S.side);
        S.side = nullptr;
        S.ev_fork = S.ev_clip = S.ev_join = nullptr;
        // the highest priority: the clip kernels' few blocks are placed
        // before the main stream's fill the SMs
        int least = 0, greatest = 0;
        FGC_CUDA(cudaDeviceGetStreamPriorityRange(&least, &greatest));
        FGC_CUDA(cudaStreamCreateWithPriority(&S.side, cudaStreamNonBlocking, greatest));
        FGC_CUDA(cudaEventCreateWithFlags(&S.ev_fork, cudaEventDisableTiming));
        FGC_CUDA(cudaEventCreateWithFlags(&S.ev_clip, cudaEventDisableTiming));
        FGC_CUDA(cudaEventCreateWithFlags(&S.ev_join, cudaEventDisableTiming));
        S.side_device = dev;
    }
    FGC_CUDA(S.host_in.ensure(TL.in_bytes() * plans.size()));
    FGC_CUDA(S.host_out.ensure(TL.out_bytes(nmax) * plans.size()));
    if (need_dbg) {
        size_t most = 0;
        for (const PassPlan& P : plans) most = std::max(most, (size_t)need_grid * P.F * 4);
        FGC_CUDA(S.dbg.ensure(most));
    }
    return FGC_OK;
}

}  // namespace

int prepare_submission(PassScratch& S, const DevLimits& D, const PassTuning& T, const Submission& sub) {
    std::vector<std::vector<uint32_t>> groups;
    std::vector<PassPlan> plans;
    uint32_t nmax = 1, need_grid = 1;
    return plan_submission(S, D, T, sub, groups, plans, nmax, need_grid);
}

int issue_submission(PassScratch& S, cudaStream_t stream, const DevLimits& D, const PassTuning& T, Submission& sub,
                     size_t first_pass) {
    if (sub.items.empty()) return FGC_OK;
    std::vector<std::vector<uint32_t>> groups;
    std::vector<PassPlan> plans;
    uint32_t nmax = 1, need_grid = 1;
    int prc = plan_submission(S, D, T, sub, groups, plans, nmax, need_grid);
    if (prc) return prc;
    if (first_pass == 0) {
        sub.passes.assign(groups.size(), PassRecord{});
        for (size_t g = 0; g < groups.size(); g++) sub.passes[g].items = groups[g];
        for (auto& v : sub.events) destroy_events(v);
        sub.events.assign(sub.timing ? groups.size() : 0, {});
    }
    const TableLayout TL = table_layout(nmax);
    unsigned char* dtab = S.table.p;
    PassHeader* dhdr = (PassHeader*)dtab;
    // the submission's status starts clear (a retry re-issues the failed
    // passes with a clear status: the earlier ones succeeded)
    FGC_CUDA(cudaMemsetAsync(&dhdr->status, 0, sizeof(unsigned int), stream));

    for (size_t g = first_pass; g < plans.size(); g++) {
        const PassPlan& P = plans[g];
        PassRecord& rec = sub.passes[g];
        const uint32_t n = (uint32_t)P.views.size();
        rec.in_off = g * TL.in_bytes();
        rec.out_off = g * TL.out_bytes(nmax);
        rec.nbands = P.nbands;
        rec.band_rows = P.band_rows;
        rec.launches = 0;
        std::vector<cudaEvent_t>* evs = nullptr;
        if (sub.timing && g < sub.events.size()) {
            destroy_events(sub.events[g]);
            evs = &sub.events[g];
        }

        // ---- table upload
        unsigned char* hin = S.host_in.p + rec.in_off;
        memcpy(hin, P.views.data(), (size_t)n * sizeof(ItemView));
        uint32_t* hst = (uint32_t*)(hin + (TL.starts - TL.views));
        memcpy(hst, P.vtile.data(), (n + 1) * 4);
        memcpy(hst + (nmax + 1), P.stile.data(), (n + 1) * 4);
        memcpy(hst + 2 * (nmax + 1), P.blk.data(), (n + 1) * 4);
        memcpy(hst + 3 * (nmax + 1), P.band.data(), (n + 1) * 4);
        FGC_CUDA(cudaMemcpyAsync(dtab + TL.views, hin, TL.in_bytes(), cudaMemcpyHostToDevice, stream));
        FGC_CUDA(cudaMemsetAsync(&dhdr->c, 0, TL.out_bytes(n) - offsetof(PassHeader, c), stream));
        const uint64_t prim_cap0 = prim_capacity(P, S.clip_cap);
        const uint64_t rs_tiles = ceil_div(prim_cap0, 2048);
        const uint64_t ntiles = (uint64_t)P.stiles + P.scan_tiles + 4 + rs_tiles + 2;
        FGC_CUDA(cudaMemsetAsync(S.tiles.p, 0, ntiles * 8, stream));

        const ItemView* items = (const ItemView*)(dtab + TL.views);
        const uint32_t* dst = (const uint32_t*)(dtab + TL.starts);
        ItemStarts starts{dst, dst + (nmax + 1), dst + 2 * (nmax + 1), dst + 3 * (nmax + 1)};
        ItemOut* iout = (ItemOut*)(dtab + TL.iout);
        PassCounters* dc = &dhdr->c;
        unsigned int* status = &dhdr->status;
        unsigned long long* t_setup = S.tiles.p;
        unsigned long long* t_scan = t_setup + P.stiles + 2;
        unsigned long long* t_rscan = t_scan + P.scan_tiles + 2;
        const uint64_t prim_cap = prim_capacity(P, S.clip_cap);

        mark(evs, stream);
        if (P.vtiles > 0) {
            VertexParams vp;
            vp.items = items;
            vp.starts = starts;
            vp.nitems = n;
            vp.ntiles = P.vtiles;
            vp.vclip = S.vclip.p;
            vp.vndc = S.vndc.p;
            vp.vscr = S.vscr.p;
            vp.vout = S.vout.p;
            vertex_kernel<<<std::min<uint32_t>(P.vtiles, 16 * D.sms), kVertexTile, 0, stream>>>(vp);
            FGC_CUDA(cudaGetLastError());
            rec.launches++;
        }
        mark(evs, stream);

        GeomParams gp;
        memset(&gp, 0, sizeof(gp));
        gp.items = items;
        gp.starts = starts;
        gp.nitems = n;
        gp.ntiles = P.stiles;
        gp.iout = iout;
        gp.vclip = S.vclip.p;
        gp.vndc = S.vndc.p;
        gp.vscr = S.vscr.p;
        gp.vout = S.vout.p;
        gp.prims = S.prims.p;
        gp.pbox = S.pbox.p;
        gp.rf = S.rf.p;
        gp.pspan = S.pspan.p;
        gp.prim_cap = prim_cap;
        gp.clip_list = S.clip_list.p;
        gp.clip_cap = S.clip_cap;
        gp.clip_count = &dc->clip_count;
        gp.lclip_list = S.lclip_list.p;
        gp.lclip_count = &dc->lclip_count;
        gp.pool = S.pool.p;
        gp.pool32 = S.pool32.p;
        gp.cpoly = S.cpoly.p;
        gp.cvert = S.cvert.p;
        gp.prim_total = &dc->prim_total;
        gp.lb = draw_lookback(t_setup, &dc->tick_setup, status, nullptr);  // setup_kernel writes the totals
        gp.status = status;
        gp.work = S.work.p;
        gp.work_cap = S.work.cap;
        gp.work_total = &dc->work_total;
        gp.smeta = S.smeta.p;
        gp.cidx = S.cidx.p;
        gp.tsum = S.tsum.p;
        // Clipped triangles: the count kernel lists them, and on the side
        // stream one kernel builds their polygons and one the polygons'
        // vertices while the scan and the list writer run; a third makes the
        // fan pieces beside the emission (they need the slots the list writer
        // assigns). Clipped lines are listed by the list writer and clipped
        // beside the emission as well.
        const bool clips = P.any_tri || P.any_line;
        setup_count_kernel<<<P.stiles, kSetupTile, 0, stream>>>(gp);
        if (P.any_tri) {
            FGC_CUDA(cudaEventRecord(S.ev_fork, stream));
            FGC_CUDA(cudaStreamWaitEvent(S.side, S.ev_fork, 0));
            // one warp per block: a few thousand clip entries still spread
            // over every SM's FP64 pipes
            clip_poly_kernel<<<grid_for(S.clip_cap, 32, D.sms * 8), 32, 0, S.side>>>(gp);
            clip_vert_kernel<<<grid_for((uint64_t)S.clip_cap * kClipPoly, 64, D.sms * 8), 64, 0, S.side>>>(gp);
            FGC_CUDA(cudaGetLastError());
            rec.launches += 2;
        }
        setup_scan_kernel<<<1, 1024, 0, stream>>>(gp);
        setup_kernel<<<P.stiles, kSetupTile, 0, stream>>>(gp);
        FGC_CUDA(cudaGetLastError());
        rec.launches += 3;
        if (clips) {
            FGC_CUDA(cudaEventRecord(S.ev_clip, stream));
            FGC_CUDA(cudaStreamWaitEvent(S.side, S.ev_clip, 0));
            if (P.any_tri) {
                clip_piece_kernel<<<grid_for((uint64_t)S.clip_cap * 7, 64, D.sms * 8), 64, 0, S.side>>>(gp);
                rec.launches++;
            }
            if (P.any_line) {
                clip_lines_kernel<<<grid_for(P.nlines, 128, D.sms * 4), 128, 0, S.side>>>(gp);
                rec.launches++;
            }
            FGC_CUDA(cudaGetLastError());
            FGC_CUDA(cudaEventRecord(S.ev_join, S.side));
        }
        setup_emit_kernel<<<grid_for(P.work_items, 256, D.sms * 16), 256, 0, stream>>>(gp);
        FGC_CUDA(cudaGetLastError());
        rec.launches++;
        if (clips) FGC_CUDA(cudaStreamWaitEvent(stream, S.ev_join, 0));
        mark(evs, stream);
        mark(evs, stream);  // the stage the primitive ranges had (now part of the emission)

        BinParams bp;
        bp.items = items;
        bp.starts = starts;
        bp.nitems = n;
        bp.iout = iout;
        bp.pbox = S.pbox.p;
        bp.mat = S.mat.p;
        bp.off = S.off.p;
        bp.pair_total = &dc->pair_total;
        bp.bins = S.bins.p;
        bp.bin_cap = S.bin_cap;
        bp.status = status;
        bp.pnb = S.pnb.p;
        const size_t hist_smem = (size_t)P.max_nbands * 4;
        if (hist_smem > 48 * 1024)
            FGC_CUDA(cudaFuncSetAttribute(bin_count_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)hist_smem));
        bin_count_kernel<<<P.nblk, 256, hist_smem, stream>>>(bp);
        FGC_CUDA(cudaGetLastError());
        ScanParams sp;
        sp.n_dev = nullptr;
        sp.in = S.mat.p;
        sp.out = S.off.p;
        sp.n = P.nmat;
        sp.lb = draw_lookback(t_scan, &dc->tick_scan, status, &dc->pair_total);
        scan_u32_kernel<<<P.scan_tiles, 256, 0, stream>>>(sp);
        FGC_CUDA(cudaGetLastError());
        const size_t scat_smem = (size_t)P.bin_warps * P.max_nbands * 4;
        if (scat_smem > 48 * 1024)
            FGC_CUDA(cudaFuncSetAttribute(bin_scatter_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)scat_smem));
        bin_scatter_kernel<<<P.nblk, P.bin_warps * 32, scat_smem, stream>>>(bp, P.bin_warps);
        FGC_CUDA(cudaGetLastError());
        // row starts per (primitive, band): slots from a scan of the
        // primitives' band counts
        if (P.row_table) {
            ScanParams rsp;
            rsp.in = S.pnb.p;
            rsp.out = S.prs.p;
            rsp.n = prim_cap0;
            rsp.lb = draw_lookback(t_rscan, &dc->tick_rscan, status, &dc->reserved);
            rsp.n_dev = &dc->prim_total;  // bin_count wrote the band counts of these
            scan_u32_kernel<<<(unsigned)rs_tiles, 256, 0, stream>>>(rsp);
            FGC_CUDA(cudaGetLastError());
            RowStartParams rq;
            rq.iout = iout;
            rq.items = items;
            rq.nitems = n;
            rq.prims = S.prims.p;
            rq.pbox = S.pbox.p;
            rq.pnb = S.pnb.p;
            rq.prs = S.prs.p;
            rq.prim_total = &dc->prim_total;
            rq.cap = S.bin_cap;
            rq.rstart = S.rstart.p;
            rq.status = status;
            row_starts_kernel<<<grid_for(prim_cap0, 256, D.sms * 8), 256, 0, stream>>>(rq);
            FGC_CUDA(cudaGetLastError());
            rec.launches += 2;
        }
        rec.launches += 3;
        mark(evs, stream);

        RasterParams rp;
        memset(&rp, 0, sizeof(rp));
        rp.items = items;
        rp.starts = starts;
        rp.nitems = n;
        rp.nbands = P.nbands;
        rp.iout = iout;
        rp.prims = S.prims.p;
        rp.pbox = S.pbox.p;
        rp.pspan = S.pspan.p;
        rp.bins = S.bins.p;
        rp.off = S.off.p;
        rp.nmat = P.nmat;
        rp.pair_total = &dc->pair_total;
        rp.F = P.F;
        rp.Lmax = P.Lmax;
        rp.win = std::max(1, std::min(T.window, 256));
        rp.su = P.su;
        rp.pool = S.pool.p;
        rp.pool32 = S.pool32.p;
        rp.rf = S.rf.p;
        rp.prs = S.prs.p;
        rp.rstart = S.rstart.p;
        rp.band_counter = &dc->band_counter;
        rp.status = status;
        rp.dbg = P.debug_shaded ? S.dbg.p : nullptr;
        const void* kfn = raster_kernel_ptr(P.precision);
        FGC_CUDA(cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)P.smem));
        int per_sm = 0;
        FGC_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kfn, kRasterThreads, P.smem));
        if (per_sm < 1) return fail(FGC_ERR_UNSUPPORTED, "raster kernel does not fit on an SM");
        int rgrid = (int)std::min<uint64_t>((uint64_t)per_sm * D.sms, P.nbands);
        if (P.debug_shaded) rgrid = std::min<int>(rgrid, (int)need_grid);
        FGC_CUDA(launch_raster(P.precision, rgrid, kRasterThreads, P.smem, stream, rp));
        rec.launches++;
        mark(evs, stream);

        // ---- results: status, counters, per-draw outputs
        FGC_CUDA(cudaMemcpyAsync(S.host_out.p + rec.out_off, dtab, TL.out_bytes(n), cudaMemcpyDeviceToHost, stream));
    }
    return FGC_OK;
}

int collect_submission(PassScratch& S, Submission& sub, size_t from, size_t* retry_from) {
    *retry_from = sub.passes.size();
    fgc_stats& st = sub.stats;
    const unsigned int overflow = ST_CLIP_OVERFLOW | ST_POOL_OVERFLOW | ST_BIN_OVERFLOW;
    size_t first_bad = sub.passes.size();
    uint32_t clip_need = 0;
    uint64_t pair_need = 0;
    for (size_t g = from; g < sub.passes.size(); g++) {
        const PassRecord& rec = sub.passes[g];
        const PassHeader* h = (const PassHeader*)(S.host_out.p + rec.out_off);
        if (h->status & ST_RASTER_INTERNAL)
            return fail(FGC_ERR_DEVICE_LIMIT, "the raster stage detected an internal inconsistency");
        if (h->status & ST_LOOKBACK_TIMEOUT)
            return fail(FGC_ERR_DEVICE_LIMIT, "a look-back wait in a scan of the binning stage timed out");
        if ((h->status & overflow) && first_bad == sub.passes.size()) first_bad = g;
        if (first_bad <= g) {
            clip_need = std::max(clip_need, h->c.clip_count);
            pair_need = std::max<uint64_t>(pair_need, h->c.pair_total);
            continue;
        }
        // a pass that succeeded: its draws' results
        const ItemOut* io = (const ItemOut*)((const unsigned char*)h + kHeaderBytes);
        for (size_t j = 0; j < rec.items.size(); j++) {
            fgc_rasterize_info& info = sub.infos[rec.items[j]];
            info.total_pixels = io[j].info[0];
            info.updated_pixels = io[j].info[1];
            st.covered_pixels += io[j].info[0];
            st.updated_pixels += io[j].info[1];
            st.visited_pixels += io[j].info[2];
            st.shaded_fragments += io[j].info[3];
        }
        st.clipped += (uint64_t)h->c.clip_count + h->c.lclip_count;
        st.primitives += h->c.prim_total;
        st.bin_entries += h->c.pair_total;
        st.bands += rec.nbands;
        if (g == 0) st.band_rows = (uint32_t)rec.band_rows;
        if (sub.timing && g < sub.events.size()) {
            const std::vector<cudaEvent_t>& evs = sub.events[g];
            for (int i = 0; i + 1 < (int)evs.size() && i < FGC_STAGE_COUNT; i++) {
                float ms = 0;
                cudaEventElapsedTime(&ms, evs[i], evs[i + 1]);
                st.stage_ms[i] += ms;
            }
        }
    }
    st.attempts++;
    for (size_t g = from; g < sub.passes.size(); g++) st.kernel_launches += sub.passes[g].launches;
    if (first_bad == sub.passes.size()) return FGC_OK;
    const unsigned int bad = ((const PassHeader*)(S.host_out.p + sub.passes[first_bad].out_off))->status;
    if (bad & (ST_CLIP_OVERFLOW | ST_POOL_OVERFLOW))
        S.clip_cap = std::max<uint32_t>(S.clip_cap * 2, clip_need + clip_need / 4 + 64);
    if (bad & ST_BIN_OVERFLOW) S.bin_cap = std::max<uint64_t>(S.bin_cap, pair_need + pair_need / 4 + 1024);
    *retry_from = first_bad;
    return FGC_OK;
}

int finish_submission(PassScratch& S, cudaStream_t stream, const DevLimits& D, const PassTuning& T, Submission& sub,
                      size_t from) {
    for (int attempt = 0; attempt < 8; attempt++) {
        FGC_CUDA(cudaStreamSynchronize(stream));
        size_t next = 0;
        int rc = collect_submission(S, sub, from, &next);
        if (rc) return rc;
        if (next == sub.passes.size()) return FGC_OK;
        from = next;
        rc = issue_submission(S, stream, D, T, sub, from);
        if (rc) return rc;
    }
    return fail(FGC_ERR_DEVICE_LIMIT, "draw buffers kept overflowing");
}

int run_submission(PassScratch& S, cudaStream_t stream, const DevLimits& D, const PassTuning& T, Submission& sub) {
    sub.reset();
    int rc = issue_submission(S, stream, D, T, sub, 0);
    if (rc) return rc;
    return finish_submission(S, stream, D, T, sub, 0);
}

// ---------------------------------------------------------------------------
// Device limits (read once per device)
// ---------------------------------------------------------------------------
int dev_limits(int device, const DevLimits** out) {
    static std::mutex mu;
    static DevLimits table[64];
    if (device < 0 || device >= 64) return fail(FGC_ERR_UNSUPPORTED, "device ordinal out of range");
    std::lock_guard<std::mutex> lock(mu);
    DevLimits& D = table[device];
    if (D.device != device) {
        FGC_CUDA(cudaDeviceGetAttribute(&D.sms, cudaDevAttrMultiProcessorCount, device));
        FGC_CUDA(cudaDeviceGetAttribute(&D.smem_per_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, device));
        FGC_CUDA(cudaDeviceGetAttribute(&D.smem_per_block_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, device));
        FGC_CUDA(cudaDeviceGetAttribute(&D.smem_reserved_per_block, cudaDevAttrReservedSharedMemoryPerBlock, device));
        for (int p = 0; p < 2; p++) {
            cudaFuncAttributes fa;
            FGC_CUDA(cudaFuncGetAttributes(&fa, raster_kernel_ptr(p == 0 ? FGC_PRECISION_PLAIN : FGC_PRECISION_MIXED)));
            D.raster_static[p] = (int)fa.sharedSizeBytes;
        }
        D.device = device;
    }
    *out = &D;
    return FGC_OK;
}

}  // namespace fgc
