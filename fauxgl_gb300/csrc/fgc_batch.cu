// fgc_batch.cu -- batches: many independent draws (views of uneven size,
// each with its own mesh range, state, shader and target context) rendered
// by the pass engine with one launch per pipeline stage for all of them,
// asynchronously, optionally as a CUDA graph, with an autotuner for the
// pipeline's shapes. No counterpart in the reference: a batch gives every
// draw exactly the output of fgc_draw_triangles / fgc_draw_lines alone.
#include "fgc_host.cuh"

#include <chrono>
#include <new>

using namespace fgc;

struct fgc_batch {
    int device = 0;
    cudaStream_t stream = nullptr;
    cudaStream_t own_stream = nullptr;
    cudaEvent_t done = nullptr;
    PassScratch scratch;
    PassTuning tuning;
    bool use_graph = false;
    cudaGraphExec_t exec = nullptr;
    Submission sub;
    struct ReadBack {
        fgc_context* ctx;
        uint8_t* dst;
        int32_t scale;
        size_t ds_off;  // offset in ds (scaled read-backs)
    };
    std::vector<ReadBack> reads;
    DevBuf<uint32_t> ds;
    std::vector<fgc_context*> contexts;  // distinct targets of the submission in flight
    bool inflight = false;
    bool timing = false;
    fgc_stats stats = {};
    std::mutex mu;
};

namespace {

// Queue the read-backs of a submission (after its passes).
int enqueue_reads(fgc_batch* b) {
    const DevLimits* D = nullptr;
    int rc = dev_limits(b->device, &D);
    if (rc) return rc;
    for (const fgc_batch::ReadBack& r : b->reads) {
        const fgc_context* c = r.ctx;
        if (r.scale <= 1) {
            FGC_CUDA(cudaMemcpyAsync(r.dst, c->color.p, (size_t)c->N * 4, cudaMemcpyDeviceToHost, b->stream));
            continue;
        }
        const uint64_t n = (uint64_t)(c->W / r.scale) * (uint64_t)(c->H / r.scale);
        uint32_t* dst = b->ds.p + r.ds_off;
        downsample_kernel<<<grid_for(n, 256, D->sms * 8), 256, 0, b->stream>>>(c->color.p, c->W, c->H, r.scale, dst);
        FGC_CUDA(cudaGetLastError());
        FGC_CUDA(cudaMemcpyAsync(r.dst, dst, n * 4, cudaMemcpyDeviceToHost, b->stream));
    }
    return FGC_OK;
}

void release_contexts(fgc_batch* b) {
    for (fgc_context* c : b->contexts) {
        std::lock_guard<std::mutex> lock(c->mu);
        if (c->busy == b) c->busy = nullptr;
    }
    b->contexts.clear();
}

// Issue the submission in b->sub (passes from the first) and its read-backs.
int issue(fgc_batch* b) {
    const DevLimits* D = nullptr;
    int rc = dev_limits(b->device, &D);
    if (rc) return rc;
    rc = prepare_submission(b->scratch, *D, b->tuning, b->sub);
    if (rc) return rc;
    if (!b->use_graph) {
        rc = issue_submission(b->scratch, b->stream, *D, b->tuning, b->sub, 0);
        if (rc) return rc;
        rc = enqueue_reads(b);
        if (rc) return rc;
        FGC_CUDA(cudaEventRecord(b->done, b->stream));
        return FGC_OK;
    }
    // Capture the submission and replay it as one graph launch; an
    // executable graph from an earlier submission is updated in place when
    // the new one has the same shape, otherwise instantiated anew.
    FGC_CUDA(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
    rc = issue_submission(b->scratch, b->stream, *D, b->tuning, b->sub, 0);
    if (rc == FGC_OK) rc = enqueue_reads(b);
    cudaGraph_t g = nullptr;
    cudaError_t ce = cudaStreamEndCapture(b->stream, &g);
    if (rc) {
        if (g) cudaGraphDestroy(g);
        return rc;
    }
    if (ce != cudaSuccess) return fail(FGC_ERR_CUDA, std::string("cudaStreamEndCapture: ") + cudaGetErrorString(ce));
    if (b->exec) {
        cudaGraphExecUpdateResultInfo info;
        if (cudaGraphExecUpdate(b->exec, g, &info) != cudaSuccess) {
            cudaGetLastError();  // clear the update failure
            cudaGraphExecDestroy(b->exec);
            b->exec = nullptr;
        }
    }
    if (!b->exec) {
        ce = cudaGraphInstantiate(&b->exec, g, 0);
        if (ce != cudaSuccess) {
            cudaGraphDestroy(g);
            b->exec = nullptr;
            return fail(FGC_ERR_CUDA, std::string("cudaGraphInstantiate: ") + cudaGetErrorString(ce));
        }
    }
    cudaGraphDestroy(g);
    FGC_CUDA(cudaGraphLaunch(b->exec, b->stream));
    FGC_CUDA(cudaEventRecord(b->done, b->stream));
    return FGC_OK;
}

// Wait for the submission in flight, re-issue failed passes (and the
// read-backs after them) until every pass has succeeded.
int finish(fgc_batch* b) {
    const DevLimits* D = nullptr;
    int rc = dev_limits(b->device, &D);
    if (rc) return rc;
    size_t from = 0;
    for (int attempt = 0; attempt < 8; attempt++) {
        FGC_CUDA(cudaStreamSynchronize(b->stream));
        size_t next = 0;
        rc = collect_submission(b->scratch, b->sub, from, &next);
        if (rc) return rc;
        if (next == b->sub.passes.size()) return FGC_OK;
        from = next;
        // a pass overflowed: it and the passes after it left their targets
        // untouched; run them again with the sizes the device measured
        rc = issue_submission(b->scratch, b->stream, *D, b->tuning, b->sub, from);
        if (rc) return rc;
        rc = enqueue_reads(b);
        if (rc) return rc;
    }
    return fail(FGC_ERR_DEVICE_LIMIT, "draw buffers kept overflowing");
}

int submit(fgc_batch* b, const fgc_batch_item* items, uint64_t n) {
    if (b->inflight) return fail(FGC_ERR_BUSY, "the batch has a submission in flight (fgc_batch_wait first)");
    Submission& sub = b->sub;
    sub.items.clear();
    sub.items.resize(n);
    b->reads.clear();
    size_t ds_total = 0;
    for (uint64_t i = 0; i < n; i++) {
        const fgc_batch_item& it = items[i];
        if (!it.context || !it.mesh || !it.state || !it.shader) return fail(FGC_ERR_INVALID_ARGUMENT, "null field in a batch item");
        const fgc_context* c = it.context;
        const fgc_mesh* m = it.mesh;
        if (c->device != b->device || m->device != b->device)
            return fail(FGC_ERR_INVALID_ARGUMENT, "batch item on another device");
        if (it.shader->texture && it.shader->texture->device != b->device)
            return fail(FGC_ERR_INVALID_ARGUMENT, "texture is on another device");
        if (it.tri_first > m->ntri || it.tri_count > m->ntri - it.tri_first)
            return fail(FGC_ERR_INVALID_ARGUMENT, "triangle range out of bounds");
        if (it.line_first > m->nline || it.line_count > m->nline - it.line_first)
            return fail(FGC_ERR_INVALID_ARGUMENT, "line range out of bounds");
        PassItem& p = sub.items[i];
        int rc = fill_views(it.state, it.shader, p.sv, p.shv);
        if (rc) return rc;
        p.ctx = it.context;
        p.mesh = m;
        p.tf = it.tri_first;
        p.tc = it.tri_count;
        p.lf = it.line_first;
        p.lc = it.line_count;
        if (it.out_nrgba) {
            const int32_t s = it.out_scale < 1 ? 1 : it.out_scale;
            if (c->W % s != 0 || c->H % s != 0) return fail(FGC_ERR_INVALID_ARGUMENT, "out_scale must divide the frame");
            fgc_batch::ReadBack r{it.context, it.out_nrgba, s, ds_total};
            if (s > 1) ds_total += (size_t)(c->W / s) * (size_t)(c->H / s);
            b->reads.push_back(r);
        }
    }
    if (ds_total) FGC_CUDA(b->ds.ensure(ds_total));
    // claim the targets; the first draw on each takes its pending clears
    std::vector<fgc_context*> claimed;
    for (uint64_t i = 0; i < n; i++) {
        fgc_context* c = sub.items[i].ctx;
        if (std::find(claimed.begin(), claimed.end(), c) != claimed.end()) continue;
        std::lock_guard<std::mutex> lock(c->mu);
        int rc = context_ready(c);
        if (rc == FGC_OK) rc = ensure_debug(c);
        if (rc == FGC_OK && c->debug) {
            cudaError_t e = cudaStreamSynchronize(c->stream);  // debug buffers initialised
            if (e != cudaSuccess) rc = fail(FGC_ERR_CUDA, std::string("cudaStreamSynchronize: ") + cudaGetErrorString(e));
        }
        if (rc) {
            for (fgc_context* d : claimed) {
                std::lock_guard<std::mutex> l2(d->mu);
                d->busy = nullptr;
            }
            return rc;
        }
        c->busy = b;
        claimed.push_back(c);
    }
    for (uint64_t i = 0; i < n; i++) {
        PassItem& p = sub.items[i];
        fgc_context* c = p.ctx;
        p.clear_color = c->clear_color_pending;
        p.clear_depth = c->clear_depth_pending;
        p.clear_color_value = c->clear_color;
        p.clear_depth_value = c->clear_depth;
        c->clear_color_pending = false;
        c->clear_depth_pending = false;
    }
    b->contexts = claimed;
    sub.timing = b->timing && !b->use_graph;
    sub.reset();
    int rc = issue(b);
    if (rc) {
        release_contexts(b);
        return rc;
    }
    b->inflight = true;
    return FGC_OK;
}

int wait(fgc_batch* b, fgc_rasterize_info* infos) {
    if (!b->inflight) return fail(FGC_ERR_INVALID_ARGUMENT, "the batch has no submission in flight");
    int rc = finish(b);
    b->inflight = false;
    release_contexts(b);
    b->stats = b->sub.stats;
    for (const PassItem& p : b->sub.items) {
        b->stats.elements += p.tc + p.lc;
        if (p.tc > 0 || p.lc > 0) b->stats.unique_vertices += p.mesh->nuniq;
    }
    if (rc) return rc;
    if (infos)
        for (size_t i = 0; i < b->sub.infos.size(); i++) infos[i] = b->sub.infos[i];
    return FGC_OK;
}

}  // namespace

extern "C" {

int fgc_batch_create(fgc_batch** out) {
    if (!out) return fail(FGC_ERR_INVALID_ARGUMENT, "out is null");
    *out = nullptr;
    fgc_batch* b = new (std::nothrow) fgc_batch();
    if (!b) return fail(FGC_ERR_OUT_OF_MEMORY, "host allocation failed");
    cudaError_t e = cudaGetDevice(&b->device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&b->own_stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->done, cudaEventDisableTiming);
    if (e != cudaSuccess) {
        if (b->own_stream) cudaStreamDestroy(b->own_stream);
        delete b;
        return fail(FGC_ERR_CUDA, std::string("batch setup: ") + cudaGetErrorString(e));
    }
    b->stream = b->own_stream;
    *out = b;
    return FGC_OK;
}

int fgc_batch_destroy(fgc_batch* b) {
    if (!b) return FGC_OK;
    {
        std::lock_guard<std::mutex> lock(b->mu);
        cudaSetDevice(b->device);
        if (b->inflight) wait(b, nullptr);
        cudaStreamSynchronize(b->stream);
        if (b->exec) cudaGraphExecDestroy(b->exec);
        if (b->done) cudaEventDestroy(b->done);
    }
    if (b->own_stream) cudaStreamDestroy(b->own_stream);
    delete b;
    return FGC_OK;
}

int fgc_batch_set_stream(fgc_batch* b, void* cuda_stream) {
    if (!b) return fail(FGC_ERR_INVALID_ARGUMENT, "null batch");
    std::lock_guard<std::mutex> lock(b->mu);
    if (b->inflight) return fail(FGC_ERR_BUSY, "the batch has a submission in flight");
    FGC_CUDA(cudaSetDevice(b->device));
    FGC_CUDA(cudaStreamSynchronize(b->stream));
    b->stream = cuda_stream ? (cudaStream_t)cuda_stream : b->own_stream;
    return FGC_OK;
}

int fgc_batch_set_tuning(fgc_batch* b, const fgc_batch_tuning* t) {
    if (!b || !t) return fail(FGC_ERR_INVALID_ARGUMENT, "null argument");
    if (t->band_pixels < 1 || t->prims_per_bin_block < 1 || t->fragment_cap < 256 || t->window < 0 ||
        t->window > 256)
        return fail(FGC_ERR_INVALID_ARGUMENT, "tuning values out of range");
    std::lock_guard<std::mutex> lock(b->mu);
    if (b->inflight) return fail(FGC_ERR_BUSY, "the batch has a submission in flight");
    b->tuning.band_pixels = t->band_pixels;
    b->tuning.prims_per_bin_block = t->prims_per_bin_block;
    b->tuning.frag_cap = t->fragment_cap;
    b->tuning.window = t->window ? t->window : 8;
    b->use_graph = t->use_graph != 0;
    return FGC_OK;
}

int fgc_batch_get_tuning(const fgc_batch* b, fgc_batch_tuning* t) {
    if (!b || !t) return fail(FGC_ERR_INVALID_ARGUMENT, "null argument");
    t->band_pixels = (int32_t)b->tuning.band_pixels;
    t->prims_per_bin_block = (int32_t)b->tuning.prims_per_bin_block;
    t->fragment_cap = b->tuning.frag_cap;
    t->use_graph = b->use_graph ? 1 : 0;
    t->window = b->tuning.window;
    t->reserved = 0;
    return FGC_OK;
}

int fgc_batch_set_timing(fgc_batch* b, int32_t enable) {
    if (!b) return fail(FGC_ERR_INVALID_ARGUMENT, "null batch");
    std::lock_guard<std::mutex> lock(b->mu);
    b->timing = enable != 0;
    return FGC_OK;
}

int fgc_batch_submit(fgc_batch* b, const fgc_batch_item* items, uint64_t n) {
    if (!b || (n && !items)) return fail(FGC_ERR_INVALID_ARGUMENT, "null argument");
    std::lock_guard<std::mutex> lock(b->mu);
    FGC_CUDA(cudaSetDevice(b->device));
    return submit(b, items, n);
}

int fgc_batch_query(fgc_batch* b, int32_t* done) {
    if (!b || !done) return fail(FGC_ERR_INVALID_ARGUMENT, "null argument");
    std::lock_guard<std::mutex> lock(b->mu);
    if (!b->inflight) {
        *done = 1;
        return FGC_OK;
    }
    FGC_CUDA(cudaSetDevice(b->device));
    cudaError_t e = cudaEventQuery(b->done);
    if (e == cudaErrorNotReady) {
        *done = 0;
        return FGC_OK;
    }
    if (e != cudaSuccess) return fail(FGC_ERR_CUDA, std::string("cudaEventQuery: ") + cudaGetErrorString(e));
    *done = 1;
    return FGC_OK;
}

int fgc_batch_wait(fgc_batch* b, fgc_rasterize_info* infos) {
    if (!b) return fail(FGC_ERR_INVALID_ARGUMENT, "null batch");
    std::lock_guard<std::mutex> lock(b->mu);
    FGC_CUDA(cudaSetDevice(b->device));
    return wait(b, infos);
}

int fgc_batch_last_stats(const fgc_batch* b, fgc_stats* out) {
    if (!b || !out) return fail(FGC_ERR_INVALID_ARGUMENT, "null argument");
    *out = b->stats;
    return FGC_OK;
}

int fgc_batch_autotune(fgc_batch* b, const fgc_batch_item* items, uint64_t n, int32_t repeats,
                       fgc_batch_tuning* best) {
    if (!b || !items || !n) return fail(FGC_ERR_INVALID_ARGUMENT, "null argument");
    if (repeats < 1) repeats = 1;
    std::lock_guard<std::mutex> lock(b->mu);
    FGC_CUDA(cudaSetDevice(b->device));
    if (b->inflight) return fail(FGC_ERR_BUSY, "the batch has a submission in flight");
    // one run per repeat after a warm-up; the median wall time from submit
    // to the end of wait
    auto measure = [&](double* ms) -> int {
        std::vector<double> t;
        for (int r = 0; r <= repeats; r++) {
            auto t0 = std::chrono::steady_clock::now();
            int rc = submit(b, items, n);
            if (rc == FGC_OK) rc = wait(b, nullptr);
            if (rc) return rc;
            auto t1 = std::chrono::steady_clock::now();
            if (r > 0) t.push_back(std::chrono::duration<double, std::milli>(t1 - t0).count());
        }
        std::sort(t.begin(), t.end());
        *ms = t[t.size() / 2];
        return FGC_OK;
    };
    // coordinate descent over the four shapes, one sweep in this order
    const int64_t bands[] = {2048, 4096, 8192};
    const int64_t blocks[] = {2048, 4096, 8192, 16384};
    const int frags[] = {512, 768, 1024};
    const int windows[] = {4, 8, 16, 32};
    PassTuning cur = b->tuning;
    double cur_ms = 0;
    int rc = measure(&cur_ms);
    if (rc) return rc;
    auto try_one = [&](PassTuning cand) -> int {
        PassTuning keep = b->tuning;
        b->tuning = cand;
        double ms = 0;
        int r = measure(&ms);
        if (r) {
            b->tuning = keep;
            return r;
        }
        if (ms < cur_ms) {
            cur_ms = ms;
            cur = cand;
        }
        b->tuning = cur;
        return FGC_OK;
    };
    for (int64_t v : bands) {
        if (v == cur.band_pixels) continue;
        PassTuning c = cur;
        c.band_pixels = v;
        if ((rc = try_one(c))) return rc;
    }
    for (int64_t v : blocks) {
        if (v == cur.prims_per_bin_block) continue;
        PassTuning c = cur;
        c.prims_per_bin_block = v;
        if ((rc = try_one(c))) return rc;
    }
    for (int v : frags) {
        if (v == cur.frag_cap) continue;
        PassTuning c = cur;
        c.frag_cap = v;
        if ((rc = try_one(c))) return rc;
    }
    for (int v : windows) {
        if (v == cur.window) continue;
        PassTuning c = cur;
        c.window = v;
        if ((rc = try_one(c))) return rc;
    }
    b->tuning = cur;
    if (best) {
        best->band_pixels = (int32_t)cur.band_pixels;
        best->prims_per_bin_block = (int32_t)cur.prims_per_bin_block;
        best->fragment_cap = cur.frag_cap;
        best->use_graph = b->use_graph ? 1 : 0;
        best->window = cur.window;
        best->reserved = 0;
    }
    return FGC_OK;
}

}  // extern "C"
