"""GPU: batches of many draws (fgc_batch_*) against the same draws run one at
a time (fgc_draw_mesh) and against the oracle.

A batch renders every draw with one launch per pipeline stage; each draw's
colour, FP64 depth (bit patterns), winner ids and RasterizeInfo must be
identical to what the draw gives alone, whatever else is in the batch and
whatever the pipeline's tuning."""
import ctypes

import numpy as np
import pytest

from fauxgl_gb300 import _abi
from fauxgl_gb300.context import NewContext, _upload_mesh, _upload_texture
from oracle import oracle as O
from tests.helpers import phong, random_scene, random_texture, scene_matrix, solid, state

pytestmark = pytest.mark.gpu

SIZES = [(97, 61), (160, 90), (33, 200), (256, 256), (640, 2), (61, 37), (300, 170), (1, 1), (4100, 9)]


def make_specs(seed, precision=_abi.FGC_PRECISION_PLAIN, sizes=SIZES, big=1):
    """One draw per frame size: seeded random scenes (some clipped), the three
    built-in shaders, wireframe, lines, alpha blending."""
    specs = []
    for k, (w, h) in enumerate(sizes):
        mesh = random_scene(seed * 100 + k, ntri=(30 + 25 * k) * big, nline=3 * k)
        m = list(scene_matrix(w / h))
        kind = k % 3
        if kind == 0:
            sh = phong(m, (0.3, 0.8, 0.5), (0.3, 0.2, 4.5), color=(0.27, 0.54, 0.4, 1) if k % 2 else (0, 0, 0, 0))
            tex = None
        elif kind == 1:
            sh = solid((0.9, 0.2, 0.1, 0.6 if k % 2 else 1.0), m)
            tex = None
        else:
            sh = _abi.FgcShader()
            sh.kind = _abi.FGC_SHADER_TEXTURE
            sh.matrix[:] = m
            tex = random_texture(seed + k)
        st = state(cull=[_abi.FGC_CULL_BACK, _abi.FGC_CULL_NONE, _abi.FGC_CULL_FRONT][k % 3],
                   wireframe=int(k == 5), alpha_blend=int(k % 2 == 1), precision=precision)
        clear = ((k * 37 % 255) / 255.0, 0.5, 0.25, 1.0 if k % 2 == 0 else 0.0)
        specs.append(dict(w=w, h=h, mesh=mesh, st=st, sh=sh, tex=tex, clear=clear))
    return specs


def shader_with_texture(spec):
    sh = _abi.FgcShader.from_buffer_copy(spec["sh"])
    if spec["tex"] is not None:
        sh.texture = _upload_texture(spec["tex"])
    return sh


def new_target(spec):
    ctx = NewContext(spec["w"], spec["h"])
    ctx.SetDebug(_abi.FGC_DEBUG_WINNER)
    ctx.ClearColorBufferWith(spec["clear"])
    return ctx


def frame(ctx):
    return ctx.Image(), ctx.DepthBuffer.view(np.uint64), ctx.Winner()


def draw_alone(spec, ctx=None):
    lib = _abi.load_library()
    ctx = ctx or new_target(spec)
    info = _abi.FgcRasterizeInfo()
    sh = shader_with_texture(spec)
    _abi.check(lib.fgc_draw_mesh(ctx.handle, _upload_mesh(spec["mesh"]), ctypes.byref(spec["st"]), ctypes.byref(sh),
                                 ctypes.byref(info)))
    return ctx, (int(info.total_pixels), int(info.updated_pixels))


class BatchRun:
    """Owns a batch handle and the structs its items point at."""

    def __init__(self, tuning=None):
        self.lib = _abi.load_library()
        h = ctypes.c_void_p()
        _abi.check(self.lib.fgc_batch_create(ctypes.byref(h)))
        self.h = h.value
        if tuning:
            t = _abi.FgcBatchTuning(*tuning)
            _abi.check(self.lib.fgc_batch_set_tuning(self.h, ctypes.byref(t)))
        self.keep = []

    def items(self, specs, ctxs, reads=None):
        items = (_abi.FgcBatchItem * len(specs))()
        for i, (sp, ctx) in enumerate(zip(specs, ctxs)):
            sh = shader_with_texture(sp)
            self.keep += [sh, sp["st"]]
            it = items[i]
            it.context = ctx.handle
            it.mesh = _upload_mesh(sp["mesh"])
            it.tri_first, it.tri_count = 0, sp["mesh"].ntri
            it.line_first, it.line_count = 0, sp["mesh"].nline
            it.state = ctypes.pointer(sp["st"])
            it.shader = ctypes.pointer(sh)
            if reads and reads[i] is not None:
                buf, scale = reads[i]
                it.out_nrgba = buf.ctypes.data
                it.out_scale = scale
        self.keep.append(items)
        return items

    def submit(self, items, n):
        _abi.check(self.lib.fgc_batch_submit(self.h, items, n))

    def wait(self, n):
        infos = (_abi.FgcRasterizeInfo * max(n, 1))()
        _abi.check(self.lib.fgc_batch_wait(self.h, infos))
        return [(int(infos[i].total_pixels), int(infos[i].updated_pixels)) for i in range(n)]

    def run(self, specs, ctxs, reads=None):
        items = self.items(specs, ctxs, reads)
        self.submit(items, len(specs))
        return self.wait(len(specs))

    def stats(self):
        st = _abi.FgcStats()
        _abi.check(self.lib.fgc_batch_last_stats(self.h, ctypes.byref(st)))
        return st

    def close(self):
        if self.h:
            self.lib.fgc_batch_destroy(self.h)
            self.h = None


def assert_same(ctx_a, ctx_b, what=""):
    a, b = frame(ctx_a), frame(ctx_b)
    for name, x, y in zip(("colour", "depth", "winner"), a, b):
        assert np.array_equal(x, y), "%s %s differs at %d pixels" % (what, name, int((x != y).sum()))


@pytest.mark.parametrize("precision", [_abi.FGC_PRECISION_PLAIN, _abi.FGC_PRECISION_MIXED])
def test_batch_matches_single_draws(gpu_lib, precision):
    specs = make_specs(1, precision)
    alone = [draw_alone(sp) for sp in specs]
    ctxs = [new_target(sp) for sp in specs]
    b = BatchRun()
    infos = b.run(specs, ctxs)
    st = b.stats()
    b.close()
    for k, (sp, (ctx1, info1), ctx2, info2) in enumerate(zip(specs, alone, ctxs, infos)):
        assert info1 == info2, (k, info1, info2)
        assert_same(ctx1, ctx2, "draw %d (%dx%d)" % (k, sp["w"], sp["h"]))
    assert st.covered_pixels == sum(i[0] for i in infos)
    assert st.updated_pixels == sum(i[1] for i in infos)
    assert st.elements == sum(sp["mesh"].ntri + sp["mesh"].nline for sp in specs)


def test_batch_against_oracle(gpu_lib):
    specs = make_specs(2, sizes=[(64, 48), (31, 77), (120, 40)])
    ctxs = [new_target(sp) for sp in specs]
    b = BatchRun()
    infos = b.run(specs, ctxs)
    b.close()
    for sp, ctx, info in zip(specs, ctxs, infos):
        ref = O.OracleContext(sp["w"], sp["h"])
        ref.clear_color(sp["clear"])
        rinfo = ref.draw(sp["mesh"], sp["st"], sp["sh"], texture=sp["tex"], what=3)
        assert info == tuple(rinfo)
        assert np.array_equal(ctx.Image(), ref.color())
        assert np.array_equal(ctx.DepthBuffer.view(np.uint64), ref.depth().view(np.uint64))
        assert np.array_equal(ctx.Winner(), ref.winner())


def test_batch_mixed_precisions_and_shared_targets(gpu_lib):
    """Draws that share a context run in order (successive passes); draws of
    both precisions in one submission."""
    base = make_specs(3, sizes=[(128, 96), (90, 90), (200, 60)])
    over = []
    for sp in base:
        o = dict(sp)
        o["mesh"] = sp["mesh"]
        o["st"] = state(cull=_abi.FGC_CULL_NONE, wireframe=1, depth_bias=1e-5, alpha_blend=1,
                        precision=_abi.FGC_PRECISION_MIXED)
        o["sh"] = solid((0, 0, 0, 0.5), list(scene_matrix(sp["w"] / sp["h"])))
        o["tex"] = None
        over.append(o)
    # sequential reference: surface then overlay on the same context
    seq = []
    for sp, o in zip(base, over):
        ctx, i1 = draw_alone(sp)
        _, i2 = draw_alone(o, ctx)
        seq.append((ctx, i1, i2))
    ctxs = [new_target(sp) for sp in base]
    b = BatchRun()
    specs = base + over
    infos = b.run(specs, ctxs + ctxs)
    st = b.stats()
    b.close()
    n = len(base)
    for k, (ctx1, i1, i2) in enumerate(seq):
        assert infos[k] == i1 and infos[n + k] == i2, (k, infos[k], i1, infos[n + k], i2)
        assert_same(ctx1, ctxs[k], "target %d" % k)
    assert st.attempts >= 1


def test_batch_read_back_and_downsample(gpu_lib):
    specs = make_specs(4, sizes=[(96, 64), (128, 128), (60, 30)])
    ctxs = [new_target(sp) for sp in specs]
    reads = [(np.zeros((64, 96, 4), np.uint8), 1), (np.zeros((32, 32, 4), np.uint8), 4),
             (np.zeros((15, 30, 4), np.uint8), 2)]
    b = BatchRun()
    b.run(specs, ctxs, reads)
    b.close()
    assert np.array_equal(reads[0][0], ctxs[0].Image())
    assert np.array_equal(reads[1][0], ctxs[1].Downsample(4))
    assert np.array_equal(reads[2][0], ctxs[2].Downsample(2))


def test_batch_contexts_are_busy_until_wait(gpu_lib):
    specs = make_specs(5, sizes=[(400, 300), (300, 200)], big=8)
    ctxs = [new_target(sp) for sp in specs]
    b = BatchRun()
    items = b.items(specs, ctxs)
    b.submit(items, len(specs))
    with pytest.raises(_abi.FauxGLError) as e:
        ctxs[0].Image()
    assert e.value.status == _abi.FGC_ERR_BUSY
    with pytest.raises(_abi.FauxGLError) as e2:
        b.submit(items, len(specs))
    assert e2.value.status == _abi.FGC_ERR_BUSY
    done = ctypes.c_int32()
    _abi.check(b.lib.fgc_batch_query(b.h, ctypes.byref(done)))
    assert done.value in (0, 1)
    infos = b.wait(len(specs))
    b.close()
    for sp, ctx, info in zip(specs, ctxs, infos):
        ctx1, info1 = draw_alone(sp)
        assert info == info1
        assert_same(ctx1, ctx)


def test_batch_overflow_is_rerun(gpu_lib):
    """More clipped triangles than the first clip list holds, spread over the
    draws: the batch re-runs from the failed pass and still matches."""
    specs = make_specs(6, sizes=[(200, 150), (150, 200), (256, 64)], big=30)
    for sp in specs:
        sp["st"].cull = _abi.FGC_CULL_NONE
    ctxs = [new_target(sp) for sp in specs]
    b = BatchRun()
    infos = b.run(specs, ctxs)
    st = b.stats()
    b.close()
    assert st.clipped > 1024
    assert st.attempts >= 2
    for sp, ctx, info in zip(specs, ctxs, infos):
        ctx1, info1 = draw_alone(sp)
        assert info == info1
        assert_same(ctx1, ctx)


@pytest.mark.parametrize("tuning", [(2048, 2048, 512, 0, 4), (8192, 16384, 768, 0, 32), (4096, 4096, 1024, 1, 8),
                                    (4096, 4096, 1024, 0, 1)])
def test_batch_tuning_and_graph_do_not_change_results(gpu_lib, tuning):
    specs = make_specs(7, sizes=[(97, 61), (300, 170), (33, 200), (1024, 16)])
    alone = [draw_alone(sp) for sp in specs]
    b = BatchRun(tuning)
    for rep in range(2):  # the second submission replays / updates the graph
        ctxs = [new_target(sp) for sp in specs]
        infos = b.run(specs, ctxs)
        for (ctx1, info1), ctx2, info2 in zip(alone, ctxs, infos):
            assert info1 == info2
            assert_same(ctx1, ctx2, "rep %d" % rep)
    b.close()


def test_batch_autotune(gpu_lib):
    specs = make_specs(8, sizes=[(256, 256), (512, 128), (128, 512)], big=4)
    ctxs = [new_target(sp) for sp in specs]
    b = BatchRun()
    items = b.items(specs, ctxs)
    t = _abi.FgcBatchTuning()
    _abi.check(b.lib.fgc_batch_autotune(b.h, items, len(specs), 1, ctypes.byref(t)))
    assert t.band_pixels in (2048, 4096, 8192) and t.fragment_cap in (512, 768, 1024)
    assert t.window in (4, 8, 16, 32)
    cur = _abi.FgcBatchTuning()
    _abi.check(b.lib.fgc_batch_get_tuning(b.h, ctypes.byref(cur)))
    assert (cur.band_pixels, cur.prims_per_bin_block, cur.fragment_cap) == \
        (t.band_pixels, t.prims_per_bin_block, t.fragment_cap)
    ctxs = [new_target(sp) for sp in specs]
    infos = b.run(specs, ctxs)
    b.close()
    for sp, ctx, info in zip(specs, ctxs, infos):
        ctx1, info1 = draw_alone(sp)
        assert info == info1
        assert_same(ctx1, ctx)


def test_batch_empty_and_degenerate_items(gpu_lib):
    """Zero-length ranges, a 1x1 frame and an empty batch."""
    specs = make_specs(9, sizes=[(1, 1), (17, 5)])
    ctxs = [new_target(sp) for sp in specs]
    b = BatchRun()
    items = b.items(specs, ctxs)
    items[1].tri_count = 0
    items[1].line_count = 0
    b.submit(items, 2)
    infos = b.wait(2)
    assert infos[1] == (0, 0)
    # the clear still applies to a draw with nothing in it
    img = ctxs[1].Image()
    assert (img == img[0, 0]).all()
    _abi.check(b.lib.fgc_batch_submit(b.h, items, 0))
    assert b.wait(0) == []
    b.close()
