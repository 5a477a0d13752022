"""GPU parity on the workloads the benchmark times, at their stated sizes.

  supersampled frame  the dense 1,310,720-triangle mesh at 7680x4320 (1920x1080
                      at scale 4), PhongShader, then the same mesh as a
                      wireframe overlay (DepthBias 1e-5, SolidColorShader black
                      at alpha 0.5, AlphaBlend), then the device box-downsample
                      to 1920x1080
  thumbnail views     a covering subset of the 1,024-view batch (every shape
                      kind at every resolution, the fewest and most segments,
                      the largest meshes) rendered through fgc_batch_submit

Plain form: RasterizeInfo, NRGBA colour, depth bits and winner ids identical
to the oracle's, FP64 shader output within 1e-12. Mixed form: RasterizeInfo,
depth bits and winner ids identical (zero mismatches), colour within 1/255
per channel."""
import ctypes

import numpy as np
import pytest

from fauxgl_gb300 import _abi, scenes
from fauxgl_gb300.context import NewContext, _upload_mesh
from fauxgl_gb300.shader import NewPhongShader, to_fgc_shader
from oracle import oracle as O
from tests.helpers import phong, solid, state

pytestmark = pytest.mark.gpu

PLAIN, MIXED = _abi.FGC_PRECISION_PLAIN, _abi.FGC_PRECISION_MIXED
SS_W, SS_H, SS = 1920 * 4, 1080 * 4, 4


def check_error(err, precision, shaded=True):
    assert err["winner_mismatch_frac"] == 0, err
    assert err["depth_mismatch_frac"] == 0, err
    if precision == PLAIN:
        assert err["max_err_steps"] == 0, err
        if shaded:
            assert err["shaded_max_err"] <= 1e-12, err
    else:
        assert err["max_err_steps"] <= 1, err


@pytest.fixture(scope="module")
def dense():
    return scenes.displaced_sphere(8)


def ss_draws():
    m = scenes.camera_matrix(SS_W, SS_H)
    return [(state(), phong(m, scenes.LIGHT, scenes.EYE, scenes.OBJECT_COLOR)),
            (state(wireframe=1, depth_bias=1e-5), solid((0, 0, 0, 0.5), m))]


@pytest.fixture(scope="module")
def ss_oracle(dense):
    ref = O.OracleContext(SS_W, SS_H)
    ref.clear_color(scenes.BACKGROUND)
    infos = [ref.draw(dense, st, sh) for st, sh in ss_draws()]
    return ref, infos


@pytest.mark.parametrize("precision", [PLAIN, MIXED])
def test_supersampled_overlay_full_size(gpu_lib, dense, ss_oracle, precision):
    ref, rinfos = ss_oracle
    mh = _upload_mesh(dense)
    ctx = NewContext(SS_W, SS_H)
    ctx.SetDebug(_abi.FGC_DEBUG_WINNER | (_abi.FGC_DEBUG_SHADED_COLOR if precision == PLAIN else 0))
    ctx.ClearColorBufferWith(scenes.BACKGROUND)
    for (st, sh), rinfo in zip(ss_draws(), rinfos):
        st.precision = precision
        info = _abi.FgcRasterizeInfo()
        _abi.check(gpu_lib.fgc_draw_mesh(ctx.handle, mh, ctypes.byref(st), ctypes.byref(sh), ctypes.byref(info)))
        assert (int(info.total_pixels), int(info.updated_pixels)) == tuple(rinfo)
    err = O.frame_error(ctx.Image(), ctx.DepthBuffer, ctx.Winner(), ref,
                        shaded=ctx.ShadedColor() if precision == PLAIN else None)
    check_error(err, precision)
    ds = ctx.Downsample(SS).astype(np.int16)
    rds = O.downsample(ref.color(), SS).astype(np.int16)
    assert np.abs(ds - rds).max() <= (0 if precision == PLAIN else 1)


def check_views():
    _, views = scenes.thumbnail_batch(build=set())
    pick = scenes.thumbnail_check_views(views)
    meshes, views = scenes.thumbnail_batch(build={views[i]["mesh"] for i in pick})
    return meshes, [views[i] for i in pick]


@pytest.mark.parametrize("precision", [MIXED, PLAIN])
def test_thumbnail_views_against_oracle(gpu_lib, precision):
    meshes, views = check_views()
    kinds = {(v["kind"], v["width"]) for v in views}
    assert len(kinds) == 12 and len(views) >= 16
    n = len(views)
    items = (_abi.FgcBatchItem * n)()
    keep, ctxs = [], []
    for i, v in enumerate(views):
        ctx = NewContext(v["width"], v["height"])
        ctx.SetDebug(_abi.FGC_DEBUG_WINNER)
        ctx.ClearColorBufferWith(scenes.BACKGROUND)
        st = state(precision=precision)
        sh = NewPhongShader(v["matrix"], scenes.LIGHT, v["eye"])
        sh.ObjectColor = v["color"]
        shs = to_fgc_shader(sh)
        keep += [st, shs]
        m = meshes[v["mesh"]]
        it = items[i]
        it.context, it.mesh = ctx.handle, _upload_mesh(m)
        it.tri_first, it.tri_count, it.line_first, it.line_count = 0, m.ntri, 0, 0
        it.state, it.shader = ctypes.pointer(st), ctypes.pointer(shs)
        ctxs.append(ctx)
    b = ctypes.c_void_p()
    _abi.check(gpu_lib.fgc_batch_create(ctypes.byref(b)))
    infos = (_abi.FgcRasterizeInfo * n)()
    try:
        _abi.check(gpu_lib.fgc_batch_submit(b, items, n))
        _abi.check(gpu_lib.fgc_batch_wait(b, infos))
    finally:
        gpu_lib.fgc_batch_destroy(b)
    for i, v in enumerate(views):
        ref = O.OracleContext(v["width"], v["height"])
        ref.clear_color(scenes.BACKGROUND)
        rinfo = ref.draw(meshes[v["mesh"]], keep[2 * i], keep[2 * i + 1])
        assert (int(infos[i].total_pixels), int(infos[i].updated_pixels)) == tuple(rinfo), (i, v["kind"])
        err = O.frame_error(ctxs[i].Image(), ctxs[i].DepthBuffer, ctxs[i].Winner(), ref)
        check_error(err, precision, shaded=False)
