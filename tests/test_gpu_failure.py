"""GPU failure path of the bounded waits, without a GPU fault.

The binning stage scans its bin counts in one pass by a decoupled
look-back: each block waits, for a bounded number of polls, until its
predecessors have published their sums. The test hook fgc_debug_lookback
shortens that bound and names a block that never publishes, so the waits of
the blocks after it run out. The draw must then
come back with FGC_ERR_DEVICE_LIMIT (not hang, not fault), leave the
framebuffer untouched, keep its pending clears, and the same context must
draw correctly once the hook is reset."""
import ctypes

import numpy as np
import pytest

from fauxgl_gb300 import _abi, scenes
from fauxgl_gb300.context import NewContext, _upload_mesh
from oracle import oracle as O
from tests.helpers import phong, state

pytestmark = pytest.mark.gpu


def draw(lib, ctx, mh, st, sh):
    info = _abi.FgcRasterizeInfo()
    rc = lib.fgc_draw_mesh(ctx.handle, mh, ctypes.byref(st), ctypes.byref(sh), ctypes.byref(info))
    return rc, (int(info.total_pixels), int(info.updated_pixels))


def test_lookback_wait_runs_out_and_context_stays_usable(gpu_lib):
    # 81,920 triangles at 1920x1080: 540 bands x 20 binning blocks, a bin
    # count matrix of six scan blocks
    w, h = 1920, 1080
    mesh = scenes.displaced_sphere(6)
    mh = _upload_mesh(mesh)
    sh = phong(scenes.camera_matrix(w, h), scenes.LIGHT, scenes.EYE, scenes.OBJECT_COLOR)
    st = state()
    ctx = NewContext(w, h)
    ctx.SetDebug(_abi.FGC_DEBUG_WINNER)
    ctx.ClearColorBufferWith(scenes.BACKGROUND)
    try:
        _abi.check(gpu_lib.fgc_debug_lookback(64, 1))  # block 1 never publishes; 64 polls
        rc, _ = draw(gpu_lib, ctx, mh, st, sh)
        assert rc == _abi.FGC_ERR_DEVICE_LIMIT
        assert b"look-back" in gpu_lib.fgc_last_error()
        rc, _ = draw(gpu_lib, ctx, mh, st, sh)  # every draw under the hook gives up the same way
        assert rc == _abi.FGC_ERR_DEVICE_LIMIT
    finally:
        _abi.check(gpu_lib.fgc_debug_lookback(0, 0xFFFFFFFF))
    # nothing was drawn, and the clear is still pending: the read applies it
    img = ctx.Image()
    assert (img == np.array(O.nrgba(scenes.BACKGROUND), dtype=np.uint8)).all()
    assert (ctx.Winner() == 0xFFFFFFFF).all()
    # the same context draws correctly afterwards
    ctx.ClearColorBufferWith(scenes.BACKGROUND)
    rc, info = draw(gpu_lib, ctx, mh, st, sh)
    assert rc == _abi.FGC_OK
    ref = O.OracleContext(w, h)
    ref.clear_color(scenes.BACKGROUND)
    assert info == ref.draw(mesh, st, sh)
    assert np.array_equal(ctx.Image(), ref.color())
    assert np.array_equal(ctx.DepthBuffer.view(np.uint64), ref.depth().view(np.uint64))
    assert np.array_equal(ctx.Winner(), ref.winner())


def test_default_lookback_limit_is_restored(gpu_lib):
    """fgc_debug_lookback(0, none) restores the default bound: a large draw
    with thousands of blocks completes."""
    _abi.check(gpu_lib.fgc_debug_lookback(0, 0xFFFFFFFF))
    mesh = scenes.displaced_sphere(6)
    ctx = NewContext(640, 360)
    sh = phong(scenes.camera_matrix(640, 360), scenes.LIGHT, scenes.EYE, scenes.OBJECT_COLOR)
    rc, info = draw(gpu_lib, ctx, _upload_mesh(mesh), state(), sh)
    assert rc == _abi.FGC_OK and info[0] > 0
    st = _abi.FgcStats()
    _abi.check(gpu_lib.fgc_context_last_stats(ctx.handle, ctypes.byref(st)))
    assert st.attempts == 1
