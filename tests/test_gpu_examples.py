"""GPU parity on the reference's own example scenes (tests/example_scenes.py):
the meshes fogleman/fauxgl ships, loaded with the library's LoadSTL kernel,
prepared with the example's own calls (BiUnitCube / Transform on the host,
SmoothNormals[Threshold] on the device) and drawn with the example's shader
fields, against the oracle fed the same file bytes.

Three things are checked: the GPU frame equals the oracle's (plain: colour,
depth bits, winner ids and RasterizeInfo identical; mixed: depth, winners and
RasterizeInfo identical, colour within 1/255); the oracle run here agrees
with the digests committed in tests/golden/examples.json (made by
tests/golden/make_examples.py on another machine); and the plain GPU frame
matches those digests too."""
import ctypes
import json
import os

import numpy as np
import pytest

from fauxgl_gb300 import _abi
from fauxgl_gb300.context import NewContext
from fauxgl_gb300.meshops import DeviceMesh
from oracle import oracle as O
from tests import example_scenes as E

pytestmark = pytest.mark.gpu

with open(os.path.join(E.GOLDEN, "examples.json")) as _f:
    GOLDEN = json.load(_f)


def prepare_device(dm, prep):
    """The preparation steps on a device mesh: smoothing by the library's
    kernels, BiUnitCube / Transform by the host mirror on a downloaded copy."""
    for step in prep:
        if step[0] in ("bi_unit_cube", "transform"):
            m = dm.download()
            if step[0] == "bi_unit_cube":
                m.BiUnitCube()
            else:
                m.Transform(step[1])
            dm = DeviceMesh.upload(m)
        elif step[0] == "smooth_threshold":
            dm.SmoothNormalsThreshold(step[1])
        elif step[0] == "smooth":
            dm.SmoothNormals()
    return dm


@pytest.fixture(scope="module")
def oracle_frames():
    cache = {}

    def get(name):
        if name not in cache:
            cache[name] = E.render_oracle(name)
        return cache[name]
    return get


@pytest.mark.parametrize("name", E.NAMES)
def test_oracle_matches_committed_digests(name, oracle_frames):
    ref, infos, mesh = oracle_frames(name)
    g = GOLDEN[name]
    assert [list(i) for i in infos] == g["infos"]
    assert mesh.ntri == g["triangles"]
    assert E.digests(ref.color(), ref.depth(), ref.winner()) == {k: g[k] for k in ("color", "depth", "winner")}


@pytest.mark.parametrize("precision", [_abi.FGC_PRECISION_PLAIN, _abi.FGC_PRECISION_MIXED])
@pytest.mark.parametrize("name", E.NAMES)
def test_example_scene(gpu_lib, oracle_frames, name, precision):
    stl, w, h, clear, prep, draws = E.scene(name)
    ref, rinfos, host_mesh = oracle_frames(name)
    dm = prepare_device(DeviceMesh.load_stl(E.stl_bytes(stl)), prep)
    got = dm.download()
    assert np.array_equal(got.tri_pos.view(np.uint64), host_mesh.tri_pos.view(np.uint64)), "positions differ"
    assert np.array_equal(got.tri_nrm.view(np.uint64), host_mesh.tri_nrm.view(np.uint64)), "normals differ"

    plain = precision == _abi.FGC_PRECISION_PLAIN
    ctx = NewContext(w, h)
    ctx.SetDebug(_abi.FGC_DEBUG_WINNER | (_abi.FGC_DEBUG_SHADED_COLOR if plain else 0))
    ctx.ClearColorBufferWith(clear)
    infos = []
    for st, sh in draws:
        st = _abi.FgcState.from_buffer_copy(st)
        st.precision = precision
        info = _abi.FgcRasterizeInfo()
        _abi.check(gpu_lib.fgc_draw_mesh(ctx.handle, dm.handle, ctypes.byref(st), ctypes.byref(sh),
                                         ctypes.byref(info)))
        infos.append((int(info.total_pixels), int(info.updated_pixels)))
    assert infos == [tuple(i) for i in rinfos]
    img, depth, win = ctx.Image(), ctx.DepthBuffer, ctx.Winner()
    err = O.frame_error(img, depth, win, ref, shaded=ctx.ShadedColor() if plain else None)
    assert err["winner_mismatch_frac"] == 0 and err["depth_mismatch_frac"] == 0, err
    if plain:
        assert err["max_err_steps"] == 0, err
        assert err["shaded_max_err"] <= 1e-12, err
        g = GOLDEN[name]
        assert E.digests(img, depth, win) == {k: g[k] for k in ("color", "depth", "winner")}
    else:
        assert err["max_err_steps"] <= 1, err
