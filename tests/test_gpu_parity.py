"""GPU parity: libfauxglcuda (through the C ABI) against the oracle on the same
inputs.

Plain form (FP64): RasterizeInfo, NRGBA colour, FP64 depth (bit patterns)
and winner ids must be identical; the FP64 shader output of each pixel's
last updating fragment must be within 1e-12 per channel (it is identical
unless a fractional SpecularPower routes through exp/log).
Mixed form: RasterizeInfo, depth and winner ids identical; NRGBA within
1/255 per channel."""
import ctypes

import numpy as np
import pytest

from fauxgl_gb300 import _abi, scenes
from fauxgl_gb300.context import NewContext, _upload_mesh, _upload_texture
from fauxgl_gb300.mesh import Mesh
from oracle import oracle as O
from tests.helpers import (phong, random_scene, random_texture, scene_matrix, screen_to_ndc, screen_triangle_mesh,
                           solid, state)

pytestmark = pytest.mark.gpu

COLOR_TOL_PLAIN = 1e-12
MAXF = 1.7976931348623157e308


class Pair:
    """A GPU context and an oracle context driven with the same calls."""

    def __init__(self, w, h, debug=3):
        self.w, self.h = w, h
        self.gpu = NewContext(w, h)
        self.gpu.SetDebug(debug)
        self.ref = O.OracleContext(w, h)

    def clear_color(self, c):
        self.gpu.ClearColorBufferWith(c)
        self.ref.clear_color(c)

    def clear_depth(self, v):
        self.gpu.ClearDepthBufferWith(v)
        self.ref.clear_depth(v)

    def draw(self, mesh, st, sh, texture=None, what=3, tri_range=None, line_range=None):
        lib = _abi.load_library()
        mh = _upload_mesh(mesh)
        sh2 = _abi.FgcShader.from_buffer_copy(sh)
        if texture is not None:
            sh2.texture = _upload_texture(texture)
        info = _abi.FgcRasterizeInfo()
        if what == 3:
            rc = lib.fgc_draw_mesh(self.gpu.handle, mh, ctypes.byref(st), ctypes.byref(sh2), ctypes.byref(info))
        elif what == 1:
            f, c = tri_range or (0, mesh.ntri)
            rc = lib.fgc_draw_triangles(self.gpu.handle, mh, f, c, ctypes.byref(st), ctypes.byref(sh2),
                                        ctypes.byref(info))
        else:
            f, c = line_range or (0, mesh.nline)
            rc = lib.fgc_draw_lines(self.gpu.handle, mh, f, c, ctypes.byref(st), ctypes.byref(sh2),
                                    ctypes.byref(info))
        _abi.check(rc)
        rinfo = self.ref.draw(mesh, st, sh, texture=texture, what=what, tri_range=tri_range, line_range=line_range)
        return (int(info.total_pixels), int(info.updated_pixels)), rinfo

    def check(self, mixed=False, tol=COLOR_TOL_PLAIN):
        g, r = self.gpu, self.ref
        gd, rd = g.DepthBuffer, r.depth()
        assert np.array_equal(gd.view(np.uint64), rd.view(np.uint64)), \
            "depth differs at %d pixels" % int((gd.view(np.uint64) != rd.view(np.uint64)).sum())
        gw, rw = g.Winner(), r.winner()
        assert np.array_equal(gw, rw), "winner ids differ at %d pixels" % int((gw != rw).sum())
        gi, ri = g.Image(), r.color()
        if mixed:
            assert np.abs(gi.astype(int) - ri.astype(int)).max() <= 1
        else:
            assert np.array_equal(gi, ri), "colour differs at %d pixels" % int((gi != ri).any(-1).sum())
            gs, rs = g.ShadedColor(), r.shaded()
            both = np.isfinite(gs) & np.isfinite(rs)
            assert np.array_equal(np.isnan(gs), np.isnan(rs))
            assert np.abs(gs[both] - rs[both]).max(initial=0) <= tol


def run_both(pair, mesh, st, sh, **kw):
    gi, ri = pair.draw(mesh, st, sh, **kw)
    assert gi == ri, (gi, ri)
    return gi


# ---------------------------------------------------------------------------
# known-answer scenes
# ---------------------------------------------------------------------------
TRI = [(1, 1), (9, 1), (1, 9)]


def test_single_triangle_and_ties(gpu_lib):
    p = Pair(16, 16)
    m = screen_triangle_mesh([TRI, TRI], 16, 16)
    assert run_both(p, m, state(cull=_abi.FGC_CULL_NONE), solid((0, 1, 0, 1))) == (72, 72)
    p.check()


@pytest.mark.parametrize("cull", [_abi.FGC_CULL_NONE, _abi.FGC_CULL_FRONT, _abi.FGC_CULL_BACK])
@pytest.mark.parametrize("face", [_abi.FGC_FACE_CW, _abi.FGC_FACE_CCW])
def test_cull_modes(gpu_lib, cull, face):
    p = Pair(16, 16)
    m = screen_triangle_mesh([TRI, TRI[::-1], [(3, 12), (14, 4), (15, 15)]], 16, 16)
    run_both(p, m, state(cull=cull, front_face=face), solid((1, 0.5, 0.25, 1)))
    p.check()


def test_discard_and_depth_flags(gpu_lib):
    p = Pair(16, 16)
    st = dict(cull=_abi.FGC_CULL_NONE)
    near = screen_triangle_mesh([TRI], 16, 16, z=-0.5)
    far = screen_triangle_mesh([TRI], 16, 16, z=0.5)
    assert run_both(p, near, state(**st), solid((0, 0, 0, 0))) == (36, 0)
    run_both(p, near, state(write_depth=0, **st), solid((1, 0, 0, 1)))
    run_both(p, near, state(**st), solid((1, 0, 0, 1)))
    run_both(p, far, state(**st), solid((0, 0, 1, 1)))
    run_both(p, far, state(read_depth=0, **st), solid((0, 0, 1, 1)))
    run_both(p, near, state(write_color=0, **st), solid((0, 1, 0, 1)))
    run_both(p, near, state(depth_bias=0.125, **st), solid((0, 1, 0, 1)))
    run_both(p, far, state(depth_bias=-0.3, **st), solid((0, 1, 1, 1)))
    p.check()


@pytest.mark.parametrize("alpha", [1.0, 0.5])
def test_row_wraparound(gpu_lib, alpha):
    w = h = 16
    pts = [((15.5, 4.0), (15.5, 10.0)), ((0.3, 2.0), (0.2, 13.0)), ((14.0, 15.8), (2.0, 15.9)),
           ((8.0, 0.1), (15.9, 0.2))]
    lp = np.array([[[*screen_to_ndc(x, y, w, h), 0.0] for (x, y) in seg] for seg in pts])
    line = Mesh(None, line_pos=lp)
    p = Pair(w, h)
    p.clear_color((0, 0, 0, 1))
    run_both(p, line, state(line_width=4.0), solid((1, 1, 1, alpha)), what=2)
    p.check()


@pytest.mark.parametrize("alpha", [1.0, 0.5])
def test_wrapped_rows_beyond_a_chunk(gpu_lib, alpha):
    """Line quads hundreds of pixels wider than a 2-pixel frame: in each band
    their wrapped rows outnumber the units one chunk holds, so the
    rasteriser takes such a primitive alone, its rows over several chunks."""
    w, h = 2, 300
    pts = [((0.5, 10.0), (1.5, 290.0)), ((1.0, 150.0), (1.2, 160.0)), ((0.1, 299.0), (1.9, 0.5))]
    lp = np.array([[[*screen_to_ndc(x, y, w, h), 0.0] for (x, y) in seg] for seg in pts])
    line = Mesh(None, line_pos=lp)
    p = Pair(w, h)
    p.clear_color((0, 0, 0, 1))
    run_both(p, line, state(line_width=400.0), solid((1, 1, 1, alpha)), what=2)
    p.check()


# ---------------------------------------------------------------------------
# seeded random scenes over the draw state space
# ---------------------------------------------------------------------------
STATES = [
    dict(),
    dict(cull=_abi.FGC_CULL_NONE),
    dict(cull=_abi.FGC_CULL_FRONT, front_face=_abi.FGC_FACE_CW),
    dict(wireframe=1),
    dict(wireframe=1, line_width=5.5, depth_bias=-1e-4),
    dict(cull=_abi.FGC_CULL_NONE, depth_bias=1e-5),
    dict(read_depth=0),
    dict(write_depth=0, cull=_abi.FGC_CULL_NONE),
]


@pytest.mark.parametrize("si", range(len(STATES)))
@pytest.mark.parametrize("shader", ["solid", "solid_alpha", "phong", "phong_vertex", "phong_pow", "texture",
                                    "phong_texture"])
def test_random_scenes(gpu_lib, si, shader):
    seed = 1000 * si + sum(ord(ch) for ch in shader)
    w, h = 97, 61
    mesh = random_scene(seed, ntri=80, nline=25)
    m = scene_matrix(w / h)
    tex = None
    if shader == "solid":
        sh = solid((0.9, 0.3, 0.2, 1.0), m)
    elif shader == "solid_alpha":
        sh = solid((0.2, 0.6, 0.9, 0.4), m)
    elif shader == "phong":
        sh = phong(m, (0.3, 0.8, 0.5), (0.3, 0.2, 4.5), (0.27, 0.54, 0.4, 1.0))
    elif shader == "phong_vertex":
        sh = phong(m, (0.3, 0.8, 0.5), (0.3, 0.2, 4.5), (0, 0, 0, 0))
    elif shader == "phong_pow":
        sh = phong(m, (0.3, 0.8, 0.5), (0.3, 0.2, 4.5), (0.27, 0.54, 0.4, 0.6), power=7.0)
    else:
        tex = random_texture(seed)
        if shader == "texture":
            sh = _abi.FgcShader()
            sh.kind = _abi.FGC_SHADER_TEXTURE
            sh.matrix[:] = list(m)
        else:
            sh = phong(m, (0.3, 0.8, 0.5), (0.3, 0.2, 4.5), (0.27, 0.54, 0.4, 1.0))
    p = Pair(w, h)
    p.clear_color((0.1, 0.2, 0.3, 1.0))
    run_both(p, mesh, state(**STATES[si]), sh, texture=tex)
    # a second draw on top exercises the loaded (not cleared) framebuffer
    run_both(p, random_scene(seed + 1, ntri=40, nline=10), state(**STATES[(si + 3) % len(STATES)]), sh, texture=tex)
    p.check()


def test_fractional_specular_power_within_tolerance(gpu_lib):
    w, h = 64, 48
    mesh = random_scene(77, ntri=60)
    m = scene_matrix(w / h)
    p = Pair(w, h)
    run_both(p, mesh, state(), phong(m, (0.3, 0.8, 0.5), (0.3, 0.2, 4.5), (0.27, 0.54, 0.4, 1.0), power=12.37))
    g, r = p.gpu.ShadedColor(), p.ref.shaded()
    assert np.nanmax(np.abs(g - r)) <= COLOR_TOL_PLAIN
    assert np.array_equal(p.gpu.Winner(), p.ref.winner())


@pytest.mark.parametrize("power", [1.0, 2.0, 3.0, 7.0, 32.0, 33.0, 255.0, 1000.0, 2.0 ** 40, 2.0 ** 63])
def test_integer_specular_powers_bit_exact(gpu_lib, power):
    """Integer SpecularPower takes the repeated-squaring path of math.Pow;
    1000 and 2^40 drive results below the normal range and the exponent
    guard's early exit, 2^63 is beyond the integer path."""
    w, h = 64, 48
    mesh = random_scene(91, ntri=60)
    m = scene_matrix(w / h)
    p = Pair(w, h)
    run_both(p, mesh, state(), phong(m, (0.3, 0.8, 0.5), (0.3, 0.2, 4.5), (0.27, 0.54, 0.4, 1.0), power=power))
    g, r = p.gpu.ShadedColor(), p.ref.shaded()
    gn, rn = np.isnan(g), np.isnan(r)
    assert np.array_equal(gn, rn)
    assert np.array_equal(np.where(gn, 0.0, g).view(np.uint64), np.where(rn, 0.0, r).view(np.uint64))
    p.check()


@pytest.mark.parametrize("w,h", [(1, 1), (3, 200), (200, 3), (640, 2), (4100, 9), (61, 37), (9000, 11), (16000, 5)])
def test_odd_frame_shapes(gpu_lib, w, h):
    mesh = random_scene(w * 7 + h, ntri=120, nline=30)
    m = scene_matrix(w / h)
    p = Pair(w, h)
    p.clear_color((1, 1, 1, 1))
    run_both(p, mesh, state(cull=_abi.FGC_CULL_NONE), phong(m, (0.3, 0.8, 0.5), (0.3, 0.2, 4.5), (0.5, 0.2, 0.1, 0.7)))
    p.check()


def test_boxes_at_pixel_centre_boundaries(gpu_lib):
    """Triangles whose extremes sit on, just inside or just outside pixel
    centres (offsets of 0, 1e-15, 1e-9, 2^-8 and 2^-8 +- 1e-12 around
    k + 1/2), needles and slivers: the setup leaves out box rows and columns
    that hold no covered centre, and the frame must not change."""
    rng = np.random.default_rng(2024)
    w = h = 96
    offs = np.array([0.0, 1e-15, -1e-15, 1e-9, -1e-9, 2.0 ** -8, -2.0 ** -8, 2.0 ** -8 + 1e-12,
                     -2.0 ** -8 - 1e-12, 2.0 ** -8 - 1e-12, 0.25, -0.25, 0.499, 0.501])
    tris = []
    for _ in range(1500):
        c = rng.integers(4, w - 8, size=2)
        pts = []
        for _ in range(3):
            d = rng.integers(-3, 4, size=2)
            o = rng.choice(offs, size=2)
            pts.append((float(c[0] + d[0]) + 0.5 + o[0], float(c[1] + d[1]) + 0.5 + o[1]))
        tris.append(pts)
    for _ in range(300):  # needles and slivers: two corners almost together
        x, y = rng.uniform(4, w - 8, size=2)
        dx, dy = rng.uniform(-6, 6, size=2)
        e = rng.choice([1e-13, 1e-9, 1e-6, 1e-3])
        tris.append([(x, y), (x + dx, y + dy), (x + dx + e, y + dy - e)])
    mesh = screen_triangle_mesh(tris, w, h)
    p = Pair(w, h)
    for prec in (_abi.FGC_PRECISION_PLAIN, _abi.FGC_PRECISION_MIXED):
        for st in (state(cull=_abi.FGC_CULL_NONE, precision=prec),
                   state(cull=_abi.FGC_CULL_NONE, wireframe=1, line_width=0.75, precision=prec)):
            p = Pair(w, h)
            run_both(p, mesh, st, solid((0.3, 0.6, 0.9, 0.7)))
            p.check(mixed=prec == _abi.FGC_PRECISION_MIXED)


def test_triangle_and_line_ranges(gpu_lib):
    mesh = random_scene(5, ntri=90, nline=40)
    m = scene_matrix(1.0)
    p = Pair(80, 80)
    sh = solid((0.3, 0.6, 0.1, 0.8), m)
    run_both(p, mesh, state(), sh, what=1, tri_range=(10, 50))
    run_both(p, mesh, state(line_width=3.0), sh, what=2, line_range=(5, 20))
    run_both(p, mesh, state(), sh, what=1, tri_range=(89, 1))
    run_both(p, mesh, state(), sh, what=1, tri_range=(0, 0))
    p.check()


def test_big_primitives(gpu_lib):
    """Triangles larger than the fragment buffer take the multi-round path."""
    for w, h in ((1920, 64), (64, 700), (2000, 3)):
        tris = [[(-5, -5), (w + 7, -3), (-4, h + 9)], [(w + 3, h + 2), (-7, h + 5), (w + 6, -8)],
                [(0.5, 0.5), (w - 0.5, h * 0.5), (w * 0.3, h - 0.25)]]
        mesh = screen_triangle_mesh(tris, w, h, z=0.25)
        p = Pair(w, h)
        run_both(p, mesh, state(cull=_abi.FGC_CULL_NONE), solid((0.2, 0.4, 0.6, 0.9)))
        p.check()


def test_clip_list_and_bin_growth(gpu_lib):
    """More clipped triangles than the initial clip list, and more bin
    entries than the initial bin array: the draw re-runs with the sizes the
    device measured and still matches."""
    rng = np.random.default_rng(3)
    n = 6000
    c = rng.uniform(-3, 3, size=(n, 1, 3))
    c[..., 2] = rng.uniform(-1.5, 1.5, size=(n, 1))
    pos = c + rng.uniform(0.3, 1.2, size=(n, 1, 1)) * rng.normal(size=(n, 3, 3))
    mesh = Mesh(pos, rng.normal(size=(n, 3, 3)))
    m = scene_matrix(1.0)
    p = Pair(300, 300)
    run_both(p, mesh, state(cull=_abi.FGC_CULL_NONE, wireframe=1, line_width=3.0), solid((0, 0, 0, 0.5), m))
    p.check()


def test_clears_between_draws(gpu_lib):
    mesh = random_scene(11, ntri=50)
    m = scene_matrix(1.0)
    p = Pair(50, 50)
    sh = solid((0.8, 0.1, 0.1, 1.0), m)
    p.clear_color((0.5, 0.5, 0.5, 1))
    run_both(p, mesh, state(), sh)
    p.clear_depth(0.9)
    run_both(p, mesh, state(), sh)
    p.clear_color((0, 0, 0, 0))
    p.clear_depth(MAXF)
    run_both(p, random_scene(12, ntri=50), state(), sh)
    p.check()
    # a clear with no draw after it is applied by the read
    p.clear_color((0.25, 0.5, 0.75, 1))
    assert np.array_equal(p.gpu.Image(), np.broadcast_to(np.array([63, 127, 191, 255], np.uint8), (50, 50, 4)))


# ---------------------------------------------------------------------------
# benchmark scenes at full size
# ---------------------------------------------------------------------------
def phong_scene_shader(w, h):
    return phong(scenes.camera_matrix(w, h), scenes.LIGHT, scenes.EYE, scenes.OBJECT_COLOR)


def test_sphere_512(gpu_lib):
    p = Pair(512, 512)
    p.clear_color(scenes.BACKGROUND)
    assert run_both(p, scenes.sphere_scene(4), state(), phong_scene_shader(512, 512))[0] == 248705
    p.check()


@pytest.fixture(scope="module")
def dense_mesh():
    return scenes.displaced_sphere(8)


def test_dense_mesh_1080p_plain_bit_exact(gpu_lib, dense_mesh):
    p = Pair(1920, 1080)
    p.clear_color(scenes.BACKGROUND)
    run_both(p, dense_mesh, state(), phong_scene_shader(1920, 1080))
    p.check()


def test_dense_mesh_1080p_mixed(gpu_lib, dense_mesh):
    p = Pair(1920, 1080)
    p.clear_color(scenes.BACKGROUND)
    run_both(p, dense_mesh, state(precision=_abi.FGC_PRECISION_MIXED), phong_scene_shader(1920, 1080))
    p.check(mixed=True)


def test_supersampled_overlay_and_downsample(gpu_lib):
    """The 16x-supersampled frame with the wireframe overlay (alpha 0.5,
    DepthBias 1e-5), checked bit-exact at a reduced mesh size, then box
    downsampled on the device."""
    w, h, s = 480 * 4, 270 * 4, 4
    mesh = scenes.displaced_sphere(6)
    p = Pair(w, h)
    p.clear_color(scenes.BACKGROUND)
    sh = phong(scenes.camera_matrix(w, h), scenes.LIGHT, scenes.EYE, scenes.OBJECT_COLOR)
    run_both(p, mesh, state(), sh)
    run_both(p, mesh, state(wireframe=1, depth_bias=1e-5), solid((0, 0, 0, 0.5), scenes.camera_matrix(w, h)))
    p.check()
    ds = p.gpu.Downsample(s)
    assert np.array_equal(ds, O.downsample(p.ref.color(), s))


def test_depth_image(gpu_lib):
    p = Pair(256, 256)
    run_both(p, scenes.sphere_scene(3), state(), phong_scene_shader(256, 256))
    assert np.array_equal(p.gpu.DepthImage(), p.ref.depth_image())


def test_unsupported_shader_kind_is_an_error(gpu_lib):
    ctx = NewContext(8, 8)
    mesh = screen_triangle_mesh([TRI], 8, 8)
    sh = solid((1, 1, 1, 1))
    sh.kind = 9
    info = _abi.FgcRasterizeInfo()
    rc = gpu_lib.fgc_draw_mesh(ctx.handle, _upload_mesh(mesh), ctypes.byref(state()), ctypes.byref(sh),
                               ctypes.byref(info))
    assert rc == _abi.FGC_ERR_UNSUPPORTED_SHADER
    rc = gpu_lib.fgc_draw_triangles(ctx.handle, _upload_mesh(mesh), 0, 5, ctypes.byref(state()),
                                    ctypes.byref(solid((1, 1, 1, 1))), ctypes.byref(info))
    assert rc == _abi.FGC_ERR_INVALID_ARGUMENT
