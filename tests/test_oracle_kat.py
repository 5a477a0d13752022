"""Known-answer tests pinning the oracle (the C restatement of the reference's
pipeline). The reference ships no tests or golden vectors for this path, so
each expected value here is derived independently of the oracle: exact
rational geometry for coverage, the reference's integer formulas restated
in Python for NRGBA and alpha blending, Go's Pow algorithm restated in
Python, and behaviour read off context.go for culling, clipping, depth
flags, Discard and the row wrap-around."""
import math
from fractions import Fraction

import numpy as np
import pytest

from fauxgl_gb300 import _abi, scenes
from fauxgl_gb300.geom import Identity
from fauxgl_gb300.mesh import Mesh
from oracle import oracle as O
from tests.helpers import screen_triangle_mesh, solid, state

MAXF = 1.7976931348623157e308
W = H = 16


def covered(ctx):
    return {(int(x), int(y)) for y, x in zip(*np.nonzero(ctx.winner() != 0xFFFFFFFF))}


def closed_triangle_pixels(tri, w, h):
    """Pixels whose centre lies in the closed triangle (exact rationals)."""
    (ax, ay), (bx, by), (cx, cy) = [(Fraction(x), Fraction(y)) for x, y in tri]

    def e(px, py, x0, y0, x1, y1):
        return (x1 - x0) * (py - y0) - (y1 - y0) * (px - x0)

    area = e(cx, cy, ax, ay, bx, by)
    out = set()
    for y in range(h):
        for x in range(w):
            px, py = Fraction(2 * x + 1, 2), Fraction(2 * y + 1, 2)
            ws = [e(px, py, ax, ay, bx, by), e(px, py, bx, by, cx, cy), e(px, py, cx, cy, ax, ay)]
            if all(v * area >= 0 for v in ws):
                out.add((x, y))
    return out


TRI = [(1, 1), (9, 1), (1, 9)]


def test_single_triangle_coverage_matches_exact_geometry():
    ctx = O.OracleContext(W, H)
    mesh = screen_triangle_mesh([TRI], W, H)
    info = ctx.draw(mesh, state(cull=_abi.FGC_CULL_NONE), solid((1, 0, 0, 1)))
    expect = closed_triangle_pixels(TRI, W, H)
    assert len(expect) == 36
    assert covered(ctx) == expect
    assert info == (36, 36)
    img = ctx.color()
    for (x, y) in expect:
        assert tuple(img[y, x]) == (255, 0, 0, 255)
    # depth: z = 0 in NDC -> 0.5 on screen
    d = ctx.depth()
    assert all(d[y, x] == 0.5 for (x, y) in expect)
    assert (d == MAXF).sum() == W * H - 36


def test_equal_depth_later_triangle_wins():
    ctx = O.OracleContext(W, H)
    mesh = screen_triangle_mesh([TRI, TRI], W, H)
    info = ctx.draw(mesh, state(cull=_abi.FGC_CULL_NONE), solid((0, 1, 0, 1)))
    assert info == (72, 72)  # the second triangle passes bz <= depth on ties
    win = ctx.winner()
    assert set(np.unique(win[win != 0xFFFFFFFF]).tolist()) == {1}


@pytest.mark.parametrize("cull,face,ccw_drawn,cw_drawn", [
    (_abi.FGC_CULL_BACK, _abi.FGC_FACE_CCW, True, False),
    (_abi.FGC_CULL_FRONT, _abi.FGC_FACE_CCW, False, True),
    (_abi.FGC_CULL_BACK, _abi.FGC_FACE_CW, False, True),
    (_abi.FGC_CULL_FRONT, _abi.FGC_FACE_CW, True, False),
    (_abi.FGC_CULL_NONE, _abi.FGC_FACE_CCW, True, True),
])
def test_cull_table(cull, face, ccw_drawn, cw_drawn):
    # NDC y points up, screen y down: TRI = (1,1),(9,1),(1,9) on screen has
    # NDC corners (-7/8,7/8),(1/8,7/8),(-7/8,-1/8) and signed area
    # (1)(-1) - (0)(0) = -1 < 0 (context.go:323): clockwise.
    cw = screen_triangle_mesh([TRI], W, H)
    ccw = screen_triangle_mesh([TRI[::-1]], W, H)
    for mesh, drawn in ((ccw, ccw_drawn), (cw, cw_drawn)):
        ctx = O.OracleContext(W, H)
        info = ctx.draw(mesh, state(cull=cull, front_face=face), solid((1, 1, 1, 1)))
        assert (info[0] > 0) == drawn


def test_discard_counts_but_writes_nothing():
    ctx = O.OracleContext(W, H)
    info = ctx.draw(screen_triangle_mesh([TRI], W, H), state(cull=_abi.FGC_CULL_NONE), solid((0, 0, 0, 0)))
    assert info == (36, 0)
    assert (ctx.depth() == MAXF).all()
    assert (ctx.color() == 0).all()


def test_depth_flags():
    near = screen_triangle_mesh([TRI], W, H, z=-0.5)   # screen z 0.25
    far = screen_triangle_mesh([TRI], W, H, z=0.5)     # screen z 0.75
    st = dict(cull=_abi.FGC_CULL_NONE)
    # WriteDepth off: colour written, depth untouched
    ctx = O.OracleContext(W, H)
    ctx.draw(near, state(write_depth=0, **st), solid((1, 0, 0, 1)))
    assert (ctx.depth() == MAXF).all() and ctx.color()[2, 2, 0] == 255
    # occlusion, then ReadDepth off lets the far triangle overwrite
    ctx = O.OracleContext(W, H)
    ctx.draw(near, state(**st), solid((1, 0, 0, 1)))
    assert ctx.draw(far, state(**st), solid((0, 0, 1, 1))) == (36, 0)
    assert ctx.color()[2, 2, 0] == 255
    assert ctx.draw(far, state(read_depth=0, **st), solid((0, 0, 1, 1))) == (36, 36)
    assert tuple(ctx.color()[2, 2]) == (0, 0, 255, 255) and ctx.depth()[2, 2] == 0.75
    # WriteColor off: depth written, colour kept
    ctx = O.OracleContext(W, H)
    ctx.draw(far, state(write_color=0, **st), solid((1, 0, 0, 1)))
    assert ctx.depth()[2, 2] == 0.75 and (ctx.color() == 0).all()


def test_depth_bias_tests_biased_depth_but_writes_unbiased():
    st = dict(cull=_abi.FGC_CULL_NONE)
    m = screen_triangle_mesh([TRI], W, H)
    ctx = O.OracleContext(W, H)
    ctx.draw(m, state(**st), solid((1, 0, 0, 1)))
    assert ctx.draw(m, state(depth_bias=0.125, **st), solid((0, 1, 0, 1))) == (36, 0)
    assert ctx.draw(m, state(depth_bias=-0.125, **st), solid((0, 0, 1, 1))) == (36, 36)
    assert ctx.depth()[2, 2] == 0.5
    assert tuple(ctx.color()[2, 2]) == (0, 0, 255, 255)


def _go_nrgba(c):
    """color.go:56-63: clamp, *255, truncate."""
    return tuple(0 if math.isnan(v) else int(min(max(v, 0.0), 1.0) * 255) for v in c)


def _go_blend(dst, c):
    """context.go:256-267 with image/color NRGBA.RGBA()."""
    n = _go_nrgba(c)
    a8 = n[3]
    src = [((v | (v << 8)) * a8) // 0xff for v in n[:3]] + [a8 | (a8 << 8)]
    a = (0xffff - src[3]) * 0x101
    return tuple(((d * a // 0xffff + s) >> 8) & 0xff for d, s in zip(dst, src))


@pytest.mark.parametrize("c", [(0.5, 1.2, -0.1, 0.999), (0.0, 1.0, 0.25, 0.5), (float("nan"), 0.7, 1e-9, 1.0),
                               (0.99999, 0.00392156862745098, 0.5019607843137255, 0.0)])
def test_nrgba_quantisation(c):
    assert O.nrgba(c) == _go_nrgba(c)


@pytest.mark.parametrize("dst,c", [((255, 0, 0, 255), (0, 0, 1, 0.5)), ((10, 20, 30, 40), (0.3, 0.6, 0.9, 0.25)),
                                   ((0, 0, 0, 0), (1, 1, 1, 0.999)), ((200, 100, 50, 255), (0.5, 0.5, 0.5, 0.0))])
def test_alpha_blend_integer_arithmetic(dst, c):
    assert O.blend(dst, c) == _go_blend(dst, c)
    if dst == (255, 0, 0, 255):
        assert _go_blend(dst, c) == (128, 0, 127, 255)


def _go_pow_int(x, n):
    """Go math.Pow for x > 0 and integer n >= 1: repeated squaring of the
    Frexp mantissa with exact renormalisation, then Ldexp."""
    x1, xe = math.frexp(x)
    a1, ae = 1.0, 0
    i = n
    while i:
        if i & 1:
            a1 *= x1
            ae += xe
        x1 *= x1
        xe <<= 1
        if x1 < 0.5:
            x1 += x1
            xe -= 1
        i >>= 1
    return math.ldexp(a1, ae)


@pytest.mark.parametrize("x", [0.9, 0.5, 0.123456789, 0.999999, 0.73, 1e-3, 0.5000001])
def test_go_pow_integer_exponent(x):
    assert O.go_pow(x, 32) == _go_pow_int(x, 32)
    assert O.go_pow(x, 7) == _go_pow_int(x, 7)


def test_go_pow_special_cases():
    assert O.go_pow(0.0, 32) == 0.0
    assert math.copysign(1, O.go_pow(-0.0, 3)) < 0
    assert O.go_pow(2.0, 0.5) == math.sqrt(2.0)
    assert O.go_pow(5.0, 0) == 1.0 and O.go_pow(1.0, float("nan")) == 1.0
    assert math.isnan(O.go_pow(-2.0, 0.5))
    assert O.go_pow(0.0, -1) == math.inf


def test_clip_triangle_piece_counts():
    inside = [0.0, 0.0, 0.5, 1.0]
    inside2 = [0.5, 0.0, 0.5, 1.0]
    # one vertex behind the near plane (z < -w): a quad -> 2 triangles
    t = O.clip_triangle([inside, inside2, [0.0, 0.5, -2.0, 1.0]])
    assert t.shape[0] == 2
    # all outside the same plane -> nothing
    assert O.clip_triangle([[2, 0, 0, 1], [3, 0, 0, 1], [2, 1, 0, 1]]).shape[0] == 0
    # crossing x = w and y = w with the hypotenuse x + y = 1.5 cutting the
    # corner: (0,1),(0,0),(1,0),(1,.5),(.5,1), a pentagon -> 3 triangles
    t = O.clip_triangle([[0.0, 0.0, 0.0, 1.0], [1.5, 0.0, 0.0, 1.0], [0.0, 1.5, 0.0, 1.0]])
    assert t.shape[0] == 3
    pts = {(float(x), float(y)) for piece in t for x, y, _, _ in piece}
    assert pts == {(0.0, 1.0), (0.0, 0.0), (1.0, 0.0), (1.0, 0.5), (0.5, 1.0)}
    # a triangle inside except its far corner: the unit square -> 2 triangles
    t = O.clip_triangle([[0.0, 0.0, 0.0, 1.0], [3.0, 0.0, 0.0, 1.0], [0.0, 3.0, 0.0, 1.0]])
    assert t.shape[0] == 2
    for piece in t:
        for x, y, z, w in piece:
            assert abs(x) <= w * (1 + 1e-12) and abs(y) <= w * (1 + 1e-12) and abs(z) <= w * (1 + 1e-12)


def test_row_wraparound_writes_depth_but_not_opaque_colour():
    """context.go:223-228 only range-checks i = y*W + x, so a fat line past
    the right edge lands on the next row; SetNRGBA ignores that (x, y), the
    alpha-blend path writes it."""
    from fauxgl_gb300.geom import Identity
    from tests.helpers import screen_to_ndc
    x0, y0 = screen_to_ndc(15.5, 4.0, W, H)
    x1, y1 = screen_to_ndc(15.5, 10.0, W, H)
    line = Mesh(None, line_pos=np.array([[[x0, y0, 0.0], [x1, y1, 0.0]]]))
    for alpha, expect_colour in ((1.0, False), (0.5, True)):
        ctx = O.OracleContext(W, H)
        ctx.clear_color((0, 0, 0, 1))
        info = ctx.draw(line, state(line_width=4.0), solid((1, 1, 1, alpha)), what=2)
        d = ctx.depth()
        assert info[0] > 0
        # pixels x = 16, 17 of rows 3..10 become x = 0, 1 of rows 4..11
        wrapped = [(y, x) for y in range(4, 12) for x in (0, 1) if d[y, x] != MAXF]
        assert len(wrapped) >= 8
        col = ctx.color()
        assert any(col[y, x, 0] != 0 for (y, x) in wrapped) == expect_colour


def test_threaded_baseline_matches_sequential_on_convex_scene():
    mesh = scenes.sphere_scene(3)
    m = scenes.camera_matrix(200, 200)
    from tests.helpers import phong
    sh = phong(m, scenes.LIGHT, scenes.EYE, scenes.OBJECT_COLOR)
    a = O.OracleContext(200, 200)
    b = O.OracleContext(200, 200)
    ia = a.draw(mesh, state(), sh)
    ib = b.draw(mesh, state(), sh, nthreads=4)
    assert ia[0] == ib[0]
    assert np.array_equal(a.color(), b.color())


def test_depth_image_normalisation():
    ctx = O.OracleContext(W, H)
    ctx.draw(screen_triangle_mesh([TRI], W, H, z=0.0), state(cull=_abi.FGC_CULL_NONE), solid((1, 1, 1, 1)))
    ctx.draw(screen_triangle_mesh([[(10, 10), (15, 10), (10, 15)]], W, H, z=0.5), state(cull=_abi.FGC_CULL_NONE),
             solid((1, 1, 1, 1)))
    g = ctx.depth_image()
    # context.go:87-117 restated over the depth buffer
    d = ctx.depth()
    vals = d[d != MAXF]
    lo, hi = float(vals.min()), float(vals.max())
    for (y, x) in [(2, 2), (11, 11), (12, 10), (0, 15), (5, 5)]:
        v = float(d[y, x])
        t = 1.0 if v == MAXF else (v - lo) / (hi - lo)
        assert g[y, x] == int(t * 0xffff)
    assert g[2, 2] == 0 and g[0, 15] == 0xffff


def test_box_downsample_rounds_to_nearest():
    img = np.zeros((4, 4, 4), dtype=np.uint8)
    img[0, 0] = (1, 2, 3, 255)
    img[0, 1] = (2, 2, 3, 255)
    img[1, 0] = (2, 2, 4, 255)
    img[1, 1] = (2, 3, 4, 254)
    out = O.downsample(img, 2)
    sums = img[:2, :2].reshape(4, 4).astype(int).sum(0)
    assert tuple(out[0, 0]) == tuple((s + 2) // 4 for s in sums)
