"""Host-side scene construction: shapes, mesh processing and camera math in
the reference's operation order."""
import math

import numpy as np
import pytest

from fauxgl_gb300 import scenes
from fauxgl_gb300.geom import HexColor, LookAt, Perspective, Screen, V, Vector
from fauxgl_gb300.mesh import Mesh, NewTriangleForPoints, smooth_normals_threshold_host
from fauxgl_gb300.shapes import NewCone, NewCube, NewCylinder, NewIcosahedron, NewSphere, cylinder_segments


@pytest.mark.parametrize("detail", [0, 1, 2, 4])
def test_sphere_counts_and_unit_radius(detail):
    m = NewSphere(detail)
    assert m.ntri == 20 * 4 ** detail
    r = np.linalg.norm(m.tri_pos, axis=-1)
    assert np.allclose(r, 1.0, atol=1e-15)


def test_sphere_recursion_order():
    """The first child triangle of the first icosahedron face is
    (v1, v12, v13) of that face (shapes.go:125-128)."""
    ico = NewIcosahedron().tri_pos
    s1 = NewSphere(1).tri_pos
    v1, v2, v3 = ico[0]

    def mid(a, b):
        m = (a + b) / 2
        return m * (1 / math.sqrt(m[0] * m[0] + m[1] * m[1] + m[2] * m[2]))

    assert np.array_equal(s1[0], np.array([v1, mid(v1, v2), mid(v1, v3)]))
    assert np.array_equal(s1[3], np.array([mid(v1, v2), mid(v2, v3), mid(v1, v3)]))


def test_face_normals_follow_triangle_normal():
    t = NewTriangleForPoints((0, 0, 0), (1, 0, 0), (0, 1, 0))
    assert tuple(t.V1.Normal) == (0.0, 0.0, 1.0)


def test_biunitcube_fits_the_cube():
    m = scenes.displaced_sphere(3, seed=7)
    lo, hi = m.tri_pos.reshape(-1, 3).min(0), m.tri_pos.reshape(-1, 3).max(0)
    assert (lo >= -1 - 1e-12).all() and (hi <= 1 + 1e-12).all()
    assert np.isclose((hi - lo).max(), 2.0)


def test_smooth_normals_threshold_properties():
    m = scenes.displaced_sphere(3, seed=7)
    n = m.tri_nrm.reshape(-1, 3)
    assert np.allclose(np.linalg.norm(n, axis=-1), 1.0, atol=1e-12)
    # corners sharing a position and a face normal within the threshold
    # end with the same smoothed normal
    m0 = scenes.sphere_scene(2)
    fn = m0.tri_nrm.copy()
    m1 = Mesh(m0.tri_pos, np.repeat(_face(m0.tri_pos)[:, None, :], 3, axis=1))
    smooth_normals_threshold_host(m1, math.radians(89))
    keys = {}
    for p, nn in zip(m1.tri_pos.reshape(-1, 3), m1.tri_nrm.reshape(-1, 3)):
        keys.setdefault(tuple(p), set()).add(tuple(nn))
    assert all(len(v) == 1 for v in keys.values())


def _face(p):
    e1, e2 = p[:, 1] - p[:, 0], p[:, 2] - p[:, 0]
    c = np.cross(e1, e2)
    return c / np.linalg.norm(c, axis=-1, keepdims=True)


def test_smooth_normals_sequential_sum_order():
    """The smoothed normal is the normalised left-to-right sum of the
    qualifying normals in corner order (mesh.go:80-88)."""
    p = np.array([[[0, 0, 0], [1, 0, 0], [0, 1, 0]], [[0, 0, 0], [0, 1, 0], [-1, 0, 0]]], dtype=float)
    n = np.array([[[0.1, 0.2, 0.97], [0, 0, 1], [0, 0, 1]], [[0.3, -0.1, 0.95], [0, 0, 1], [0, 0, 1]]])
    m = Mesh(p, n)
    smooth_normals_threshold_host(m, math.radians(30))
    a, b = Vector(*n[0, 0]), Vector(*n[1, 0])
    expect = Vector(0, 0, 0).Add(a).Add(b).Normalize()
    assert tuple(m.tri_nrm[0, 0]) == tuple(expect)
    assert tuple(m.tri_nrm[1, 0]) == tuple(expect)


def test_camera_matrix_matches_reference_formulas():
    m = scenes.camera_matrix(512, 512)
    # Perspective(30, 1, 1, 10): ymax = tan(15 deg)
    ymax = 1 * math.tan(30 * math.pi / 360)
    p = Perspective(30, 1, 1, 10)
    assert p[0] == 2 / (2 * ymax) and p[5] == 2 / (2 * ymax)
    assert p[10] == (-10 - 1) / 9 and p[11] == (-2 * 10) / 9 and p[14] == -1
    l = LookAt(scenes.EYE, scenes.CENTER, scenes.UP)
    assert m == l.Perspective(30, 1, 1, 10)
    # the eye maps to the origin of view space
    e = l.MulPosition(scenes.EYE)
    assert max(abs(v) for v in e) < 1e-15
    assert Screen(512, 256) == (256, 0, 0, 256, 0, -128, 0, 128, 0, 0, 0.5, 0.5, 0, 0, 0, 1)


def test_hexcolor():
    c = HexColor("#468966")
    assert c == (0x46 / 255, 0x89 / 255, 0x66 / 255, 1.0)
    assert HexColor("FFF8E3").A == 1.0 and HexColor("#abc") == HexColor("aabbcc")


def test_shapes():
    assert NewCube().ntri == 12
    assert NewCylinder(30, True).ntri == 48 and NewCone(30, False).ntri == 12
    assert cylinder_segments(7, capped=True).ntri == 28 and cylinder_segments(513, cone=True).ntri == 1026


def test_displacement_is_seeded_and_keeps_shared_vertices():
    a = scenes.displaced_sphere(2, seed=5)
    b = scenes.displaced_sphere(2, seed=5)
    c = scenes.displaced_sphere(2, seed=6)
    assert np.array_equal(a.tri_pos, b.tri_pos) and not np.array_equal(a.tri_pos, c.tri_pos)
    # the closed surface still has 10*4^d + 2 distinct positions
    assert np.unique(a.tri_pos.reshape(-1, 3), axis=0).shape[0] == 10 * 4 ** 2 + 2


def test_thumbnail_batch_shapes():
    meshes, views = scenes.thumbnail_batch(nmeshes=6, views_per_mesh=2, seed=3, tri_max=5000)
    assert len(meshes) == 6 and len(views) == 12
    assert all(v["width"] in (256, 512, 768, 1024) for v in views)
    assert all(200 // 4 <= m.ntri <= 4 * 5000 for m in meshes)
