"""CPU checks of the oracle's mesh-preparation restatement
(oracle/fauxgl_oracle_mesh.c): known answers for LoadSTL, SharpEdges and
Silhouette, and agreement of its smoothing with the independent host
restatement in fauxgl_gb300.mesh (both follow mesh.go:80-120)."""
import math
import struct

import numpy as np

from fauxgl_gb300 import scenes
from fauxgl_gb300.mesh import Mesh, face_normals, smooth_normals_host, smooth_normals_threshold_host
from fauxgl_gb300.shapes import NewCube, NewSphere
from oracle import oracle as O


def same(a, b):
    a, b = np.asarray(a, dtype=np.float64), np.asarray(b, dtype=np.float64)
    na, nb = np.isnan(a), np.isnan(b)
    return (a.shape == b.shape and np.array_equal(na, nb)
            and np.array_equal(np.where(na, 0.0, a).view(np.uint64), np.where(nb, 0.0, b).view(np.uint64)))


def one_triangle_binary():
    rec = struct.pack("<3f", 9, 9, 9) + struct.pack("<9f", 0, 0, 0, 1, 0, 0, 0, 1, 0) + struct.pack("<H", 0)
    return b"x" * 80 + struct.pack("<I", 1) + rec


def test_stl_known_answers():
    pos, nrm = O.stl_parse(one_triangle_binary())
    assert pos.tolist() == [[[0, 0, 0], [1, 0, 0], [0, 1, 0]]]
    assert nrm.tolist() == [[[0, 0, 1]] * 3]  # the stored normal (9,9,9) is ignored
    text = b"solid s\n facet normal 0 0 0\n  outer loop\n   vertex 0 0 0\n   vertex 0 1 0\n   vertex 1 0 0\n" \
           b"  endloop\n endfacet\nendsolid s\n"
    pos, nrm = O.stl_parse(text)
    assert nrm.tolist() == [[[0, 0, -1]] * 3]
    # FP32 widening: 0.1 is stored as the nearest float
    rec = struct.pack("<3f", 0, 0, 0) + struct.pack("<9f", 0.1, 0, 0, 1, 0, 0, 0, 1, 0) + struct.pack("<H", 0)
    pos, _ = O.stl_parse(b"y" * 80 + struct.pack("<I", 1) + rec)
    assert pos[0, 0, 0] == float(np.float32(0.1)) != 0.1


def test_smoothing_agrees_with_host_restatement():
    for detail, seed in ((3, 1), (4, 2)):
        pos = scenes.displace(scenes.sphere_positions(detail), seed)
        m = Mesh(pos)
        m.BiUnitCube()
        m.tri_nrm = np.ascontiguousarray(np.repeat(face_normals(m.tri_pos)[:, None, :], 3, axis=1))
        for deg in (0.0, 30.0, 75.0):
            h = Mesh(m.tri_pos, m.tri_nrm.copy())
            smooth_normals_threshold_host(h, math.radians(deg))
            assert same(h.tri_nrm, O.smooth_normals_threshold(m.tri_pos, m.tri_nrm, math.cos(math.radians(deg))))
        h = Mesh(m.tri_pos, m.tri_nrm.copy())
        smooth_normals_host(h)
        assert same(h.tri_nrm, O.smooth_normals(m.tri_pos, m.tri_nrm))


def test_map_key_semantics():
    """-0 and +0 are one key; a NaN position finds nothing (SmoothNormals: the
    zero vector; SmoothNormalsThreshold: the normalised zero vector, NaN)."""
    p = np.array([[[0.0, 0, 0], [1, 0, 0], [0, 1, 0]], [[-0.0, 0, 0], [0, 0, 1], [1, 0, 0]],
                  [[np.nan, 0, 0], [1, 0, 0], [0, 1, 0]]])
    n = np.array([[[0, 0, 1.0]] * 3, [[0, 1.0, 0]] * 3, [[0, 0, 1.0]] * 3])
    s = O.smooth_normals(p, n)
    r = 1 / math.sqrt(2)
    assert s[0, 0].tolist() == s[1, 0].tolist() == [0.0, 1 * r, 1 * r]
    assert s[2, 0].tolist() == [0.0, 0.0, 0.0]
    t = O.smooth_normals_threshold(p, n, math.cos(math.radians(100)))
    assert t[0, 0].tolist() == [0.0, r, r] and np.isnan(t[2, 0]).all()


def test_sharp_edges_and_silhouette_known_answers():
    cube = NewCube()
    lines = O.sharp_edges(cube.tri_pos, math.radians(45))
    assert lines.shape == (12, 2, 3)
    d = lines[:, 1] - lines[:, 0]
    assert (np.count_nonzero(d, axis=1) == 1).all()  # every line runs along one axis
    assert O.sharp_edges(cube.tri_pos, math.radians(95)).shape[0] == 0
    s = NewSphere(3)
    eye = np.array([0.0, 0.0, 50.0])
    sil = O.silhouette(s.tri_pos, s.tri_nrm, eye, 0.0)
    assert sil.shape[0] > 0
    pts = sil.reshape(-1, 3)
    nrm = pts / np.linalg.norm(pts, axis=1, keepdims=True)
    # on the unit sphere the silhouette is where the view ray grazes the surface
    assert np.abs(np.einsum("ij,ij->i", nrm, pts - eye)).max() < 0.05 * np.linalg.norm(eye)
