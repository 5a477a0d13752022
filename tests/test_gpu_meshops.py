"""GPU parity of the mesh preparation kernels (fgc_meshops.cu) against the
oracle's C restatement (oracle/fauxgl_oracle_mesh.c): LoadSTL, SmoothNormals,
SmoothNormalsThreshold, SharpEdges, Silhouette. Positions and normals are
compared bit for bit; SharpEdges excludes dihedral angles within 1e-9 rad of
the threshold, where CUDA's acos and the C library's may round differently."""
import math
import struct

import numpy as np
import pytest

from fauxgl_gb300 import _abi, scenes
from fauxgl_gb300.meshops import DeviceMesh, LoadSTL
from fauxgl_gb300.mesh import Mesh, face_normals
from fauxgl_gb300.shapes import NewCone, NewCube, NewSphere
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def bits(a):
    return np.ascontiguousarray(a, dtype=np.float64).view(np.uint64)


def same_bits(a, b):
    """Equal bit patterns, any NaN equal to any NaN (payloads differ between
    the CPU and the GPU)."""
    a, b = np.asarray(a, dtype=np.float64), np.asarray(b, dtype=np.float64)
    if a.shape != b.shape:
        return False
    na, nb = np.isnan(a), np.isnan(b)
    return np.array_equal(na, nb) and np.array_equal(bits(np.where(na, 0.0, a)), bits(np.where(nb, 0.0, b)))


def binary_stl(tri_pos, seed=0):
    rng = np.random.default_rng(seed)
    t = np.asarray(tri_pos, dtype=np.float32).reshape(-1, 3, 3)
    out = bytearray(b"fauxgl test solid".ljust(80, b" "))
    out += struct.pack("<I", t.shape[0])
    for tri in t:
        stored = rng.normal(size=3).astype(np.float32)  # ignored by the reader
        out += stored.tobytes() + tri.astype("<f4").tobytes() + struct.pack("<H", 0)
    return bytes(out)


def ascii_stl(tri_pos, fmt="%.9g"):
    lines = ["solid test"]
    for tri in np.asarray(tri_pos).reshape(-1, 3, 3):
        lines.append("  facet normal 0 0 0")
        lines.append("    outer loop")
        for v in tri:
            lines.append("      vertex " + " ".join(fmt % c for c in v))
        lines.append("    endloop")
        lines.append("  endfacet")
    lines.append("endsolid test")
    return ("\n".join(lines) + "\n").encode()


def seeded_mesh(detail=3, seed=5):
    pos = scenes.displace(scenes.sphere_positions(detail), seed)
    m = Mesh(pos)
    m.BiUnitCube()
    m.tri_nrm = np.ascontiguousarray(np.repeat(face_normals(m.tri_pos)[:, None, :], 3, axis=1))
    return m


def tricky_mesh():
    """Shared positions written as -0 and +0, NaN positions, degenerate and
    duplicated triangles."""
    m = seeded_mesh(2, seed=9)
    p = m.tri_pos.copy()
    n = m.tri_nrm.copy()
    extra = np.array([[[0.0, 0.0, 0.0], [1.0, 0.0, 0.0], [0.0, 1.0, 0.0]],
                      [[-0.0, 0.0, -0.0], [0.0, 1.0, 0.0], [-1.0, 0.0, 0.0]],
                      [[0.0, -0.0, 0.0], [0.0, 0.0, 1.0], [1.0, 0.0, 0.0]],
                      [[np.nan, 0.0, 0.0], [1.0, 0.0, 0.0], [0.0, 1.0, 0.0]],
                      [[np.nan, 0.0, 0.0], [1.0, 0.0, 0.0], [0.0, 0.0, 1.0]],
                      [[2.0, 2.0, 2.0], [2.0, 2.0, 2.0], [3.0, 2.0, 2.0]],
                      [[0.0, 0.0, 0.0], [1.0, 0.0, 0.0], [0.0, 1.0, 0.0]]])
    en = np.array([[[0.0, 0.0, 1.0]] * 3, [[0.0, 0.0, 1.0]] * 3, [[0.0, -1.0, 0.0]] * 3,
                   [[0.0, 0.0, 1.0]] * 3, [[0.0, 1.0, 0.0]] * 3, [[0.0, 0.0, 1.0]] * 3,
                   [[0.1, 0.0, 0.99]] * 3])
    return Mesh(np.concatenate([p, extra]), np.concatenate([n, en]))


# ---------------------------------------------------------------------------
# LoadSTL
# ---------------------------------------------------------------------------
def test_load_binary_stl(gpu_lib, tmp_path):
    m = seeded_mesh(4, seed=2)
    data = binary_stl(m.tri_pos)
    path = tmp_path / "mesh.stl"
    path.write_bytes(data)
    got = LoadSTL(str(path))
    pos, nrm = O.stl_parse(data)
    assert got.ntri == m.ntri == pos.shape[0]
    assert same_bits(got.tri_pos, pos)
    assert same_bits(got.tri_nrm, nrm)
    assert same_bits(pos, np.asarray(m.tri_pos, dtype=np.float32).astype(np.float64))


def test_load_ascii_stl(gpu_lib):
    m = seeded_mesh(2, seed=4)
    for fmt in ("%.9g", "%.17e", "%+.3f"):
        data = ascii_stl(m.tri_pos, fmt)
        d = DeviceMesh.load_stl(data)
        got = d.download()
        pos, nrm = O.stl_parse(data)
        assert same_bits(got.tri_pos, pos)
        assert same_bits(got.tri_nrm, nrm)
    # fields that are not numbers read as 0; other lines are ignored
    text = b"solid x\nvertex 1 2 3\n  vertex\t4 abc 6\nvertex 7 8 9 10\nvertex 0x1p-2 1e400 -0\nendsolid\n"
    got = DeviceMesh.load_stl(text).download()
    pos, nrm = O.stl_parse(text)
    assert got.ntri == 1
    assert same_bits(got.tri_pos, pos) and same_bits(got.tri_nrm, nrm)


def test_stl_errors_and_empty(gpu_lib):
    with pytest.raises(_abi.FauxGLError):
        DeviceMesh.load_stl(b"short")
    with pytest.raises(_abi.FauxGLError):
        DeviceMesh.load_stl(b"solid x\n" + b" " * 80 + b"\nvertex 1 2 3\nvertex 4 5 6\n")
    empty = binary_stl(np.zeros((0, 3, 3)))
    assert DeviceMesh.load_stl(empty).ntri == 0


# ---------------------------------------------------------------------------
# smoothing
# ---------------------------------------------------------------------------
@pytest.mark.parametrize("degrees", [0.0, 30.0, 60.0, 180.0])
def test_smooth_normals_threshold(gpu_lib, degrees):
    for m in (seeded_mesh(4, seed=3), tricky_mesh(), NewCube(), NewCone(20, True)):
        d = DeviceMesh.upload(m)
        d.SmoothNormalsThreshold(math.radians(degrees))
        got = d.download().tri_nrm
        want = O.smooth_normals_threshold(m.tri_pos, m.tri_nrm, math.cos(math.radians(degrees)))
        assert same_bits(got, want)


def test_smooth_normals(gpu_lib):
    for m in (seeded_mesh(4, seed=8), tricky_mesh(), NewSphere(2)):
        d = DeviceMesh.upload(m)
        d.SmoothNormals()
        assert same_bits(d.download().tri_nrm, O.smooth_normals(m.tri_pos, m.tri_nrm))
    # the host Mesh method runs the same kernels
    m = tricky_mesh()
    want = O.smooth_normals_threshold(m.tri_pos, m.tri_nrm, math.cos(math.radians(30)))
    m.SmoothNormalsThreshold(math.radians(30))
    assert same_bits(m.tri_nrm, want)


def test_smoothing_keeps_lines_and_draws(gpu_lib):
    """Smoothing changes only triangle normals; a smoothed DeviceMesh draws
    exactly like the host mesh with the same normals."""
    from fauxgl_gb300 import NewContext, NewPhongShader
    m = seeded_mesh(3, seed=6)
    lines = np.array([[[0.0, 0.0, 0.0], [0.5, 0.5, 0.5]], [[-0.5, 0.2, 0.1], [0.3, -0.4, 0.2]]])
    mesh = Mesh(m.tri_pos, m.tri_nrm, line_pos=lines, line_nrm=np.ones_like(lines))
    d = DeviceMesh.upload(mesh)
    d.SmoothNormalsThreshold(math.radians(30))
    back = d.download()
    assert same_bits(back.line_nrm, np.ones_like(lines))
    host = Mesh(back.tri_pos, back.tri_nrm, line_pos=back.line_pos, line_nrm=back.line_nrm)
    sh = NewPhongShader(scenes.camera_matrix(160, 120), scenes.LIGHT, scenes.EYE)
    out = []
    for src in (d, host):
        ctx = NewContext(160, 120)
        ctx.ClearColorBufferWith(scenes.BACKGROUND)
        ctx.Shader = sh
        info = ctx.DrawMesh(src)
        out.append((info.TotalPixels, info.UpdatedPixels, ctx.Image().copy(), ctx.DepthBuffer.copy()))
    assert out[0][:2] == out[1][:2]
    assert np.array_equal(out[0][2], out[1][2])
    assert same_bits(out[0][3], out[1][3])


# ---------------------------------------------------------------------------
# SharpEdges / Silhouette
# ---------------------------------------------------------------------------
def _borderline(tri_pos, threshold):
    fn = face_normals(np.asarray(tri_pos)).reshape(-1, 3)
    ang = []
    edges = {}
    for t, tri in enumerate(np.asarray(tri_pos).reshape(-1, 3, 3)):
        for k in range(3):
            a, b = tuple(tri[k] + 0.0), tuple(tri[(k + 1) % 3] + 0.0)
            key = (min(a, b), max(a, b))
            if key in edges:
                u = edges[key]
                ang.append(math.acos(max(-1.0, min(1.0, float(np.dot(fn[t], fn[u]))))))
        for k in range(3):
            a, b = tuple(tri[k] + 0.0), tuple(tri[(k + 1) % 3] + 0.0)
            edges[(min(a, b), max(a, b))] = t
    return any(abs(x - threshold) < 1e-9 for x in ang)


@pytest.mark.parametrize("degrees", [10.0, 25.0, 44.0, 89.0])
def test_sharp_edges(gpu_lib, degrees):
    thr = math.radians(degrees)
    for m in (seeded_mesh(4, seed=11), NewCube(), NewCone(15, True), tricky_mesh()):
        if _borderline(m.tri_pos, thr):
            continue
        got = DeviceMesh.upload(m).SharpEdges(thr).download()
        want = O.sharp_edges(m.tri_pos, thr)
        assert got.nline == want.shape[0]
        assert same_bits(got.line_pos, want.reshape(-1, 2, 3))
    # a cube has twelve edges at 90 degrees, each reported once
    cube = DeviceMesh.upload(NewCube()).SharpEdges(math.radians(45)).download()
    assert cube.nline == 12


def test_silhouette(gpu_lib):
    for m, eye, off in ((seeded_mesh(4, seed=12), (-3.0, 1.0, -0.75), 0.001),
                        (NewSphere(3), (0.0, 0.0, 5.0), 0.0), (tricky_mesh(), (2.0, 3.0, 4.0), -0.01)):
        got = DeviceMesh.upload(m).Silhouette(eye, off).download()
        want = O.silhouette(m.tri_pos, m.tri_nrm, eye, off)
        assert got.nline == want.shape[0] > 0
        assert same_bits(got.line_pos, want.reshape(-1, 2, 3))
    # the host Mesh method returns the same line mesh
    m = seeded_mesh(3, seed=13)
    assert same_bits(m.Silhouette((1, 2, 3), 0.0).line_pos, O.silhouette(m.tri_pos, m.tri_nrm, (1, 2, 3), 0.0))


def test_line_meshes_draw(gpu_lib):
    """Sharp-edge and silhouette line meshes are drawn like uploaded ones."""
    from fauxgl_gb300 import NewContext, NewSolidColorShader
    m = seeded_mesh(4, seed=14)
    d = DeviceMesh.upload(m)
    edges = d.SharpEdges(math.radians(20))
    host = edges.download()
    sh = NewSolidColorShader(scenes.camera_matrix(200, 150), (0, 0, 0, 1))
    imgs = []
    for src in (edges, host):
        ctx = NewContext(200, 150)
        ctx.Shader = sh
        ctx.DrawMesh(src)
        imgs.append(ctx.Image().copy())
    assert np.array_equal(imgs[0], imgs[1])
