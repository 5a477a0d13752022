"""Built-in shapes of package fauxgl (shapes.go), generated as arrays.

Every shape keeps the reference's triangle order and per-vertex arithmetic,
and each triangle gets its face normal as NewTriangleForPoints ->
NewTriangle -> FixNormals gives it (triangle.go:7-11, 46-58).
"""
import math

import numpy as np

from .geom import Radians
from .mesh import Mesh, _normalize, face_normals

# NewIcosahedron (shapes.go:189-236).
_ICO_A = 0.8506507174597755
_ICO_B = 0.5257312591858783
_ICO_VERTS = np.array([
    [-_ICO_A, -_ICO_B, 0], [-_ICO_A, _ICO_B, 0], [-_ICO_B, 0, -_ICO_A], [-_ICO_B, 0, _ICO_A],
    [0, -_ICO_A, -_ICO_B], [0, -_ICO_A, _ICO_B], [0, _ICO_A, -_ICO_B], [0, _ICO_A, _ICO_B],
    [_ICO_B, 0, -_ICO_A], [_ICO_B, 0, _ICO_A], [_ICO_A, -_ICO_B, 0], [_ICO_A, _ICO_B, 0],
], dtype=np.float64)
_ICO_FACES = np.array([
    [0, 3, 1], [1, 3, 7], [2, 0, 1], [2, 1, 6], [4, 0, 2], [4, 5, 0], [5, 3, 0], [6, 1, 7],
    [6, 7, 11], [7, 3, 9], [8, 2, 6], [8, 4, 2], [8, 6, 11], [8, 10, 4], [8, 11, 10], [9, 3, 5],
    [10, 5, 4], [10, 9, 5], [11, 7, 9], [11, 9, 10],
], dtype=np.int64)


def _with_face_normals(tri_pos):
    tri_pos = np.ascontiguousarray(tri_pos, dtype=np.float64)
    n = face_normals(tri_pos)
    return Mesh(tri_pos, np.repeat(n[:, None, :], 3, axis=1))


def NewIcosahedron():
    return _with_face_normals(_ICO_VERTS[_ICO_FACES])


def sphere_positions(detail):
    """NewSphere's triangle positions (shapes.go:107-133).

    The recursion emits, for each triangle, its four children
    (v1,v12,v13), (v2,v23,v12), (v3,v13,v23), (v12,v23,v13) in that order,
    depth first. Expanding every triangle of a level into its four children
    in place yields the same order, so the levels are computed as arrays.
    """
    tris = _ICO_VERTS[_ICO_FACES]
    for _ in range(detail):
        v1, v2, v3 = tris[:, 0], tris[:, 1], tris[:, 2]
        v12 = _normalize((v1 + v2) / 2)  # v1.Add(v2).DivScalar(2).Normalize()
        v13 = _normalize((v1 + v3) / 2)
        v23 = _normalize((v2 + v3) / 2)
        kids = np.stack([np.stack([v1, v12, v13], 1), np.stack([v2, v23, v12], 1),
                         np.stack([v3, v13, v23], 1), np.stack([v12, v23, v13], 1)], axis=1)
        tris = kids.reshape(-1, 3, 3)
    return np.ascontiguousarray(tris)


def NewSphere(detail):
    """shapes.go:107-117: icosphere with 20 * 4**detail triangles."""
    return _with_face_normals(sphere_positions(detail))


def NewPlane():
    """shapes.go:5-14."""
    v1, v2, v3, v4 = (-0.5, -0.5, 0), (0.5, -0.5, 0), (0.5, 0.5, 0), (-0.5, 0.5, 0)
    return _with_face_normals(np.array([[v1, v2, v3], [v1, v3, v4]], dtype=np.float64))


def NewCube():
    """shapes.go:16-37 (unit cube scaled by 0.5)."""
    v = np.array([[-1, -1, -1], [-1, -1, 1], [-1, 1, -1], [-1, 1, 1],
                  [1, -1, -1], [1, -1, 1], [1, 1, -1], [1, 1, 1]], dtype=np.float64)
    idx = [[3, 5, 7], [5, 3, 1], [0, 6, 4], [6, 0, 2], [0, 5, 1], [5, 0, 4],
           [5, 6, 7], [6, 5, 4], [6, 3, 7], [3, 6, 2], [0, 3, 2], [3, 0, 1]]
    m = _with_face_normals(v[np.array(idx)])
    from .geom import Scale
    m.Transform(Scale((0.5, 0.5, 0.5)))
    return m


def _ring(a0, a1):
    r0, r1 = Radians(float(a0)), Radians(float(a1))
    return math.cos(r0), math.sin(r0), math.cos(r1), math.sin(r1)


def NewCylinder(step, capped):
    """shapes.go:135-163 (integer degree step)."""
    tris = []
    for a0 in range(0, 360, step):
        a1 = (a0 + step) % 360
        x0, y0, x1, y1 = _ring(a0, a1)
        p00, p10, p11, p01 = (x0, y0, -0.5), (x1, y1, -0.5), (x1, y1, 0.5), (x0, y0, 0.5)
        tris += [[p00, p10, p11], [p00, p11, p01]]
        if capped:
            tris += [[(0, 0, -0.5), p10, p00], [(0, 0, 0.5), p01, p11]]
    return _with_face_normals(np.array(tris, dtype=np.float64))


def NewCone(step, capped):
    """shapes.go:165-187 (integer degree step)."""
    tris = []
    for a0 in range(0, 360, step):
        a1 = (a0 + step) % 360
        x0, y0, x1, y1 = _ring(a0, a1)
        p00, p10 = (x0, y0, -0.5), (x1, y1, -0.5)
        tris.append([p00, p10, (0, 0, 0.5)])
        if capped:
            tris.append([(0, 0, -0.5), p10, p00])
    return _with_face_normals(np.array(tris, dtype=np.float64))


def cylinder_segments(segments, capped=True, cone=False):
    """NewCylinder / NewCone restated with a real-valued angle step so any
    segment count can be built (the reference's integer degree step only
    expresses divisors of 360). Segment k spans angles 2*pi*k/n to
    2*pi*(k+1)/n; the triangle pattern per segment is the reference's."""
    k = np.arange(segments, dtype=np.float64)
    a0 = 2 * math.pi * k / segments
    a1 = 2 * math.pi * ((k + 1) % segments) / segments
    x0, y0, x1, y1 = np.cos(a0), np.sin(a0), np.cos(a1), np.sin(a1)
    lo, hi = np.full_like(x0, -0.5), np.full_like(x0, 0.5)
    zero = np.zeros_like(x0)
    p00 = np.stack([x0, y0, lo], -1)
    p10 = np.stack([x1, y1, lo], -1)
    p11 = np.stack([x1, y1, hi], -1)
    p01 = np.stack([x0, y0, hi], -1)
    c0 = np.stack([zero, zero, lo], -1)
    c1 = np.stack([zero, zero, hi], -1)
    if cone:
        per = [np.stack([p00, p10, c1], 1)]
        if capped:
            per.append(np.stack([c0, p10, p00], 1))
    else:
        per = [np.stack([p00, p10, p11], 1), np.stack([p00, p11, p01], 1)]
        if capped:
            per += [np.stack([c0, p10, p00], 1), np.stack([c1, p01, p11], 1)]
    tris = np.stack(per, axis=1).reshape(-1, 3, 3)
    return _with_face_normals(tris)
