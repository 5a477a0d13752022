"""Shared builders for the tests: fgc_state / fgc_shader structs, screen-space
triangles, seeded random scenes."""
import math

import numpy as np

from fauxgl_gb300 import _abi
from fauxgl_gb300.geom import Identity
from fauxgl_gb300.mesh import Mesh


def state(**kw):
    s = _abi.FgcState(1, 1, 1, 1, 0, _abi.FGC_FACE_CCW, _abi.FGC_CULL_BACK, 0, 2.0, 0.0)
    for k, v in kw.items():
        setattr(s, k, v)
    return s


def solid(color, matrix=None):
    s = _abi.FgcShader()
    s.kind = _abi.FGC_SHADER_SOLID_COLOR
    s.matrix[:] = list(matrix if matrix is not None else Identity())
    s.color[:] = list(color)
    return s


def phong(matrix, light, eye, color=(0, 0, 0, 0), power=32.0):
    s = _abi.FgcShader()
    s.kind = _abi.FGC_SHADER_PHONG
    s.matrix[:] = list(matrix)
    s.color[:] = list(color)
    s.light_direction[:] = list(light)
    s.camera_position[:] = list(eye)
    s.ambient_color[:] = [0.2, 0.2, 0.2, 1]
    s.diffuse_color[:] = [0.8, 0.8, 0.8, 1]
    s.specular_color[:] = [1, 1, 1, 1]
    s.specular_power = power
    return s


def screen_to_ndc(sx, sy, w, h):
    """Inverse of Screen(w, h) for x and y (exact for dyadic w/2, h/2)."""
    w2, h2 = w / 2.0, h / 2.0
    return (sx - w2) / w2, (h2 - sy) / h2


def screen_triangle_mesh(tris, w, h, z=0.0):
    """Triangles given as screen-space (x, y) corners, drawn with an identity
    matrix: Output = (ndc, 1)."""
    pos = []
    for t in tris:
        pos.append([[*screen_to_ndc(x, y, w, h), z] for (x, y) in t])
    return Mesh(np.array(pos, dtype=np.float64))


def random_scene(seed, ntri=60, nline=0, spread=1.6, with_attrs=True):
    """Seeded random triangles and lines in clip space around the view volume
    (some cross the frustum planes and get clipped), drawn with a matrix that
    puts them in front of the camera."""
    rng = np.random.default_rng(seed)
    centers = rng.uniform(-spread, spread, size=(ntri, 1, 3))
    centers[..., 2] = rng.uniform(-0.9, 1.2, size=(ntri, 1))
    size = rng.uniform(0.02, 0.8, size=(ntri, 1, 1))
    pos = centers + size * rng.normal(size=(ntri, 3, 3))
    nrm = rng.normal(size=(ntri, 3, 3))
    nrm /= np.linalg.norm(nrm, axis=-1, keepdims=True)
    tex = rng.uniform(-0.5, 1.5, size=(ntri, 3, 2)) if with_attrs else None
    col = rng.uniform(0, 1, size=(ntri, 3, 4)) if with_attrs else None
    lp = rng.uniform(-spread, spread, size=(nline, 2, 3))
    lp[..., 2] = rng.uniform(-0.9, 1.2, size=(nline, 2))
    ln = rng.normal(size=(nline, 2, 3))
    return Mesh(pos, nrm, tex, col, lp, ln, rng.uniform(0, 1, size=(nline, 2, 2)),
                rng.uniform(0, 1, size=(nline, 2, 4)))


def scene_matrix(aspect=1.0):
    """A perspective camera looking down -z at the random scenes' volume."""
    from fauxgl_gb300.geom import LookAt, Perspective, V
    return LookAt(V(0.3, 0.2, 4.5), V(0, 0, 0), V(0, 1, 0)).Perspective(45.0, aspect, 1.0, 10.0)


def random_texture(seed, w=13, h=9, transparent_fraction=0.2):
    from fauxgl_gb300.shader import ImageTexture
    rng = np.random.default_rng(seed)
    img = rng.integers(0, 256, size=(h, w, 4), dtype=np.uint16).astype(np.uint8)
    mask = rng.uniform(size=(h, w)) < transparent_fraction
    img[mask] = 0
    return ImageTexture.from_nrgba8(img)
