"""Seeded synthetic scenes for the benchmark workloads.

The reference's own benchmark mesh (the Stanford Dragon, README.md:36) is not
available, so these procedurally built meshes of the same scale stand in for
it. Camera, light and colours follow README.md:61-76.

  sphere_scene(detail=4)        icosphere, 5,120 triangles, normals = normalised
                                positions, 512x512
  displaced_sphere(detail=8)    icosphere subdivided 8x (1,310,720 triangles),
                                radius displaced by 8 sine octaves, fit to the
                                bi-unit cube, normals smoothed at 30 degrees
  frame(...)                    camera matrix + Phong shader parameters
  thumbnail_batch(...)          256 seeded meshes x 4 views (batched renders)
"""
import math

import numpy as np

from .geom import HexColor, LookAt, Perspective, Radians, V, Vector
from .mesh import Mesh, _normalize, face_normals, group_rows, smooth_normals_threshold_host
from .shapes import cylinder_segments, sphere_positions

EYE = V(-3, 1, -0.75)
CENTER = V(0, -0.07, 0)
UP = V(0, 1, 0)
LIGHT = V(-0.75, 1, 0.25).Normalize()
OBJECT_COLOR = HexColor("#468966")
BACKGROUND = HexColor("#FFF8E3")
FOVY, NEAR, FAR = 30.0, 1.0, 10.0

_M64 = (1 << 64) - 1


class SplitMix64:
    """splitmix64 generator (Steele, Lea, Flood 2014)."""

    def __init__(self, seed):
        self.state = seed & _M64

    def next(self):
        self.state = (self.state + 0x9E3779B97F4A7C15) & _M64
        z = self.state
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & _M64
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & _M64
        return z ^ (z >> 31)

    def uniform(self):
        """Uniform float in [0, 1) from the top 53 bits."""
        return (self.next() >> 11) * (1.0 / 9007199254740992.0)

    def unit_vector(self):
        """Uniform direction on the unit sphere (z uniform, azimuth uniform)."""
        z = 2 * self.uniform() - 1
        phi = 2 * math.pi * self.uniform()
        r = math.sqrt(max(0.0, 1 - z * z))
        return (r * math.cos(phi), r * math.sin(phi), z)


def camera_matrix(width, height, eye=EYE, center=CENTER, up=UP, fovy=FOVY, near=NEAR, far=FAR):
    """LookAt(eye, center, up).Perspective(fovy, aspect, near, far) as in the examples."""
    aspect = float(width) / float(height)
    return LookAt(eye, center, up).Perspective(fovy, aspect, near, far)


def sphere_scene(detail=4):
    """Unit icosphere with vertex normals equal to the normalised positions."""
    pos = sphere_positions(detail)
    return Mesh(pos, _normalize(pos))


def displace(pos, seed, octaves=8, amplitude=0.15, base_frequency=3.0):
    """Scale each unit-sphere point p by
    1 + sum_k amplitude * 2^-k * sin(K_k . p + phase_k), with |K_k| =
    2^k * base_frequency, K_k's direction and phase_k drawn from
    splitmix64(seed). Equal input positions give equal outputs, so shared
    vertices stay shared."""
    rng = SplitMix64(seed)
    waves = []
    for k in range(octaves):
        d = rng.unit_vector()
        mag = (2.0 ** k) * base_frequency
        waves.append((d[0] * mag, d[1] * mag, d[2] * mag, 2 * math.pi * rng.uniform(), amplitude * 2.0 ** -k))
    flat = np.ascontiguousarray(pos.reshape(-1, 3), dtype=np.float64)
    inv = group_rows(flat)
    first = np.zeros(int(inv.max()) + 1 if inv.size else 0, dtype=np.int64)
    first[inv[::-1]] = np.arange(inv.size)[::-1]  # each group's first row
    uniq = flat[first]
    r = np.ones(uniq.shape[0])
    for kx, ky, kz, ph, amp in waves:
        r = r + amp * np.sin(kx * uniq[:, 0] + ky * uniq[:, 1] + kz * uniq[:, 2] + ph)
    out = uniq * r[:, None]
    return out[inv].reshape(pos.shape)


def displaced_sphere(detail=8, seed=1, smooth_degrees=30.0):
    """Dense-mesh workload: displaced icosphere fit to the bi-unit cube with
    face normals smoothed at the given threshold (the dragon example's
    BiUnitCube + SmoothNormalsThreshold(Radians(30)) preparation)."""
    pos = displace(sphere_positions(detail), seed)
    mesh = Mesh(pos)
    mesh.BiUnitCube()
    fn = face_normals(mesh.tri_pos)
    mesh.tri_nrm = np.ascontiguousarray(np.repeat(fn[:, None, :], 3, axis=1))
    smooth_normals_threshold_host(mesh, Radians(smooth_degrees))
    return mesh


def phong_params(matrix, light=LIGHT, eye=EYE, color=OBJECT_COLOR):
    """NewPhongShader(matrix, light, eye) with ObjectColor = color."""
    return dict(matrix=matrix, light=light, eye=eye, color=color)


def thumbnail_batch(nmeshes=256, views_per_mesh=4, seed=3, tri_min=200, tri_max=200000,
                    resolutions=(256, 512, 768, 1024), build=None):
    """Batched-thumbnail workload: nmeshes seeded meshes whose triangle counts
    are log-uniform in [tri_min, tri_max] (displaced icospheres at the nearest
    subdivision level, cylinders and cones with 8-512 segments), each seen by
    views_per_mesh cameras at radius 3 (azimuth in [0, 2pi), elevation in
    [-30, 45] degrees), per-view square resolution drawn from resolutions,
    random Phong object colour.

    Returns (meshes, views) where views is a list of dicts with keys
    mesh, kind ("sphere", "cylinder" or "cone"), segments (0 for spheres),
    triangles, width, height, matrix, eye, color. build: a set of mesh indices to build
    (the others are None; the draws of the seeded generator are the same)."""
    rng = SplitMix64(seed)
    meshes, kinds = [], []
    for i in range(nmeshes):
        t = math.exp(math.log(tri_min) + rng.uniform() * (math.log(tri_max) - math.log(tri_min)))
        kind = int(rng.uniform() * 3)
        seg = detail = 0
        if kind != 0:
            seg = int(math.exp(math.log(8) + rng.uniform() * (math.log(512) - math.log(8))))
            ntri = seg * (4 if kind == 1 else 2)
        else:
            detail = int(min(6, max(2, round(math.log(t / 20.0, 4)))))
            ntri = 20 * 4 ** detail
        kinds.append((("sphere", "cylinder", "cone")[kind], seg, ntri))
        if build is not None and i not in build:
            meshes.append(None)
        elif kind == 0:
            pos = displace(sphere_positions(detail), seed * 1000003 + i)
            m = Mesh(pos)
            m.BiUnitCube()
            fn = face_normals(m.tri_pos)
            m.tri_nrm = np.ascontiguousarray(np.repeat(fn[:, None, :], 3, axis=1))
            smooth_normals_threshold_host(m, Radians(30.0))
        else:
            m = cylinder_segments(seg, capped=True, cone=(kind == 2))
            m.BiUnitCube()
        if build is None or i in build:
            meshes.append(m)
    views = []
    for i in range(nmeshes):
        for _ in range(views_per_mesh):
            az = 2 * math.pi * rng.uniform()
            el = Radians(-30.0 + 75.0 * rng.uniform())
            eye = Vector(3 * math.cos(el) * math.cos(az), 3 * math.sin(el), 3 * math.cos(el) * math.sin(az))
            res = resolutions[int(rng.uniform() * len(resolutions))]
            color = (rng.uniform(), rng.uniform(), rng.uniform(), 1.0)
            views.append(dict(mesh=i, kind=kinds[i][0], segments=kinds[i][1], triangles=kinds[i][2], width=res, height=res, eye=eye,
                              matrix=camera_matrix(res, res, eye=eye, center=V(0, 0, 0)), color=color))
    return meshes, views


def thumbnail_check_views(views, count=16):
    """A seeded subset of the thumbnail batch that covers it: the first view
    of every (shape kind, resolution) pair, then views of the cylinders and
    cones with the fewest and the most segments and of the largest meshes,
    until count views are taken. Returns view indices in batch order."""
    picked, seen = [], set()
    for i, v in enumerate(views):
        key = (v["kind"], v["width"])
        if key not in seen:
            seen.add(key)
            picked.append(i)
    lathe = [i for i, v in enumerate(views) if v["kind"] != "sphere"]
    cands = []
    if lathe:
        cands += [min(lathe, key=lambda i: views[i]["segments"]), max(lathe, key=lambda i: views[i]["segments"])]
    cands += sorted(range(len(views)), key=lambda i: (-views[i]["triangles"], -views[i]["width"], i))
    for i in cands:
        if len(picked) >= count:
            break
        if i not in picked:
            picked.append(i)
    return sorted(picked)
