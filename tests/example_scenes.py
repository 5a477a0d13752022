"""The reference's example scenes as parity inputs: the meshes shipped with
fogleman/fauxgl (examples/*.stl, committed gzipped under tests/golden/examples/)
drawn with the exact call sequence and shader fields of the example program
that uses each one.

  bowser   examples/bowser.go:25-55   LoadSTL, BiUnitCube, SmoothNormalsThreshold(30 deg),
                                      4096x4096 (1024 at scale 4), up +Z, Phong with
                                      ObjectColor FFD34E, DiffuseColor Gray(0.9),
                                      SpecularColor Gray(0.25), SpecularPower 100
  hello    examples/hello.go:19-40    LoadSTL (ASCII), BiUnitCube, SmoothNormalsThreshold(30 deg),
                                      2000x1000, Phong with ObjectColor (0.5, 1, 0.65, 1)
  sphere   examples/shapes.go:68-78   LoadSTL, SmoothNormals, Transform(Scale(2.5)), Phong with
                                      ObjectColor FFFF9D at alpha 0.65 and SpecularPower 0,
                                      then the same mesh again with Wireframe and
                                      DepthBias -1e-5; 1600x1600 (the example's output size;
                                      its scale-4 buffer and its 1,500 randomly placed cubes,
                                      drawn with Go's math/rand, are left out)
  cube     examples/cube.stl          LoadSTL, BiUnitCube; no example draws it: the
                                      benchmark's camera and Phong shader at 512x512

Each scene is one mesh, prepared once, drawn by a list of draws on one
context: (draw state, shader). prepare_host() runs the preparation on the oracle's host mesh (the
checker side); the GPU side uses the library's own LoadSTL and smoothing
kernels (tests/test_gpu_examples.py).
"""
import gzip
import math
import os

from fauxgl_gb300 import _abi, scenes
from fauxgl_gb300.geom import Color, Gray, HexColor, LookAt, Radians, Scale, V
from fauxgl_gb300.shader import NewPhongShader, to_fgc_shader

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
EXAMPLES = os.path.join(GOLDEN, "examples")
BLACK = (0.0, 0.0, 0.0, 1.0)


def stl_bytes(name):
    with gzip.open(os.path.join(EXAMPLES, name + ".stl.gz"), "rb") as f:
        return f.read()


def _state(**kw):
    st = _abi.state_default()
    for k, v in kw.items():
        setattr(st, k, v)
    return st


def _phong(matrix, light, eye, color, **fields):
    sh = NewPhongShader(matrix, light, eye)
    sh.ObjectColor = color
    for k, v in fields.items():
        setattr(sh, k, v)
    return to_fgc_shader(sh)


def scene(name):
    """(stl name, width, height, clear colour, prep, [(state, shader), ...]).
    prep is a list of steps: ("bi_unit_cube",), ("smooth_threshold", radians),
    ("smooth",), ("transform", matrix)."""
    if name == "bowser":
        w = h = 1024 * 4
        eye, center, up = V(3, 1, 0.5), V(0, -0.1, 0), V(0, 0, 1)
        m = LookAt(eye, center, up).Perspective(30, 1024 / 1024, 1, 10)
        sh = _phong(m, V(0.75, 0.25, 1).Normalize(), eye, HexColor("FFD34E"), DiffuseColor=Gray(0.9),
                    SpecularColor=Gray(0.25), SpecularPower=100.0)
        prep = [("bi_unit_cube",), ("smooth_threshold", Radians(30))]
        return "bowser", w, h, BLACK, prep, [(_state(), sh)]
    if name == "hello":
        w, h = 2000, 1000
        eye, center, up = V(-1, -2, 2), V(-0.07, 0, 0), V(0, 0, 1)
        m = LookAt(eye, center, up).Perspective(20, w / h, 1, 50)
        sh = _phong(m, V(-2, 0, 1).Normalize(), eye, Color(0.5, 1, 0.65, 1))
        prep = [("bi_unit_cube",), ("smooth_threshold", Radians(30))]
        return "hello", w, h, BLACK, prep, [(_state(), sh)]
    if name == "sphere":
        w = h = 1600
        eye, center, up = V(3 * 4, 3 * 4, 1.5 * 4), V(0, 0, 0), V(0, 0, 1)
        m = LookAt(eye, center, up).Perspective(30, w / h, 1, 100)
        sh = _phong(m, V(0.75, 0.5, 1).Normalize(), eye, HexColor("FFFF9D").Alpha(0.65), SpecularPower=0.0)
        prep = [("smooth",), ("transform", Scale(V(2.5, 2.5, 2.5)))]
        return "sphere", w, h, BLACK, prep, [(_state(), sh), (_state(wireframe=1, depth_bias=-0.00001), sh)]
    if name == "cube":
        w = h = 512
        sh = _phong(scenes.camera_matrix(w, h), scenes.LIGHT, scenes.EYE, scenes.OBJECT_COLOR)
        return "cube", w, h, scenes.BACKGROUND, [("bi_unit_cube",)], [(_state(), sh)]
    raise KeyError(name)


NAMES = ("bowser", "hello", "sphere", "cube")


def prepare_host(mesh, prep):
    """The preparation steps on a host Mesh, smoothing by the oracle's C
    restatement (mesh.go:80-120); BiUnitCube and Transform are the host
    mirror's (mesh.go:127-130, 167-175)."""
    from oracle import oracle as O
    for step in prep:
        if step[0] == "bi_unit_cube":
            mesh.BiUnitCube()
        elif step[0] == "transform":
            mesh.Transform(step[1])
        elif step[0] == "smooth_threshold":
            mesh.tri_nrm = O.smooth_normals_threshold(mesh.tri_pos, mesh.tri_nrm, math.cos(step[1]))
            mesh.dirty()
        elif step[0] == "smooth":
            mesh.tri_nrm = O.smooth_normals(mesh.tri_pos, mesh.tri_nrm)
            mesh.dirty()
        else:
            raise ValueError(step)
    return mesh


def digests(color, depth, winner):
    """sha256 of the NRGBA bytes, the FP64 depth (little-endian) and the
    winner ids (u32 little-endian) of a frame."""
    import hashlib

    import numpy as np
    return {
        "color": hashlib.sha256(np.ascontiguousarray(color, dtype=np.uint8).tobytes()).hexdigest(),
        "depth": hashlib.sha256(np.ascontiguousarray(depth, dtype="<f8").tobytes()).hexdigest(),
        "winner": hashlib.sha256(np.ascontiguousarray(winner, dtype="<u4").tobytes()).hexdigest(),
    }


def render_oracle(name):
    """The scene on the oracle in the reference's sequential order: (oracle
    context, [RasterizeInfo per draw], prepared host mesh)."""
    from fauxgl_gb300.mesh import Mesh
    from oracle import oracle as O
    stl, w, h, clear, prep, draws = scene(name)
    pos, nrm = O.stl_parse(stl_bytes(stl))
    mesh = prepare_host(Mesh(pos, nrm), prep)
    ref = O.OracleContext(w, h)
    ref.clear_color(clear)
    infos = [ref.draw(mesh, st, sh) for st, sh in draws]
    return ref, infos, mesh
