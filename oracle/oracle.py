"""TEST INFRASTRUCTURE ONLY: ctypes access to the C restatement of the
reference pipeline (oracle/fauxgl_oracle.c).

Used by tests/ as the checker, by __graft_entry__.smoke() to check one small
draw, and by bench.py's CPU-baseline leg. Never used by the product.

Parity unpinned: the reference has no golden vectors for this path and cannot
be built on either machine (no Go toolchain); the restatement is pinned by the
hand-derived known-answer tests in tests/test_oracle_kat.py.
"""
import ctypes
import os
import subprocess

import numpy as np

from fauxgl_gb300 import _abi

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "libfauxgl_oracle.so")
_lib = None


def build():
    """Compile the oracle with its Makefile (gcc, -ffp-contract=off)."""
    subprocess.run(["make", "-s", "-C", _HERE], check=True)


def load():
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        build()
    lib = ctypes.CDLL(LIB_PATH)
    P = ctypes.c_void_p
    D = ctypes.POINTER(ctypes.c_double)
    U8 = ctypes.POINTER(ctypes.c_uint8)
    U16 = ctypes.POINTER(ctypes.c_uint16)
    lib.oracle_create.restype = P
    lib.oracle_create.argtypes = [ctypes.c_int32, ctypes.c_int32]
    lib.oracle_destroy.argtypes = [P]
    lib.oracle_clear_color.argtypes = [P, D]
    lib.oracle_clear_depth.argtypes = [P, ctypes.c_double]
    lib.oracle_draw.restype = ctypes.c_int
    lib.oracle_draw.argtypes = [P, ctypes.POINTER(_abi.FgcState), ctypes.POINTER(_abi.FgcShader), U16,
                                ctypes.c_int32, ctypes.c_int32, D, D, D, D, ctypes.c_int64, ctypes.c_int64,
                                D, D, D, D, ctypes.c_int64, ctypes.c_int64, ctypes.c_int32, ctypes.c_int32,
                                ctypes.POINTER(_abi.FgcRasterizeInfo)]
    for name, t in (("oracle_color", U8), ("oracle_depth", D), ("oracle_winner", ctypes.POINTER(ctypes.c_uint32)),
                    ("oracle_shaded", D)):
        getattr(lib, name).restype = t
        getattr(lib, name).argtypes = [P]
    lib.oracle_downsample.argtypes = [U8, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, U8]
    lib.oracle_depth_image.argtypes = [P, U16]
    lib.oracle_go_pow.restype = ctypes.c_double
    lib.oracle_go_pow.argtypes = [ctypes.c_double, ctypes.c_double]
    lib.oracle_nrgba.argtypes = [D, U8]
    lib.oracle_blend.argtypes = [U8, D]
    lib.oracle_clip_triangle.restype = ctypes.c_int
    lib.oracle_clip_triangle.argtypes = [D, D]
    U64 = ctypes.c_uint64
    lib.oracle_stl_parse.restype = ctypes.c_int64
    lib.oracle_stl_parse.argtypes = [U8, U64, D, D, U64]
    lib.oracle_smooth_normals_threshold.argtypes = [D, D, U64, ctypes.c_double]
    lib.oracle_smooth_normals.argtypes = [D, D, U64]
    lib.oracle_sharp_edges.restype = ctypes.c_int64
    lib.oracle_sharp_edges.argtypes = [D, U64, ctypes.c_double, D, U64]
    lib.oracle_silhouette.restype = ctypes.c_int64
    lib.oracle_silhouette.argtypes = [D, D, U64, D, ctypes.c_double, D, U64]
    _lib = lib
    return lib


def _d(a):
    return None if a is None else np.ascontiguousarray(a, dtype=np.float64).ctypes.data_as(
        ctypes.POINTER(ctypes.c_double))


class OracleContext:
    """NewContext(width, height) on the CPU restatement."""

    def __init__(self, width, height):
        self.lib = load()
        self.width, self.height = int(width), int(height)
        self.h = self.lib.oracle_create(self.width, self.height)

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.oracle_destroy(self.h)
            self.h = None

    def clear_color(self, rgba):
        c = np.asarray(rgba, dtype=np.float64)
        self.lib.oracle_clear_color(self.h, _d(c))

    def clear_depth(self, value):
        self.lib.oracle_clear_depth(self.h, float(value))

    def draw(self, mesh, state, shader, texture=None, what=3, nthreads=0,
             tri_range=None, line_range=None):
        """Draw a Mesh with an fgc_state / fgc_shader pair; returns
        (total_pixels, updated_pixels). what: 1 triangles, 2 lines, 3 both."""
        keep = []

        def arr(a):
            if a is None:
                return None
            a = np.ascontiguousarray(a, dtype=np.float64)
            keep.append(a)
            return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))

        tf, tc = tri_range if tri_range is not None else (0, mesh.ntri)
        lf, lc = line_range if line_range is not None else (0, mesh.nline)
        tex_ptr, tw, th = None, 0, 0
        if texture is not None:
            t = np.ascontiguousarray(texture.texels, dtype=np.uint16)
            keep.append(t)
            tex_ptr = t.ctypes.data_as(ctypes.POINTER(ctypes.c_uint16))
            tw, th = texture.Width, texture.Height
        info = _abi.FgcRasterizeInfo()
        rc = self.lib.oracle_draw(self.h, ctypes.byref(state), ctypes.byref(shader), tex_ptr, tw, th,
                                  arr(mesh.tri_pos), arr(mesh.tri_nrm), arr(mesh.tri_tex), arr(mesh.tri_col),
                                  tf, tc, arr(mesh.line_pos), arr(mesh.line_nrm), arr(mesh.line_tex),
                                  arr(mesh.line_col), lf, lc, what, nthreads, ctypes.byref(info))
        if rc != 0:
            raise RuntimeError("oracle_draw failed with status %d" % rc)
        return int(info.total_pixels), int(info.updated_pixels)

    def _view(self, fn, dtype, count):
        p = fn(self.h)
        return np.ctypeslib.as_array(p, shape=(count,)).astype(dtype, copy=True)

    def color(self):
        return self._view(self.lib.oracle_color, np.uint8, self.width * self.height * 4).reshape(
            self.height, self.width, 4)

    def depth(self):
        return self._view(self.lib.oracle_depth, np.float64, self.width * self.height).reshape(
            self.height, self.width)

    def winner(self):
        return self._view(self.lib.oracle_winner, np.uint32, self.width * self.height).reshape(
            self.height, self.width)

    def shaded(self):
        return self._view(self.lib.oracle_shaded, np.float64, self.width * self.height * 4).reshape(
            self.height, self.width, 4)

    def depth_image(self):
        out = np.empty(self.width * self.height, dtype=np.uint16)
        self.lib.oracle_depth_image(self.h, out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint16)))
        return out.reshape(self.height, self.width)


def frame_error(image, depth, winner, ref, shaded=None):
    """Accuracy of a rendered frame against the oracle's frame `ref` (an
    OracleContext drawn with the same calls): the checker behind the parity
    tests and the benchmark's accuracy report.

    Colour errors are per channel of the NRGBA bytes, as fractions of full
    scale (1/255 = one step): max_err is the largest, mean_err the mean over
    every channel of every pixel. winner_mismatch_frac is the fraction of
    pixels whose last updating element differs, depth_mismatch_frac the
    fraction whose FP64 depth differs in any bit. With `shaded` (the FP64 /
    FP32 shader output the GPU kept per pixel), shaded_max_err is the largest
    per-channel difference from the oracle's FP64 shader output over the
    pixels whose winners agree and whose values are finite."""
    img = np.asarray(image, dtype=np.uint8)
    rc = ref.color()
    diff = np.abs(img.astype(np.int16) - rc.astype(np.int16))
    npx = img.shape[0] * img.shape[1]
    gw, rw = np.asarray(winner), ref.winner()
    gd = np.ascontiguousarray(depth, dtype=np.float64).view(np.uint64)
    rd = ref.depth().view(np.uint64)
    out = {
        "pixels": int(npx),
        "max_err": round(float(diff.max(initial=0)) / 255.0, 6),
        "mean_err": float("%.3g" % (float(diff.mean()) / 255.0)) if diff.size else 0.0,
        "max_err_steps": int(diff.max(initial=0)),
        "channels_off": int((diff != 0).sum()),
        "winner_mismatch_frac": float(int((gw != rw).sum())) / max(npx, 1),
        "depth_mismatch_frac": float(int((gd != rd).sum())) / max(npx, 1),
    }
    if shaded is not None:
        gs, rs = np.asarray(shaded, dtype=np.float64), ref.shaded()
        ok = (gw == rw)[..., None] & np.isfinite(gs) & np.isfinite(rs)
        d = np.abs(gs - rs)[ok]
        out["shaded_max_err"] = float("%.3g" % float(d.max(initial=0.0)))
        out["shaded_mean_err"] = float("%.3g" % float(d.mean())) if d.size else 0.0
    return out


def downsample(img, scale):
    """Box downsample of an (H, W, 4) uint8 image (the project's definition)."""
    lib = load()
    img = np.ascontiguousarray(img, dtype=np.uint8)
    h, w = img.shape[:2]
    out = np.empty((h // scale, w // scale, 4), dtype=np.uint8)
    lib.oracle_downsample(img.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)), w, h, scale,
                          out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)))
    return out


def go_pow(x, y):
    return load().oracle_go_pow(float(x), float(y))


def nrgba(c):
    out = np.zeros(4, dtype=np.uint8)
    load().oracle_nrgba(_d(np.asarray(c, dtype=np.float64)), out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)))
    return tuple(int(v) for v in out)


def blend(dst, src):
    d = np.asarray(dst, dtype=np.uint8).copy()
    s = np.asarray(src, dtype=np.float64)
    load().oracle_blend(d.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)), _d(s))
    return tuple(int(v) for v in d)


def clip_triangle(clip):
    """ClipTriangle on clip-space outputs only: (3,4) -> (n,3,4)."""
    c = np.ascontiguousarray(clip, dtype=np.float64).reshape(12)
    out = np.zeros(7 * 3 * 4)
    n = load().oracle_clip_triangle(_d(c), _d(out))
    return out.reshape(7, 3, 4)[:n].copy()


# ---------------------------------------------------------------------------
# mesh preparation (fauxgl_oracle_mesh.c)
# ---------------------------------------------------------------------------
def stl_parse(data):
    """LoadSTL on bytes: (tri_pos (T,3,3), tri_nrm (T,3,3)); raises ValueError
    where the reference errors."""
    lib = load()
    buf = np.frombuffer(bytes(data), dtype=np.uint8)
    ptr = buf.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8))
    n = lib.oracle_stl_parse(ptr, buf.size, None, None, 0)
    if n < 0:
        raise ValueError("not an STL file the reference reads (%d)" % n)
    pos = np.zeros((max(n, 1), 3, 3))
    nrm = np.zeros((max(n, 1), 3, 3))
    lib.oracle_stl_parse(ptr, buf.size, _d2(pos), _d2(nrm), n)
    return pos[:n], nrm[:n]


def _d2(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def smooth_normals_threshold(tri_pos, tri_nrm, threshold):
    """Mesh.SmoothNormalsThreshold with threshold = cos(radians) given."""
    pos = np.ascontiguousarray(tri_pos, dtype=np.float64)
    nrm = np.ascontiguousarray(tri_nrm, dtype=np.float64).copy()
    load().oracle_smooth_normals_threshold(_d2(pos), _d2(nrm), pos.shape[0], float(threshold))
    return nrm


def smooth_normals(tri_pos, tri_nrm):
    pos = np.ascontiguousarray(tri_pos, dtype=np.float64)
    nrm = np.ascontiguousarray(tri_nrm, dtype=np.float64).copy()
    load().oracle_smooth_normals(_d2(pos), _d2(nrm), pos.shape[0])
    return nrm


def sharp_edges(tri_pos, angle_threshold):
    """Mesh.SharpEdges: line positions (L, 2, 3) in the reference's order."""
    lib = load()
    pos = np.ascontiguousarray(tri_pos, dtype=np.float64)
    n = lib.oracle_sharp_edges(_d2(pos), pos.shape[0], float(angle_threshold), None, 0)
    out = np.zeros((max(n, 1), 2, 3))
    lib.oracle_sharp_edges(_d2(pos), pos.shape[0], float(angle_threshold), _d2(out), n)
    return out[:n]


def silhouette(tri_pos, tri_nrm, eye, offset):
    """Mesh.Silhouette: line positions (L, 2, 3) in the reference's order."""
    lib = load()
    pos = np.ascontiguousarray(tri_pos, dtype=np.float64)
    nrm = np.ascontiguousarray(tri_nrm, dtype=np.float64)
    e = np.ascontiguousarray(eye, dtype=np.float64)
    n = lib.oracle_silhouette(_d2(pos), _d2(nrm), pos.shape[0], _d2(e), float(offset), None, 0)
    out = np.zeros((max(n, 1), 2, 3))
    lib.oracle_silhouette(_d2(pos), _d2(nrm), pos.shape[0], _d2(e), float(offset), _d2(out), n)
    return out[:n]
