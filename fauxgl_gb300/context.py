"""Context: the drawing API of package fauxgl (context.go) on libfauxglcuda.

Context mirrors the reference's public fields and methods:

    ctx = NewContext(width, height)
    ctx.ClearColorBufferWith(HexColor("#FFF8E3"))
    ctx.Shader = shader                 # a built-in shader
    info = ctx.DrawMesh(mesh)           # RasterizeInfo(TotalPixels, UpdatedPixels)
    img = ctx.Image()                   # (H, W, 4) uint8 NRGBA

Every draw snapshots ReadDepth, WriteDepth, WriteColor, AlphaBlend,
Wireframe, FrontFace, Cull, LineWidth and DepthBias (context.go:40-58) into
an fgc_state and the shader into an fgc_shader, then runs on the GPU. A
shader that is not SolidColorShader, TextureShader or PhongShader raises
UnsupportedShaderError; nothing runs on the CPU. Precision selects the
arithmetic form: PRECISION_PLAIN (FP64 throughout, the reference's results)
or PRECISION_MIXED (FP64 geometry/edges/depth, FP32 shading).
"""
import ctypes
from collections import namedtuple

import numpy as np

from . import _abi
from .geom import Color, Transparent
from .mesh import Line, Mesh, Triangle
from .shader import SolidColorShader, shader_texture, to_fgc_shader
from .geom import Identity

FaceCW = _abi.FGC_FACE_CW
FaceCCW = _abi.FGC_FACE_CCW
CullNone = _abi.FGC_CULL_NONE
CullFront = _abi.FGC_CULL_FRONT
CullBack = _abi.FGC_CULL_BACK
PRECISION_PLAIN = _abi.FGC_PRECISION_PLAIN
PRECISION_MIXED = _abi.FGC_PRECISION_MIXED


class RasterizeInfo(namedtuple("RasterizeInfo", "TotalPixels UpdatedPixels")):
    """context.go:28-38."""

    def Add(self, other):
        return RasterizeInfo(self.TotalPixels + other.TotalPixels, self.UpdatedPixels + other.UpdatedPixels)


def _upload_mesh(mesh):
    """Device handle of a Mesh, uploaded once and cached on the mesh (a
    meshops.DeviceMesh is already on the device)."""
    lib = _abi.load_library()
    from .meshops import DeviceMesh
    if isinstance(mesh, DeviceMesh):
        return mesh.handle
    if mesh._device is not None:
        return mesh._device.handle
    keep = []

    def arr(a):
        if a is None:
            return None
        a = np.ascontiguousarray(a, dtype=np.float64)
        keep.append(a)
        return _abi.dptr(a)

    h = ctypes.c_void_p()
    tri_pos = mesh.tri_pos if mesh.ntri else None
    line_pos = mesh.line_pos if mesh.nline else None
    _abi.check(lib.fgc_mesh_upload(arr(tri_pos), arr(mesh.tri_nrm if mesh.ntri else None),
                                   arr(mesh.tri_tex if mesh.ntri else None), arr(mesh.tri_col if mesh.ntri else None),
                                   mesh.ntri, arr(line_pos), arr(mesh.line_nrm if mesh.nline else None),
                                   arr(mesh.line_tex if mesh.nline else None),
                                   arr(mesh.line_col if mesh.nline else None), mesh.nline, ctypes.byref(h)))
    mesh._device = _DeviceHandle(h.value, lib.fgc_mesh_release)
    return mesh._device.handle


def _draw_handle(mesh):
    """(device handle, owner) of the mesh for one draw: the kept copy of a
    DeviceMesh or a resident Mesh (owner None), else a copy uploaded now from
    the mesh's current arrays and released with its owner -- DrawMesh reads
    the mesh's triangles on every call (context.go:435-439), so an edit
    between draws is always drawn."""
    from .meshops import DeviceMesh
    if isinstance(mesh, DeviceMesh) or getattr(mesh, "resident", False):
        return _upload_mesh(mesh), None
    dm = DeviceMesh.upload(mesh)
    return dm.handle, dm


def _upload_texture(tex):
    lib = _abi.load_library()
    if tex._device is None:
        h = ctypes.c_void_p()
        _abi.check(lib.fgc_texture_upload(tex.texels.ctypes.data_as(ctypes.POINTER(ctypes.c_uint16)),
                                          tex.Width, tex.Height, ctypes.byref(h)))
        tex._device = _DeviceHandle(h.value, lib.fgc_texture_release)
    return tex._device.handle


class _DeviceHandle:
    """Owns a device resource and releases it when collected."""

    def __init__(self, handle, release):
        self.handle = handle
        self._release = release

    def __del__(self):
        if self.handle:
            try:
                self._release(self.handle)
            except Exception:
                pass
            self.handle = None


class Context:
    """Context (context.go:40-58); buffers live on the GPU."""

    def __init__(self, width, height):
        self._lib = _abi.load_library()
        self.Width = int(width)
        self.Height = int(height)
        h = ctypes.c_void_p()
        _abi.check(self._lib.fgc_context_create(self.Width, self.Height, ctypes.byref(h)))
        self._h = _DeviceHandle(h.value, self._lib.fgc_context_destroy)
        self.ClearColor = Transparent
        self.Shader = SolidColorShader(Identity(), Color(1, 0, 1, 1))
        self.ReadDepth = True
        self.WriteDepth = True
        self.WriteColor = True
        self.AlphaBlend = True
        self.Wireframe = False
        self.FrontFace = FaceCCW
        self.Cull = CullBack
        self.LineWidth = 2.0
        self.DepthBias = 0.0
        self.Precision = PRECISION_PLAIN

    @property
    def handle(self):
        return self._h.handle

    # -- state ---------------------------------------------------------------
    def state(self):
        """fgc_state snapshot of the public fields."""
        s = _abi.FgcState()
        s.read_depth = int(bool(self.ReadDepth))
        s.write_depth = int(bool(self.WriteDepth))
        s.write_color = int(bool(self.WriteColor))
        s.alpha_blend = int(bool(self.AlphaBlend))
        s.wireframe = int(bool(self.Wireframe))
        s.front_face = int(self.FrontFace)
        s.cull = int(self.Cull)
        s.precision = int(self.Precision)
        s.line_width = float(self.LineWidth)
        s.depth_bias = float(self.DepthBias)
        return s

    def shader_struct(self):
        tex = shader_texture(self.Shader)
        th = _upload_texture(tex) if tex is not None else None
        return to_fgc_shader(self.Shader, th)

    # -- clears ----------------------------------------------------------------
    def ClearColorBufferWith(self, color):
        c = (ctypes.c_double * 4)(*[float(v) for v in color])
        _abi.check(self._lib.fgc_clear_color(self.handle, c))

    def ClearColorBuffer(self):
        self.ClearColorBufferWith(self.ClearColor)

    def ClearDepthBufferWith(self, value):
        _abi.check(self._lib.fgc_clear_depth(self.handle, float(value)))

    def ClearDepthBuffer(self):
        self.ClearDepthBufferWith(1.7976931348623157e308)

    # -- drawing ---------------------------------------------------------------
    def _info(self, fn, *args):
        info = _abi.FgcRasterizeInfo()
        st = self.state()
        sh = self.shader_struct()
        _abi.check(fn(self.handle, *args, ctypes.byref(st), ctypes.byref(sh), ctypes.byref(info)))
        return RasterizeInfo(int(info.total_pixels), int(info.updated_pixels))

    def DrawMesh(self, mesh):
        """context.go:435-439. A Mesh that is not resident (Mesh.MakeResident)
        is uploaded for this draw from its current arrays."""
        h, _owner = _draw_handle(mesh)
        return self._info(self._lib.fgc_draw_mesh, h)

    def DrawTriangles(self, mesh, first=0, count=None):
        """context.go:413-433 over mesh triangles [first, first+count)."""
        count = mesh.ntri - first if count is None else count
        h, _owner = _draw_handle(mesh)
        return self._info(self._lib.fgc_draw_triangles, h, int(first), int(count))

    def DrawLines(self, mesh, first=0, count=None):
        """context.go:391-411 over mesh lines [first, first+count)."""
        count = mesh.nline - first if count is None else count
        h, _owner = _draw_handle(mesh)
        return self._info(self._lib.fgc_draw_lines, h, int(first), int(count))

    def DrawTriangle(self, t):
        """context.go:370-389 for one Triangle object."""
        assert isinstance(t, Triangle)
        return self.DrawTriangles(Mesh.from_objects([t]))

    def DrawLine(self, l):
        """context.go:351-368 for one Line object."""
        assert isinstance(l, Line)
        return self.DrawLines(Mesh.from_objects([], [l]))

    # -- buffers ---------------------------------------------------------------
    def Image(self):
        """NRGBA colour buffer as an (H, W, 4) uint8 array (context.go:83-85)."""
        out = np.empty((self.Height, self.Width, 4), dtype=np.uint8)
        _abi.check(self._lib.fgc_read_color(self.handle, out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8))))
        return out

    @property
    def ColorBuffer(self):
        return self.Image()

    @property
    def DepthBuffer(self):
        out = np.empty((self.Height, self.Width), dtype=np.float64)
        _abi.check(self._lib.fgc_read_depth(self.handle, _abi.dptr(out)))
        return out

    def SetColorBuffer(self, nrgba):
        a = np.ascontiguousarray(nrgba, dtype=np.uint8)
        _abi.check(self._lib.fgc_write_color(self.handle, a.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8))))

    def SetDepthBuffer(self, depth):
        a = np.ascontiguousarray(depth, dtype=np.float64)
        _abi.check(self._lib.fgc_write_depth(self.handle, _abi.dptr(a)))

    def DepthImage(self):
        """Gray16 depth visualisation (context.go:87-117) as (H, W) uint16."""
        out = np.empty((self.Height, self.Width), dtype=np.uint16)
        _abi.check(self._lib.fgc_depth_image(self.handle, out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint16))))
        return out

    def Downsample(self, scale):
        """Box-downsampled colour buffer, (H/scale, W/scale, 4) uint8."""
        out = np.empty((self.Height // scale, self.Width // scale, 4), dtype=np.uint8)
        _abi.check(self._lib.fgc_downsample(self.handle, int(scale), out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8))))
        return out

    # -- instrumentation ----------------------------------------------------------
    def SetTiming(self, enable):
        """Record CUDA events between the pipeline stages of each draw."""
        _abi.check(self._lib.fgc_context_set_timing(self.handle, int(bool(enable))))

    def LastStats(self):
        """Work counters and stage times (ms) of the last draw."""
        st = _abi.FgcStats()
        _abi.check(self._lib.fgc_context_last_stats(self.handle, ctypes.byref(st)))
        d = {name: int(getattr(st, name)) for name, _ in _abi.FgcStats._fields_ if name != "stage_ms"}
        d["stage_ms"] = {n: float(st.stage_ms[i]) for i, n in enumerate(_abi.STAGE_NAMES)}
        return d

    def SetStream(self, cuda_stream):
        """Issue this context's work on a caller-owned CUDA stream handle (int
        or None for the context's own stream)."""
        _abi.check(self._lib.fgc_context_set_stream(self.handle, cuda_stream or None))

    # -- parity instrumentation -------------------------------------------------
    def SetDebug(self, flags):
        _abi.check(self._lib.fgc_context_set_debug(self.handle, int(flags)))

    def Winner(self):
        out = np.empty((self.Height, self.Width), dtype=np.uint32)
        _abi.check(self._lib.fgc_read_winner(self.handle, out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32))))
        return out

    def ShadedColor(self):
        out = np.empty((self.Height, self.Width, 4), dtype=np.float64)
        _abi.check(self._lib.fgc_read_shaded_color(self.handle, _abi.dptr(out)))
        return out


def NewContext(width, height):
    """context.go:60-81."""
    return Context(width, height)
