"""ctypes view of the libfauxglcuda C ABI (include/fauxglcuda.h).

The structs here are the exact layouts of fgc_state, fgc_shader and
fgc_rasterize_info. Loading the library fails loudly when it has not been
built: there is no CPU fallback for any drawing call.
"""
import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libfauxglcuda.so")

FGC_OK = 0
FGC_ERR_INVALID_ARGUMENT = 1
FGC_ERR_UNSUPPORTED_SHADER = 2
FGC_ERR_CUDA = 3
FGC_ERR_OUT_OF_MEMORY = 4
FGC_ERR_DEVICE_LIMIT = 5
FGC_ERR_UNSUPPORTED = 6
FGC_ERR_BUSY = 7

FGC_FACE_CW = 1
FGC_FACE_CCW = 2
FGC_CULL_NONE = 1
FGC_CULL_FRONT = 2
FGC_CULL_BACK = 3
FGC_SHADER_SOLID_COLOR = 1
FGC_SHADER_TEXTURE = 2
FGC_SHADER_PHONG = 3
FGC_PRECISION_PLAIN = 0
FGC_PRECISION_MIXED = 1
FGC_DEBUG_WINNER = 1
FGC_DEBUG_SHADED_COLOR = 2


class FgcRasterizeInfo(ctypes.Structure):
    _fields_ = [("total_pixels", ctypes.c_uint64), ("updated_pixels", ctypes.c_uint64)]


class FgcState(ctypes.Structure):
    _fields_ = [
        ("read_depth", ctypes.c_int32),
        ("write_depth", ctypes.c_int32),
        ("write_color", ctypes.c_int32),
        ("alpha_blend", ctypes.c_int32),
        ("wireframe", ctypes.c_int32),
        ("front_face", ctypes.c_int32),
        ("cull", ctypes.c_int32),
        ("precision", ctypes.c_int32),
        ("line_width", ctypes.c_double),
        ("depth_bias", ctypes.c_double),
    ]


def state_default():
    """An fgc_state holding NewContext's defaults (context.go:66-77): ReadDepth,
    WriteDepth, WriteColor and AlphaBlend on, Wireframe off, FaceCCW, CullBack,
    LineWidth 2, DepthBias 0, plain precision. The same values as the
    library's fgc_state_default, built without loading the library."""
    return FgcState(1, 1, 1, 1, 0, FGC_FACE_CCW, FGC_CULL_BACK, FGC_PRECISION_PLAIN, 2.0, 0.0)


class FgcShader(ctypes.Structure):
    _fields_ = [
        ("kind", ctypes.c_int32),
        ("reserved", ctypes.c_int32),
        ("matrix", ctypes.c_double * 16),
        ("color", ctypes.c_double * 4),
        ("light_direction", ctypes.c_double * 3),
        ("camera_position", ctypes.c_double * 3),
        ("ambient_color", ctypes.c_double * 4),
        ("diffuse_color", ctypes.c_double * 4),
        ("specular_color", ctypes.c_double * 4),
        ("specular_power", ctypes.c_double),
        ("texture", ctypes.c_void_p),
    ]


FGC_STAGE_VERTEX, FGC_STAGE_SETUP, FGC_STAGE_CLIP, FGC_STAGE_BIN, FGC_STAGE_RASTER = range(5)
FGC_STAGE_COUNT = 5
STAGE_NAMES = ("vertex", "setup", "clip", "bin", "raster")


class FgcStats(ctypes.Structure):
    _fields_ = [
        ("elements", ctypes.c_uint64),
        ("unique_vertices", ctypes.c_uint64),
        ("clipped", ctypes.c_uint64),
        ("primitives", ctypes.c_uint64),
        ("bin_entries", ctypes.c_uint64),
        ("visited_pixels", ctypes.c_uint64),
        ("covered_pixels", ctypes.c_uint64),
        ("shaded_fragments", ctypes.c_uint64),
        ("updated_pixels", ctypes.c_uint64),
        ("kernel_launches", ctypes.c_uint64),
        ("bands", ctypes.c_uint32),
        ("band_rows", ctypes.c_uint32),
        ("attempts", ctypes.c_uint32),
        ("reserved", ctypes.c_uint32),
        ("stage_ms", ctypes.c_double * FGC_STAGE_COUNT),
    ]


class FgcBatchItem(ctypes.Structure):
    _fields_ = [
        ("context", ctypes.c_void_p),
        ("mesh", ctypes.c_void_p),
        ("tri_first", ctypes.c_uint64),
        ("tri_count", ctypes.c_uint64),
        ("line_first", ctypes.c_uint64),
        ("line_count", ctypes.c_uint64),
        ("state", ctypes.POINTER(FgcState)),
        ("shader", ctypes.POINTER(FgcShader)),
        ("out_nrgba", ctypes.c_void_p),
        ("out_scale", ctypes.c_int32),
        ("reserved", ctypes.c_int32),
    ]


class FgcBatchTuning(ctypes.Structure):
    _fields_ = [
        ("band_pixels", ctypes.c_int32),
        ("prims_per_bin_block", ctypes.c_int32),
        ("fragment_cap", ctypes.c_int32),
        ("use_graph", ctypes.c_int32),
        ("window", ctypes.c_int32),
        ("reserved", ctypes.c_int32),
    ]


# Every exported symbol of include/fauxglcuda.h, with (restype, argtypes).
_P = ctypes.c_void_p
_PP = ctypes.POINTER(ctypes.c_void_p)
_D = ctypes.POINTER(ctypes.c_double)
_I = ctypes.c_int
_I32 = ctypes.c_int32
_U64 = ctypes.c_uint64
_ST = ctypes.POINTER(FgcState)
_SH = ctypes.POINTER(FgcShader)
_INFO = ctypes.POINTER(FgcRasterizeInfo)

SIGNATURES = {
    "fgc_abi_version": (_I32, []),
    "fgc_state_default": (None, [_ST]),
    "fgc_shader_solid_color": (None, [_SH, _D, _D]),
    "fgc_shader_texture": (None, [_SH, _D, _P]),
    "fgc_shader_phong": (None, [_SH, _D, _D, _D]),
    "fgc_last_error": (ctypes.c_char_p, []),
    "fgc_context_create": (_I, [_I32, _I32, _PP]),
    "fgc_context_destroy": (_I, [_P]),
    "fgc_context_size": (_I, [_P, ctypes.POINTER(_I32), ctypes.POINTER(_I32)]),
    "fgc_context_set_debug": (_I, [_P, _I32]),
    "fgc_clear_color": (_I, [_P, _D]),
    "fgc_clear_depth": (_I, [_P, ctypes.c_double]),
    "fgc_mesh_upload": (_I, [_D, _D, _D, _D, _U64, _D, _D, _D, _D, _U64, _PP]),
    "fgc_mesh_release": (_I, [_P]),
    "fgc_mesh_counts": (_I, [_P, ctypes.POINTER(_U64), ctypes.POINTER(_U64)]),
    "fgc_mesh_load_stl": (_I, [ctypes.c_void_p, _U64, _PP]),
    "fgc_mesh_smooth_normals_threshold": (_I, [_P, ctypes.c_double]),
    "fgc_mesh_smooth_normals": (_I, [_P]),
    "fgc_mesh_sharp_edges": (_I, [_P, ctypes.c_double, _PP]),
    "fgc_mesh_silhouette": (_I, [_P, _D, ctypes.c_double, _PP]),
    "fgc_mesh_download": (_I, [_P, _D, _D, _D, _D]),
    "fgc_texture_upload": (_I, [ctypes.POINTER(ctypes.c_uint16), _I32, _I32, _PP]),
    "fgc_texture_release": (_I, [_P]),
    "fgc_draw_mesh": (_I, [_P, _P, _ST, _SH, _INFO]),
    "fgc_draw_triangles": (_I, [_P, _P, _U64, _U64, _ST, _SH, _INFO]),
    "fgc_draw_lines": (_I, [_P, _P, _U64, _U64, _ST, _SH, _INFO]),
    "fgc_read_color": (_I, [_P, ctypes.POINTER(ctypes.c_uint8)]),
    "fgc_read_depth": (_I, [_P, _D]),
    "fgc_write_color": (_I, [_P, ctypes.POINTER(ctypes.c_uint8)]),
    "fgc_write_depth": (_I, [_P, _D]),
    "fgc_depth_image": (_I, [_P, ctypes.POINTER(ctypes.c_uint16)]),
    "fgc_depth_image_noalloc": (_I, [_P, ctypes.POINTER(ctypes.c_uint16)]),
    "fgc_downsample": (_I, [_P, _I32, ctypes.POINTER(ctypes.c_uint8)]),
    "fgc_read_winner": (_I, [_P, ctypes.POINTER(ctypes.c_uint32)]),
    "fgc_read_shaded_color": (_I, [_P, _D]),
    "fgc_context_set_timing": (_I, [_P, _I32]),
    "fgc_context_last_stats": (_I, [_P, ctypes.POINTER(FgcStats)]),
    "fgc_context_set_stream": (_I, [_P, _P]),
    "fgc_debug_lookback": (_I, [ctypes.c_uint32, ctypes.c_uint32]),
    "fgc_measure_fp64_rate": (_I, [_D]),
    "fgc_batch_create": (_I, [_PP]),
    "fgc_batch_destroy": (_I, [_P]),
    "fgc_batch_set_stream": (_I, [_P, _P]),
    "fgc_batch_set_tuning": (_I, [_P, ctypes.POINTER(FgcBatchTuning)]),
    "fgc_batch_get_tuning": (_I, [_P, ctypes.POINTER(FgcBatchTuning)]),
    "fgc_batch_set_timing": (_I, [_P, _I32]),
    "fgc_batch_submit": (_I, [_P, ctypes.POINTER(FgcBatchItem), _U64]),
    "fgc_batch_query": (_I, [_P, ctypes.POINTER(_I32)]),
    "fgc_batch_wait": (_I, [_P, _INFO]),
    "fgc_batch_last_stats": (_I, [_P, ctypes.POINTER(FgcStats)]),
    "fgc_batch_autotune": (_I, [_P, ctypes.POINTER(FgcBatchItem), _U64, _I32, ctypes.POINTER(FgcBatchTuning)]),
}

_lib = None


class FauxGLError(RuntimeError):
    """A libfauxglcuda call returned a non-zero fgc_status."""

    def __init__(self, status, message):
        super().__init__("fgc status %d: %s" % (status, message))
        self.status = status


def load_library(path=None):
    """Load libfauxglcuda.so once and bind every exported symbol.

    Raises RuntimeError when the shared library is missing: the CUDA
    extension is the only implementation of the drawing calls.
    """
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise RuntimeError(
            "libfauxglcuda.so is not built (%s); run __graft_entry__.build() "
            "or python -m fauxgl_gb300.build" % p)
    lib = ctypes.CDLL(p)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib


def check(status):
    """Raise FauxGLError for a non-zero fgc_status."""
    if status != FGC_OK:
        msg = load_library().fgc_last_error()
        raise FauxGLError(status, msg.decode() if msg else "")
    return status


def dptr(a):
    """ctypes double* of a C-contiguous float64 numpy array (or None)."""
    if a is None:
        return None
    return a.ctypes.data_as(_D)
