"""The C-ABI library builds, loads and exports every symbol the public header
declares; host-side argument checking works without a GPU."""
import ctypes
import os
import re

import pytest

from fauxgl_gb300 import _abi
from fauxgl_gb300.shader import NewPhongShader, SolidColorShader, UnsupportedShaderError, to_fgc_shader

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "fauxglcuda.h")


def header_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(fgc_[a-z0-9_]+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib():
    from fauxgl_gb300 import build
    build.build()
    return _abi.load_library()


def test_header_declares_the_reference_surface():
    names = header_functions()
    for n in ("fgc_context_create", "fgc_draw_mesh", "fgc_draw_triangles", "fgc_draw_lines", "fgc_clear_color",
              "fgc_clear_depth", "fgc_read_color", "fgc_read_depth", "fgc_downsample", "fgc_mesh_upload",
              "fgc_texture_upload", "fgc_depth_image"):
        assert n in names


def test_library_exports_every_declared_symbol(lib):
    missing = [n for n in header_functions() if not hasattr(lib, n)]
    assert not missing, missing
    # and the Python binding knows each of them
    assert set(header_functions()) == set(_abi.SIGNATURES)


def test_struct_layouts_match_the_header(lib):
    assert ctypes.sizeof(_abi.FgcState) == 8 * 4 + 16
    assert ctypes.sizeof(_abi.FgcShader) == 8 + 8 * (16 + 4 + 3 + 3 + 4 + 4 + 4 + 1) + 8
    assert ctypes.sizeof(_abi.FgcRasterizeInfo) == 16
    assert ctypes.sizeof(_abi.FgcBatchItem) == 8 * 2 + 8 * 4 + 8 * 3 + 4 * 2
    assert ctypes.sizeof(_abi.FgcBatchTuning) == 24


def test_defaults_without_gpu(lib):
    st = _abi.FgcState()
    lib.fgc_state_default(ctypes.byref(st))
    assert (st.read_depth, st.write_depth, st.write_color, st.alpha_blend, st.wireframe) == (1, 1, 1, 1, 0)
    assert (st.front_face, st.cull, st.line_width, st.depth_bias) == (_abi.FGC_FACE_CCW, _abi.FGC_CULL_BACK, 2.0, 0.0)
    sh = _abi.FgcShader()
    m = (ctypes.c_double * 16)(*[1.0 if i % 5 == 0 else 0.0 for i in range(16)])
    lib.fgc_shader_phong(ctypes.byref(sh), m, (ctypes.c_double * 3)(0, 0, 1), (ctypes.c_double * 3)(0, 0, 5))
    assert sh.kind == _abi.FGC_SHADER_PHONG and sh.specular_power == 32.0
    assert list(sh.ambient_color) == [0.2, 0.2, 0.2, 1.0] and list(sh.diffuse_color) == [0.8, 0.8, 0.8, 1.0]
    declared = int(re.search(r"#define FGC_ABI_VERSION (\d+)", open(HEADER).read()).group(1))
    assert lib.fgc_abi_version() == declared
    # the Python-side defaults (used where the library must not be mapped) agree
    assert bytes(_abi.state_default()) == bytes(st)


def test_argument_errors_without_gpu(lib):
    out = ctypes.c_void_p()
    assert lib.fgc_context_create(0, 10, ctypes.byref(out)) == _abi.FGC_ERR_INVALID_ARGUMENT
    assert b"positive" in lib.fgc_last_error()
    assert lib.fgc_draw_mesh(None, None, None, None, None) == _abi.FGC_ERR_INVALID_ARGUMENT


def test_custom_shader_is_rejected_not_run_on_cpu():
    class MyShader:
        def Vertex(self, v):
            return v

        def Fragment(self, v):
            return (1, 1, 1, 1)

    with pytest.raises(UnsupportedShaderError):
        to_fgc_shader(MyShader())
    # a subclass of a built-in is also custom code
    class Sub(SolidColorShader):
        pass
    with pytest.raises(UnsupportedShaderError):
        to_fgc_shader(Sub([1] * 16, (1, 1, 1, 1)))
    assert to_fgc_shader(NewPhongShader([1] * 16, (0, 0, 1), (0, 0, 5))).kind == _abi.FGC_SHADER_PHONG
