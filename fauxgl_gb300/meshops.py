"""Mesh preparation on the GPU through libfauxglcuda: LoadSTL, SmoothNormalsThreshold,
SmoothNormals, SharpEdges and Silhouette (stl.go:23-154, mesh.go:80-120, 207-209,
258-292, silhouette.go:3-53).

DeviceMesh is a mesh resident on the GPU (an fgc_mesh handle). Context.DrawMesh,
DrawTriangles, DrawLines and Batch.Add accept it like a Mesh, so a loaded and
smoothed mesh is drawn without a round trip through the host:

    m = DeviceMesh.load_stl("bunny.stl")
    m.SmoothNormalsThreshold(Radians(30))
    edges = m.SharpEdges(Radians(40))        # a line mesh, also on the GPU
    ctx.DrawMesh(m); ctx.DrawMesh(edges)

The host Mesh methods of the same names run these kernels too (upload, operate,
download). Results carry the reference's FP64 bits; SharpEdges compares CUDA's acos
with the threshold (an angle within an ulp or two of it may be decided differently
from Go's math.Acos).
"""
import ctypes
import os

import numpy as np

from . import _abi


def _lib():
    return _abi.load_library()


class DeviceMesh:
    """A mesh on the GPU (fgc_mesh)."""

    def __init__(self, handle):
        from .context import _DeviceHandle
        self._h = _DeviceHandle(handle, _lib().fgc_mesh_release)

    @property
    def handle(self):
        return self._h.handle

    # -- construction ------------------------------------------------------------
    @classmethod
    def upload(cls, mesh):
        """A device copy of a host Mesh (triangles, lines and their attributes)."""
        lib = _lib()
        keep = []

        def arr(a):
            if a is None:
                return None
            a = np.ascontiguousarray(a, dtype=np.float64)
            keep.append(a)
            return _abi.dptr(a)

        h = ctypes.c_void_p()
        t, l = mesh.ntri, mesh.nline
        _abi.check(lib.fgc_mesh_upload(arr(mesh.tri_pos if t else None), arr(mesh.tri_nrm if t else None),
                                       arr(mesh.tri_tex if t else None), arr(mesh.tri_col if t else None), t,
                                       arr(mesh.line_pos if l else None), arr(mesh.line_nrm if l else None),
                                       arr(mesh.line_tex if l else None), arr(mesh.line_col if l else None), l,
                                       ctypes.byref(h)))
        return cls(h.value)

    @classmethod
    def load_stl(cls, source):
        """LoadSTL (stl.go:23-57) from a path or the file's bytes: binary when the
        size is 84 + 50 * count, else ASCII; face normals computed on the GPU."""
        if isinstance(source, (bytes, bytearray, memoryview)):
            data = bytes(source)
        else:
            with open(os.fspath(source), "rb") as f:
                data = f.read()
        buf = ctypes.create_string_buffer(data, len(data))
        h = ctypes.c_void_p()
        _abi.check(_lib().fgc_mesh_load_stl(buf, len(data), ctypes.byref(h)))
        return cls(h.value)

    # -- counts --------------------------------------------------------------------
    def _counts(self):
        t, l = ctypes.c_uint64(), ctypes.c_uint64()
        _abi.check(_lib().fgc_mesh_counts(self.handle, ctypes.byref(t), ctypes.byref(l)))
        return int(t.value), int(l.value)

    @property
    def ntri(self):
        return self._counts()[0]

    @property
    def nline(self):
        return self._counts()[1]

    # -- operations (mesh.go, silhouette.go) ----------------------------------------
    def SmoothNormalsThreshold(self, radians):
        """mesh.go:80-103, in place."""
        _abi.check(_lib().fgc_mesh_smooth_normals_threshold(self.handle, float(radians)))

    def SmoothNormals(self):
        """mesh.go:105-120, in place."""
        _abi.check(_lib().fgc_mesh_smooth_normals(self.handle))

    def SharpEdges(self, angle_threshold):
        """mesh.go:258-292: a new line mesh of the edges whose faces meet at more
        than angle_threshold radians."""
        h = ctypes.c_void_p()
        _abi.check(_lib().fgc_mesh_sharp_edges(self.handle, float(angle_threshold), ctypes.byref(h)))
        return DeviceMesh(h.value)

    def Silhouette(self, eye, offset):
        """mesh.go:207-209 / silhouette.go:3-53: a new line mesh along the
        silhouette seen from eye, pushed out by offset along the smoothed normals."""
        e = (ctypes.c_double * 3)(*[float(v) for v in eye])
        h = ctypes.c_void_p()
        _abi.check(_lib().fgc_mesh_silhouette(self.handle, e, float(offset), ctypes.byref(h)))
        return DeviceMesh(h.value)

    # -- read back -------------------------------------------------------------------
    def download(self):
        """A host Mesh with this mesh's positions and normals."""
        from .mesh import Mesh
        t, l = self._counts()
        tp, tn = np.zeros((t, 3, 3)), np.zeros((t, 3, 3))
        lp, ln = np.zeros((l, 2, 3)), np.zeros((l, 2, 3))
        _abi.check(_lib().fgc_mesh_download(self.handle, _abi.dptr(tp), _abi.dptr(tn), _abi.dptr(lp),
                                            _abi.dptr(ln)))
        return Mesh(tp if t else None, tn if t else None, line_pos=lp if l else None, line_nrm=ln if l else None)


def LoadSTL(path):
    """LoadSTL (stl.go:23-57): a host Mesh, decoded and given face normals on the GPU."""
    return DeviceMesh.load_stl(path).download()
