"""Batch: many independent draws rendered by one set of GPU launches.

No counterpart in package fauxgl. A batch takes draws -- each a Context (its
current state and Shader), a Mesh and a triangle / line range -- and renders
all of them with one launch per pipeline stage; every draw's framebuffer and
RasterizeInfo equal what Context.DrawTriangles / DrawLines would give alone.

    b = Batch()
    b.Add(ctx1, mesh1)                       # DrawMesh-like: triangles, then lines
    b.Add(ctx2, mesh2, read_back=True)       # frame copied to the host afterwards
    b.Submit()                               # returns once queued
    infos = b.Wait()                         # [RasterizeInfo, ...]
    img = b.Result(1)                        # (H, W, 4) uint8 of the second draw

Between Submit and Wait the draws' contexts are busy (any call on them raises
FauxGLError with FGC_ERR_BUSY).
"""
import ctypes

import numpy as np

from . import _abi
from .context import RasterizeInfo, _DeviceHandle, _draw_handle


class Batch:
    def __init__(self, use_graph=False):
        self._lib = _abi.load_library()
        h = ctypes.c_void_p()
        _abi.check(self._lib.fgc_batch_create(ctypes.byref(h)))
        self._h = _DeviceHandle(h.value, self._lib.fgc_batch_destroy)
        self._draws = []
        self._submitted = None
        if use_graph:
            t = self.Tuning()
            t["use_graph"] = 1
            self.SetTuning(**t)

    @property
    def handle(self):
        return self._h.handle

    def Clear(self):
        """Forget the queued draws (not the submission in flight)."""
        self._draws = []

    def Add(self, ctx, mesh, tri_first=0, tri_count=None, line_first=0, line_count=None, read_back=False,
            scale=1):
        """Queue a draw of mesh triangles [tri_first, tri_first+tri_count) then
        lines [line_first, ...) into ctx with ctx's current state and shader.
        read_back: copy the frame (box-downsampled by scale) to the host after
        the batch. Returns the draw's index."""
        tri_count = mesh.ntri - tri_first if tri_count is None else tri_count
        line_count = mesh.nline - line_first if line_count is None else line_count
        st = ctx.state()
        sh = ctx.shader_struct()
        out = None
        if read_back:
            out = np.empty((ctx.Height // scale, ctx.Width // scale, 4), dtype=np.uint8)
        # a mesh that is not resident is copied to the device now (its owner
        # stays with the draw until the batch is done)
        handle, owner = _draw_handle(mesh)
        self._draws.append((ctx, owner or mesh, handle, int(tri_first), int(tri_count), int(line_first),
                            int(line_count), st, sh, out, int(scale)))
        return len(self._draws) - 1

    def _items(self):
        n = len(self._draws)
        items = (_abi.FgcBatchItem * n)()
        for i, (ctx, _mesh, mh, tf, tc, lf, lc, st, sh, out, scale) in enumerate(self._draws):
            it = items[i]
            it.context = ctx.handle
            it.mesh = mh
            it.tri_first, it.tri_count, it.line_first, it.line_count = tf, tc, lf, lc
            it.state = ctypes.pointer(st)
            it.shader = ctypes.pointer(sh)
            it.out_nrgba = out.ctypes.data if out is not None else None
            it.out_scale = scale
        return items

    def Submit(self):
        """Queue every added draw on the GPU; returns without waiting."""
        items = self._items()
        _abi.check(self._lib.fgc_batch_submit(self.handle, items, len(self._draws)))
        self._submitted = (items, list(self._draws))

    def Done(self):
        d = ctypes.c_int32()
        _abi.check(self._lib.fgc_batch_query(self.handle, ctypes.byref(d)))
        return bool(d.value)

    def Wait(self):
        """Block until the submission has finished; one RasterizeInfo per draw."""
        n = len(self._submitted[1]) if self._submitted else 0
        infos = (_abi.FgcRasterizeInfo * max(n, 1))()
        _abi.check(self._lib.fgc_batch_wait(self.handle, infos))
        return [RasterizeInfo(int(infos[i].total_pixels), int(infos[i].updated_pixels)) for i in range(n)]

    def Result(self, index):
        """The read-back frame of draw `index` of the last submission."""
        return self._submitted[1][index][9]

    def Render(self):
        self.Submit()
        return self.Wait()

    # -- tuning / instrumentation ----------------------------------------------
    def Tuning(self):
        t = _abi.FgcBatchTuning()
        _abi.check(self._lib.fgc_batch_get_tuning(self.handle, ctypes.byref(t)))
        return {name: int(getattr(t, name)) for name, _ in _abi.FgcBatchTuning._fields_}

    def SetTuning(self, band_pixels=4096, prims_per_bin_block=4096, fragment_cap=1024, use_graph=0, window=8,
                  reserved=0):
        t = _abi.FgcBatchTuning(int(band_pixels), int(prims_per_bin_block), int(fragment_cap), int(use_graph),
                                int(window), 0)
        _abi.check(self._lib.fgc_batch_set_tuning(self.handle, ctypes.byref(t)))

    def Autotune(self, repeats=2):
        """Time the added draws under candidate shapes and keep the fastest."""
        items = self._items()
        t = _abi.FgcBatchTuning()
        _abi.check(self._lib.fgc_batch_autotune(self.handle, items, len(self._draws), int(repeats), ctypes.byref(t)))
        return {name: int(getattr(t, name)) for name, _ in _abi.FgcBatchTuning._fields_}

    def SetTiming(self, enable):
        _abi.check(self._lib.fgc_batch_set_timing(self.handle, int(bool(enable))))

    def SetStream(self, cuda_stream):
        _abi.check(self._lib.fgc_batch_set_stream(self.handle, cuda_stream or None))

    def LastStats(self):
        st = _abi.FgcStats()
        _abi.check(self._lib.fgc_batch_last_stats(self.handle, ctypes.byref(st)))
        d = {name: int(getattr(st, name)) for name, _ in _abi.FgcStats._fields_ if name != "stage_ms"}
        d["stage_ms"] = {n: float(st.stage_ms[i]) for i, n in enumerate(_abi.STAGE_NAMES)}
        return d
