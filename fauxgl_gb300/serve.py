"""Render serving loop on libfauxglcuda (no counterpart in package fauxgl).

A Server keeps a pool of meshes resident on the GPU and renders requests --
(mesh, camera, width, height, supersampling scale) -- as they arrive:

  * admission by HBM budget: a request is admitted when its framebuffers
    (colour 4 B + depth 8 B per supersampled pixel, plus the downsampled
    result) and its share of the pipeline scratch fit in what the requests
    already on the GPU leave of the budget;
  * continuous batching: admitted requests are grouped into a batch (one
    launch per pipeline stage for all of them) as soon as a batch slot is
    free; several slots, each with its own CUDA stream, keep batches in
    flight at once, so requests that arrive while others are on the GPU
    start as slots and memory free up and their work overlaps on the device;
  * results: each request's frame is cleared, drawn, box-downsampled by its
    scale on the device and copied to the host; its latency runs from arrival
    to that copy's completion;
  * deadlines and cancellation: a request still waiting for admission
    request_timeout seconds after its arrival expires (load shedding when the
    offered rate is above what the GPU sustains), and cancel() withdraws a
    waiting request at once or discards a running one's result when its
    batch finishes (work on the GPU is never interrupted).

Each request's result does not depend on what it is batched with: every draw
of a batch gives exactly what it gives alone (same kernels, same per-draw
arithmetic), which the tests check.

    srv = Server(meshes, hbm_budget=64 << 30)
    t = srv.submit(Request(mesh=3, matrix=m, eye=e, color=c, width=512, height=512, scale=2))
    while not t.done: srv.poll()
    t.image, t.info, t.latency_s
"""
import ctypes
import time
from collections import deque
from dataclasses import dataclass, field

import numpy as np

from . import _abi
from .context import _DeviceHandle, _upload_mesh

# Pipeline scratch a request may need per submitted triangle (raster primitive
# record, box, span, bins, vertex-stage records), used for admission.
SCRATCH_BYTES_PER_TRIANGLE = 256


@dataclass
class Request:
    mesh: int                      # index into the server's mesh pool
    matrix: tuple                  # 16 row-major values (Shader matrix)
    eye: tuple                     # camera position (PhongShader)
    color: tuple                   # PhongShader ObjectColor
    width: int                     # result size (after downsampling)
    height: int
    scale: int = 1                 # supersampling factor per axis
    light: tuple = (0.0, 0.0, 1.0)
    background: tuple = (1.0, 1.0, 1.0, 1.0)


@dataclass(eq=False)  # tickets are compared by identity (two requests may be alike)
class Ticket:
    request: Request
    arrival: float
    admitted: float = 0.0
    finished: float = 0.0
    done: bool = False             # the result is ready
    status: str = "pending"        # pending, running, done, cancelled or expired
    image: np.ndarray = None
    info: tuple = None
    bytes: int = 0
    scratch: int = 0
    cancel_requested: bool = False
    _ctx: object = field(default=None, repr=False)

    @property
    def latency_s(self):
        return self.finished - self.arrival if self.done else None

    @property
    def dropped(self):
        return self.status in ("cancelled", "expired")


def _pinned(nbytes):
    """Page-locked host buffer (falls back to ordinary memory without torch)."""
    try:
        import torch
        t = torch.empty(int(nbytes), dtype=torch.uint8, pin_memory=True)
        return t, t.numpy()
    except Exception:
        a = np.empty(int(nbytes), dtype=np.uint8)
        return a, a


class _Slot:
    """One batch in flight: a batch handle with its own CUDA stream."""

    def __init__(self, lib):
        self.lib = lib
        h = ctypes.c_void_p()
        _abi.check(lib.fgc_batch_create(ctypes.byref(h)))
        self.h = _DeviceHandle(h.value, lib.fgc_batch_destroy)
        self.tickets = []
        self.keep = []

    @property
    def busy(self):
        return bool(self.tickets)

    def done(self):
        d = ctypes.c_int32()
        _abi.check(self.lib.fgc_batch_query(self.h.handle, ctypes.byref(d)))
        return bool(d.value)


class Server:
    """Continuous-batching render server over a resident mesh pool."""

    def __init__(self, meshes, hbm_budget=32 << 30, slots=3, max_batch=64, precision=_abi.FGC_PRECISION_MIXED,
                 tuning=None, lib=None, upload=None, request_timeout=None, clock=time.perf_counter,
                 max_batch_triangles=16 << 20):
        # lib / upload stand in for libfauxglcuda and the mesh upload in the
        # host-logic tests
        self.lib = lib or _abi.load_library()
        self.meshes = list(meshes)
        self.mesh_handles = [(upload or _upload_mesh)(m) for m in self.meshes]
        self.budget = int(hbm_budget)
        self.max_batch = int(max_batch)
        self.max_batch_triangles = int(max_batch_triangles)  # a batch's scratch grows with its triangles
        self.precision = precision
        self.slots = [_Slot(self.lib) for _ in range(max(1, slots))]
        if tuning:
            t = _abi.FgcBatchTuning(*tuning)
            for s in self.slots:
                _abi.check(self.lib.fgc_batch_set_tuning(s.h.handle, ctypes.byref(t)))
        self.request_timeout = request_timeout  # seconds a request may wait for admission (None: forever)
        self.clock = clock
        self.pending = deque()
        self.dropped = []    # cancelled and expired tickets
        self.contexts = {}   # (W, H) -> [idle contexts], kept for reuse
        self.fb_bytes = 0    # framebuffers of every live context (idle or in use)
        self.scratch = 0     # scratch share of the requests on the GPU
        self.completed = []

    # -- requests -------------------------------------------------------------
    @staticmethod
    def framebuffer_bytes(W, H):
        return W * H * 12  # NRGBA + FP64 depth

    def request_bytes(self, r):
        W, H = r.width * r.scale, r.height * r.scale
        return (self.framebuffer_bytes(W, H) + r.width * r.height * 4
                + SCRATCH_BYTES_PER_TRIANGLE * self.meshes[r.mesh].ntri)

    def submit(self, request, arrival=None):
        t = Ticket(request, self.clock() if arrival is None else arrival)
        t.bytes = self.request_bytes(request)
        if t.bytes > self.budget:
            raise ValueError("request needs %d bytes, above the HBM budget %d" % (t.bytes, self.budget))
        self.pending.append(t)
        return t

    @property
    def in_use(self):
        return self.fb_bytes + self.scratch

    def cancel(self, ticket):
        """Withdraw a request: a waiting one leaves the queue now; a running
        one's result is discarded when its batch finishes. Returns False when
        the result was already delivered (or the ticket already dropped)."""
        if ticket.status == "pending":
            self.pending.remove(ticket)
            self._drop(ticket, "cancelled")
            return True
        if ticket.status == "running":
            ticket.cancel_requested = True
            return True
        return False

    def _drop(self, t, status):
        t.status = status
        t.finished = self.clock()
        self.dropped.append(t)

    def _expire(self, now):
        """Requests that waited for admission longer than request_timeout."""
        if self.request_timeout is None:
            return
        # the queue is in arrival order: the oldest waiting requests lead it
        while self.pending and now - self.pending[0].arrival > self.request_timeout:
            self._drop(self.pending.popleft(), "expired")

    # -- contexts ---------------------------------------------------------------
    def _fits(self, t):
        """Admit t if its framebuffer (unless an idle one of its size is kept),
        its downsampled result and its scratch fit the budget; idle contexts
        of other sizes are freed to make room."""
        r = t.request
        W, H = r.width * r.scale, r.height * r.scale
        extra = t.bytes - (self.framebuffer_bytes(W, H) if self.contexts.get((W, H)) else 0)
        while self.in_use + extra > self.budget:
            victim = next(((k, v) for k, v in self.contexts.items() if v and k != (W, H)), None)
            if victim is None:
                return False
            (vw, vh), lst = victim
            lst.pop()  # released when collected
            self.fb_bytes -= self.framebuffer_bytes(vw, vh)
        return True

    def _context(self, W, H):
        free = self.contexts.setdefault((W, H), [])
        if free:
            return free.pop()
        h = ctypes.c_void_p()
        _abi.check(self.lib.fgc_context_create(W, H, ctypes.byref(h)))
        self.fb_bytes += self.framebuffer_bytes(W, H)
        return _DeviceHandle(h.value, self.lib.fgc_context_destroy)

    def _release(self, W, H, ctx):
        self.contexts.setdefault((W, H), []).append(ctx)

    def trim(self):
        """Free the idle contexts (their framebuffers)."""
        for (W, H), lst in self.contexts.items():
            self.fb_bytes -= self.framebuffer_bytes(W, H) * len(lst)
        self.contexts = {}

    # -- the loop ---------------------------------------------------------------
    def poll(self):
        """Finish the batches that are done, then admit pending requests into
        free slots. Returns the tickets finished by this call."""
        finished = []
        for s in self.slots:
            if s.busy and s.done():
                finished += self._finish(s)
        self._expire(self.clock())
        for s in self.slots:
            if not self.pending:
                break
            if not s.busy:
                self._admit(s)
        return finished

    def drain(self):
        while self.pending or any(s.busy for s in self.slots):
            self.poll()
        return self.completed

    def _admit(self, slot):
        batch, ctxs = [], []
        tris = 0
        while self.pending and len(batch) < self.max_batch:
            t = self.pending[0]
            ntri = self.meshes[t.request.mesh].ntri
            if batch and tris + ntri > self.max_batch_triangles:
                break
            if not self._fits(t):
                break
            tris += ntri
            self.pending.popleft()
            r = t.request
            ctxs.append(self._context(r.width * r.scale, r.height * r.scale))
            t.scratch = t.bytes - self.framebuffer_bytes(r.width * r.scale, r.height * r.scale)
            self.scratch += t.scratch
            batch.append(t)
        if not batch:
            return
        n = len(batch)
        items = (_abi.FgcBatchItem * n)()
        keep = [items]
        now = self.clock()
        for i, t in enumerate(batch):
            r = t.request
            ctx = ctxs[i]
            t._ctx = ctx
            t.admitted = now
            t.status = "running"
            c = (ctypes.c_double * 4)(*r.background)
            _abi.check(self.lib.fgc_clear_color(ctx.handle, c))
            _abi.check(self.lib.fgc_clear_depth(ctx.handle, 1.7976931348623157e308))
            st = _abi.FgcState()
            self.lib.fgc_state_default(ctypes.byref(st))
            st.precision = self.precision
            sh = _abi.FgcShader()
            m16 = (ctypes.c_double * 16)(*[float(x) for x in r.matrix])
            self.lib.fgc_shader_phong(ctypes.byref(sh), m16, (ctypes.c_double * 3)(*r.light),
                                      (ctypes.c_double * 3)(*r.eye))
            sh.color[:] = list(r.color)
            raw, arr = _pinned(r.width * r.height * 4)
            t.image = arr.reshape(r.height, r.width, 4)
            keep += [st, sh, raw]
            mesh = self.meshes[r.mesh]
            it = items[i]
            it.context = ctx.handle
            it.mesh = self.mesh_handles[r.mesh]
            it.tri_first, it.tri_count, it.line_first, it.line_count = 0, mesh.ntri, 0, mesh.nline
            it.state = ctypes.pointer(st)
            it.shader = ctypes.pointer(sh)
            it.out_nrgba = arr.ctypes.data
            it.out_scale = r.scale
        _abi.check(self.lib.fgc_batch_submit(slot.h.handle, items, n))
        slot.tickets = batch
        slot.keep = keep

    def _finish(self, slot):
        n = len(slot.tickets)
        infos = (_abi.FgcRasterizeInfo * n)()
        _abi.check(self.lib.fgc_batch_wait(slot.h.handle, infos))
        now = self.clock()
        out = []
        for i, t in enumerate(slot.tickets):
            r = t.request
            self._release(r.width * r.scale, r.height * r.scale, t._ctx)
            t._ctx = None
            self.scratch -= t.scratch
            if t.cancel_requested:
                t.image = None
                self._drop(t, "cancelled")
                continue
            t.info = (int(infos[i].total_pixels), int(infos[i].updated_pixels))
            t.finished = now
            t.done = True
            t.status = "done"
            out.append(t)
        self.completed += out
        slot.tickets = []
        slot.keep = []
        return out


def render_alone(mesh, request, precision=_abi.FGC_PRECISION_MIXED):
    """The request rendered by itself through the plain drawing API
    (NewContext, ClearColorBufferWith, DrawMesh, box downsample): the reference
    result a served request must equal."""
    lib = _abi.load_library()
    r = request
    W, H = r.width * r.scale, r.height * r.scale
    h = ctypes.c_void_p()
    _abi.check(lib.fgc_context_create(W, H, ctypes.byref(h)))
    ctx = _DeviceHandle(h.value, lib.fgc_context_destroy)
    _abi.check(lib.fgc_clear_color(ctx.handle, (ctypes.c_double * 4)(*r.background)))
    st = _abi.FgcState()
    lib.fgc_state_default(ctypes.byref(st))
    st.precision = precision
    sh = _abi.FgcShader()
    lib.fgc_shader_phong(ctypes.byref(sh), (ctypes.c_double * 16)(*[float(x) for x in r.matrix]),
                         (ctypes.c_double * 3)(*r.light), (ctypes.c_double * 3)(*r.eye))
    sh.color[:] = list(r.color)
    info = _abi.FgcRasterizeInfo()
    _abi.check(lib.fgc_draw_mesh(ctx.handle, _upload_mesh(mesh), ctypes.byref(st), ctypes.byref(sh),
                                 ctypes.byref(info)))
    out = np.empty((r.height, r.width, 4), dtype=np.uint8)
    _abi.check(lib.fgc_downsample(ctx.handle, r.scale, out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8))))
    return out, (int(info.total_pixels), int(info.updated_pixels))


def poisson_arrivals(rate, duration, seed):
    """Arrival times (seconds from 0) of a Poisson process of the given rate."""
    rng = np.random.default_rng(seed)
    t, out = 0.0, []
    while True:
        t += rng.exponential(1.0 / rate)
        if t >= duration:
            return out
        out.append(t)


def run_load(server, requests, arrivals, timeout=None, sleep=time.sleep):
    """Drive the server with requests arriving at the given times (seconds
    from start); returns (tickets in arrival order, elapsed seconds). With a
    timeout (seconds), requests not finished by then are cancelled: arrivals
    after it are never submitted, waiting ones leave the queue and running
    batches are finished with their results discarded, so the server is idle
    and reusable on return."""
    clock = server.clock
    start = clock()
    tickets = []
    i = 0
    deadline = None if timeout is None else start + timeout
    while i < len(requests) or server.pending or any(s.busy for s in server.slots):
        now = clock()
        if deadline is not None and now > deadline:
            for t in list(server.pending) + [t for s in server.slots for t in s.tickets]:
                server.cancel(t)
            server.drain()
            break
        while i < len(requests) and now - start >= arrivals[i]:
            tickets.append(server.submit(requests[i], arrival=start + arrivals[i]))
            i += 1
        server.poll()
        if i < len(requests) and not server.pending and not any(s.busy for s in server.slots):
            # idle until the next arrival
            wait = start + arrivals[i] - clock()
            if wait > 0:
                sleep(min(wait, 0.002))
    return tickets, clock() - start


def latency_summary(tickets):
    """p50 / p99 latency of the delivered results (dropped requests excluded)."""
    lat = sorted(t.latency_s for t in tickets if t.done)
    if not lat:
        return {"p50_ms": None, "p99_ms": None, "n": 0}

    def pct(q):
        return lat[min(len(lat) - 1, int(round(q * (len(lat) - 1))))] * 1e3
    return {"p50_ms": round(pct(0.5), 3), "p99_ms": round(pct(0.99), 3), "n": len(lat)}
