"""Host logic of the serving loop (admission by HBM budget, continuous
batching over several batch slots, context reuse) against a fake of the
library's batch interface: no GPU."""
import ctypes
import itertools

import numpy as np
import pytest

from fauxgl_gb300 import _abi
from fauxgl_gb300.serve import Request, Server, latency_summary, poisson_arrivals


class FakeMesh:
    def __init__(self, ntri):
        self.ntri, self.nline = ntri, 0


class FakeLib:
    """The calls Server makes, with a batch that finishes `latency` queries
    after its submission."""

    def __init__(self, latency=2):
        self.ids = itertools.count(1)
        self.latency = latency
        self.contexts = {}        # handle -> (W, H)
        self.created = 0
        self.batches = {}         # handle -> dict(items, polls)
        self.submissions = []     # list of lists of context handles
        self.peak_inflight = 0

    def _out(self, ref, v):
        ctypes.cast(ref, ctypes.POINTER(ctypes.c_void_p))[0] = v

    def fgc_batch_create(self, ref):
        h = next(self.ids)
        ref._obj.value = h
        self.batches[h] = None
        return 0

    def fgc_batch_destroy(self, h):
        return 0

    def fgc_batch_set_tuning(self, h, t):
        return 0

    def fgc_context_create(self, w, h, ref):
        c = next(self.ids)
        ref._obj.value = c
        self.contexts[c] = (w, h)
        self.created += 1
        return 0

    def fgc_context_destroy(self, c):
        self.contexts.pop(c, None)
        return 0

    def fgc_clear_color(self, c, rgba):
        assert c in self.contexts
        return 0

    def fgc_clear_depth(self, c, v):
        assert c in self.contexts
        return 0

    def fgc_state_default(self, st):
        return None

    def fgc_shader_phong(self, sh, m, light, eye):
        return None

    def fgc_batch_submit(self, h, items, n):
        assert self.batches[h] is None, "one submission in flight per batch"
        ctxs = [items[i].context for i in range(n)]
        assert len(set(ctxs)) == n
        self.batches[h] = dict(items=[(items[i].context, items[i].out_nrgba, items[i].out_scale) for i in range(n)],
                               polls=0)
        self.submissions.append(ctxs)
        self.peak_inflight = max(self.peak_inflight, sum(1 for b in self.batches.values() if b))
        return 0

    def fgc_batch_query(self, h, ref):
        b = self.batches[h]
        b["polls"] += 1
        ref._obj.value = 1 if b["polls"] >= self.latency else 0
        return 0

    def fgc_batch_wait(self, h, infos):
        b = self.batches[h]
        for i, (c, out, scale) in enumerate(b["items"]):
            infos[i].total_pixels = c
            infos[i].updated_pixels = scale
        self.batches[h] = None
        return 0


def make_server(budget, slots=2, max_batch=4, latency=2, meshes=(1000, 2000)):
    lib = FakeLib(latency)
    srv = Server([FakeMesh(n) for n in meshes], hbm_budget=budget, slots=slots, max_batch=max_batch, lib=lib,
                 upload=lambda m: id(m))
    return srv, lib


def req(mesh=0, w=64, h=32, scale=1):
    return Request(mesh=mesh, matrix=tuple(float(i % 5 == 0) for i in range(16)), eye=(0, 0, 5),
                   color=(0.5, 0.5, 0.5, 1), width=w, height=h, scale=scale)


def test_admission_keeps_within_the_budget():
    probe, _ = make_server(1 << 40)
    one = probe.request_bytes(req())
    srv, lib = make_server(2 * one, slots=3, max_batch=4)
    ts = [srv.submit(req()) for _ in range(7)]
    peak = 0
    for _ in range(200):
        srv.poll()
        peak = max(peak, srv.in_use)
        assert srv.in_use <= srv.budget
        if all(t.done for t in ts):
            break
    assert all(t.done for t in ts)
    assert peak == 2 * one
    # admitted in arrival order, two at a time
    assert [len(s) for s in lib.submissions] == [2, 2, 2, 1]
    assert all(a.admitted <= b.admitted for a, b in zip(ts, ts[1:]))


def test_continuous_batching_fills_free_slots():
    srv, lib = make_server(1 << 40, slots=3, max_batch=2, latency=3)
    first = [srv.submit(req()) for _ in range(4)]
    srv.poll()                       # slots 0 and 1 take two each
    assert [len(s) for s in lib.submissions] == [2, 2]
    late = [srv.submit(req()) for _ in range(2)]
    srv.poll()                       # arrives while the first batches run: slot 2
    assert [len(s) for s in lib.submissions] == [2, 2, 2]
    assert lib.peak_inflight == 3
    srv.drain()
    assert all(t.done for t in first + late)
    assert all(t.latency_s is not None and t.latency_s >= 0 for t in first + late)


def test_contexts_are_reused_and_trimmed():
    srv, lib = make_server(1 << 40, slots=1, max_batch=8)
    for _ in range(3):
        ts = [srv.submit(req(w=64, h=32, scale=2)) for _ in range(3)]
        srv.drain()
        assert all(t.done for t in ts)
    assert lib.created == 3            # three 128x64 contexts, reused by every round
    assert srv.fb_bytes == 3 * 128 * 64 * 12
    srv.trim()
    assert srv.fb_bytes == 0


def test_idle_contexts_of_other_sizes_are_freed_for_room():
    probe, _ = make_server(1 << 40)
    big = probe.request_bytes(req(w=256, h=256, scale=2))
    srv, lib = make_server(big + 1000, slots=1, max_batch=4)
    small = srv.submit(req(w=16, h=16))
    srv.drain()
    assert small.done and srv.fb_bytes == 16 * 16 * 12
    t = srv.submit(req(w=256, h=256, scale=2))
    srv.drain()
    assert t.done
    assert srv.fb_bytes == 512 * 512 * 12   # the idle 16x16 context was released


def test_oversized_request_is_rejected():
    srv, _ = make_server(1000)
    with pytest.raises(ValueError):
        srv.submit(req(w=512, h=512))


def test_poisson_arrivals_and_summary():
    a = poisson_arrivals(200.0, 2.0, seed=4)
    assert all(0 <= x < 2.0 for x in a) and a == sorted(a)
    assert 300 < len(a) < 500
    assert latency_summary([]) == {"p50_ms": None, "p99_ms": None, "n": 0}


class FakeClock:
    """A clock the test moves by hand (and run_load's sleep moves too)."""

    def __init__(self):
        self.t = 0.0

    def __call__(self):
        return self.t

    def sleep(self, dt):
        self.t += dt


def make_timed_server(budget=1 << 40, slots=1, max_batch=2, latency=3, request_timeout=None):
    lib = FakeLib(latency)
    clock = FakeClock()
    srv = Server([FakeMesh(1000)], hbm_budget=budget, slots=slots, max_batch=max_batch, lib=lib,
                 upload=lambda m: id(m), request_timeout=request_timeout, clock=clock)
    return srv, lib, clock


def test_cancel_waiting_and_running_requests():
    srv, lib, clock = make_timed_server(slots=1, max_batch=2, latency=3)
    ts = [srv.submit(req()) for _ in range(5)]
    srv.poll()  # the first two run, three wait
    assert [t.status for t in ts] == ["running", "running", "pending", "pending", "pending"]
    assert srv.cancel(ts[3])            # waiting: leaves the queue at once
    assert ts[3].status == "cancelled" and ts[3] not in srv.pending
    assert srv.cancel(ts[1])            # running: the batch finishes, its result is dropped
    assert ts[1].status == "running" and ts[1].cancel_requested
    srv.drain()
    assert [t.status for t in ts] == ["done", "cancelled", "done", "cancelled", "done"]
    assert ts[1].image is None and not ts[1].done and ts[1].latency_s is None
    assert not srv.cancel(ts[0])        # delivered results cannot be withdrawn
    assert len(lib.submissions) == 2    # the cancelled waiting request never reached the GPU
    assert srv.scratch == 0             # every admitted request released its share
    assert latency_summary(ts)["n"] == 3
    assert {id(t) for t in srv.dropped} == {id(ts[1]), id(ts[3])}


def test_waiting_requests_expire_after_the_request_timeout():
    srv, lib, clock = make_timed_server(slots=1, max_batch=1, latency=2, request_timeout=0.5)
    ts = [srv.submit(req()) for _ in range(4)]
    srv.poll()                # one runs, three wait
    clock.t = 0.4
    srv.poll()                # the first finishes after two queries; the second is admitted
    srv.poll()
    clock.t = 0.6             # the two still waiting are now past the timeout
    srv.drain()
    assert [t.status for t in ts] == ["done", "done", "expired", "expired"]
    assert len(lib.submissions) == 2
    assert all(t.finished == 0.6 for t in ts[2:])


def test_run_load_timeout_cancels_unfinished_work():
    from fauxgl_gb300.serve import run_load
    srv, lib, clock = make_timed_server(slots=1, max_batch=1, latency=1000000)  # batches never finish by themselves
    reqs = [req() for _ in range(4)]
    lib.latency = 4
    arrivals = [0.0, 0.0, 0.01, 10.0]       # the last arrives after the deadline
    orig_poll = srv.poll

    def slow_poll():                        # each poll takes 5 ms of the fake clock
        clock.t += 0.005
        return orig_poll()
    srv.poll = slow_poll
    tickets, elapsed = run_load(srv, reqs, arrivals, timeout=0.012, sleep=clock.sleep)
    assert len(tickets) == 3                # the fourth was never submitted
    assert tickets[0].status in ("done", "cancelled")
    assert all(t.status in ("done", "cancelled") for t in tickets)
    assert any(t.status == "cancelled" for t in tickets)
    assert not srv.pending and not any(s.busy for s in srv.slots)  # idle and reusable
    assert srv.scratch == 0
    t = srv.submit(req())
    srv.drain()
    assert t.status == "done"


def test_batches_stop_at_their_triangle_cap():
    lib = FakeLib(2)
    srv = Server([FakeMesh(1000), FakeMesh(2000)], hbm_budget=1 << 40, slots=1, max_batch=8, lib=lib,
                 upload=lambda m: id(m), max_batch_triangles=3500)
    ts = [srv.submit(req(mesh=m)) for m in (0, 1, 0, 1, 1)]
    srv.drain()
    assert all(t.done for t in ts)
    # 1000 + 2000 fit, the next 1000 would pass 3500; a lone request always runs
    assert [len(s) for s in lib.submissions] == [2, 2, 1]
