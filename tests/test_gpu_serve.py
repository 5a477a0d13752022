"""GPU: the serving loop renders every request exactly as the request alone
(NewContext, clear, DrawMesh, box downsample) gives it, whatever it is
batched and overlapped with, in both arithmetic forms; admission keeps the
requests on the GPU within the HBM budget."""
import math

import numpy as np
import pytest

from fauxgl_gb300 import _abi, scenes
from fauxgl_gb300.geom import V, Vector
from fauxgl_gb300.serve import Request, Server, latency_summary, poisson_arrivals, render_alone, run_load
from fauxgl_gb300.shapes import cylinder_segments

pytestmark = pytest.mark.gpu


def pool():
    a = scenes.displaced_sphere(3, seed=11)
    b = scenes.sphere_scene(4)
    c = cylinder_segments(40, capped=True)
    c.BiUnitCube()
    return [a, b, c]


def requests(n, seed):
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        w, h = [(64, 48), (96, 96), (120, 80), (33, 70)][rng.integers(4)]
        scale = [1, 2, 4][rng.integers(3)]
        az, el = 2 * math.pi * rng.uniform(), math.radians(-30 + 75 * rng.uniform())
        eye = Vector(3 * math.cos(el) * math.cos(az), 3 * math.sin(el), 3 * math.cos(el) * math.sin(az))
        m = scenes.camera_matrix(w * scale, h * scale, eye=eye, center=V(0, 0, 0))
        out.append(Request(mesh=int(rng.integers(3)), matrix=tuple(m), eye=tuple(eye),
                           color=(rng.uniform(), rng.uniform(), rng.uniform(), 1.0), width=w, height=h,
                           scale=scale, light=tuple(scenes.LIGHT), background=(1.0, 0.97, 0.89, 1.0)))
    return out


@pytest.mark.parametrize("precision", [_abi.FGC_PRECISION_MIXED, _abi.FGC_PRECISION_PLAIN])
def test_served_requests_equal_the_request_alone(gpu_lib, precision):
    meshes = pool()
    reqs = requests(24, seed=precision + 1)
    srv = Server(meshes, hbm_budget=4 << 30, slots=3, max_batch=5, precision=precision)
    arrivals = poisson_arrivals(2000.0, 1.0, seed=5)[:len(reqs)]
    arrivals += [arrivals[-1]] * (len(reqs) - len(arrivals))
    tickets, elapsed = run_load(srv, reqs, arrivals)
    assert len(tickets) == len(reqs) and all(t.done for t in tickets)
    for t in tickets:
        img, info = render_alone(meshes[t.request.mesh], t.request, precision)
        assert t.info == info
        assert np.array_equal(t.image, img)
    s = latency_summary(tickets)
    assert s["n"] == len(reqs) and s["p50_ms"] <= s["p99_ms"]


def test_admission_bounds_device_memory(gpu_lib):
    meshes = pool()
    reqs = requests(10, seed=9)
    probe = Server(meshes, hbm_budget=1 << 40, slots=1)
    need = max(probe.request_bytes(r) for r in reqs)
    srv = Server(meshes, hbm_budget=2 * need, slots=3, max_batch=4)
    for r in reqs:
        srv.submit(r)
    peak = 0
    while srv.pending or any(s.busy for s in srv.slots):
        srv.poll()
        peak = max(peak, srv.in_use)
        assert srv.in_use <= srv.budget
    assert len(srv.completed) == len(reqs)
    for t in srv.completed:
        img, info = render_alone(meshes[t.request.mesh], t.request)
        assert t.info == info and np.array_equal(t.image, img)
