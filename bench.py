#!/usr/bin/env python
"""Benchmark of FauxGL's triangle pipeline on GB300.

Workload (one step = one frame): the dense-mesh 1080p frame -- a displaced
icosphere of 1,310,720 triangles fit to the bi-unit cube with normals
smoothed at 30 degrees, 1920x1080, PhongShader (light (-0.75,1,0.25), object
#468966), back-face culling, colour cleared to #FFF8E3 and depth to
MaxFloat64 every frame. Seeded synthetic data (the reference's benchmark
mesh, the Stanford Dragon, is not available).

value   frames/s of the plain FP64 form (the reference's arithmetic, bit-exact
        to it) with the mesh resident in HBM; CUDA events on the stream the
        library launches on bracket the K timed frames.
e2e     the same frames through the C ABI with a host readback each frame:
        fgc_clear_color + fgc_clear_depth + fgc_draw_mesh + fgc_read_color
        into pinned host memory (H2D: the draw-state and shader structs;
        D2H: the NRGBA frame and RasterizeInfo).
Also reported: the mixed form at 1x, both forms at 16x supersampling with the
wireframe overlay and device box-downsample (7680x4320 -> 1920x1080), per-stage
times, the roofline of the dominant stage, the CPU baseline, and the clocks
sampled during the timed region.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
"""
import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "frames/s at 1.3M tris 1080p 1x/16xSS, mixed vs FP64-plain; batch p99 latency"
WORKLOAD = ("dense-mesh 1080p frame: displaced icosphere 1,310,720 triangles (subdivision 8, seed 1), "
            "1920x1080, PhongShader, back-face culling, colour+depth clear per frame")
W, H = 1920, 1080
SS = 4

# Algorithmic FP64 operations (add, subtract, multiply, divide, sqrt: one
# each; compares not counted) of the reference's rasterize loop
# (context.go:184-278) per event, for the Phong shader with an object colour,
# no texture and SpecularPower 32 (shader.go:75-96, vertex.go:18-47).
FLOPS_PER_VISITED = 6        # b_k = w_k*ra (3), w_k += a_k (3)
FLOPS_PER_COVERED = 6        # z (3 mul, 2 add), bz (1)
FLOPS_PER_SHADED_PHONG = 119  # perspective 6, position 21, normal 31, Phong 61
FLOPS_PER_SHADED_SOLID = 0
# Triangle setup (drawClippedTriangle + rasterize prologue): NDC area per
# triangle, edge setup per surviving primitive.
FLOPS_SETUP_PER_TRIANGLE = 7
FLOPS_SETUP_PER_PRIM = 40
FLOPS_VERTEX_PER_UNIQUE = 34  # MulPositionW 24, NDC 3 divides, screen 6, 1/W


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--ss-steps", type=int, default=5, help="timed frames of the 16x supersampled variants")
    ap.add_argument("--cpu-frames", type=int, default=5)
    ap.add_argument("--batch-steps", type=int, default=5, help="timed batches of the 1,024-view thumbnail batch")
    ap.add_argument("--batch-views", type=int, default=0,
                    help="render only the first N views of the thumbnail batch (0: all; for profiler runs)")
    ap.add_argument("--batch-tuning", default="auto",
                    help="'auto' (autotune) or band_pixels,prims_per_bin_block,fragment_cap,window")
    ap.add_argument("--serve-seconds", type=float, default=2.0, help="arrival window per rate of the serving loop")
    ap.add_argument("--serve-timeout", type=float, default=1.0,
                    help="seconds a serving request may wait for admission before it is shed")
    ap.add_argument("--serve-budget-gb", type=int, default=96, help="HBM budget of the serving loop")
    ap.add_argument("--only", choices=["all", "plain", "mixed", "ss16", "batch", "serve", "meshprep", "accuracy"],
                    default="all",
                    help="plain / mixed / ss16 / batch / serve / meshprep: time only that workload (for profiler "
                         "runs); accuracy: only the per-configuration comparison with the oracle")
    ap.add_argument("--no-accuracy", action="store_true", help="skip the comparison with the oracle")
    ap.add_argument("--detail", type=int, default=8,
                    help="subdivision of the dense mesh (8: the benchmark's 1,310,720 triangles; a smaller value "
                         "gives a smaller case of the same scene for profiler counter captures, not a bench line)")
    return ap.parse_args()


def dist_env():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), int(
        os.environ.get("LOCAL_RANK", "0"))


def reduce_max(values, device):
    """Max over ranks of each value: N replicas each render their own frames,
    so the job's step time is the slowest rank's (no data-path collective)."""
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(v) for v in values], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(x) for x in t]


def replica_rate(max_ms, world):
    """Whole-job frames/s of world replicas whose slowest frame takes max_ms."""
    return world * 1e3 / max_ms


def build_scene(detail=8):
    from fauxgl_gb300 import scenes
    t = time.time()
    mesh = scenes.displaced_sphere(detail, seed=1)
    log("scene: %d triangles in %.1fs" % (mesh.ntri, time.time() - t))
    return mesh


def phong_struct(w, h):
    from fauxgl_gb300 import scenes
    from fauxgl_gb300.shader import NewPhongShader, to_fgc_shader
    sh = NewPhongShader(scenes.camera_matrix(w, h), scenes.LIGHT, scenes.EYE)
    sh.ObjectColor = scenes.OBJECT_COLOR
    return to_fgc_shader(sh)


def overlay_struct(w, h):
    from fauxgl_gb300 import scenes
    from fauxgl_gb300.shader import NewSolidColorShader, to_fgc_shader
    return to_fgc_shader(NewSolidColorShader(scenes.camera_matrix(w, h), (0, 0, 0, 0.5)))


class ClockSampler:
    """nvidia-smi clock / throttle samples taken while the timed region runs."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *exc):
        self.rows = []
        if self.proc is None:
            return False
        self.proc.terminate()
        try:
            out, _ = self.proc.communicate(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
            out, _ = self.proc.communicate()
        for line in out.splitlines():
            parts = [p.strip() for p in line.split(",")]
            if len(parts) == 9:
                self.rows.append(parts)
        return False

    def summary(self):
        rows = getattr(self, "rows", [])
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            for n, v in zip(names, r[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(rows),
                "power_w_max": max(float(r[3]) for r in rows if r[3].replace(".", "").isdigit()) if rows else None}


def work_dict(s):
    return {k: int(getattr(s, k)) for k in ("elements", "clipped", "primitives", "bin_entries", "visited_pixels",
                                            "covered_pixels", "shaded_fragments", "updated_pixels", "attempts",
                                            "kernel_launches")}


class Frame:
    """A context plus the draws of one benchmark frame."""

    def __init__(self, lib, mesh_h, w, h, precision, overlay=False, scale=1):
        from fauxgl_gb300 import _abi, scenes
        self.lib, self.mesh_h, self.w, self.h = lib, mesh_h, w, h
        self.ctx = ctypes.c_void_p()
        _abi.check(lib.fgc_context_create(w, h, ctypes.byref(self.ctx)))
        self.st = _abi.FgcState()
        lib.fgc_state_default(ctypes.byref(self.st))
        self.st.precision = precision
        self.sh = phong_struct(w, h)
        self.overlay = overlay
        if overlay:
            self.st2 = _abi.FgcState.from_buffer_copy(self.st)
            self.st2.wireframe = 1
            self.st2.depth_bias = 1e-5
            self.sh2 = overlay_struct(w, h)
        self.scale = scale
        self.pass_ms = [[0.0] * 5, [0.0] * 5]  # stage times summed over runs: main pass, overlay
        self.pass_work = [None, None]
        self.bg = (ctypes.c_double * 4)(*scenes.BACKGROUND)
        self.info = _abi.FgcRasterizeInfo()
        self.launches = 0
        self.ds = None
        if scale > 1:
            import numpy as np
            self.ds = np.empty((h // scale, w // scale, 4), dtype=np.uint8)

    def set_stream(self, stream):
        from fauxgl_gb300 import _abi
        _abi.check(self.lib.fgc_context_set_stream(self.ctx, stream))

    def set_timing(self, on):
        self.lib.fgc_context_set_timing(self.ctx, int(on))

    def stats(self):
        from fauxgl_gb300 import _abi
        s = _abi.FgcStats()
        _abi.check(self.lib.fgc_context_last_stats(self.ctx, ctypes.byref(s)))
        return s

    def run(self, record=True):
        """One frame: clears, the draw(s), the downsample. With record, also the
        draws' statistics (stage times, work, kernel launches); without, only
        the library calls (the timed frames), and the launches of the last
        recorded frame are returned."""
        from fauxgl_gb300 import _abi
        lib = self.lib
        _abi.check(lib.fgc_clear_color(self.ctx, self.bg))
        _abi.check(lib.fgc_clear_depth(self.ctx, 1.7976931348623157e308))
        _abi.check(lib.fgc_draw_mesh(self.ctx, self.mesh_h, ctypes.byref(self.st), ctypes.byref(self.sh),
                                     ctypes.byref(self.info)))
        if record:
            s = self.stats()
            launches = s.kernel_launches
            self.pass_ms[0] = [a + b for a, b in zip(self.pass_ms[0], s.stage_ms)]
            self.pass_work[0] = work_dict(s)
        if self.overlay:
            _abi.check(lib.fgc_draw_mesh(self.ctx, self.mesh_h, ctypes.byref(self.st2), ctypes.byref(self.sh2),
                                         ctypes.byref(self.info)))
            if record:
                s = self.stats()
                launches += s.kernel_launches
                self.pass_ms[1] = [a + b for a, b in zip(self.pass_ms[1], s.stage_ms)]
                self.pass_work[1] = work_dict(s)
        if self.ds is not None:
            _abi.check(lib.fgc_downsample(self.ctx, self.scale,
                                          self.ds.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8))))
            if record:
                launches += 1
        if record:
            self.launches = launches
        return self.launches

    def close(self):
        self.lib.fgc_context_destroy(self.ctx)


def time_frames(frame, steps, warmup, torch, dist_barrier, stage_acc=None, record=False):
    """Device-timed frames on torch's current stream (the library launches on
    it). Returns (ms per frame, launches per frame). The timed frames read the
    draws' statistics only with stage_acc or record."""
    stream = torch.cuda.current_stream()
    frame.set_stream(stream.cuda_stream)
    for _ in range(warmup):
        frame.run()
    dist_barrier()
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    launches = 0
    e0.record(stream)
    for _ in range(steps):
        launches += frame.run(record=record or stage_acc is not None)
        if stage_acc is not None:
            s = frame.stats()
            for i in range(5):
                stage_acc[i] += s.stage_ms[i]
    e1.record(stream)
    torch.cuda.synchronize()
    dist_barrier()
    return e0.elapsed_time(e1) / steps, launches // max(steps, 1)


BATCH_WORKLOAD = ("batched thumbnails: 256 seeded meshes (displaced icospheres, cylinders, cones; 200-200k "
                  "triangles log-uniform, seed 3) x 4 cameras = 1,024 views at 256^2-1024^2, PhongShader with a "
                  "random object colour, back-face culling, mixed precision, colour+depth clear per view")


def bench_batch(lib, args, torch):
    """Config-3 batch: every step renders all 1,024 views (clears included)
    through fgc_batch_submit / fgc_batch_wait. Returns the 'batch' JSON object."""
    import numpy as np
    from fauxgl_gb300 import _abi, scenes
    from fauxgl_gb300.context import _upload_mesh
    from fauxgl_gb300.shader import NewPhongShader, to_fgc_shader
    t0 = time.time()
    meshes, views = scenes.thumbnail_batch()
    if args.batch_views > 0:
        views = views[:args.batch_views]
    handles = [_upload_mesh(m) for m in meshes]
    log("batch scene: %d meshes, %d views, %d triangles drawn per batch (%.1fs)" % (
        len(meshes), len(views), sum(meshes[v["mesh"]].ntri for v in views), time.time() - t0))
    ctxs, keep = [], []
    items = (_abi.FgcBatchItem * len(views))()
    bg = (ctypes.c_double * 4)(*scenes.BACKGROUND)
    out_bytes = 0
    for i, v in enumerate(views):
        c = ctypes.c_void_p()
        _abi.check(lib.fgc_context_create(v["width"], v["height"], ctypes.byref(c)))
        ctxs.append(c)
        st = _abi.FgcState()
        lib.fgc_state_default(ctypes.byref(st))
        st.precision = _abi.FGC_PRECISION_MIXED
        sh = NewPhongShader(v["matrix"], scenes.LIGHT, v["eye"])
        sh.ObjectColor = v["color"]
        shs = to_fgc_shader(sh)
        keep += [st, shs]
        m = meshes[v["mesh"]]
        it = items[i]
        it.context, it.mesh = c.value, handles[v["mesh"]]
        it.tri_first, it.tri_count, it.line_first, it.line_count = 0, m.ntri, 0, m.nline
        it.state, it.shader = ctypes.pointer(st), ctypes.pointer(shs)
        out_bytes += v["width"] * v["height"] * 4
    n = len(views)
    b = ctypes.c_void_p()
    _abi.check(lib.fgc_batch_create(ctypes.byref(b)))
    stream = torch.cuda.current_stream()
    _abi.check(lib.fgc_batch_set_stream(b, stream.cuda_stream))
    infos = (_abi.FgcRasterizeInfo * n)()

    def clears():
        for c in ctxs:
            lib.fgc_clear_color(c, bg)
            lib.fgc_clear_depth(c, 1.7976931348623157e308)

    def step():
        clears()
        _abi.check(lib.fgc_batch_submit(b, items, n))
        _abi.check(lib.fgc_batch_wait(b, infos))

    def timed(steps, warmup):
        for _ in range(warmup):
            step()
        torch.cuda.synchronize()
        lat = []
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(steps):
            t = time.perf_counter()
            step()
            lat.append((time.perf_counter() - t) * 1e3)
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / steps, lat

    # autotune the pipeline shapes on this batch (results never depend on them)
    tuned = _abi.FgcBatchTuning()
    if args.batch_tuning == "auto":
        clears()
        _abi.check(lib.fgc_batch_autotune(b, items, n, 1, ctypes.byref(tuned)))
    else:
        bp, pb, fc, win = (int(x) for x in args.batch_tuning.split(","))
        tuned = _abi.FgcBatchTuning(bp, pb, fc, 0, win, 0)
        _abi.check(lib.fgc_batch_set_tuning(b, ctypes.byref(tuned)))
    tuning = {k: int(getattr(tuned, k)) for k, _ in _abi.FgcBatchTuning._fields_}
    log("batch tuning:", tuning)
    steps = max(3, args.batch_steps)
    ms, lat = timed(steps, 2)
    st = _abi.FgcStats()
    _abi.check(lib.fgc_batch_last_stats(b, ctypes.byref(st)))
    _abi.check(lib.fgc_batch_set_timing(b, 1))
    step()
    stt = _abi.FgcStats()
    _abi.check(lib.fgc_batch_last_stats(b, ctypes.byref(stt)))
    _abi.check(lib.fgc_batch_set_timing(b, 0))
    # the same submission as a CUDA graph
    tuned.use_graph = 1
    _abi.check(lib.fgc_batch_set_tuning(b, ctypes.byref(tuned)))
    g_ms, g_lat = timed(steps, 2)
    tuned.use_graph = 0
    _abi.check(lib.fgc_batch_set_tuning(b, ctypes.byref(tuned)))
    # end to end: every view's frame read back into pinned host memory
    pinned = torch.empty(out_bytes, dtype=torch.uint8, pin_memory=True)
    base, off = pinned.data_ptr(), 0
    for i, v in enumerate(views):
        items[i].out_nrgba = base + off
        items[i].out_scale = 1
        off += v["width"] * v["height"] * 4
    e_ms, e_lat = timed(steps, 1)
    for i in range(n):
        items[i].out_nrgba = None
    # unbatched: the same views one fgc_draw_mesh each
    info1 = _abi.FgcRasterizeInfo()
    for c in ctxs:
        _abi.check(lib.fgc_context_set_stream(c, stream.cuda_stream))

    def one_by_one():
        clears()
        for i in range(n):
            it = items[i]
            _abi.check(lib.fgc_draw_triangles(ctxs[i], it.mesh, 0, it.tri_count, it.state, it.shader,
                                              ctypes.byref(info1)))
    one_by_one()
    torch.cuda.synchronize()
    t = time.perf_counter()
    one_by_one()
    torch.cuda.synchronize()
    single_ms = (time.perf_counter() - t) * 1e3
    lib.fgc_batch_destroy(b)
    for c in ctxs:
        lib.fgc_context_destroy(c)
    tris = sum(meshes[v["mesh"]].ntri for v in views)

    def pct(x, q):
        x = sorted(x)
        return x[min(len(x) - 1, int(round(q * (len(x) - 1))))]
    return {
        "workload": BATCH_WORKLOAD, "views_per_batch": n, "triangles_per_batch": tris,
        "value": round(n * 1e3 / ms, 1), "unit": "views/s", "ms_per_batch": round(ms, 3),
        "latency_ms": {"p50": round(pct(lat, 0.5), 3), "p99": round(pct(lat, 0.99), 3), "steps": steps},
        "mtri_per_s": round(tris / ms / 1e3, 1), "gfragments_per_s": round(st.covered_pixels / ms / 1e6, 3),
        "graph": {"value": round(n * 1e3 / g_ms, 1), "ms_per_batch": round(g_ms, 3),
                  "latency_ms": {"p50": round(pct(g_lat, 0.5), 3), "p99": round(pct(g_lat, 0.99), 3)}},
        "e2e": {"value": round(n * 1e3 / e_ms, 1), "unit": "views/s", "ms_per_batch": round(e_ms, 3),
                "latency_ms": {"p50": round(pct(e_lat, 0.5), 3), "p99": round(pct(e_lat, 0.99), 3)},
                "d2h_bytes_per_step": out_bytes,
                "h2d_bytes_per_step": n * (ctypes.sizeof(_abi.FgcState) + ctypes.sizeof(_abi.FgcShader))},
        "unbatched": {"value": round(n * 1e3 / single_ms, 1), "ms_per_batch": round(single_ms, 3),
                      "how": "the same views, one fgc_draw_triangles call each"},
        "tuning": tuning, "dtype": "f64+f32",
        "stages_ms": {k: round(v, 3) for k, v in zip(_abi.STAGE_NAMES, stt.stage_ms)},
        "work": {"passes_kernel_launches": int(st.kernel_launches), "bands": int(st.bands),
                 **{k: int(getattr(st, k)) for k in ("elements", "clipped", "primitives", "bin_entries",
                                                     "visited_pixels", "covered_pixels", "shaded_fragments",
                                                     "updated_pixels")}},
    }


MESHPREP_WORKLOAD = ("mesh preparation around the draw path on the dense 1,310,720-triangle mesh: LoadSTL of its "
                     "binary STL (62.9 MB, decode + face normals + weld on the GPU), SmoothNormalsThreshold(30 deg), "
                     "SmoothNormals, SharpEdges(30 deg), Silhouette(eye, 0.001); host wall time per call (each call "
                     "synchronises), against the oracle's single-threaded C restatement on the same data")


def bench_meshprep(lib, mesh, torch, cpu=True):
    """The §8(f) mesh-preparation rows, each one library call, timed end to
    end on the host (median of 5 after 1 warm-up); the oracle's C
    restatement timed once on the same inputs."""
    import struct
    import numpy as np
    from fauxgl_gb300 import scenes
    from fauxgl_gb300.meshops import DeviceMesh
    t0 = time.time()
    pos32 = np.ascontiguousarray(mesh.tri_pos, dtype="<f4").reshape(-1, 9)
    rec = np.zeros((mesh.ntri, 50), dtype=np.uint8)
    rec[:, 12:48] = pos32.view(np.uint8).reshape(-1, 36)
    data = b"meshprep".ljust(80, b" ") + struct.pack("<I", mesh.ntri) + rec.tobytes()
    log("meshprep: %d-byte STL built (%.1fs)" % (len(data), time.time() - t0))

    def med(fn, reps=5):
        fn()
        torch.cuda.synchronize()
        ts = []
        for _ in range(reps):
            t = time.perf_counter()
            fn()
            ts.append((time.perf_counter() - t) * 1e3)
        return round(statistics.median(ts), 3)

    eye = tuple(scenes.EYE)
    dm = DeviceMesh.load_stl(data)
    out = {"workload": MESHPREP_WORKLOAD, "triangles": mesh.ntri, "unit": "ms per call (host wall time)"}
    out["load_stl_ms"] = med(lambda: DeviceMesh.load_stl(data))
    out["smooth_normals_threshold_ms"] = med(lambda: dm.SmoothNormalsThreshold(scenes.Radians(30.0)))
    out["smooth_normals_ms"] = med(lambda: dm.SmoothNormals())
    dm = DeviceMesh.load_stl(data)
    out["sharp_edges_ms"] = med(lambda: dm.SharpEdges(scenes.Radians(30.0)))
    out["silhouette_ms"] = med(lambda: dm.Silhouette(eye, 0.001))
    out["sharp_edges_lines"] = dm.SharpEdges(scenes.Radians(30.0)).nline
    out["silhouette_lines"] = dm.Silhouette(eye, 0.001).nline
    out["mtri_per_s"] = {k[:-3]: round(mesh.ntri / v / 1e3, 1) for k, v in list(out.items()) if k.endswith("_ms")}
    if cpu:
        from oracle import oracle as O
        import math
        c = {}
        t = time.perf_counter()
        p, n = O.stl_parse(data)
        c["load_stl_ms"] = round((time.perf_counter() - t) * 1e3, 1)
        t = time.perf_counter()
        O.smooth_normals_threshold(p, n, math.cos(scenes.Radians(30.0)))
        c["smooth_normals_threshold_ms"] = round((time.perf_counter() - t) * 1e3, 1)
        t = time.perf_counter()
        O.smooth_normals(p, n)
        c["smooth_normals_ms"] = round((time.perf_counter() - t) * 1e3, 1)
        t = time.perf_counter()
        O.sharp_edges(p, scenes.Radians(30.0))
        c["sharp_edges_ms"] = round((time.perf_counter() - t) * 1e3, 1)
        t = time.perf_counter()
        O.silhouette(p, n, eye, 0.001)
        c["silhouette_ms"] = round((time.perf_counter() - t) * 1e3, 1)
        out["cpu_baseline"] = {"kind": "port", "cores": 1, "unit": "ms per call", **c,
                               "sample": "the same mesh, once each, oracle C restatement (sorting-based grouping)"}
    return out


SERVE_WORKLOAD = ("serving loop: pool of 64 resident meshes built as the dense and thumbnail workloads build them "
                  "(displaced icospheres of 5k-1.31M triangles log-uniform, capped cylinders and cones with 8-512 "
                  "segments; seed 4), "
                  "Poisson arrivals over the whole window at each rate, each request a random mesh, camera at "
                  "radius 3, resolution in {512^2, 1920x1080, 3840x2160}, supersampling scale in {1, 2, 4} "
                  "(box-downsampled on the device, result copied to the host), PhongShader with a random object "
                  "colour; requests waiting longer than the request timeout are shed")


def _pool_mesh(args):
    from fauxgl_gb300 import scenes
    from fauxgl_gb300.shapes import cylinder_segments
    kind, size, seed = args
    if kind == "sphere":
        m = scenes.displaced_sphere(size, seed=seed)
    else:
        m = cylinder_segments(size, capped=True, cone=(kind == "cone"))
        m.BiUnitCube()
    m.kind = kind
    return m


def serve_pool(n=64, seed=4, tri_min=5000, tri_max=1310720):
    """The serving workload's resident meshes, built on all host cores as the
    dense and thumbnail workloads build theirs: displaced icospheres at the
    subdivision nearest a triangle count drawn log-uniform from
    [tri_min, tri_max], and capped cylinders and cones with 8-512 segments."""
    import math
    import multiprocessing as mp
    from fauxgl_gb300 import scenes
    rng = scenes.SplitMix64(seed)
    jobs = []
    for i in range(n):
        t = math.exp(math.log(tri_min) + rng.uniform() * (math.log(tri_max) - math.log(tri_min)))
        kind = ("sphere", "cylinder", "cone")[int(rng.uniform() * 3)]
        if kind == "sphere":
            size = int(min(8, max(2, round(math.log(t / 20.0, 4)))))
        else:
            size = int(math.exp(math.log(8) + rng.uniform() * (math.log(512) - math.log(8))))
        jobs.append((kind, size, seed * 1000003 + i))
    weight = [20 * 4 ** j[1] if j[0] == "sphere" else j[1] for j in jobs]
    order = sorted(range(n), key=lambda i: -weight[i])  # biggest first
    with mp.get_context("spawn").Pool(min(n, os.cpu_count() or 1)) as p:
        built = p.map(_pool_mesh, [jobs[i] for i in order], chunksize=1)
    meshes = [None] * n
    for i, m in zip(order, built):
        meshes[i] = m
    return meshes


def serve_requests(meshes, n, seed):
    import math
    from fauxgl_gb300 import scenes
    from fauxgl_gb300.geom import V, Vector
    from fauxgl_gb300.serve import Request
    rng = scenes.SplitMix64(seed)
    sizes = [(512, 512), (1920, 1080), (3840, 2160)]
    out = []
    for _ in range(n):
        mi = int(rng.uniform() * len(meshes))
        az = 2 * math.pi * rng.uniform()
        el = math.radians(-30.0 + 75.0 * rng.uniform())
        eye = Vector(3 * math.cos(el) * math.cos(az), 3 * math.sin(el), 3 * math.cos(el) * math.sin(az))
        w, h = sizes[int(rng.uniform() * 3)]
        s = [1, 2, 4][int(rng.uniform() * 3)]
        m = scenes.camera_matrix(w * s, h * s, eye=eye, center=V(0, 0, 0))
        out.append(Request(mesh=mi, matrix=tuple(m), eye=tuple(eye),
                           color=(rng.uniform(), rng.uniform(), rng.uniform(), 1.0), width=w, height=h, scale=s,
                           light=tuple(scenes.LIGHT), background=tuple(scenes.BACKGROUND)))
    return out


def bench_serve(args, meshes):
    """Config-4 serving loop, mixed and plain forms: the saturation throughput
    of a closed loop (the queue never runs dry), then each offered rate over
    its whole arrival window with load shedding (requests that wait longer
    than the request timeout expire)."""
    from fauxgl_gb300 import _abi
    from fauxgl_gb300.serve import Server, latency_summary, poisson_arrivals, run_load
    rates = [50, 200, 500, 1000, 2000]
    out = {"workload": SERVE_WORKLOAD, "pool_triangles": sum(m.ntri for m in meshes),
           "pool_kinds": {k: sum(1 for m in meshes if getattr(m, "kind", None) == k)
                          for k in ("sphere", "cylinder", "cone")},
           "window_s": args.serve_seconds, "request_timeout_s": args.serve_timeout, "saturation": {}, "rates": {}}
    for form, prec in (("mixed", _abi.FGC_PRECISION_MIXED), ("plain", _abi.FGC_PRECISION_PLAIN)):
        srv = Server(meshes, hbm_budget=args.serve_budget_gb << 30, slots=3, max_batch=32, precision=prec,
                     request_timeout=args.serve_timeout)
        warm = serve_requests(meshes, 6, seed=99)
        run_load(srv, warm, [0.0] * len(warm))
        # saturation: keep the queue full for the window, after a window of
        # the same load that creates the contexts the mix needs
        reqs = iter(serve_requests(meshes, 100000, seed=77))
        for measured in (False, True):
            t0 = time.perf_counter()
            done, frags = 0, 0
            while time.perf_counter() - t0 < args.serve_seconds:
                while len(srv.pending) < 2 * srv.max_batch:
                    srv.submit(next(reqs))
                for t in srv.poll():
                    done += 1
                    frags += t.info[0]
        el = time.perf_counter() - t0
        for t in list(srv.pending):  # the queue's remainder is not part of the measurement
            srv.cancel(t)
        srv.drain()
        out["saturation"][form] = {"frames_per_s": round(done / el, 2), "gfragments_per_s": round(frags / el / 1e9, 3),
                                   "window_s": round(el, 3)}
        log("serve %s saturation: %s" % (form, out["saturation"][form]))
        res = {}
        for k, rate in enumerate(rates):
            arr = poisson_arrivals(float(rate), args.serve_seconds, seed=40 + k)
            reqs = serve_requests(meshes, len(arr), seed=400 + k)
            tickets, elapsed = run_load(srv, reqs, arr)
            lat = latency_summary(tickets)
            served = [t for t in tickets if t.done]
            frags = sum(t.info[0] for t in served)
            res[str(rate)] = {"offered": len(reqs), "served": len(served),
                              "expired": sum(1 for t in tickets if t.status == "expired"),
                              "elapsed_s": round(elapsed, 3), "frames_per_s": round(len(served) / elapsed, 2),
                              "gfragments_per_s": round(frags / elapsed / 1e9, 3), **lat}
            log("serve %s %4d req/s: %s" % (form, rate, res[str(rate)]))
        out["rates"][form] = res
        srv.trim()
        del srv
    return out


ACCURACY_NOTE = ("checker leg, outside every timed region: each configuration drawn once per form through the C ABI "
                 "and compared with the oracle (the FP64 C restatement in the reference's sequential order) on the "
                 "same inputs; colour errors per NRGBA channel as fractions of full scale (1/255 = 0.00392), "
                 "shaded_* the pre-quantisation shader output where the winners agree")


def _accuracy_frame(lib, mesh_h, w, h, draws, precision, ref, shaded, clear):
    """One GPU frame of the draws with winner (and shaded-colour) debug
    outputs, compared with the oracle frame ref."""
    from fauxgl_gb300 import _abi
    from fauxgl_gb300.context import NewContext
    from oracle import oracle as O
    ctx = NewContext(w, h)
    ctx.SetDebug(_abi.FGC_DEBUG_WINNER | (_abi.FGC_DEBUG_SHADED_COLOR if shaded else 0))
    ctx.ClearColorBufferWith(clear)
    for st, sh in draws:
        st = _abi.FgcState.from_buffer_copy(st)
        st.precision = precision
        info = _abi.FgcRasterizeInfo()
        _abi.check(lib.fgc_draw_mesh(ctx.handle, mesh_h, ctypes.byref(st), ctypes.byref(sh), ctypes.byref(info)))
    err = O.frame_error(ctx.Image(), ctx.DepthBuffer, ctx.Winner(), ref, shaded=ctx.ShadedColor() if shaded else None)
    return ctx, err


def bench_accuracy(lib, dense, dense_h):
    """Max and mean per-channel colour error and the winner-mismatch fraction
    of both forms against the FP64 oracle, for the 512^2 icosphere frame, the
    dense 1080p frame, the 16x supersampled frame with its overlay (and its
    downsampled image) and a covering subset of the thumbnail views."""
    import numpy as np
    from fauxgl_gb300 import _abi, scenes
    from fauxgl_gb300.context import _upload_mesh
    from fauxgl_gb300.shader import NewPhongShader, to_fgc_shader
    from oracle import oracle as O
    forms = (("plain", _abi.FGC_PRECISION_PLAIN), ("mixed", _abi.FGC_PRECISION_MIXED))
    out = {"note": ACCURACY_NOTE}
    t0 = time.time()

    def one(name, mesh, mesh_h, w, h, draws, shaded=True, scale=1):
        ref = O.OracleContext(w, h)
        ref.clear_color(scenes.BACKGROUND)
        for st, sh in draws:
            ref.draw(mesh, st, sh)
        res = {}
        for form, prec in forms:
            ctx, err = _accuracy_frame(lib, mesh_h, w, h, draws, prec, ref, shaded, scenes.BACKGROUND)
            if scale > 1:
                d = np.abs(ctx.Downsample(scale).astype(np.int16) - O.downsample(ref.color(), scale).astype(np.int16))
                err["downsampled"] = {"max_err": round(float(d.max()) / 255.0, 6),
                                      "mean_err": float("%.3g" % (float(d.mean()) / 255.0))}
            res[form] = err
        out[name] = res

    st0 = _abi.state_default()
    c0 = scenes.sphere_scene(4)
    one("c0_sphere_512", c0, _upload_mesh(c0), 512, 512, [(st0, phong_struct(512, 512))])
    one("c1_dense_1080p", dense, dense_h, W, H, [(st0, phong_struct(W, H))])
    st2 = _abi.state_default()
    st2.wireframe, st2.depth_bias = 1, 1e-5
    one("c2_dense_16xss_overlay", dense, dense_h, W * SS, H * SS,
        [(st0, phong_struct(W * SS, H * SS)), (st2, overlay_struct(W * SS, H * SS))], shaded=False, scale=SS)
    # a covering subset of the thumbnail batch, each view compared on its own
    _, views = scenes.thumbnail_batch(build=set())
    pick = scenes.thumbnail_check_views(views)
    meshes, views = scenes.thumbnail_batch(build={views[i]["mesh"] for i in pick})
    agg = {form: {"pixels": 0, "max_err": 0.0, "sum_err": 0.0, "winner_mismatches": 0, "depth_mismatches": 0,
                  "shaded_max_err": 0.0} for form, _ in forms}
    for i in pick:
        v = views[i]
        m = meshes[v["mesh"]]
        sh = NewPhongShader(v["matrix"], scenes.LIGHT, v["eye"])
        sh.ObjectColor = v["color"]
        shs = to_fgc_shader(sh)
        ref = O.OracleContext(v["width"], v["height"])
        ref.clear_color(scenes.BACKGROUND)
        ref.draw(m, st0, shs)
        for form, prec in forms:
            _, err = _accuracy_frame(lib, _upload_mesh(m), v["width"], v["height"], [(st0, shs)], prec, ref, True,
                                     scenes.BACKGROUND)
            a = agg[form]
            n = err["pixels"]
            a["pixels"] += n
            a["max_err"] = max(a["max_err"], err["max_err"])
            a["sum_err"] += err["mean_err"] * n
            a["winner_mismatches"] += round(err["winner_mismatch_frac"] * n)
            a["depth_mismatches"] += round(err["depth_mismatch_frac"] * n)
            a["shaded_max_err"] = max(a["shaded_max_err"], err["shaded_max_err"])
    out["c3_thumbnail_views"] = {"views": len(pick), "kinds_x_resolutions": len({(views[i]["kind"], views[i]["width"])
                                                                                  for i in pick})}
    for form, _ in forms:
        a = agg[form]
        out["c3_thumbnail_views"][form] = {
            "pixels": a["pixels"], "max_err": a["max_err"],
            "mean_err": float("%.3g" % (a["sum_err"] / max(a["pixels"], 1))),
            "winner_mismatch_frac": a["winner_mismatches"] / max(a["pixels"], 1),
            "depth_mismatch_frac": a["depth_mismatches"] / max(a["pixels"], 1),
            "shaded_max_err": a["shaded_max_err"]}
    out["seconds"] = round(time.time() - t0, 1)
    return out


def cpu_frames(mesh, nframes, nthreads):
    """The oracle's threaded form (the reference's own worker split) on the
    host cores: one warm-up frame, then the median of nframes."""
    from fauxgl_gb300 import _abi, scenes
    from oracle import oracle as O
    st = _abi.state_default()
    sh = phong_struct(W, H)
    ctx = O.OracleContext(W, H)
    times = []
    for i in range(nframes + 1):
        ctx.clear_color(scenes.BACKGROUND)
        ctx.clear_depth(1.7976931348623157e308)
        t = time.perf_counter()
        ctx.draw(mesh, st, sh, nthreads=nthreads)
        dt = time.perf_counter() - t
        if i > 0:
            times.append(dt)
    return statistics.median(times), times


# Algorithmic HBM bytes of a frame (each byte the frame must move once): the
# mesh's per-corner records the plain form reads (position + normal, 2 x 3
# FP64 per corner, 144 B per triangle) and one fused clear-and-write pass of
# the NRGBA colour (4 B) and FP64 depth (8 B) of every pixel.
BYTES_PER_TRIANGLE_PLAIN = 144
BYTES_PER_PIXEL = 12


def load_profile(name):
    """A committed ncu summary (profiles/<name>.json): the DRAM traffic per
    launch of a kernel of this version, with the command that measured it."""
    p = os.path.join(ROOT, "profiles", name + ".json")
    if not os.path.exists(p):
        return None
    with open(p) as f:
        return json.load(f)


def hbm_peak():
    """(GB/s, source): the measured copy bandwidth of the GB300s
    (MEASURED_PEAKS.json hbm_gbs) when the file is present, else the value it
    held when it was last present here."""
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            d = json.load(f)
        for k in ("hbm_gbs", "hbm_GBps", "hbm"):
            if isinstance(d.get(k), (int, float)):
                return float(d[k]), "measured (MEASURED_PEAKS.json %s)" % k
    except (OSError, ValueError, AttributeError):
        pass
    return 6694.5, "measured copy bandwidth of this pool's GB300s (MEASURED_PEAKS.json hbm_gbs, as last recorded)"


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    nthreads = os.cpu_count() or 1
    mesh = build_scene()
    from fauxgl_gb300 import _abi, scenes
    from oracle import oracle as O
    st = _abi.state_default()
    sh = phong_struct(W, H)
    ctx = O.OracleContext(W, H)

    def frame():
        ctx.clear_color(scenes.BACKGROUND)
        ctx.clear_depth(1.7976931348623157e308)
        ctx.draw(mesh, st, sh, nthreads=nthreads)

    for _ in range(args.warmup):
        frame()
    t = time.perf_counter()
    for _ in range(args.steps):
        frame()
    dt = (time.perf_counter() - t) / args.steps
    fps = 1.0 / dt
    out = {
        "impl": "reference", "metric": METRIC, "value": round(fps, 3), "unit": "frames/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(dt * 1e3, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": WORKLOAD, "form": "reference arithmetic (FP64)",
                   "implementation": "C restatement of the reference's rasterizer run with the reference's own "
                                     "worker split (i %% %d), 256 striped locks; no Go toolchain on this "
                                     "machine" % nthreads},
        "cpu_baseline": {"value": round(fps, 3), "unit": "frames/s", "cores": nthreads, "kind": "port",
                         "sample": "%d frames after %d warm-up frames" % (args.steps, args.warmup)},
        "e2e": {"value": round(fps, 3), "unit": "frames/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out), flush=True)
    return 0


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    # the serving pool is built by spawned workers before any GPU work
    single = dist_env()[1] == 1  # the batch and serving workloads run at N=1 only
    pool = serve_pool() if args.only in ("all", "serve") and args.serve_seconds > 0 and single else None
    import numpy as np
    import torch
    from fauxgl_gb300 import _abi
    from fauxgl_gb300.context import _upload_mesh

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

        def barrier():
            dist.barrier()
    else:
        def barrier():
            pass
    lib = _abi.load_library()
    mesh = build_scene(args.detail)
    mesh_h = _upload_mesh(mesh)
    gops = ctypes.c_double()
    _abi.check(lib.fgc_measure_fp64_rate(ctypes.byref(gops)))
    fp64_peak_tflops = gops.value / 1e3

    if args.only == "ss16":
        f = Frame(lib, mesh_h, W * SS, H * SS, _abi.FGC_PRECISION_PLAIN, overlay=True, scale=SS)
        ss_ms, _ = time_frames(f, args.steps, args.warmup, torch, barrier)
        print(json.dumps({"ss16_plain_ms_per_frame": round(ss_ms, 3), "steps": args.steps,
                          "work": {"surface": f.pass_work[0], "overlay": f.pass_work[1]}}), flush=True)
        f.close()
        return 0
    if args.only == "batch":
        print(json.dumps({"batch": bench_batch(lib, args, torch)}), flush=True)
        return 0
    if args.only == "mixed":
        f = Frame(lib, mesh_h, W, H, _abi.FGC_PRECISION_MIXED)
        f.set_timing(True)
        stage = [0.0] * 5
        mixed_ms, _ = time_frames(f, args.steps, args.warmup, torch, barrier, stage)
        print(json.dumps({"mixed_ms_per_frame": round(mixed_ms, 4), "value": round(1e3 / mixed_ms, 3),
                          "stages_ms": {k: round(v / args.steps, 4) for k, v in zip(_abi.STAGE_NAMES, stage)},
                          "work": work_dict(f.stats()), "steps": args.steps}), flush=True)
        f.close()
        return 0
    if args.only == "serve":
        print(json.dumps({"serve": bench_serve(args, pool)}), flush=True)
        return 0
    if args.only == "meshprep":
        print(json.dumps({"meshprep": bench_meshprep(lib, mesh, torch)}), flush=True)
        return 0
    if args.only == "accuracy":
        print(json.dumps({"accuracy": bench_accuracy(lib, mesh, mesh_h)}), flush=True)
        return 0

    # ---- headline: plain FP64 at 1080p, mesh resident ------------------------
    # nvidia-smi samples the clocks over all GPU measurements below.
    clocks = ClockSampler(local)
    clocks.__enter__()
    plain = Frame(lib, mesh_h, W, H, _abi.FGC_PRECISION_PLAIN)
    ms, launches = time_frames(plain, args.steps, args.warmup, torch, barrier)
    # the stage breakdown comes from a second, shorter run with the library's
    # per-stage events on (they cost host time between frames, so the
    # headline frames above run without them)
    plain.set_timing(True)
    n_stage = max(3, min(args.steps, 10))
    stage = [0.0] * 5
    time_frames(plain, n_stage, 1, torch, barrier, stage)
    stage = [s / n_stage for s in stage]
    st = plain.stats()
    info = (plain.info.total_pixels, plain.info.updated_pixels)
    plain.set_timing(False)

    e2e_ms = mixed_ms = e2e_upload = None
    ss = {}
    h2d = ctypes.sizeof(_abi.FgcState) + ctypes.sizeof(_abi.FgcShader) + 2 * 32
    d2h = W * H * 4 + ctypes.sizeof(_abi.FgcRasterizeInfo)
    if args.only == "all":
        # ---- e2e through the C ABI with the frame read back each step -------
        pinned = torch.empty((H, W, 4), dtype=torch.uint8, pin_memory=True)
        ptr = ctypes.cast(pinned.data_ptr(), ctypes.POINTER(ctypes.c_uint8))

        def e2e_frame():
            plain.run()
            _abi.check(lib.fgc_read_color(plain.ctx, ptr))

        for _ in range(args.warmup):
            e2e_frame()
        barrier()
        torch.cuda.synchronize()
        stream = torch.cuda.current_stream()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.steps):
            e2e_frame()
        e1.record(stream)
        torch.cuda.synchronize()
        barrier()
        e2e_ms = e0.elapsed_time(e1) / args.steps

        # ---- the same with the mesh uploaded every frame (not resident) ----
        # fgc_mesh_upload from the host arrays (positions + normals), clears,
        # the draw, the read-back, fgc_mesh_release: what DrawMesh of a mesh
        # that was not made resident costs
        tp = np.ascontiguousarray(mesh.tri_pos)
        tn = np.ascontiguousarray(mesh.tri_nrm)
        up_steps = max(3, min(args.steps, 5))

        def upload_frame():
            h = ctypes.c_void_p()
            _abi.check(lib.fgc_mesh_upload(_abi.dptr(tp), _abi.dptr(tn), None, None, mesh.ntri, None, None, None,
                                           None, 0, ctypes.byref(h)))
            plain.mesh_h = h.value
            plain.run()
            _abi.check(lib.fgc_read_color(plain.ctx, ptr))
            _abi.check(lib.fgc_mesh_release(h))
            plain.mesh_h = mesh_h

        upload_frame()
        torch.cuda.synchronize()
        t_up = time.perf_counter()
        for _ in range(up_steps):
            upload_frame()
        torch.cuda.synchronize()
        upload_ms = (time.perf_counter() - t_up) * 1e3 / up_steps
        e2e_upload = {"value": round(world * 1e3 / upload_ms, 3), "unit": "frames/s", "steps": up_steps,
                      "h2d_bytes_per_step": h2d + tp.nbytes + tn.nbytes, "d2h_bytes_per_step": d2h,
                      "how": "fgc_mesh_upload of the 1,310,720 triangles' positions and normals from pageable host "
                             "memory, clears, fgc_draw_mesh, fgc_read_color, fgc_mesh_release every frame; host wall "
                             "time (the upload is synchronous)"}

        # ---- mixed form at 1080p --------------------------------------------
        mixed = Frame(lib, mesh_h, W, H, _abi.FGC_PRECISION_MIXED)
        mixed_ms, _ = time_frames(mixed, args.steps, args.warmup, torch, barrier)
        mixed.close()

        # ---- 16x supersampled frame + wireframe overlay + box downsample ----
        for name, prec in (("plain", _abi.FGC_PRECISION_PLAIN), ("mixed", _abi.FGC_PRECISION_MIXED)):
            f = Frame(lib, mesh_h, W * SS, H * SS, prec, overlay=True, scale=SS)
            f.set_timing(True)
            ss_ms, ss_launch = time_frames(f, args.ss_steps, 1, torch, barrier, record=True)
            n = args.ss_steps + 1
            ss[name] = {"value": round(1e3 / ss_ms, 3), "unit": "frames/s", "ms_per_frame": round(ss_ms, 3),
                        "stages_ms": {"surface": {k: round(v / n, 3) for k, v in zip(_abi.STAGE_NAMES, f.pass_ms[0])},
                                      "overlay": {k: round(v / n, 3) for k, v in zip(_abi.STAGE_NAMES, f.pass_ms[1])}},
                        "work": {"surface": f.pass_work[0], "overlay": f.pass_work[1]}}
            f.close()
    batch = serve = meshprep = None
    if args.only == "all" and args.batch_steps > 0 and single:
        batch = bench_batch(lib, args, torch)
    if args.only == "all" and single:
        meshprep = bench_meshprep(lib, mesh, torch, cpu=rank == 0)
    if args.only == "all" and pool is not None:
        serve = bench_serve(args, pool)
    clocks.__exit__(None, None, None)
    accuracy = None
    if args.only == "all" and not args.no_accuracy and rank == 0 and world == 1:
        accuracy = bench_accuracy(lib, mesh, mesh_h)
        log("accuracy:", json.dumps(accuracy))

    # ---- roofline of the dominant stage --------------------------------------
    names = list(_abi.STAGE_NAMES)
    dom = max(range(5), key=lambda i: stage[i])
    if names[dom] == "raster":
        flops = (FLOPS_PER_VISITED * st.visited_pixels + FLOPS_PER_COVERED * st.covered_pixels
                 + FLOPS_PER_SHADED_PHONG * st.shaded_fragments + st.shaded_fragments)
    elif names[dom] == "setup":
        flops = FLOPS_SETUP_PER_TRIANGLE * st.elements + FLOPS_SETUP_PER_PRIM * st.primitives
    elif names[dom] == "vertex":
        flops = FLOPS_VERTEX_PER_UNIQUE * st.unique_vertices
    else:
        flops = 0
    achieved = flops / (stage[dom] * 1e-3) / 1e12 if stage[dom] > 0 else 0.0
    # HBM view of the frame: algorithmic bytes (mesh records once, one
    # framebuffer pass) over the whole frame's time, and the raster kernel's
    # measured DRAM traffic per launch from the committed ncu summary
    frame_bytes = st.elements * BYTES_PER_TRIANGLE_PLAIN + W * H * BYTES_PER_PIXEL
    gbs_peak, gbs_src = hbm_peak()
    prof = load_profile("raster_kernel_dense1080p")
    traffic = prof.get("plain", {}).get("dram_bytes_per_launch") if prof else None

    # ---- CPU baseline (rank 0, N=1 only) ------------------------------------
    cpu = None
    if rank == 0 and world == 1 and args.cpu_frames > 0 and args.only == "all":
        nthreads = os.cpu_count() or 1
        cpu_dt, _ = cpu_frames(mesh, args.cpu_frames, nthreads)
        cpu = {"value": round(1.0 / cpu_dt, 3), "unit": "frames/s", "cores": nthreads, "kind": "port",
               "sample": "median of %d frames of this workload after 1 warm-up frame, the reference's "
                         "worker split over %d threads" % (args.cpu_frames, nthreads)}

    # max over ranks of the per-frame time
    if world > 1:
        ms, e2e_max, mixed_max = reduce_max([ms, e2e_ms or 0.0, mixed_ms or 0.0], "cuda")
        e2e_ms = e2e_max if e2e_ms else None
        mixed_ms = mixed_max if mixed_ms else None
    fps = replica_rate(ms, world)
    if rank == 0:
        out = {
            "metric": METRIC, "value": round(fps, 3), "unit": "frames/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(ms, 4), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": WORKLOAD, "form": "plain FP64 (bit-exact to the reference)",
                       "parallelism": "replicas" if world > 1 else "single GPU",
                       "l2": "inputs larger than L2 (mesh ~300 MB + framebuffer 25 MB resident; L2 129 MB)",
                       "rasterize_info": list(info)},
            "e2e": ({"value": round(world * 1e3 / e2e_ms, 3), "unit": "frames/s", "h2d_bytes_per_step": h2d,
                     "d2h_bytes_per_step": d2h, "mesh": "resident"} if e2e_ms else None),
            "e2e_upload": e2e_upload,
            "gpu_launches": launches * args.steps,
            "roofline": {"bound": "fp64", "kernel": names[dom] + "_kernel", "achieved": round(achieved, 4),
                         "peak": round(fp64_peak_tflops, 4), "unit": "TFLOP/s",
                         "frac": round(achieved / fp64_peak_tflops, 4) if fp64_peak_tflops else None,
                         "traffic": traffic,
                         "traffic_source": ("ncu dram__bytes_read.sum + dram__bytes_write.sum per launch, "
                                            "profiles/raster_kernel_dense1080p.json (%s)" % prof.get("version", "?"))
                         if prof else None,
                         "peak_source": "FP64 add (DADD) rate measured in this run by the library's own probe "
                                        "(fgc_measure_fp64_rate): the issue rate of the adds and multiplies the "
                                        "reference's arithmetic consists of, 84 % of ncu's FP64 pipe peak (which only "
                                        "DFMAs of general operands reach); the pool's MEASURED_PEAKS.json has no FP64 "
                                        "figure",
                         "flops_per_launch": int(flops),
                         "hbm": {"bound_of": "whole frame", "algorithmic_bytes": int(frame_bytes),
                                 "achieved": round(frame_bytes / (ms * 1e-3) / 1e9, 1),
                                 "peak": gbs_peak, "unit": "GB/s",
                                 "frac": round(frame_bytes / (ms * 1e-3) / 1e9 / gbs_peak, 4),
                                 "peak_source": gbs_src}},
            "stages_ms": {n: round(v, 4) for n, v in zip(names, stage)},
            "work": {"elements": st.elements, "unique_vertices": st.unique_vertices, "clipped": st.clipped,
                     "primitives": st.primitives, "bin_entries": st.bin_entries,
                     "visited_pixels": st.visited_pixels, "covered_pixels": st.covered_pixels,
                     "shaded_fragments": st.shaded_fragments, "updated_pixels": st.updated_pixels},
            "mixed": ({"value": round(world * 1e3 / mixed_ms, 3), "unit": "frames/s", "dtype": "f64+f32"}
                      if mixed_ms else None),
            "ss16": ss,
            "batch": batch,
            "serve": serve,
            "meshprep": meshprep,
            "accuracy": accuracy,
            "clocks": clocks.summary(),
        }
        if cpu is not None:
            out["cpu_baseline"] = cpu
        if args.detail != 8:
            out["config"]["workload"] = ("profiler case, not the benchmark's workload: displaced icosphere of "
                                         "subdivision %d (%d triangles), 1920x1080" % (args.detail, mesh.ntri))
        print(json.dumps(out), flush=True)
    plain.close()
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
