"""fgc_depth_image_noalloc: DepthImage for callers that may not let the
library allocate device memory once they run (a render service that
reserves every buffer before admitting work, a host application that owns
its plugins' GPU memory). fgc_depth_image grows device staging buffers on
first use; the no-allocation variant keeps that scratch in one static 16 MiB
device array instead, which limits it to 2^23-pixel frames. That array, and
the kernels the call launches, are made resident when the first context on a
GPU is created, so the call itself leaves the device's free memory unchanged.

This file is collected last so that, if it fails, a run that stops at the
first failure has already run every other test."""
import ctypes

import numpy as np
import pytest

from fauxgl_gb300 import _abi, scenes
from fauxgl_gb300.context import NewContext
from fauxgl_gb300.shader import NewPhongShader

pytestmark = pytest.mark.gpu


def noalloc_image(lib, ctx):
    out = np.empty((ctx.Height, ctx.Width), dtype=np.uint16)
    _abi.check(lib.fgc_depth_image_noalloc(ctx.handle, out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint16))))
    return out


def draw_frame(ctx, mesh, eye):
    ctx.ClearColorBufferWith(scenes.BACKGROUND)
    ctx.ClearDepthBuffer()
    sh = NewPhongShader(scenes.camera_matrix(ctx.Width, ctx.Height, eye=eye), scenes.LIGHT, eye)
    sh.ObjectColor = scenes.OBJECT_COLOR
    ctx.Shader = sh
    ctx.DrawMesh(mesh)


def test_noalloc_depth_image_matches_depth_image_twice(gpu_lib):
    ctx = NewContext(640, 360)
    mesh = scenes.displaced_sphere(4)
    # two calls in a row, on two different frames: the shared scratch must
    # not carry the first frame's depth range into the second
    for eye in (scenes.EYE, scenes.V(2.5, -1.5, 2.0)):
        draw_frame(ctx, mesh, eye)
        expect = ctx.DepthImage()
        got = noalloc_image(gpu_lib, ctx)
        assert np.array_equal(got, expect)
        assert len(np.unique(got)) > 100  # a real depth gradient, not a constant image


def test_noalloc_depth_image_leaves_free_memory_unchanged(gpu_lib):
    import torch
    ctx = NewContext(512, 384)
    draw_frame(ctx, scenes.displaced_sphere(3), scenes.EYE)  # the draw's own buffers exist before the check
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    got = noalloc_image(gpu_lib, ctx)
    got2 = noalloc_image(gpu_lib, ctx)
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0, "the call changed free device memory by %d bytes" % (free0 - free1)
    assert np.array_equal(got, got2)
    assert np.array_equal(got, ctx.DepthImage())


def test_noalloc_depth_image_rejects_frames_above_its_limit(gpu_lib):
    ctx = NewContext(4097, 2048)  # 8,390,656 > 8,388,608 pixels
    out = np.empty((2048, 4097), dtype=np.uint16)
    rc = gpu_lib.fgc_depth_image_noalloc(ctx.handle, out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint16)))
    assert rc == _abi.FGC_ERR_INVALID_ARGUMENT
    assert b"8388608" in gpu_lib.fgc_last_error()
