"""Meshes that change between draws, through the Python mirror of the Go API.

The reference's DrawMesh reads mesh.Triangles on every call
(context.go:435-439), so a program may edit a mesh between draws. The
binding uploads a mesh for each draw unless it was made resident; a resident
mesh is kept on the device and its copy is dropped by the Mesh methods that
change it, or by dirty() after an edit of its arrays in place."""
import numpy as np
import pytest

from fauxgl_gb300 import scenes
from fauxgl_gb300.context import NewContext
from fauxgl_gb300.geom import Translate, V
from fauxgl_gb300.shader import NewPhongShader
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def frame(mesh, w=200, h=150):
    ctx = NewContext(w, h)
    ctx.SetDebug(1)
    ctx.ClearColorBufferWith(scenes.BACKGROUND)
    sh = NewPhongShader(scenes.camera_matrix(w, h), scenes.LIGHT, scenes.EYE)
    sh.ObjectColor = scenes.OBJECT_COLOR
    ctx.Shader = sh
    info = ctx.DrawMesh(mesh)
    ref = O.OracleContext(w, h)
    ref.clear_color(scenes.BACKGROUND)
    rinfo = ref.draw(mesh, ctx.state(), ctx.shader_struct())
    assert tuple(info) == rinfo
    assert np.array_equal(ctx.Image(), ref.color())
    assert np.array_equal(ctx.Winner(), ref.winner())
    return ctx.Image()


def test_mesh_edited_in_place_between_draws(gpu_lib):
    mesh = scenes.sphere_scene(3)
    first = frame(mesh)
    mesh.tri_pos[: mesh.ntri // 2] *= 0.8  # shrink half the sphere, in place
    second = frame(mesh)
    assert not np.array_equal(first, second)


def test_resident_mesh_keeps_its_copy_until_dropped(gpu_lib):
    mesh = scenes.sphere_scene(3).MakeResident()
    frame(mesh)
    mesh.Transform(Translate(V(0.2, 0.0, 0.0)))  # a Mesh method drops the copy itself
    moved = frame(mesh)
    mesh.tri_pos[:] = mesh.tri_pos * 0.9          # an edit in place: dirty() before the next draw
    mesh.dirty()
    smaller = frame(mesh)
    assert not np.array_equal(moved, smaller)
