"""Clears folded into the tile kernel against the oracle and against unfolded fills: a cleared
target the segment never draws into, a render target that two views share, a non-default clear
depth, custom visibility clear values, and the null pixel shader over a folded colour clear."""
import ctypes

import numpy as np
import pytest

from helpers import assert_color_close
from malevich_gb300 import api, scenes
from oracle import pyoracle

pytestmark = pytest.mark.gpu


def encoded(rgba):
    return np.uint32(pyoracle.oracle_lib().orc_encode_clear_color((ctypes.c_float * 4)(*rgba)))


def test_cleared_target_without_draws_is_still_cleared(device):
    """Clear two render targets in one command list and draw into one of them: the other's clear
    is not folded (no view binds it) and must still happen."""
    fr = scenes.small_scene(41, 64, 48, n_objects=2, level=2)
    r = api.FrameRenderer(device, fr)
    other_rt = api.Texture2D(device, 64, 48, api.FORMAT_R8G8B8A8_UNORM, bind=api.BIND_RENDER_TARGET)
    other_ds = api.Texture2D(device, 64, 48, api.FORMAT_D32_FLOAT, bind=api.BIND_DEPTH_STENCIL)
    dctx = device.create_deferred_context()
    dctx.clear_render_target(other_rt, (0.1, 0.2, 0.3, 0.4))
    dctx.clear_depth(other_ds, 0.25)
    r._issue(dctx, fr, r.targets[0])
    cl = dctx.finish_command_list()
    dctx.destroy()
    for _ in range(2):                       # eager, then graph replay
        device.immediate.execute_command_list(cl)
        ctx = device.immediate
        assert np.all(ctx.read_texture(other_rt) == encoded((0.1, 0.2, 0.3, 0.4)))
        assert np.all(ctx.read_texture(other_ds) == np.float32(0.25))
        got, want = r.read(0), pyoracle.render_oracle(fr)
        assert np.array_equal(got["depth"].view(np.uint32), want["depth"].view(np.uint32))
        assert_color_close(got["color"], want["color"])
    cl.destroy()
    other_rt.destroy()
    other_ds.destroy()
    r.destroy()


def test_render_target_shared_by_two_views_keeps_its_fill(device):
    """One render target with two depth buffers (two views of one batch): its clear is not
    folded; the batch must equal the same draws issued one by one."""
    fr = scenes.small_scene(42, 64, 48, n_objects=2, level=2)
    r = api.FrameRenderer(device, fr)
    rt, ds, _ = r.targets[0]
    ds2 = api.Texture2D(device, 64, 48, api.FORMAT_D32_FLOAT, bind=api.BIND_DEPTH_STENCIL)

    def issue(ctx):
        ctx.clear_render_target(rt, fr.clear_color)
        ctx.clear_depth(ds, fr.clear_depth)
        ctx.clear_depth(ds2, fr.clear_depth)
        for k, d in enumerate(fr.draws):
            ctx.om_set_render_targets(rt, ds if k % 2 == 0 else ds2)
            ctx.ia_set_vertex_buffer(r._buffer(d.vb, api.BIND_VERTEX_BUFFER), d.vb_stride)
            ctx.ia_set_index_buffer(r._buffer(d.ib, api.BIND_INDEX_BUFFER))
            ctx.vs_set_shader(d.vs)
            ctx.ps_set_shader(d.ps)
            ctx.vs_set_constant_buffer(0, r._buffer(d.cb, api.BIND_CONSTANT_BUFFER))
            ctx.vs_set_shader_resource(0, r._texture(d.vs_tex))
            ctx.ps_set_shader_resource(0, r._texture(d.ps_tex))
            ctx.rs_set_viewport(d.viewport)
            ctx.rs_set_cull(d.cull)
            ctx.om_set_depth_func(d.depth_func)
            ctx.draw_indexed(d.index_count)

    ctx = device.immediate
    issue(ctx)
    ctx.finish()
    want = (ctx.read_texture(rt), ctx.read_texture(ds), ctx.read_texture(ds2))
    dctx = device.create_deferred_context()
    issue(dctx)
    cl = dctx.finish_command_list()
    dctx.destroy()
    for _ in range(2):
        ctx.execute_command_list(cl)
        got = (ctx.read_texture(rt), ctx.read_texture(ds), ctx.read_texture(ds2))
        for a, b in zip(got, want):
            assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
    cl.destroy()
    ds2.destroy()
    r.destroy()


@pytest.mark.parametrize("clear_depth", [0.0, 0.3])
def test_folded_clear_depth_values_match_the_oracle(device, clear_depth):
    fr = scenes.small_scene(43, 80, 56, n_objects=3, level=2)
    fr.clear_depth = clear_depth
    r = api.FrameRenderer(device, fr, visibility=True)
    r.render_batched()
    got, want = r.read(0), pyoracle.render_oracle(fr)
    for key in ("depth", "vis_tri", "vis_draw", "vis_bary"):
        assert np.array_equal(got[key].view(np.uint32), want[key].view(np.uint32)), key
    assert_color_close(got["color"], want["color"])
    r.destroy()


def test_folded_visibility_clears_and_null_pixel_shader(device):
    """Visibility targets cleared to custom values and a null-pixel-shader pass: pixels no draw
    wrote hold the clear values, and the colour target holds the clear colour everywhere."""
    sc = scenes.diff_scene(seed=12, n_views=2, size=64, freq=6, tex_size=16)
    frames = scenes.diff_frames(sc, shade=False)
    for f in frames:
        f.clear_color = (0.5, 0.25, 0.75, 1.0)
    r = api.FrameRenderer(device, frames, visibility=True, primitive_ids=True)
    ctx = device.immediate
    dctx = device.create_deferred_context()
    for f, tg, pr in zip(r.frames, r.targets, r.prim_targets):
        r._issue(dctx, f, tg, pr)
        dctx.clear_u32(tg[2][1], 0x12345678)     # the draw-id target, cleared again after the draws
    cl_a = dctx.finish_command_list()
    dctx.destroy()
    ctx.execute_command_list(cl_a)
    for k, f in enumerate(frames):
        got = r.read(k)
        want = pyoracle.render_oracle(f)
        assert np.array_equal(got["vis_prim"], want["vis_prim"])
        assert np.array_equal(got["depth"].view(np.uint32), want["depth"].view(np.uint32))
        assert np.all(got["color"] == encoded((0.5, 0.25, 0.75, 1.0)))
        assert np.all(got["vis_draw"] == np.uint32(0x12345678))   # cleared after the draws
    cl_a.destroy()
    r.destroy()
