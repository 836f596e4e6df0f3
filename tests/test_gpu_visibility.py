"""The visibility pass of the differentiable path through the C ABI: the null pixel shader
(MLV_PS_NONE, depth and visibility only) and primitive-id targets placed on caller memory
(mlv_create_texture2d_on_memory), against the shaded pass and the oracle."""
import numpy as np
import pytest

from malevich_gb300 import api, scenes
from oracle import pyoracle

pytestmark = pytest.mark.gpu


def small_diff_scene():
    return scenes.diff_scene(seed=9, n_views=4, size=96, freq=12, tex_size=64)


def test_null_pixel_shader_keeps_colour_and_matches_depth_and_ids(device):
    sc = small_diff_scene()
    shaded = scenes.diff_frames(sc)
    bare = scenes.diff_frames(sc, shade=False)
    r1 = api.FrameRenderer(device, shaded, visibility=True, primitive_ids=True)
    r1.render_batched()
    r2 = api.FrameRenderer(device, bare, visibility=True, primitive_ids=True)
    ctx = device.immediate
    for rt, _, _ in r2.targets:
        ctx.clear_render_target(rt, (0.25, 0.5, 0.75, 1.0))
    r2.render_batched()
    import ctypes
    sentinel = np.uint32(pyoracle.oracle_lib().orc_encode_clear_color((ctypes.c_float * 4)(0.25, 0.5, 0.75, 1.0)))
    for k in range(len(shaded)):
        a, b = r1.read(k), r2.read(k)
        for key in ("depth", "vis_tri", "vis_draw", "vis_bary", "vis_prim"):
            assert np.array_equal(a[key].view(np.uint32), b[key].view(np.uint32)), key
        assert np.all(b["color"] == sentinel)
        o = pyoracle.render_oracle(bare[k])
        assert np.array_equal(b["vis_prim"], o["vis_prim"])
        assert np.array_equal(b["depth"].view(np.uint32), o["depth"].view(np.uint32))
    r1.destroy()
    r2.destroy()


def test_primitive_ids_placed_on_caller_memory(device):
    import torch
    sc = small_diff_scene()
    frames = scenes.diff_frames(sc, shade=False)
    n, s = len(frames), sc["width"]
    prim = torch.full((n, s, s), 7, dtype=torch.int32, device="cuda")
    r = api.FrameRenderer(device, frames, primitive_id_memory=[prim[i].data_ptr() for i in range(n)])
    r.render_batched()
    device.immediate.finish()
    placed = prim.cpu().numpy().view(np.uint32)
    for k in range(n):
        assert np.array_equal(placed[k], r.read(k)["vis_prim"])
        assert np.array_equal(placed[k], pyoracle.render_oracle(frames[k])["vis_prim"])
    r.destroy()
    # the library does not own placed memory: the tensor stays valid after destroy
    assert int(prim[0, 0, 0].item()) in (-1, int(placed[0, 0, 0].view(np.int32)))


def test_placed_texture_rejects_unaligned_memory(device):
    import ctypes
    import torch
    buf = torch.zeros(64 * 64 + 4, dtype=torch.int32, device="cuda")
    with pytest.raises(api.MalevichError):
        api.Texture2D(device, 64, 64, api.FORMAT_R32_UINT, bind=api.BIND_UNORDERED_ACCESS,
                      device_memory=buf.data_ptr() + 4)
    lib = api.load_library()
    h = ctypes.c_void_p()
    assert lib.mlv_create_texture2d_on_memory(device.handle, None, ctypes.c_void_p(buf.data_ptr()),
                                              ctypes.byref(h)) != 0


def test_queued_uploads_keep_queued_work_on_the_old_contents(device):
    """A queued upload after a queued draw does not change what that draw reads (the context
    synchronises first), and the next draw reads the new contents."""
    fr = scenes.small_scene(31, 64, 48, n_objects=2, level=2)
    r = api.FrameRenderer(device, fr)
    ctx = device.immediate
    r.render_per_draw()
    want_old = r.read(0)
    vb_buf, vb_arr = next(v for k, v in r._buffers.items() if k[1] == api.BIND_VERTEX_BUFFER)
    moved = np.ascontiguousarray(vb_arr.copy())
    moved[:, 0] += 0.25                       # shift the first mesh's object-space x
    r.render_per_draw()                       # queued
    ctx.update_buffer_async(vb_buf, moved)    # queued behind it
    ctx.finish()
    assert np.array_equal(r.read(0)["depth"].view(np.uint32), want_old["depth"].view(np.uint32))
    r.render_per_draw()
    new = r.read(0)
    for d in fr.draws:
        if d.vb is vb_arr:
            d.vb = moved
    want_new = pyoracle.render_oracle(fr)
    assert np.array_equal(new["depth"].view(np.uint32), want_new["depth"].view(np.uint32))
    assert not np.array_equal(new["depth"], want_old["depth"])
    ctx.update_buffer_async(vb_buf, np.ascontiguousarray(vb_arr))
    ctx.finish()
    r.destroy()


@pytest.mark.parametrize("batched", [True, False])
def test_null_pixel_shader_among_shaded_draws_of_one_view(device, batched):
    """A view whose draws mix the null pixel shader with shaded ones: depth, ids and barycentrics
    of every draw, the colour of the shaded draws' pixels (the null shader's pixels keep the
    colour below them)."""
    fr = scenes.small_scene(61, 80, 56, n_objects=4, level=3)
    for k, d in enumerate(fr.draws):
        if k % 2 == 1:
            d.ps = scenes.PS_NONE
    want = pyoracle.render_oracle(fr)
    r = api.FrameRenderer(device, fr, visibility=True)
    for _ in range(2 if batched else 1):
        r.render_batched() if batched else r.render_per_draw()
    got = r.read(0)
    r.destroy()
    for key in ("depth", "vis_tri", "vis_draw", "vis_bary"):
        assert np.array_equal(got[key].view(np.uint32), want[key].view(np.uint32)), key
    from helpers import assert_color_close
    assert_color_close(got["color"], want["color"])
