"""The tile kernel with several warps sharing one tile's triangles (mlv_tuning.warps_per_tile 2, 4
and 8) against the oracle and against one warp per tile: every output bit for bit, colour included
(the same fragments are shaded by the same code). Covers multi-draw hierarchical Z, both depth
functions, partial tiles, the fill-rule and sample-point modes, the null pixel shader with
primitive ids, folded clears, multi-view batches and the TileInfo capture."""
import numpy as np
import pytest

from helpers import assert_bits_equal, assert_color_close, sort_infos
from malevich_gb300 import api, scenes
from oracle import pyoracle

pytestmark = pytest.mark.gpu

KEYS = ("color", "depth", "vis_tri", "vis_draw", "vis_bary")


def render(device, frames, warps_per_tile, tile_warps=4, **kw):
    ctx = device.immediate
    base = ctx.tuning()
    ctx.set_tuning(warps_per_tile=warps_per_tile, tile_warps_per_block=tile_warps)
    try:
        r = api.FrameRenderer(device, frames, visibility=True, **kw)
        r.render_batched()   # eager, then graph replay
        r.render_batched()
        outs = [r.read(i) for i in range(len(r.frames))]
        r.destroy()
    finally:
        ctx.set_tuning(**base)
    return outs


def check(got, want_gpu, want_oracle):
    for k in KEYS:
        assert np.array_equal(got[k].view(np.uint32), want_gpu[k].view(np.uint32)), k
    assert_bits_equal(got["depth"], want_oracle["depth"], "depth")
    assert np.array_equal(got["vis_tri"], want_oracle["vis_tri"])
    assert_bits_equal(got["vis_bary"], want_oracle["vis_bary"], "barycentrics")
    assert_color_close(got["color"], want_oracle["color"])


SCENES = {
    "multi_draw_ge": lambda: scenes.small_scene(31, 64, 64, n_objects=5, level=3),
    "multi_draw_less": lambda: scenes.small_scene(32, 64, 64, n_objects=4, native=False),
    "partial_tiles": lambda: scenes.small_scene(33, 61, 45, n_objects=3),
    "lighting": lambda: scenes.small_scene(34, 80, 48, vs=scenes.VS_VERTEX_LIGHTING, ps=scenes.PS_ENV_LIGHTING,
                                           n_objects=3),
    "single_sphere": lambda: scenes.config1_plain(seed=1, width=320, height=192, tex_size=64, level=4),
}


@pytest.mark.parametrize("name", sorted(SCENES))
@pytest.mark.parametrize("wpt", [2, 4, 8])
def test_shared_tiles_match(device, name, wpt):
    fr = SCENES[name]()
    want = pyoracle.render_oracle(fr)
    base = render(device, [fr], 1)[0]
    got = render(device, [fr], wpt)[0]
    check(got, base, want)


@pytest.mark.parametrize("fill_rule,sample_center", [(1, 0), (0, 1), (1, 1)])
def test_shared_tiles_raster_modes(device, fill_rule, sample_center):
    fr = scenes.small_scene(35, 64, 64, n_objects=4, level=3)
    for d in fr.draws:
        d.fill_rule, d.sample_center = fill_rule, sample_center
    want = pyoracle.render_oracle(fr)
    base = render(device, [fr], 1)[0]
    for wpt in (4, 8):
        check(render(device, [fr], wpt)[0], base, want)


def test_shared_tiles_multiview_and_null_pixel_shader(device):
    sc = scenes.diff_scene(seed=13, n_views=3, size=96, freq=12, tex_size=16)
    frames = scenes.diff_frames(sc, shade=False)
    base = render(device, frames, 1, primitive_ids=True)
    got = render(device, frames, 2, primitive_ids=True)
    for k, f in enumerate(frames):
        want = pyoracle.render_oracle(f)
        assert np.array_equal(got[k]["vis_prim"], want["vis_prim"])
        assert np.array_equal(got[k]["vis_prim"], base[k]["vis_prim"])
        check(got[k], base[k], want)


def test_shared_tiles_batch_of_views(device):
    frames = scenes.config3_batched(seed=14, n_views=4, n_meshes=4, resolutions=(64, 96), tri_range=(300, 3000),
                                    draws_per_view=(2, 3), tex_size=32, n_textures=2)
    base = render(device, frames, 1, tile_warps=8)
    got = render(device, frames, 8)
    for k, f in enumerate(frames):
        check(got[k], base[k], pyoracle.render_oracle(f))


def test_shared_tiles_tile_infos(device):
    fr = scenes.small_scene(36, 64, 64, n_objects=1, level=4)
    want = pyoracle.render_oracle(fr, capture=True)["captures"][0]
    ctx = device.immediate
    base = ctx.tuning()
    ctx.set_tuning(warps_per_tile=4)
    r = api.FrameRenderer(device, fr, visibility=False)
    ctx.set_debug_capture(True)
    try:
        r.render_per_draw()
        tile, tri, mask = ctx.tile_infos()
    finally:
        ctx.set_debug_capture(False)
        ctx.set_tuning(**base)
        r.destroy()
    wt, wtri, wm = sort_infos(want["info_bin"], want["info_tri"], want["info_mask"])
    assert np.array_equal(tile, wt) and np.array_equal(tri, wtri)
    assert np.array_equal(mask, wm)


def test_warps_per_tile_is_validated(device):
    ctx = device.immediate
    with pytest.raises(api.MalevichError):
        ctx.set_tuning(warps_per_tile=3)
    assert ctx.tuning()["warps_per_tile"] == 1
