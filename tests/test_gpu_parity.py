"""GPU draw path (through the C ABI) against the checkers: the reference's golden outputs and
the oracle restatement. Coverage, triangle ids, draw ids, barycentrics and depth are compared
bit for bit; UNORM8 colour within +-1 LSB (see helpers.COLOR_TOL)."""
import ctypes
import os

import numpy as np
import pytest

from conftest import GOLDEN
from helpers import assert_bits_equal, assert_color_close, color_diff, reference_nan_pixels, sort_infos
from malevich_gb300 import api, scenes
from oracle import pyoracle

pytestmark = pytest.mark.gpu

STATS = ("vertex_count", "input_triangle_count", "assembled_triangle_count", "active_bin_count",
         "total_triangle_count_in_bins")


def render_gpu(device, frame, batched=False):
    r = api.FrameRenderer(device, frame, visibility=True)
    ctx = device.immediate
    ctx.reset_stats()
    if batched:
        r.render_batched()
    else:
        r.render_per_draw()
    out = r.read(0)
    out["stats"] = ctx.stats()
    r.destroy()
    return out


def check_against_oracle(got, want, colour_outliers=0.0):
    assert_bits_equal(got["depth"], want["depth"], "depth")
    assert np.array_equal(got["vis_tri"], want["vis_tri"]), "triangle ids differ"
    assert np.array_equal(got["vis_draw"], want["vis_draw"]), "draw ids differ"
    assert_bits_equal(got["vis_bary"], want["vis_bary"], "barycentrics")
    assert_color_close(got["color"], want["color"], max_outlier_frac=colour_outliers)
    for k in STATS:
        assert got["stats"][k] == want["stats"][k], k


@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p)[:-4] for p in GOLDEN])
def test_gpu_matches_reference_golden(device, path):
    z = np.load(path)
    frame = scenes.frame_from_arrays(z)
    got = render_gpu(device, frame)
    assert_bits_equal(got["depth"], z["out/depth"], "depth")
    assert np.array_equal(got["vis_tri"], z["out/vis_tri"]), "triangle ids differ"
    assert np.array_equal(got["vis_draw"], z["out/vis_draw"]), "draw ids differ"
    assert [got["stats"][k] for k in STATS] == list(z["out/stats"])
    nan = reference_nan_pixels(z["out/color"])
    d = color_diff(got["color"], z["out/color"]).max(axis=-1)[~nan]
    # as the oracle's comparison with the same fixtures (tests/test_oracle.py): +-1 LSB with rare
    # outliers where the reference's approximate rsqrt moves a lat-long lookup across the seam or
    # a pole threshold; their fraction is bounded, and printed
    print("%s: %d of %d pixels beyond +-1 LSB of the reference, max %d, %d reference NaN pixels" % (
        os.path.basename(path), (d > 1).sum(), d.size, d.max(), nan.sum()))
    assert (d > 1).mean() <= 1e-3, np.bincount(d.ravel())
    assert d.max() <= 3 or path.endswith("scene_frame_480x272.npz"), np.bincount(d.ravel())


CASES = []
for seed in range(3):
    for vs, ps in [(1, 1), (2, 3), (2, 2), (1, 3)]:
        for inside in (False, True):
            CASES.append((seed, vs, ps, inside, True))
    CASES.append((seed, 1, 1, False, False))   # depth LESS, standard projection
    CASES.append((seed, 1, 3, True, False))


@pytest.mark.parametrize("seed,vs,ps,inside,native", CASES)
def test_gpu_matches_oracle_small(device, seed, vs, ps, inside, native):
    fr = scenes.small_scene(1000 + seed, 64, 64, vs=vs, ps=ps, inside=inside, native=native)
    check_against_oracle(render_gpu(device, fr), pyoracle.render_oracle(fr))


@pytest.mark.parametrize("w,h", [(60, 44), (8, 8), (1, 1), (13, 77)])
def test_gpu_partial_tiles(device, w, h):
    fr = scenes.small_scene(77, w, h, n_objects=3)
    check_against_oracle(render_gpu(device, fr), pyoracle.render_oracle(fr))


@pytest.mark.parametrize("cull", [scenes.CULL_NONE, scenes.CULL_FRONT, scenes.CULL_BACK])
def test_gpu_cull_modes(device, cull):
    fr = scenes.small_scene(5, 64, 64, n_objects=4)
    for d in fr.draws:
        d.cull = cull
    check_against_oracle(render_gpu(device, fr), pyoracle.render_oracle(fr))


def test_gpu_start_index_base_vertex_and_nonindexed(device):
    fr = scenes.small_scene(6, 64, 64, n_objects=2)
    d0 = fr.draws[0]
    # shift the vertices by 5 and the indices by 3 triangles: same triangles via start/base
    pad_v = np.zeros((5, 8), np.float32)
    d0.vb = np.concatenate([pad_v, d0.vb])
    d0.ib = np.concatenate([np.zeros(9, np.uint32), d0.ib])
    d0.start_index, d0.base_vertex = 9, 5
    # second draw non-indexed: de-index its triangles
    d1 = fr.draws[1]
    d1.vb = d1.vb[d1.ib[:d1.index_count - d1.index_count % 3]]
    d1.ib = None
    d1.index_count = len(d1.vb)
    check_against_oracle(render_gpu(device, fr), pyoracle.render_oracle(fr))


def test_gpu_index_count_not_multiple_of_8(device):
    fr = scenes.small_scene(8, 64, 64, n_objects=2)
    for d in fr.draws:
        d.index_count -= 2 * 3 + 1   # drop two triangles and leave a stray index
    check_against_oracle(render_gpu(device, fr), pyoracle.render_oracle(fr))


def test_gpu_tile_infos_match_oracle(device):
    """The per-(tile, triangle) coverage masks after hierarchical Z (TileInfo, main.c:159-162)."""
    fr = scenes.small_scene(12, 64, 64, n_objects=1, level=3)
    want = pyoracle.render_oracle(fr, capture=True)["captures"][0]
    r = api.FrameRenderer(device, fr, visibility=False)
    ctx = device.immediate
    ctx.set_debug_capture(True)
    try:
        r.render_per_draw()
        tile, tri, mask = ctx.tile_infos()
    finally:
        ctx.set_debug_capture(False)
        r.destroy()
    wt, wtri, wm = sort_infos(want["info_bin"], want["info_tri"], want["info_mask"])
    assert np.array_equal(tile, wt) and np.array_equal(tri, wtri)
    assert np.array_equal(mask, wm)


def test_gpu_fullscreen_triangles_use_block_binning(device):
    # two triangles covering a 1280x720 target: the cooperative path for triangles spanning many tiles
    z = np.load(os.path.join(os.path.dirname(__file__), "golden", "fullscreen_env.npz"))
    fr = scenes.frame_from_arrays(z)
    fr.width, fr.height = 1280, 720
    for d in fr.draws:
        d.viewport = (0.0, 0.0, 1280.0, 720.0, 0.0, 1.0)
    check_against_oracle(render_gpu(device, fr), pyoracle.render_oracle(fr))


def test_gpu_config1_plain_less(device):
    fr = scenes.config1_plain(seed=1, native=False)
    want = pyoracle.render_oracle(fr)
    got = render_gpu(device, fr)
    check_against_oracle(got, want, colour_outliers=1e-3)
    assert want["stats"]["assembled_triangle_count"] > 5000


def test_gpu_config1_plain_reference_mode(device):
    fr = scenes.config1_plain(seed=1, native=True)
    check_against_oracle(render_gpu(device, fr), pyoracle.render_oracle(fr), colour_outliers=1e-3)


def test_gpu_batched_equals_per_draw_and_oracle_scene(device):
    fr = scenes.config2_scene(seed=2, width=480, height=272, ground_cells=96, counts=[3000, 5000, 8000, 2000],
                              radiance_size=(256, 128), ground_tex=0)
    a = render_gpu(device, fr, batched=False)
    b = render_gpu(device, fr, batched=True)
    for k in ("color", "depth", "vis_tri", "vis_draw", "vis_bary"):
        assert np.array_equal(a[k], b[k]), k
    check_against_oracle(b, pyoracle.render_oracle(fr), colour_outliers=1e-3)


def test_gpu_batched_multi_view(device):
    frames = scenes.config3_batched(seed=3, n_views=6, n_meshes=5, resolutions=(64, 96, 128),
                                    tri_range=(500, 6000), draws_per_view=(2, 4), tex_size=128, n_textures=2)
    r = api.FrameRenderer(device, frames, visibility=True)
    r.render_batched()
    r.render_batched()   # second execution replays the captured graph
    outs = [r.read(i) for i in range(len(frames))]
    r.destroy()
    for fr, got in zip(frames, outs):
        want = pyoracle.render_oracle(fr)
        assert_bits_equal(got["depth"], want["depth"], "depth")
        assert np.array_equal(got["vis_tri"], want["vis_tri"])
        assert np.array_equal(got["vis_draw"], want["vis_draw"])
        assert_color_close(got["color"], want["color"])


def test_gpu_repeat_is_deterministic(device):
    fr = scenes.small_scene(31, 64, 64, vs=2, ps=3)
    a = render_gpu(device, fr)
    b = render_gpu(device, fr)
    for k in ("color", "depth", "vis_tri", "vis_bary"):
        assert np.array_equal(a[k], b[k])


def test_gpu_status_codes(device):
    ctx = device.immediate
    rt = api.Texture2D(device, 16, 16, api.FORMAT_R8G8B8A8_UNORM)
    ds = api.Texture2D(device, 16, 16, api.FORMAT_D32_FLOAT)
    try:
        with pytest.raises(api.MalevichError) as e:
            ctx.om_set_render_targets(rt, rt)      # depth target of the wrong format
        assert e.value.status == 1
        ctx.om_set_render_targets(None, None)
        with pytest.raises(api.MalevichError) as e:
            ctx.draw_indexed(3)                    # nothing bound
        assert e.value.status == 7
        big = api.Texture2D(device, 32, 32, api.FORMAT_D32_FLOAT)
        with pytest.raises(api.MalevichError):
            ctx.om_set_render_targets(rt, big)     # size mismatch
        big.destroy()
    finally:
        rt.destroy()
        ds.destroy()


def test_destroyed_resources_are_unbound(device):
    """A destroyed texture or buffer no longer counts as bound on any context of its device (the
    next draw reports the missing binding instead of reaching freed memory)."""
    ctx = device.immediate
    dctx = device.create_deferred_context()
    rt = api.Texture2D(device, 16, 16, api.FORMAT_R8G8B8A8_UNORM, bind=api.BIND_RENDER_TARGET)
    ds = api.Texture2D(device, 16, 16, api.FORMAT_D32_FLOAT, bind=api.BIND_DEPTH_STENCIL)
    vb = api.Buffer(device, np.zeros((3, 8), np.float32), bind=api.BIND_VERTEX_BUFFER)
    try:
        for c in (ctx, dctx):
            c.om_set_render_targets(rt, ds)
            c.ia_set_vertex_buffer(vb, 32)
            c.vs_set_shader(scenes.VS_PASSTHROUGH)
            c.ps_set_shader(scenes.PS_PASSTHROUGH)
            c.rs_set_viewport((0.0, 0.0, 16.0, 16.0, 0.0, 1.0))
        rt.destroy()
        rt = None
        for c in (ctx, dctx):
            with pytest.raises(api.MalevichError) as e:
                c.draw(3)
            assert e.value.status == 7 and "render target" in str(e.value)
        vb.destroy()
        vb = None
        rt = api.Texture2D(device, 16, 16, api.FORMAT_R8G8B8A8_UNORM, bind=api.BIND_RENDER_TARGET)
        for c in (ctx, dctx):
            c.om_set_render_targets(rt, ds)
            with pytest.raises(api.MalevichError) as e:
                c.draw(3)
            assert e.value.status == 7 and "vertex buffer" in str(e.value)
    finally:
        for r in (rt, ds, vb):
            if r is not None:
                r.destroy()
        dctx.destroy()


def test_gpu_copy_arguments_are_checked(device):
    """Copies outside a buffer (also where offset + size wraps around 64 bits) and row pitches
    shorter than a row are INVALID_ARG, refused before any copy is issued."""
    ctx, lib = device.immediate, api.load_library()
    buf = api.Buffer(device, byte_width=64)
    tex = api.Texture2D(device, 8, 4, api.FORMAT_R8G8B8A8_UNORM)
    src = np.zeros(64, np.uint8)
    img = np.zeros((4, 8), np.uint32)
    p = src.ctypes.data_as(ctypes.c_void_p)
    q = img.ctypes.data_as(ctypes.c_void_p)
    try:
        for offset, size in ((60, 8), (65, 0), (2 ** 64 - 4, 8)):
            assert lib.mlv_update_buffer(ctx.handle, buf.handle, offset, p, size) == 1, (offset, size)
            assert lib.mlv_update_buffer_async(ctx.handle, buf.handle, offset, p, size) == 1, (offset, size)
        assert lib.mlv_update_buffer(ctx.handle, buf.handle, 56, p, 8) == 0
        assert lib.mlv_update_texture2d(ctx.handle, tex.handle, q, 28) == 1
        assert lib.mlv_update_texture2d_async(ctx.handle, tex.handle, q, 16) == 1
        assert lib.mlv_read_texture2d(ctx.handle, tex.handle, q, 31) == 1
        desc = api.Texture2DDesc(8, 4, api.FORMAT_R8G8B8A8_UNORM, api.BIND_SHADER_RESOURCE)
        h = ctypes.c_void_p()
        assert lib.mlv_create_texture2d(device.handle, ctypes.byref(desc), q, 4, ctypes.byref(h)) == 1
        img[:] = np.arange(32, dtype=np.uint32).reshape(4, 8)
        assert lib.mlv_update_texture2d(ctx.handle, tex.handle, q, 32) == 0
        assert np.array_equal(ctx.read_texture(tex), img)
    finally:
        buf.destroy()
        tex.destroy()


def test_gpu_workspace_overflow_is_regrown_and_rerun():
    """Tiny first buffers: batches overflow, skip their writes, and are re-run after regrowing;
    the image and the statistics come out as if nothing happened."""
    from malevich_gb300 import build
    build.build()
    dev = api.Device(0)
    try:
        dev.immediate.set_tuning(initial_bin_entries=64, initial_clip_fan_slots=1)
        fr = scenes.small_scene(3, 64, 64, n_objects=4, inside=True)
        fr.draws += scenes.small_scene(4, 64, 64, n_objects=3).draws
        got = render_gpu(dev, fr)
        check_against_oracle(got, pyoracle.render_oracle(fr))
    finally:
        dev.destroy()
