"""The persistent launch (mlv_tuning.persistent_launch: a batch's binned pipeline as one launch of
resident CTAs, with a grid-wide barrier between its stages) against the kernel-per-stage form and
the oracle: every output bit for bit, colour included (the same bodies shade the same fragments),
and the reference's Stats. Covers the shader pairings, clipping, both depth modes, partial tiles,
the raster modes, tiles shared by 8 warps, the triangle-id, draw-id and barycentric targets (the
rank stage), the null pixel shader with primitive ids, the TileInfo capture, multi-view batches,
eager and graph-replayed command lists and per-draw batches, overflow re-runs, the 1920x1080 scene
frame, and a grid barrier whose bounded wait runs out (MLV_DEBUG_STALL_GRID): MLV_ERROR_TIMEOUT
within seconds, after which the same context renders correctly again."""
import time

import numpy as np
import pytest

from helpers import assert_bits_equal, assert_color_close, sort_infos
from malevich_gb300 import api, scenes
from oracle import pyoracle

pytestmark = pytest.mark.gpu

KEYS = ("color", "depth", "vis_tri", "vis_draw", "vis_bary", "vis_prim")
STATS = ("vertex_count", "input_triangle_count", "assembled_triangle_count", "active_bin_count",
         "total_triangle_count_in_bins")
TIMEOUT = 5


def render(device, frames, persistent, warps_per_tile=1, per_draw=False, visibility=True, **kw):
    """The frames on the binned path, as a kernel per stage (persistent 0) or one launch (1):
    batched (eager, then graph replay) or per draw. Returns the outputs and the last run's Stats."""
    ctx = device.immediate
    base = ctx.tuning()
    ctx.set_tuning(persistent_launch=persistent, warps_per_tile=warps_per_tile, small_draw_triangles=0)
    try:
        r = api.FrameRenderer(device, frames, visibility=visibility, **kw)
        for _ in range(1 if per_draw else 2):
            ctx.reset_stats()
            r.render_per_draw() if per_draw else r.render_batched()
        outs = [r.read(i) for i in range(len(r.frames))]
        st = ctx.stats()
        r.destroy()
    finally:
        ctx.set_tuning(**base)
    return outs, st


def check_same(got, want):
    for k in KEYS:
        if k in want:
            assert np.array_equal(got[k].view(np.uint32), want[k].view(np.uint32)), k


def check_oracle(got, want):
    assert_bits_equal(got["depth"], want["depth"], "depth")
    assert_color_close(got["color"], want["color"])
    if "vis_tri" in got:
        assert np.array_equal(got["vis_tri"], want["vis_tri"]), "triangle ids"
        assert np.array_equal(got["vis_draw"], want["vis_draw"]), "draw ids"
        assert_bits_equal(got["vis_bary"], want["vis_bary"], "barycentrics")


SCENES = {
    "multi_draw_ge": lambda: scenes.small_scene(41, 64, 64, n_objects=5, level=3),
    "multi_draw_less": lambda: scenes.small_scene(42, 64, 64, n_objects=4, native=False),
    "clipped": lambda: scenes.small_scene(43, 72, 56, n_objects=4, inside=True),
    "clipped_less": lambda: scenes.small_scene(44, 72, 56, n_objects=3, inside=True, native=False),
    "partial_tiles": lambda: scenes.small_scene(45, 61, 45, n_objects=3),
    "lighting": lambda: scenes.small_scene(46, 80, 48, vs=scenes.VS_VERTEX_LIGHTING, ps=scenes.PS_ENV_LIGHTING,
                                           n_objects=3),
    "lighting_basic_ps": lambda: scenes.small_scene(47, 64, 64, vs=scenes.VS_VERTEX_LIGHTING, ps=scenes.PS_BASIC,
                                                    n_objects=2, inside=True),
    "single_sphere": lambda: scenes.config1_plain(seed=1, width=320, height=192, tex_size=64, level=4),
}


@pytest.mark.parametrize("name", sorted(SCENES))
@pytest.mark.parametrize("wpt", [1, 8])
def test_persistent_matches_chained_and_oracle(device, name, wpt):
    fr = SCENES[name]()
    want = pyoracle.render_oracle(fr)
    (base,), st_base = render(device, [fr], 0)
    (got,), st = render(device, [fr], 1, warps_per_tile=wpt)
    check_same(got, base)
    check_oracle(got, want)
    for k in STATS:
        assert st[k] == st_base[k] == want["stats"][k], (k, st[k], st_base[k], want["stats"][k])
    # one launch (the clears are folded into its tile stage) against one per stage
    assert st["kernel_launches"] == 1 and st_base["kernel_launches"] >= 6, (st["kernel_launches"],
                                                                          st_base["kernel_launches"])


def test_persistent_per_draw_batches(device):
    # one batch per draw on the immediate context: unfolded clears, each draw's hierarchical-Z
    # snapshot from the draws before it
    fr = scenes.small_scene(48, 64, 64, n_objects=4, inside=True)
    want = pyoracle.render_oracle(fr)
    (base,), _ = render(device, [fr], 0, per_draw=True)
    (got,), st = render(device, [fr], 1, per_draw=True)
    check_same(got, base)
    check_oracle(got, want)
    for k in STATS:
        assert st[k] == want["stats"][k], k


@pytest.mark.parametrize("fill_rule,sample_center", [(1, 0), (0, 1), (1, 1)])
def test_persistent_raster_modes(device, fill_rule, sample_center):
    fr = scenes.small_scene(49, 64, 64, n_objects=4, level=3)
    for d in fr.draws:
        d.fill_rule, d.sample_center = fill_rule, sample_center
    (base,), _ = render(device, [fr], 0)
    (got,), _ = render(device, [fr], 1)
    check_same(got, base)
    check_oracle(got, pyoracle.render_oracle(fr))


def test_persistent_without_visibility_targets(device):
    # no triangle-id target: no rank stage
    fr = scenes.small_scene(50, 64, 64, n_objects=4, inside=True)
    (base,), _ = render(device, [fr], 0, visibility=False)
    (got,), _ = render(device, [fr], 1, visibility=False)
    check_same(got, base)
    check_oracle(got, pyoracle.render_oracle(fr))


def test_persistent_null_pixel_shader_multiview(device):
    sc = scenes.diff_scene(seed=15, n_views=3, size=96, freq=12, tex_size=16)
    frames = scenes.diff_frames(sc, shade=False)
    base, _ = render(device, frames, 0, visibility=False, primitive_ids=True)
    got, _ = render(device, frames, 1, visibility=False, primitive_ids=True)
    for k, f in enumerate(frames):
        want = pyoracle.render_oracle(f)
        assert np.array_equal(got[k]["vis_prim"], want["vis_prim"])
        check_same(got[k], base[k])
        assert_bits_equal(got[k]["depth"], want["depth"], "depth")


@pytest.mark.parametrize("wpt", [1, 8])
def test_persistent_batch_of_views(device, wpt):
    frames = scenes.config3_batched(seed=16, n_views=6, n_meshes=5, resolutions=(64, 96, 128),
                                    tri_range=(300, 4000), draws_per_view=(2, 4), tex_size=32, n_textures=2)
    base, st_base = render(device, frames, 0)
    got, st = render(device, frames, 1, warps_per_tile=wpt)
    want_stats = {k: 0 for k in STATS}
    for k, f in enumerate(frames):
        want = pyoracle.render_oracle(f)
        check_same(got[k], base[k])
        check_oracle(got[k], want)
        for s in STATS:
            want_stats[s] += want["stats"][s]
    for s in STATS:
        assert st[s] == st_base[s] == want_stats[s], s


def test_persistent_tile_infos(device):
    fr = scenes.small_scene(51, 64, 64, n_objects=1, level=4)
    want = pyoracle.render_oracle(fr, capture=True)["captures"][0]
    ctx = device.immediate
    base = ctx.tuning()
    ctx.set_tuning(persistent_launch=1, small_draw_triangles=0)
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


def test_persistent_overflow_is_regrown_and_rerun():
    """Tiny first buffers on a fresh device: the persistent batch overflows (clip fans, then bin
    entries), skips its writes at the next grid barrier, and is re-run after regrowing."""
    dev = api.Device(0)
    try:
        dev.immediate.set_tuning(initial_bin_entries=64, initial_clip_fan_slots=1, persistent_launch=1,
                                 small_draw_triangles=0)
        fr = scenes.small_scene(52, 64, 64, n_objects=4, inside=True)
        fr.draws += scenes.small_scene(53, 64, 64, n_objects=3).draws
        want = pyoracle.render_oracle(fr)
        r = api.FrameRenderer(dev, fr, visibility=True)
        for run in (r.render_per_draw, r.render_batched, r.render_batched):
            dev.immediate.reset_stats()
            run()
            got = r.read(0)
            check_oracle(got, want)
            st = dev.immediate.stats()
            for k in STATS:
                assert st[k] == want["stats"][k], k
        r.destroy()
    finally:
        dev.destroy()


def test_persistent_scene_frame_full_size(device):
    # the 1920x1080 scene frame (1.03M input triangles, 12 draws): bit for bit against the
    # kernel-per-stage form, whose full-size parity with the oracle is tested elsewhere
    fr = scenes.config2_scene(seed=2)
    (base,), st_base = render(device, [fr], 0, visibility=False)
    for wpt in (1, 8):
        (got,), st = render(device, [fr], 1, warps_per_tile=wpt, visibility=False)
        check_same(got, base)
        for k in STATS:
            assert st[k] == st_base[k], k


def test_bounded_grid_barrier_wait_runs_out_and_context_recovers(device):
    fr = scenes.small_scene(54, 256, 192, n_objects=2)
    ctx = device.immediate
    base = ctx.tuning()
    r = api.FrameRenderer(device, fr)
    try:
        ctx.set_tuning(small_draw_triangles=0, persistent_launch=1, debug_flags=api.DEBUG_STALL_GRID)
        t0 = time.perf_counter()
        with pytest.raises(api.MalevichError) as err:
            r.render_per_draw()
            ctx.finish()
        elapsed = time.perf_counter() - t0
        assert err.value.status == TIMEOUT, str(err.value)
        assert "grid barrier" in str(err.value)
        assert elapsed < 60.0, elapsed
        print("the grid barrier's bounded waits gave up after %.2f s" % elapsed)
        # the same context works again: flag off (both launch forms), frame rendered and checked
        want = pyoracle.render_oracle(fr)
        for persistent in (1, 0):
            ctx.set_tuning(**dict(base, persistent_launch=persistent, small_draw_triangles=0))
            r.render_per_draw()
            got = r.read(0)
            assert_bits_equal(got["depth"], want["depth"], "depth after the timeout")
        assert np.count_nonzero(want["depth"] != np.float32(fr.clear_depth)) > 1000
    finally:
        ctx.set_tuning(**base)
        r.destroy()


def test_bounded_lookback_wait_in_the_persistent_launch(device):
    # the bin scan's stall (MLV_DEBUG_STALL_LOOKBACK) inside the persistent launch: its scan blocks
    # give up and publish, and the next grid barrier stops the batch
    fr = scenes.small_scene(55, 1920, 1080, n_objects=2, native=True)
    ctx = device.immediate
    base = ctx.tuning()
    r = api.FrameRenderer(device, fr)
    try:
        ctx.set_tuning(small_draw_triangles=0, persistent_launch=1, debug_flags=api.DEBUG_STALL_LOOKBACK)
        with pytest.raises(api.MalevichError) as err:
            r.render_per_draw()
            ctx.finish()
        assert err.value.status == TIMEOUT, str(err.value)
        ctx.set_tuning(**dict(base, persistent_launch=1, small_draw_triangles=0))
        r.render_per_draw()
        assert_bits_equal(r.read(0)["depth"], pyoracle.render_oracle(fr)["depth"], "depth after the timeout")
    finally:
        ctx.set_tuning(**base)
        r.destroy()


def test_autotune_searches_the_persistent_launch(device):
    # the sweep times the persistent points too; whichever form wins, the image is the same
    from malevich_gb300 import autotune
    fr = scenes.small_scene(56, 64, 64, n_objects=2, level=2)
    (want,), _ = render(device, [fr], 0)
    ctx = device.immediate
    base = ctx.tuning()
    r = api.FrameRenderer(device, fr, visibility=True)
    try:
        ctx.set_tuning(small_draw_triangles=0)
        r.render_batched()
        out = autotune.autotune(device, r, repeats=3, warmup=1, choose_path=False)
        assert sum(1 for p, _ in out["results"] if p["persistent_launch"]) == 8
        assert ctx.tuning()["persistent_launch"] == out["best"]["persistent_launch"]
        r.render_batched()
        r.render_batched()
        check_same(r.read(0), want)
    finally:
        ctx.set_tuning(**base)
        r.destroy()


def test_persistent_launch_is_validated(device):
    ctx = device.immediate
    with pytest.raises(api.MalevichError):
        ctx.set_tuning(persistent_launch=2)
    assert ctx.tuning()["persistent_launch"] == 0
