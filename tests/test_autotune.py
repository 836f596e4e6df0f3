"""The autotuner's search (CPU, with a fake timer) and, on the GPU, that tuning changes only the
speed: the batched outputs after autotuning equal the default launch shapes' bit for bit."""
import numpy as np
import pytest

from malevich_gb300 import autotune, scenes


def test_candidates_cover_the_space_in_order():
    space = {"b": (1, 2), "a": (3, 4, 5)}
    pts = autotune.candidates(space)
    assert len(pts) == 6
    assert pts[0] == {"a": 3, "b": 1} and pts[-1] == {"a": 5, "b": 2}
    # several warps per tile make the warps-per-CTA knob moot: (3 + 3) tile shapes; the persistent
    # launch has fixed shapes but for warps per tile (1 or all 8) and the big-triangle threshold
    assert len(autotune.candidates()) == (3 + 3) * 3 * 4 + 2 * 4
    pts = autotune.candidates({"tile_warps_per_block": (2, 8), "warps_per_tile": (1, 4)})
    assert pts == [{"tile_warps_per_block": 2, "warps_per_tile": 1}, {"tile_warps_per_block": 2, "warps_per_tile": 4},
                   {"tile_warps_per_block": 8, "warps_per_tile": 1}]


def test_persistent_points_take_its_fixed_shapes():
    pts = [p for p in autotune.candidates() if p["persistent_launch"]]
    assert len(pts) == 8
    assert all(p["tile_warps_per_block"] == 8 and p["geometry_block"] == 256 for p in pts)
    assert sorted({p["warps_per_tile"] for p in pts}) == [1, 8]
    assert sorted({p["big_triangle_tiles"] for p in pts}) == [4, 8, 16, 32]
    # without the knobs it fixes, only warps per tile is filtered
    pts = autotune.candidates({"persistent_launch": (0, 1), "warps_per_tile": (1, 2, 4)})
    assert pts == [{"persistent_launch": 0, "warps_per_tile": 1}, {"persistent_launch": 0, "warps_per_tile": 2},
                   {"persistent_launch": 0, "warps_per_tile": 4}, {"persistent_launch": 1, "warps_per_tile": 1},
                   {"persistent_launch": 1, "warps_per_tile": 4}]


def test_autotune_picks_the_persistent_launch_when_it_is_fastest():
    dev = _FakeDevice()
    cost = lambda: (1.0 if dev.immediate.t["persistent_launch"] else 2.0) + dev.immediate.t["big_triangle_tiles"] * 0.01
    out = autotune.autotune(dev, _FakeRenderer(), time_fn=lambda fn: (fn(), cost())[1])
    assert out["best"]["persistent_launch"] == 1 and out["best"]["big_triangle_tiles"] == 4
    assert dev.immediate.t["persistent_launch"] == 1 and dev.immediate.t["tile_warps_per_block"] == 8


def test_the_path_choice_counts_launches_of_the_chained_form():
    # a context left on the persistent launch runs 1 binned launch a batch: the path choice must
    # compare the chained form's 6 with the small-draw path's 3, and keep the context's form after
    class _Ctx(_FakeCtx):
        def reset_stats(self):
            pass

        def stats(self):
            if self.t.get("small_draw_triangles"):
                return {"kernel_launches": 3}
            return {"kernel_launches": 1 if self.t.get("persistent_launch") else 6}

    dev = _FakeDevice()
    dev.immediate = _Ctx()
    dev.immediate.t["persistent_launch"] = 1
    cost = lambda: 1.0 if dev.immediate.t.get("small_draw_triangles") else 2.0
    out = autotune.autotune(dev, _FakeRenderer(), time_fn=lambda fn: (fn(), cost())[1])
    assert out["results"] == [] and out["best"] == {"small_draw_triangles": autotune.PATHS[1]}
    assert dev.immediate.t["persistent_launch"] == 1


def test_pick_takes_the_fastest_and_keeps_the_first_tie():
    res = [({"x": 1}, 3.0), ({"x": 2}, 1.5), ({"x": 3}, 1.5), ({"x": 4}, 2.0)]
    assert autotune.pick(res) == ({"x": 2}, 1.5)


class _FakeCtx:
    def __init__(self):
        self.t = {"tile_warps_per_block": 4, "warps_per_tile": 1, "geometry_block": 256, "big_triangle_tiles": 16,
                  "small_draw_triangles": 0xFFFFFFFF, "persistent_launch": 0}
        self.history = []

    def tuning(self):
        return dict(self.t)

    def set_tuning(self, **kw):
        self.t.update(kw)
        self.history.append(dict(self.t))


class _FakeDevice:
    def __init__(self):
        self.immediate = _FakeCtx()


class _FakeRenderer:
    def render_batched(self):
        pass


def test_autotune_sets_the_fastest_point():
    dev = _FakeDevice()
    cost = lambda: dev.immediate.t["tile_warps_per_block"] * 10 + abs(dev.immediate.t["geometry_block"] - 128) + \
        dev.immediate.t["big_triangle_tiles"] * 0.1
    out = autotune.autotune(dev, _FakeRenderer(), time_fn=lambda fn: (fn(), cost())[1])
    # a context without launch statistics cannot tell whether the small-draw path applies: its
    # path setting stays, and the sweep runs
    assert out["best"] == {"big_triangle_tiles": 4, "geometry_block": 128, "tile_warps_per_block": 2,
                           "warps_per_tile": 1, "persistent_launch": 0, "small_draw_triangles": 0xFFFFFFFF}
    assert dev.immediate.t == out["best"]
    assert len(out["results"]) == 80 and len(out["path"]) == 2


def test_autotune_skips_the_sweep_when_the_small_draw_path_wins():
    class _Ctx(_FakeCtx):
        def reset_stats(self):
            self.launches = 0

        def stats(self):
            return {"batch_count": 1, "kernel_launches": 3 if self.t.get("small_draw_triangles") else 4}

    dev = _FakeDevice()
    dev.immediate = _Ctx()
    cost = lambda: 1.0 if dev.immediate.t.get("small_draw_triangles") else 2.0
    out = autotune.autotune(dev, _FakeRenderer(), time_fn=lambda fn: (fn(), cost())[1])
    assert out["best"] == {"small_draw_triangles": autotune.PATHS[1]} and out["results"] == []
    assert dev.immediate.t["small_draw_triangles"] == autotune.PATHS[1]
    assert dev.immediate.t["tile_warps_per_block"] == 4   # not swept


def test_autotune_restores_the_tuning_on_error():
    dev = _FakeDevice()
    calls = []

    def bad_timer(fn):
        calls.append(1)
        if len(calls) == 3:
            raise RuntimeError("timer failed")
        return 1.0

    with pytest.raises(RuntimeError):
        autotune.autotune(dev, _FakeRenderer(), time_fn=bad_timer)
    assert dev.immediate.t == {"tile_warps_per_block": 4, "warps_per_tile": 1, "geometry_block": 256,
                               "big_triangle_tiles": 16, "small_draw_triangles": 0xFFFFFFFF, "persistent_launch": 0}


@pytest.mark.gpu
def test_autotuned_batched_output_equals_default(device):
    from malevich_gb300 import api
    frames = scenes.config3_batched(seed=11, n_views=6, n_meshes=5, resolutions=(128, 192), tri_range=(500, 8000),
                                    draws_per_view=(2, 4), tex_size=64, n_textures=2)
    ctx = device.immediate
    base = ctx.tuning()
    r = api.FrameRenderer(device, frames, visibility=True)
    r.render_batched()
    want = [r.read(i) for i in range(len(frames))]
    out = autotune.autotune(device, r, space={"tile_warps_per_block": (2, 8), "geometry_block": (128, 512),
                                              "big_triangle_tiles": (1, 32)}, repeats=2, warmup=1)
    assert out["best"] == {k: ctx.tuning()[k] for k in out["best"]}
    r.render_batched()
    for i in range(len(frames)):
        got = r.read(i)
        for key in ("color", "depth", "vis_tri", "vis_draw", "vis_bary"):
            assert np.array_equal(got[key].view(np.uint32), want[i][key].view(np.uint32)), (i, key)
    r.destroy()
    ctx.set_tuning(**base)


@pytest.mark.gpu
def test_autotune_picks_a_path_for_a_single_draw_and_keeps_the_output(device):
    from malevich_gb300 import api
    frame = scenes.config1_plain(seed=2, width=320, height=192, tex_size=64, level=4)
    ctx = device.immediate
    base = ctx.tuning()
    r = api.FrameRenderer(device, frame)   # no triangle-id targets: the small-draw path applies
    try:
        r.render_batched()
        want = r.read(0)
        out = autotune.autotune(device, r, repeats=2, warmup=1)
        assert [p["small_draw_triangles"] for p, _ in out["path"]] == list(autotune.PATHS)
        assert ctx.tuning()["small_draw_triangles"] == out["best"]["small_draw_triangles"]
        # no sweep when the small-draw path won; a sweep when the binned path did
        if out["best"]["small_draw_triangles"] == 0:
            assert out["results"]
        else:
            assert out["results"] == []
        r.render_batched()
        got = r.read(0)
        for key in ("color", "depth"):
            assert np.array_equal(got[key].view(np.uint32), want[key].view(np.uint32)), key
    finally:
        r.destroy()
        ctx.set_tuning(**base)


def test_autotune_keeps_the_path_setting_when_the_small_draw_path_does_not_apply():
    class _Ctx(_FakeCtx):
        def reset_stats(self):
            pass

        def stats(self):
            return {"batch_count": 1, "kernel_launches": 6}   # the same kernels either way

    dev = _FakeDevice()
    dev.immediate = _Ctx()
    cost = lambda: 1.0 if not dev.immediate.t.get("small_draw_triangles") else 2.0   # noise favouring 0
    out = autotune.autotune(dev, _FakeRenderer(), space={"geometry_block": (128, 256)},
                            time_fn=lambda fn: (fn(), cost())[1])
    assert dev.immediate.t["small_draw_triangles"] == 0xFFFFFFFF and len(out["results"]) == 2


@pytest.mark.gpu
def test_autotune_sweeps_when_the_small_draw_path_does_not_apply(device):
    from malevich_gb300 import api
    frame = scenes.config1_plain(seed=3, width=160, height=96, tex_size=32, level=3)
    ctx = device.immediate
    base = ctx.tuning()
    r = api.FrameRenderer(device, frame, visibility=True)   # triangle ids: binned path only
    try:
        r.render_batched()
        out = autotune.autotune(device, r, space={"tile_warps_per_block": (2, 4)}, repeats=1, warmup=1)
        assert len(out["results"]) == 2
    finally:
        r.destroy()
        ctx.set_tuning(**base)


@pytest.mark.gpu
@pytest.mark.parametrize("first,then", [(autotune.PATHS[1], 0), (0, autotune.PATHS[1])])
def test_a_tuning_change_that_moves_the_path_sizes_its_buffers_before_the_capture(first, then):
    """A fresh context that has run a command list on one path only: a tuning change moves the list
    to the other path, whose buffers (the binned path's job and clip lists, the small-draw path's
    keys) did not exist yet, and the graph captured for it must see them allocated."""
    from malevich_gb300 import api
    dev = api.Device(0)
    try:
        ctx = dev.immediate
        ctx.set_tuning(small_draw_triangles=first)
        frame = scenes.config1_plain(seed=4, width=192, height=128, tex_size=32, level=3)
        r = api.FrameRenderer(dev, frame)
        r.render_batched()   # eager: sizes the workspace for the first path only
        r.render_batched()   # graph
        want = r.read(0)
        ctx.set_tuning(small_draw_triangles=then)
        r.render_batched()   # captured again, on the other path
        r.render_batched()
        got = r.read(0)
        for key in ("color", "depth"):
            assert np.array_equal(got[key].view(np.uint32), want[key].view(np.uint32)), key
        r.destroy()
    finally:
        dev.destroy()
