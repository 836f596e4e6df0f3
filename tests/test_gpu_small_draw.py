"""The small-draw path (one draw of few triangles: three kernels, no binning) against the oracle and
against the binned path on the same inputs: depth bit for bit, colour within +-1 LSB of the oracle
and bit for bit against the binned path, the reference's Stats equal. Covers every shader pairing,
clipping (clip fans go through the kernel's queue), both depth modes, the cull modes, the fill rule
and sample position, partial edge tiles, the null pixel shader, the primitive-id, draw-id and
barycentric targets, folded clears (command lists) and unfolded ones (per draw, where each draw's
hierarchical-Z snapshot comes from the draws before it), full-screen triangles (queued chunks), the
queue's overflow and re-run, and the 1280x720 single draw at full size."""
import numpy as np
import pytest

from helpers import assert_bits_equal, assert_color_close
from malevich_gb300 import api, scenes
from oracle import pyoracle

pytestmark = pytest.mark.gpu

STATS = ("vertex_count", "input_triangle_count", "assembled_triangle_count", "active_bin_count",
         "total_triangle_count_in_bins")


def render(device, frame, small, batched=False, prim=False):
    """Renders with the small-draw path allowed up to `small` triangles (0: always binned)."""
    ctx = device.immediate
    base = ctx.tuning()
    ctx.set_tuning(small_draw_triangles=small)
    try:
        r = api.FrameRenderer(device, frame, primitive_ids=prim)
        ctx.reset_stats()
        for _ in range(2 if batched else 1):   # batched: eager, then graph replay
            ctx.reset_stats()
            r.render_batched() if batched else r.render_per_draw()
        out = r.read(0)
        out["stats"] = ctx.stats()
        r.destroy()
    finally:
        ctx.set_tuning(**base)
    return out


def check(got, want, exact_colour=False):
    assert_bits_equal(got["depth"], want["depth"], "depth")
    if exact_colour:
        assert np.array_equal(got["color"], want["color"]), "colour differs"
    else:
        assert_color_close(got["color"], want["color"])
    if "vis_prim" in got and "vis_prim" in want:
        assert np.array_equal(got["vis_prim"], want["vis_prim"]), "primitive ids differ"
    for k in STATS:
        assert got["stats"][k] == want["stats"][k], (k, got["stats"][k], want["stats"][k])


def one_draw_frames(frame):
    """Each draw of a frame as a frame of its own (a single-draw batch)."""
    return [scenes.Frame(frame.width, frame.height, [d], clear_color=frame.clear_color, clear_depth=frame.clear_depth)
            for d in frame.draws]


CASES = []
for seed in range(2):
    for vs, ps in [(1, 1), (2, 3), (2, 2), (1, 3)]:
        for inside in (False, True):
            CASES.append((seed, vs, ps, inside, True))
    CASES.append((seed, 1, 1, False, False))
    CASES.append((seed, 1, 3, True, False))


@pytest.mark.parametrize("seed,vs,ps,inside,native", CASES)
@pytest.mark.parametrize("batched", [False, True])
def test_small_draw_matches_oracle_and_binned(device, seed, vs, ps, inside, native, batched):
    fr = scenes.small_scene(2000 + seed, 72, 56, vs=vs, ps=ps, inside=inside, native=native, n_objects=1)
    got = render(device, fr, 1 << 20, batched=batched, prim=True)
    check(got, pyoracle.render_oracle(fr))
    check(got, render(device, fr, 0, batched=batched, prim=True), exact_colour=True)


def test_small_draw_per_draw_sequence(device):
    # several single-draw batches into one target: each draw's depth test and hierarchical-Z
    # snapshot come from the draws before it (unfolded clears: the per-draw path)
    for native in (True, False):
        fr = scenes.small_scene(2100, 96, 64, n_objects=5, native=native, inside=False)
        got = render(device, fr, 1 << 20)
        check(got, pyoracle.render_oracle(fr))
        check(got, render(device, fr, 0), exact_colour=True)


@pytest.mark.parametrize("w,h", [(1, 1), (13, 77), (60, 44), (8, 8)])
def test_small_draw_partial_tiles(device, w, h):
    fr = scenes.small_scene(2200, w, h, n_objects=2)
    got = render(device, fr, 1 << 20, prim=True)
    check(got, pyoracle.render_oracle(fr))


@pytest.mark.parametrize("cull", [scenes.CULL_NONE, scenes.CULL_FRONT, scenes.CULL_BACK])
@pytest.mark.parametrize("fill_rule,center", [(0, 0), (1, 0), (0, 1), (1, 1)])
def test_small_draw_raster_modes(device, cull, fill_rule, center):
    fr = scenes.small_scene(2300, 80, 64, n_objects=1, inside=True)
    for d in fr.draws:
        d.cull, d.fill_rule, d.sample_center = cull, fill_rule, center
    got = render(device, fr, 1 << 20, prim=True)
    check(got, pyoracle.render_oracle(fr))
    check(got, render(device, fr, 0, prim=True), exact_colour=True)


def test_small_draw_null_pixel_shader(device):
    fr = scenes.small_scene(2400, 80, 64, n_objects=1, inside=True)
    for d in fr.draws:
        d.ps = scenes.PS_NONE
    for batched in (False, True):
        got = render(device, fr, 1 << 20, batched=batched, prim=True)
        check(got, pyoracle.render_oracle(fr), exact_colour=True)


def test_small_draw_visibility_targets(device):
    # draw ids and barycentrics (the triangle-id target keeps the binned path: it needs the ranks)
    fr = scenes.small_scene(2500, 64, 48, n_objects=1)
    ctx = device.immediate
    outs = []
    for small in (1 << 20, 0):
        base = ctx.tuning()
        ctx.set_tuning(small_draw_triangles=small)
        r = api.FrameRenderer(device, fr)
        rt, ds, _ = r.targets[0]
        vd = api.Texture2D(device, fr.width, fr.height, api.FORMAT_R32_UINT, bind=api.BIND_UNORDERED_ACCESS)
        vb = api.Texture2D(device, fr.width, fr.height, api.FORMAT_R32G32_FLOAT, bind=api.BIND_UNORDERED_ACCESS)
        ctx.clear_u32(vd, 0xFFFFFFFF)
        ctx.clear_u32(vb, 0)
        ctx.clear_render_target(rt, fr.clear_color)
        ctx.clear_depth(ds, fr.clear_depth)
        ctx.om_set_render_targets(rt, ds)
        ctx.om_set_visibility_targets(None, vd, vb)
        ctx.om_set_primitive_id_target(None)
        d = fr.draws[0]
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
        outs.append((ctx.read_texture(rt), ctx.read_texture(ds), ctx.read_texture(vd), ctx.read_texture(vb)))
        ctx.om_set_visibility_targets(None, None, None)
        vd.destroy()
        vb.destroy()
        r.destroy()
        ctx.set_tuning(**base)
    want = pyoracle.render_oracle(fr)
    assert_bits_equal(outs[0][1], want["depth"], "depth")
    assert np.array_equal(outs[0][2], want["vis_draw"]), "draw ids differ"
    assert_bits_equal(outs[0][3], want["vis_bary"], "barycentrics")
    for a, b in zip(outs[0], outs[1]):
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32))


def _full_screen(n_tris, size, depth_func=scenes.DEPTH_GREATER_EQUAL):
    corners = [((0.0, 0.0), (1.0, 0.0), (0.0, 1.0)), ((1.0, 0.0), (1.0, 1.0), (0.0, 1.0)),
               ((0.1, 0.9), (0.95, 0.2), (0.5, 0.05)), ((0.0, 0.0), (1.0, 1.0), (0.0, 1.0))]
    vb = []
    for t in range(n_tris):
        z = 0.2 + 0.6 * ((t * 7) % n_tris) / n_tris
        for (x, y) in corners[t % len(corners)]:
            vb.append([x, y, z, 1.0, 0.2 + 0.05 * (t % 10), 0.5, 0.7, 0.0])
    vb = np.asarray(vb, np.float32)
    vp = (0.0, 0.0, float(size), float(size), 0.0, 1.0)
    d = scenes.Draw(scenes.VS_PASSTHROUGH, scenes.PS_PASSTHROUGH, vb, np.arange(len(vb), dtype=np.uint32), len(vb),
                    viewport=vp, cull=scenes.CULL_NONE, depth_func=depth_func)
    cd = 1.0 if depth_func == scenes.DEPTH_LESS else 0.0
    return scenes.Frame(size, size, [d], clear_color=(0.25, 0.5, 0.75, 1.0), clear_depth=cd)


@pytest.mark.parametrize("depth_func", [scenes.DEPTH_GREATER_EQUAL, scenes.DEPTH_LESS])
def test_small_draw_full_screen_triangles(device, depth_func):
    # triangles over the whole target go through the queue in chunks
    fr = _full_screen(6, 256, depth_func)
    for batched in (False, True):
        got = render(device, fr, 1 << 20, batched=batched, prim=True)
        check(got, pyoracle.render_oracle(fr), exact_colour=True)


def test_small_draw_queue_overflow_reruns(device):
    # more queued chunks than the first queue holds (16,384 entries): the batch is detected on the
    # device, regrown and re-run at the next synchronisation, with the same result
    fr = _full_screen(12, 1024)
    got = render(device, fr, 1 << 20)
    check(got, render(device, fr, 0), exact_colour=True)


@pytest.mark.parametrize("native", [False, True])
def test_small_draw_single_draw_full_size(device, native):
    fr = scenes.config1_plain(seed=1, native=native)
    want = pyoracle.render_oracle(fr)
    for batched in (False, True):
        got = render(device, fr, 1 << 20, batched=batched, prim=True)
        check(got, want)
    assert want["stats"]["assembled_triangle_count"] > 5000


def render_views(device, frames, small, prim=False):
    """All views in one command list (one draw each), read back view by view."""
    ctx = device.immediate
    base = ctx.tuning()
    ctx.set_tuning(small_draw_triangles=small)
    try:
        r = api.FrameRenderer(device, frames, primitive_ids=prim)
        for _ in range(2):   # eager, then graph replay
            ctx.reset_stats()
            r.render_batched()
        outs = [r.read(i) for i in range(len(frames))]
        stats = ctx.stats()
        r.destroy()
    finally:
        ctx.set_tuning(**base)
    return outs, stats


def test_small_draw_multi_view_batch(device):
    # views of different sizes and depth modes, one draw each, in one batch
    sizes = [(64, 48), (40, 72), (96, 96), (17, 33), (80, 64)]
    frames = [scenes.small_scene(2700 + k, w, h, n_objects=1, native=(k % 2 == 0), inside=(k % 3 == 0),
                                 vs=(1, 2)[k % 2], ps=(1, 3)[k % 2]) for k, (w, h) in enumerate(sizes)]
    got, st = render_views(device, frames, 1 << 20, prim=True)
    ref, st_ref = render_views(device, frames, 0, prim=True)
    want_stats = {k: 0 for k in STATS}
    for fr, g, b in zip(frames, got, ref):
        want = pyoracle.render_oracle(fr)
        assert_bits_equal(g["depth"], want["depth"], "depth")
        assert_color_close(g["color"], want["color"])
        assert np.array_equal(g["vis_prim"], want["vis_prim"])
        assert np.array_equal(g["color"], b["color"])
        assert np.array_equal(g["depth"].view(np.uint32), b["depth"].view(np.uint32))
        for k in STATS:
            want_stats[k] += want["stats"][k]
    for k in STATS:
        assert st[k] == want_stats[k] == st_ref[k], k


def test_small_draw_visibility_pass_keys_only(device):
    # the differentiable loop's visibility pass in small: many views of one mesh, the null pixel
    # shader and primitive-id targets only (the resolve reads no records)
    sc = scenes.diff_scene(seed=9, n_views=6, size=64, freq=12, tex_size=64)
    frames = scenes.diff_frames(sc, shade=False)
    got, st = render_views(device, frames, 1 << 20, prim=True)
    ref, st_ref = render_views(device, frames, 0, prim=True)
    for fr, g, b in zip(frames, got, ref):
        want = pyoracle.render_oracle(fr)
        assert np.array_equal(g["vis_prim"], want["vis_prim"])
        assert_bits_equal(g["depth"], want["depth"], "depth")
        assert np.array_equal(g["color"], b["color"])
    for k in STATS:
        assert st[k] == st_ref[k], k
