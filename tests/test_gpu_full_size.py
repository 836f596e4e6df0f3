"""The benchmark workloads at their full sizes against the oracle: the 1920x1080 scene frame
(1,032,584 input triangles) batched and per draw, views of the 64-view batch, and views of the
differentiable loop's 256-view visibility pass. Depth, ids and barycentrics bit for bit, colour
within +-1 LSB (normalising shaders: at most 0.1% of pixels beyond, see helpers), statistics equal."""
import numpy as np
import pytest

from helpers import assert_bits_equal, assert_color_close, outlier_report
from malevich_gb300 import api, scenes
from oracle import pyoracle

pytestmark = pytest.mark.gpu

STATS = ("vertex_count", "input_triangle_count", "assembled_triangle_count", "active_bin_count",
         "total_triangle_count_in_bins")


@pytest.fixture(scope="module")
def scene_frame():
    fr = scenes.config2_scene(seed=2)
    return fr, pyoracle.render_oracle(fr)


@pytest.mark.parametrize("batched", [True, False])
def test_full_scene_frame(device, scene_frame, batched):
    fr, want = scene_frame
    r = api.FrameRenderer(device, fr, visibility=True)
    ctx = device.immediate
    for _ in range(2 if batched else 1):   # batched: eager, then graph replay
        ctx.reset_stats()
        r.render_batched() if batched else r.render_per_draw()
    got = r.read(0)
    stats = ctx.stats()
    r.destroy()
    assert want["stats"]["input_triangle_count"] == 1032584
    assert_bits_equal(got["depth"], want["depth"], "depth")
    assert np.array_equal(got["vis_tri"], want["vis_tri"])
    assert np.array_equal(got["vis_draw"], want["vis_draw"])
    assert_bits_equal(got["vis_bary"], want["vis_bary"], "barycentrics")
    rep = outlier_report(got["color"], want["color"])
    print("scene frame (%s): %d of %d pixels (%.5f%%) beyond +-1 LSB of the oracle, max diff %d" % (
        "batched" if batched else "per draw", rep["pixels_beyond_1lsb"], fr.width * fr.height,
        100 * rep["fraction"], rep["max_diff"]))
    assert_color_close(got["color"], want["color"], max_outlier_frac=1e-3)
    for k in STATS:
        assert stats[k] == want["stats"][k], k


def test_multiview_batch_views(device):
    frames = scenes.config3_batched(seed=3)
    pick = [0, 17, 40, 63]
    r = api.FrameRenderer(device, frames)
    r.render_batched()
    r.render_batched()
    outs = {i: r.read(i) for i in pick}
    r.destroy()
    for i in pick:
        want = pyoracle.render_oracle(frames[i])
        assert_bits_equal(outs[i]["depth"], want["depth"], "depth of view %d" % i)
        assert_color_close(outs[i]["color"], want["color"])


def test_differentiable_loop_visibility_views(device):
    sc = scenes.diff_scene(seed=5, n_views=256, size=256, tex_size=2048, heightfield_cells=316)
    frames = scenes.diff_frames(sc, shade=False)
    r = api.FrameRenderer(device, frames, primitive_ids=True)
    r.render_batched()
    for i in (0, 255):
        got = r.read(i)
        want = pyoracle.render_oracle(frames[i])
        assert np.array_equal(got["vis_prim"], want["vis_prim"])
        assert_bits_equal(got["depth"], want["depth"], "depth of view %d" % i)
    r.destroy()
