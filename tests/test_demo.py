"""The headless application loop: PNG round trip, the reference's camera, and (GPU) a few frames of
the synthetic scene through the C ABI, each written as a PNG that matches the oracle's render."""
import numpy as np
import pytest

from malevich_gb300 import demo, scenes
from oracle import pyoracle


def test_png_round_trip(tmp_path):
    rng = np.random.default_rng(3)
    img = rng.integers(0, 256, (7, 11, 4), dtype=np.uint8)
    p = tmp_path / "x.png"
    demo.write_png(p, img)
    assert p.read_bytes()[:8] == b"\x89PNG\r\n\x1a\n"
    assert np.array_equal(demo.read_png(p), img)


def test_reference_camera_looks_down_minus_x_from_its_start():
    clip_from_view, view_from_world = demo.reference_camera(1200, 720)
    # the camera sits at (3.5, 1, 1); view space +z (forward) is world -x at yaw = pitch = 0
    assert np.allclose(view_from_world @ [3.5, 1.0, 1.0, 1.0], [0, 0, 0, 1])
    assert np.allclose(view_from_world @ [2.5, 1.0, 1.0, 1.0], [0, 0, 1, 1])
    assert np.allclose(view_from_world @ [3.5, 1.0, 2.0, 1.0], [0, 1, 0, 1])     # world +z is up
    # reversed-Z infinite: depth = near / z_view
    c = clip_from_view @ [0, 0, 2.0, 1.0]
    assert np.isclose(c[2] / c[3], 0.01 / 2.0)


def test_target_words_become_display_rgb():
    words = np.array([[0x00FF8010]], np.uint32)
    assert demo.target_to_rgba8(words)[0, 0].tolist() == [0xFF, 0x80, 0x10, 255]


@pytest.mark.gpu
def test_demo_frames_match_the_oracle(device, tmp_path):
    objects = demo.synthetic_scene(seed=4)
    paths, stats = demo.run(device, objects, frames=2, width=160, height=96, out_dir=str(tmp_path))
    assert len(paths) == 2 and all(s["assembled_triangle_count"] > 0 for s in stats)
    for k, p in enumerate(paths):
        got = demo.read_png(p)
        want = pyoracle.render_oracle(demo.scene_frame(objects, 160, 96, yaw=k * 0.15))["color"]
        diff = np.abs(got[..., :3].astype(int) - demo.target_to_rgba8(want)[..., :3].astype(int))
        assert diff.max() <= 1 and (diff > 0).mean() < 0.01
