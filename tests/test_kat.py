"""Known-answer and property tests of the oracle's building blocks and of the GPU formulations
that replace the reference's double-precision steps (checked on the CPU in numpy)."""
import ctypes

import numpy as np

from malevich_gb300 import scenes
from oracle import pyoracle


def snap_gpu_formulation(v32):
    """numpy model of the float-only snap the GPU uses for floor(x*16 + 0.5) (main.c:843-848)."""
    v = (v32.astype(np.float32) * np.float32(16.0)).astype(np.float32)
    out = np.empty(v.shape, np.int64)
    small = np.abs(v) < np.float32(8388608.0)
    f = np.floor(v[small]).astype(np.float32)
    out[small] = f.astype(np.int64) + (v[small] >= (f + np.float32(0.5))).astype(np.int64)
    big = ~small
    vb = v[big].astype(np.float64)
    ok = (vb >= -2147483648.0) & (vb < 2147483648.0)
    res = np.full(vb.shape, -2147483648, np.int64)
    res[ok] = vb[ok].astype(np.int64)
    out[big] = res
    return out.astype(np.int32)


def test_snap_float_formulation_matches_double():
    lib = pyoracle.oracle_lib()
    rng = np.random.default_rng(0)
    vals = np.concatenate([
        rng.uniform(-4000, 4000, 20000).astype(np.float32),
        (np.arange(-4096, 4096) / np.float32(32.0)).astype(np.float32),           # exact half-steps
        np.nextafter((np.arange(-2048, 2048) / np.float32(32.0)).astype(np.float32), np.float32(np.inf)),
        np.nextafter((np.arange(-2048, 2048) / np.float32(32.0)).astype(np.float32), np.float32(-np.inf)),
        np.array([0.0, -0.0, 1e-30, -1e-30, 0.03124999, 0.03125, 524288.0, 1e9, -1e9, 3e10], np.float32),
    ])
    want = np.array([lib.orc_snap(float(v)) for v in vals], np.int32)
    got = snap_gpu_formulation(vals)
    assert np.array_equal(got, want)


def test_cvt_rn_is_round_half_even_with_integer_indefinite():
    lib = pyoracle.oracle_lib()
    for x, want in [(0.5, 0), (1.5, 2), (2.5, 2), (-0.5, 0), (-1.5, -2), (254.5, 254), (255.49, 255),
                    (float("nan"), -2 ** 31), (3e9, -2 ** 31), (-3e9, -2 ** 31)]:
        assert lib.orc_cvt_rn(x) == want, x


def test_clear_color_packs_r_low_with_truncation():
    lib = pyoracle.oracle_lib()
    c = (ctypes.c_float * 4)(*scenes.REFERENCE_CLEAR_COLOR)
    v = lib.orc_encode_clear_color(c)
    # 227/255*255 etc. truncate; alpha 0 (main.c:1271, math.h:322-324)
    r, g, b, a = v & 0xFF, (v >> 8) & 0xFF, (v >> 16) & 0xFF, v >> 24
    assert a == 0 and abs(r - 227) <= 1 and abs(g - 223) <= 1 and abs(b - 216) <= 1


def _one_triangle_frame(pts, w=32, h=32, cull=scenes.CULL_BACK, depth_func=scenes.DEPTH_GREATER_EQUAL):
    """passthrough_vs input: position in [0,1] screen space (x*2-1 in the VS), colour."""
    vb = np.zeros((3, 8), np.float32)
    for i, (x, y, z) in enumerate(pts):
        vb[i] = [x, y, z, 1.0, 0.25 * (i + 1), 0.5, 0.75, 0.0]
    ib = np.array([0, 1, 2, 0, 0, 0, 0, 0], np.uint32)
    d = scenes.Draw(scenes.VS_PASSTHROUGH, scenes.PS_PASSTHROUGH, vb, ib, 8, viewport=(0, 0, w, h, 0, 1),
                    cull=cull, depth_func=depth_func)
    return scenes.Frame(w, h, [d], clear_depth=0.0 if depth_func == scenes.DEPTH_GREATER_EQUAL else 1.0)


def test_shared_edge_is_covered_by_both_triangles():
    # the reference's coverage test is (E0|E1|E2) > 0: edges are inclusive (main.c:1027-1028)
    a = _one_triangle_frame([(0.1, 0.1, 0.5), (0.1, 0.9, 0.5), (0.9, 0.9, 0.5)], cull=scenes.CULL_NONE)
    b = _one_triangle_frame([(0.1, 0.1, 0.5), (0.9, 0.9, 0.5), (0.9, 0.1, 0.5)], cull=scenes.CULL_NONE)
    ma = pyoracle.render_oracle(a, capture=True)["vis_tri"] != 0xFFFFFFFF
    mb = pyoracle.render_oracle(b, capture=True)["vis_tri"] != 0xFFFFFFFF
    assert ma.any() and mb.any()
    assert (ma & mb).sum() > 0, "pixels on the shared diagonal belong to both triangles"


def test_winding_culling_modes():
    ccw = [(0.1, 0.1, 0.5), (0.1, 0.9, 0.5), (0.9, 0.9, 0.5)]
    cw = [ccw[0], ccw[2], ccw[1]]
    cov = lambda pts, cull: (pyoracle.render_oracle(_one_triangle_frame(pts, cull=cull))["vis_tri"] != 0xFFFFFFFF).sum()
    kept_back = [cov(p, scenes.CULL_BACK) for p in (ccw, cw)]
    assert sorted(kept_back)[0] == 0 and sorted(kept_back)[1] > 0, "back-face culling keeps exactly one winding"
    assert cov(ccw, scenes.CULL_NONE) > 0 and cov(cw, scenes.CULL_NONE) > 0
    kept_front = [cov(p, scenes.CULL_FRONT) for p in (ccw, cw)]
    assert (kept_front[0] > 0) != (kept_back[0] > 0)


def test_zero_area_triangle_is_assembled_but_covers_nothing():
    fr = _one_triangle_frame([(0.5, 0.5, 0.5)] * 3)
    o = pyoracle.render_oracle(fr, capture=True)
    assert o["stats"]["assembled_triangle_count"] >= 1
    assert (o["vis_tri"] == 0xFFFFFFFF).all()


def test_w_zero_vertex_rejects_triangle():
    fr = _one_triangle_frame([(0.1, 0.1, 0.5), (0.1, 0.9, 0.5), (0.9, 0.9, 0.5)], cull=scenes.CULL_NONE)
    fr.draws[0].vb[1, 3] = 0.0
    o = pyoracle.render_oracle(fr)
    # triangle 0 rejected (main.c:759-761); the padding triangle still assembles
    assert (o["vis_tri"] != 0).all()


def test_icosphere_and_config_sizes():
    v, f = scenes.icosphere(5)
    assert len(v) == 10242 and len(f) == 20480
    fr = scenes.config1_plain(seed=1)
    assert fr.draws[0].index_count == 61440 and fr.width == 1280 and fr.height == 720
    assert fr.draws[0].ps_tex.width == 1024
