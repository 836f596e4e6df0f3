"""The rasterizer modes the reference lacks, as the oracle defines them: the top-left fill rule and
pixel-centre sampling (MLV_FILL_TOP_LEFT, MLV_SAMPLE_PIXEL_CENTER; the reference's rule and sample
point stay the default). CPU tests check the oracle against coverage worked out by hand; the GPU
tests check the kernels against the oracle in every mode combination."""
import numpy as np
import pytest

from helpers import sort_infos
from malevich_gb300 import api, scenes
from oracle import pyoracle

W = H = 64


def grid_frame(fill_rule=0, sample_center=0, x0=8, y0=8, cells=4, cell=8, cull=scenes.CULL_NONE):
    """cells x cells quads of cell x cell pixels from pixel corner (x0, y0), each split along its
    main diagonal; every vertex sits exactly on a pixel corner (passthrough screen space)."""
    verts = []
    for j in range(cells + 1):
        for i in range(cells + 1):
            x, y = x0 + i * cell, y0 + j * cell
            verts.append([x / W, 1.0 - y / H, 0.5, 1.0, 0.2, 0.6, 0.9, 0.0])
    vb = np.array(verts, np.float32)
    faces = []
    n = cells + 1
    for j in range(cells):
        for i in range(cells):
            a, b, c, d = j * n + i, j * n + i + 1, (j + 1) * n + i, (j + 1) * n + i + 1
            faces += [[a, b, d], [a, d, c]]
    ib = scenes.pad_indices(np.array(faces))
    d = scenes.Draw(scenes.VS_PASSTHROUGH, scenes.PS_PASSTHROUGH, vb, ib, 3 * len(faces),
                    viewport=(0.0, 0.0, float(W), float(H), 0.0, 1.0), cull=cull, depth_func=scenes.DEPTH_LESS,
                    fill_rule=fill_rule, sample_center=sample_center)
    return scenes.Frame(W, H, [d], clear_color=(0.0, 0.0, 0.0, 0.0), clear_depth=1.0)


def triangle_frame(pts, fill_rule=0, sample_center=0):
    vb = np.array([[x / W, 1.0 - y / H, 0.5, 1.0, 1.0, 1.0, 1.0, 0.0] for x, y in pts], np.float32)
    ib = scenes.pad_indices(np.array([[0, 1, 2]]))
    d = scenes.Draw(scenes.VS_PASSTHROUGH, scenes.PS_PASSTHROUGH, vb, ib, 3,
                    viewport=(0.0, 0.0, float(W), float(H), 0.0, 1.0), cull=scenes.CULL_NONE,
                    depth_func=scenes.DEPTH_LESS, fill_rule=fill_rule, sample_center=sample_center)
    return scenes.Frame(W, H, [d], clear_color=(0.0, 0.0, 0.0, 0.0), clear_depth=1.0)


def coverage_count(frame):
    """How many (triangle) coverage tests pass at each pixel, from the oracle's TileInfo masks."""
    cap = pyoracle.render_oracle(frame, capture=True)["captures"][0]
    count = np.zeros((H, W), np.int32)
    tiles_x = (W + 7) // 8
    for b, m in zip(cap["info_bin"], cap["info_mask"]):
        tx, ty = int(b) % tiles_x, int(b) // tiles_x
        for p in range(64):
            if int(m) >> p & 1:
                count[ty * 8 + p // 8, tx * 8 + p % 8] += 1
    return count


def test_top_left_covers_every_sample_of_a_mesh_exactly_once():
    c = coverage_count(grid_frame(fill_rule=1))
    inside = np.zeros((H, W), bool)
    inside[8:40, 8:40] = True               # corners (x, y) with 8 <= x, y < 40
    assert np.all(c[inside] == 1)
    assert np.all(c[~inside] == 0)


def test_inclusive_rule_covers_shared_edges_twice():
    c = coverage_count(grid_frame(fill_rule=0))
    assert np.all(c[8:41, 8:41] >= 1)       # the closed square, right and bottom edges included
    assert np.all(c[:8] == 0) and np.all(c[41:] == 0)
    assert c[12, 12] >= 2                   # on a diagonal shared by two triangles of a quad
    assert c[16, 12] >= 2                   # on a horizontal grid line
    assert c[13, 12] == 1                   # strictly inside one triangle


def test_pixel_centre_sampling_of_a_right_triangle():
    # legs along x and y from (0, 0) to 8 pixels: the corner (x, y) is covered for x + y <= 8
    # (inclusive rule), the centre (x + 1/2, y + 1/2) for x + y <= 7
    pts = [(0, 0), (8, 0), (0, 8)]
    corner = coverage_count(triangle_frame(pts))
    centre = coverage_count(triangle_frame(pts, sample_center=1))
    yy, xx = np.mgrid[0:H, 0:W]
    assert np.array_equal(corner > 0, (xx + yy <= 8))
    assert np.array_equal(centre > 0, (xx + yy <= 7))
    # top-left at the centre: the hypotenuse (interior up-left of it) is neither top nor left, so
    # centres on it (x + y == 7) drop out; the legs are top and left edges
    tl = coverage_count(triangle_frame(pts, fill_rule=1, sample_center=1))
    assert np.array_equal(tl > 0, (xx + yy <= 6))


def test_pixel_centre_barycentrics_are_taken_at_the_centre():
    pts = [(0, 0), (16, 0), (0, 16)]
    a = pyoracle.render_oracle(triangle_frame(pts))
    b = pyoracle.render_oracle(triangle_frame(pts, sample_center=1))
    # quantised barycentrics (E >> 8) * inv_area at (2, 3): corner E1 ~ x, centre ~ x + 1/2
    assert a["vis_bary"][3, 2].tolist() != b["vis_bary"][3, 2].tolist()
    assert np.allclose(b["vis_bary"][3, 2], [2.5 / 16, 3.5 / 16], atol=1.0 / 16) or \
        np.allclose(b["vis_bary"][3, 2], [3.5 / 16, 2.5 / 16], atol=1.0 / 16)


MODES = [(0, 0), (1, 0), (0, 1), (1, 1)]


@pytest.mark.gpu
@pytest.mark.parametrize("fill_rule,sample_center", MODES)
def test_gpu_raster_modes_match_oracle(device, fill_rule, sample_center):
    frames = [grid_frame(fill_rule, sample_center), scenes.small_scene(21, 96, 80, n_objects=3, level=3)]
    for d in frames[1].draws:
        d.fill_rule, d.sample_center = fill_rule, sample_center
    for fr in frames:
        want = pyoracle.render_oracle(fr, capture=True)
        r = api.FrameRenderer(device, fr, visibility=True)
        ctx = device.immediate
        ctx.set_debug_capture(True)
        try:
            r.render_per_draw()
            tile, tri, mask = ctx.tile_infos()
            got = r.read(0)
        finally:
            ctx.set_debug_capture(False)
            r.destroy()
        for key in ("depth", "vis_tri", "vis_bary"):
            assert np.array_equal(got[key].view(np.uint32), want[key].view(np.uint32)), key
        if len(fr.draws) == 1:
            cap = want["captures"][0]
            wt, wtri, wm = sort_infos(cap["info_bin"], cap["info_tri"], cap["info_mask"])
            assert np.array_equal(tile, wt) and np.array_equal(tri, wtri) and np.array_equal(mask, wm)


@pytest.mark.gpu
def test_gpu_rasterizer_state_rejects_unknown_modes(device):
    import ctypes
    lib = api.load_library()
    ctx = device.immediate
    for desc in (api.RasterizerDesc(api.CULL_BACK, 2, 0), api.RasterizerDesc(api.CULL_BACK, 0, 7)):
        assert lib.mlv_rs_set_state(ctx.handle, ctypes.byref(desc)) != 0
    assert lib.mlv_rs_set_state(ctx.handle, ctypes.byref(api.RasterizerDesc(api.CULL_BACK, 1, 1))) == 0
    assert lib.mlv_rs_set_state(ctx.handle, None) == 0
