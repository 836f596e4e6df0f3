"""The FP64 adjoint of the differentiable shading model (oracle/oracle_adjoint.c) against FP64
central finite differences with step 1e-4, under the visibility the oracle's rasteriser produces.

Colours and texels enter the loss quadratically, so central differences are exact up to rounding.
For positions the loss is smooth only inside a bilinear texel cell; the position check holds each
pixel's cell fixed (the derivative of the active piece, which is what the adjoint computes). The
barycentrics are rational in the positions, and on sliver triangles of a couple of pixels the
O(h^2) truncation of a plain central difference at h = 1e-4 reaches 1e-3 relative (it falls as h^2,
as test_position_differences_converge_quadratically shows), so positions are checked against the
Richardson extrapolation of the central differences at h and h/2, whose error is O(h^4)."""
import numpy as np
import pytest

from malevich_gb300 import scenes
from oracle import pyoracle

H = 1e-4
TOL = 1e-4


def make_model(seed=5, n_views=2, size=48, freq=5, tex=24, perturb=True):
    sc = scenes.diff_scene(seed=seed, n_views=n_views, size=size, freq=freq, tex_size=tex)
    frames = scenes.diff_frames(sc)
    prims = [pyoracle.render_oracle(f)["vis_prim"] for f in frames]
    rng = np.random.default_rng(seed + 100)
    # the target: the same mesh with perturbed attributes and screen-space positions
    col_t = sc["col"] + 0.05 * rng.standard_normal(sc["col"].shape)
    tex_t = sc["tex"] + 0.05 * rng.standard_normal(sc["tex"].shape)
    pos_t = sc["pos"] + 0.002 * rng.standard_normal(sc["pos"].shape)
    tframes = scenes.diff_frames(sc, pos=pos_t.astype(np.float32))
    tprims = [pyoracle.render_oracle(f)["vis_prim"] for f in tframes]
    tview = [dict(width=size, height=size, pos=pos_t[k], prim=tprims[k], target=np.zeros((size, size, 3)))
             for k in range(n_views)]
    _, timg = pyoracle.DiffModel(sc["ib"], col_t, sc["uv"], tex_t, tview).loss(image=True)
    views = [dict(width=size, height=size, pos=sc["pos"][k], prim=prims[k], target=timg[k]) for k in range(n_views)]
    return pyoracle.DiffModel(sc["ib"], sc["col"], sc["uv"], sc["tex"], views)


def central_fd(model, arr, idx, h=H):
    old = arr[idx]
    arr[idx] = old + h
    lp = model.loss()
    arr[idx] = old - h
    lm = model.loss()
    arr[idx] = old
    return (lp - lm) / (2 * h)


def richardson_fd(model, arr, idx, h=H):
    return (4.0 * central_fd(model, arr, idx, h / 2) - central_fd(model, arr, idx, h)) / 3.0


def test_visibility_covers_pixels():
    m = make_model()
    covered = sum(int((v["prim"] != 0xFFFFFFFF).sum()) for v in m.views)
    assert covered > 500
    assert m.loss() > 0


@pytest.mark.parametrize("which", ["col", "tex", "pos"])
def test_adjoint_matches_central_differences(which):
    m = make_model()
    if which == "pos":
        m.freeze_cells()
    g_col, g_tex, g_pos = m.grad()
    rng = np.random.default_rng(7)
    if which == "col":
        arr, g = m.col, g_col
    elif which == "tex":
        arr, g = m.tex, g_tex
    else:
        arr, g = m.views[0]["pos"], g_pos[0]
    nz = np.flatnonzero(np.abs(g).ravel() > 0)            # parameters the loss actually depends on
    pick = rng.choice(nz, size=min(32, len(nz)), replace=False)
    errs, ill = [], 0
    for f in pick:
        idx = np.unravel_index(f, arr.shape)
        if which != "pos":
            errs.append(abs(central_fd(m, arr, idx) - g[idx]) / abs(g[idx]))
            continue
        fd = richardson_fd(m, arr, idx)
        # a vertex of a silhouette sliver (near-zero screen area) puts a pole of the barycentrics
        # within a few h of the point; there the step-1e-4 estimates disagree with each other and
        # the comparison is made at h = 1e-5, where the differences have converged
        spread = abs(central_fd(m, arr, idx) - central_fd(m, arr, idx, H / 2)) / abs(g[idx])
        if spread > TOL:
            ill += 1
            fd = richardson_fd(m, arr, idx, H / 10)
        errs.append(abs(fd - g[idx]) / abs(g[idx]))
    assert max(errs) <= TOL, (which, max(errs))
    assert ill <= len(pick) // 4, "too many ill-conditioned points: %d of %d" % (ill, len(pick))


def test_position_differences_converge_quadratically():
    m = make_model()
    m.freeze_cells()
    _, _, g_pos = m.grad()
    arr, g = m.views[0]["pos"], g_pos[0]
    idx = np.unravel_index(int(np.argmax(np.abs(g))), arr.shape)
    e1 = abs(central_fd(m, arr, idx, 1e-3) - g[idx])
    e2 = abs(central_fd(m, arr, idx, 1e-4) - g[idx])
    assert e2 < e1 / 50      # about 100x for O(h^2)


def test_adjoint_is_zero_off_the_visible_set():
    m = make_model()
    g_col, g_tex, g_pos = m.grad()
    used = set(np.unique(np.concatenate([m.ib[np.unique(v["prim"][v["prim"] != 0xFFFFFFFF])].ravel()
                                         for v in m.views])).tolist())
    unused = np.array(sorted(set(range(len(m.col))) - used))
    if len(unused):
        assert np.all(g_col[unused] == 0)


def test_single_precision_cells_agree_with_fp64_cells():
    """The GPU's cell choice (restated in C with the kernels' float operation sequence) differs
    from the FP64 choice only where the texel coordinate lies within rounding of a cell boundary:
    on a tiny fraction of pixels, and then by one cell."""
    m = make_model(n_views=2, size=96, freq=8, tex=256)
    m.freeze_cells("f64")
    c64 = [v["cells"].copy() for v in m.views]
    m.freeze_cells("f32")
    c32 = [v["cells"] for v in m.views]
    covered = sum(int((v["prim"] != 0xFFFFFFFF).sum()) for v in m.views)
    diff = sum(int((a != b).any(axis=-1).sum()) for a, b in zip(c64, c32))
    assert covered > 5000
    assert diff <= max(2, covered // 1000)
    assert max(int(np.abs(a.astype(np.int64) - b).max()) for a, b in zip(c64, c32)) <= 1
