"""The hand-written adjoint on the GPU (through the C ABI, wrapped in a torch.autograd.Function in
diffrender.py) against the FP64 oracle adjoint, on the differentiable configuration: 16 views at
512x512 of a 50,000-triangle sphere with per-vertex colours and a 1024x1024 RGBA32F texture, the
target rendered from attributes perturbed by N(0, 0.05) and screen positions by N(0, 0.002).
Tolerance: 1e-4 relative error (norm of the difference over the norm of the FP64 gradient)."""
import numpy as np
import pytest

from malevich_gb300 import scenes
from oracle import pyoracle

pytestmark = pytest.mark.gpu

REL_TOL = 1e-4


def rel_err(a, b):
    return float(np.linalg.norm((a - b).ravel()) / max(np.linalg.norm(b.ravel()), 1e-30))


@pytest.fixture(scope="module")
def setup(device):
    import torch
    from diffrender import DiffRender, DiffScene, l2_loss, visibility
    sc = scenes.diff_scene(seed=4)
    rng = np.random.default_rng(104)
    col_t = (sc["col"] + 0.05 * rng.standard_normal(sc["col"].shape)).astype(np.float32)
    tex_t = (sc["tex"] + 0.05 * rng.standard_normal(sc["tex"].shape)).astype(np.float32)
    pos_t = (sc["pos"] + 0.002 * rng.standard_normal(sc["pos"].shape)).astype(np.float32)
    prims = visibility(device, sc)
    tprims = visibility(device, sc, pos=pos_t)
    tscene = DiffScene(sc, tprims)
    with torch.no_grad():
        target = DiffRender.apply(torch.from_numpy(col_t).cuda(), torch.from_numpy(tex_t).cuda(),
                                  torch.from_numpy(pos_t).cuda(), tscene)
    dscene = DiffScene(sc, prims)
    return dict(sc=sc, prims=prims, target=target, dscene=dscene, DiffRender=DiffRender, l2_loss=l2_loss)


def test_visibility_matches_oracle_rasteriser(setup):
    sc = setup["sc"]
    frames = scenes.diff_frames(sc)
    for k in (0, 7):
        want = pyoracle.render_oracle(frames[k])["vis_prim"]
        assert np.array_equal(setup["prims"][k], want)


def test_forward_and_adjoint_match_fp64_oracle(setup):
    import torch
    sc, DiffRender = setup["sc"], setup["DiffRender"]
    col = torch.from_numpy(sc["col"]).cuda().requires_grad_()
    tex = torch.from_numpy(sc["tex"]).cuda().requires_grad_()
    pos = torch.from_numpy(sc["pos"]).cuda().requires_grad_()
    image = DiffRender.apply(col, tex, pos, setup["dscene"])
    loss = setup["l2_loss"](image, setup["target"], setup["dscene"])
    loss.backward()
    target = setup["target"].cpu().numpy().astype(np.float64)
    views = [dict(width=sc["width"], height=sc["height"], pos=sc["pos"][k], prim=setup["prims"][k], target=target[k])
             for k in range(sc["pos"].shape[0])]
    model = pyoracle.DiffModel(sc["ib"], sc["col"], sc["uv"], sc["tex"], views)
    # bilinear cells as the GPU's single-precision arithmetic picks them: the position derivative
    # jumps at cell boundaries, so both sides must differentiate inside the same cell
    model.freeze_cells(rule="f32")
    ref_loss, ref_img = model.loss(image=True)
    g_col, g_tex, g_pos = model.grad()
    errs = {"image": rel_err(image.detach().cpu().numpy(), ref_img),
            "loss": abs(loss.item() - ref_loss) / ref_loss,
            "colors": rel_err(col.grad.cpu().numpy(), g_col), "texels": rel_err(tex.grad.cpu().numpy(), g_tex),
            "positions": rel_err(pos.grad.cpu().numpy(), g_pos)}
    print("relative errors vs FP64:", errs)
    assert max(errs.values()) <= REL_TOL, errs


def test_autograd_backward_equals_direct_call_and_is_repeatable(setup):
    import torch
    sc, DiffRender = setup["sc"], setup["DiffRender"]
    grads = []
    for _ in range(2):
        tex = torch.from_numpy(sc["tex"]).cuda().requires_grad_()
        col = torch.from_numpy(sc["col"]).cuda()
        pos = torch.from_numpy(sc["pos"]).cuda()
        setup["l2_loss"](DiffRender.apply(col, tex, pos, setup["dscene"]), setup["target"], setup["dscene"]).backward()
        grads.append(tex.grad.clone())
    # float atomics make the summation order vary; the results agree far inside the tolerance
    assert rel_err(grads[0].cpu().numpy(), grads[1].cpu().numpy().astype(np.float64)) < 1e-6


def test_adam_on_texture_and_colours_reduces_the_loss(setup):
    import torch
    sc, DiffRender = setup["sc"], setup["DiffRender"]
    col = torch.full_like(torch.from_numpy(sc["col"]), 0.5).cuda().requires_grad_()
    tex = torch.full_like(torch.from_numpy(sc["tex"]), 0.5).cuda().requires_grad_()
    pos = torch.from_numpy(sc["pos"]).cuda()
    opt = torch.optim.Adam([col, tex], lr=1e-2)
    losses = []
    for _ in range(20):
        opt.zero_grad()
        loss = setup["l2_loss"](DiffRender.apply(col, tex, pos, setup["dscene"]), setup["target"], setup["dscene"])
        loss.backward()
        opt.step()
        losses.append(loss.item())
    assert losses[-1] < 0.8 * losses[0]
