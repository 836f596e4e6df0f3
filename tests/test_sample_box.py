"""The tile kernel walks each triangle's pixel box shrunk to the samples it can cover (setup's
sample box) instead of the reference's box (main.c:888-904). This checks the argument on the CPU
with the same integer arithmetic: for random snapped triangles (tiny, sliver, degenerate, up to
1024 pixels wide) under both fill rules and both sample points, every sample the reference's
coverage test accepts inside the reference's box lies inside the sample box, and the 6-bit
shrinks give the reference's box back exactly."""
import numpy as np
import pytest

W = H = 4096   # viewport; boxes are clamped to it as setup does
M32 = np.int64(0xFFFFFFFF)


def wrap32(v):
    v = np.asarray(v, dtype=np.int64) & M32
    return np.where(v >= 2 ** 31, v - 2 ** 32, v)


def edges(x, y, area):
    """set_edge (main.c:563-575) for the three edges, wrapping int32: (a, b, c) per edge."""
    out = []
    for (i, j) in ((1, 2), (2, 0), (0, 1)):
        a = wrap32(y[i] - y[j])
        b = wrap32(x[j] - x[i])
        if area < 0:
            a, b = wrap32(-a), wrap32(-b)
        c = wrap32(wrap32(-a * x[i]) - wrap32(b * y[i]))
        out.append((int(a), int(b), int(c)))
    return out


def boxes(x, y, center):
    """Setup's reference box and sample box, and the shrinks (the kernel's formulas)."""
    mnx, mny = min(x) >> 4, min(y) >> 4
    mxx, mxy = max(x) >> 4, max(y) >> 4
    mnx, mny = min(max(mnx, 0), W - 1), min(max(mny, 0), H - 1)
    mxx, mxy = max(min(mxx + 1, W - 1), -8), max(min(mxy + 1, H - 1), -8)
    dlx = dly = dhx = dhy = 0
    if max(x) - min(x) <= 16384 and max(y) - min(y) <= 16384:
        off = 8 if center else 0
        dlx = min(max(((min(x) - off + 15) >> 4) - mnx, 0), 1)
        dly = min(max(((min(y) - off + 15) >> 4) - mny, 0), 1)
        dhx = min(max(mxx - ((max(x) - off) >> 4), 0), 3)
        dhy = min(max(mxy - ((max(y) - off) >> 4), 0), 3)
    ref = (mnx, mny, mxx, mxy)
    tight = (mnx + dlx, mny + dly, mxx - dhx, mxy - dhy)
    return ref, tight, (dlx, dly, dhx, dhy)


def covered_samples(x, y, ref, center, top_left):
    area = int(wrap32((x[1] - x[0]) * (y[2] - y[0]) - (x[2] - x[0]) * (y[1] - y[0])))
    e = edges(x, y, area)
    if center:   # E at (x + 1/2, y + 1/2): c += 8 (a + b)
        e = [(a, b, int(wrap32(c + 8 * (a + b)))) for a, b, c in e]
    xs = np.arange(ref[0], ref[2] + 1, dtype=np.int64)
    ys = np.arange(ref[1], ref[3] + 1, dtype=np.int64)
    if len(xs) == 0 or len(ys) == 0:
        return np.zeros((0, 2), np.int64)
    X, Y = np.meshgrid(xs, ys)
    E = [wrap32(wrap32(wrap32(a * X) * 16) + wrap32(wrap32(b * Y) * 16) + c) for a, b, c in e]
    if top_left:
        bias = [0 if (a > 0 or (a == 0 and b > 0)) else 1 for a, b, _ in e]
        cov = (E[0] >= bias[0]) & (E[1] >= bias[1]) & (E[2] >= bias[2])
    else:
        cov = ((E[0] | E[1] | E[2]) > 0)   # main.c:1028: none negative, not all zero
    return np.stack([X[cov], Y[cov]], axis=1)


def random_triangles(rng, n):
    out = []
    for k in range(n):
        kind = k % 5
        cx, cy = rng.integers(0, (W - 64) * 16, size=2)
        if kind == 0:      # sub-pixel
            pts = rng.integers(-12, 13, size=(3, 2))
        elif kind == 1:    # a few pixels
            pts = rng.integers(-80, 81, size=(3, 2))
        elif kind == 2:    # sliver: nearly collinear
            d = rng.integers(-400, 401, size=2)
            t = rng.uniform(0, 1, size=3)
            pts = np.stack([np.round(t * d[0]), np.round(t * d[1])], 1).astype(np.int64)
            pts[:, 0] += rng.integers(-1, 2, size=3)
        elif kind == 3:    # exactly degenerate (collinear or coincident)
            d = rng.integers(-300, 301, size=2)
            t = rng.integers(-3, 4, size=3)
            pts = np.stack([t * d[0], t * d[1]], 1)
        else:              # large, up to about 1024 pixels
            pts = rng.integers(-8000, 8001, size=(3, 2))
        x = [int(cx + p[0]) for p in pts]
        y = [int(cy + p[1]) for p in pts]
        out.append((x, y))
    return out


@pytest.mark.parametrize("center", [0, 1])
@pytest.mark.parametrize("top_left", [0, 1])
def test_covered_samples_lie_in_the_sample_box(center, top_left):
    rng = np.random.default_rng(100 + 2 * center + top_left)
    shrunk = 0
    for x, y in random_triangles(rng, 600):
        ref, tight, (dlx, dly, dhx, dhy) = boxes(x, y, center)
        # the shrinks fit their bits and give the reference's box back (k_scatter, clip fans)
        assert 0 <= dlx <= 1 and 0 <= dly <= 1 and 0 <= dhx <= 3 and 0 <= dhy <= 3
        assert (tight[0] - dlx, tight[1] - dly, tight[2] + dhx, tight[3] + dhy) == ref
        pts = covered_samples(x, y, ref, center, top_left)
        if len(pts):
            assert pts[:, 0].min() >= tight[0] and pts[:, 0].max() <= tight[2], (x, y, ref, tight)
            assert pts[:, 1].min() >= tight[1] and pts[:, 1].max() <= tight[3], (x, y, ref, tight)
        shrunk += (ref[2] - ref[0] + 1) * (ref[3] - ref[1] + 1) - max(tight[2] - tight[0] + 1, 0) * max(
            tight[3] - tight[1] + 1, 0)
    assert shrunk > 0   # the shrink does remove samples the reference tests


def test_degenerate_triangles_cover_nothing():
    rng = np.random.default_rng(7)
    for _ in range(300):
        d = rng.integers(-200, 201, size=2)
        t = rng.integers(-4, 5, size=3)
        base = rng.integers(0, 1000 * 16, size=2)
        x = [int(base[0] + k * d[0]) for k in t]
        y = [int(base[1] + k * d[1]) for k in t]
        for center in (0, 1):
            ref, _, _ = boxes(x, y, center)
            for top_left in (0, 1):
                assert len(covered_samples(x, y, ref, center, top_left)) == 0
