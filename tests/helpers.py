"""Comparison helpers shared by the parity tests."""
import numpy as np

# Colour tolerance: +-1 LSB per UNORM8 channel. Colour goes through powf/expf/acosf, which the
# reference takes from Intel SVML, the CPU checkers from libm and the GPU from CUDA's libdevice;
# these differ by a few ulp, which moves a rounded 8-bit channel by at most one step.
COLOR_TOL = 1


def channels(c):
    return c.view(np.uint8).reshape(c.shape + (4,)).astype(np.int16)


def color_diff(a, b):
    return np.abs(channels(a) - channels(b))


def assert_color_close(got, want, tol=COLOR_TOL, max_outlier_frac=0.0):
    d = color_diff(got, want)
    bad = (d > tol).any(axis=-1)
    frac = bad.mean() if bad.size else 0.0
    assert frac <= max_outlier_frac, "colour: %d pixels (%.4f%%) beyond +-%d LSB, max diff %d" % (
        bad.sum(), 100 * frac, tol, d.max())
    return d


def reference_nan_pixels(color):
    """Pixels where the reference wrote NaN colour: _mm256_cvtps_epi32 turns a NaN channel into
    0x80000000 (main.c:1176-1178), which its approximate rsqrt produces where a cosine exceeds 1
    before acos (common_shader_core.h:232-240). Compared apart from the +-1 LSB bound."""
    return np.ascontiguousarray(color).view(np.uint32) == 0x80000000


def outlier_report(got, want):
    """Counts for the colour-outlier report: pixels beyond +-1 LSB (excluding the reference's NaN
    pixels when `want` comes from the reference), their fraction and the largest difference."""
    d = color_diff(got, want).max(axis=-1)
    n = int((d > COLOR_TOL).sum())
    return {"pixels_beyond_1lsb": n, "fraction": n / d.size if d.size else 0.0, "max_diff": int(d.max()) if d.size else 0}


def assert_bits_equal(got, want, what):
    g = np.ascontiguousarray(got).view(np.uint32)
    w = np.ascontiguousarray(want).view(np.uint32)
    if not np.array_equal(g, w):
        idx = np.argwhere(g != w)
        raise AssertionError("%s differs at %d positions, first %s: got %r want %r" % (
            what, len(idx), tuple(idx[0]), got[tuple(idx[0])], want[tuple(idx[0])]))


def sort_infos(tile, tri, mask):
    order = np.lexsort((tri, tile))
    return tile[order], tri[order], mask[order]
