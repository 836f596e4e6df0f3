"""The .octrn asset format (data only): round trips of meshes and images, rejection of malformed
files, the reference's sRGB-to-linear load step, and - where the reference's asset folder is
present on this machine - a parse of every shipped mesh and image with consistency checks."""
import glob
import os
import struct

import numpy as np
import pytest

from malevich_gb300 import octrn

from oracle import ref_build

# the reference's shipped assets, when its checkout is on this machine ($MALEVICH_ASSETS overrides)
ASSETS = os.environ.get("MALEVICH_ASSETS") or os.path.join(ref_build.reference_dir() or "", "assets")


def test_mesh_round_trip(tmp_path):
    rng = np.random.default_rng(1)
    v = rng.standard_normal((37, 8)).astype(np.float32)
    i = rng.integers(0, 37, 60).astype(np.uint32)
    p = tmp_path / "m.octrn"
    octrn.write_mesh(p, v, i)
    assert os.path.getsize(p) == 28 + 37 * 32 + 60 * 4
    v2, i2 = octrn.read_mesh(p)
    assert np.array_equal(v, v2) and np.array_equal(i, i2)


@pytest.mark.parametrize("fmt", [octrn.FORMAT_R8G8B8A8_UNORM, octrn.FORMAT_R16G16B16A16_FLOAT,
                                 octrn.FORMAT_R32G32B32A32_FLOAT])
def test_image_round_trip(tmp_path, fmt):
    rng = np.random.default_rng(2)
    dt = {octrn.FORMAT_R8G8B8A8_UNORM: np.uint8, octrn.FORMAT_R16G16B16A16_FLOAT: np.float16,
          octrn.FORMAT_R32G32B32A32_FLOAT: np.float32}[fmt]
    t = (rng.random((5, 7, 4)) * 200).astype(dt)
    p = tmp_path / "t.octrn"
    octrn.write_image(p, t, fmt)
    t2, f2 = octrn.read_image(p)
    assert f2 == fmt and t2.dtype == dt and np.array_equal(t, t2)


def test_malformed_files_are_rejected(tmp_path):
    p = tmp_path / "bad.octrn"
    p.write_bytes(b"notoctrn" + bytes(40))
    with pytest.raises(octrn.OctrnError):
        octrn.read_mesh(p)
    octrn.write_mesh(p, np.zeros((4, 8), np.float32), np.array([0, 1, 9], np.uint32))
    with pytest.raises(octrn.OctrnError):
        octrn.read_mesh(p)                                   # index 9 >= 4 vertices
    octrn.write_mesh(p, np.zeros((4, 8), np.float32), np.array([0, 1, 2], np.uint32))
    p.write_bytes(p.read_bytes()[:-4])
    with pytest.raises(octrn.OctrnError):
        octrn.read_mesh(p)                                   # truncated
    with pytest.raises(octrn.OctrnError):
        octrn.read_image(p)                                  # a mesh is not an image


def test_srgb_to_linear_matches_the_reference_formula():
    b = np.arange(256, dtype=np.uint8)
    got = octrn.srgb_to_linear_rgba8(b)
    v = np.float32(b.astype(np.float32) * np.float32(1.0 / 255.0))
    for k in (0, 10, 11, 100, 128, 254, 255):
        d = float(v[k])
        lin = d / 12.92 if d <= 0.04045 else ((d + 0.055) / 1.055) ** 2.4
        assert got[k] == int(np.float32(np.float32(lin) * np.float32(255.0)))
    assert got[0] == 0 and got[255] in (254, 255) and np.all(np.diff(got.astype(int)) >= 0)


@pytest.mark.skipif(not glob.glob(os.path.join(ASSETS, "*.octrn")), reason="the reference's assets are not here")
def test_reference_assets_parse():
    meshes = [p for p in glob.glob(os.path.join(ASSETS, "*.octrn")) if "_mesh" in os.path.basename(p)]
    assert meshes
    for p in meshes:
        v, i = octrn.read_mesh(p)
        assert os.path.getsize(p) == 28 + v.nbytes + i.nbytes
        assert np.all(np.isfinite(v))
        n = np.linalg.norm(v[:, 3:6], axis=1)
        assert np.mean(np.abs(n - 1.0) < 1e-2) > 0.99, p    # unit normals
        assert len(i) % 3 == 0
    for p in glob.glob(os.path.join(ASSETS, "*irradiance*.octrn")):
        t, fmt = octrn.read_image(p)
        assert fmt == octrn.FORMAT_R32G32B32A32_FLOAT and t.shape == (128, 256, 4)
        assert np.all(np.isfinite(t)) and np.all(t[..., :3] >= 0)
