"""Generates the golden fixtures in this folder by running the reference's own pipeline core,
compiled headless from its sources by oracle/ref_build.py (x86-64, this container only).

Each fixture holds the input frame (vertex/index buffers, constant buffer, textures, state) and
the reference's outputs: colour, depth, triangle-ID and draw-ID buffers, hierarchical-Z tile
minima, Stats (main.c:199-206), and for every draw the assembled triangles' setup and the
per-(bin, triangle) TileInfo masks. The reference runs with one OpenMP thread, which gives the
serial primitive order (main.c:874-875).

Scenes: seeded small icosphere scenes for every reference shader pairing, with the camera outside
(no clipping) and inside the geometry (near/side-plane clipping), and the reference's own fixed
inputs - the Suprematism quads (main.c:232-254) with passthrough_vs/ps, and the fullscreen quad
(main.c:255-270) with fullscreen_vs + env_lighting_ps - parsed from source/main.c at generation
time, never written out by hand.

Usage: python tests/golden/make_golden.py [--reference DIR]   (default: oracle/ref_build.py's reference_dir())
"""
import argparse
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from malevich_gb300 import scenes  # noqa: E402
from oracle import pyoracle, ref_build  # noqa: E402


def _parse_c_array(src, name):
    m = re.search(r"%s\[\]\s*=\s*\{(.*?)\};" % re.escape(name), src, re.S)
    if not m:
        raise RuntimeError("array %s not found" % name)
    nums = re.findall(r"-?\d+\.?\d*(?:[eE][-+]?\d+)?", m.group(1))
    return [float(x) for x in nums]


def reference_fixed_frames(reference, w, h):
    src = open(os.path.join(reference, "source", "main.c"), encoding="utf-8", errors="replace").read()
    vb = np.array(_parse_c_array(src, "suprematist_vertex_buffer"), np.float32).reshape(-1, 8)
    ib = np.array(_parse_c_array(src, "suprematist_index_buffer"), np.uint32)
    vp = (0.0, 0.0, float(w), float(h), 0.0, 1.0)
    supre = scenes.Frame(w, h, [scenes.Draw(scenes.VS_PASSTHROUGH, scenes.PS_PASSTHROUGH, vb, ib, len(ib), viewport=vp)],
                         clear_color=scenes.REFERENCE_CLEAR_COLOR, clear_depth=0.0)
    fvb = np.array(_parse_c_array(src, "fullscreen_vertex_buffer"), np.float32).reshape(-1, 8)
    fib = np.array(_parse_c_array(src, "fullscreen_index_buffer"), np.uint32)
    rng = np.random.default_rng(11)
    rad = scenes.smooth_hdr(rng, 64, 32, scenes.FMT_RGBA32F, base_cells=4)
    cb = scenes.per_frame_cb(scenes.reversed_z_infinite(75.0, w / h, 0.01),
                             scenes.look_at_lh((3.5, 1.0, 1.0), (0.0, 1.0, 1.0)))
    full = scenes.Frame(w, h, [scenes.Draw(scenes.VS_FULLSCREEN, scenes.PS_ENV_LIGHTING, fvb, fib, len(fib), cb=cb,
                                           ps_tex=rad, viewport=vp)],
                        clear_color=scenes.REFERENCE_CLEAR_COLOR, clear_depth=0.0)
    return {"suprematism": supre, "fullscreen_env": full}


def scene_list():
    out = {}
    pairs = [(scenes.VS_BASIC, scenes.PS_BASIC), (scenes.VS_VERTEX_LIGHTING, scenes.PS_ENV_LIGHTING),
             (scenes.VS_VERTEX_LIGHTING, scenes.PS_PASSTHROUGH), (scenes.VS_BASIC, scenes.PS_ENV_LIGHTING)]
    for k, (vs, ps) in enumerate(pairs):
        for inside in (False, True):
            name = "icospheres_vs%d_ps%d_%s" % (vs, ps, "inside" if inside else "outside")
            seed = 100 + 10 * k + int(inside)
            while True:   # inside scenes must actually clip and show something
                fr = scenes.small_scene(seed, 64, 64, vs=vs, ps=ps, inside=inside)
                st = pyoracle.render_oracle(fr)["stats"]
                if st["assembled_triangle_count"] > 0 and (not inside or st["clipped_triangle_count"] > 0):
                    break
                seed += 1000
            out[name] = fr
    out["icospheres_32x32_level3"] = scenes.small_scene(300, 32, 32, level=3, n_objects=5)
    return out


def scene_frame_reduced():
    """The scene-scale frame's construction at 480x272: a 100x100-cell heightfield (20,000
    triangles) and 11 icospheres/boxes of 800-3,000 triangles in the 20 m cube, seen from a seeded
    pose inside it (so the ground crosses the near and side planes and is clipped heavily),
    vertex_lighting_vs + env_lighting_ps with the reference's depth mode. Smaller textures than the
    full frame (256x128 RGBA16F radiance) keep the fixture small; the full-size frame is pinned
    live where the reference is built (tests/test_oracle.py)."""
    seed = 12
    while True:
        rng = np.random.default_rng(seed)
        counts = (800 + 2200 * rng.random(11)).astype(int)
        fr = scenes.config2_scene(seed=seed, width=480, height=272, ground_cells=100, counts=counts,
                                  radiance_size=(256, 128), irradiance_size=(64, 32), ground_tex=0)
        st = pyoracle.render_oracle(fr)["stats"]
        if st["clipped_triangle_count"] >= 300 and st["assembled_triangle_count"] >= 3000:
            return {"scene_frame_480x272": fr}
        seed += 1000


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=ref_build.reference_dir())
    ap.add_argument("--only", default="", help="comma-separated fixture names to (re)generate (default: all)")
    args = ap.parse_args(argv)
    ref_build.main(["--reference", args.reference, "--sizes", "64x64,32x32,480x272"])
    frames = scene_list()
    frames.update(reference_fixed_frames(args.reference, 64, 64))
    big = scene_frame_reduced()
    frames.update(big)
    only = [n for n in args.only.split(",") if n]
    for name, fr in frames.items():
        if only and name not in only:
            continue
        # the reduced scene frame keeps no per-triangle captures (they would dwarf the fixture);
        # the small fixtures cover the setup words and TileInfo masks
        r = pyoracle.render_reference(fr, capture=name not in big, threads=1)
        arrays = scenes.frame_to_arrays(fr)
        for k in ("color", "depth", "vis_tri", "vis_draw", "tile_min"):
            arrays["out/" + k] = r[k]
        arrays["out/stats"] = np.array([r["stats"][k] for k in ("vertex_count", "input_triangle_count",
                                                                 "assembled_triangle_count", "active_bin_count",
                                                                 "total_triangle_count_in_bins")], np.int64)
        for i, c in enumerate(r["captures"]):
            for k, v in c.items():
                arrays["out/cap%d/%s" % (i, k)] = v
        path = os.path.join(HERE, name + ".npz")
        np.savez_compressed(path, **arrays)
        print("wrote", path, os.path.getsize(path), "bytes; stats", r["stats"])


if __name__ == "__main__":
    main()
