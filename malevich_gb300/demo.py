"""Headless counterpart of the reference's application loop (source/main.c:1265-1299 render(),
1422-1477 camera set-up, 1480-1562 update()): the scene's objects are drawn with basic_vs +
basic_ps into a render target cleared to the reference's colour and a reversed-Z depth buffer
cleared to 0, through the C ABI, and each frame is written as a PNG instead of being presented
through GDI (no window system here).

Scenes: the reference's `.octrn` meshes from an asset folder (their textures are loaded when the
folder has them, converted from sRGB as main.c:546-557 does, else a seeded noise texture stands in),
or, without a folder, a seeded synthetic scene. The camera starts where the reference's does and
turns by a fixed yaw step per frame, as if the mouse had moved.

    python -m malevich_gb300.demo --assets <folder> --frames 4 --out demo_out
"""
import argparse
import math
import os
import struct
import zlib

import numpy as np

from . import api, octrn, scenes

REFERENCE_SCENES = {
    "ftm": ["ftm_piedras", "ftm_madera", "ftm_leaves", "ftm_dec", "ftm_roof", "ftm_ground", "ftm_sky"],
    "toon": ["toon_house", "toon_sky"],
}


def write_png(path, rgba8):
    """An 8-bit RGBA PNG of an (H, W, 4) uint8 array (zlib from the standard library)."""
    rgba8 = np.ascontiguousarray(rgba8, np.uint8)
    h, w = rgba8.shape[:2]
    raw = b"".join(b"\x00" + rgba8[y].tobytes() for y in range(h))

    def chunk(tag, data):
        return struct.pack(">I", len(data)) + tag + data + struct.pack(">I", zlib.crc32(tag + data) & 0xFFFFFFFF)

    with open(path, "wb") as f:
        f.write(b"\x89PNG\r\n\x1a\n")
        f.write(chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, 8, 6, 0, 0, 0)))
        f.write(chunk(b"IDAT", zlib.compress(raw, 6)))
        f.write(chunk(b"IEND", b""))


def read_png(path):
    """The (H, W, 4) uint8 pixels of a PNG written by write_png (filter type 0 only)."""
    data = open(path, "rb").read()
    assert data[:8] == b"\x89PNG\r\n\x1a\n"
    pos, idat, w, h = 8, b"", 0, 0
    while pos < len(data):
        n = struct.unpack(">I", data[pos:pos + 4])[0]
        tag, body = data[pos + 4:pos + 8], data[pos + 8:pos + 8 + n]
        if tag == b"IHDR":
            w, h = struct.unpack(">II", body[:8])
        elif tag == b"IDAT":
            idat += body
        pos += 12 + n
    raw = np.frombuffer(zlib.decompress(idat), np.uint8).reshape(h, 1 + 4 * w)
    return raw[:, 1:].reshape(h, w, 4).copy()


def target_to_rgba8(color_u32):
    """Render-target words to RGBA pixels as the reference's window shows them: the output merger
    packs R << 16 | G << 8 | B (main.c:1176-1178), which the GDI surface displays as RGB
    (main.c:286-357), so red is byte 2 and blue byte 0. (The clear packs R in the low byte,
    math.h:321-323, so cleared pixels show red and blue swapped, as in the reference.)"""
    c = color_u32.astype(np.uint32)
    out = np.empty(c.shape + (4,), np.uint8)
    out[..., 0] = (c >> 16) & 0xFF
    out[..., 1] = (c >> 8) & 0xFF
    out[..., 2] = c & 0xFF
    out[..., 3] = 255
    return out


def reference_camera(width, height, pos=(3.5, 1.0, 1.0), yaw=0.0, pitch=0.0, fov_y_deg=75.0, near=0.01):
    """(clip_from_view, view_from_world) as the reference builds them: a left-handed reversed-Z
    infinite projection (main.c:1431-1441) and world_from_view = change_of_basis * yaw * pitch
    with the camera position as translation (main.c:1516-1550), inverted."""
    clip_from_view = scenes.reversed_z_infinite(fov_y_deg, width / height, near)
    cp, sp = math.cos(-pitch), math.sin(-pitch)
    cy, sy = math.cos(-yaw), math.sin(-yaw)
    rot_pitch = np.array([[1, 0, 0, 0], [0, cp, sp, 0], [0, -sp, cp, 0], [0, 0, 0, 1]], np.float64)
    rot_yaw = np.array([[cy, 0, -sy, 0], [0, 1, 0, 0], [sy, 0, cy, 0], [0, 0, 0, 1]], np.float64)
    change_of_basis = np.array([[0, 0, -1, 0], [1, 0, 0, 0], [0, 1, 0, 0], [0, 0, 0, 1]], np.float64)
    world_from_view = change_of_basis @ (rot_yaw @ rot_pitch)
    world_from_view[:3, 3] = pos
    return clip_from_view, np.linalg.inv(world_from_view)


def load_reference_scene(assets, scene="ftm", seed=0):
    """[(vertices (n, 8) float32, indices uint32, RGBA8 texture)] of a reference scene's objects
    that the folder has."""
    rng = np.random.default_rng(seed)
    objects = []
    for name in REFERENCE_SCENES[scene]:
        mesh = os.path.join(assets, name + "_mesh.octrn")
        if not os.path.exists(mesh):
            continue
        v, i = octrn.read_mesh(mesh)
        tex_path = os.path.join(assets, name + "_tex.octrn")
        if os.path.exists(tex_path):
            t, fmt = octrn.read_image(tex_path)
            if fmt not in (octrn.FORMAT_R8G8B8A8_UNORM, octrn.FORMAT_R8G8B8A8_UNORM_SRGB):
                raise octrn.OctrnError("%s: basic_ps samples RGBA8 textures" % tex_path)
            t = octrn.srgb_to_linear_rgba8(t)
        else:
            t = _noise_texture(rng, 256)
        objects.append((v, i, t))
    return objects


def _noise_texture(rng, size):
    return rng.integers(0, 256, (size, size, 4), dtype=np.uint8)


def synthetic_scene(seed=0):
    """A few seeded icospheres and a heightfield around the reference camera's target."""
    rng = np.random.default_rng(seed)
    objects = []
    v, f = scenes.heightfield(rng, 64, 6.0, 0.4, center=(0.0, 0.0, -0.5))
    objects.append((v, f.astype(np.uint32).ravel(), _noise_texture(rng, 256)))
    for k in range(4):
        dirs, faces = scenes.icosphere(3)
        vv = scenes.sphere_vertices(dirs, 1.0 + 0.03 * rng.standard_normal(len(dirs)))
        vv[:, 0:3] = vv[:, 0:3] * rng.uniform(0.3, 0.7) + rng.uniform([-1.5, -1.5, 0.0], [0.5, 1.5, 1.0])
        objects.append((vv, faces.astype(np.uint32).ravel(), _noise_texture(rng, 256)))
    return objects


def scene_frame(objects, width, height, yaw=0.0, pitch=0.0):
    """render()'s frame (main.c:1265-1299): reference clear colour, depth cleared to 0 (reversed Z,
    GREATER_EQUAL), one basic_vs + basic_ps draw per object with its texture bound to both stages."""
    cb = scenes.per_frame_cb(*reference_camera(width, height, yaw=yaw, pitch=pitch))
    vp = (0.0, 0.0, float(width), float(height), 0.0, 1.0)
    draws = []
    for v, i, t in objects:
        tex = scenes.Texture(np.ascontiguousarray(t, np.uint8).view(np.uint32).reshape(t.shape[0], t.shape[1]),
                             scenes.FMT_RGBA8)
        ib = scenes.pad_indices(np.asarray(i, np.int64).reshape(-1, 3))
        draws.append(scenes.Draw(scenes.VS_BASIC, scenes.PS_BASIC, np.ascontiguousarray(v, np.float32), ib,
                                 (len(i) // 3) * 3, cb=cb, vs_tex=tex, ps_tex=tex, viewport=vp))
    return scenes.Frame(width, height, draws, clear_color=scenes.REFERENCE_CLEAR_COLOR, clear_depth=0.0)


def run(device, objects, frames=4, width=1200, height=720, out_dir="demo_out", yaw_step=0.15):
    """Renders `frames` frames, turning the camera by yaw_step radians each, and writes
    frame_000.png ...; returns the paths and each frame's statistics."""
    os.makedirs(out_dir, exist_ok=True)
    ctx = device.immediate
    paths, stats = [], []
    for k in range(frames):
        fr = scene_frame(objects, width, height, yaw=k * yaw_step)
        r = api.FrameRenderer(device, fr)
        ctx.reset_stats()
        r.render_per_draw()
        color = r.read(0)["color"]
        stats.append(ctx.stats())
        r.destroy()
        p = os.path.join(out_dir, "frame_%03d.png" % k)
        write_png(p, target_to_rgba8(color))
        paths.append(p)
    return paths, stats


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--assets", default=None, help="folder with the reference's .octrn assets")
    ap.add_argument("--scene", default="ftm", choices=sorted(REFERENCE_SCENES))
    ap.add_argument("--frames", type=int, default=4)
    ap.add_argument("--width", type=int, default=1200)
    ap.add_argument("--height", type=int, default=720)
    ap.add_argument("--out", default="demo_out")
    a = ap.parse_args(argv)
    objects = load_reference_scene(a.assets, a.scene) if a.assets else synthetic_scene()
    if not objects:
        raise SystemExit("no meshes of scene %r in %s" % (a.scene, a.assets))
    dev = api.Device(0)
    try:
        paths, stats = run(dev, objects, a.frames, a.width, a.height, a.out)
    finally:
        dev.destroy()
    for p, s in zip(paths, stats):
        print(p, s["assembled_triangle_count"], "triangles assembled")


if __name__ == "__main__":
    main()
