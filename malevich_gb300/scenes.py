"""Frame descriptions and seeded synthetic scenes for the draw path.

A `Frame` is what the reference's `render()` does in one call (source/main.c:1265-1299): clear
the render target and depth buffer, then a sequence of draws, each with its own pipeline state
(shaders, vertex/index buffers, constant buffer, SRV slot 0, viewport, cull and depth modes).
The GPU path renders a Frame through the C ABI (`malevich_gb300.api.render_frame`); the checkers
render the same description on the CPU.

All scenes are synthetic and seeded (the reference's own assets are not used): icospheres,
geodesic spheres, subdivided boxes and value-noise heightfields, RGBA8 uniform-noise textures and
smooth-noise HDR maps. Cameras follow the reference's conventions: row-major matrices applied to
column vectors, a left-handed view space (+x right, +y up, +z forward) and either the reference's
reversed-Z infinite projection (source/main.c:1436-1441, depth GREATER_EQUAL, cleared to 0) or a
standard [0,1] projection (depth LESS, cleared to 1).
"""
from dataclasses import dataclass, field
from typing import List, Optional

import numpy as np

# shader ids (same numbering as include/malevich.h)
VS_BASIC, VS_VERTEX_LIGHTING, VS_PASSTHROUGH, VS_FULLSCREEN, VS_PASSTHROUGH_UV = 1, 2, 3, 4, 5
PS_BASIC, PS_PASSTHROUGH, PS_ENV_LIGHTING, PS_COLOR_TIMES_TEXEL, PS_NONE = 1, 2, 3, 4, 5
FMT_RGBA8, FMT_RGBA16F, FMT_RGBA32F = 1, 2, 3
CULL_NONE, CULL_BACK, CULL_FRONT = 0, 1, 2
DEPTH_GREATER_EQUAL, DEPTH_LESS = 0, 1

REFERENCE_CLEAR_COLOR = (227.0 / 255.0, 223.0 / 255.0, 216.0 / 255.0, 0.0)


@dataclass
class Texture:
    data: np.ndarray          # (H, W) uint32 for RGBA8 (R in the low byte); (H, W, 4) float16/float32
    format: int

    @property
    def width(self):
        return int(self.data.shape[1])

    @property
    def height(self):
        return int(self.data.shape[0])


@dataclass
class Draw:
    vs: int
    ps: int
    vb: np.ndarray            # (N, stride/4) float32 or raw bytes (N, stride) uint8
    ib: Optional[np.ndarray]  # uint32 indices, or None for Draw(vertex_count)
    index_count: int
    cb: Optional[np.ndarray] = None      # 48 float32: clip_from_world, view_from_clip, world_from_view
    vs_tex: Optional[Texture] = None
    ps_tex: Optional[Texture] = None
    viewport: tuple = (0.0, 0.0, 0.0, 0.0, 0.0, 1.0)
    cull: int = CULL_BACK
    depth_func: int = DEPTH_GREATER_EQUAL
    start_index: int = 0
    base_vertex: int = 0
    fill_rule: int = 0        # 0: the reference's inclusive rule; 1: top-left
    sample_center: int = 0    # 0: sample at the pixel corner (the reference); 1: at its centre

    @property
    def vb_stride(self):
        a = self.vb
        return int(a.shape[1] * a.itemsize)

    def vb_bytes(self):
        return self.vb

    def vertex_count(self):
        return int(self.vb.shape[0])

    @property
    def triangle_count(self):
        return self.index_count // 3


@dataclass
class Frame:
    width: int
    height: int
    draws: List[Draw] = field(default_factory=list)
    clear_color: Optional[tuple] = REFERENCE_CLEAR_COLOR
    clear_depth: Optional[float] = 0.0
    initial_color: Optional[np.ndarray] = None
    initial_depth: Optional[np.ndarray] = None

    @property
    def input_triangles(self):
        return sum(d.triangle_count for d in self.draws)


# ------------------------------------------------------------------ matrices

def look_at_lh(eye, target, up=(0.0, 0.0, 1.0)):
    """view_from_world for a left-handed view space (+x right, +y up, +z forward) in the
    reference's right-handed, z-up world."""
    eye, target, up = (np.asarray(v, np.float64) for v in (eye, target, up))
    f = target - eye
    f /= np.linalg.norm(f)
    r = np.cross(f, up)
    if np.linalg.norm(r) < 1e-9:
        r = np.cross(f, np.array([0.0, 1.0, 0.0]))
    r /= np.linalg.norm(r)
    u = np.cross(r, f)
    m = np.eye(4)
    m[0, :3], m[1, :3], m[2, :3] = r, u, f
    m[0, 3], m[1, 3], m[2, 3] = -r @ eye, -u @ eye, -f @ eye
    return m


def reversed_z_infinite(fov_y_deg, aspect, near):
    """The reference's projection, source/main.c:1431-1441."""
    sy = 1.0 / np.tan(np.radians(fov_y_deg) / 2.0)
    sx = sy / aspect
    return np.array([[sx, 0, 0, 0], [0, sy, 0, 0], [0, 0, 0, near], [0, 0, 1, 0]], np.float64)


def perspective_lh(fov_y_deg, aspect, near, far):
    """Standard left-handed [0,1] depth projection (for depth LESS, cleared to 1)."""
    sy = 1.0 / np.tan(np.radians(fov_y_deg) / 2.0)
    sx = sy / aspect
    q = far / (far - near)
    return np.array([[sx, 0, 0, 0], [0, sy, 0, 0], [0, 0, q, -near * q], [0, 0, 1, 0]], np.float64)


def per_frame_cb(clip_from_view, view_from_world):
    """PerFrameCB (source/main.c:169-173): clip_from_world, view_from_clip, world_from_view."""
    clip_from_world = clip_from_view @ view_from_world
    return np.concatenate([clip_from_world.ravel(), np.linalg.inv(clip_from_view).ravel(),
                           np.linalg.inv(view_from_world).ravel()]).astype(np.float32)


# ------------------------------------------------------------------ meshes

def _icosahedron():
    t = (1.0 + 5.0 ** 0.5) / 2.0
    v = np.array([[-1, t, 0], [1, t, 0], [-1, -t, 0], [1, -t, 0], [0, -1, t], [0, 1, t], [0, -1, -t],
                  [0, 1, -t], [t, 0, -1], [t, 0, 1], [-t, 0, -1], [-t, 0, 1]], np.float64)
    f = np.array([[0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11], [1, 5, 9], [5, 11, 4],
                  [11, 10, 2], [10, 7, 6], [7, 1, 8], [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8],
                  [3, 8, 9], [4, 9, 5], [2, 4, 11], [6, 2, 10], [8, 6, 7], [9, 8, 1]], np.int64)
    return v / np.linalg.norm(v, axis=1, keepdims=True), f


def geodesic_sphere(freq):
    """Icosahedron with every face split into freq^2 triangles, projected to the unit sphere:
    20*freq^2 triangles (freq = 2^level gives the level-`level` icosphere)."""
    v0, f0 = _icosahedron()
    verts, index = [], {}

    def vid(key, p):
        if key not in index:
            index[key] = len(verts)
            verts.append(p)
        return index[key]

    faces = []
    for (a, b, c) in f0:
        A, B, C = v0[a], v0[b], v0[c]
        grid = {}
        for i in range(freq + 1):
            for j in range(freq + 1 - i):
                k = freq - i - j
                p = (A * k + B * i + C * j) / freq
                # canonical key so shared edges/corners are shared vertices
                wts = {a: k, b: i, c: j}
                key = tuple(sorted((vv, ww) for vv, ww in wts.items() if ww))
                grid[(i, j)] = vid(key, p)
        for i in range(freq):
            for j in range(freq - i):
                faces.append((grid[(i, j)], grid[(i + 1, j)], grid[(i, j + 1)]))
                if i + j + 1 < freq:
                    faces.append((grid[(i + 1, j)], grid[(i + 1, j + 1)], grid[(i, j + 1)]))
    v = np.array(verts, np.float64)
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    return v, np.array(faces, np.int64)


def icosphere(level):
    return geodesic_sphere(2 ** level)


def sphere_vertices(dirs, radii):
    """pos3, nrm3, uv2 per vertex (the basic_vs input layout, basic_vs.c:3-7)."""
    pos = dirs * radii[:, None]
    u = 0.5 + np.arctan2(dirs[:, 1], dirs[:, 0]) / (2 * np.pi)
    v = 0.5 + np.arcsin(np.clip(dirs[:, 2], -1, 1)) / np.pi
    return np.concatenate([pos, dirs, u[:, None], v[:, None]], axis=1).astype(np.float32)


def subdivided_box(n):
    """Axis-aligned unit cube [-1,1]^3 with each face split into n x n quads: 12*n^2 triangles,
    outward winding; per-face normals and UVs."""
    verts, faces = [], []
    axes = [(0, 1, 2, 1), (0, 1, 2, -1), (1, 2, 0, 1), (1, 2, 0, -1), (2, 0, 1, 1), (2, 0, 1, -1)]
    g = np.linspace(-1, 1, n + 1)
    for (ua, va, na, s) in axes:
        base = len(verts)
        for j in range(n + 1):
            for i in range(n + 1):
                p = np.zeros(3)
                p[ua], p[va], p[na] = g[i], g[j], s
                nrm = np.zeros(3)
                nrm[na] = s
                verts.append(np.concatenate([p, nrm, [i / n, j / n]]))
        for j in range(n):
            for i in range(n):
                a = base + j * (n + 1) + i
                b, c, d = a + 1, a + n + 1, a + n + 2
                if s > 0:
                    faces += [(a, b, d), (a, d, c)]
                else:
                    faces += [(a, d, b), (a, c, d)]
    return np.array(verts, np.float32), np.array(faces, np.int64)


def value_noise_2d(rng, shape, octaves=4, base_cells=8):
    """Sum of `octaves` bilinearly upsampled random grids (frequency doubling, amplitude halving),
    normalised to [0, 1]."""
    h, w = shape
    out = np.zeros((h, w), np.float64)
    amp, total = 1.0, 0.0
    for o in range(octaves):
        cells = base_cells * (2 ** o)
        grid = rng.random((cells + 1, cells + 1))
        ys = np.linspace(0, cells, h, endpoint=False) if h > 1 else np.zeros(1)
        xs = np.linspace(0, cells, w, endpoint=False) if w > 1 else np.zeros(1)
        y0 = np.floor(ys).astype(int)
        x0 = np.floor(xs).astype(int)
        fy = (ys - y0)[:, None]
        fx = (xs - x0)[None, :]
        g00 = grid[y0][:, x0]
        g10 = grid[y0][:, x0 + 1]
        g01 = grid[y0 + 1][:, x0]
        g11 = grid[y0 + 1][:, x0 + 1]
        out += amp * ((g00 * (1 - fx) + g10 * fx) * (1 - fy) + (g01 * (1 - fx) + g11 * fx) * fy)
        total += amp
        amp *= 0.5
    out /= total
    lo, hi = out.min(), out.max()
    return (out - lo) / max(hi - lo, 1e-12)


def heightfield(rng, cells, size, height, center=(0.0, 0.0, 0.0)):
    """cells x cells grid (2*cells^2 triangles) over a size x size square in the world xy plane
    (z up), heights from 4-octave value noise; outward (+z) winding; pos3, nrm3, uv2."""
    n = cells + 1
    hgt = value_noise_2d(rng, (n, n), octaves=4, base_cells=8) * height
    xs = np.linspace(-size / 2, size / 2, n)
    X, Y = np.meshgrid(xs, xs)
    Z = hgt
    gy, gx = np.gradient(Z, xs, xs)
    nrm = np.stack([-gx, -gy, np.ones_like(Z)], axis=-1)
    nrm /= np.linalg.norm(nrm, axis=-1, keepdims=True)
    U, V = np.meshgrid(np.linspace(0, 1, n), np.linspace(0, 1, n))
    verts = np.concatenate([np.stack([X + center[0], Y + center[1], Z + center[2]], -1), nrm,
                            np.stack([U, V], -1)], axis=-1).reshape(-1, 8).astype(np.float32)
    j, i = np.meshgrid(np.arange(cells), np.arange(cells), indexing="ij")
    a = (j * n + i).ravel()
    b, c, d = a + 1, a + n, a + n + 1
    faces = np.stack([np.stack([a, b, d], 1), np.stack([a, d, c], 1)], 1).reshape(-1, 3)
    return verts, faces.astype(np.int64)


def pad_indices(faces, multiple=8):
    """Flatten to an index buffer padded with (0,0,0) triangles to a multiple of 8 indices, as the
    reference's own index buffers are (source/main.c:245-254)."""
    ib = faces.reshape(-1).astype(np.uint32)
    pad = (-len(ib)) % multiple
    while pad % 3:
        pad += multiple
    return np.concatenate([ib, np.zeros(pad, np.uint32)])


# ------------------------------------------------------------------ textures

def noise_rgba8(rng, w, h):
    return Texture(rng.integers(0, 2 ** 32, size=(h, w), dtype=np.uint64).astype(np.uint32), FMT_RGBA8)


def smooth_hdr(rng, w, h, fmt, lo=0.0, hi=4.0, base_cells=8):
    chans = [value_noise_2d(rng, (h, w), octaves=4, base_cells=base_cells) for _ in range(3)]
    data = np.stack(chans + [np.ones((h, w))], -1) * np.array([hi - lo] * 3 + [1.0]) + np.array([lo] * 3 + [0.0])
    dt = np.float16 if fmt == FMT_RGBA16F else np.float32
    return Texture(data.astype(dt), fmt)


def uniform_rgba32f(rng, w, h):
    return Texture(rng.random((h, w, 4)).astype(np.float32), FMT_RGBA32F)


# ------------------------------------------------------------------ configurations

def config1_plain(seed=1, native=False, width=1280, height=720, tex_size=1024, level=5):
    """Plain single draw: level-5 icosphere (20,480 triangles), radius 1+0.05*N(0,1) per vertex,
    basic_vs + basic_ps over a uniform-noise RGBA8 texture, camera at distance 3, 60 degree FOV,
    back-face culling. native=False: depth LESS cleared to 1.0 with a standard projection;
    native=True: the reference's depth mode (GREATER_EQUAL, cleared to 0, reversed-Z)."""
    rng = np.random.default_rng(seed)
    dirs, faces = icosphere(level)
    radii = 1.0 + 0.05 * rng.standard_normal(len(dirs))
    vb = sphere_vertices(dirs, radii)
    ib = pad_indices(faces)
    tex = noise_rgba8(rng, tex_size, tex_size)
    aspect = width / height
    view = look_at_lh((3.0, 0.0, 0.0), (0.0, 0.0, 0.0))
    if native:
        proj, depth_func, clear_depth = reversed_z_infinite(60.0, aspect, 0.01), DEPTH_GREATER_EQUAL, 0.0
    else:
        proj, depth_func, clear_depth = perspective_lh(60.0, aspect, 0.1, 100.0), DEPTH_LESS, 1.0
    d = Draw(VS_BASIC, PS_BASIC, vb, ib, len(ib), cb=per_frame_cb(proj, view), vs_tex=tex, ps_tex=tex,
             viewport=(0.0, 0.0, float(width), float(height), 0.0, 1.0), cull=CULL_BACK, depth_func=depth_func)
    return Frame(width, height, [d], clear_color=REFERENCE_CLEAR_COLOR, clear_depth=clear_depth)


def _object_transform(vb, scale, pos):
    out = vb.copy()
    out[:, 0:3] = vb[:, 0:3] * scale + pos
    return out


def config2_scene(seed=2, width=1920, height=1080, ground_cells=512, counts=None,
                  radiance_size=(2048, 1024), irradiance_size=(64, 32), ground_tex=2048, fov=75.0):
    """Scene-scale frame: a ground heightfield of ground_cells^2 cells (2*512^2 = 524,288
    triangles) plus 11 seeded icospheres/boxes of 5k-60k triangles placed uniformly in a 20 m cube
    (so many triangles cover under a pixel); vertex_lighting_vs (irradiance 64x32 RGBA32F) +
    env_lighting_ps (radiance 2048x1024 RGBA16F), both smooth noise in [0,4]; a seeded camera pose
    inside the cube; the reference's depth mode."""
    rng = np.random.default_rng(seed)
    irr = smooth_hdr(rng, irradiance_size[0], irradiance_size[1], FMT_RGBA32F, base_cells=4)
    rad = smooth_hdr(rng, radiance_size[0], radiance_size[1], FMT_RGBA16F)
    # the 2048x2048 RGBA8 ground texture of this configuration is generated to keep the seeded
    # stream stable, but no shader of this frame samples an RGBA8 texture, so it is not bound
    if ground_tex:
        noise_rgba8(rng, ground_tex, ground_tex)
    eye = np.array([rng.uniform(-6, 6), rng.uniform(-6, 6), rng.uniform(1.5, 4.0)])
    yaw = rng.uniform(0, 2 * np.pi)
    target = eye + np.array([np.cos(yaw), np.sin(yaw), rng.uniform(-0.35, -0.1)])
    proj = reversed_z_infinite(fov, width / height, 0.01)
    cb = per_frame_cb(proj, look_at_lh(eye, target))
    vp = (0.0, 0.0, float(width), float(height), 0.0, 1.0)
    draws = []
    gv, gf = heightfield(rng, ground_cells, 20.0, 1.5, center=(0.0, 0.0, -0.5))
    draws.append(Draw(VS_VERTEX_LIGHTING, PS_ENV_LIGHTING, gv, pad_indices(gf), 0, cb=cb, vs_tex=irr, ps_tex=rad,
                      viewport=vp))
    draws[-1].index_count = len(draws[-1].ib)
    if counts is None:
        counts = (5000 + 55000 * rng.random(11) ** 0.25).astype(int)
    for k, target_count in enumerate(counts):
        if rng.random() < 0.5:
            freq = max(1, int(round(np.sqrt(target_count / 20.0))))
            dirs, faces = geodesic_sphere(freq)
            v = sphere_vertices(dirs, np.ones(len(dirs)))
        else:
            n = max(1, int(round(np.sqrt(target_count / 12.0))))
            v, faces = subdivided_box(n)
        scale = rng.uniform(0.3, 2.0)
        pos = np.array([rng.uniform(-10, 10), rng.uniform(-10, 10), rng.uniform(-0.5, 8.0)])
        vb = _object_transform(v, scale, pos)
        ib = pad_indices(faces)
        draws.append(Draw(VS_VERTEX_LIGHTING, PS_ENV_LIGHTING, vb, ib, len(ib), cb=cb, vs_tex=irr, ps_tex=rad,
                          viewport=vp))
    return Frame(width, height, draws, clear_color=REFERENCE_CLEAR_COLOR, clear_depth=0.0)


def config3_batched(seed=3, n_views=64, n_meshes=16, resolutions=(256, 384, 512, 768, 1024),
                    tri_range=(2000, 200000), draws_per_view=(4, 16), tex_size=1024, n_textures=4):
    """Batched multi-view: n_views views at seeded square resolutions, n_meshes icosphere/heightfield
    meshes with log-uniform triangle counts, each view draws a seeded subset of 4-16 meshes with
    basic_vs + basic_ps over RGBA8 noise textures; reference depth mode. Returns a list of Frames."""
    rng = np.random.default_rng(seed)
    texes = [noise_rgba8(rng, tex_size, tex_size) for _ in range(n_textures)]
    meshes = []
    for m in range(n_meshes):
        target = int(np.exp(rng.uniform(np.log(tri_range[0]), np.log(tri_range[1]))))
        if rng.random() < 0.5:
            freq = max(1, int(round(np.sqrt(target / 20.0))))
            dirs, faces = geodesic_sphere(freq)
            radii = 1.0 + 0.03 * rng.standard_normal(len(dirs))
            v = sphere_vertices(dirs, radii)
        else:
            cells = max(1, int(round(np.sqrt(target / 2.0))))
            v, faces = heightfield(rng, cells, 2.5, 0.4)
        pos = rng.uniform(-3, 3, size=3)
        meshes.append((_object_transform(v, rng.uniform(0.6, 1.6), pos), pad_indices(faces)))
    frames = []
    for vi in range(n_views):
        res = int(rng.choice(resolutions))
        k = int(rng.integers(draws_per_view[0], draws_per_view[1] + 1))
        subset = rng.choice(n_meshes, size=k, replace=False)
        az, el = rng.uniform(0, 2 * np.pi), rng.uniform(0.2, 0.9)
        dist = rng.uniform(8, 14)
        eye = dist * np.array([np.cos(az) * np.cos(el), np.sin(az) * np.cos(el), np.sin(el)])
        cb = per_frame_cb(reversed_z_infinite(60.0, 1.0, 0.01), look_at_lh(eye, (0, 0, 0)))
        vp = (0.0, 0.0, float(res), float(res), 0.0, 1.0)
        draws = []
        for m in subset:
            vb, ib = meshes[m]
            t = texes[int(m) % n_textures]
            draws.append(Draw(VS_BASIC, PS_BASIC, vb, ib, len(ib), cb=cb, vs_tex=t, ps_tex=t, viewport=vp))
        frames.append(Frame(res, res, draws, clear_color=REFERENCE_CLEAR_COLOR, clear_depth=0.0))
    return frames


def small_scene(seed, width=64, height=64, vs=VS_BASIC, ps=PS_BASIC, n_objects=4, level=2, native=True,
                inside=False, tex_size=64):
    """A few perturbed icospheres in a small render target, for parity tests that must finish in
    seconds on the CPU checkers. inside=True puts the camera among the objects so that triangles
    cross the near and side planes and get clipped."""
    rng = np.random.default_rng(seed)
    tex8 = noise_rgba8(rng, tex_size, tex_size)
    irr = smooth_hdr(rng, 16, 8, FMT_RGBA32F, base_cells=2)
    rad = smooth_hdr(rng, 64, 32, FMT_RGBA32F, base_cells=4)
    if inside:
        eye = np.zeros(3)
        target = rng.standard_normal(3)
    else:
        eye = np.array([4.0 + rng.uniform(0, 1), rng.uniform(-1, 1), rng.uniform(-1, 1)])
        target = np.zeros(3)
    aspect = width / height
    if native:
        proj, df, cd = reversed_z_infinite(60.0, aspect, 0.01), DEPTH_GREATER_EQUAL, 0.0
    else:
        proj, df, cd = perspective_lh(60.0, aspect, 0.05, 50.0), DEPTH_LESS, 1.0
    cb = per_frame_cb(proj, look_at_lh(eye, target))
    vp = (0.0, 0.0, float(width), float(height), 0.0, 1.0)
    draws = []
    for k in range(n_objects):
        dirs, faces = icosphere(level)
        radii = rng.uniform(0.4, 1.0) * (1.0 + 0.05 * rng.standard_normal(len(dirs)))
        vb = sphere_vertices(dirs, radii)
        if inside:   # spheres around the eye, some straddling the camera plane
            off = rng.standard_normal(3)
            vb[:, 0:3] += off / np.linalg.norm(off) * rng.uniform(0.6, 1.3)
        else:
            vb[:, 0:3] += rng.uniform(-1.2, 1.2, size=3)
        ib = pad_indices(faces)
        vs_tex = irr if vs == VS_VERTEX_LIGHTING else tex8
        ps_tex = rad if ps == PS_ENV_LIGHTING else tex8
        draws.append(Draw(vs, ps, vb, ib, len(ib), cb=cb, vs_tex=vs_tex, ps_tex=ps_tex, viewport=vp,
                          depth_func=df))
    return Frame(width, height, draws, clear_color=REFERENCE_CLEAR_COLOR, clear_depth=cd)


# ------------------------------------------------------------------ (de)serialisation

def frame_to_arrays(frame, prefix="frame"):
    """Flattens a Frame into a dict of numpy arrays (for .npz fixtures)."""
    out = {prefix + "/size": np.array([frame.width, frame.height], np.int64),
           prefix + "/ndraws": np.array([len(frame.draws)], np.int64)}
    if frame.clear_color is not None:
        out[prefix + "/clear_color"] = np.array(frame.clear_color, np.float32)
    if frame.clear_depth is not None:
        out[prefix + "/clear_depth"] = np.array([frame.clear_depth], np.float32)
    stored = {}   # texture already written: id(data) -> (draw, slot); later uses refer to it
    for i, d in enumerate(frame.draws):
        p = "%s/draw%d/" % (prefix, i)
        out[p + "ints"] = np.array([d.vs, d.ps, d.index_count, d.cull, d.depth_func, d.start_index, d.base_vertex],
                                   np.int64)
        out[p + "vb"] = d.vb
        if d.ib is not None:
            out[p + "ib"] = d.ib
        if d.cb is not None:
            out[p + "cb"] = d.cb
        out[p + "viewport"] = np.array(d.viewport, np.float32)
        for slot, name in enumerate(("vs_tex", "ps_tex")):
            t = getattr(d, name)
            if t is None:
                continue
            if id(t.data) in stored:
                out[p + name + "_same_as"] = np.array(stored[id(t.data)], np.int64)
                continue
            stored[id(t.data)] = (i, slot)
            out[p + name] = t.data
            out[p + name + "_fmt"] = np.array([t.format], np.int64)
    return out


def frame_from_arrays(z, prefix="frame"):
    w, h = (int(v) for v in z[prefix + "/size"])
    cc = tuple(float(v) for v in z[prefix + "/clear_color"]) if prefix + "/clear_color" in z else None
    cd = float(z[prefix + "/clear_depth"][0]) if prefix + "/clear_depth" in z else None
    fr = Frame(w, h, [], clear_color=cc, clear_depth=cd)
    texcache = {}
    for i in range(int(z[prefix + "/ndraws"][0])):
        p = "%s/draw%d/" % (prefix, i)
        vs, ps, n, cull, df, si, bv = (int(v) for v in z[p + "ints"])
        texs = {}
        for name in ("vs_tex", "ps_tex"):
            if p + name + "_same_as" in z:   # the texture of an earlier draw's slot
                j, slot = (int(v) for v in z[p + name + "_same_as"])
                texs[name] = getattr(fr.draws[j], ("vs_tex", "ps_tex")[slot])
            elif p + name in z:
                data = z[p + name]
                key = (data.shape, data.dtype.str, hash(data.tobytes()))
                if key not in texcache:
                    texcache[key] = Texture(data, int(z[p + name + "_fmt"][0]))
                texs[name] = texcache[key]
        fr.draws.append(Draw(vs, ps, z[p + "vb"], z[p + "ib"] if p + "ib" in z else None, n,
                             cb=z[p + "cb"] if p + "cb" in z else None, vs_tex=texs.get("vs_tex"),
                             ps_tex=texs.get("ps_tex"), viewport=tuple(float(v) for v in z[p + "viewport"]),
                             cull=cull, depth_func=df, start_index=si, base_vertex=bv))
    return fr


# ------------------------------------------------------------------ differentiable scenes

def diff_scene(seed=4, n_views=16, size=512, freq=50, tex_size=1024, heightfield_cells=None):
    """The differentiable configuration: a geodesic sphere of 20*freq^2 triangles (freq 50: 50,000)
    with planar UVs (0.5 + 0.5 (x, y)) or, with heightfield_cells, a heightfield of 2*cells^2
    triangles with its grid UVs; per-vertex colours U(0,1), an RGBA32F texture U(0,1); per view a seeded rotation and perspective projection into the
    passthrough screen space [0,1]^2 (x, y) with depth z in (0,1). Returns a dict of arrays."""
    rng = np.random.default_rng(seed)
    if heightfield_cells:
        v, faces = heightfield(rng, heightfield_cells, 2.0, 0.4)
        P = v[:, 0:3].astype(np.float64)
        uv = v[:, 6:8].astype(np.float32)
    else:
        dirs, faces = geodesic_sphere(freq)
        P = dirs
        # a seam-free planar map: the spherical map's seam triangles interpolate across the whole
        # texture (and its poles leave u undefined), which makes their texel lookups, and any
        # gradient through them, ill-conditioned in single precision
        uv = 0.5 + 0.5 * dirs[:, 0:2]
    n = len(P)
    col = rng.random((n, 3)).astype(np.float32)
    tex = rng.random((tex_size, tex_size, 4)).astype(np.float32)
    pos = np.zeros((n_views, n, 2), np.float32)
    z = np.zeros((n_views, n), np.float32)
    f = 1.0 / np.tan(np.radians(50.0) / 2)
    for k in range(n_views):
        if heightfield_cells:
            # a camera over the heightfield at a seeded azimuth and an elevation of 45-90 degrees,
            # 2.4 from its centre, looking at it (the grid spans most of the view)
            az, el = rng.uniform(0, 2 * np.pi), np.radians(rng.uniform(45.0, 90.0))
            cam = 2.4 * np.array([np.cos(el) * np.cos(az), np.cos(el) * np.sin(az), np.sin(el)])
            fwd = -cam / np.linalg.norm(cam)
            right = np.array([-np.sin(az), np.cos(az), 0.0])
            up = np.cross(right, fwd)
            D = P - cam
            Q = np.stack([D @ right, D @ up, D @ fwd], axis=1)
            depth, dist = Q[:, 2], 2.4
        else:
            q = rng.standard_normal(4)
            q /= np.linalg.norm(q)
            a, b, c, d = q
            R = np.array([[a * a + b * b - c * c - d * d, 2 * (b * c - a * d), 2 * (b * d + a * c)],
                          [2 * (b * c + a * d), a * a - b * b + c * c - d * d, 2 * (c * d - a * b)],
                          [2 * (b * d - a * c), 2 * (c * d + a * b), a * a - b * b - c * c + d * d]])
            Q = P @ R.T
            dist = 3.0
            depth = Q[:, 2] + dist
        pos[k, :, 0] = 0.5 + 0.5 * f * Q[:, 0] / depth
        pos[k, :, 1] = 0.5 + 0.5 * f * Q[:, 1] / depth
        z[k] = (depth / (dist + 2.0)).astype(np.float32)
    return {"ib": faces.astype(np.uint32), "col": col, "uv": uv.astype(np.float32), "tex": tex, "pos": pos, "z": z,
            "width": size, "height": size}


def diff_frames(scene, pos=None, col=None, uv=None, shade=True):
    """One frame per view drawing the scene with MLV_VS_PASSTHROUGH_UV + COLOR_TIMES_TEXEL (depth LESS
    cleared to 1, no culling): the exact rasteriser's visibility for the differentiable path.
    shade=False: the null pixel shader and no colour clear (depth and visibility only)."""
    pos = scene["pos"] if pos is None else pos
    col = scene["col"] if col is None else col
    uv = scene["uv"] if uv is None else uv
    tex = Texture(scene["tex"], FMT_RGBA32F)
    ib = pad_indices(scene["ib"])
    n_tris = len(scene["ib"])
    frames = []
    for k in range(pos.shape[0]):
        vb = np.concatenate([pos[k], scene["z"][k][:, None], col, uv], axis=1).astype(np.float32)
        d = Draw(VS_PASSTHROUGH_UV, PS_COLOR_TIMES_TEXEL if shade else PS_NONE, vb, ib, 3 * n_tris,
                 ps_tex=tex if shade else None,
                 viewport=(0.0, 0.0, float(scene["width"]), float(scene["height"]), 0.0, 1.0),
                 cull=CULL_NONE, depth_func=DEPTH_LESS)
        frames.append(Frame(scene["width"], scene["height"], [d], clear_color=(0.0, 0.0, 0.0, 0.0) if shade else None,
                            clear_depth=1.0))
    return frames
