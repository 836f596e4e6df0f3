"""ctypes front ends for the two CPU checkers (TEST INFRASTRUCTURE ONLY).

- `render_oracle(frame)` drives the C restatement in oracle.c (built by oracle/build.py).
- `render_reference(frame)` drives the reference's own pipeline core, compiled headless from its
  sources by oracle/ref_build.py into oracle/_ref/ (x86-64 only; absent on other hosts).

Both take the `Frame` description from `malevich_gb300.scenes` (a list of draws with their
pipeline state), the same description the GPU path renders, and return numpy arrays.
Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import this module.
"""
import ctypes
import glob
import os

import numpy as np

from . import build as _build

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(HERE, "_ref")

_u32p = ctypes.POINTER(ctypes.c_uint32)
_f32p = ctypes.POINTER(ctypes.c_float)


class OrcTexture(ctypes.Structure):
    _fields_ = [("data", ctypes.c_void_p), ("width", ctypes.c_uint32), ("height", ctypes.c_uint32),
                ("format", ctypes.c_int32)]


class OrcDraw(ctypes.Structure):
    _fields_ = [("vs", ctypes.c_int32), ("ps", ctypes.c_int32), ("vb", ctypes.c_void_p),
                ("vb_stride", ctypes.c_uint32), ("vertex_count", ctypes.c_uint32),
                ("ib", ctypes.c_void_p), ("index_count", ctypes.c_uint32), ("start_index", ctypes.c_uint32),
                ("base_vertex", ctypes.c_int32), ("cb", ctypes.c_void_p), ("vs_tex", OrcTexture),
                ("ps_tex", OrcTexture), ("viewport", ctypes.c_float * 6), ("cull", ctypes.c_int32),
                ("depth_func", ctypes.c_int32), ("fill_rule", ctypes.c_int32), ("sample_center", ctypes.c_int32)]


class OrcTarget(ctypes.Structure):
    _fields_ = [("color", ctypes.c_void_p), ("depth", ctypes.c_void_p), ("width", ctypes.c_uint32),
                ("height", ctypes.c_uint32), ("tile_min", ctypes.c_void_p), ("tile_max", ctypes.c_void_p),
                ("vis_tri", ctypes.c_void_p), ("vis_draw", ctypes.c_void_p), ("vis_bary", ctypes.c_void_p),
                ("vis_prim", ctypes.c_void_p)]


class OrcStats(ctypes.Structure):
    _fields_ = [("vertex_count", ctypes.c_uint64), ("input_triangle_count", ctypes.c_uint64),
                ("assembled_triangle_count", ctypes.c_uint64), ("active_bin_count", ctypes.c_uint64),
                ("total_triangle_count_in_bins", ctypes.c_uint64), ("fragments_written", ctypes.c_uint64),
                ("clipped_triangle_count", ctypes.c_uint64)]


class OrcCapture(ctypes.Structure):
    _fields_ = [("n_tris", ctypes.c_uint32), ("edges", ctypes.c_void_p), ("rw", ctypes.c_void_p),
                ("inv_area", ctypes.c_void_p), ("depth_bound", ctypes.c_void_p), ("bounds", ctypes.c_void_p),
                ("attrs", ctypes.c_void_p), ("n_infos", ctypes.c_uint32), ("info_bin", ctypes.c_void_p),
                ("info_tri", ctypes.c_void_p), ("info_mask", ctypes.c_void_p)]


_orc = None


def oracle_lib():
    global _orc
    if _orc is None:
        lib = ctypes.CDLL(_build.build_oracle())
        lib.orc_draw_indexed.argtypes = [ctypes.POINTER(OrcTarget), ctypes.POINTER(OrcDraw), ctypes.c_uint32,
                                         ctypes.POINTER(OrcStats), ctypes.POINTER(OrcCapture)]
        lib.orc_draw_indexed.restype = ctypes.c_int
        lib.orc_clear_color.argtypes = [ctypes.POINTER(OrcTarget), _f32p]
        lib.orc_clear_depth.argtypes = [ctypes.POINTER(OrcTarget), ctypes.c_float]
        lib.orc_capture_free.argtypes = [ctypes.POINTER(OrcCapture)]
        lib.orc_encode_clear_color.argtypes = [_f32p]
        lib.orc_encode_clear_color.restype = ctypes.c_uint32
        lib.orc_cvt_rn.argtypes = [ctypes.c_float]
        lib.orc_cvt_rn.restype = ctypes.c_int32
        lib.orc_snap.argtypes = [ctypes.c_float]
        lib.orc_snap.restype = ctypes.c_int32
        lib.orc_run_vs.argtypes = [ctypes.c_int32, _f32p, _f32p, ctypes.POINTER(OrcTexture), _f32p]
        lib.orc_run_ps.argtypes = [ctypes.c_int32, _f32p, ctypes.POINTER(OrcTexture), _f32p]
        lib.orc_set_threads.argtypes = [ctypes.c_int]
        lib.orc_max_threads.restype = ctypes.c_int
        _orc = lib
    return _orc


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p) if a is not None else None


def _tex(t, keep):
    if t is None:
        return OrcTexture(None, 0, 0, 0)
    data = np.ascontiguousarray(t.data)
    keep.append(data)
    return OrcTexture(_ptr(data), t.width, t.height, t.format)


def _draw_struct(d, keep):
    vb = np.ascontiguousarray(d.vb_bytes())
    keep.append(vb)
    ib = None
    if d.ib is not None:
        ib = np.ascontiguousarray(d.ib, dtype=np.uint32)
        keep.append(ib)
    cb = None
    if d.cb is not None:
        cb = np.ascontiguousarray(d.cb, dtype=np.float32)
        keep.append(cb)
    s = OrcDraw()
    s.vs, s.ps = d.vs, d.ps
    s.vb = _ptr(vb)
    s.vb_stride = d.vb_stride
    s.vertex_count = d.vertex_count()
    s.ib = _ptr(ib)
    s.index_count = d.index_count
    s.start_index = d.start_index
    s.base_vertex = d.base_vertex
    s.fill_rule = getattr(d, "fill_rule", 0)
    s.sample_center = getattr(d, "sample_center", 0)
    s.cb = _ptr(cb)
    s.vs_tex = _tex(d.vs_tex, keep)
    s.ps_tex = _tex(d.ps_tex, keep)
    s.viewport = (ctypes.c_float * 6)(*d.viewport)
    s.cull = d.cull
    s.depth_func = d.depth_func
    return s


def render_oracle(frame, capture=False, threads=None):
    """Render `frame` on the CPU restatement. Returns a dict of numpy arrays and stats; with
    capture=True also the per-draw assembled triangles and TileInfo masks."""
    lib = oracle_lib()
    if threads is not None:
        lib.orc_set_threads(int(threads))
    w, h = frame.width, frame.height
    ntx, nty = (w + 7) // 8, (h + 7) // 8
    color = np.zeros((h, w), np.uint32)
    depth = np.zeros((h, w), np.float32)
    tile_min = np.zeros(ntx * nty, np.float32)
    tile_max = np.ones(ntx * nty, np.float32)
    vis_tri = np.full((h, w), 0xFFFFFFFF, np.uint32)
    vis_draw = np.full((h, w), 0xFFFFFFFF, np.uint32)
    vis_bary = np.zeros((h, w, 2), np.float32)
    vis_prim = np.full((h, w), 0xFFFFFFFF, np.uint32)
    if frame.initial_color is not None:
        color[...] = frame.initial_color
    if frame.initial_depth is not None:
        depth[...] = frame.initial_depth
    tgt = OrcTarget(_ptr(color), _ptr(depth), w, h, _ptr(tile_min), _ptr(tile_max), _ptr(vis_tri),
                    _ptr(vis_draw), _ptr(vis_bary), _ptr(vis_prim))
    if frame.clear_color is not None:
        lib.orc_clear_color(ctypes.byref(tgt), (ctypes.c_float * 4)(*frame.clear_color))
    if frame.clear_depth is not None:
        lib.orc_clear_depth(ctypes.byref(tgt), ctypes.c_float(frame.clear_depth))
    stats = OrcStats()
    caps = []
    for seq, d in enumerate(frame.draws):
        keep = []
        ds = _draw_struct(d, keep)
        cap = OrcCapture() if capture else None
        rc = lib.orc_draw_indexed(ctypes.byref(tgt), ctypes.byref(ds), seq, ctypes.byref(stats),
                                  ctypes.byref(cap) if cap is not None else None)
        if rc != 0:
            raise ValueError("oracle rejected draw %d" % seq)
        if cap is not None:
            caps.append(_read_capture(cap))
            lib.orc_capture_free(ctypes.byref(cap))
    return {
        "color": color, "depth": depth, "vis_tri": vis_tri, "vis_draw": vis_draw, "vis_bary": vis_bary,
        "vis_prim": vis_prim, "tile_min": tile_min, "tile_max": tile_max,
        "stats": {k: int(getattr(stats, k)) for k, _ in OrcStats._fields_},
        "captures": caps,
    }


def _arr(ptr, n, dtype):
    if n == 0 or not ptr:
        return np.zeros(0, dtype)
    ct = np.ctypeslib.as_ctypes_type(dtype)
    return np.ctypeslib.as_array(ctypes.cast(ptr, ctypes.POINTER(ct)), shape=(n,)).copy()


def _read_capture(c):
    n, m = c.n_tris, c.n_infos
    return {
        "edges": _arr(c.edges, 9 * n, np.int32).reshape(n, 3, 3),
        "rw": _arr(c.rw, 3 * n, np.float32).reshape(n, 3),
        "inv_area": _arr(c.inv_area, n, np.float32),
        "depth_bound": _arr(c.depth_bound, n, np.float32),
        "bounds": _arr(c.bounds, 4 * n, np.int32).reshape(n, 4),
        "attrs": _arr(c.attrs, 36 * n, np.float32).reshape(n, 3, 3, 4),
        "info_bin": _arr(c.info_bin, m, np.uint32),
        "info_tri": _arr(c.info_tri, m, np.uint32),
        "info_mask": _arr(c.info_mask, m, np.uint64),
    }


# ------------------------------------------------------------------ the reference itself

_ref_libs = {}


def reference_available(width, height):
    return os.path.exists(os.path.join(REF_DIR, "libmalevich_ref_%dx%d.so" % (width, height)))


def reference_sizes():
    out = []
    for p in glob.glob(os.path.join(REF_DIR, "libmalevich_ref_*x*.so")):
        wh = os.path.basename(p)[len("libmalevich_ref_"):-3]
        w, h = wh.split("x")
        out.append((int(w), int(h)))
    return out


def reference_lib(width, height):
    key = (width, height)
    if key not in _ref_libs:
        path = os.path.join(REF_DIR, "libmalevich_ref_%dx%d.so" % key)
        if not os.path.exists(path):
            raise FileNotFoundError(path)
        lib = ctypes.CDLL(path)
        lib.ref_clear.argtypes = [_f32p, ctypes.c_float]
        lib.ref_set_viewport.argtypes = [_f32p]
        lib.ref_set_shaders.argtypes = [ctypes.c_int, ctypes.c_int]
        lib.ref_set_cb.argtypes = [ctypes.c_void_p]
        lib.ref_set_vs_texture.argtypes = [ctypes.c_void_p, ctypes.c_uint, ctypes.c_uint]
        lib.ref_set_ps_texture.argtypes = [ctypes.c_void_p, ctypes.c_uint, ctypes.c_uint]
        lib.ref_draw_indexed.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint]
        lib.ref_set_threads.argtypes = [ctypes.c_int]
        lib.ref_get_stats.argtypes = [_u32p]
        lib.ref_color.restype = ctypes.c_void_p
        lib.ref_depth.restype = ctypes.c_void_p
        lib.ref_ids.restype = ctypes.c_void_p
        lib.ref_tile_min.restype = ctypes.c_void_p
        lib.ref_last_triangle_count.restype = ctypes.c_uint
        lib.ref_last_tile_info_count.restype = ctypes.c_uint
        lib.ref_last_triangles.argtypes = [ctypes.c_void_p] * 6
        lib.ref_last_tile_infos.argtypes = [ctypes.c_void_p] * 3
        _ref_libs[key] = lib
    return _ref_libs[key]


def _ref_texture(t, keep):
    """The reference fetches RGBA8 as u32 and float textures as float4 (common_shader_core.h:26-53);
    an RGBA16F texture is handed to it widened to float, which is exact."""
    if t is None:
        return None, 0, 0
    data = t.data
    if t.format == 2:
        data = data.astype(np.float32)
    data = np.ascontiguousarray(data)
    keep.append(data)
    return _ptr(data), t.width, t.height


def render_reference(frame, capture=False, threads=1):
    """Render `frame` on the reference's own pipeline core (reference-native modes only: depth
    GREATER_EQUAL, back-face culling, 32-byte vertices, no start/base offsets, index counts that
    are a multiple of 8). threads=1 gives the serial primitive order the parity tests use."""
    lib = reference_lib(frame.width, frame.height)
    lib.ref_set_threads(int(threads))
    w, h = frame.width, frame.height
    for d in frame.draws:
        if d.depth_func != 0 or d.cull != 1 or d.vb_stride != 32 or d.start_index or d.base_vertex:
            raise ValueError("draw uses a mode the reference does not have")
        if d.index_count % 8 or d.ib is None or d.vs > 4 or d.ps > 3:
            raise ValueError("draw uses a mode the reference does not have")
    lib.ref_clear((ctypes.c_float * 4)(*frame.clear_color), ctypes.c_float(frame.clear_depth))
    lib.ref_reset_stats()
    caps = []
    for d in frame.draws:
        keep = []
        lib.ref_set_viewport((ctypes.c_float * 6)(*d.viewport))
        if lib.ref_set_shaders(d.vs, d.ps) != 0:
            raise ValueError("unknown shader")
        cb = np.zeros(48, np.float32) if d.cb is None else np.ascontiguousarray(d.cb, np.float32)
        lib.ref_set_cb(_ptr(cb))
        p, tw, th = _ref_texture(d.vs_tex, keep)
        lib.ref_set_vs_texture(p, tw, th)
        p, tw, th = _ref_texture(d.ps_tex, keep)
        lib.ref_set_ps_texture(p, tw, th)
        vb = np.ascontiguousarray(d.vb_bytes())
        ib = np.ascontiguousarray(d.ib, np.uint32)
        lib.ref_draw_indexed(_ptr(vb), _ptr(ib), d.index_count)
        if capture:
            n = lib.ref_last_triangle_count()
            edges = np.zeros((max(n, 1), 3, 3), np.int32)
            rw = np.zeros((max(n, 1), 3), np.float32)
            inv_area = np.zeros(max(n, 1), np.float32)
            maxd = np.zeros(max(n, 1), np.float32)
            bounds = np.zeros((max(n, 1), 4), np.int32)
            attrs = np.zeros((max(n, 1), 3, 3, 4), np.float32)
            lib.ref_last_triangles(_ptr(edges), _ptr(rw), _ptr(inv_area), _ptr(maxd), _ptr(bounds), _ptr(attrs))
            m = lib.ref_last_tile_info_count()
            ib_ = np.zeros(max(m, 1), np.uint32)
            it_ = np.zeros(max(m, 1), np.uint32)
            im_ = np.zeros(max(m, 1), np.uint64)
            lib.ref_last_tile_infos(_ptr(ib_), _ptr(it_), _ptr(im_))
            caps.append({"edges": edges[:n], "rw": rw[:n], "inv_area": inv_area[:n], "depth_bound": maxd[:n],
                         "bounds": bounds[:n], "attrs": attrs[:n], "info_bin": ib_[:m], "info_tri": it_[:m],
                         "info_mask": im_[:m]})
    st = (ctypes.c_uint32 * 5)()
    lib.ref_get_stats(st)
    color = _arr(lib.ref_color(), w * h, np.uint32).reshape(h, w)
    depth = _arr(lib.ref_depth(), w * h, np.float32).reshape(h, w)
    ids = _arr(lib.ref_ids(), w * h, np.uint64).reshape(h, w)
    vis_tri = (ids & 0xFFFFFFFF).astype(np.uint32)
    vis_draw = (ids >> 32).astype(np.uint32)
    ntx, nty = w // 8, h // 8
    tile_min = _arr(lib.ref_tile_min(), ntx * nty, np.float32)
    return {
        "color": color, "depth": depth, "vis_tri": vis_tri, "vis_draw": vis_draw, "tile_min": tile_min,
        "stats": {"vertex_count": st[0], "input_triangle_count": st[1], "assembled_triangle_count": st[2],
                  "active_bin_count": st[3], "total_triangle_count_in_bins": st[4]},
        "captures": caps,
    }


# ------------------------------------------------------------------ differentiable model (FP64)

class OrcDiffScene(ctypes.Structure):
    _fields_ = [("n_verts", ctypes.c_uint32), ("n_tris", ctypes.c_uint32), ("ib", ctypes.c_void_p),
                ("col", ctypes.c_void_p), ("uv", ctypes.c_void_p), ("tex", ctypes.c_void_p),
                ("tw", ctypes.c_uint32), ("th", ctypes.c_uint32)]


class OrcDiffView(ctypes.Structure):
    _fields_ = [("width", ctypes.c_uint32), ("height", ctypes.c_uint32), ("pos", ctypes.c_void_p),
                ("prim", ctypes.c_void_p), ("target", ctypes.c_void_p), ("cells", ctypes.c_void_p)]


class DiffModel:
    """FP64 differentiable shading (oracle_adjoint.c) over fixed visibility: loss, image, adjoint."""

    def __init__(self, ib, col, uv, tex, views):
        """ib (T,3) uint32; col (N,3); uv (N,2); tex (th,tw,4); views: list of dicts with keys
        width, height, pos (N,2), prim (H,W) uint32, target (H,W,3)."""
        self.lib = oracle_lib()
        self.lib.orc_diff_loss.restype = ctypes.c_double
        self.lib.orc_diff_loss.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint32, ctypes.c_void_p]
        self.lib.orc_diff_grad.argtypes = [ctypes.c_void_p] * 2 + [ctypes.c_uint32] + [ctypes.c_void_p] * 3
        self.lib.orc_diff_cells.argtypes = [ctypes.c_void_p] * 3
        self.lib.orc_diff_cells_f32.argtypes = [ctypes.c_void_p] * 3
        self.ib = np.ascontiguousarray(ib, np.uint32)
        self.col = np.ascontiguousarray(col, np.float64)
        self.uv = np.ascontiguousarray(uv, np.float64)
        self.tex = np.ascontiguousarray(tex, np.float64)
        self.views = [dict(v) for v in views]
        for v in self.views:
            v["pos"] = np.ascontiguousarray(v["pos"], np.float64)
            v["prim"] = np.ascontiguousarray(v["prim"], np.uint32)
            v["target"] = np.ascontiguousarray(v["target"], np.float64)
            v["cells"] = None

    def _structs(self):
        sc = OrcDiffScene(len(self.col), len(self.ib), _ptr(self.ib), _ptr(self.col), _ptr(self.uv), _ptr(self.tex),
                          self.tex.shape[1], self.tex.shape[0])
        arr = (OrcDiffView * len(self.views))()
        for i, v in enumerate(self.views):
            arr[i] = OrcDiffView(v["width"], v["height"], _ptr(v["pos"]), _ptr(v["prim"]), _ptr(v["target"]),
                                 _ptr(v["cells"]) if v["cells"] is not None else None)
        return sc, arr

    def freeze_cells(self, rule="f64"):
        """Holds each pixel's bilinear cell fixed (the loss becomes smooth in the positions).
        rule "f64" picks the cells in FP64; "f32" with the GPU kernels' single-precision sequence."""
        fn = {"f64": self.lib.orc_diff_cells, "f32": self.lib.orc_diff_cells_f32}[rule]
        sc, arr = self._structs()
        for i, v in enumerate(self.views):
            cells = np.zeros((v["height"], v["width"], 2), np.int32)
            fn(ctypes.byref(sc), ctypes.byref(arr[i]), _ptr(cells))
            v["cells"] = cells

    def loss(self, image=False):
        sc, arr = self._structs()
        img = None
        if image:
            img = np.zeros((len(self.views), self.views[0]["height"], self.views[0]["width"], 3), np.float64)
        val = self.lib.orc_diff_loss(ctypes.byref(sc), arr, len(self.views), _ptr(img) if img is not None else None)
        return (val, img) if image else val

    def grad(self):
        sc, arr = self._structs()
        g_col = np.zeros_like(self.col)
        g_tex = np.zeros_like(self.tex)
        g_pos = np.zeros((len(self.views),) + self.col.shape[:1] + (2,), np.float64)
        self.lib.orc_diff_grad(ctypes.byref(sc), arr, len(self.views), _ptr(g_col), _ptr(g_tex), _ptr(g_pos))
        return g_col, g_tex, g_pos
