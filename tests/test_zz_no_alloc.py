"""The allocation-free entry point, mlv_draw_indexed_noalloc, against mlv_draw_indexed.

It exists for callers that cannot call cudaMalloc (a host that owns all device memory through its
own allocator, a render loop with a no-allocation rule, work issued while another component
captures a CUDA graph): it draws with the same kernels, keeping its scratch in one static device
array. This test allocates the inputs and outputs itself, as such a caller would, then renders
the same frame twice in a row through the C ABI and compares both results with the normal path:
depth, bit for bit; colour within the +-1 LSB the other parity tests use. It also drives the
overflows only the device can detect (more (tile, triangle) pairs than the scratch holds: the call
must report MLV_ERROR_CAPACITY_EXCEEDED, leave the render target unwritten, and the next call must
work), the non-indexed path, per-index shading of vertex buffers beyond the scratch's vertex limit
and the null pixel shader. This file is collected last so that a failure here comes after every
other test has run.
"""
import ctypes

import numpy as np
import pytest

from helpers import assert_bits_equal, assert_color_close
from malevich_gb300 import api, build, scenes

pytestmark = pytest.mark.gpu


class NoallocTexture(ctypes.Structure):
    _fields_ = [("data", ctypes.c_void_p), ("width", ctypes.c_uint32), ("height", ctypes.c_uint32),
                ("format", ctypes.c_int)]


class NoallocDraw(ctypes.Structure):
    _fields_ = [("vertex_buffer", ctypes.c_void_p), ("vertex_stride", ctypes.c_uint32),
                ("vertex_count", ctypes.c_uint32), ("index_buffer", ctypes.c_void_p),
                ("index_buffer_count", ctypes.c_uint32), ("index_count", ctypes.c_uint32),
                ("start_index", ctypes.c_uint32), ("base_vertex", ctypes.c_int32),
                ("vs", ctypes.c_int), ("ps", ctypes.c_int), ("per_frame_cb", ctypes.c_void_p),
                ("vs_texture", NoallocTexture), ("ps_texture", NoallocTexture), ("viewport", api.Viewport),
                ("cull_mode", ctypes.c_int), ("depth_func", ctypes.c_int), ("color", ctypes.c_void_p),
                ("depth", ctypes.c_void_p), ("tile_min", ctypes.c_void_p), ("tile_max", ctypes.c_void_p),
                ("width", ctypes.c_uint32), ("height", ctypes.c_uint32), ("flags", ctypes.c_uint32)]


RESET_HIZ = 0x1
MAX_TRIANGLES = 32768
MAX_VERTICES = 32768
MAX_BIN_ENTRIES = 131072
INVALID_ARG = 1
CAPACITY_EXCEEDED = 3


def _texture(renderer, t):
    if t is None:
        return NoallocTexture(None, 0, 0, 0)
    tex = renderer._texture(t)
    return NoallocTexture(tex.device_pointer(), tex.width, tex.height, tex.format)


def _describe(renderer, frame, d, rt, ds, tile_min, tile_max, keep, flags):
    """The caller-side descriptor of one draw: inputs, outputs and state, all caller-owned."""
    cb = np.ascontiguousarray(d.cb, np.float32) if d.cb is not None else None
    keep.append(cb)
    nd = NoallocDraw()
    nd.vertex_buffer = renderer._buffer(d.vb, api.BIND_VERTEX_BUFFER).device_pointer()
    nd.vertex_stride = d.vb_stride
    nd.vertex_count = d.vertex_count()
    nd.index_buffer = renderer._buffer(d.ib, api.BIND_INDEX_BUFFER).device_pointer() if d.ib is not None else None
    nd.index_buffer_count = len(d.ib) if d.ib is not None else 0
    nd.index_count, nd.start_index, nd.base_vertex = d.index_count, d.start_index, d.base_vertex
    nd.vs, nd.ps = d.vs, d.ps
    nd.per_frame_cb = cb.ctypes.data_as(ctypes.c_void_p) if cb is not None else None
    nd.vs_texture = _texture(renderer, d.vs_tex)
    nd.ps_texture = _texture(renderer, d.ps_tex)
    nd.viewport = api.Viewport(*d.viewport)
    nd.cull_mode = {scenes.CULL_NONE: api.CULL_NONE, scenes.CULL_BACK: api.CULL_BACK,
                    scenes.CULL_FRONT: api.CULL_FRONT}[d.cull]
    nd.depth_func = api.COMPARISON_LESS if d.depth_func == scenes.DEPTH_LESS else api.COMPARISON_GREATER_EQUAL
    nd.color, nd.depth = rt.device_pointer(), ds.device_pointer()
    nd.tile_min, nd.tile_max = tile_min.data_ptr(), tile_max.data_ptr()
    nd.width, nd.height = frame.width, frame.height
    nd.flags = flags
    return nd


def _render_noalloc(lib, dev, renderer, frame, rt, ds, tile_min, tile_max, keep, expect=0):
    ctx = dev.immediate
    ctx.clear_render_target(rt, frame.clear_color)
    ctx.clear_depth(ds, frame.clear_depth)
    ctx.finish()
    for k, d in enumerate(frame.draws):
        nd = _describe(renderer, frame, d, rt, ds, tile_min, tile_max, keep, RESET_HIZ if k == 0 else 0)
        status = lib.mlv_draw_indexed_noalloc(ctypes.byref(nd), None)
        assert status == expect, lib.mlv_get_last_error_string()
    return ctx.read_texture(rt), ctx.read_texture(ds)


class _Targets:
    """A caller's render target, depth target and hierarchical-Z arrays for one frame size."""

    def __init__(self, dev, frame):
        import torch
        self.rt = api.Texture2D(dev, frame.width, frame.height, api.FORMAT_R8G8B8A8_UNORM, bind=api.BIND_RENDER_TARGET)
        self.ds = api.Texture2D(dev, frame.width, frame.height, api.FORMAT_D32_FLOAT, bind=api.BIND_DEPTH_STENCIL)
        tiles = ((frame.width + 7) // 8) * ((frame.height + 7) // 8)
        self.tile_min = torch.zeros(tiles, dtype=torch.float32, device="cuda")
        self.tile_max = torch.ones(tiles, dtype=torch.float32, device="cuda")

    def render(self, lib, dev, renderer, frame, keep, expect=0):
        return _render_noalloc(lib, dev, renderer, frame, self.rt, self.ds, self.tile_min, self.tile_max, keep,
                               expect)

    def destroy(self):
        self.rt.destroy()
        self.ds.destroy()


def _compare_two_calls(lib, dev, frame):
    keep = []
    ref = api.FrameRenderer(dev, frame)
    ref.render_per_draw()
    want = ref.read(0)
    tg = _Targets(dev, frame)
    for call in range(2):
        color, depth = tg.render(lib, dev, ref, frame, keep)
        assert_bits_equal(depth, want["depth"], "depth (call %d)" % call)
        assert_color_close(color, want["color"])
    tg.destroy()
    ref.destroy()


@pytest.mark.parametrize("native", [True, False])
def test_noalloc_matches_draw_indexed_on_two_calls(native):
    build.build()
    lib = api.load_library()
    dev = api.Device(0)
    try:
        frame = scenes.small_scene(21, 96, 80, vs=scenes.VS_BASIC, ps=scenes.PS_BASIC, n_objects=3, native=native)
        frame.draws += scenes.small_scene(22, 96, 80, vs=scenes.VS_VERTEX_LIGHTING, ps=scenes.PS_ENV_LIGHTING,
                                          n_objects=2, native=native, inside=True).draws
        _compare_two_calls(lib, dev, frame)
    finally:
        dev.destroy()


def _variant(kind):
    frame = scenes.small_scene(23, 88, 72, vs=scenes.VS_BASIC, ps=scenes.PS_BASIC, n_objects=3, native=True)
    out = []
    for d in frame.draws:
        if kind == "non_indexed":
            # de-indexed vertices, drawn with implicit indices (index_buffer NULL)
            vb = np.ascontiguousarray(d.vb[d.ib[:d.index_count]])
            out.append(scenes.Draw(d.vs, d.ps, vb, None, d.index_count, cb=d.cb, vs_tex=d.vs_tex, ps_tex=d.ps_tex,
                                   viewport=d.viewport, depth_func=d.depth_func))
        elif kind == "large_vertex_buffer":
            # more vertices than the scratch shades once each: the call shades them per index
            pad = np.zeros((MAX_VERTICES + 1000 - len(d.vb), d.vb.shape[1]), np.float32)
            vb = np.ascontiguousarray(np.concatenate([d.vb, pad]))
            out.append(scenes.Draw(d.vs, d.ps, vb, d.ib, d.index_count, cb=d.cb, vs_tex=d.vs_tex, ps_tex=d.ps_tex,
                                   viewport=d.viewport, depth_func=d.depth_func))
        elif kind == "null_ps":
            out.append(scenes.Draw(d.vs, scenes.PS_NONE, d.vb, d.ib, d.index_count, cb=d.cb, vs_tex=d.vs_tex,
                                   ps_tex=None, viewport=d.viewport, depth_func=d.depth_func))
    frame.draws = out
    return frame


@pytest.mark.parametrize("kind", ["non_indexed", "large_vertex_buffer", "null_ps"])
def test_noalloc_variants_match_draw_indexed(kind):
    build.build()
    lib = api.load_library()
    dev = api.Device(0)
    try:
        frame = _variant(kind)
        if kind == "large_vertex_buffer":
            assert all(d.vertex_count() > MAX_VERTICES for d in frame.draws)
        _compare_two_calls(lib, dev, frame)
    finally:
        dev.destroy()


def _full_screen_frame(n_tris, size=1024):
    """n_tris triangles that each span the whole size x size target (passthrough positions in
    [0,1] screen space), so that every one of them is binned into every 8x8 tile."""
    corners = [((0.0, 0.0), (1.0, 0.0), (0.0, 1.0)), ((1.0, 0.0), (1.0, 1.0), (0.0, 1.0)),
               ((0.0, 1.0), (1.0, 1.0), (1.0, 0.0)), ((0.0, 0.0), (1.0, 1.0), (0.0, 1.0))]
    vb = []
    for t in range(n_tris):
        z = 0.1 + 0.8 * t / max(1, n_tris)
        for (x, y) in corners[t % len(corners)]:
            vb.append([x, y, z, 1.0, 0.2 + 0.05 * t, 0.5, 0.7, 0.0])
    vb = np.asarray(vb, np.float32)
    ib = np.arange(len(vb), dtype=np.uint32)
    vp = (0.0, 0.0, float(size), float(size), 0.0, 1.0)
    d = scenes.Draw(scenes.VS_PASSTHROUGH, scenes.PS_PASSTHROUGH, vb, ib, len(ib), viewport=vp, cull=scenes.CULL_NONE,
                    depth_func=scenes.DEPTH_GREATER_EQUAL)
    return scenes.Frame(size, size, [d], clear_color=(0.25, 0.5, 0.75, 1.0), clear_depth=0.0)


def test_noalloc_bin_overflow_reports_and_recovers():
    """More (tile, triangle) pairs than MLV_NOALLOC_MAX_BIN_ENTRIES, which only the device can
    count: the call returns MLV_ERROR_CAPACITY_EXCEEDED and leaves the render target as cleared;
    the next call, within the limits, matches mlv_draw_indexed."""
    build.build()
    lib = api.load_library()
    dev = api.Device(0)
    keep = []
    try:
        big = _full_screen_frame(9)
        tiles = (big.width // 8) * (big.height // 8)
        assert 9 * tiles > MAX_BIN_ENTRIES
        ref = api.FrameRenderer(dev, big)
        tg = _Targets(dev, big)
        color, _ = tg.render(lib, dev, ref, big, keep, expect=CAPACITY_EXCEEDED)
        assert b"MAX_BIN_ENTRIES" in lib.mlv_get_last_error_string()
        ctx = dev.immediate
        ctx.clear_render_target(tg.rt, big.clear_color)
        ctx.finish()
        cleared = ctx.read_texture(tg.rt)
        assert np.array_equal(color, cleared), "the render target was written although the call overflowed"
        # the next call works and matches the normal path
        ok = _full_screen_frame(4)
        assert 4 * tiles < MAX_BIN_ENTRIES
        ref2 = api.FrameRenderer(dev, ok)
        ref2.render_per_draw()
        want = ref2.read(0)
        color, depth = tg.render(lib, dev, ref2, ok, keep)
        assert_bits_equal(depth, want["depth"], "depth after the overflow")
        assert_color_close(color, want["color"])
        tg.destroy()
        ref.destroy()
        ref2.destroy()
    finally:
        dev.destroy()


def test_noalloc_rejects_sizes_beyond_its_limits():
    build.build()
    lib = api.load_library()
    nd = NoallocDraw()
    nd.vertex_buffer = nd.color = nd.depth = nd.tile_min = nd.tile_max = 16   # never dereferenced
    nd.vertex_stride, nd.vertex_count = 32, 3
    nd.index_count = 3 * (MAX_TRIANGLES + 1)
    nd.vs, nd.ps = scenes.VS_PASSTHROUGH, scenes.PS_PASSTHROUGH
    nd.viewport = api.Viewport(0, 0, 64, 64, 0, 1)
    nd.cull_mode, nd.depth_func = api.CULL_BACK, api.COMPARISON_GREATER_EQUAL
    nd.width, nd.height = 64, 64
    assert lib.mlv_draw_indexed_noalloc(ctypes.byref(nd), None) == CAPACITY_EXCEEDED
    assert b"MAX_TRIANGLES" in lib.mlv_get_last_error_string()
    nd.index_count = 3
    nd.width, nd.height = 2048, 2048    # more 8x8 tiles than the scratch holds
    nd.viewport = api.Viewport(0, 0, 2048, 2048, 0, 1)
    assert lib.mlv_draw_indexed_noalloc(ctypes.byref(nd), None) == CAPACITY_EXCEEDED
    # indices past the end of the caller's index buffer are refused on the host
    nd.width, nd.height = 64, 64
    nd.viewport = api.Viewport(0, 0, 64, 64, 0, 1)
    nd.index_buffer = 16
    nd.index_buffer_count = 6
    nd.index_count, nd.start_index = 6, 3
    assert lib.mlv_draw_indexed_noalloc(ctypes.byref(nd), None) == INVALID_ARG
    assert b"index buffer" in lib.mlv_get_last_error_string()
