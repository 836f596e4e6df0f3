"""The allocation-free entry point, mlv_draw_indexed_noalloc, against mlv_draw_indexed.

It exists for callers that cannot call cudaMalloc (a host that owns all device memory through its
own allocator, a render loop with a no-allocation rule, work issued while another component
captures a CUDA graph): it draws with the same kernels, keeping its scratch in one static device
array. This test allocates the inputs and outputs itself, as such a caller would, then renders
the same frame twice in a row through the C ABI and compares both results with the normal path:
depth, bit for bit; colour within the +-1 LSB the other parity tests use. This file is collected
last so that a failure here comes after every other test has run.
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
                ("index_count", ctypes.c_uint32), ("start_index", ctypes.c_uint32), ("base_vertex", ctypes.c_int32),
                ("vs", ctypes.c_int), ("ps", ctypes.c_int), ("per_frame_cb", ctypes.c_void_p),
                ("vs_texture", NoallocTexture), ("ps_texture", NoallocTexture), ("viewport", api.Viewport),
                ("cull_mode", ctypes.c_int), ("depth_func", ctypes.c_int), ("color", ctypes.c_void_p),
                ("depth", ctypes.c_void_p), ("tile_min", ctypes.c_void_p), ("tile_max", ctypes.c_void_p),
                ("width", ctypes.c_uint32), ("height", ctypes.c_uint32), ("flags", ctypes.c_uint32)]


RESET_HIZ = 0x1
MAX_TRIANGLES = 32768
CAPACITY_EXCEEDED = 3


def _texture(renderer, t):
    if t is None:
        return NoallocTexture(None, 0, 0, 0)
    tex = renderer._texture(t)
    return NoallocTexture(tex.device_pointer(), tex.width, tex.height, tex.format)


def _render_noalloc(lib, dev, renderer, frame, rt, ds, tile_min, tile_max, keep):
    ctx = dev.immediate
    ctx.clear_render_target(rt, frame.clear_color)
    ctx.clear_depth(ds, frame.clear_depth)
    ctx.finish()
    for k, d in enumerate(frame.draws):
        cb = np.ascontiguousarray(d.cb, np.float32) if d.cb is not None else None
        keep.append(cb)
        nd = NoallocDraw()
        vb = renderer._buffer(d.vb, api.BIND_VERTEX_BUFFER)
        nd.vertex_buffer = vb.device_pointer()
        nd.vertex_stride = d.vb_stride
        nd.vertex_count = d.vertex_count()
        nd.index_buffer = renderer._buffer(d.ib, api.BIND_INDEX_BUFFER).device_pointer() if d.ib is not None else None
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
        nd.flags = RESET_HIZ if k == 0 else 0
        status = lib.mlv_draw_indexed_noalloc(ctypes.byref(nd), None)
        assert status == 0, lib.mlv_get_last_error_string()
    return ctx.read_texture(rt), ctx.read_texture(ds)


@pytest.mark.parametrize("native", [True, False])
def test_noalloc_matches_draw_indexed_on_two_calls(native):
    import torch
    build.build()
    lib = api.load_library()
    dev = api.Device(0)
    keep = []
    try:
        frame = scenes.small_scene(21, 96, 80, vs=scenes.VS_BASIC, ps=scenes.PS_BASIC, n_objects=3, native=native)
        frame.draws += scenes.small_scene(22, 96, 80, vs=scenes.VS_VERTEX_LIGHTING, ps=scenes.PS_ENV_LIGHTING,
                                          n_objects=2, native=native, inside=True).draws
        ref = api.FrameRenderer(dev, frame)
        ref.render_per_draw()
        want = ref.read(0)
        rt = api.Texture2D(dev, frame.width, frame.height, api.FORMAT_R8G8B8A8_UNORM, bind=api.BIND_RENDER_TARGET)
        ds = api.Texture2D(dev, frame.width, frame.height, api.FORMAT_D32_FLOAT, bind=api.BIND_DEPTH_STENCIL)
        tiles = ((frame.width + 7) // 8) * ((frame.height + 7) // 8)
        tile_min = torch.zeros(tiles, dtype=torch.float32, device="cuda")
        tile_max = torch.ones(tiles, dtype=torch.float32, device="cuda")
        for call in range(2):
            color, depth = _render_noalloc(lib, dev, ref, frame, rt, ds, tile_min, tile_max, keep)
            assert_bits_equal(depth, want["depth"], "depth (call %d)" % call)
            assert_color_close(color, want["color"])
        rt.destroy()
        ds.destroy()
        ref.destroy()
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
