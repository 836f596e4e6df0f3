"""Python front end of the C ABI (include/malevich.h), loaded with ctypes.

The objects mirror the API one to one (Device, Context, Buffer, Texture2D, CommandList); the
`FrameRenderer` plays a `scenes.Frame` through them the way the reference's render() does
(source/main.c:1265-1299): clear the targets, then for each draw set the pipeline state and call
DrawIndexed. It can also record the same frame into a deferred context and execute the resulting
command list as one batched, graph-captured launch sequence.

There is no CPU fallback: if the CUDA library is missing, `load_library` raises.
"""
import ctypes
import os

import numpy as np

from . import scenes

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libmalevich_gb300.so")

MLV_OK = 0
STATUS_NAMES = {0: "OK", 1: "INVALID_ARG", 2: "OUT_OF_MEMORY", 3: "CAPACITY_EXCEEDED", 4: "DEVICE",
                5: "TIMEOUT", 6: "UNSUPPORTED", 7: "INVALID_STATE"}

FORMAT_R8G8B8A8_UNORM, FORMAT_R16G16B16A16_FLOAT, FORMAT_R32G32B32A32_FLOAT = 1, 2, 3
FORMAT_D32_FLOAT, FORMAT_R32_UINT, FORMAT_R32G32_FLOAT = 4, 5, 6
BIND_VERTEX_BUFFER, BIND_INDEX_BUFFER, BIND_CONSTANT_BUFFER, BIND_SHADER_RESOURCE = 0x1, 0x2, 0x4, 0x8
BIND_RENDER_TARGET, BIND_DEPTH_STENCIL, BIND_UNORDERED_ACCESS = 0x20, 0x40, 0x80
CULL_NONE, CULL_FRONT, CULL_BACK = 1, 2, 3
COMPARISON_LESS, COMPARISON_GREATER_EQUAL = 2, 7
STAGES = ("clear", "geometry", "bin_scan", "bin_scatter", "tile", "vertex")

# every function the header declares (tests check the library exports all of them)
EXPORTS = [
    "mlv_get_last_error_string", "mlv_get_abi_version", "mlv_create_device", "mlv_destroy_device",
    "mlv_get_immediate_context", "mlv_create_deferred_context", "mlv_destroy_context", "mlv_create_buffer",
    "mlv_destroy_buffer", "mlv_create_texture2d", "mlv_create_texture2d_on_memory", "mlv_destroy_texture2d", "mlv_buffer_device_pointer",
    "mlv_texture2d_device_pointer", "mlv_update_buffer", "mlv_update_texture2d", "mlv_read_texture2d",
    "mlv_update_buffer_async", "mlv_update_texture2d_async", "mlv_update_resources_async",
    "mlv_ia_set_primitive_topology", "mlv_ia_set_index_buffer", "mlv_ia_set_vertex_buffers",
    "mlv_vs_set_shader", "mlv_vs_set_constant_buffers", "mlv_vs_set_shader_resources", "mlv_ps_set_shader",
    "mlv_ps_set_shader_resources", "mlv_rs_set_viewports", "mlv_rs_set_state", "mlv_om_set_depth_stencil_state",
    "mlv_om_set_render_targets", "mlv_om_set_visibility_targets", "mlv_clear_render_target_view",
    "mlv_clear_depth_stencil_view", "mlv_clear_texture_u32", "mlv_draw_indexed", "mlv_draw", "mlv_flush",
    "mlv_finish", "mlv_finish_command_list", "mlv_execute_command_list", "mlv_destroy_command_list",
    "mlv_get_stream", "mlv_get_stats", "mlv_reset_stats", "mlv_get_tuning", "mlv_set_tuning",
    "mlv_set_profiling", "mlv_get_stage_times", "mlv_set_debug_capture", "mlv_get_tile_infos",
    "mlv_draw_indexed_noalloc", "mlv_diff_forward", "mlv_diff_backward", "mlv_om_set_primitive_id_target",
]


class MalevichError(RuntimeError):
    def __init__(self, status, message):
        super().__init__("%s: %s" % (STATUS_NAMES.get(status, status), message))
        self.status = status


UPLOAD_BUFFER, UPLOAD_TEXTURE2D = 0, 1


class Upload(ctypes.Structure):
    """One range of a grouped upload (mlv_upload)."""
    _fields_ = [("kind", ctypes.c_uint32), ("pad", ctypes.c_uint32), ("resource", ctypes.c_void_p),
                ("src_offset", ctypes.c_uint64), ("dst_offset", ctypes.c_uint64), ("size", ctypes.c_uint64)]


class BufferDesc(ctypes.Structure):
    _fields_ = [("byte_width", ctypes.c_uint64), ("bind_flags", ctypes.c_uint32), ("reserved", ctypes.c_uint32)]


class Texture2DDesc(ctypes.Structure):
    _fields_ = [("width", ctypes.c_uint32), ("height", ctypes.c_uint32), ("format", ctypes.c_int),
                ("bind_flags", ctypes.c_uint32)]


class Viewport(ctypes.Structure):
    _fields_ = [(n, ctypes.c_float) for n in ("top_left_x", "top_left_y", "width", "height", "min_depth",
                                               "max_depth")]


class RasterizerDesc(ctypes.Structure):
    _fields_ = [("cull_mode", ctypes.c_int), ("fill_rule", ctypes.c_int), ("sample_position", ctypes.c_int)]


class DepthStencilDesc(ctypes.Structure):
    _fields_ = [("depth_enable", ctypes.c_int32), ("depth_func", ctypes.c_int)]


class Stats(ctypes.Structure):
    _fields_ = [(n, ctypes.c_uint64) for n in ("vertex_count", "input_triangle_count", "assembled_triangle_count",
                                               "active_bin_count", "total_triangle_count_in_bins", "draw_count",
                                               "batch_count", "kernel_launches")]

    def as_dict(self):
        return {n: int(getattr(self, n)) for n, _ in self._fields_}


class Tuning(ctypes.Structure):
    _fields_ = [("tile_warps_per_block", ctypes.c_uint32), ("warps_per_tile", ctypes.c_uint32),
                ("big_triangle_tiles", ctypes.c_uint32), ("geometry_block", ctypes.c_uint32),
                ("initial_bin_entries", ctypes.c_uint32), ("initial_clip_fan_slots", ctypes.c_uint32),
                ("small_draw_triangles", ctypes.c_uint32), ("debug_flags", ctypes.c_uint32),
                ("persistent_launch", ctypes.c_uint32)]


DEBUG_STALL_LOOKBACK = 0x1
DEBUG_STALL_GRID = 0x2


_lib = None


def load_library(path=LIB_PATH):
    """Loads the in-tree CUDA library. Raises if it has not been built: there is no fallback."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise ImportError("malevich_gb300 CUDA library not built (%s); run __graft_entry__.build()" % path)
    lib = ctypes.CDLL(path)
    vp = ctypes.c_void_p
    lib.mlv_get_last_error_string.restype = ctypes.c_char_p
    lib.mlv_get_abi_version.restype = ctypes.c_int
    for name in EXPORTS:
        f = getattr(lib, name)
        if name not in ("mlv_get_last_error_string", "mlv_get_abi_version"):
            f.restype = ctypes.c_int
    lib.mlv_create_device.argtypes = [ctypes.c_int, ctypes.POINTER(vp)]
    lib.mlv_destroy_device.argtypes = [vp]
    lib.mlv_get_immediate_context.argtypes = [vp, ctypes.POINTER(vp)]
    lib.mlv_create_deferred_context.argtypes = [vp, ctypes.POINTER(vp)]
    lib.mlv_destroy_context.argtypes = [vp]
    lib.mlv_create_buffer.argtypes = [vp, ctypes.POINTER(BufferDesc), vp, ctypes.POINTER(vp)]
    lib.mlv_destroy_buffer.argtypes = [vp]
    lib.mlv_create_texture2d.argtypes = [vp, ctypes.POINTER(Texture2DDesc), vp, ctypes.c_uint32, ctypes.POINTER(vp)]
    lib.mlv_create_texture2d_on_memory.argtypes = [vp, ctypes.POINTER(Texture2DDesc), vp, ctypes.POINTER(vp)]
    lib.mlv_destroy_texture2d.argtypes = [vp]
    lib.mlv_buffer_device_pointer.argtypes = [vp, ctypes.POINTER(vp)]
    lib.mlv_texture2d_device_pointer.argtypes = [vp, ctypes.POINTER(vp)]
    lib.mlv_update_buffer.argtypes = [vp, vp, ctypes.c_uint64, vp, ctypes.c_uint64]
    lib.mlv_update_texture2d.argtypes = [vp, vp, vp, ctypes.c_uint32]
    lib.mlv_update_buffer_async.argtypes = [vp, vp, ctypes.c_uint64, vp, ctypes.c_uint64]
    lib.mlv_update_texture2d_async.argtypes = [vp, vp, vp, ctypes.c_uint32]
    lib.mlv_update_resources_async.argtypes = [vp, vp, ctypes.c_uint64, ctypes.POINTER(Upload), ctypes.c_uint32]
    lib.mlv_read_texture2d.argtypes = [vp, vp, vp, ctypes.c_uint32]
    lib.mlv_ia_set_primitive_topology.argtypes = [vp, ctypes.c_int]
    lib.mlv_ia_set_index_buffer.argtypes = [vp, vp, ctypes.c_int, ctypes.c_uint32]
    lib.mlv_ia_set_vertex_buffers.argtypes = [vp, ctypes.c_uint32, ctypes.c_uint32, ctypes.POINTER(vp),
                                              ctypes.POINTER(ctypes.c_uint32), ctypes.POINTER(ctypes.c_uint32)]
    lib.mlv_vs_set_shader.argtypes = [vp, ctypes.c_int]
    lib.mlv_ps_set_shader.argtypes = [vp, ctypes.c_int]
    for n in ("mlv_vs_set_constant_buffers", "mlv_vs_set_shader_resources", "mlv_ps_set_shader_resources"):
        getattr(lib, n).argtypes = [vp, ctypes.c_uint32, ctypes.c_uint32, ctypes.POINTER(vp)]
    lib.mlv_rs_set_viewports.argtypes = [vp, ctypes.c_uint32, ctypes.POINTER(Viewport)]
    lib.mlv_rs_set_state.argtypes = [vp, ctypes.POINTER(RasterizerDesc)]
    lib.mlv_om_set_depth_stencil_state.argtypes = [vp, ctypes.POINTER(DepthStencilDesc)]
    lib.mlv_om_set_render_targets.argtypes = [vp, vp, vp]
    lib.mlv_om_set_visibility_targets.argtypes = [vp, vp, vp, vp]
    lib.mlv_clear_render_target_view.argtypes = [vp, vp, ctypes.POINTER(ctypes.c_float)]
    lib.mlv_clear_depth_stencil_view.argtypes = [vp, vp, ctypes.c_float]
    lib.mlv_clear_texture_u32.argtypes = [vp, vp, ctypes.c_uint32]
    lib.mlv_draw_indexed.argtypes = [vp, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_int32]
    lib.mlv_draw.argtypes = [vp, ctypes.c_uint32, ctypes.c_uint32]
    lib.mlv_flush.argtypes = [vp]
    lib.mlv_finish.argtypes = [vp]
    lib.mlv_finish_command_list.argtypes = [vp, ctypes.POINTER(vp)]
    lib.mlv_execute_command_list.argtypes = [vp, vp]
    lib.mlv_destroy_command_list.argtypes = [vp]
    lib.mlv_get_stream.argtypes = [vp, ctypes.POINTER(vp)]
    lib.mlv_get_stats.argtypes = [vp, ctypes.POINTER(Stats)]
    lib.mlv_reset_stats.argtypes = [vp]
    lib.mlv_get_tuning.argtypes = [vp, ctypes.POINTER(Tuning)]
    lib.mlv_set_tuning.argtypes = [vp, ctypes.POINTER(Tuning)]
    lib.mlv_set_profiling.argtypes = [vp, ctypes.c_int]
    lib.mlv_get_stage_times.argtypes = [vp, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_uint64)]
    lib.mlv_set_debug_capture.argtypes = [vp, ctypes.c_int]
    lib.mlv_get_tile_infos.argtypes = [vp, vp, vp, vp, ctypes.c_uint64, ctypes.POINTER(ctypes.c_uint64)]
    lib.mlv_draw_indexed_noalloc.argtypes = [vp, vp]
    lib.mlv_diff_forward.argtypes = [vp, vp]
    lib.mlv_diff_backward.argtypes = [vp, vp]
    lib.mlv_om_set_primitive_id_target.argtypes = [vp, vp]
    _lib = lib
    return lib


def _check(status):
    if status != MLV_OK:
        msg = _lib.mlv_get_last_error_string().decode("utf-8", "replace")
        raise MalevichError(status, msg)


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p)


class Buffer:
    def __init__(self, device, data=None, byte_width=None, bind=BIND_VERTEX_BUFFER):
        lib = load_library()
        arr = None if data is None else np.ascontiguousarray(data)
        size = arr.nbytes if arr is not None else int(byte_width)
        h = ctypes.c_void_p()
        _check(lib.mlv_create_buffer(device.handle, ctypes.byref(BufferDesc(size, bind, 0)),
                                     _ptr(arr) if arr is not None else None, ctypes.byref(h)))
        self.handle, self.size, self.device = h, size, device

    def destroy(self):
        if self.handle:
            _check(load_library().mlv_destroy_buffer(self.handle))
            self.handle = None

    def device_pointer(self):
        p = ctypes.c_void_p()
        _check(load_library().mlv_buffer_device_pointer(self.handle, ctypes.byref(p)))
        return p.value


class Texture2D:
    def __init__(self, device, width, height, fmt, data=None, bind=BIND_SHADER_RESOURCE, device_memory=None):
        """device_memory: place the texture on that caller-owned device address instead."""
        lib = load_library()
        arr = None if data is None else np.ascontiguousarray(data)
        h = ctypes.c_void_p()
        desc = Texture2DDesc(width, height, fmt, bind)
        if device_memory is not None:
            _check(lib.mlv_create_texture2d_on_memory(device.handle, ctypes.byref(desc), device_memory, ctypes.byref(h)))
        else:
            _check(lib.mlv_create_texture2d(device.handle, ctypes.byref(desc), _ptr(arr) if arr is not None else None,
                                            0, ctypes.byref(h)))
        self.handle, self.width, self.height, self.format, self.device = h, width, height, fmt, device

    def destroy(self):
        if self.handle:
            _check(load_library().mlv_destroy_texture2d(self.handle))
            self.handle = None

    def device_pointer(self):
        p = ctypes.c_void_p()
        _check(load_library().mlv_texture2d_device_pointer(self.handle, ctypes.byref(p)))
        return p.value


_DTYPES = {FORMAT_R8G8B8A8_UNORM: (np.uint32, ()), FORMAT_D32_FLOAT: (np.float32, ()),
           FORMAT_R32_UINT: (np.uint32, ()), FORMAT_R32G32_FLOAT: (np.float32, (2,)),
           FORMAT_R16G16B16A16_FLOAT: (np.float16, (4,)), FORMAT_R32G32B32A32_FLOAT: (np.float32, (4,))}


class Context:
    def __init__(self, handle, device, deferred=False):
        self.handle, self.device, self.deferred = handle, device, deferred
        self.lib = load_library()
        self._queued = []   # sources of queued uploads: alive until the context next synchronises

    def _synchronised(self):
        self._queued.clear()

    # state (Pipeline fields, source/main.c:109-115)
    def ia_set_index_buffer(self, buf, offset=0):
        _check(self.lib.mlv_ia_set_index_buffer(self.handle, buf.handle if buf else None, FORMAT_R32_UINT, offset))

    def ia_set_vertex_buffer(self, buf, stride, offset=0):
        arr = (ctypes.c_void_p * 1)(buf.handle if buf else None)
        _check(self.lib.mlv_ia_set_vertex_buffers(self.handle, 0, 1, arr, (ctypes.c_uint32 * 1)(stride),
                                                  (ctypes.c_uint32 * 1)(offset)))

    def vs_set_shader(self, vs):
        _check(self.lib.mlv_vs_set_shader(self.handle, vs))

    def ps_set_shader(self, ps):
        _check(self.lib.mlv_ps_set_shader(self.handle, ps))

    def vs_set_constant_buffer(self, slot, buf):
        _check(self.lib.mlv_vs_set_constant_buffers(self.handle, slot, 1, (ctypes.c_void_p * 1)(buf.handle if buf else None)))

    def vs_set_shader_resource(self, slot, tex):
        _check(self.lib.mlv_vs_set_shader_resources(self.handle, slot, 1, (ctypes.c_void_p * 1)(tex.handle if tex else None)))

    def ps_set_shader_resource(self, slot, tex):
        _check(self.lib.mlv_ps_set_shader_resources(self.handle, slot, 1, (ctypes.c_void_p * 1)(tex.handle if tex else None)))

    def rs_set_viewport(self, vp):
        _check(self.lib.mlv_rs_set_viewports(self.handle, 1, ctypes.byref(Viewport(*vp))))

    def rs_set_cull(self, cull_internal, fill_rule=0, sample_center=0):
        mode = {scenes.CULL_NONE: CULL_NONE, scenes.CULL_BACK: CULL_BACK, scenes.CULL_FRONT: CULL_FRONT}[cull_internal]
        _check(self.lib.mlv_rs_set_state(self.handle, ctypes.byref(RasterizerDesc(mode, fill_rule, sample_center))))

    def om_set_depth_func(self, depth_func_internal):
        f = COMPARISON_LESS if depth_func_internal == scenes.DEPTH_LESS else COMPARISON_GREATER_EQUAL
        _check(self.lib.mlv_om_set_depth_stencil_state(self.handle, ctypes.byref(DepthStencilDesc(1, f))))

    def om_set_render_targets(self, rt, ds):
        _check(self.lib.mlv_om_set_render_targets(self.handle, rt.handle if rt else None, ds.handle if ds else None))

    def om_set_visibility_targets(self, tri=None, draw=None, bary=None):
        h = lambda t: t.handle if t else None
        _check(self.lib.mlv_om_set_visibility_targets(self.handle, h(tri), h(draw), h(bary)))

    def om_set_primitive_id_target(self, tex):
        _check(self.lib.mlv_om_set_primitive_id_target(self.handle, tex.handle if tex else None))

    def clear_render_target(self, rt, rgba):
        _check(self.lib.mlv_clear_render_target_view(self.handle, rt.handle, (ctypes.c_float * 4)(*rgba)))

    def clear_depth(self, ds, depth):
        _check(self.lib.mlv_clear_depth_stencil_view(self.handle, ds.handle, ctypes.c_float(depth)))

    def clear_u32(self, tex, value):
        _check(self.lib.mlv_clear_texture_u32(self.handle, tex.handle, ctypes.c_uint32(value)))

    def draw_indexed(self, count, start=0, base_vertex=0):
        _check(self.lib.mlv_draw_indexed(self.handle, count, start, base_vertex))

    def draw(self, count, start=0):
        _check(self.lib.mlv_draw(self.handle, count, start))

    def finish(self):
        _check(self.lib.mlv_finish(self.handle))
        self._synchronised()

    def read_texture(self, tex):
        dt, extra = _DTYPES[tex.format]
        out = np.empty((tex.height, tex.width) + extra, dt)
        _check(self.lib.mlv_read_texture2d(self.handle, tex.handle, _ptr(out), 0))
        self._synchronised()
        return out

    def update_buffer(self, buf, data, offset=0):
        arr = np.ascontiguousarray(data)
        _check(self.lib.mlv_update_buffer(self.handle, buf.handle, offset, _ptr(arr), arr.nbytes))
        self._synchronised()

    def update_texture(self, tex, data):
        arr = np.ascontiguousarray(data)
        _check(self.lib.mlv_update_texture2d(self.handle, tex.handle, _ptr(arr), 0))
        self._synchronised()

    def update_buffer_async(self, buf, arr, offset=0):
        """Queued upload: `arr` (C-contiguous) must stay unchanged until the next synchronisation;
        the context keeps a reference to it until then."""
        if not arr.flags["C_CONTIGUOUS"]:
            raise ValueError("update_buffer_async needs a C-contiguous array it can keep")
        _check(self.lib.mlv_update_buffer_async(self.handle, buf.handle, offset, _ptr(arr), arr.nbytes))
        self._queued.append(arr)

    def update_texture_async(self, tex, arr):
        if not arr.flags["C_CONTIGUOUS"]:
            raise ValueError("update_texture_async needs a C-contiguous array it can keep")
        _check(self.lib.mlv_update_texture2d_async(self.handle, tex.handle, _ptr(arr), 0))
        self._queued.append(arr)

    def update_resources_async(self, block, uploads):
        """Queued uploads of several resources from one C-contiguous byte array `block`:
        `uploads` is a list of (resource, src_offset, size) for Buffer/Texture objects (buffers may
        add a dst_offset as a fourth item). One copy moves the block, one kernel places the ranges;
        the context keeps `block` alive until its next synchronisation."""
        if not block.flags["C_CONTIGUOUS"]:
            raise ValueError("update_resources_async needs a C-contiguous array it can keep")
        arr = (Upload * max(len(uploads), 1))()
        for i, u in enumerate(uploads):
            res, src, size = u[0], u[1], u[2]
            dst = u[3] if len(u) > 3 else 0
            kind = UPLOAD_TEXTURE2D if isinstance(res, Texture2D) else UPLOAD_BUFFER
            arr[i] = Upload(kind, 0, res.handle, src, dst, size)
        _check(self.lib.mlv_update_resources_async(self.handle, _ptr(block), block.nbytes, arr, len(uploads)))
        self._queued.append(block)

    def finish_command_list(self):
        h = ctypes.c_void_p()
        _check(self.lib.mlv_finish_command_list(self.handle, ctypes.byref(h)))
        return CommandList(h)

    def execute_command_list(self, cl):
        _check(self.lib.mlv_execute_command_list(self.handle, cl.handle))

    def stream(self):
        p = ctypes.c_void_p()
        _check(self.lib.mlv_get_stream(self.handle, ctypes.byref(p)))
        return p.value

    def stats(self):
        s = Stats()
        _check(self.lib.mlv_get_stats(self.handle, ctypes.byref(s)))
        self._synchronised()
        return s.as_dict()

    def reset_stats(self):
        _check(self.lib.mlv_reset_stats(self.handle))
        self._synchronised()

    def tuning(self):
        t = Tuning()
        _check(self.lib.mlv_get_tuning(self.handle, ctypes.byref(t)))
        return {n: int(getattr(t, n)) for n, _ in Tuning._fields_}

    def set_tuning(self, **kw):
        cur = self.tuning()
        cur.update(kw)
        _check(self.lib.mlv_set_tuning(self.handle, ctypes.byref(Tuning(**cur))))

    def set_profiling(self, enable):
        _check(self.lib.mlv_set_profiling(self.handle, int(bool(enable))))

    def stage_times(self):
        ms = (ctypes.c_double * len(STAGES))()
        n = (ctypes.c_uint64 * len(STAGES))()
        _check(self.lib.mlv_get_stage_times(self.handle, ms, n))
        return {STAGES[i]: (float(ms[i]), int(n[i])) for i in range(len(STAGES))}

    def set_debug_capture(self, enable):
        _check(self.lib.mlv_set_debug_capture(self.handle, int(bool(enable))))

    def tile_infos(self):
        n = ctypes.c_uint64()
        _check(self.lib.mlv_get_tile_infos(self.handle, None, None, None, 0, ctypes.byref(n)))
        m = int(n.value)
        tiles = np.zeros(max(m, 1), np.uint32)
        tris = np.zeros(max(m, 1), np.uint32)
        masks = np.zeros(max(m, 1), np.uint64)
        _check(self.lib.mlv_get_tile_infos(self.handle, _ptr(tiles), _ptr(tris), _ptr(masks), m, ctypes.byref(n)))
        return tiles[:m], tris[:m], masks[:m]

    def destroy(self):
        if self.deferred and self.handle:
            _check(self.lib.mlv_destroy_context(self.handle))
            self.handle = None


class CommandList:
    def __init__(self, handle):
        self.handle = handle

    def destroy(self):
        if self.handle:
            _check(load_library().mlv_destroy_command_list(self.handle))
            self.handle = None


class Device:
    def __init__(self, ordinal=0):
        lib = load_library()
        h = ctypes.c_void_p()
        _check(lib.mlv_create_device(ordinal, ctypes.byref(h)))
        self.handle = h
        self.ordinal = ordinal
        c = ctypes.c_void_p()
        _check(lib.mlv_get_immediate_context(h, ctypes.byref(c)))
        self.immediate = Context(c, self)

    def create_deferred_context(self):
        c = ctypes.c_void_p()
        _check(load_library().mlv_create_deferred_context(self.handle, ctypes.byref(c)))
        return Context(c, self, deferred=True)

    def destroy(self):
        if self.handle:
            _check(load_library().mlv_destroy_device(self.handle))
            self.handle = None


# ------------------------------------------------------------------ frames

_FMT = {scenes.FMT_RGBA8: FORMAT_R8G8B8A8_UNORM, scenes.FMT_RGBA16F: FORMAT_R16G16B16A16_FLOAT,
        scenes.FMT_RGBA32F: FORMAT_R32G32B32A32_FLOAT}


class FrameRenderer:
    """Uploads a Frame's (or several Frames') resources once and renders them through the C ABI,
    either per draw on the immediate context or as one command list (batched)."""

    def __init__(self, device, frames, visibility=False, primitive_ids=False, primitive_id_memory=None):
        """primitive_id_memory: one device address per frame on which to place its primitive-id
        target (e.g. the slices of a [frames][height][width] int32 tensor)."""
        self.device = device
        self.frames = frames if isinstance(frames, (list, tuple)) else [frames]
        self._buffers, self._textures = {}, {}
        self.targets = []
        self.prim_targets = []
        for fr in self.frames:
            rt = Texture2D(device, fr.width, fr.height, FORMAT_R8G8B8A8_UNORM, bind=BIND_RENDER_TARGET)
            ds = Texture2D(device, fr.width, fr.height, FORMAT_D32_FLOAT, bind=BIND_DEPTH_STENCIL)
            vis = None
            if visibility:
                vis = (Texture2D(device, fr.width, fr.height, FORMAT_R32_UINT, bind=BIND_UNORDERED_ACCESS),
                       Texture2D(device, fr.width, fr.height, FORMAT_R32_UINT, bind=BIND_UNORDERED_ACCESS),
                       Texture2D(device, fr.width, fr.height, FORMAT_R32G32_FLOAT, bind=BIND_UNORDERED_ACCESS))
            self.targets.append((rt, ds, vis))
            mem = primitive_id_memory[len(self.prim_targets)] if primitive_id_memory is not None else None
            self.prim_targets.append(Texture2D(device, fr.width, fr.height, FORMAT_R32_UINT, bind=BIND_UNORDERED_ACCESS,
                                               device_memory=mem) if primitive_ids or mem else None)
            for d in fr.draws:
                self._buffer(d.vb, BIND_VERTEX_BUFFER)
                if d.ib is not None:
                    self._buffer(d.ib, BIND_INDEX_BUFFER)
                if d.cb is not None:
                    self._buffer(d.cb, BIND_CONSTANT_BUFFER)
                for t in (d.vs_tex, d.ps_tex):
                    if t is not None:
                        self._texture(t)
        self.command_list = None

    def _buffer(self, arr, bind):
        key = (id(arr), bind)
        if key not in self._buffers:
            self._buffers[key] = (Buffer(self.device, np.ascontiguousarray(arr), bind=bind), arr)
        return self._buffers[key][0]

    def _texture(self, t):
        key = id(t.data)
        if key not in self._textures:
            self._textures[key] = (Texture2D(self.device, t.width, t.height, _FMT[t.format], data=t.data), t)
        return self._textures[key][0]

    def _issue(self, ctx, fr, targets, prim=None):
        rt, ds, vis = targets
        if fr.clear_color is not None:
            ctx.clear_render_target(rt, fr.clear_color)
        if fr.clear_depth is not None:
            ctx.clear_depth(ds, fr.clear_depth)
        if vis is not None:
            ctx.clear_u32(vis[0], 0xFFFFFFFF)
            ctx.clear_u32(vis[1], 0xFFFFFFFF)
            ctx.clear_u32(vis[2], 0)
        if prim is not None:
            ctx.clear_u32(prim, 0xFFFFFFFF)
        ctx.om_set_render_targets(rt, ds)
        ctx.om_set_visibility_targets(*(vis if vis is not None else (None, None, None)))
        ctx.om_set_primitive_id_target(prim)
        for d in fr.draws:
            ctx.ia_set_vertex_buffer(self._buffer(d.vb, BIND_VERTEX_BUFFER), d.vb_stride)
            ctx.ia_set_index_buffer(self._buffer(d.ib, BIND_INDEX_BUFFER) if d.ib is not None else None)
            ctx.vs_set_shader(d.vs)
            ctx.ps_set_shader(d.ps)
            ctx.vs_set_constant_buffer(0, self._buffer(d.cb, BIND_CONSTANT_BUFFER) if d.cb is not None else None)
            ctx.vs_set_shader_resource(0, self._texture(d.vs_tex) if d.vs_tex is not None else None)
            ctx.ps_set_shader_resource(0, self._texture(d.ps_tex) if d.ps_tex is not None else None)
            ctx.rs_set_viewport(d.viewport)
            ctx.rs_set_cull(d.cull, d.fill_rule, d.sample_center)
            ctx.om_set_depth_func(d.depth_func)
            if d.ib is not None:
                ctx.draw_indexed(d.index_count, d.start_index, d.base_vertex)
            else:
                ctx.draw(d.index_count, d.start_index)

    def render_per_draw(self):
        """Immediate context: one launch sequence per draw (the reference's draw_indexed loop)."""
        ctx = self.device.immediate
        for fr, tg, pr in zip(self.frames, self.targets, self.prim_targets):
            self._issue(ctx, fr, tg, pr)

    def record(self):
        """Records every frame into one deferred context and returns the command list."""
        if self.command_list is None:
            dctx = self.device.create_deferred_context()
            for fr, tg, pr in zip(self.frames, self.targets, self.prim_targets):
                self._issue(dctx, fr, tg, pr)
            self.command_list = dctx.finish_command_list()
            dctx.destroy()
        return self.command_list

    def record_repeated(self, times):
        """A command list that plays the frames `times` times in a row on the same targets (each
        repetition clears and draws again): back-to-back frames in one graph launch."""
        dctx = self.device.create_deferred_context()
        for _ in range(times):
            for fr, tg, pr in zip(self.frames, self.targets, self.prim_targets):
                self._issue(dctx, fr, tg, pr)
        lst = dctx.finish_command_list()
        dctx.destroy()
        return lst

    def render_batched(self):
        """All draws of all frames as one batched launch sequence (a CUDA graph after the first run)."""
        self.device.immediate.execute_command_list(self.record())

    def read(self, index=0):
        ctx = self.device.immediate
        rt, ds, vis = self.targets[index]
        out = {"color": ctx.read_texture(rt), "depth": ctx.read_texture(ds)}
        if vis is not None:
            out["vis_tri"] = ctx.read_texture(vis[0])
            out["vis_draw"] = ctx.read_texture(vis[1])
            out["vis_bary"] = ctx.read_texture(vis[2])
        if self.prim_targets[index] is not None:
            out["vis_prim"] = ctx.read_texture(self.prim_targets[index])
        return out

    def destroy(self):
        if self.command_list is not None:
            self.command_list.destroy()
        for b, _ in self._buffers.values():
            b.destroy()
        for t, _ in self._textures.values():
            t.destroy()
        for rt, ds, vis in self.targets:
            rt.destroy()
            ds.destroy()
            for v in vis or ():
                v.destroy()
        for p in self.prim_targets:
            if p is not None:
                p.destroy()
