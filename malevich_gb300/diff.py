"""Host-side descriptors for the differentiable path's C ABI (mlv_diff_forward / mlv_diff_backward).

DiffDesc mirrors `mlv_diff_desc` (include/malevich.h). DiffScene keeps a scene's device-side
topology, UVs, visibility (per-view primitive ids from the exact rasteriser) and the checkpoint
buffer of per-pixel barycentrics, and fills a DiffDesc for given parameter tensors. The reference
has no differentiable path; these are the library side of the additions that the tests wrap in a
torch.autograd.Function.
"""
import ctypes

import numpy as np
import torch

from malevich_gb300 import api, scenes


class DiffDesc(ctypes.Structure):
    _fields_ = [("n_verts", ctypes.c_uint32), ("n_tris", ctypes.c_uint32), ("index_buffer", ctypes.c_void_p),
                ("colors", ctypes.c_void_p), ("uvs", ctypes.c_void_p), ("texture", ctypes.c_void_p),
                ("tex_width", ctypes.c_uint32), ("tex_height", ctypes.c_uint32), ("num_views", ctypes.c_uint32),
                ("width", ctypes.c_uint32), ("height", ctypes.c_uint32), ("positions", ctypes.c_void_p),
                ("primitive_ids", ctypes.c_void_p), ("barycentrics", ctypes.c_void_p), ("image", ctypes.c_void_p),
                ("grad_image", ctypes.c_void_p), ("grad_colors", ctypes.c_void_p), ("grad_texture", ctypes.c_void_p),
                ("grad_positions", ctypes.c_void_p)]


def _p(t):
    return t.data_ptr() if t is not None else None


def visibility(device, scene, pos=None):
    """Per-view primitive ids (the input triangle each pixel shows) from the exact rasteriser,
    all views in one batched command list, with the null pixel shader."""
    frames = scenes.diff_frames(scene, pos=pos, shade=False)
    r = api.FrameRenderer(device, frames, primitive_ids=True)
    r.render_batched()
    prims = np.stack([r.read(i)["vis_prim"] for i in range(len(frames))])
    r.destroy()
    return prims


class DiffScene:
    """Device-side topology, UVs, visibility and the checkpoint (barycentric) buffer."""

    def __init__(self, scene, prims):
        """prims: per-view primitive ids, a numpy array or an int32 device tensor used in place."""
        dev = "cuda"
        self.ib = torch.from_numpy(np.ascontiguousarray(scene["ib"]).view(np.int32)).to(dev)
        self.uv = torch.from_numpy(np.ascontiguousarray(scene["uv"], np.float32)).to(dev)
        if isinstance(prims, torch.Tensor):
            self.prim = prims
        else:
            self.prim = torch.from_numpy(np.ascontiguousarray(prims).view(np.int32)).to(dev)
        self.views, self.height, self.width = prims.shape
        self.n_verts = scene["col"].shape[0]
        self.n_tris = scene["ib"].shape[0]
        self.bary = torch.zeros((self.views, self.height, self.width, 2), dtype=torch.float32, device=dev)
        self.mask = (self.prim != -1).unsqueeze(-1).float()

    def desc(self, col, tex, pos, image=None, grad_image=None, g_col=None, g_tex=None, g_pos=None):
        return DiffDesc(self.n_verts, self.n_tris, _p(self.ib), _p(col), _p(self.uv), _p(tex), tex.shape[1],
                        tex.shape[0], self.views, self.width, self.height, _p(pos), _p(self.prim), _p(self.bary),
                        _p(image), _p(grad_image), _p(g_col), _p(g_tex), _p(g_pos))
