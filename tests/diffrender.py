"""Test harness for the differentiable path: a torch.autograd.Function over the C ABI's
mlv_diff_forward / mlv_diff_backward. The descriptors and the visibility pass it drives live in
the package (malevich_gb300/diff.py); the product is the C ABI."""
import ctypes

import torch

from malevich_gb300 import api
from malevich_gb300.diff import DiffScene, visibility  # noqa: F401  (re-exported for the tests)


class DiffRender(torch.autograd.Function):
    """image = render(colors, texture, positions) under the scene's fixed visibility."""

    @staticmethod
    def forward(ctx, col, tex, pos, scene):
        lib = api.load_library()
        col, tex, pos = col.contiguous(), tex.contiguous(), pos.contiguous()
        image = torch.empty((scene.views, scene.height, scene.width, 3), dtype=torch.float32, device=col.device)
        d = scene.desc(col, tex, pos, image=image)
        st = lib.mlv_diff_forward(ctypes.byref(d), ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
        if st != 0:
            raise api.MalevichError(st, lib.mlv_get_last_error_string().decode())
        ctx.scene = scene
        ctx.save_for_backward(col, tex, pos)
        return image

    @staticmethod
    def backward(ctx, grad_image):
        lib = api.load_library()
        col, tex, pos = ctx.saved_tensors
        scene = ctx.scene
        g_col = torch.zeros_like(col) if ctx.needs_input_grad[0] else None
        g_tex = torch.zeros_like(tex) if ctx.needs_input_grad[1] else None
        g_pos = torch.zeros_like(pos) if ctx.needs_input_grad[2] else None
        gi = grad_image.contiguous()
        d = scene.desc(col, tex, pos, grad_image=gi, g_col=g_col, g_tex=g_tex, g_pos=g_pos)
        st = lib.mlv_diff_backward(ctypes.byref(d), ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
        if st != 0:
            raise api.MalevichError(st, lib.mlv_get_last_error_string().decode())
        return g_col, g_tex, g_pos, None


def l2_loss(image, target, scene):
    return (((image - target) * scene.mask) ** 2).sum()
