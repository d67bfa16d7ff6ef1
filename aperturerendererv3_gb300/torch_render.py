"""PyTorch binding of the replay adjoint: rendering as a differentiable function
of the albedo texels.

    img = render_textures(texels, renderer, (W, H), origin, direction, spp, fov=40, max_depth=8)
    loss = ((img - target) ** 2).sum()
    loss.backward()              # texels.grad from ar_adjoint

Forward uploads the texels into the renderer's scene and renders the per-pixel
mean XYZ (float64, on the texels' device).  Backward re-uploads the texels the
forward saw and calls the C ABI's replay adjoint with d(loss)/d(image); the
gradient comes back as float64 sums and is cast to the texels' dtype.  Both
directions go through the same C entry points a C++ caller would use; there is
no Python or CPU fallback.
"""
from __future__ import annotations

import torch

from .scene import SceneRenderer


class RenderTextures(torch.autograd.Function):
    @staticmethod
    def forward(ctx, texels: torch.Tensor, renderer: SceneRenderer, size, origin, direction, spp: int, kw: dict):
        if not texels.is_cuda:
            raise ValueError("texels must be a CUDA tensor")
        renderer.update_texels(texels)
        w, h = int(size[0]), int(size[1])
        img = torch.empty((h, w, 3), dtype=torch.float64, device=texels.device)
        renderer.render_into(img, size, origin, direction, spp, **kw)
        ctx.save_for_backward(texels)
        ctx.args = (renderer, size, origin, direction, spp, kw)
        return img

    @staticmethod
    def backward(ctx, grad_img: torch.Tensor):
        (texels,) = ctx.saved_tensors
        renderer, size, origin, direction, spp, kw = ctx.args
        renderer.update_texels(texels)
        grad = torch.empty(texels.numel(), dtype=torch.float64, device=texels.device)
        renderer.adjoint(grad_img, grad, size, origin, direction, spp, **kw)
        return grad.to(texels.dtype).view_as(texels), None, None, None, None, None, None


def render_textures(texels: torch.Tensor, renderer: SceneRenderer, size, origin, direction, spp: int, **kw):
    """Differentiable render of the per-pixel mean XYZ with respect to `texels`
    (all of the renderer's texture texels, float32, texel_count() elements in any shape)."""
    return RenderTextures.apply(texels, renderer, size, origin, direction, spp, kw)
