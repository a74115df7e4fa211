"""Differentiable rendering through the path-replay adjoint.

``render_albedo(texture, tracer, tex_id, params)`` returns the rendered image
(weight-normalised RGB, (H, W, 3)) as a function of an f32 RGBA albedo
texture that the tracer reads directly (``PathTracer.add_texture`` with a CUDA
tensor).  Its backward pass is ``mrg_pt_adjoint``: the image gradient goes in
as dLoss/dPixel and the texture gradient comes out, recomputing every path
from its sample index instead of storing it.  Russian roulette's
throughput-dependent probability is a constant to the adjoint, so gradient
checks render with ``rr_start == max_depth``.
"""
import torch


class AlbedoRender(torch.autograd.Function):
    @staticmethod
    def forward(ctx, texture, tracer, tex_id, params):
        image = tracer.render(params)
        ctx.tracer, ctx.tex_id, ctx.params = tracer, tex_id, params
        ctx.tex_shape = texture.shape
        return image[..., :3] / image[..., 3:]

    @staticmethod
    def backward(ctx, grad_image):
        h, w = grad_image.shape[0], grad_image.shape[1]
        delta = torch.zeros((h, w, 4), dtype=torch.float32, device=grad_image.device)
        delta[..., :3] = grad_image.float()
        grad = ctx.tracer.adjoint(ctx.params, ctx.tex_id, delta)
        return grad[..., :ctx.tex_shape[-1]].reshape(ctx.tex_shape), None, None, None


def render_albedo(texture, tracer, tex_id, params):
    """Image = render(texture); differentiable in ``texture``."""
    return AlbedoRender.apply(texture, tracer, tex_id, params)
