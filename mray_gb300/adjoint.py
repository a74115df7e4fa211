"""Differentiable rendering through the path-replay adjoint.

``render_albedo(texture, tracer, tex_id, params)`` returns the rendered image
(weight-normalised RGB, (H, W, 3)) as a function of an f32 RGBA albedo
texture that the tracer reads directly (``PathTracer.add_texture`` with a CUDA
tensor).  ``render_scene(texture, emission, tracer, tex_id, lights, params)``
is the same image as a function of the texture and of the RGB radiance of the
area-light instances ``lights`` ((len(lights), 3); the forward pass sets them
on the tracer).  Their backward pass is ``mrg_pt_adjoint``: the image gradient
goes in as dLoss/dPixel and the texture (and emission) gradients come out,
recomputing every path from its sample index instead of storing it.  Russian
roulette's throughput-dependent probability is a constant to the adjoint, so
gradient checks render with ``rr_start == max_depth``.
"""
import torch


def _delta(grad_image):
    h, w = grad_image.shape[0], grad_image.shape[1]
    delta = torch.zeros((h, w, 4), dtype=torch.float32, device=grad_image.device)
    delta[..., :3] = grad_image.float()
    return delta


class AlbedoRender(torch.autograd.Function):
    @staticmethod
    def forward(ctx, texture, tracer, tex_id, params):
        image = tracer.render(params)
        ctx.tracer, ctx.tex_id, ctx.params = tracer, tex_id, params
        ctx.tex_shape = texture.shape
        return image[..., :3] / image[..., 3:]

    @staticmethod
    def backward(ctx, grad_image):
        grad = ctx.tracer.adjoint(ctx.params, ctx.tex_id, _delta(grad_image))
        return grad[..., :ctx.tex_shape[-1]].reshape(ctx.tex_shape), None, None, None


class SceneRender(torch.autograd.Function):
    @staticmethod
    def forward(ctx, texture, emission, tracer, tex_id, lights, params):
        for inst, r in zip(lights, emission.detach().double().cpu().tolist()):
            tracer.set_area_light(inst, r)
        image = tracer.render(params)
        ctx.tracer, ctx.tex_id, ctx.lights, ctx.params = tracer, tex_id, list(lights), params
        ctx.tex_shape = None if texture is None else texture.shape
        ctx.em_dtype, ctx.em_device = emission.dtype, emission.device
        return image[..., :3] / image[..., 3:]

    @staticmethod
    def backward(ctx, grad_image):
        t = ctx.tracer
        ge = torch.zeros((t.n_instances, 4), dtype=torch.float32, device=grad_image.device)
        grad = t.adjoint(ctx.params, ctx.tex_id, _delta(grad_image), grad_emission=ge)
        g_tex = None if grad is None else grad[..., :ctx.tex_shape[-1]].reshape(ctx.tex_shape)
        g_em = ge[ctx.lights, :3].to(device=ctx.em_device, dtype=ctx.em_dtype)
        return g_tex, g_em, None, None, None, None


def render_albedo(texture, tracer, tex_id, params):
    """Image = render(texture); differentiable in ``texture``."""
    return AlbedoRender.apply(texture, tracer, tex_id, params)


def render_scene(texture, emission, tracer, tex_id, lights, params):
    """Image = render(texture, emission of ``lights``); differentiable in
    both (texture / tex_id None: emission only)."""
    return SceneRender.apply(texture, emission, tracer, tex_id, lights, params)
