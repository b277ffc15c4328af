"""Differentiable rendering: material parameters -> image, with gradients
from the adjoint kernel (path replay) behind a torch.autograd.Function.

Parameters are a float64 tensor [materials, 7] per scene: reflectance
(r, g, b) -- the albedo of a Diffuse material, F0 of a GGX material --,
GGX roughness, and emission (r, g, b).  Values that a material's type does
not use are ignored (zero gradient).  The forward pass writes them into the
scene (path_scene_set_material; the BVH stays) and renders with the
streaming integrator; the backward pass runs path_render_adjoint with
dLoss/dImage.
"""

import numpy as np

from . import api, capi

PARAMS = ("refl_r", "refl_g", "refl_b", "roughness", "emit_r", "emit_g", "emit_b")
N_PARAMS = len(PARAMS)


def params_of(materials):
    """[materials, 7] float64 parameters of a list of capi.PathMaterial."""
    out = np.zeros((len(materials), N_PARAMS), np.float64)
    for i, m in enumerate(materials):
        refl = m.specular if m.type == capi.BSDF["GGX"] else m.diffuse
        out[i, 0:3] = list(refl)
        out[i, 3] = m.roughness
        out[i, 4:7] = list(m.emission)
    return out


def apply_params(scene, materials, params):
    """Write params [materials, 7] into the scene's materials (based on
    `materials`, the scene's material records)."""
    params = np.asarray(params, np.float64)
    for i, base in enumerate(materials):
        m = capi.PathMaterial()
        ctypes_copy(m, base)
        p = params[i]
        if m.type == capi.BSDF["GGX"]:
            m.specular[:] = [float(v) for v in p[0:3]]
            m.roughness = float(p[3])
        elif m.type == capi.BSDF["Diffuse"]:
            m.diffuse[:] = [float(v) for v in p[0:3]]
        m.emission[:] = [float(v) for v in p[4:7]]
        scene.set_material(i, m)


def ctypes_copy(dst, src):
    import ctypes
    ctypes.memmove(ctypes.byref(dst), ctypes.byref(src), ctypes.sizeof(src))


class Renderable:
    """A scene, its material records, camera and settings: what the
    autograd function renders."""

    def __init__(self, scene, materials, spec, samples_per, settings, renderer=None):
        self.scene = scene
        self.materials = materials
        self.spec = spec
        self.spp = int(samples_per)
        self.settings = settings.copy()
        self.settings.kernel_approach = 1
        self.renderer = renderer or api.Renderer()

    def render(self, params):
        apply_params(self.scene, self.materials, params)
        img = np.zeros((self.spec.y_dim, self.spec.x_dim, 3), np.float32)
        self.renderer.render(api.ExecutionModel.GPU, self.spec, img, self.scene, self.spp,
                             self.settings)
        return img

    def adjoint(self, params, d_image):
        apply_params(self.scene, self.materials, params)
        return self.renderer.render_adjoint(self.spec, self.scene, self.spp, self.settings,
                                            d_image)


def _function():
    import torch

    class RenderFunction(torch.autograd.Function):
        """image = render(params); d params = adjoint(dLoss/dImage)."""

        @staticmethod
        def forward(ctx, params, renderable):
            p = params.detach().cpu().numpy().astype(np.float64)
            ctx.renderable = renderable
            ctx.p = p
            ctx.dtype = params.dtype
            img = renderable.render(p)
            return torch.from_numpy(img).to(params.device)

        @staticmethod
        def backward(ctx, grad_image):
            g = grad_image.detach().to(torch.float32).contiguous()
            d = ctx.renderable.adjoint(ctx.p, g)
            return torch.from_numpy(d).to(device=grad_image.device, dtype=ctx.dtype), None

    return RenderFunction


_RENDER_FN = None


def render(params, renderable):
    """Differentiable render: params torch tensor [materials, 7] -> image
    torch tensor [H, W, 3] (float32)."""
    global _RENDER_FN
    if _RENDER_FN is None:
        _RENDER_FN = _function()
    return _RENDER_FN.apply(params, renderable)
