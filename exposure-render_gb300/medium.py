"""Differentiable medium over the C ABI (er_medium_*): a float density grid
and opacity parameters rendered by a bound tracer's camera and lights, with
gradients from the path-replay adjoint kernel behind a
torch.autograd.Function.

    m = Medium(renderer, density, opacity, scale=40.0)        # majorant built once
    img = m(density, opacity, spp=32)                          # (H, W, 3) mean, differentiable
    loss = ((img - target) ** 2).mean(); loss.backward()       # density.grad, opacity.grad

model="spline" (C.ER_MEDIUM_SPLINE): opacity holds B-spline values over the
density, isotropic phase with `albedo`.  model="tracer" (C.ER_MEDIUM_TRACER):
the grid holds intensities in the tracer's transfer-function domain and
opacity holds the values of the tracer's opacity nodes (at the tracer's node
positions); diffuse, specular, glossiness and emission are the tracer's, the
shading its BRDF / phase / hybrid (the hybrid as the expected value over its
shader choice) - the transport model of the tracer, with its opacity nodes
and intensity grid as the parameters.  `gradient_magnitude_inv` normalises
the hybrid switch (a constant of the estimator: 1 / the grid's largest
gradient magnitude when the Medium is made, by default).

The majorant grid is fixed when the Medium is made (or on rebuild_majorant):
the estimator's random numbers then do not depend on the medium, so for a
fixed seed the image is a smooth function of density and opacity.  The
forward keeps every sample for the adjoint (spp * H * W * 12 bytes); with
keep_samples=False the adjoint recomputes each sample first.

Every call goes through libexposurerender.so; there is no other path.
"""
from __future__ import annotations

import ctypes
from ctypes import byref

import torch

from . import capi as C


class Medium:
    def __init__(self, renderer, density: torch.Tensor, opacity: torch.Tensor, scale: float,
                 albedo=(0.8, 0.8, 0.8), nee_probability: float = 0.5, brick: int = 8, margin: float = 1.25,
                 floor: float = 1e-3, keep_samples: bool = True, model: str = "spline", gradient_magnitude_inv: float = None):
        self.r = renderer
        self.lib = renderer.lib
        self.model = {"spline": C.ER_MEDIUM_SPLINE, "tracer": C.ER_MEDIUM_TRACER}[model]
        self.gm_inv = 0.0
        if self.model == C.ER_MEDIUM_TRACER:
            if gradient_magnitude_inv is None:
                from . import scenes
                v = renderer.scene
                gradient_magnitude_inv = scenes.gradient_magnitude_range(density.detach().cpu().numpy(), v.spacing)
            self.gm_inv = float(gradient_magnitude_inv)
        self.scale = float(scale)
        self.albedo = tuple(float(a) for a in albedo)
        self.q = float(nee_probability)
        self.brick = int(brick)
        self.keep_samples = keep_samples
        # the kernels address the density grid with the tracer volume's resolution
        if tuple(density.shape) != tuple(renderer.scene.volume.shape):
            raise ValueError(f"density grid {tuple(density.shape)} differs from the tracer volume {renderer.scene.volume.shape}")
        self.shape = tuple(density.shape)
        self.n_opacity = opacity.numel()
        z, y, x = density.shape
        nb = [(d + brick - 1) // brick for d in (z, y, x)]
        self.majorant = torch.zeros(nb, dtype=torch.float32, device=density.device)
        self.rebuild_majorant(density, opacity, margin, floor)

    def desc(self, density: torch.Tensor, opacity: torch.Tensor) -> C.er_medium_desc:
        assert density.is_cuda and density.dtype == torch.float32 and density.is_contiguous()
        assert opacity.is_cuda and opacity.dtype == torch.float32 and opacity.is_contiguous()
        if tuple(density.shape) != self.shape or opacity.numel() != self.n_opacity:
            raise ValueError("density or opacity shape differs from the medium's")
        d = C.er_medium_desc()
        d.d_density = density.data_ptr()
        d.d_opacity = opacity.data_ptr()
        d.n_opacity = opacity.numel()
        d.scale = self.scale
        for i in range(3):
            d.albedo[i] = self.albedo[i]
        d.nee_probability = self.q
        d.d_majorant = self.majorant.data_ptr()
        d.brick = self.brick
        d.model = self.model
        d.gradient_magnitude_inv = self.gm_inv
        return d

    def rebuild_majorant(self, density, opacity, margin=1.25, floor=1e-3):
        d = self.desc(density.detach(), opacity.detach())
        C.check(self.lib.er_medium_majorant(self.r.tracer_id, byref(d), margin, floor, self.majorant.data_ptr(),
                                            ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)))

    def render_samples(self, density, opacity, spp, view=0, first=0):
        """(samples (spp, H, W, 3), per-pixel sums (H, W, 3))"""
        H, W = self.r.height, self.r.width
        smp = torch.empty((spp, H, W, 3), dtype=torch.float32, device=density.device)
        s = torch.empty((H, W, 3), dtype=torch.float32, device=density.device)
        d = self.desc(density, opacity)
        C.check(self.lib.er_medium_render(self.r.tracer_id, byref(d), spp, view, first, smp.data_ptr(), s.data_ptr(),
                                          ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)))
        return smp, s

    def render_sums64(self, density, opacity, spp, view=0, first=0):
        """per-pixel sums (H, W, 3) of the binary64 evaluation of the same samples"""
        H, W = self.r.height, self.r.width
        smp = torch.empty((spp, H, W, 3), dtype=torch.float64, device=density.device)
        s = torch.empty((H, W, 3), dtype=torch.float64, device=density.device)
        d = self.desc(density, opacity)
        C.check(self.lib.er_medium_render_f64(self.r.tracer_id, byref(d), spp, view, first, smp.data_ptr(), s.data_ptr(),
                                              ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)))
        return s

    def adjoint(self, density, opacity, spp, dloss_dsum, samples=None, view=0, first=0):
        """(dLoss/d density, dLoss/d opacity) given dLoss/d(pixel sums)"""
        g_rho = torch.zeros_like(density)
        g_tf = torch.zeros_like(opacity)
        d = self.desc(density, opacity)
        dl = dloss_dsum.contiguous().float()
        C.check(self.lib.er_medium_adjoint(self.r.tracer_id, byref(d), spp, view, first, dl.data_ptr(),
                                           samples.data_ptr() if samples is not None else None, g_rho.data_ptr(),
                                           g_tf.data_ptr(), ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)))
        return g_rho, g_tf

    def __call__(self, density, opacity, spp, view=0, first=0):
        return RenderMedium.apply(density, opacity, self, spp, view, first)


class RenderMedium(torch.autograd.Function):
    """image mean (H, W, 3) of spp samples per pixel; backward = the adjoint kernel"""

    @staticmethod
    def forward(ctx, density, opacity, medium, spp, view, first):
        density = density.detach().contiguous()
        opacity = opacity.detach().contiguous()
        smp, s = medium.render_samples(density, opacity, spp, view, first)
        ctx.medium, ctx.spp, ctx.view, ctx.first = medium, spp, view, first
        ctx.save_for_backward(density, opacity, smp if medium.keep_samples else torch.empty(0))
        return s / spp

    @staticmethod
    def backward(ctx, grad_img):
        density, opacity, smp = ctx.saved_tensors
        m = ctx.medium
        g_rho, g_tf = m.adjoint(density, opacity, ctx.spp, grad_img / ctx.spp, smp if smp.numel() else None, ctx.view, ctx.first)
        return g_rho, g_tf, None, None, None, None
