"""torch.autograd.Function over crt_render / crt_adjoint_lambert.

Differentiable Lambert rendering with respect to the vertex positions, the
light position and the per-material albedo (kd).  The forward pass is the
ordinary pixel kernel (double mean colour, ``rgb_f64``); the backward pass is
the hand-written adjoint kernel, which recomputes each tile's hits instead of
storing them.  Interior gradients only: visibility (which triangle a sample
hits, whether its shadow ray is blocked) is held fixed.

This wrapper exists to check the adjoint (against central finite differences
and the oracle's float64 gradient); the kernels themselves are reachable from
C through include/crt.h.
"""
from __future__ import annotations

import numpy as np
import torch

from . import Scene
from .data import Light


class LambertRender(torch.autograd.Function):
    """image = LambertRender.apply(verts, light_pos, albedo, ctx_obj)

    verts: (V, 3) float32 CUDA tensor; light_pos: (3,) float64; albedo: (M, 3)
    float64 (the kd of every material).  Returns the (H*W, 3) float64 mean
    colour in the reference's bottom-up pixel order and the (H*W,) mean depth."""

    @staticmethod
    def forward(ctx, verts, light_pos, albedo, r):
        r.set_inputs(verts, light_pos, albedo)
        img, depth = r.forward()
        ctx.r = r
        ctx.devs = (verts.device, light_pos.device, albedo.device)
        return img, depth

    @staticmethod
    def backward(ctx, grad_img, grad_depth):
        r = ctx.r
        g = r.adjoint(grad_img, grad_depth)
        dv, dl, da = ctx.devs
        return g["vertices"].to(dv, torch.float32), g["light"].to(dl), g["kd"].to(da), None


class Renderer:
    """Holds the scene and the fixed camera/image parameters for LambertRender."""

    def __init__(self, mesh, camera, light, width, height, spp):
        self.scene = Scene(mesh)
        self.mats = np.ascontiguousarray(np.asarray(mesh.materials, np.float64).reshape(-1, 16)).copy()
        self.camera, self.light = camera, light
        self.W, self.H, self.spp = width, height, spp

    def set_inputs(self, verts, light_pos, albedo):
        self.scene.set_vertices(verts.detach().contiguous(), rebuild=True)
        self.mats[:, 3:6] = albedo.detach().cpu().numpy()
        self.scene.set_materials(self.mats)
        lp = tuple(float(x) for x in light_pos.detach().cpu().numpy())
        self.cur_light = Light(position=lp, color=self.light.color, radius=self.light.radius,
                               constant_term=self.light.constant_term, linear_term=self.light.linear_term,
                               quadratic_term=self.light.quadratic_term)

    def forward(self):
        n = self.W * self.H
        img = torch.empty((n, 3), dtype=torch.float64, device="cuda")
        depth = torch.empty(n, dtype=torch.float64, device="cuda")
        self.scene.render(self.camera, self.cur_light, self.W, self.H, self.spp, out={"rgb_f64": img, "depth": depth})
        return img, depth

    def adjoint(self, grad_img, grad_depth=None):
        dev = "cuda"
        out = dict(vertices=torch.zeros((self.scene.nv, 3), dtype=torch.float64, device=dev),
                   light=torch.zeros(3, dtype=torch.float64, device=dev),
                   kd=torch.zeros((self.scene.nmat, 3), dtype=torch.float64, device=dev))
        gd = None if grad_depth is None else grad_depth.contiguous().to(torch.float64)
        self.scene.adjoint(self.camera, self.cur_light, self.W, self.H, self.spp,
                           grad_img.contiguous().to(torch.float64), gd, out=out)
        return out


def render(verts, light_pos, albedo, renderer: Renderer):
    return LambertRender.apply(verts, light_pos, albedo, renderer)
