"""Levis approximate gradient and its automatic-differentiation wrapper.

``levis_approximation_grad`` mirrors
``at3d.gradient.LevisApproxGradient.levis_approximation_grad``
(at3d/gradient.py:164-415) for one solver and one sensor with one ray per
pixel, the L2 cost and unit uncertainties: it returns the gradient of the
cost with respect to the extinction and single-scattering albedo of one
species on the property grid, the cost and the rendered radiances.  The
derivative is the reference's Levis approximation (the radiance field is
frozen; LEVISAPPROX_GRADIENT, src/polarized/shdomsub4.f:288-809) computed
by the GPU adjoint behind ``shdom_levis_gradient``.

``LevisRender`` is a ``torch.autograd.Function``: its forward renders the
frozen solution along the rays, its backward runs the same adjoint with
the incoming gradient as ray weights (``shdom_levis_adjoint``) and returns
d/d(extinction) and d/d(albedo).
"""
from __future__ import annotations

import numpy as np

from .solver import RTE


def levis_approximation_grad(rte_solver: RTE, sensor: dict, measurements, species: int = 0,
                             cost_function: str = "L2"):
    """(gradient [npx, npy, npz, 2] (extinction, ssalb), loss, radiances)."""
    if cost_function != "L2":
        raise NotImplementedError("only the L2 cost function is supported")
    rays = (sensor["ray_x"], sensor["ray_y"], sensor["ray_z"], sensor["ray_mu"], sensor["ray_phi"])
    grad, loss, radiances = rte_solver.levis_gradient(rays, measurements, species)
    return grad, loss, radiances


def _torch():
    import torch
    return torch


class _LevisRenderFn:
    """Built lazily so that importing this module does not import torch."""
    cls = None

    @classmethod
    def get(cls):
        if cls.cls is None:
            torch = _torch()

            class LevisRender(torch.autograd.Function):
                @staticmethod
                def forward(ctx, extinction, ssalb, rte, rays, species):
                    x, y, z, mu, phi = rays
                    out = rte.render(x, y, z, mu, phi)
                    ctx.rte, ctx.rays, ctx.species = rte, rays, species
                    ctx.shape = tuple(extinction.shape)
                    ctx.device, ctx.dtype = extinction.device, extinction.dtype
                    return torch.as_tensor(out, device=extinction.device, dtype=extinction.dtype)

                @staticmethod
                def backward(ctx, grad_out):
                    w = grad_out.detach().to("cpu", torch.float64).numpy()
                    g = ctx.rte.levis_adjoint(ctx.rays, w, ctx.species)
                    g = torch.as_tensor(g, device=ctx.device, dtype=ctx.dtype)
                    return g[..., 0].reshape(ctx.shape), g[..., 1].reshape(ctx.shape), None, None, None

            cls.cls = LevisRender
        return cls.cls


def render_differentiable(rte: RTE, extinction, ssalb, rays, species: int = 0):
    """Radiances along `rays` from the solved (frozen) field, differentiable
    with respect to `extinction` and `ssalb` (torch tensors shaped like the
    species' property grid) through the Levis adjoint."""
    return _LevisRenderFn.get().apply(extinction, ssalb, rte, tuple(rays), species)
