"""torch.autograd binding of the blob-window adjoint.

``window(mesh, material, x0, steps, every, **params)`` runs ``steps`` CG_nomass
steps of ``mesh`` with per-element SI ``material`` (the columns of
``Mesh.material``: density, shear viscosity, bulk viscosity, shear modulus,
bulk modulus, dielectric) from positions ``x0`` (meso units, all nodes) and
returns the final positions. ``material`` and ``x0`` may require grad: the
backward pass is the C ABI's adjoint (ffea_gpu_adjoint_backward), one adjoint
CG solve per step with the noise replayed from the same stream. Density and
dielectric do not enter a CG_nomass step, so their gradient is zero.
"""
from __future__ import annotations

import copy

import numpy as np
import torch

from . import lib


class BlobWindow(torch.autograd.Function):
    @staticmethod
    def forward(ctx, material: torch.Tensor, x0: torch.Tensor, mesh, steps: int, every: int, params: dict):
        m = copy.copy(mesh)
        m.material = material.detach().cpu().numpy().astype(np.float64)
        blob = lib.Blob(m, solver="CG_nomass", **params)
        blob.set_state(pos=x0.detach().cpu().numpy())
        adj = lib.Adjoint(blob, steps, every)
        adj.forward()
        ctx.blob, ctx.adj = blob, adj
        return torch.from_numpy(blob.pos()).to(x0.dtype)

    @staticmethod
    def backward(ctx, grad_out: torch.Tensor):
        g = ctx.adj.backward(grad_out.detach().cpu().numpy())
        si = lib.meso_to_si_gradients(g)
        gm = np.zeros((len(g["G"]), 6))
        gm[:, 1], gm[:, 2], gm[:, 3], gm[:, 4] = si["shear_visc"], si["bulk_visc"], si["shear_mod"], si["bulk_mod"]
        ctx.adj.close()
        ctx.blob.close()
        return torch.from_numpy(gm), torch.from_numpy(g["x0"]), None, None, None, None


def window(mesh, material: torch.Tensor, x0: torch.Tensor, steps: int, every: int, **params) -> torch.Tensor:
    """Final positions after ``steps`` steps; differentiable in ``material`` and ``x0``."""
    return BlobWindow.apply(material, x0, mesh, steps, every, params)
