"""torch.autograd binding of the blob-window adjoint.

``window(mesh, material, x0, steps, every, **params)`` runs ``steps`` CG_nomass
steps of ``mesh`` with per-element SI ``material`` (the columns of
``Mesh.material``: density, shear viscosity, bulk viscosity, shear modulus,
bulk modulus, dielectric) from positions ``x0`` (meso units, all nodes) and
returns the final positions. ``material`` and ``x0`` may require grad: the
backward pass is the C ABI's adjoint (ffea_gpu_adjoint_backward), one adjoint
CG solve per step with the noise replayed from the same stream. Density and
dielectric do not enter a CG_nomass step, so their gradient is zero.

Device memory: the blob and its checkpoints live only as long as a backward
pass can still need them. A forward whose inputs need no gradient (or that
runs under ``torch.no_grad``) frees them before it returns; otherwise they are
freed by the backward pass, or when the graph that holds them is dropped.
"""
from __future__ import annotations

import copy

import numpy as np
import torch

from . import lib


class _Window:
    """The device state of one differentiated window: the blob and its adjoint (checkpoints). ``release``
    frees both (adjoint first) and may be called more than once; dropping the last reference releases too."""

    def __init__(self, blob: lib.Blob, adj: lib.Adjoint):
        self.blob, self.adj = blob, adj

    def release(self) -> None:
        if self.adj is not None:
            self.adj.close()
            self.adj = None
        if self.blob is not None:
            self.blob.close()
            self.blob = None

    def __del__(self):
        self.release()


class BlobWindow(torch.autograd.Function):
    @staticmethod
    def forward(ctx, material: torch.Tensor, x0: torch.Tensor, mesh, steps: int, every: int, params: dict,
                keep: bool):
        m = copy.copy(mesh)
        m.material = material.detach().cpu().numpy().astype(np.float64)
        blob = lib.Blob(m, solver="CG_nomass", **params)
        w = _Window(blob, None)
        blob.set_state(pos=x0.detach().cpu().numpy())
        w.adj = lib.Adjoint(blob, steps, every)
        w.adj.forward()
        out = torch.from_numpy(blob.pos()).to(x0.dtype)
        if keep:
            ctx.window = w  # freed by backward, or with the graph (ctx) if backward never runs
        else:
            w.release()
        return out

    @staticmethod
    def backward(ctx, grad_out: torch.Tensor):
        w = ctx.window
        g = w.adj.backward(grad_out.detach().cpu().numpy())
        w.release()
        si = lib.meso_to_si_gradients(g)
        gm = np.zeros((len(g["G"]), 6))
        gm[:, 1], gm[:, 2], gm[:, 3], gm[:, 4] = si["shear_visc"], si["bulk_visc"], si["shear_mod"], si["bulk_mod"]
        return torch.from_numpy(gm), torch.from_numpy(g["x0"]), None, None, None, None, None


def window(mesh, material: torch.Tensor, x0: torch.Tensor, steps: int, every: int, **params) -> torch.Tensor:
    """Final positions after ``steps`` steps; differentiable in ``material`` and ``x0``."""
    # forward runs with grad mode off, so whether a backward can follow is decided here
    keep = torch.is_grad_enabled() and (material.requires_grad or x0.requires_grad)
    return BlobWindow.apply(material, x0, mesh, steps, every, params, keep)
