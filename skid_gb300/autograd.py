"""torch.autograd.Function wrappers of the density and group-potential
adjoints.

Thin on purpose: every forward and every backward is one libskidgpu call
through the ctypes binding, and torch only carries the tensors (there is no
torch arithmetic on the path).  Used to check the hand-written adjoint
kernels in a framework's own autograd loop.

    rho = sph_density(pos, mass, nSmooth=64, period=1.0)
    (w * rho).sum().backward()          # pos.grad = d/dx sum w_i rho_i

    E = group_potential(pos, mass, soft, grp, sel, G=1.0)
    (v * E).sum().backward()            # pos.grad = d/dx sum v_s E_s
"""
from __future__ import annotations

import numpy as np
import torch

from . import gpu, tipsy


def _snapshot(pos: np.ndarray, mass: np.ndarray, soft: np.ndarray | None = None) -> tipsy.Snapshot:
    n = len(pos)
    soft = np.zeros(n, np.float32) if soft is None else soft
    return tipsy.Snapshot(0.0, 0, n, 0, pos, np.zeros((n, 3), np.float32), mass, soft,
                          np.zeros(n, np.float32))


def _np32(t: torch.Tensor, shape=None) -> np.ndarray:
    a = np.ascontiguousarray(t.detach().cpu().numpy(), np.float32)
    return a.reshape(shape) if shape is not None else a


class SPHDensity(torch.autograd.Function):
    """rho_i of skid_density over dark-matter particles at pos (n, 3); the
    backward pass is skid_density_adjoint."""

    @staticmethod
    def forward(ctx, pos, mass, nSmooth=64, period=None, mode=gpu.ADJ_AUTO):
        snap = _snapshot(_np32(pos, (-1, 3)), _np32(mass))
        g = gpu.Context(period=period, nSmooth=nSmooth)
        g.set_particles(snap)
        g.scatter_active(False, False)
        g.density()
        rho, _ = g.get_density()
        ctx.skid = g
        ctx.mode = mode
        return torch.from_numpy(rho).to(pos.device)

    @staticmethod
    def backward(ctx, grad_rho):
        d = ctx.skid.density_adjoint(_np32(grad_rho), ctx.mode)
        ctx.skid.close()
        return torch.from_numpy(d).to(grad_rho.device), None, None, None, None


class GroupPotential(torch.autograd.Function):
    """Potential energy E_s (FP64) of the groups sel of the grouping grp
    (ids by particle, 0 = none), centres from the centre of mass; the
    backward pass is skid_potential_adjoint."""

    @staticmethod
    def forward(ctx, pos, mass, soft, grp, sel, G=1.0, soft_type=2, period=None):
        snap = _snapshot(_np32(pos, (-1, 3)), _np32(mass), _np32(soft))
        g = gpu.Context(period=period, nSmooth=2)
        g.set_particles(snap)
        g.set_groups(np.ascontiguousarray(grp.detach().cpu().numpy(), np.int32))
        s = np.ascontiguousarray(sel.detach().cpu().numpy(), np.int32)
        E, _ = g.potential_adjoint(s, None, G=G, soft_type=soft_type)
        ctx.skid, ctx.sel, ctx.G, ctx.soft_type = g, s, G, soft_type
        return torch.from_numpy(E).to(pos.device)

    @staticmethod
    def backward(ctx, grad_E):
        v = _np32(grad_E)
        _, d = ctx.skid.potential_adjoint(ctx.sel, v, G=ctx.G, soft_type=ctx.soft_type)
        ctx.skid.close()
        return torch.from_numpy(d).to(grad_E.device), None, None, None, None, None, None, None


def sph_density(pos, mass, nSmooth=64, period=None, mode=gpu.ADJ_AUTO):
    return SPHDensity.apply(pos, mass, nSmooth, period, mode)


def group_potential(pos, mass, soft, grp, sel, G=1.0, soft_type=2, period=None):
    return GroupPotential.apply(pos, mass, soft, grp, sel, G, soft_type, period)
