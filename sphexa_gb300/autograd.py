"""torch.autograd harness over the hand-written adjoint (sphgb_adjoint_std).

A thin test/analysis harness: the forward runs the std pair passes (density, EOS, IAD,
momentum-energy) through the C ABI on the neighbour lists frozen by ``FrozenStdSweep.freeze``,
and the backward calls the adjoint kernels.  Gradients are taken with respect to positions,
velocities, smoothing lengths and internal energy; masses are constants.
"""

from __future__ import annotations

import ctypes as C

import torch

from . import _lib, sph
from ._lib import check


class FrozenStdSweep:
    """Context + particle set whose SFC order, tree and neighbour lists are fixed at freeze()."""

    def __init__(self, ctx: sph.Context, d: sph.ParticlesData, box: sph.Box, deterministic: bool = False):
        if d.precision != "fp64":
            raise ValueError("the adjoint runs in the FP64 form")
        self.ctx, self.d, self.box = ctx, d, box
        self.deterministic = deterministic

    def freeze(self) -> None:
        """domain sync + neighbour search; afterwards the order and the lists stay as they are."""
        sph.Domain(self.ctx, self.box).sync(self.d)
        sph.find_neighbors_sfc(self.ctx, 0, self.d.n, self.d)

    def inputs(self) -> tuple[torch.Tensor, ...]:
        f = self.d.f
        return tuple(f[k].clone() for k in ("x", "y", "z", "vx", "vy", "vz", "h", "u"))

    def forward(self, x, y, z, vx, vy, vz, h, u):
        f = self.d.f
        for k, t in zip(("x", "y", "z", "vx", "vy", "vz", "h", "u"), (x, y, z, vx, vy, vz, h, u)):
            f[k].copy_(t.detach())
        sph.compute_density(self.ctx, self.d)
        sph.compute_eos_hydro_std(self.ctx, self.d)
        sph.compute_iad(self.ctx, self.d)
        sph.compute_momentum_energy_std(self.ctx, self.d)
        return tuple(f[k].clone() for k in ("rho", "ax", "ay", "az", "du"))

    def backward(self, g_rho, g_ax, g_ay, g_az, g_du):
        n = self.d.n
        dev = self.d.device
        seeds = _lib.SphgbSeeds()
        keep = []
        for name, g in (("rho", g_rho), ("ax", g_ax), ("ay", g_ay), ("az", g_az), ("du", g_du)):
            if g is not None:
                g = g.detach().to(torch.float64).contiguous()
                keep.append(g)
                setattr(seeds, name, g.data_ptr())
        out = {k: torch.zeros(n, dtype=torch.float64, device=dev) for k in ("x", "y", "z", "vx", "vy", "vz", "h", "u")}
        grads = _lib.SphgbGrads()
        for k, t in out.items():
            setattr(grads, k, t.data_ptr())
        s = self.d.c_struct()
        check(self.ctx.lib.sphgb_adjoint_std(self.ctx.h, C.byref(s), C.byref(seeds), C.byref(grads),
                                            int(self.deterministic)),
              "sphgb_adjoint_std")
        return tuple(out[k] for k in ("x", "y", "z", "vx", "vy", "vz", "h", "u"))


class StdSweepFunction(torch.autograd.Function):
    """(x, y, z, vx, vy, vz, h, u) -> (rho, ax, ay, az, du) on frozen lists, with the adjoint backward."""

    @staticmethod
    def forward(fctx, sweep: FrozenStdSweep, x, y, z, vx, vy, vz, h, u):
        fctx.sweep = sweep
        return sweep.forward(x, y, z, vx, vy, vz, h, u)

    @staticmethod
    def backward(fctx, g_rho, g_ax, g_ay, g_az, g_du):
        grads = fctx.sweep.backward(g_rho, g_ax, g_ay, g_az, g_du)
        return (None,) + grads


def loss_rho_a(rho, ax, ay, az, rho_target):
    """L = sum_i (rho_i - rho_target_i)^2 + sum_i |a_i|^2"""
    return ((rho - rho_target) ** 2).sum() + (ax * ax + ay * ay + az * az).sum()
