"""torch.autograd harness over the hand-written adjoints (sphgb_adjoint_std, sphgb_adjoint_ve).

A thin test/analysis harness: the forward runs the std pair passes (density, EOS, IAD,
momentum-energy) or the VE pair passes (xmass, gradh, EOS, IAD + divv/curlv, AV switches,
momentum-energy) through the C ABI on the neighbour lists frozen by ``freeze``, and the backward
calls the adjoint kernels.  Gradients are taken with respect to positions, velocities, smoothing
lengths and internal energy; masses and the alpha before the AV switch are constants.
"""

from __future__ import annotations

import ctypes as C

import torch

from . import _lib, sph
from ._lib import check


class FrozenStdSweep:
    """Context + particle set whose SFC order, tree and neighbour lists are fixed at freeze()."""

    def __init__(self, ctx: sph.Context, d: sph.ParticlesData, box: sph.Box, deterministic: bool = False):
        # the std adjoint runs in both forms (mixed: FP32 pair arithmetic, scatter form only)
        if d.precision not in ("fp64", "mixed") or (deterministic and d.precision != "fp64"):
            raise ValueError("the std adjoint runs in the FP64 form, or in the mixed form without deterministic")
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
        return _run_adjoint(self, g_rho, g_ax, g_ay, g_az, g_du, "sphgb_adjoint_std",
                            lambda s, seeds, grads: (C.byref(s), C.byref(seeds), C.byref(grads),
                                                     int(self.deterministic)))


def _run_adjoint(sweep, g_rho, g_ax, g_ay, g_az, g_du, fn, args):
    """call the adjoint entry ``fn`` with the output seeds; returns the input gradients"""
    n = sweep.d.n
    dev = sweep.d.device
    seeds = _lib.SphgbSeeds()
    keep = []
    for name, g in (("rho", g_rho), ("ax", g_ax), ("ay", g_ay), ("az", g_az), ("du", g_du)):
        if g is not None:  # seeds in the output field's type (du is FP64 in both forms)
            g = g.detach().to(sweep.d.f[name].dtype).contiguous()
            keep.append(g)
            setattr(seeds, name, g.data_ptr())
    out = {k: torch.zeros(n, dtype=torch.float64, device=dev) for k in ("x", "y", "z", "vx", "vy", "vz", "h", "u")}
    grads = _lib.SphgbGrads()
    for k, t in out.items():
        setattr(grads, k, t.data_ptr())
    s = sweep.d.c_struct()
    check(getattr(sweep.ctx.lib, fn)(sweep.ctx.h, *args(s, seeds, grads)), fn)
    # FP64 gradients, returned in each input's type (float for the mixed form's h and v)
    return tuple(out[k].to(sweep.d.f[k].dtype) for k in ("x", "y", "z", "vx", "vy", "vz", "h", "u"))


class FrozenVeSweep(FrozenStdSweep):
    """VE chain on frozen lists.  The alpha before the AV switch is kept from freeze() on, so that
    every forward starts from the same alpha; av_clean selects momentumAndEnergy<avClean>.  With
    tape (default) the context's forward passes keep the sums the backward needs
    (sphgb_set_adjoint_tape); the backward then reads them from the last forward."""

    def __init__(self, ctx, d, box, av_clean: bool = False, deterministic: bool = False, tape: bool = True):
        if d.precision != "fp64":
            raise ValueError("the VE adjoint runs in the FP64 form")
        super().__init__(ctx, d, box, deterministic)
        self.av_clean = av_clean
        self.alpha0 = None
        ctx.set_adjoint_tape(tape)

    def freeze(self) -> None:
        super().freeze()
        self.alpha0 = self.d.f["alpha"].clone()

    def forward(self, x, y, z, vx, vy, vz, h, u):
        f = self.d.f
        for k, t in zip(("x", "y", "z", "vx", "vy", "vz", "h", "u"), (x, y, z, vx, vy, vz, h, u)):
            f[k].copy_(t.detach())
        f["alpha"].copy_(self.alpha0)
        sph.compute_xmass(self.ctx, self.d)
        sph.compute_ve_def_gradh(self.ctx, self.d)
        sph.compute_eos(self.ctx, self.d)
        sph.compute_iad_divv_curlv(self.ctx, self.d)
        sph.compute_av_switches(self.ctx, self.d)
        sph.compute_momentum_energy(self.ctx, self.d, self.av_clean)
        return tuple(f[k].clone() for k in ("rho", "ax", "ay", "az", "du"))

    def backward(self, g_rho, g_ax, g_ay, g_az, g_du):
        a0 = self.alpha0
        return _run_adjoint(self, g_rho, g_ax, g_ay, g_az, g_du, "sphgb_adjoint_ve",
                            lambda s, seeds, grads: (C.byref(s), a0.data_ptr(), int(self.av_clean), C.byref(seeds),
                                                     C.byref(grads), int(self.deterministic)))


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


class VeSweepFunction(StdSweepFunction):
    """(x, y, z, vx, vy, vz, h, u) -> (rho, ax, ay, az, du) of the VE chain on frozen lists."""


def loss_rho_a(rho, ax, ay, az, rho_target):
    """L = sum_i (rho_i - rho_target_i)^2 + sum_i |a_i|^2"""
    return ((rho - rho_target) ** 2).sum() + (ax * ax + ay * ay + az * az).sum()
