"""Central-difference check of the std and VE adjoints at the adjoint configuration's full size.

Workload: 100^3 = 1,000,000 particles on a jittered periodic lattice (+-0.3 spacing, seed 5), density
from a seeded sum of Fourier modes (seed 55), velocities N(0, 0.1^2) per component (seed 555), and a
target density from an independent Fourier field (seed 5555).  Loss L = sum_i (rho_i - rho_target_i)^2
+ sum_i |a_i|^2 on the neighbour lists frozen after one search.

The FP64 forward runs with the smooth kernel form (sphgb_set_kernel_form: W and dW/dv continuously
differentiable), so the only kinks left are the branches of the physics (artificial viscosity, AV
switch, Atwood ramp, max(0, .), signal-velocity maxima, the avClean clamp).  The adjoint's gradient
comes from the default forms (one evaluation per mutual pair, forward tape); the central differences
from the deterministic forward (bitwise reproducible sums).  64 coordinates are drawn from
PCG64(55555) over (x y z vx vy vz h u) x particles, eps = 1e-6 (times h for h); each
coordinate whose +-eps / +-2 eps stencil straddles a kink of the forward is reported and replaced by
the next draw (tests/fd_check.py).  Bar: |adjoint - central difference| <= 1e-6 |central difference|
on every one of the 64 checked coordinates, positions and smoothing lengths included.
"""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

BAR = 1e-6


def _setup(chain, av_clean=False):
    import torch
    from sphexa_gb300 import autograd as AG, sph, workloads as W
    wl = W.fourier(100, seed=5, rho_seed=55, v_seed=555, target_seed=5555)
    ctx = sph.Context(0)
    ctx.set_kernel_form(True)
    d = sph.ParticlesData.from_workload(wl, "fp64", "cuda:0", av_clean=av_clean)
    box = sph.Box(wl.box.copy(), wl.bc.copy())
    if chain == "std":
        sw = AG.FrozenStdSweep(ctx, d, box)
    else:
        sw = AG.FrozenVeSweep(ctx, d, box, av_clean=av_clean)
    sw.freeze()
    order = sph.Domain(ctx, box).order(wl.n)
    rho_t = torch.tensor(wl.fields["rho_target"][order], dtype=torch.float64, device="cuda:0")
    return wl, ctx, sw, rho_t


@pytest.mark.parametrize("chain,av_clean", [("std", False), ("ve", False), ("ve", True)])
def test_adjoint_matches_central_differences_at_1M(chain, av_clean):
    from fd_check import adjoint_gradient, fd_check, report
    wl, ctx, sw, rho_t = _setup(chain, av_clean)
    assert wl.n == 1_000_000
    grads = adjoint_gradient(sw, rho_t, [t.detach().clone() for t in sw.inputs()])
    ctx.set_deterministic(True)
    rows, straddles = fd_check(sw, rho_t, wl.n, grads)
    report(rows, straddles, f"{chain} chain{' avClean' if av_clean else ''}, 1M particles")
    assert len(rows) == 64
    assert {r[0] for r in rows} >= {"x", "y", "z", "h"}
    worst = max(rows, key=lambda r: r[4])
    assert worst[4] <= BAR, f"{worst[0]} of particle {worst[1]}: adjoint {worst[2]:.12e} vs FD {worst[3]:.12e}"
    ctx.close()


def test_smooth_form_stays_close_to_the_table_form():
    """the smooth kernel form changes the forward by the table's interpolation error only"""
    import torch
    from sphexa_gb300 import sph, workloads as W
    wl = W.fourier(20, seed=5, rho_seed=55, v_seed=555)
    out = {}
    for smooth in (False, True):
        ctx = sph.Context(0)
        ctx.set_kernel_form(smooth)
        d = sph.ParticlesData.from_workload(wl, "fp64", "cuda:0")
        sph.sweep(ctx, d, sph.Box(wl.box.copy(), wl.bc.copy()), "ve", False)
        out[smooth] = {k: d.f[k].cpu().numpy() for k in ("rho", "c11", "divv", "alpha", "ax", "du")}
        ctx.close()
    for k in out[False]:
        a, b = out[True][k], out[False][k]
        err = np.max(np.abs(a - b)) / np.max(np.abs(b))
        print(f"smooth vs table {k:5s}: {err:.2e}")
        assert err <= 1e-6, k
