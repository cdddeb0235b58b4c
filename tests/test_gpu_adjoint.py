"""The hand-written adjoint of the std chain against an FP64 reference gradient and FP64 central
differences.

Workload: the adjoint configuration's generator (jittered periodic lattice, Fourier density
field, Gaussian velocities, an independent target density field) at 10^3 to 12^3 particles.  Loss
L = sum (rho - rho_target)^2 + sum |a|^2 on the frozen neighbour lists.

* Reference gradient: torch autograd through the FP64 torch restatement of the same chain on the
  same edges (tests/torch_reference.py), in both kernel forms (the reference's linear table and the
  smooth cubic pieces); bar normwise 1e-9 per field.
* Central differences: smooth kernel form, eps = 1e-6 (times h for h), 64 coordinates from
  PCG64(55555); a coordinate whose stencil straddles a kink of the forward (the viscosity branch) is
  reported and replaced by the next draw (tests/fd_check.py).  Bar: relative agreement <= 1e-6 on
  every checked coordinate.  The full-size version (1M particles) is tests/test_gpu_adjoint_fd.py.
"""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FIELDS = ("x", "y", "z", "vx", "vy", "vz", "h", "u")


def setup(side=12, seed=5, deterministic=False, ordered_forward=False, precision="fp64", smooth=False):
    import torch
    from sphexa_gb300 import autograd as AG, sph, workloads as W
    wl = W.fourier(side, seed=seed, rho_seed=55, v_seed=555, target_seed=5555)
    ctx = sph.Context(0)
    ctx.set_kernel_form(smooth)
    if ordered_forward:  # the scatter adjoint then walks the full lists (no owned lists in use)
        ctx.set_deterministic(True)
    d = sph.ParticlesData.from_workload(wl, precision, "cuda:0")
    box = sph.Box(wl.box.copy(), wl.bc.copy())
    sw = AG.FrozenStdSweep(ctx, d, box, deterministic=deterministic)
    sw.freeze()
    order = sph.Domain(ctx, box).order(wl.n)
    rho_t = torch.tensor(wl.fields["rho_target"][order], dtype=torch.float64, device="cuda:0")
    return wl, ctx, sw, rho_t


def loss_of(sw, rho_t, vals):
    from sphexa_gb300 import autograd as AG
    rho, ax, ay, az, du = sw.forward(*vals)
    return float(AG.loss_rho_a(rho, ax, ay, az, rho_t).item())


@pytest.mark.parametrize("smooth", [False, True])
@pytest.mark.parametrize("form", ["pair-once", "scatter", "two-sided"])
def test_adjoint_matches_fp64_reference_gradient(port, form, smooth):
    """Every gradient component of every particle against torch autograd through the FP64 torch
    restatement of the same chain on the same frozen edges (tests/torch_reference.py).  pair-once:
    one evaluation per mutual pair of the owned lists; scatter: every list entry once with atomics;
    two-sided: the bit-reproducible form."""
    import torch
    from sphexa_gb300 import autograd as AG, sph
    from torch_reference import std_chain
    wl, ctx, sw, rho_t = setup(side=10, seed=7, deterministic=form == "two-sided", ordered_forward=form == "scatter",
                               smooth=smooth)
    n = wl.n
    ng = int(ctx.params.ngmax)
    nb = sph.export_neighbors(ctx, n, ng).cpu().numpy().reshape(n, ng).astype(np.int64)
    cnt = np.minimum(sw.d.nc.cpu().numpy().astype(np.int64) - 1, ng)
    ei = np.repeat(np.arange(n), cnt)
    ej = np.concatenate([nb[k, :cnt[k]] for k in range(n)])
    dev = "cuda:0"
    ei_t, ej_t = torch.tensor(ei, device=dev), torch.tensor(ej, device=dev)
    if smooth:
        from torch_reference import hermite_tables
        wh, _ = hermite_tables(6.0)
    else:
        wh, _ = port.tables(6.0)
    tab = torch.tensor(wh, dtype=torch.float64, device=dev)
    inp = [t.clone().requires_grad_(True) for t in sw.inputs()]
    m = sw.d.m.clone()
    out_ref = std_chain(*inp, m, ei_t, ej_t, tab, ctx.K, float(ctx.params.gamma),
                        torch.tensor(wl.box[1::2] - wl.box[0::2], dtype=torch.float64), [True, True, True])
    L_ref = AG.loss_rho_a(*out_ref[:4], rho_t)
    L_ref.backward()
    g_ref = {f: inp[k].grad.detach().cpu().numpy() for k, f in enumerate(FIELDS)}

    base = [t.detach().clone().requires_grad_(True) for t in sw.inputs()]
    out = AG.StdSweepFunction.apply(sw, *base)
    for a, b in zip(out, out_ref):
        ref = b.detach().cpu().numpy()
        assert np.max(np.abs(a.detach().cpu().numpy() - ref)) <= 1e-10 * (np.max(np.abs(ref)) + 1e-300)
    L = AG.loss_rho_a(*out[:4], rho_t)
    L.backward()
    for k, f in enumerate(FIELDS):
        g = base[k].grad.detach().cpu().numpy()
        err = np.linalg.norm(g - g_ref[f]) / (np.linalg.norm(g_ref[f]) + 1e-300)
        print(f"reference gradient {f:3s}: normwise rel {err:.3e}")
        assert err <= 1e-9, f
    ctx.close()


def test_deterministic_adjoint_is_bit_reproducible():
    import torch
    wl, ctx, sw, rho_t = setup(side=10, seed=9, deterministic=True)
    vals = sw.inputs()
    rho, ax, ay, az, du = sw.forward(*vals)
    seeds = (2.0 * (rho - rho_t), 2.0 * ax, 2.0 * ay, 2.0 * az, None)
    g1 = [t.cpu().numpy() for t in sw.backward(*seeds)]
    g2 = [t.cpu().numpy() for t in sw.backward(*seeds)]
    for a, b in zip(g1, g2):
        np.testing.assert_array_equal(a, b)
    ctx.close()


def test_adjoint_matches_central_differences():
    from fd_check import adjoint_gradient, fd_check, report
    wl, ctx, sw, rho_t = setup(smooth=True)
    grads = adjoint_gradient(sw, rho_t, [t.detach().clone() for t in sw.inputs()])
    ctx.set_deterministic(True)  # bitwise reproducible forward for the differences
    rows, straddles = fd_check(sw, rho_t, wl.n, grads)
    report(rows, straddles, "std chain, 12^3")
    assert len(rows) == 64
    worst = max(rows, key=lambda r: r[4])
    assert worst[4] <= 1e-6, worst
    ctx.close()


def test_mixed_adjoint_matches_fp64_gradient():
    """The mixed form's adjoint (FP32 pair arithmetic on FP64 coordinate differences, FP64 sums) on
    the mixed forward's state against the FP64 adjoint on the same inputs (the workload's h, m and v
    are FP32 values, so both forms start from identical inputs).  Bar: normwise 1e-4 per field."""
    import torch
    from sphexa_gb300 import autograd as AG
    grads = {}
    for prec in ("fp64", "mixed"):
        wl, ctx, sw, rho_t = setup(side=10, seed=7, precision=prec)
        base = [t.clone().requires_grad_(True) for t in sw.inputs()]
        out = AG.StdSweepFunction.apply(sw, *base)
        L = AG.loss_rho_a(*[o.to(torch.float64) for o in out[:4]], rho_t)
        L.backward()
        grads[prec] = [b.grad.detach().to(torch.float64).cpu().numpy() for b in base]
        ctx.close()
    for k, f in enumerate(FIELDS):
        g64, g32 = grads["fp64"][k], grads["mixed"][k]
        err = np.linalg.norm(g32 - g64) / np.linalg.norm(g64)
        print(f"mixed adjoint {f:3s}: normwise rel {err:.3e}")
        assert err <= 1e-4, f


def test_mixed_adjoint_once_form_matches_scatter_form_after_moves():
    """The mixed adjoint evaluates its momentum-energy term once per owned entry of owned lists
    built from list membership (a mutual pair gives both directed terms); in deterministic-context
    mode it walks the full lists instead (every directed pair evaluated by its owner).  On frozen
    lists whose particles moved after the search (positions jittered by 1e-3 of the spacing, so the
    geometry no longer decides which pairs are mutual), both walks evaluate the same pairs: the
    gradients agree to FP32 summation order.  Bar: normwise 1e-5 per field."""
    import torch
    from sphexa_gb300 import autograd as AG
    grads = {}
    for det in (False, True):
        wl, ctx, sw, rho_t = setup(side=10, seed=9, precision="mixed")
        if det:
            ctx.set_deterministic(True)
        base = [t.clone() for t in sw.inputs()]
        gen = torch.Generator(device="cpu").manual_seed(91)
        for k in range(3):  # move x, y, z by 1e-3 of the lattice spacing
            base[k] = base[k] + (torch.rand(base[k].shape, generator=gen, dtype=torch.float64) - 0.5).to(
                base[k].device) * (2e-3 / 10)
        base = [b.requires_grad_(True) for b in base]
        out = AG.StdSweepFunction.apply(sw, *base)
        L = AG.loss_rho_a(*[o.to(torch.float64) for o in out[:4]], rho_t)
        L.backward()
        grads[det] = [b.grad.detach().to(torch.float64).cpu().numpy() for b in base]
        ctx.close()
    for k, f in enumerate(FIELDS):
        g1, g0 = grads[False][k], grads[True][k]
        err = np.linalg.norm(g1 - g0) / np.linalg.norm(g0)
        print(f"mixed adjoint once vs scatter {f:3s}: normwise rel {err:.3e}")
        assert err <= 1e-5, f
