"""The hand-written adjoint of the VE chain (sphgb_adjoint_ve) against torch autograd through the FP64
torch restatement of the same chain (tests/torch_reference.py ve_chain) and against FP64 central
differences.

Workload: the adjoint configuration's generator (jittered periodic lattice, Fourier density
field, Gaussian velocities) at 10^3 to 12^3 particles, with u, h and the alpha before the AV switch
varied per particle (so that the AV switch takes both of its branches, the Atwood weights all three
of theirs and no two h coincide) and an AV time step of 1e-2.  Loss L = sum (rho - rho_target)^2 +
sum |a|^2 (+ a seed on du for the reference-gradient test) on the frozen neighbour lists.

* Reference gradient: every form of the adjoint, avClean on and off, in both kernel forms (the
  reference's linear table, the smooth cubic pieces); bar normwise 1e-9 per field.
* Central differences: smooth kernel form, eps = 1e-6 (times h for h), 64 coordinates from
  PCG64(55555); a coordinate whose stencil straddles a kink of the forward (AV switch, Atwood ramp,
  signal-velocity maximum, max(0, .), avClean clamp) is reported and replaced by the next draw
  (tests/fd_check.py).  Bar: relative agreement <= 1e-6 on every checked coordinate.  The full-size
  version (1M particles) is tests/test_gpu_adjoint_fd.py.
"""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FIELDS = ("x", "y", "z", "vx", "vy", "vz", "h", "u")


def setup(side=10, seed=7, av_clean=False, deterministic=False, ordered_forward=False, smooth=False):
    import torch
    from sphexa_gb300 import autograd as AG, sph, workloads as W
    wl = W.fourier(side, seed=seed, rho_seed=55, v_seed=555, target_seed=5555)
    rng = np.random.Generator(np.random.PCG64(seed + 100))
    wl.fields["u"] = wl.fields["u"] * rng.uniform(0.8, 1.2, wl.n)
    wl.fields["h"] = wl.fields["h"] * rng.uniform(0.97, 1.03, wl.n)
    wl.fields["alpha"] = rng.uniform(0.05, 0.5, wl.n)
    ctx = sph.Context(0)
    ctx.set_params(minDt=1e-2)
    ctx.set_kernel_form(smooth)
    if ordered_forward:  # forward passes in list order; the scatter adjoint then walks the full lists
        ctx.set_deterministic(True)
    d = sph.ParticlesData.from_workload(wl, "fp64", "cuda:0", av_clean=av_clean)
    box = sph.Box(wl.box.copy(), wl.bc.copy())
    sw = AG.FrozenVeSweep(ctx, d, box, av_clean=av_clean, deterministic=deterministic)
    sw.freeze()
    order = sph.Domain(ctx, box).order(wl.n)
    rho_t = torch.tensor(wl.fields["rho_target"][order], dtype=torch.float64, device="cuda:0")
    return wl, ctx, sw, rho_t


@pytest.mark.parametrize("smooth", [False, True])
@pytest.mark.parametrize("av_clean", [False, True])
@pytest.mark.parametrize("form", ["pair-once", "scatter", "two-sided"])
def test_ve_adjoint_matches_fp64_reference_gradient(port, av_clean, form, smooth):
    """pair-once: one evaluation per mutual pair of the owned lists; scatter: every list entry
    once with atomics (context in deterministic mode); two-sided: bit-reproducible form"""
    import torch
    from sphexa_gb300 import autograd as AG, sph
    from torch_reference import ve_chain
    wl, ctx, sw, rho_t = setup(side=10, seed=7, av_clean=av_clean, deterministic=form == "two-sided",
                               ordered_forward=form == "scatter", smooth=smooth)
    n = wl.n
    ng = int(ctx.params.ngmax)
    nb = sph.export_neighbors(ctx, n, ng).cpu().numpy().reshape(n, ng).astype(np.int64)
    cnt = np.minimum(sw.d.nc.cpu().numpy().astype(np.int64) - 1, ng)
    ei = np.repeat(np.arange(n), cnt)
    ej = np.concatenate([nb[k, :cnt[k]] for k in range(n)])
    dev = "cuda:0"
    if smooth:
        from torch_reference import hermite_tables
        wh, whd = hermite_tables(6.0)
    else:
        wh, whd = port.tables(6.0)
    tab = torch.tensor(wh, dtype=torch.float64, device=dev)
    tabd = torch.tensor(whd, dtype=torch.float64, device=dev)
    p = ctx.params
    inp = [t.clone().requires_grad_(True) for t in sw.inputs()]
    out_ref = ve_chain(*inp, sw.d.m.clone(), sw.alpha0.clone(), torch.tensor(ei, device=dev),
                       torch.tensor(ej, device=dev), tab, tabd, ctx.K, float(p.gamma),
                       torch.tensor(wl.box[1::2] - wl.box[0::2], dtype=torch.float64), [True, True, True],
                       float(p.minDt), float(p.alphamin), float(p.alphamax), float(p.decay_constant), av_clean)
    gen = torch.Generator(device="cpu").manual_seed(3)
    s_du = torch.randn(n, generator=gen, dtype=torch.float64).to(dev)
    L_ref = AG.loss_rho_a(*out_ref[:4], rho_t) + (s_du * out_ref[4]).sum()
    L_ref.backward()
    g_ref = {f: inp[k].grad.detach().cpu().numpy() for k, f in enumerate(FIELDS)}

    base = [t.detach().clone().requires_grad_(True) for t in sw.inputs()]
    out = AG.VeSweepFunction.apply(sw, *base)
    for name, a, b in zip(("rho", "ax", "ay", "az", "du"), out, out_ref):
        ref = b.detach().cpu().numpy()
        err = np.max(np.abs(a.detach().cpu().numpy() - ref)) / (np.max(np.abs(ref)) + 1e-300)
        assert err <= 1e-10, name
    L = AG.loss_rho_a(*out[:4], rho_t) + (s_du * out[4]).sum()
    L.backward()
    for k, f in enumerate(FIELDS):
        g = base[k].grad.detach().cpu().numpy()
        err = np.linalg.norm(g - g_ref[f]) / (np.linalg.norm(g_ref[f]) + 1e-300)
        print(f"VE reference gradient {f:3s}: normwise rel {err:.3e}")
        assert err <= 1e-9, f
    ctx.close()


def test_deterministic_ve_adjoint_is_bit_reproducible():
    wl, ctx, sw, rho_t = setup(side=10, seed=9, av_clean=True, deterministic=True)
    vals = sw.inputs()
    rho, ax, ay, az, du = sw.forward(*vals)
    seeds = (2.0 * (rho - rho_t), 2.0 * ax, 2.0 * ay, 2.0 * az, du)
    g1 = [t.cpu().numpy() for t in sw.backward(*seeds)]
    g2 = [t.cpu().numpy() for t in sw.backward(*seeds)]
    for a, b in zip(g1, g2):
        np.testing.assert_array_equal(a, b)
    ctx.close()


def test_ve_adjoint_requires_alpha_before_the_switch():
    import ctypes as C
    from sphexa_gb300 import _lib
    wl, ctx, sw, rho_t = setup(side=8, seed=11)
    s = sw.d.c_struct()
    seeds = _lib.SphgbSeeds()
    grads = _lib.SphgbGrads()
    assert ctx.lib.sphgb_adjoint_ve(ctx.h, C.byref(s), None, 0, C.byref(seeds), C.byref(grads), 0) == 1  # SPHGB_ERR_ARG
    ctx.close()


@pytest.mark.parametrize("av_clean", [False, True])
def test_ve_adjoint_matches_central_differences(av_clean):
    from fd_check import adjoint_gradient, fd_check, report
    wl, ctx, sw, rho_t = setup(side=12, seed=5, av_clean=av_clean, smooth=True)
    grads = adjoint_gradient(sw, rho_t, [t.detach().clone() for t in sw.inputs()])
    ctx.set_deterministic(True)  # bitwise reproducible forward for the differences
    rows, straddles = fd_check(sw, rho_t, wl.n, grads)
    report(rows, straddles, f"VE chain{' avClean' if av_clean else ''}, 12^3")
    assert len(rows) == 64
    worst = max(rows, key=lambda r: r[4])
    assert worst[4] <= 1e-6, worst
    ctx.close()


@pytest.mark.parametrize("av_clean", [False, True])
@pytest.mark.parametrize("form", ["pair-once", "scatter", "two-sided", "large-h"])
def test_ve_adjoint_tape_matches_recomputed_sums(av_clean, form):
    """the forward passes' tape (sphgb_set_adjoint_tape) against the adjoint's own re-summation:
    same gradients to rounding (vsig_i and its pair found through the FP32 filter, or in FP64 when
    2h > L/4 as in the 5^3 set), and with a du seed the energy pre-pass is not launched"""
    wl, ctx, sw, rho_t = setup(side=5 if form == "large-h" else 10, seed=13, av_clean=av_clean,
                               deterministic=form == "two-sided", ordered_forward=form == "scatter")
    if form == "large-h":
        assert 2.0 * float(sw.d.h.min()) > 0.25 * float(wl.box[1] - wl.box[0])
    _tape_vs_resummed(ctx, sw, wl.n, rho_t)
    ctx.close()


def _tape_vs_resummed(ctx, sw, n, rho_t):
    """backward with the forward tape, then with the tape off: same gradients to rounding, and
    without the energy pre-pass when the tape holds the momentum-energy sums"""
    import torch
    gen = torch.Generator(device="cpu").manual_seed(4)
    s_du = torch.randn(n, generator=gen, dtype=torch.float64).to("cuda:0")

    def grads():
        vals = sw.inputs()
        rho, ax, ay, az, du = sw.forward(*vals)
        l0 = ctx.launches()
        g = [t.cpu().numpy() for t in sw.backward(2.0 * (rho - rho_t), 2.0 * ax, 2.0 * ay, 2.0 * az, s_du)]
        return g, ctx.launches() - l0

    grads()  # the first backward also builds the transposed lists of the two-sided form
    g_tape, n_tape = grads()
    ctx.set_adjoint_tape(False)
    g_sum, n_sum = grads()
    assert n_tape == n_sum - 1  # no energy pre-pass with the tape
    for f, a, b in zip(FIELDS, g_tape, g_sum):
        err = np.linalg.norm(a - b) / (np.linalg.norm(b) + 1e-300)
        print(f"tape vs re-summed {f:3s}: normwise rel {err:.3e}")
        assert err <= 1e-12, f


def test_ve_adjoint_tape_open_box():
    """the tape and the FP32-filtered signal-velocity walk in an open box (no periodic images),
    random positions with Gaussian velocities"""
    import torch
    from sphexa_gb300 import autograd as AG, sph, workloads as W
    wl = W.random_cube(3000, seed=61, periodic=False)
    ctx = sph.Context(0)
    ctx.set_params(minDt=1e-2, ngmax=250)
    d = sph.ParticlesData.from_workload(wl, "fp64", "cuda:0")
    box = sph.Box(wl.box.copy(), wl.bc.copy())
    sw = AG.FrozenVeSweep(ctx, d, box)
    sw.freeze()
    assert ctx.stats()["capped"] == 0
    rho_t = torch.ones(wl.n, dtype=torch.float64, device="cuda:0") * float(d.m.sum().item())
    _tape_vs_resummed(ctx, sw, wl.n, rho_t)
    ctx.close()
