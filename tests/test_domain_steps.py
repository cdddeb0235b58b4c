"""Domain syncs as the steps of one simulation: the open box shrinks by at most 5 % of its previous
length per side and sync (cstone::limitBoxShrinking, box.hpp:397-414, from the second sync on)."""

import numpy as np
import pytest

from oracle import oracle as O


def limit_box_shrinking(fit, prev, shrink=0.05):
    """restatement of limitBoxShrinking on limits [xmin xmax ymin ymax zmin zmax]"""
    out = np.empty(6)
    for k in range(3):
        lo, hi = prev[2 * k], prev[2 * k + 1]
        ln = hi - lo
        out[2 * k] = min(fit[2 * k], lo + shrink * ln)
        out[2 * k + 1] = max(fit[2 * k + 1], hi - shrink * ln)
    return out


def test_limit_box_shrinking_restatement_equals_reference():
    r = O.reference("fp64")
    if r is None:
        pytest.skip("reference-compiled oracle not built (reference sources absent)")
    import ctypes as C
    fn = r.lib.oracle_limit_box_shrinking
    fn.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
    fn.restype = C.c_int
    rng = np.random.Generator(np.random.PCG64(21))
    for _ in range(200):
        prev = np.sort(rng.uniform(-2, 2, (3, 2)), axis=1).ravel()
        fit = prev + rng.normal(0, 0.2, 6)
        fit = np.stack([np.minimum(fit[0::2], fit[1::2] - 1e-3), fit[1::2]], 1).ravel()
        out = np.zeros(6)
        assert fn(fit.ctypes.data, prev.ctypes.data, out.ctypes.data) == 0
        np.testing.assert_array_equal(out, limit_box_shrinking(fit, prev))


@pytest.mark.gpu
def test_multi_step_sync_box_and_keys(gpu_ctx, port):
    import torch
    from sphexa_gb300 import sph, workloads as W
    wl0 = W.sphere(30000, seed=23)
    ctx = gpu_ctx
    ctx.set_domain_mode(1)
    prev = None
    for step, scale in enumerate((1.0, 0.8, 1.2, 0.97)):
        wl = W.sphere(30000, seed=23)
        for k in ("x", "y", "z"):
            wl.fields[k] = wl0.fields[k] * scale
        fit = np.array([f(wl.fields[k]) for k in ("x", "y", "z") for f in (np.min, np.max)])
        want = fit if prev is None else limit_box_shrinking(fit, prev)
        d = sph.ParticlesData.from_workload(wl, "fp64", "cuda:0")
        box = sph.Box(fit.copy(), np.zeros(3, dtype=np.uint8))
        dom = sph.Domain(ctx, box)
        dom.sync(d)
        torch.cuda.synchronize()
        np.testing.assert_array_equal(box.lim, want, err_msg=f"step {step}")
        # keys and order are those of the limited box
        wl.box = want.copy()
        ref = port.sweep(wl, "ve", stages=O.OS_KEYS, want_nbr=False, want_tree=False, fit_box=False)
        np.testing.assert_array_equal(d.keys.cpu().numpy().view(np.uint64), ref["keys"])
        np.testing.assert_array_equal(dom.order(wl.n), ref["order"].astype(np.int64))
        prev = want
    assert not np.array_equal(prev, fit)  # the shrink limit was active on the last steps
    ctx.set_domain_mode(0)
