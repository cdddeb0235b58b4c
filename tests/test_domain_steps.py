"""Domain syncs as the steps of one simulation: the open box shrinks by at most 5 % of its previous
length per side and sync (cstone::limitBoxShrinking, box.hpp:397-414, from the second sync on), and
the tree is the reference's single-rank focus tree, converged at the first sync and updated once per
sync from the previous tree and counts (focus/octree_focus_mpi.hpp:88-253, domain/domain.hpp:199-211)."""

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


def sphere_steps(scales, n=30000, seed=23):
    from sphexa_gb300 import workloads as W
    wl0 = W.sphere(n, seed=seed)
    for scale in scales:
        wl = W.sphere(n, seed=seed)
        for k in ("x", "y", "z"):
            wl.fields[k] = wl0.fields[k] * scale
        yield wl


def test_focus_tree_restatement_equals_reference(port):
    """the numpy restatement of one focus-tree update against the reference's CombinedUpdate::updateFocus
    driven over a sequence of syncs that both splits and merges; the first sync's converged tree
    against the oracle's converged cornerstone tree"""
    import ctypes as C
    r = O.reference("fp64")
    if r is None:
        pytest.skip("reference-compiled oracle not built (reference sources absent)")
    fn = r.lib.oracle_focus_steps
    fn.argtypes = [C.c_int64, C.c_int32, C.c_void_p, C.c_uint32, C.c_void_p, C.c_int64, C.c_void_p]
    box = np.array([-1.3, 1.3, -1.3, 1.3, -1.3, 1.3])
    keys, first = [], None
    for s, wl in enumerate(sphere_steps((1.0, 0.8, 0.6, 1.2, 0.97, 0.97))):
        wl.box = box.copy()
        res = port.sweep(wl, "ve", stages=O.OS_KEYS | O.OS_TREE, want_nbr=False, want_tree=s == 0, fit_box=False)
        keys.append(np.sort(res["keys"]))
        if s == 0:
            first = res["leaves"]
    n, bucket = len(keys[0]), 64
    cap = 20 * n
    out = np.zeros(cap, np.uint64)
    nl = np.zeros(len(keys), np.int64)
    assert fn(n, len(keys), np.concatenate(keys).ctypes.data, bucket, out.ctypes.data, cap, nl.ctypes.data) == 0
    ref, pos = [], 0
    for s in range(len(keys)):
        ref.append(out[pos:pos + nl[s] + 1])
        pos += nl[s] + 1
    np.testing.assert_array_equal(ref[0], first)
    leaves, merged, split = ref[0], False, False
    for s in range(1, len(keys)):
        nxt = O.focus_rebalance_once(leaves, O.leaf_counts(leaves, keys[s - 1]), bucket)
        np.testing.assert_array_equal(nxt, ref[s], err_msg=f"step {s}")
        merged |= not np.all(np.isin(leaves, nxt))
        split |= not np.all(np.isin(nxt, leaves))
        leaves = nxt
    assert merged and split  # the sequence exercises both kinds of update


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
        # the focus tree: converged at the first sync, then one update from the previous tree
        t = dom.tree()
        keys = np.sort(ref["keys"])
        if step == 0:
            conv = port.sweep(wl, "ve", stages=O.OS_KEYS | O.OS_TREE, want_nbr=False, fit_box=False)
            want_leaves = conv["leaves"]
        else:
            want_leaves = O.focus_rebalance_once(prev_leaves, O.leaf_counts(prev_leaves, prev_keys),
                                                 int(ctx.params.bucket))
        np.testing.assert_array_equal(t["leaves"], want_leaves, err_msg=f"step {step}")
        np.testing.assert_array_equal(np.diff(t["layout"].astype(np.int64)), O.leaf_counts(want_leaves, keys))
        prev_leaves, prev_keys = want_leaves, keys
        prev = want
    assert not np.array_equal(prev, fit)  # the shrink limit was active on the last steps
    # neighbour search on the last tree (updated, not converged): counts and lists against brute force
    ng = 150
    nb, nc = sph.find_neighbors(ctx, d.x, d.y, d.z, d.h, 0, wl.n, ng)
    torch.cuda.synchronize()
    x, y, z, h = (d.f[k].cpu().numpy() for k in ("x", "y", "z", "h"))
    nbh, nch = nb.cpu().numpy().reshape(wl.n, ng), nc.cpu().numpy()
    for i in range(0, wl.n, 101):
        r2 = (x - x[i]) ** 2 + (y - y[i]) ** 2 + (z - z[i]) ** 2
        inside = np.flatnonzero(r2 < 4 * h[i] * h[i])
        inside = inside[inside != i]
        assert nch[i] == len(inside)
        np.testing.assert_array_equal(nbh[i, :min(len(inside), ng)], inside[:ng])
    ctx.set_domain_mode(0)
