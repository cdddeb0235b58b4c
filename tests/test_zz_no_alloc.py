"""The allocation-free key entry point against the regular one.

sphgb_sfc_keys_noalloc serves callers whose device memory is owned by their own allocator (or
who cannot afford the device synchronisation of cudaMalloc/cudaFree in a step loop): it fits
the box and computes Hilbert keys with only the caller's buffers and a fixed scratch array
inside the library.  Its keys and box must equal what a first sphgb_domain_sync produces for the
same particles: keys bit-exact (the integer bar of every parity test here), box limits bit-exact.

The calls run back to back on the shared scratch array: first an open box of 600,000 particles
(147 blocks of partials, so the final reduction folds several partials per lane), then a smaller
open set (its 8 blocks must not see the larger call's stale partials), then a box that is periodic
in x and open in y and z (the per-axis merge of fitted and given limits), then an all-periodic box
(no extrema pass at all).  This file is collected last so that a stop-at-first-failure run has
already run every other test.
"""

import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _noalloc_keys(lib, d, box):
    from sphexa_gb300 import _lib
    b = box.to_c()
    keys = d.f["keys"].clone()
    rc = lib.sphgb_sfc_keys_noalloc(d.x.data_ptr(), d.y.data_ptr(), d.z.data_ptr(), d.n, C.byref(b),
                                    keys.data_ptr(), None)
    assert rc == 0, _lib.load().sphgb_status_string(rc)
    return keys.cpu().numpy().view(np.uint64), np.array(b.lim[:])


def _regular_keys(ctx, wl):
    from sphexa_gb300 import sph
    d = sph.ParticlesData.from_workload(wl, "fp64", "cuda:0")
    box = sph.Box(wl.box.copy(), wl.bc.copy())
    dom = sph.Domain(ctx, box)
    dom.sync(d)
    return d.keys.cpu().numpy().view(np.uint64), dom.order(wl.n), box.lim.copy()


def _mixed_boundaries(wl):
    """periodic in x over the generator's box, open in y and z"""
    wl.bc = np.array([1, 0, 0], dtype=wl.bc.dtype)
    return wl


def test_noalloc_keys_match_domain_sync_in_a_row():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from sphexa_gb300 import _lib, sph, workloads as W
    lib = _lib.load()
    ctx = sph.Context(0)
    cases = [W.sphere(600_000, seed=63), W.sphere(30_000, seed=62),
             _mixed_boundaries(W.random_cube(40_000, seed=64, periodic=False)),
             W.random_cube(50_000, seed=61, periodic=True)]
    for k, wl in enumerate(cases):
        d = sph.ParticlesData.from_workload(wl, "fp64", "cuda:0")
        box = sph.Box(wl.box.copy(), wl.bc.copy())
        keys, lim = _noalloc_keys(lib, d, box)
        ref_sorted, order, ref_lim = _regular_keys(ctx, wl)
        np.testing.assert_array_equal(lim, ref_lim)
        np.testing.assert_array_equal(keys[order], ref_sorted)
        if k == 2:  # periodic x keeps the given limits, open y and z take the particle extrema
            np.testing.assert_array_equal(lim[:2], wl.box[:2])
            for a, f in ((1, "y"), (2, "z")):
                assert lim[2 * a] == np.min(wl.fields[f]) and lim[2 * a + 1] == np.max(wl.fields[f])
    # too large is refused before any work
    b = sph.Box(cases[3].box.copy(), cases[3].bc.copy()).to_c()
    assert lib.sphgb_sfc_keys_noalloc(1, 1, 1, 268_435_457, C.byref(b), 1, None) == _lib.SPHGB_ERR_TOO_LARGE
    ctx.close()
