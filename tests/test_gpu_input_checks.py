"""Invalid inputs are refused with SPHGB_ERR_INPUT before any key, tree or search kernel runs.

A NaN or infinite coordinate, a NaN, zero or negative smoothing length, or a non-finite box limit
would otherwise flow silently into the Hilbert keys and the neighbour search.  Each case checks the
status and that the call launched nothing but the one check kernel (the context's launch counter),
and that the context still works on valid data afterwards (no sticky CUDA error)."""

import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ERR_INPUT = 9


def _data(wl, precision="fp64"):
    from sphexa_gb300 import sph
    return sph.ParticlesData.from_workload(wl, precision, "cuda:0")


def _sync_status(ctx, d, box):
    from sphexa_gb300 import _lib
    lib = _lib.load()
    b = box.to_c()
    return lib.sphgb_domain_sync(ctx.h, C.byref(d.c_struct()), C.byref(b))


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("field,value", [("x", np.inf), ("y", np.nan), ("z", -np.inf), ("h", np.nan),
                                         ("h", 0.0), ("h", -1e-3), ("h", np.inf)])
def test_sync_refuses_bad_particle(field, value, precision):
    from sphexa_gb300 import sph, workloads as W
    ctx = sph.Context(0)
    wl = W.random_cube(5000, seed=301, periodic=True)
    d = _data(wl, precision)
    d.f[field][1234] = value
    box = sph.Box(wl.box.copy(), wl.bc.copy())
    before = ctx.launches()
    assert _sync_status(ctx, d, box) == ERR_INPUT
    assert ctx.launches() - before == 1  # the check kernel only
    # the same context then syncs a valid set
    d2 = _data(wl, precision)
    assert _sync_status(ctx, d2, sph.Box(wl.box.copy(), wl.bc.copy())) == 0
    ctx.close()


def test_sync_refuses_non_finite_box():
    from sphexa_gb300 import sph, workloads as W
    ctx = sph.Context(0)
    wl = W.random_cube(2000, seed=302, periodic=True)
    d = _data(wl)
    lim = wl.box.copy()
    lim[3] = np.nan
    before = ctx.launches()
    assert _sync_status(ctx, d, sph.Box(lim, wl.bc.copy())) == ERR_INPUT
    assert ctx.launches() == before
    ctx.close()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_neighbour_searches_refuse_bad_h_after_a_valid_sync(precision):
    """h (or x) changed to an invalid value after a valid sync: the searches refuse it before the
    grid-form and search kernels run; then a repaired h searches normally"""
    from sphexa_gb300 import _lib, sph, workloads as W
    lib = _lib.load()
    ctx = sph.Context(0)
    wl = W.random_cube(8000, seed=303, periodic=False)
    d = _data(wl, precision)
    box = sph.Box(wl.box.copy(), wl.bc.copy())
    sph.Domain(ctx, box).sync(d)
    h_ok = d.h.clone()
    d.h[77] = float("nan")
    before = ctx.launches()
    assert lib.sphgb_find_neighbors_sph(ctx.h, C.byref(d.c_struct()), 0, d.n) == ERR_INPUT
    assert ctx.launches() - before == 1
    # the fixed-h search of cstone::findNeighbors, with an infinite x
    d.h.copy_(h_ok)
    x_ok = d.x.clone()
    d.x[5] = float("inf")
    import torch
    nc = torch.zeros(d.n, dtype=torch.int32, device="cuda:0")
    hp = _lib.SPHGB_MIXED if precision == "mixed" else _lib.SPHGB_FP64
    before = ctx.launches()
    rc = lib.sphgb_find_neighbors(ctx.h, d.x.data_ptr(), d.y.data_ptr(), d.z.data_ptr(), d.h.data_ptr(), hp, 0, d.n,
                                  150, None, nc.data_ptr())
    assert rc == ERR_INPUT
    assert ctx.launches() - before == 1
    d.x.copy_(x_ok)
    assert sph.find_neighbors_sfc(ctx, 0, d.n, d) in (0, _lib.SPHGB_ERR_NOCONV)
    assert int(d.nc.max().item()) > 1
    ctx.close()


def test_sweep_refuses_bad_h():
    from sphexa_gb300 import _lib, sph, workloads as W
    ctx = sph.Context(0)
    wl = W.random_cube(3000, seed=304, periodic=True)
    d = _data(wl)
    d.h[0] = 0.0
    with pytest.raises(_lib.SphgbError) as e:
        sph.sweep(ctx, d, sph.Box(wl.box.copy(), wl.bc.copy()), "ve", False)
    assert e.value.status == ERR_INPUT
    ctx.close()
