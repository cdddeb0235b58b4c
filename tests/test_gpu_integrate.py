"""The integration step and global reductions on the GPU against the oracle.

Positions, velocities, x_m1, u and du_m1 are bit-exact against the oracle's step (itself bit-exact
against the reference's positionUpdate / energyUpdate, tests/test_integrate_oracle.py) in both
precisions, except u on the u < 0 branch (CUDA exp against glibc exp: 1e-15 relative); h updates
agree to the last bits of pow; the conserved sums and time-step limits to 1e-13.
"""

import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

from test_integrate_oracle import FIELDS, step_inputs  # noqa: E402
from oracle import oracle as O  # noqa: E402

HYDRO = ("vx", "vy", "vz", "ax", "ay", "az", "h")


def load(d, f):
    import torch
    for k in ("x", "y", "z", "u", "du") + HYDRO:
        d.f[k].copy_(torch.as_tensor(f[k], dtype=d.f[k].dtype))


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("bc", [(1, 1, 1), (0, 0, 0), (2, 1, 0)])
def test_positions_match_oracle(gpu_ctx, port, precision, bc):
    import torch
    from sphexa_gb300 import sph
    f = step_inputs(frozen=40)
    if precision == "mixed":  # the hydro-type inputs are FP32 values
        for k in HYDRO + ("xm1", "ym1", "zm1", "dum1"):
            f[k] = f[k].astype(np.float32).astype(np.float64)
    n = len(f["x"])
    d = sph.ParticlesData(n, precision, "cuda:0")
    load(d, f)
    dt = d.f["vx"].dtype
    m1 = {k: torch.as_tensor(f[k], dtype=dt, device="cuda:0").clone() for k in ("xm1", "ym1", "zm1", "dum1")}
    box = sph.Box(np.array([-0.5, 0.5, -0.5, 0.5, -0.5, 0.5]), np.array(bc, dtype=np.uint8))
    ts = sph.Timestep(minDt=1e-3, minDt_m1=8e-4)
    sph.compute_positions(gpu_ctx, d, box, m1["xm1"], m1["ym1"], m1["zm1"], m1["dum1"], ts)
    ref = {k: v.copy() for k, v in f.items()}
    O.run_positions(port.lib, ref, 1e-3, 8e-4, box.lim, bc)
    cast = (lambda a: a.astype(np.float32).astype(np.float64)) if precision == "mixed" else (lambda a: a)
    got = {k: d.f[k].double().cpu().numpy() for k in ("x", "y", "z", "vx", "vy", "vz", "u")}
    got.update({k: m1[k].double().cpu().numpy() for k in m1})
    for k in ("x", "y", "z"):
        np.testing.assert_array_equal(got[k], ref[k], err_msg=k)
    for k in ("vx", "vy", "vz", "xm1", "ym1", "zm1", "dum1"):
        np.testing.assert_array_equal(got[k], cast(ref[k]), err_msg=k)
    neg = slice(50, 100)  # u < 0 branch: exp of the two libraries
    keep = np.ones(n, bool)
    keep[neg] = False
    np.testing.assert_array_equal(got["u"][keep], ref["u"][keep])
    np.testing.assert_allclose(got["u"][neg], ref["u"][neg], rtol=1e-15)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_update_smoothing_length(gpu_ctx, port, precision):
    import torch
    from sphexa_gb300 import sph
    rng = np.random.Generator(np.random.PCG64(11))
    n = 20000
    h = rng.uniform(0.01, 0.05, n)
    if precision == "mixed":
        h = h.astype(np.float32).astype(np.float64)
    nc = rng.integers(1, 400, n).astype(np.uint32)
    d = sph.ParticlesData(n, precision, "cuda:0")
    d.f["h"].copy_(torch.as_tensor(h, dtype=d.f["h"].dtype))
    d.f["nc"].copy_(torch.as_tensor(nc.astype(np.int32)))
    gpu_ctx.set_params(ng0=100)
    sph.update_smoothing_length(gpu_ctx, d)
    got = d.f["h"].double().cpu().numpy()
    if precision == "fp64":
        ref = h.copy()
        O.run_update_h(port.lib, 100, nc, ref)
        np.testing.assert_allclose(got, ref, rtol=4.5e-16)
    else:  # updateH in float arithmetic (kernels.hpp:26-32 with T = float)
        hf, ncf = h.astype(np.float32), nc.astype(np.float32)
        ref = hf * np.float32(0.5) * np.power(np.float32(1) + np.float32(1023.0) * np.float32(100) / ncf,
                                               np.float32(0.1))
        np.testing.assert_allclose(got, ref.astype(np.float64), rtol=3e-7)


def test_conserved_and_timesteps(gpu_ctx, port):
    import torch
    from sphexa_gb300 import sph
    f = step_inputs(n=300000, seed=12)
    n = len(f["x"])
    f["m"] = np.full(n, 1.0 / n)
    d = sph.ParticlesData(n, "fp64", "cuda:0")
    load(d, f)
    d.f["m"].copy_(torch.as_tensor(f["m"]))
    divv = np.random.Generator(np.random.PCG64(13)).normal(0.0, 2.0, n)
    d.f["divv"].copy_(torch.as_tensor(divv))
    got = sph.conserved_quantities(gpu_ctx, d)
    ref = O.run_conserved(port.lib, f)
    vec = np.array([got["eKin"], got["eInt"]] + got["linmom"] + got["angmom"])
    np.testing.assert_allclose(vec, ref, rtol=1e-12, atol=1e-16)
    # identical on a second call (fixed reduction order)
    again = sph.conserved_quantities(gpu_ctx, d)
    assert again == got
    assert sph.rho_timestep(gpu_ctx, d, 0.06) == pytest.approx(0.06 / abs(divv.max()), rel=1e-15)
    amax = np.max(f["ax"] ** 2 + f["ay"] ** 2 + f["az"] ** 2)
    assert sph.acceleration_timestep(gpu_ctx, d, 0.2, 0.005) == pytest.approx(
        0.2 * math.sqrt(0.005 / math.sqrt(amax)), rel=1e-14)
    # computeTimestep (ts_global.hpp:97-113): min of the limits, growth limit 1.1 minDt
    ts = sph.Timestep(minDt=1e-4, minDt_m1=9e-5, ttot=0.5, minDtCourant=3e-4, minDtRho=2e-4)
    sph.compute_timestep(gpu_ctx, d, ts)
    assert ts.minDt == pytest.approx(1.1e-4, rel=1e-15) and ts.minDt_m1 == 1e-4
    assert ts.ttot == pytest.approx(0.5 + 1.1e-4, rel=1e-15)
    ts2 = sph.Timestep(minDt=1e-2, minDtCourant=3e-4, minDtRho=2e-4, g=1.0)
    sph.compute_timestep(gpu_ctx, d, ts2)
    dt_acc = 0.2 * math.sqrt(0.005 / math.sqrt(amax))
    assert ts2.minDt == pytest.approx(min(dt_acc, 2e-4), rel=1e-14)
