"""Pins of the integration-step oracle (CPU).

The port's one-step integration (positions, velocities, x_m1, u, du_m1) and h update equal the
reference's own sph::positionUpdate / energyUpdate / fbcCheck / updateH compiled from its headers
bit for bit, on periodic, open and fixed boundaries and on the u < 0 branch; the conserved-quantity
restatement equals numpy sums (the reference's conserved_quantities.hpp needs MPI headers).
"""

import numpy as np
import pytest

from oracle import oracle as O

FIELDS = ["x", "y", "z", "vx", "vy", "vz", "ax", "ay", "az", "xm1", "ym1", "zm1", "u", "du", "dum1", "h"]


def step_inputs(n=5000, seed=7, frozen=0):
    rng = np.random.Generator(np.random.PCG64(seed))
    f = {k: rng.uniform(-0.5, 0.5, n) for k in ("x", "y", "z")}
    for k in ("vx", "vy", "vz"):
        f[k] = rng.normal(0.0, 1.0, n)
    for k in ("ax", "ay", "az"):
        f[k] = rng.normal(0.0, 30.0, n)
    for k in ("xm1", "ym1", "zm1"):
        f[k] = rng.normal(0.0, 1e-3, n)
    f["u"] = rng.uniform(0.5, 2.0, n)
    f["du"] = rng.normal(0.0, 5.0, n)
    f["dum1"] = rng.normal(0.0, 5.0, n)
    f["h"] = rng.uniform(0.01, 0.03, n)
    # some particles leave the box in one step, some drive u negative (the exp branch)
    f["vx"][:50] = 400.0
    f["du"][50:100] = -5e3
    if frozen:
        for k in ("vx", "vy", "vz"):
            f[k][-frozen:] = 0.0
        f["x"][-frozen:] = 0.5 - 0.5 * f["h"][-frozen:]
    return f


@pytest.fixture(scope="module")
def ref_lib():
    r = O.reference("fp64")
    if r is None:
        pytest.skip("reference-compiled oracle not built (reference sources absent)")
    return r.lib


@pytest.mark.parametrize("bc", [(1, 1, 1), (0, 0, 0), (2, 1, 0)])
def test_port_positions_equal_reference(port, ref_lib, bc):
    box = [-0.5, 0.5, -0.5, 0.5, -0.5, 0.5]
    a = step_inputs(frozen=40)
    b = {k: v.copy() for k, v in a.items()}
    O.run_positions(port.lib, a, 1e-3, 8e-4, box, bc)
    O.run_positions(ref_lib, b, 1e-3, 8e-4, box, bc)
    for k in FIELDS:
        np.testing.assert_array_equal(a[k], b[k], err_msg=k)
    if 2 in bc:  # frozen particles next to the fixed boundary did not move
        c = step_inputs(frozen=40)
        np.testing.assert_array_equal(a["x"][-40:], c["x"][-40:])


def test_port_update_h_equals_reference(port, ref_lib):
    rng = np.random.Generator(np.random.PCG64(8))
    h1 = rng.uniform(0.01, 0.05, 4000)
    h2 = h1.copy()
    nc = rng.integers(1, 400, 4000).astype(np.uint32)
    O.run_update_h(port.lib, 100, nc, h1)
    O.run_update_h(ref_lib, 100, nc, h2)
    np.testing.assert_array_equal(h1, h2)


def test_conserved_restatement_equals_numpy(port):
    f = step_inputs()
    f["m"] = np.full(len(f["x"]), 1.0 / len(f["x"]))
    out = O.run_conserved(port.lib, f)
    X = np.stack([f["x"], f["y"], f["z"]], 1)
    V = np.stack([f["vx"], f["vy"], f["vz"]], 1)
    m = f["m"]
    want = np.concatenate([[0.5 * np.sum(m * np.sum(V * V, 1)), np.sum(m * f["u"])], (m[:, None] * V).sum(0),
                           (m[:, None] * np.cross(X, V)).sum(0)])
    np.testing.assert_allclose(out, want, rtol=1e-12, atol=1e-15)
