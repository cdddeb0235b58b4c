"""Central-difference check of an adjoint gradient, with detection of kinks in the forward.

Test infrastructure.  The forward is evaluated at x0 +- eps and x0 +- 2 eps for one coordinate at
a time; the loss differences are summed per particle (L = sum_i l_i with
l_i = (rho_i - rho_target_i)^2 + |a_i|^2), so particles the coordinate does not reach contribute
exactly zero and the differences carry only the rounding of the particles that change (the forward
must then be bitwise reproducible: the context in deterministic mode).

A coordinate whose stencil straddles a kink of the forward (a branch of the artificial viscosity,
the AV switch, the Atwood ramp, max(0, .), a signal-velocity maximum, or a node of a kernel table
in its linear form) is detected from the forward values alone, without looking at the adjoint.
For a smooth loss f
    D1 = (f(+e) - f(-e)) / 2e and D2 = (f(+2e) - f(-2e)) / 4e differ by e^2 f''' / 2, and
    S2 - 4 S1, with Sk = f(+ke) + f(-ke) - 2 f(0), is O(e^4 f'''').
A slope jump J at an offset s in (-e, e) adds -J s / 4e to D2 - D1 and J (3|s| - 2e) to S2 - 4 S1,
while it moves the central difference D1 away from either one-sided derivative by up to J / 2;
these two never vanish together, and J / 2 <= max(6 |D2 - D1|, |S2 - 4 S1| / 2e) =: kink.  A
coordinate with kink > kink_tol |D1| is reported as a straddle and another is drawn from the same
seeded stream; every other coordinate must satisfy |adjoint - D1| <= tol |D1|.  With kink_tol = 5e-7
and tol = 1e-6 an undetected kink moves D1 by at most half the bar, and the smooth part of the kink
estimate (3 e^2 |f'''| ~ 1e-7 |f'| for pair distances of about h = 0.014) stays below kink_tol.
"""

from __future__ import annotations

import numpy as np

FIELDS = ("x", "y", "z", "vx", "vy", "vz", "h", "u")


def particle_loss(out, rho_t):
    rho, ax, ay, az = out[:4]
    return (rho - rho_t) ** 2 + ax * ax + ay * ay + az * az


def adjoint_gradient(sw, rho_t, base):
    """dL/d(inputs) by the hand-written adjoint at `base` (the forward runs first: the VE adjoint
    reads the sums its forward left)"""
    rho, ax, ay, az, du = sw.forward(*base)
    seeds = (2.0 * (rho - rho_t), 2.0 * ax, 2.0 * ay, 2.0 * az, None)
    return [g.detach().cpu().numpy() for g in sw.backward(*seeds)]


def fd_check(sw, rho_t, n, grads, count=64, seed=55555, eps=1e-6, kink_tol=5e-7, max_draws=1000,
             relative=("h",)):
    """Draw coordinates (field, particle) from PCG64(seed) until `count` of them are free of kinks;
    returns (rows, straddles), rows = (field, i, adjoint, central difference, relative difference),
    straddles = (field, i, kink / |D1|).  The step is eps for every field, times the value itself for
    the fields in `relative` (h: a length scale of about 0.014, whose every pair distance ratio r/h
    an absolute step of 1e-6 would move by 7e-5 at once)."""
    base = [t.detach().clone() for t in sw.inputs()]
    l0 = particle_loss(sw.forward(*base), rho_t)
    rng = np.random.Generator(np.random.PCG64(seed))
    rows, straddles = [], []
    while len(rows) < count and len(rows) + len(straddles) < max_draws:
        k = int(rng.integers(0, len(FIELDS)))
        i = int(rng.integers(0, n))
        field = FIELDS[k]
        x0 = float(base[k][i])
        step = eps * abs(x0) if field in relative else eps
        at, ls = {}, {}
        for s in (1, -1, 2, -2):
            at[s] = x0 + s * step
            base[k][i] = at[s]
            ls[s] = particle_loss(sw.forward(*base), rho_t)
        base[k][i] = x0
        d1 = float((ls[1] - ls[-1]).sum().item()) / (at[1] - at[-1])
        d2 = float((ls[2] - ls[-2]).sum().item()) / (at[2] - at[-2])
        s1 = float(((ls[1] - l0) + (ls[-1] - l0)).sum().item())
        s2 = float(((ls[2] - l0) + (ls[-2] - l0)).sum().item())
        kink = max(6.0 * abs(d2 - d1), abs(s2 - 4.0 * s1) / (2.0 * step))
        scale = max(abs(d1), 1e-300)
        if kink > kink_tol * scale:
            straddles.append((field, i, kink / scale))
            continue
        ad = float(grads[k][i])
        rows.append((field, i, ad, d1, abs(ad - d1) / scale))
    sw.forward(*base)  # leave the state of the base point
    return rows, straddles


def report(rows, straddles, label):
    print(f"{label}: {len(rows)} coordinates checked, {len(straddles)} straddling a kink")
    for f in FIELDS:
        e = [r[4] for r in rows if r[0] == f]
        if e:
            print(f"  {f:3s} n={len(e):2d} max rel {max(e):.3e} median {np.median(e):.3e}")
    for f, i, q in straddles:
        print(f"  straddle: {f} of particle {i}, kink bound / |D1| = {q:.2e}")
