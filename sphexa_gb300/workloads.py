"""Seeded synthetic particle sets for the single-rank SPH hydro sweep.

The reference runs its Sedov / Evrard test cases from glass blocks downloaded at run time;
none are available offline, so every workload here is a lattice or an analytic distribution
with a fixed seed.  The formulas follow the reference initialisers:

* lattice placement: cell-centred ``regularGrid`` (main/src/init/grid.hpp:100-131);
* Sedov smoothing length ``h0 = 0.5 * cbrt(3/(4 pi) * ng0 * V / N)`` and the Gaussian energy
  spike ``u = u0 + E0 exp(-r^2/w^2)``, ``E0 = E / (pi^1.5 w^3)``
  (main/src/init/sedov_init.hpp:55-80, main/src/init/sedov_constants.hpp:14-19);
* alpha starts at ``alphamin`` (sedov_init.hpp:65);
* the clustered sphere uses the Evrard-style h from the local number density
  (main/src/init/evrard_init.hpp:80-92).

All hydro inputs (h, m, v, alpha) are rounded to FP32-representable values so that the
FP64 form and the mixed (FP32 hydro field) form of the sweep see bit-identical inputs and
therefore identical neighbour lists.  Coordinates and u stay FP64, as in the reference's
default ``SphTypes`` (sph/include/sph/types.hpp:39-46).
"""

from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

BC_OPEN = 0
BC_PERIODIC = 1


@dataclass
class Workload:
    name: str
    n: int
    box: np.ndarray            # [xmin, xmax, ymin, ymax, zmin, zmax] float64
    bc: np.ndarray             # [3] uint8, 0 open / 1 periodic
    fields: dict = field(default_factory=dict)   # name -> np.ndarray (float64)
    params: dict = field(default_factory=dict)

    def nbytes(self) -> int:
        return sum(a.nbytes for a in self.fields.values())


def default_params(**over) -> dict:
    """Physics constants of ``sphexa::ParticlesData`` (sph/include/sph/particles_data.hpp:90-146)."""
    p = dict(ng0=100, ngmax=150, gamma=5.0 / 3.0, Kcour=0.2, sincIndex=6.0,
             alphamin=0.05, alphamax=1.0, decay_constant=0.2, minDt=1e-6, bucket=64)
    p.update(over)
    return p


def _f32(a: np.ndarray) -> np.ndarray:
    return np.asarray(a, dtype=np.float32).astype(np.float64)


def lattice(side: int, r: float = 0.5) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
    """Cell-centred cubic lattice in [-r, r]^3, x fastest (grid.hpp:100-131)."""
    step = 2.0 * r / side
    c = -r + 0.5 * step + step * np.arange(side, dtype=np.float64)
    z, y, x = np.meshgrid(c, c, c, indexing="ij")
    return x.ravel().copy(), y.ravel().copy(), z.ravel().copy()


def _wrap(a: np.ndarray, lo: float, hi: float) -> np.ndarray:
    L = hi - lo
    a = np.where(a < lo, a + L, a)
    return np.where(a >= hi, a - L, a)


def sedov(side: int = 50, jitter: float = 0.0, seed: int = 2, ng0: int = 100) -> Workload:
    """Sedov blast on a (optionally jittered) periodic lattice in [-0.5, 0.5]^3."""
    n = side ** 3
    x, y, z = lattice(side)
    step = 1.0 / side
    if jitter > 0.0:
        rng = np.random.Generator(np.random.PCG64(seed))
        x = _wrap(x + rng.uniform(-jitter, jitter, n) * step, -0.5, 0.5)
        y = _wrap(y + rng.uniform(-jitter, jitter, n) * step, -0.5, 0.5)
        z = _wrap(z + rng.uniform(-jitter, jitter, n) * step, -0.5, 0.5)
    h0 = 0.5 * math.cbrt(3.0 / (4.0 * math.pi) * ng0 * 1.0 / n)
    w = 2.0 * h0
    e0 = 1.0 / (math.pi ** 1.5 * w ** 3)
    r2 = x * x + y * y + z * z
    u = 1e-8 + e0 * np.exp(-r2 / (w * w))
    prm = default_params(ng0=ng0)
    f = dict(x=x, y=y, z=z,
             h=_f32(np.full(n, h0)), m=_f32(np.full(n, 1.0 / n)), u=u,
             vx=np.zeros(n), vy=np.zeros(n), vz=np.zeros(n),
             alpha=_f32(np.full(n, prm["alphamin"])))
    return Workload(f"sedov{side}^3" + (f"_jit{jitter}" if jitter else ""), n,
                    np.array([-0.5, 0.5, -0.5, 0.5, -0.5, 0.5]),
                    np.array([BC_PERIODIC] * 3, dtype=np.uint8), f, prm)


def _fourier_density(x, y, z, seed: int, modes: int = 8, amp: float = 0.1) -> np.ndarray:
    """1 + amp * sum_m a_m cos(2 pi k_m . x + phi_m) / sum a_m, integer k (periodic in the unit box)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    ks = []
    while len(ks) < modes:
        k = rng.integers(-4, 5, 3)
        if np.any(k != 0):
            ks.append(k)
    a = rng.uniform(0.5, 1.0, modes)
    phi = rng.uniform(0.0, 2.0 * math.pi, modes)
    s = np.zeros_like(x)
    for m in range(modes):
        s += a[m] * np.cos(2.0 * math.pi * (ks[m][0] * x + ks[m][1] * y + ks[m][2] * z) + phi[m])
    return 1.0 + amp * s / a.sum()


def fourier(side: int = 300, jitter: float = 0.3, seed: int = 3, rho_seed: int = 33,
            v_seed: int = 333, target_seed: int | None = None, ng0: int = 100) -> Workload:
    """Jittered periodic lattice with a Fourier density field and Gaussian velocities."""
    n = side ** 3
    x, y, z = lattice(side)
    step = 1.0 / side
    rng = np.random.Generator(np.random.PCG64(seed))
    x = _wrap(x + rng.uniform(-jitter, jitter, n) * step, -0.5, 0.5)
    y = _wrap(y + rng.uniform(-jitter, jitter, n) * step, -0.5, 0.5)
    z = _wrap(z + rng.uniform(-jitter, jitter, n) * step, -0.5, 0.5)
    rho = _fourier_density(x, y, z, rho_seed)
    vr = np.random.Generator(np.random.PCG64(v_seed))
    vx, vy, vz = (vr.normal(0.0, 0.1, n) for _ in range(3))
    h0 = 0.5 * math.cbrt(3.0 / (4.0 * math.pi) * ng0 / n)
    prm = default_params(ng0=ng0)
    f = dict(x=x, y=y, z=z, h=_f32(np.full(n, h0)), m=_f32(rho / n), u=np.ones(n),
             vx=_f32(vx), vy=_f32(vy), vz=_f32(vz), alpha=_f32(np.full(n, prm["alphamin"])))
    if target_seed is not None:
        f["rho_target"] = _fourier_density(x, y, z, target_seed)
    return Workload(f"fourier{side}^3", n, np.array([-0.5, 0.5, -0.5, 0.5, -0.5, 0.5]),
                    np.array([BC_PERIODIC] * 3, dtype=np.uint8), f, prm)


def sphere(n: int = 10_000_000, seed: int = 4, ng0: int = 100) -> Workload:
    """Clustered sphere, open boundaries: r = sqrt(U) so that density ~ 1/r."""
    rng = np.random.Generator(np.random.PCG64(seed))
    r = np.sqrt(rng.uniform(0.0, 1.0, n))
    d = rng.normal(0.0, 1.0, (n, 3))
    d /= np.linalg.norm(d, axis=1)[:, None]
    x, y, z = (r * d[:, k] for k in range(3))
    ndens = n / (2.0 * math.pi * np.maximum(r, 1e-6))
    h = 0.5 * np.cbrt(3.0 / (4.0 * math.pi) * ng0 / ndens)
    prm = default_params(ng0=ng0)
    f = dict(x=x, y=y, z=z, h=_f32(h), m=_f32(np.full(n, 1.0 / n)), u=np.full(n, 0.05),
             vx=np.zeros(n), vy=np.zeros(n), vz=np.zeros(n),
             alpha=_f32(np.full(n, prm["alphamin"])))
    box = np.array([x.min(), x.max(), y.min(), y.max(), z.min(), z.max()])
    return Workload(f"sphere{n}", n, box, np.array([BC_OPEN] * 3, dtype=np.uint8), f, prm)


def random_cube(n: int, seed: int = 42, periodic: bool = True, h: float | None = None,
                gaussian: bool = False) -> Workload:
    """Small uniform / Gaussian random sets in the unit box, like the reference's
    ``RandomCoordinates`` fixtures (domain/test/coord_samples/random.hpp:30-140)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    if gaussian:
        pts = np.clip(rng.normal(0.5, 0.15, (n, 3)), 0.0, 1.0 - 1e-12)
    else:
        pts = rng.uniform(0.0, 1.0, (n, 3))
    if h is None:
        h = 0.5 * math.cbrt(3.0 / (4.0 * math.pi) * 100 / n)
    prm = default_params()
    v = rng.normal(0.0, 0.1, (n, 3))
    f = dict(x=pts[:, 0].copy(), y=pts[:, 1].copy(), z=pts[:, 2].copy(),
             h=_f32(rng.uniform(0.9, 1.1, n) * h), m=_f32(rng.uniform(0.5, 1.5, n) / n),
             u=rng.uniform(0.5, 1.5, n), vx=_f32(v[:, 0]), vy=_f32(v[:, 1]), vz=_f32(v[:, 2]),
             alpha=_f32(rng.uniform(0.05, 1.0, n)))
    bc = BC_PERIODIC if periodic else BC_OPEN
    box = np.array([0.0, 1.0, 0.0, 1.0, 0.0, 1.0])
    return Workload(f"random{n}", n, box, np.array([bc] * 3, dtype=np.uint8), f, prm)


CONFIGS = {
    # config name -> factory; sizes are the ones the scope table quotes
    "sedov50": lambda: sedov(50),
    "sedov200_jit": lambda: sedov(200, jitter=0.25, seed=2),
    "fourier300": lambda: fourier(300),
    "sphere10M": lambda: sphere(10_000_000),
    "adjoint100": lambda: fourier(100, seed=5, rho_seed=55, v_seed=555, target_seed=5555),
}
