"""Generate the golden fixtures under tests/golden/ from the reference's own CPU code.

Run here, where the reference sources exist: it builds oracle/_ref/libref_fp64.so from the
reference headers (oracle/Makefile) and records
  * kat_std.npz   - the 5-particle known-answer inputs of sph/test/std.cpp:40-91 and the
                    reference j-loop outputs on them;
  * kat_ve.npz    - the 99-particle inputs of sph/test/ve.cpp:52-104 (read from the reference's
                    sph/test/example_data.txt, derived fields formed as in its SetUp) and the
                    reference j-loop outputs;
  * sweep_*.npz   - small seeded workloads (sphexa_gb300/workloads.py) run through the full
                    reference chain: keys, order, cornerstone leaves, octree, neighbour counts
                    and sorted sets, and every output field.
Where the reference sources are absent, the tests compare against these files.

    python tests/golden/make_golden.py
"""

from __future__ import annotations

import ctypes as C
import math
import os
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path.insert(0, str(ROOT))

from oracle import oracle as O  # noqa: E402
from sphexa_gb300 import workloads as W  # noqa: E402

REF = Path(os.environ.get("SPHGB_REFERENCE", Path(__file__).resolve().parents[3] / "reference"))

OJ = dict(xmass=0, gradh=1, iad_std=2, iad_ve=3, divv=4, av=5, me_std=6, me_ve=7)


class JIn(C.Structure):
    _fields_ = [("n", C.c_int64), ("f", C.c_void_p * O.NF), ("neighbors", C.c_void_p), ("count", C.c_uint32),
                ("K", C.c_double), ("box", C.c_double * 6), ("bc", C.c_uint8 * 3), ("sincIndex", C.c_double),
                ("dt", C.c_double), ("alphamin", C.c_double), ("alphamax", C.c_double), ("decay", C.c_double),
                ("loop", C.c_int32), ("avclean", C.c_int32)]


def sphynx_k(n: float) -> float:
    """SPHYNX fit of the sinc-kernel normalisation (Cabezon et al. 2017), used by the reference tests."""
    b0, b1, b2, b3 = 2.7012593e-2, 2.0410827e-2, 3.7451957e-3, 4.7013839e-2
    return b0 + b1 * math.sqrt(n) + b2 * n + b3 * math.sqrt(n * n * n)


def run_jloop(lib, fields: dict, neighbors, loop: str, K: float, box, bc=(0, 0, 0), avclean=False,
              dt=0.0, alphamin=0.05, alphamax=1.0, decay=0.2) -> np.ndarray:
    lib.oracle_jloop.argtypes = [C.POINTER(JIn), C.c_void_p]
    lib.oracle_jloop.restype = C.c_int
    n = len(fields["x"])
    j = JIn()
    j.n = n
    keep = []
    for k, name in enumerate(O.FIELDS):
        if name in fields:
            a = np.ascontiguousarray(fields[name], dtype=np.float64)
            keep.append(a)
            j.f[k] = a.ctypes.data
    nb = np.ascontiguousarray(neighbors, dtype=np.uint32)
    j.neighbors = nb.ctypes.data
    j.count = len(nb)
    j.K = K
    for k in range(6):
        j.box[k] = box[k]
    for k in range(3):
        j.bc[k] = bc[k]
    j.sincIndex = 6.0
    j.dt, j.alphamin, j.alphamax, j.decay = dt, alphamin, alphamax, decay
    j.loop = OJ[loop]
    j.avclean = int(avclean)
    out = np.zeros(16)
    rc = lib.oracle_jloop(C.byref(j), out.ctypes.data)
    assert rc == 0, rc
    return out


def std_kat_inputs() -> dict:
    """Inputs of the std known-answer fixture (sph/test/std.cpp:58-84)."""
    f = dict(x=[1.0, 1.1, 3.2, 1.3, 2.4], y=[1.1, 1.2, 1.3, 4.4, 5.5], z=[1.2, 2.3, 1.4, 1.5, 1.6],
             h=[5.0, 5.1, 5.2, 5.3, 5.4], m=[1.1, 1.2, 1.3, 1.4, 1.5], rho=[0.014, 0.015, 0.016, 0.017, 0.018],
             vx=[0.010, -0.020, 0.030, -0.040, 0.050], vy=[-0.011, 0.021, -0.031, 0.041, -0.051],
             vz=[0.091, -0.081, 0.071, -0.061, 0.055], c=[0.4, 0.5, 0.6, 0.7, 0.8], p=[0.2, 0.3, 0.4, 0.5, 0.6],
             c11=[0.21, 0.27, 0.10, 0.45, 0.46], c12=[-0.22, -0.29, -0.11, -0.44, -0.47],
             c13=[-0.23, -0.31, -0.12, -0.43, -0.48], c22=[0.24, 0.32, 0.13, 0.42, 0.49],
             c23=[-0.25, -0.33, -0.14, -0.41, -0.50], c33=[0.26, 0.34, 0.15, 0.40, 0.51])
    return {k: np.array(v, dtype=np.float64) for k, v in f.items()}


def ve_kat_inputs() -> dict:
    """Inputs of the VE known-answer fixture (sph/test/ve.cpp:58-86) from example_data.txt."""
    cols = ["x", "y", "z", "vx", "vy", "vz", "h", "c", "c11", "c12", "c13", "c22", "c23", "c33", "p", "gradh",
            "rho0", "sumwhrho0", "sumwh", "dvxdx", "dvxdy", "dvxdz", "dvydx", "dvydy", "dvydz", "dvzdx", "dvzdy",
            "dvzdz", "alpha", "u", "divv"]
    data = np.loadtxt(REF / "sph" / "test" / "example_data.txt")
    assert data.shape == (99, 31), data.shape
    f = {c: data[:, k].copy() for k, c in enumerate(cols)}
    mpart = 3.781038064465603e26
    K = sphynx_k(6.0)
    f["m"] = np.full(99, mpart)
    f["xm"] = mpart / f["rho0"]
    f["kx"] = K * f["xm"] / np.power(f["h"], 3)
    f["prho"] = f["p"] / (f["kx"] * f["m"] * f["m"] * f["gradh"])
    f["dV11"] = f["dvxdx"]
    f["dV12"] = f["dvxdy"] + f["dvydx"]
    f["dV13"] = f["dvxdz"] + f["dvzdx"]
    f["dV22"] = f["dvydy"]
    f["dV23"] = f["dvydz"] + f["dvzdy"]
    f["dV33"] = f["dvzdz"]
    keep = ["x", "y", "z", "vx", "vy", "vz", "h", "c", "c11", "c12", "c13", "c22", "c23", "c33", "p", "gradh",
            "alpha", "u", "divv", "m", "xm", "kx", "prho", "dV11", "dV12", "dV13", "dV22", "dV23", "dV33"]
    return {k: f[k] for k in keep}


def kat_outputs(lib) -> tuple[dict, dict]:
    K = sphynx_k(6.0)
    fs = std_kat_inputs()
    std_out = dict(
        iad_std=run_jloop(lib, fs, [1, 2, 3, 4], "iad_std", K, (0, 6, 0, 6, 0, 6))[:6],
        me_std=run_jloop(lib, fs, [1, 2, 3, 4], "me_std", K, (0, 6, 0, 6, 0, 6))[:5])
    fv = ve_kat_inputs()
    nb = np.arange(1, 99)
    box = (-1e9, 1e9) * 3
    ve_out = dict(
        av=run_jloop(lib, fv, nb, "av", K, box, dt=0.3)[:1],
        divv=run_jloop(lib, fv, nb, "divv", K, box)[:8],
        iad_ve=run_jloop(lib, fv, nb, "iad_ve", K, box)[:6],
        me_ve_clean=run_jloop(lib, fv, nb, "me_ve", K, box, avclean=True)[:5],
        me_ve=run_jloop(lib, fv, nb, "me_ve", K, box, avclean=False)[:5],
        gradh=run_jloop(lib, fv, nb, "gradh", K, box)[:2],
        xmass=run_jloop(lib, fv, nb, "xmass", K, box)[:1])
    return ({"in_" + k: v for k, v in fs.items()} | {"out_" + k: v for k, v in std_out.items()} | {"K": K},
            {"in_" + k: v for k, v in fv.items()} | {"out_" + k: v for k, v in ve_out.items()} | {"K": K})


SWEEPS = {
    # name: (workload factory, variant, avclean)
    "sedov10_std": (lambda: W.sedov(10), "std", False),
    "random2000_ve_clean": (lambda: W.random_cube(2000, seed=7), "ve", True),
    "sphere2000_ve": (lambda: W.sphere(2000, seed=9), "ve", False),
    "fourier10_ve": (lambda: W.fourier(10, seed=11, rho_seed=12, v_seed=13), "ve", False),
}


def sweep_fixture(ref, wl, variant, avclean) -> dict:
    r = ref.sweep(wl, variant, avclean)
    ng = wl.params["ngmax"]
    sets = O.sorted_sets(r["nbr"], r["nc"], ng)
    cnt = np.minimum(r["nc"].astype(np.int64) - 1, ng)
    flat = np.concatenate([sets[i, :cnt[i]] for i in range(wl.n)]).astype(np.uint32)
    out = {"in_" + k: v for k, v in wl.fields.items()}
    out |= dict(box_in=wl.box, bc=wl.bc, box=r["box"], keys=r["keys"], order=r["order"], leaves=r["leaves"],
                counts=r["counts"], prefixes=r["prefixes"], child_offsets=r["child_offsets"],
                internal_to_leaf=r["internal_to_leaf"], level_range=r["level_range"], nc=r["nc"],
                nbr_flat=flat, minDtCourant=np.array(r["minDtCourant"]),
                variant=np.array(variant), avclean=np.array(avclean))
    for k in O.FIELDS:
        if np.any(r[k] != 0):
            out["out_" + k] = r[k]
    for k, v in wl.params.items():
        out["param_" + k] = np.array(v)
    return out


def main() -> None:
    if not O.build_reference():
        raise SystemExit(f"reference sources not found under {REF}")
    ref = O.reference("fp64")
    std, ve = kat_outputs(ref.lib)
    np.savez_compressed(HERE / "kat_std.npz", **std)
    np.savez_compressed(HERE / "kat_ve.npz", **ve)
    for name, (factory, variant, avclean) in SWEEPS.items():
        np.savez_compressed(HERE / f"sweep_{name}.npz", **sweep_fixture(ref, factory(), variant, avclean))
    for p in sorted(HERE.glob("*.npz")):
        print(p.name, p.stat().st_size)


if __name__ == "__main__":
    main()
