"""Flops per pair of every pair pass, counted on the reference's own j-loops.

MEASUREMENT INFRASTRUCTURE: builds oracle/_ref/libref_flops.so (oracle/ref/flop_count.cpp,
the reference j-loop templates instantiated on a counting scalar), runs my oracle port for the
inputs and neighbour lists of a workload, counts every loop over every particle, and writes
oracle/flop_table.json.  Needs the reference sources (SPHGB_REFERENCE, default the mounted
reference) — the committed json is what the rest of the repository uses.

Per particle i the count is flops_i = a + b * pairs_i on a smooth piece; the table gives the
least-squares b (flop per pair), a (flop per particle: the loop's prologue and epilogue) and the
workload mean sum(flops) / sum(pairs), which is what a roofline over pairs uses.

    python oracle/flop_table.py            # writes oracle/flop_table.json, prints a table
"""

from __future__ import annotations

import ctypes as C
import json
import os
import subprocess
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path[0] = str(HERE.parent)  # import `oracle` as the package at the repository root

from oracle import oracle as O  # noqa: E402
from sphexa_gb300 import workloads as W  # noqa: E402

REF = Path(os.environ.get("SPHGB_REFERENCE", Path(__file__).resolve().parents[2] / "reference"))
OJ = dict(xmass=0, gradh=1, iad_std=2, iad_ve=3, divv=4, av=5, me_std=6, me_ve=7)
OPS = ["add", "mul", "div", "sqrt", "transc", "cmp"]


class JIn(C.Structure):
    _fields_ = [("n", C.c_int64), ("f", C.c_void_p * O.NF), ("neighbors", C.c_void_p), ("count", C.c_uint32),
                ("K", C.c_double), ("box", C.c_double * 6), ("bc", C.c_uint8 * 3), ("sincIndex", C.c_double),
                ("dt", C.c_double), ("alphamin", C.c_double), ("alphamax", C.c_double), ("decay", C.c_double),
                ("loop", C.c_int32), ("avclean", C.c_int32)]


def build() -> Path:
    subprocess.run(["make", "-s", "-C", str(HERE), f"REF={REF}", "flops"], check=True)
    return HERE / "_ref" / "libref_flops.so"


# (pass name, loop, avclean, which sweep provides its inputs)
PASSES = [("density_std", "xmass", 0, "std"), ("iad_std", "iad_std", 0, "std"), ("me_std", "me_std", 0, "std"),
          ("xmass", "xmass", 0, "ve"), ("gradh", "gradh", 0, "ve"), ("iad_ve", "iad_ve", 0, "ve"),
          ("divv_curlv", "divv", 0, "ve"), ("divv_curlv_clean", "divv", 1, "ve_clean"), ("av", "av", 0, "ve"),
          ("me_ve", "me_ve", 0, "ve"), ("me_ve_clean", "me_ve", 1, "ve_clean")]


def count_workload(lib, port, wl) -> dict:
    params = wl.params
    sweeps = {"std": port.sweep(wl, "std"), "ve": port.sweep(wl, "ve"), "ve_clean": port.sweep(wl, "ve", avclean=True)}
    K = port.kernel_K(6.0)
    fn = lib.oracle_count_jloop
    fn.argtypes = [C.POINTER(JIn), C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p, C.c_void_p]
    fn.restype = C.c_int
    out = {}
    for name, loop, avclean, src in PASSES:
        res = sweeps[src]
        n = wl.n
        j = JIn()
        j.n = n
        keep = []
        for k, fname in enumerate(O.FIELDS):
            a = np.ascontiguousarray(res[fname], dtype=np.float64)
            keep.append(a)
            j.f[k] = a.ctypes.data
        j.K = K
        for k in range(6):
            j.box[k] = res["box"][k]
        for k in range(3):
            j.bc[k] = int(wl.bc[k])
        j.sincIndex = 6.0
        j.dt, j.alphamin, j.alphamax, j.decay = params["minDt"], params["alphamin"], params["alphamax"], params["decay_constant"]
        j.loop = OJ[loop]
        j.avclean = avclean
        nbr = np.ascontiguousarray(res["nbr"], dtype=np.uint32)
        nc = np.ascontiguousarray(res["nc"], dtype=np.uint32)
        flops = np.zeros(n, np.uint64)
        tot = np.zeros(6, np.uint64)
        rc = fn(C.byref(j), nbr.ctypes.data, nc.ctypes.data, params["ngmax"], flops.ctypes.data, tot.ctypes.data)
        assert rc == 0, rc
        pairs = np.minimum(nc.astype(np.int64) - 1, params["ngmax"])
        A = np.stack([np.ones(n), pairs.astype(np.float64)], axis=1)
        (a0, b0), *_ = np.linalg.lstsq(A, flops.astype(np.float64), rcond=None)
        P = int(pairs.sum())
        out[name] = dict(flop_per_pair_mean=float(flops.sum()) / P, flop_per_pair_fit=float(b0),
                         flop_per_particle_fit=float(a0),
                         ops_per_pair={op: float(tot[k]) / P for k, op in enumerate(OPS)},
                         pairs=P, particles=n)
    return out


def main() -> None:
    lib = C.CDLL(str(build()))
    port = O.port()
    table = {"convention": "reference j-loops on a counting scalar (oracle/ref/flop_count.cpp): + - * / sqrt and "
                           "transcendental calls 1 flop each (an FMA is 2), comparisons counted apart, not flops",
             "workloads": {}}
    for label, wl in (("sedov_jit_20", W.sedov(20, jitter=0.25, seed=2)),
                      ("fourier_jit_20", W.fourier(20, seed=3))):
        table["workloads"][label] = count_workload(lib, port, wl)
    (HERE / "flop_table.json").write_text(json.dumps(table, indent=1) + "\n")
    print(f"{'pass':18s} " + " ".join(f"{w:>26s}" for w in table["workloads"]))
    for name, *_ in PASSES:
        cells = []
        for w in table["workloads"].values():
            r = w[name]
            cells.append(f"{r['flop_per_pair_mean']:7.1f} ({r['flop_per_pair_fit']:6.1f}+{r['flop_per_particle_fit']:5.0f}/i)")
        print(f"{name:18s} " + " ".join(f"{c:>26s}" for c in cells))


if __name__ == "__main__":
    main()
