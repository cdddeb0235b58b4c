"""ctypes driver for the oracle interface (oracle/oracle_api.h).

TEST INFRASTRUCTURE ONLY: tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg
import this module; the product package never does.

``port()`` loads my C++/OpenMP restatement (oracle/liboracle.so).  ``reference(kind)`` loads
the reference's own CPU code compiled from its headers (oracle/_ref/libref_{fp64,f32}.so);
those exist only where the reference sources were present at build time.
"""

from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
# the reference checkout: $SPHGB_REFERENCE, else a directory "reference" beside the repository
REFERENCE_DEFAULT = HERE.parent.parent / "reference"

FIELDS = ["x", "y", "z", "h", "m", "u", "vx", "vy", "vz", "alpha",
          "rho", "p", "c", "c11", "c12", "c13", "c22", "c23", "c33",
          "ax", "ay", "az", "du", "xm", "kx", "gradh", "prho", "divv", "curlv",
          "dV11", "dV12", "dV13", "dV22", "dV23", "dV33"]
NF = len(FIELDS)
INPUT_FIELDS = ["x", "y", "z", "h", "m", "u", "vx", "vy", "vz", "alpha"]

OS_KEYS, OS_TREE, OS_NBR, OS_HYDRO = 1, 2, 4, 8
ALL_STAGES = 15


class OracleIn(C.Structure):
    _fields_ = [("n", C.c_int64), ("f", C.c_void_p * NF), ("box", C.c_double * 6), ("bc", C.c_uint8 * 3),
                ("fit_box", C.c_uint8), ("ng0", C.c_uint32), ("ngmax", C.c_uint32), ("bucket", C.c_uint32),
                ("gamma", C.c_double), ("Kcour", C.c_double), ("minDt", C.c_double),
                ("alphamin", C.c_double), ("alphamax", C.c_double), ("decay", C.c_double),
                ("sincIndex", C.c_double), ("variant", C.c_int32), ("avclean", C.c_int32),
                ("stages", C.c_int32), ("nthreads", C.c_int32)]


class OracleOut(C.Structure):
    _fields_ = [("keys", C.c_void_p), ("order", C.c_void_p), ("leaves_cap", C.c_int64),
                ("leaves", C.c_void_p), ("counts", C.c_void_p), ("nodes_cap", C.c_int64),
                ("prefixes", C.c_void_p), ("child_offsets", C.c_void_p), ("internal_to_leaf", C.c_void_p),
                ("nc", C.c_void_p), ("nbr", C.c_void_p), ("f", C.c_void_p * NF),
                ("box", C.c_double * 6), ("num_leaves", C.c_int64), ("num_nodes", C.c_int64),
                ("num_internal", C.c_int64), ("level_range", C.c_int32 * 23), ("h_iter_fails", C.c_int64),
                ("minDtCourant", C.c_double), ("t_keys", C.c_double), ("t_tree", C.c_double),
                ("t_nbr", C.c_double), ("t_hydro", C.c_double), ("threads_used", C.c_int32),
                ("centers", C.c_void_p), ("sizes", C.c_void_p)]


def build_port() -> Path:
    """Compile liboracle.so from oracle/sph_oracle.cpp (g++ -fopenmp -ffp-contract=off)."""
    subprocess.run(["make", "-s", "-C", str(HERE), "liboracle.so"], check=True)
    return HERE / "liboracle.so"


def build_port_timed() -> Path:
    """Compile liboracle_o3.so: the same restatement with release flags, for the timed CPU baseline."""
    subprocess.run(["make", "-s", "-C", str(HERE), "liboracle_o3.so"], check=True)
    return HERE / "liboracle_o3.so"


def build_reference() -> bool:
    """Compile the reference-driven oracle if the reference sources are present here."""
    ref = Path(os.environ.get("SPHGB_REFERENCE", REFERENCE_DEFAULT))
    if not (ref / "domain" / "include" / "cstone").is_dir():
        return False
    subprocess.run(["make", "-s", "-C", str(HERE), "ref", f"REF={ref}"], check=True)
    return True


class Oracle:
    def __init__(self, lib_path: Path, name: str):
        self.name = name
        self.path = Path(lib_path)
        self.lib = C.CDLL(str(self.path))
        self.lib.oracle_sweep.argtypes = [C.POINTER(OracleIn), C.POINTER(OracleOut)]
        self.lib.oracle_sweep.restype = C.c_int
        self.lib.oracle_kernel_K.argtypes = [C.c_double]
        self.lib.oracle_kernel_K.restype = C.c_double
        self.lib.oracle_tables.argtypes = [C.c_double, C.c_void_p, C.c_void_p]

    def kernel_K(self, sinc_index: float = 6.0) -> float:
        return self.lib.oracle_kernel_K(sinc_index)

    def tables(self, sinc_index: float = 6.0):
        wh = np.zeros(20000)
        whd = np.zeros(20000)
        self.lib.oracle_tables(sinc_index, wh.ctypes.data, whd.ctypes.data)
        return wh, whd

    def sweep(self, wl, variant: str = "ve", avclean: bool = False, stages: int = ALL_STAGES,
              want_nbr: bool = True, want_tree: bool = True, nthreads: int = 0, fit_box: bool | None = None):
        """Run the chain on a Workload; returns a dict of numpy arrays (sorted order) + scalars."""
        n = wl.n
        p = wl.params
        inp = OracleIn()
        inp.n = n
        keep = []
        for k, name in enumerate(FIELDS):
            if name in INPUT_FIELDS and name in wl.fields:
                a = np.ascontiguousarray(wl.fields[name], dtype=np.float64)
                keep.append(a)
                inp.f[k] = a.ctypes.data
        for k in range(6):
            inp.box[k] = float(wl.box[k])
        for k in range(3):
            inp.bc[k] = int(wl.bc[k])
        inp.fit_box = int(fit_box if fit_box is not None else any(b == 0 for b in wl.bc))
        inp.ng0, inp.ngmax, inp.bucket = p["ng0"], p["ngmax"], p["bucket"]
        inp.gamma, inp.Kcour, inp.minDt = p["gamma"], p["Kcour"], p["minDt"]
        inp.alphamin, inp.alphamax, inp.decay = p["alphamin"], p["alphamax"], p["decay_constant"]
        inp.sincIndex = p["sincIndex"]
        inp.variant = 0 if variant == "std" else 1
        inp.avclean = int(avclean)
        inp.stages = stages
        inp.nthreads = nthreads

        out = OracleOut()
        res = {"keys": np.zeros(n, np.uint64), "order": np.zeros(n, np.uint32)}
        out.keys = res["keys"].ctypes.data
        out.order = res["order"].ctypes.data
        if want_tree:
            cap = n + 2
            res["leaves"] = np.zeros(cap + 1, np.uint64)
            res["counts"] = np.zeros(cap, np.uint32)
            ncap = 2 * cap + 8
            res["prefixes"] = np.zeros(ncap, np.uint64)
            res["child_offsets"] = np.zeros(ncap, np.int32)
            res["internal_to_leaf"] = np.zeros(ncap, np.int32)
            res["centers"] = np.zeros(3 * ncap)
            res["sizes"] = np.zeros(3 * ncap)
            out.centers = res["centers"].ctypes.data
            out.sizes = res["sizes"].ctypes.data
            out.leaves_cap = cap
            out.nodes_cap = ncap
            out.leaves = res["leaves"].ctypes.data
            out.counts = res["counts"].ctypes.data
            out.prefixes = res["prefixes"].ctypes.data
            out.child_offsets = res["child_offsets"].ctypes.data
            out.internal_to_leaf = res["internal_to_leaf"].ctypes.data
        res["nc"] = np.zeros(n, np.uint32)
        out.nc = res["nc"].ctypes.data
        if want_nbr:
            res["nbr"] = np.zeros(n * p["ngmax"], np.uint32)
            out.nbr = res["nbr"].ctypes.data
        for k, name in enumerate(FIELDS):
            res[name] = np.zeros(n)
            out.f[k] = res[name].ctypes.data
        rc = self.lib.oracle_sweep(C.byref(inp), C.byref(out))
        if rc != 0:
            raise RuntimeError(f"oracle_sweep failed with {rc}")
        L = out.num_leaves
        if want_tree:
            res["leaves"] = res["leaves"][:L + 1]
            res["counts"] = res["counts"][:L]
            nn = out.num_nodes
            for k in ("prefixes", "child_offsets", "internal_to_leaf"):
                res[k] = res[k][:nn]
            for k in ("centers", "sizes"):
                res[k] = res[k][:3 * nn].reshape(nn, 3)
        res["num_leaves"] = L
        res["num_nodes"] = out.num_nodes
        res["num_internal"] = out.num_internal
        res["level_range"] = np.array(out.level_range[:], dtype=np.int32)
        res["box"] = np.array(out.box[:])
        res["minDtCourant"] = out.minDtCourant
        res["h_iter_fails"] = out.h_iter_fails
        res["times"] = dict(keys=out.t_keys, tree=out.t_tree, nbr=out.t_nbr, hydro=out.t_hydro)
        res["threads"] = out.threads_used
        return res


def port() -> Oracle:
    path = HERE / "liboracle.so"
    if not path.exists():
        build_port()
    return Oracle(path, "port")


def port_timed() -> Oracle:
    """the restatement built with release flags (timed CPU baseline only; parity uses port())"""
    path = HERE / "liboracle_o3.so"
    if not path.exists():
        build_port_timed()
    return Oracle(path, "port-O3")


def reference(kind: str = "fp64") -> Oracle | None:
    path = HERE / "_ref" / f"libref_{kind}.so"
    if not path.exists():
        return None
    return Oracle(path, f"reference-{kind}")


def sorted_sets(nbr: np.ndarray, nc: np.ndarray, ngmax: int) -> np.ndarray:
    """Neighbour lists sorted per particle, entries beyond min(nc-1, ngmax) zeroed."""
    n = nc.shape[0]
    a = nbr.reshape(n, ngmax).astype(np.int64).copy()
    cnt = np.minimum(nc.astype(np.int64) - 1, ngmax)
    mask = np.arange(ngmax)[None, :] >= cnt[:, None]
    a[mask] = np.iinfo(np.int64).max
    a.sort(axis=1)
    a[mask] = -1
    return a

def _dptr(a):
    return a.ctypes.data if a is not None else None


def run_positions(lib, f: dict, dt: float, dt_m1: float, box, bc) -> None:
    """oracle_positions on numpy float64 arrays in f (x y z vx vy vz ax ay az xm1 ym1 zm1 u du dum1 h),
    updated in place"""
    fn = lib.oracle_positions
    fn.argtypes = [C.c_int64] + [C.c_void_p] * 16 + [C.c_double, C.c_double, C.c_void_p, C.c_void_p]
    fn.restype = C.c_int
    b = np.ascontiguousarray(box, dtype=np.float64)
    c = np.ascontiguousarray(bc, dtype=np.uint8)
    names = ["x", "y", "z", "vx", "vy", "vz", "ax", "ay", "az", "xm1", "ym1", "zm1", "u", "du", "dum1", "h"]
    rc = fn(len(f["x"]), *[_dptr(f.get(k)) for k in names], dt, dt_m1, b.ctypes.data, c.ctypes.data)
    assert rc == 0


def run_update_h(lib, ng0: int, nc: np.ndarray, h: np.ndarray) -> None:
    fn = lib.oracle_update_h
    fn.argtypes = [C.c_int64, C.c_uint32, C.c_void_p, C.c_void_p]
    fn.restype = C.c_int
    assert fn(len(h), ng0, nc.ctypes.data, h.ctypes.data) == 0


def run_conserved(lib, f: dict) -> np.ndarray:
    fn = lib.oracle_conserved
    fn.argtypes = [C.c_int64] + [C.c_void_p] * 9
    fn.restype = C.c_int
    out = np.zeros(8)
    names = ["x", "y", "z", "vx", "vy", "vz", "m", "u"]
    assert fn(len(f["x"]), *[_dptr(f.get(k)) for k in names], out.ctypes.data) == 0
    return out


# ---- single-rank focus tree across syncs (restatement, numpy) ----
KEY_END = np.uint64(1) << np.uint64(63)
MAX_LEVEL = 21


def _node_range(level: int) -> int:
    return 1 << (3 * (MAX_LEVEL - level))


def focus_rebalance_once(leaves: np.ndarray, counts: np.ndarray, bucket: int) -> np.ndarray:
    """One update of the single-rank focus tree (CombinedUpdate::updateFocus,
    domain/include/cstone/focus/octree_focus.hpp:65-113, with the decisions of
    focus/rebalance.hpp:32-66 and protectAncestors :152-165 at one rank, where the focus range is
    the whole key range, so the MAC criterion never decides and the mandatory keys 0 and 2^63 are
    always present).  leaves: cornerstone leaves (L + 1 keys); counts: particle counts of the L
    leaves from the previous sync.  A leaf whose parent holds more than bucket particles splits in
    8 (if it holds more than bucket itself and lies above the last level) or stays; otherwise the
    whole subtree under its highest ancestor holding at most bucket particles collapses into that
    ancestor, whose left-most leaf keeps the start key."""
    lv = [int(k) for k in leaves]
    L = len(lv) - 1
    layout = np.concatenate([[0], np.cumsum(np.asarray(counts, dtype=np.int64))])
    import bisect

    def count(start: int, level: int) -> int:
        a = bisect.bisect_left(lv, start)
        b = bisect.bisect_left(lv, start + _node_range(level))
        return int(layout[b] - layout[a])

    out = []
    for k in range(L):
        s, span = lv[k], lv[k + 1] - lv[k]
        level = MAX_LEVEL - (span.bit_length() - 1) // 3
        if level == 0:
            op = 8 if counts[k] > bucket else 1
        else:
            ps = s & ~(_node_range(level - 1) - 1)
            if count(ps, level - 1) > bucket:
                op = 8 if (counts[k] > bucket and level < MAX_LEVEL) else 1
            else:
                a_s, a_l = ps, level - 1
                while a_l > 0:
                    pp = a_s & ~(_node_range(a_l - 1) - 1)
                    if count(pp, a_l - 1) > bucket:
                        break
                    a_s, a_l = pp, a_l - 1
                op = 1 if s == a_s else 0
        if op == 1:
            out.append(s)
        elif op == 8:
            out.extend(s + c * _node_range(level + 1) for c in range(8))
    out.append(int(KEY_END))
    return np.array(out, dtype=np.uint64)


def leaf_counts(leaves: np.ndarray, sorted_keys: np.ndarray) -> np.ndarray:
    """particles per leaf cell of a cornerstone leaf array"""
    pos = np.searchsorted(sorted_keys, leaves)
    return np.diff(pos)
