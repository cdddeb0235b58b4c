"""The arithmetic of the hand-written adjoints (sphexa_gb300/csrc/adjoint_ve.cuh and adjoint_std.cuh,
the functions the device kernels call) against torch autograd on the CPU, without a GPU.

tests/adjoint_host/ve_adjoint_host.cpp runs the device pass sequence as sequential loops over the
oracle's neighbour lists and forward state (the oracle port's VE sweep); the reference gradient is
torch autograd through tests/torch_reference.py::ve_chain on the same edges.  Both the one-term
form (every list entry) and the mutual-pair form (each pair whose ends list each other once) are
checked, with and without the avClean correction, on a set where the AV switch takes both of its
branches and the Atwood weights all three of theirs.
"""

import ctypes as C
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
P = C.c_void_p


class HostIn(C.Structure):
    _fields_ = ([("n", C.c_int64)]
                + [(k, P) for k in "x y z vx vy vz h u m alpha0 alpha xm kx gradh prho c divv".split()]
                + [("C", P * 6), ("dV", P * 6), ("off", P), ("idx", P), ("wh", P), ("whd", P), ("ntab", C.c_int64),
                   ("K", C.c_double), ("gamma", C.c_double), ("L", C.c_double * 3), ("pbc", C.c_int * 3),
                   ("dt", C.c_double), ("amin", C.c_double), ("amax", C.c_double), ("decay", C.c_double),
                   ("avClean", C.c_int)]
                + [(k, P) for k in "sRho sAx sAy sAz sDu gx gy gz gvx gvy gvz gh gu".split()])


def _build(tmp_path_factory, name: str) -> C.CDLL:
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    so = tmp_path_factory.mktemp("adjhost") / f"lib{name}.so"
    cmd = [gxx, "-O2", "-std=c++17", "-shared", "-fPIC", "-I", str(ROOT / "sphexa_gb300" / "csrc"),
           str(ROOT / "tests" / "adjoint_host" / f"{name}.cpp"), "-o", str(so)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return C.CDLL(str(so))


@pytest.fixture(scope="module")
def host_lib(tmp_path_factory):
    lib = _build(tmp_path_factory, "ve_adjoint_host")
    lib.ve_adj_host.argtypes = [C.POINTER(HostIn), C.c_int]
    lib.ve_adj_host.restype = C.c_int
    return lib


class StdHostIn(C.Structure):
    _fields_ = ([("n", C.c_int64)] + [(k, P) for k in "x y z vx vy vz h u m rho p c".split()]
                + [("C", P * 6), ("off", P), ("idx", P), ("wh", P), ("ntab", C.c_int64), ("K", C.c_double),
                   ("gamma", C.c_double), ("L", C.c_double * 3), ("pbc", C.c_int * 3)]
                + [(k, P) for k in "sRho sAx sAy sAz sDu gx gy gz gvx gvy gvz gh gu".split()])


def test_std_adjoint_arithmetic_matches_autograd(port, tmp_path_factory):
    torch = pytest.importorskip("torch")
    from sphexa_gb300 import workloads as W
    from torch_reference import std_chain
    lib = _build(tmp_path_factory, "std_adjoint_host")
    lib.std_adj_host.argtypes = [C.POINTER(StdHostIn), C.c_int]
    port.lib.oracle_kernel_K.restype = C.c_double
    wl = W.fourier(10, seed=7, rho_seed=55, v_seed=555)
    rng = np.random.Generator(np.random.PCG64(2))
    wl.fields["u"] = wl.fields["u"] * rng.uniform(0.8, 1.2, wl.n)
    wl.fields["h"] = wl.fields["h"] * rng.uniform(0.97, 1.03, wl.n)
    ref = port.sweep(wl, "std", False)
    n, ng, p = wl.n, wl.params["ngmax"], wl.params
    nb = ref["nbr"].reshape(n, ng).astype(np.int64)
    cnt = np.minimum(ref["nc"].astype(np.int64) - 1, ng)
    off = np.concatenate([[0], np.cumsum(cnt)]).astype(np.int64)
    ej = np.concatenate([nb[k, :cnt[k]] for k in range(n)]).astype(np.int64)
    ei = np.repeat(np.arange(n), cnt)
    wh, _ = port.tables(6.0)
    K = port.lib.oracle_kernel_K(6.0)
    seeds = {k: rng.normal(size=n) for k in ("rho", "ax", "ay", "az", "du")}
    t = lambda a: torch.tensor(np.ascontiguousarray(a), dtype=torch.float64)
    names = ("x", "y", "z", "vx", "vy", "vz", "h", "u")
    inp = [t(ref[k]).requires_grad_(True) for k in names]
    out = std_chain(*inp, t(ref["m"]), torch.tensor(ei), torch.tensor(ej), t(wh), K, p["gamma"],
                    t(wl.box[1::2] - wl.box[0::2]), [True] * 3)
    L = sum((o * t(seeds[k])).sum() for o, k in zip(out, ("rho", "ax", "ay", "az", "du")))
    L.backward()
    a = StdHostIn()
    keep = []

    def ptr(arr):
        arr = np.ascontiguousarray(arr, dtype=np.float64)
        keep.append(arr)
        return arr.ctypes.data

    a.n = n
    for k in "x y z vx vy vz h u m rho p c".split():
        setattr(a, k, ptr(ref[k]))
    for q, k in enumerate(("c11", "c12", "c13", "c22", "c23", "c33")):
        a.C[q] = ptr(ref[k])
    a.off, a.idx, a.wh, a.ntab, a.K, a.gamma = off.ctypes.data, ej.ctypes.data, ptr(wh), len(wh), K, p["gamma"]
    for k in range(3):
        a.L[k] = wl.box[2 * k + 1] - wl.box[2 * k]
        a.pbc[k] = 1
    a.sRho, a.sAx, a.sAy, a.sAz, a.sDu = (ptr(seeds[k]) for k in ("rho", "ax", "ay", "az", "du"))
    g = {k: np.zeros(n) for k in names}
    a.gx, a.gy, a.gz, a.gvx, a.gvy, a.gvz, a.gh, a.gu = (g[k].ctypes.data for k in names)
    for mode in (0, 1):
        assert lib.std_adj_host(C.byref(a), mode) == 0
        for k, ti in zip(names, inp):
            gr = ti.grad.numpy()
            err = np.linalg.norm(g[k] - gr) / np.linalg.norm(gr)
            assert err <= 1e-12, f"mode {mode} {k}: {err:.3e}"


@pytest.mark.parametrize("av_clean", [False, True])
def test_ve_adjoint_arithmetic_matches_autograd(port, host_lib, av_clean):
    torch = pytest.importorskip("torch")
    from sphexa_gb300 import workloads as W
    from torch_reference import ve_chain
    port.lib.oracle_kernel_K.restype = C.c_double
    wl = W.fourier(10, seed=7, rho_seed=55, v_seed=555)
    rng = np.random.Generator(np.random.PCG64(2))
    wl.fields["u"] = wl.fields["u"] * rng.uniform(0.8, 1.2, wl.n)
    wl.fields["h"] = wl.fields["h"] * rng.uniform(0.97, 1.03, wl.n)
    wl.fields["alpha"] = rng.uniform(0.05, 0.5, wl.n)
    wl.params["minDt"] = 1e-2
    ref = port.sweep(wl, "ve", av_clean)
    n, ng, p = wl.n, wl.params["ngmax"], wl.params
    nb = ref["nbr"].reshape(n, ng).astype(np.int64)
    cnt = np.minimum(ref["nc"].astype(np.int64) - 1, ng)
    off = np.concatenate([[0], np.cumsum(cnt)]).astype(np.int64)
    ej = np.concatenate([nb[k, :cnt[k]] for k in range(n)]).astype(np.int64)
    ei = np.repeat(np.arange(n), cnt)
    wh, whd = port.tables(6.0)
    K = port.lib.oracle_kernel_K(6.0)
    alpha0 = np.ascontiguousarray(wl.fields["alpha"][ref["order"]])
    seeds = {k: rng.normal(size=n) for k in ("rho", "ax", "ay", "az", "du")}

    # branch coverage of the set: all three Atwood ranges, alpha rising and decaying
    rho = ref["kx"] * ref["m"] / ref["xm"]
    At = np.abs(rho[ei] - rho[ej]) / (rho[ei] + rho[ej])
    assert np.any(At < 0.1) and np.any((At > 0.1) & (At < 0.2)) and np.any(At > 0.2)
    assert np.any(ref["alpha"] > alpha0) and np.any(ref["alpha"] < alpha0)

    t = lambda a: torch.tensor(np.ascontiguousarray(a), dtype=torch.float64)
    names = ("x", "y", "z", "vx", "vy", "vz", "h", "u")
    inp = [t(ref[k]).requires_grad_(True) for k in names]
    out = ve_chain(*inp, t(ref["m"]), t(alpha0), torch.tensor(ei), torch.tensor(ej), t(wh), t(whd), K, p["gamma"],
                   t(wl.box[1::2] - wl.box[0::2]), [True] * 3, p["minDt"], p["alphamin"], p["alphamax"],
                   p["decay_constant"], av_clean)
    for name, o in zip(("rho", "ax", "ay", "az", "du"), out):  # the restatement is the oracle's chain
        assert np.max(np.abs(o.detach().numpy() - ref[name])) <= 1e-13 * np.max(np.abs(ref[name])), name
    L = sum((o * t(seeds[k])).sum() for o, k in zip(out, ("rho", "ax", "ay", "az", "du")))
    L.backward()

    a = HostIn()
    keep = []

    def ptr(arr):
        arr = np.ascontiguousarray(arr, dtype=np.float64)
        keep.append(arr)
        return arr.ctypes.data

    a.n = n
    for k in "x y z vx vy vz h u m alpha xm kx gradh prho c divv".split():
        setattr(a, k, ptr(ref[k]))
    a.alpha0 = ptr(alpha0)
    for q, k in enumerate(("c11", "c12", "c13", "c22", "c23", "c33")):
        a.C[q] = ptr(ref[k])
    for q, k in enumerate(("dV11", "dV12", "dV13", "dV22", "dV23", "dV33")):
        a.dV[q] = ptr(ref[k])
    a.off, a.idx = off.ctypes.data, ej.ctypes.data
    a.wh, a.whd, a.ntab = ptr(wh), ptr(whd), len(wh)
    a.K, a.gamma = K, p["gamma"]
    for k in range(3):
        a.L[k] = wl.box[2 * k + 1] - wl.box[2 * k]
        a.pbc[k] = 1
    a.dt, a.amin, a.amax, a.decay = p["minDt"], p["alphamin"], p["alphamax"], p["decay_constant"]
    a.avClean = int(av_clean)
    a.sRho, a.sAx, a.sAy, a.sAz, a.sDu = (ptr(seeds[k]) for k in ("rho", "ax", "ay", "az", "du"))
    g = {k: np.zeros(n) for k in names}
    a.gx, a.gy, a.gz, a.gvx, a.gvy, a.gvz, a.gh, a.gu = (g[k].ctypes.data for k in names)
    for mode in (0, 1):
        assert host_lib.ve_adj_host(C.byref(a), mode) == 0
        for k, ti in zip(names, inp):
            gr = ti.grad.numpy()
            err = np.linalg.norm(g[k] - gr) / np.linalg.norm(gr)
            assert err <= 1e-12, f"mode {mode} {k}: {err:.3e}"
