"""ctypes declarations of the C ABI in include/sphgb.h and the loader of libsphgb.so.

The library is the only compute path: if it is missing or cannot be loaded, every entry
point raises.  There is no CPU fallback.
"""

from __future__ import annotations

import ctypes as C
from pathlib import Path

PKG = Path(__file__).resolve().parent
LIB_PATH = PKG / "libsphgb.so"

SPHGB_OK = 0
SPHGB_ERR_ARG = 1
SPHGB_ERR_NOCONV = 6
SPHGB_ERR_TOO_LARGE = 8
SPHGB_ERR_INPUT = 9
SPHGB_ERR_TIMEOUT = 10
SPHGB_FP64, SPHGB_MIXED = 0, 1
SPHGB_STD, SPHGB_VE = 0, 1
SPHGB_KERNEL_TABLE, SPHGB_KERNEL_SMOOTH = 0, 1

STATUS_NAMES = {0: "ok", 1: "invalid argument", 2: "CUDA runtime error", 3: "device allocation failed",
                4: "call out of order", 5: "octree traversal stack overflow",
                6: "h / neighbour-count iteration did not converge", 7: "no usable CUDA device",
                8: "request exceeds a fixed capacity",
                9: "non-finite coordinate, smoothing length or box limit, or h <= 0"}


class SphgbBox(C.Structure):
    _fields_ = [("lim", C.c_double * 6), ("bc", C.c_uint8 * 3)]


class SphgbParams(C.Structure):
    _fields_ = [("ng0", C.c_uint32), ("ngmax", C.c_uint32), ("bucket", C.c_uint32),
                ("gamma", C.c_double), ("Kcour", C.c_double), ("sincIndex", C.c_double),
                ("alphamin", C.c_double), ("alphamax", C.c_double), ("decay_constant", C.c_double),
                ("minDt", C.c_double)]


# order of the pointer members of sphgb_particles after n / precision / keys
DOUBLE_FIELDS = ["x", "y", "z", "u", "du"]
HYDRO_FIELDS = ["h", "m", "vx", "vy", "vz", "alpha", "rho", "p", "c", "xm", "kx", "gradh", "prho", "divv",
                "curlv", "c11", "c12", "c13", "c22", "c23", "c33", "ax", "ay", "az",
                "dV11", "dV12", "dV13", "dV22", "dV23", "dV33"]


class SphgbParticles(C.Structure):
    _fields_ = ([("n", C.c_int64), ("precision", C.c_int32), ("keys", C.c_void_p)]
                + [(f, C.c_void_p) for f in DOUBLE_FIELDS]
                + [(f, C.c_void_p) for f in HYDRO_FIELDS]
                + [("nc", C.c_void_p)])


class SphgbOctreeView(C.Structure):
    _fields_ = [("num_leaf_nodes", C.c_int64), ("num_nodes", C.c_int64), ("num_internal", C.c_int64),
                ("prefixes", C.c_void_p), ("child_offsets", C.c_void_p), ("internal_to_leaf", C.c_void_p),
                ("level_range", C.c_void_p), ("leaves", C.c_void_p), ("layout", C.c_void_p),
                ("centers", C.c_void_p), ("sizes", C.c_void_p), ("max_depth", C.c_int32)]


class SphgbStats(C.Structure):
    _fields_ = [("num_leaves", C.c_int64), ("num_nodes", C.c_int64), ("num_internal", C.c_int64),
                ("level_range", C.c_int32 * 23), ("nc_sum", C.c_int64), ("nc_max", C.c_uint32),
                ("capped", C.c_int64), ("h_iterations", C.c_int64), ("h_fails", C.c_int64),
                ("candidates", C.c_int64), ("fp64_rechecks", C.c_int64), ("refined_gradh", C.c_int64),
                ("refined_divv", C.c_int64)]


class SphgbSeeds(C.Structure):
    _fields_ = [("rho", C.c_void_p), ("ax", C.c_void_p), ("ay", C.c_void_p), ("az", C.c_void_p), ("du", C.c_void_p)]


class SphgbGrads(C.Structure):
    _fields_ = [(f, C.c_void_p) for f in ("x", "y", "z", "vx", "vy", "vz", "h", "u")]


class SphgbTimestep(C.Structure):
    _fields_ = [(f, C.c_double) for f in ("minDt", "minDt_m1", "ttot", "minDtCourant", "minDtRho", "maxDtIncrease",
                                          "g", "etaAcc", "eps")]


# name -> (argtypes); every function returns int status unless listed in RESTYPES
_P = C.c_void_p
_I64 = C.c_int64
SIGNATURES = {
    "sphgb_status_string": [C.c_int],
    "sphgb_last_cuda_error": [],
    "sphgb_version": [],
    "sphgb_create": [C.POINTER(C.c_void_p), C.c_int],
    "sphgb_destroy": [_P],
    "sphgb_set_stream": [_P, _P],
    "sphgb_set_params": [_P, C.POINTER(SphgbParams)],
    "sphgb_default_params": [C.POINTER(SphgbParams)],
    "sphgb_set_deterministic": [_P, C.c_int32],
    "sphgb_set_adjoint_tape": [_P, C.c_int32],
    "sphgb_set_mixed_refinement": [_P, C.c_int32],
    "sphgb_set_domain_mode": [_P, C.c_int32],
    "sphgb_set_kernel_form": [_P, C.c_int32],
    "sphgb_get_kernel_K": [_P, C.POINTER(C.c_double)],
    "sphgb_domain_sync": [_P, C.POINTER(SphgbParticles), C.POINTER(SphgbBox)],
    "sphgb_get_tree": [_P, C.POINTER(C.c_void_p), C.POINTER(C.c_void_p), C.POINTER(C.c_void_p),
                       C.POINTER(C.c_void_p), C.POINTER(C.c_void_p), C.POINTER(SphgbStats)],
    "sphgb_get_order": [_P, C.POINTER(C.c_void_p)],
    "sphgb_get_octree_view": [_P, C.POINTER(SphgbOctreeView)],
    "sphgb_get_params": [_P, C.POINTER(SphgbParams)],
    "sphgb_target_groups": [_P, C.c_int64, C.c_int64, C.c_void_p, C.c_int64, C.POINTER(C.c_int64)],
    "sphgb_apply_order": [_P, _P, C.c_int32],
    "sphgb_sort_by_key": [_P, _P, _P, _P, _P, _I64, C.c_int32],
    "sphgb_find_neighbors": [_P, _P, _P, _P, _P, C.c_int32, _I64, _I64, C.c_uint32, _P, _P],
    "sphgb_find_neighbors_sph": [_P, C.POINTER(SphgbParticles), _I64, _I64],
    "sphgb_export_neighbors": [_P, _P],
    "sphgb_compute_density": [_P, C.POINTER(SphgbParticles), _I64, _I64],
    "sphgb_compute_eos_std": [_P, C.POINTER(SphgbParticles), _I64, _I64],
    "sphgb_compute_iad": [_P, C.POINTER(SphgbParticles), _I64, _I64],
    "sphgb_compute_momentum_energy_std": [_P, C.POINTER(SphgbParticles), _I64, _I64, C.POINTER(C.c_double)],
    "sphgb_compute_xmass": [_P, C.POINTER(SphgbParticles), _I64, _I64],
    "sphgb_compute_ve_def_gradh": [_P, C.POINTER(SphgbParticles), _I64, _I64],
    "sphgb_compute_eos": [_P, C.POINTER(SphgbParticles), _I64, _I64],
    "sphgb_compute_iad_divv_curlv": [_P, C.POINTER(SphgbParticles), _I64, _I64],
    "sphgb_compute_av_switches": [_P, C.POINTER(SphgbParticles), _I64, _I64],
    "sphgb_compute_momentum_energy": [_P, C.POINTER(SphgbParticles), _I64, _I64, C.c_int32, _P,
                                      C.POINTER(C.c_double)],
    "sphgb_sweep": [_P, C.POINTER(SphgbParticles), C.POINTER(SphgbBox), C.c_int32, C.c_int32,
                    C.POINTER(C.c_double)],
    "sphgb_sweep_passes": [_P, C.POINTER(SphgbParticles), C.c_int32, C.c_int32, C.POINTER(C.c_double)],
    "sphgb_adjoint_std": [_P, C.POINTER(SphgbParticles), C.POINTER(SphgbSeeds), C.POINTER(SphgbGrads),
                          C.c_int32],
    "sphgb_adjoint_ve": [_P, C.POINTER(SphgbParticles), _P, C.c_int32, C.POINTER(SphgbSeeds),
                         C.POINTER(SphgbGrads), C.c_int32],
    "sphgb_get_stats": [_P, C.POINTER(SphgbStats)],
    "sphgb_get_timings": [_P, C.POINTER(C.c_float), C.c_int32],
    "sphgb_kernel_launches": [_P, C.POINTER(C.c_int64)],
    "sphgb_measure_fma_peak": [_P, C.c_int32, C.POINTER(C.c_double)],
    "sphgb_sfc_keys_noalloc": [_P, _P, _P, _I64, C.POINTER(SphgbBox), _P, _P],
    "sphgb_compute_positions": [_P, C.POINTER(SphgbParticles), C.POINTER(SphgbBox), _P, _P, _P, _P,
                                C.POINTER(SphgbTimestep), _I64, _I64],
    "sphgb_update_smoothing_length": [_P, C.POINTER(SphgbParticles), _I64, _I64],
    "sphgb_rho_timestep": [_P, C.POINTER(SphgbParticles), _I64, _I64, C.c_double, C.POINTER(C.c_double)],
    "sphgb_acceleration_timestep": [_P, C.POINTER(SphgbParticles), _I64, _I64, C.c_double, C.c_double,
                                    C.POINTER(C.c_double)],
    "sphgb_compute_timestep": [_P, C.POINTER(SphgbParticles), _I64, _I64, C.POINTER(SphgbTimestep)],
    "sphgb_conserved_quantities": [_P, C.POINTER(SphgbParticles), _I64, _I64, C.POINTER(C.c_double)],
}
RESTYPES = {"sphgb_status_string": C.c_char_p, "sphgb_last_cuda_error": C.c_char_p}

_lib = None


def load(path: Path | None = None) -> C.CDLL:
    """Load libsphgb.so once; raises OSError when it is absent (build it with __graft_entry__.build())."""
    global _lib
    if _lib is not None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise OSError(f"{p} not found: the sm_103a extension must be built (python -c "
                      f"'import __graft_entry__ as g; g.build()')")
    lib = C.CDLL(str(p))
    for name, args in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = RESTYPES.get(name, C.c_int)
    _lib = lib
    return lib


class SphgbError(RuntimeError):
    def __init__(self, status: int, where: str):
        lib = load()
        msg = lib.sphgb_status_string(status).decode()
        if status == 2:
            msg += ": " + lib.sphgb_last_cuda_error().decode()
        super().__init__(f"{where}: {msg} (status {status})")
        self.status = status


def check(status: int, where: str, allow=(SPHGB_OK,)) -> int:
    if status not in allow:
        raise SphgbError(status, where)
    return status
