"""Host-side mirror of the reference's hot-path interface over the C ABI.

Names follow the reference: ``ParticlesData`` holds the SoA fields of
``sphexa::ParticlesData<GpuTag>`` (sph/include/sph/particles_data.hpp:63-391) as torch device
tensors; ``Domain`` stands in for ``cstone::Domain::sync`` + ``octreeProperties`` at one rank;
``find_neighbors`` / ``find_neighbors_sfc`` / ``compute_*`` take the arguments of
``cstone::findNeighbors`` and the ``sph::compute*`` drivers.  Every call goes through
libsphgb.so; nothing here computes physics.
"""

from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np
import torch

from . import _lib
from ._lib import SPHGB_FP64, SPHGB_MIXED, SPHGB_STD, SPHGB_VE, check

PRECISIONS = {"fp64": SPHGB_FP64, "mixed": SPHGB_MIXED}

# fields that are FP64 in both precisions (the reference's RealType fields)
REAL_FIELDS = ("x", "y", "z", "u", "du")
HYDRO_FIELDS = _lib.HYDRO_FIELDS
STD_OUT = ("rho", "p", "c", "c11", "c12", "c13", "c22", "c23", "c33", "ax", "ay", "az")
VE_OUT = ("xm", "kx", "gradh", "prho", "c", "rho", "p", "c11", "c12", "c13", "c22", "c23", "c33", "divv", "curlv",
          "ax", "ay", "az")
DV = ("dV11", "dV12", "dV13", "dV22", "dV23", "dV33")
INPUTS = ("x", "y", "z", "h", "m", "u", "vx", "vy", "vz", "alpha")


@dataclass
class Box:
    """cstone::Box: limits [xmin xmax ymin ymax zmin zmax] and boundary per axis (0 open, 1 periodic)."""
    lim: np.ndarray
    bc: np.ndarray

    def to_c(self) -> _lib.SphgbBox:
        b = _lib.SphgbBox()
        for k in range(6):
            b.lim[k] = float(self.lim[k])
        for k in range(3):
            b.bc[k] = int(self.bc[k])
        return b

    def update_from(self, b: _lib.SphgbBox) -> None:
        self.lim = np.array(b.lim[:], dtype=np.float64)


class Context:
    """An sphgb context on one CUDA device (tree, neighbour lists, tables, scratch)."""

    def __init__(self, device: int = 0, stream: torch.cuda.Stream | None = None, **params):
        self.lib = _lib.load()
        self.device = device
        h = C.c_void_p()
        check(self.lib.sphgb_create(C.byref(h), device), "sphgb_create")
        self.h = h
        self.params = _lib.SphgbParams()
        self.lib.sphgb_default_params(C.byref(self.params))
        if params:
            self.set_params(**params)
        if stream is not None:
            self.set_stream(stream)

    def set_stream(self, stream: torch.cuda.Stream) -> None:
        check(self.lib.sphgb_set_stream(self.h, C.c_void_p(stream.cuda_stream)), "sphgb_set_stream")

    def set_params(self, **kw) -> None:
        for k, v in kw.items():
            if not hasattr(self.params, k):
                continue
            setattr(self.params, k, v)
        check(self.lib.sphgb_set_params(self.h, C.byref(self.params)), "sphgb_set_params")

    def set_deterministic(self, on: bool) -> None:
        """True: every pass sums in list order (bitwise reproducible); False (default): the FP64 VE
        xmass, gradh, IAD + divv/curlv, AV and momentum-energy passes evaluate mutual pairs once and
        scatter with FP64 atomics."""
        check(self.lib.sphgb_set_deterministic(self.h, int(bool(on))), "sphgb_set_deterministic")

    def set_adjoint_tape(self, on: bool) -> None:
        """FP64 VE passes keep the sums the VE adjoint needs (sphgb_set_adjoint_tape)."""
        check(self.lib.sphgb_set_adjoint_tape(self.h, int(bool(on))), "sphgb_set_adjoint_tape")

    def set_mixed_refinement(self, on: bool) -> None:
        """Mixed form: recompute ill-conditioned particles (gradh near 0, divv sign within the FP32
        error) in FP64 from the exact inputs (default True)."""
        check(self.lib.sphgb_set_mixed_refinement(self.h, int(bool(on))), "sphgb_set_mixed_refinement")

    def set_kernel_form(self, smooth: bool) -> None:
        """Kernel function of the FP64 passes and adjoints: the reference's linear table interpolant
        (False, default) or C1 cubic pieces through the closed form (True, sphgb_set_kernel_form)."""
        check(self.lib.sphgb_set_kernel_form(self.h, int(bool(smooth))), "sphgb_set_kernel_form")

    def set_domain_mode(self, mode: int) -> None:
        """0: every sync stands alone; 1: syncs are the steps of one simulation (box shrink limit)."""
        check(self.lib.sphgb_set_domain_mode(self.h, int(mode)), "sphgb_set_domain_mode")

    @property
    def K(self) -> float:
        k = C.c_double()
        check(self.lib.sphgb_get_kernel_K(self.h, C.byref(k)), "sphgb_get_kernel_K")
        return k.value

    def stats(self) -> dict:
        s = _lib.SphgbStats()
        check(self.lib.sphgb_get_stats(self.h, C.byref(s)), "sphgb_get_stats")
        return {f: (list(getattr(s, f)) if f == "level_range" else getattr(s, f)) for f, _ in s._fields_}

    def timings(self) -> list[float]:
        buf = (C.c_float * 8)()
        check(self.lib.sphgb_get_timings(self.h, buf, 8), "sphgb_get_timings")
        return list(buf)

    def launches(self) -> int:
        n = C.c_int64()
        check(self.lib.sphgb_kernel_launches(self.h, C.byref(n)), "sphgb_kernel_launches")
        return n.value

    def fma_peak(self, fp64: bool) -> float:
        """device FMA throughput in FLOP/s of the FP64 or FP32 pipe (probe kernel)."""
        v = C.c_double()
        check(self.lib.sphgb_measure_fma_peak(self.h, int(fp64), C.byref(v)), "sphgb_measure_fma_peak")
        return v.value

    def close(self) -> None:
        if getattr(self, "h", None):
            self.lib.sphgb_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class ParticlesData:
    """SoA particle fields on one device, in the reference's field names and types.

    precision "fp64": every field float64 (HydroType = double); "mixed": the reference default
    SphTypes, x y z u du float64 and every other hydro field float32.
    """

    def __init__(self, n: int, precision: str = "fp64", device: str | torch.device = "cuda:0",
                 av_clean: bool = False):
        self.n = int(n)
        self.precision = precision
        self.prec_id = PRECISIONS[precision]
        self.device = torch.device(device)
        self.hydro_dtype = torch.float64 if precision == "fp64" else torch.float32
        self.av_clean = av_clean
        self.f: dict[str, torch.Tensor] = {}
        for name in REAL_FIELDS:
            self.f[name] = torch.zeros(self.n, dtype=torch.float64, device=self.device)
        for name in HYDRO_FIELDS:
            if name in DV and not av_clean:
                continue
            self.f[name] = torch.zeros(self.n, dtype=self.hydro_dtype, device=self.device)
        self.f["nc"] = torch.zeros(self.n, dtype=torch.int32, device=self.device)
        self.f["keys"] = torch.zeros(self.n, dtype=torch.int64, device=self.device)
        self.minDtCourant = float("inf")

    def __getattr__(self, name):
        f = self.__dict__.get("f")
        if f is not None and name in f:
            return f[name]
        raise AttributeError(name)

    @classmethod
    def from_workload(cls, wl, precision: str = "fp64", device="cuda:0", av_clean: bool = False,
                      pinned: bool = False):
        d = cls(wl.n, precision, device, av_clean)
        d.load(wl.fields)
        return d

    def load(self, host_fields: dict) -> None:
        for name in INPUTS:
            if name in host_fields:
                t = torch.as_tensor(np.asarray(host_fields[name]), dtype=self.f[name].dtype)
                self.f[name].copy_(t, non_blocking=False)

    def c_struct(self) -> _lib.SphgbParticles:
        s = _lib.SphgbParticles()
        s.n = self.n
        s.precision = self.prec_id
        s.keys = self.f["keys"].data_ptr()
        for name in REAL_FIELDS + tuple(HYDRO_FIELDS):
            t = self.f.get(name)
            setattr(s, name, t.data_ptr() if t is not None else None)
        s.nc = self.f["nc"].data_ptr()
        return s

    def numpy(self, names=None) -> dict:
        names = names or [k for k in self.f]
        return {k: self.f[k].detach().cpu().numpy() for k in names}


class Domain:
    """Single-rank stand-in for cstone::Domain: sync() fits the box, sorts by Hilbert key,
    permutes the conserved fields and builds the cornerstone tree (domain.hpp:181-234)."""

    def __init__(self, ctx: Context, box: Box, bucket_size: int = 64):
        self.ctx = ctx
        self.box_ = box
        if bucket_size != ctx.params.bucket:
            ctx.set_params(bucket=bucket_size)

    def sync(self, d: ParticlesData) -> None:
        s = d.c_struct()
        b = self.box_.to_c()
        check(self.ctx.lib.sphgb_domain_sync(self.ctx.h, C.byref(s), C.byref(b)), "Domain::sync")
        self.box_.update_from(b)

    def box(self) -> Box:
        return self.box_

    def start_index(self) -> int:
        return 0

    def tree_stats(self) -> dict:
        return self.ctx.stats()

    def order(self, n: int) -> torch.Tensor:
        """sorted order of the last sync as a host int64 array: order[i] = pre-sync index."""
        p = C.c_void_p()
        check(self.ctx.lib.sphgb_get_order(self.ctx.h, C.byref(p)), "sphgb_get_order")
        return _device_u32(p.value, n)

    def tree(self) -> dict:
        """cornerstone leaves, layout, and octree arrays of the last sync, copied to the host."""
        ptrs = [C.c_void_p() for _ in range(5)]
        st = _lib.SphgbStats()
        check(self.ctx.lib.sphgb_get_tree(self.ctx.h, *[C.byref(p) for p in ptrs], C.byref(st)), "sphgb_get_tree")
        L, NN = st.num_leaves, st.num_nodes
        return dict(leaves=_device_array(ptrs[0].value, L + 1, np.uint64),
                    layout=_device_array(ptrs[1].value, L + 1, np.uint32),
                    prefixes=_device_array(ptrs[2].value, NN, np.uint64),
                    child_offsets=_device_array(ptrs[3].value, NN, np.int32),
                    internal_to_leaf=_device_array(ptrs[4].value, NN, np.int32),
                    num_leaves=L, num_nodes=NN, num_internal=st.num_internal,
                    level_range=np.array(st.level_range[:], dtype=np.int32))


    def octree_properties(self) -> dict:
        """Domain::octreeProperties (domain.hpp:416-428): the OctreeNsView arrays of the last sync
        (incl. the FP64 node centers and half sizes), copied to the host."""
        v = _lib.SphgbOctreeView()
        check(self.ctx.lib.sphgb_get_octree_view(self.ctx.h, C.byref(v)), "sphgb_get_octree_view")
        L, NN = v.num_leaf_nodes, v.num_nodes
        return dict(num_leaf_nodes=L, num_nodes=NN, num_internal=v.num_internal, max_depth=v.max_depth,
                    prefixes=_device_array(v.prefixes, NN, np.uint64),
                    child_offsets=_device_array(v.child_offsets, NN, np.int32),
                    internal_to_leaf=_device_array(v.internal_to_leaf, NN, np.int32),
                    level_range=_device_array(v.level_range, 23, np.int32),
                    leaves=_device_array(v.leaves, L + 1, np.uint64),
                    layout=_device_array(v.layout, L + 1, np.uint32),
                    centers=_device_array(v.centers, 3 * NN, np.float64).reshape(NN, 3),
                    sizes=_device_array(v.sizes, 3 * NN, np.float64).reshape(NN, 3))


def target_groups(ctx: Context, first: int, last: int) -> np.ndarray:
    """sph::computeGroups: boundaries of the 32-particle target groups of [first, last) (host copy)"""
    g = C.c_int64()
    check(ctx.lib.sphgb_target_groups(ctx.h, first, last, None, 0, C.byref(g)), "sphgb_target_groups")
    out = torch.zeros(g.value + 1, dtype=torch.int32, device=f"cuda:{ctx.device}")
    check(ctx.lib.sphgb_target_groups(ctx.h, first, last, out.data_ptr(), g.value + 1, C.byref(g)),
          "sphgb_target_groups")
    return out.cpu().numpy().view(np.uint32).astype(np.int64)


class _DeviceView:
    """borrowed view of library-owned device memory for torch.as_tensor"""

    def __init__(self, ptr: int, n: int, typestr: str):
        self.__cuda_array_interface__ = {"shape": (n,), "typestr": typestr, "data": (ptr, False), "version": 2,
                                         "strides": None}


def _device_array(ptr: int, n: int, dtype) -> np.ndarray:
    dtype = np.dtype(dtype)
    if n == 0:
        return np.empty(0, dtype=dtype)
    signed = {8: "<i8", 4: "<i4"}[dtype.itemsize]
    torch.cuda.synchronize()
    t = torch.as_tensor(_DeviceView(ptr, n, signed), device="cuda")
    return t.cpu().numpy().view(dtype).copy()


def _device_u32(ptr: int, n: int) -> np.ndarray:
    return _device_array(ptr, n, np.uint32).astype(np.int64)


# ---------------------------------------------------------------- reference-named entry points
def find_neighbors(ctx: Context, x: torch.Tensor, y: torch.Tensor, z: torch.Tensor, h: torch.Tensor,
                   first: int, last: int, ngmax: int):
    """cstone::findNeighbors (findneighbors.hpp:149-170): returns (neighbors[(last-first)*ngmax], nc)
    with nc excluding self; lists are sorted ascending."""
    nw = last - first
    nb = torch.zeros(nw * ngmax, dtype=torch.int32, device=x.device)
    nc = torch.zeros(nw, dtype=torch.int32, device=x.device)
    prec = SPHGB_FP64 if h.dtype == torch.float64 else SPHGB_MIXED
    check(ctx.lib.sphgb_find_neighbors(ctx.h, x.data_ptr(), y.data_ptr(), z.data_ptr(), h.data_ptr(), prec,
                                       first, last, ngmax, nb.data_ptr(), nc.data_ptr()), "findNeighbors")
    return nb, nc


def find_neighbors_sfc(ctx: Context, first: int, last: int, d: ParticlesData) -> int:
    """sph::findNeighborsSfc (sph/include/sph/find_neighbors.hpp:47-56) with the coupled h iteration;
    returns the status (0, or 6 when some particles did not converge, which the reference prints)."""
    s = d.c_struct()
    return check(ctx.lib.sphgb_find_neighbors_sph(ctx.h, C.byref(s), first, last), "findNeighborsSfc",
                 allow=(0, _lib.SPHGB_ERR_NOCONV))


def export_neighbors(ctx: Context, n_work: int, ngmax: int) -> torch.Tensor:
    out = torch.zeros(n_work * ngmax, dtype=torch.int32, device=f"cuda:{ctx.device}")
    check(ctx.lib.sphgb_export_neighbors(ctx.h, out.data_ptr()), "export_neighbors")
    return out


def _pass(fn_name: str, ctx: Context, d: ParticlesData, first: int, last: int, *extra):
    s = d.c_struct()
    fn = getattr(ctx.lib, fn_name)
    check(fn(ctx.h, C.byref(s), first, last, *extra), fn_name)


def compute_density(ctx, d, first=0, last=None):
    _pass("sphgb_compute_density", ctx, d, first, d.n if last is None else last)


def compute_eos_hydro_std(ctx, d, first=0, last=None):
    _pass("sphgb_compute_eos_std", ctx, d, first, d.n if last is None else last)


def compute_iad(ctx, d, first=0, last=None):
    _pass("sphgb_compute_iad", ctx, d, first, d.n if last is None else last)


def compute_momentum_energy_std(ctx, d, first=0, last=None):
    dt = C.c_double()
    _pass("sphgb_compute_momentum_energy_std", ctx, d, first, d.n if last is None else last, C.byref(dt))
    d.minDtCourant = dt.value


def compute_xmass(ctx, d, first=0, last=None):
    _pass("sphgb_compute_xmass", ctx, d, first, d.n if last is None else last)


def compute_ve_def_gradh(ctx, d, first=0, last=None):
    _pass("sphgb_compute_ve_def_gradh", ctx, d, first, d.n if last is None else last)


def compute_eos(ctx, d, first=0, last=None):
    _pass("sphgb_compute_eos", ctx, d, first, d.n if last is None else last)


def compute_iad_divv_curlv(ctx, d, first=0, last=None):
    _pass("sphgb_compute_iad_divv_curlv", ctx, d, first, d.n if last is None else last)


def compute_av_switches(ctx, d, first=0, last=None):
    _pass("sphgb_compute_av_switches", ctx, d, first, d.n if last is None else last)


def compute_momentum_energy(ctx, d, av_clean: bool, first=0, last=None, group_dt: torch.Tensor | None = None):
    dt = C.c_double()
    _pass("sphgb_compute_momentum_energy", ctx, d, first, d.n if last is None else last, int(av_clean),
          group_dt.data_ptr() if group_dt is not None else None, C.byref(dt))
    d.minDtCourant = dt.value


def sweep(ctx: Context, d: ParticlesData, box: Box, variant: str = "ve", av_clean: bool = False) -> int:
    """One hydro step's sweep: Domain::sync + findNeighborsSfc + the variant's pair passes."""
    s = d.c_struct()
    b = box.to_c()
    dt = C.c_double()
    st = check(ctx.lib.sphgb_sweep(ctx.h, C.byref(s), C.byref(b), SPHGB_STD if variant == "std" else SPHGB_VE,
                                   int(av_clean), C.byref(dt)), "sweep", allow=(0, _lib.SPHGB_ERR_NOCONV))
    box.update_from(b)
    d.minDtCourant = dt.value
    return st


def sweep_passes(ctx: Context, d: ParticlesData, variant: str = "ve", av_clean: bool = False) -> int:
    """Neighbour lists + pair passes on the tree of the last sync (frozen positions)."""
    s = d.c_struct()
    dt = C.c_double()
    st = check(ctx.lib.sphgb_sweep_passes(ctx.h, C.byref(s), SPHGB_STD if variant == "std" else SPHGB_VE,
                                          int(av_clean), C.byref(dt)), "sweep_passes",
               allow=(0, _lib.SPHGB_ERR_NOCONV))
    d.minDtCourant = dt.value
    return st

# ---------------------------------------------------------------- time integration and reductions
@dataclass
class Timestep:
    """sphexa::ParticlesData time-step state (particles_data.hpp:96-141): current and previous step,
    elapsed time, the pass limits and the limiter constants."""
    minDt: float = 1e-12
    minDt_m1: float = 1e-12
    ttot: float = 0.0
    minDtCourant: float = float("inf")
    minDtRho: float = float("inf")
    maxDtIncrease: float = 1.1
    g: float = 0.0
    etaAcc: float = 0.2
    eps: float = 0.005

    def to_c(self) -> _lib.SphgbTimestep:
        t = _lib.SphgbTimestep()
        for f, _ in t._fields_:
            setattr(t, f, float(getattr(self, f)))
        return t

    def update_from(self, t: _lib.SphgbTimestep) -> None:
        for f, _ in t._fields_:
            setattr(self, f, getattr(t, f))


def compute_positions(ctx: Context, d: ParticlesData, box: Box, x_m1: torch.Tensor, y_m1: torch.Tensor,
                      z_m1: torch.Tensor, du_m1: torch.Tensor | None, ts: Timestep, first: int = 0,
                      last: int | None = None) -> None:
    """sph::computePositions (positions.hpp:180-200) with dt = ts.minDt, dt_m1 = ts.minDt_m1."""
    last = d.n if last is None else last
    s = d.c_struct()
    b = box.to_c()
    t = ts.to_c()
    check(ctx.lib.sphgb_compute_positions(ctx.h, C.byref(s), C.byref(b), x_m1.data_ptr(), y_m1.data_ptr(),
                                          z_m1.data_ptr(), du_m1.data_ptr() if du_m1 is not None else None,
                                          C.byref(t), first, last), "computePositions")


def update_smoothing_length(ctx: Context, d: ParticlesData, first: int = 0, last: int | None = None) -> None:
    """sph::updateSmoothingLength (update_h.hpp:26-45)"""
    last = d.n if last is None else last
    s = d.c_struct()
    check(ctx.lib.sphgb_update_smoothing_length(ctx.h, C.byref(s), first, last), "updateSmoothingLength")


def rho_timestep(ctx: Context, d: ParticlesData, Krho: float = 0.06, first: int = 0, last: int | None = None) -> float:
    """sph::rhoTimestep (ts_global.hpp:72-95)"""
    last = d.n if last is None else last
    s = d.c_struct()
    v = C.c_double()
    check(ctx.lib.sphgb_rho_timestep(ctx.h, C.byref(s), first, last, Krho, C.byref(v)), "rhoTimestep")
    return v.value


def acceleration_timestep(ctx: Context, d: ParticlesData, etaAcc: float = 0.2, eps: float = 0.005, first: int = 0,
                          last: int | None = None) -> float:
    """sph::accelerationTimestep (ts_global.hpp:36-57)"""
    last = d.n if last is None else last
    s = d.c_struct()
    v = C.c_double()
    check(ctx.lib.sphgb_acceleration_timestep(ctx.h, C.byref(s), first, last, etaAcc, eps, C.byref(v)),
          "accelerationTimestep")
    return v.value


def compute_timestep(ctx: Context, d: ParticlesData, ts: Timestep, first: int = 0, last: int | None = None) -> None:
    """sph::computeTimestep at one rank (ts_global.hpp:97-113): updates ts in place."""
    last = d.n if last is None else last
    s = d.c_struct()
    t = ts.to_c()
    check(ctx.lib.sphgb_compute_timestep(ctx.h, C.byref(s), first, last, C.byref(t)), "computeTimestep")
    ts.update_from(t)


def conserved_quantities(ctx: Context, d: ParticlesData, first: int = 0, last: int | None = None) -> dict:
    """sphexa::localConservedQuantities (conserved_quantities.hpp:49-113)"""
    last = d.n if last is None else last
    s = d.c_struct()
    out = (C.c_double * 8)()
    check(ctx.lib.sphgb_conserved_quantities(ctx.h, C.byref(s), first, last, out), "conservedQuantities")
    return {"eKin": out[0], "eInt": out[1], "linmom": list(out[2:5]), "angmom": list(out[5:8])}
