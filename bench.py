"""Benchmark of the single-rank SPH hydro sweep on one GB300 (or N replicas under torchrun).

Workload (the configuration the metric is quoted on): Sedov blast on a 200^3 = 8.0M particle
lattice in [-0.5, 0.5]^3, periodic, positions jittered by U(+-0.25) lattice spacings (seed 2),
h frozen at h0; one step = one full sweep: box, Hilbert keys, key sort and field permutation,
cornerstone tree, neighbour lists (with the h check), and the volume-element pair passes
(xmass, gradh, EOS, IAD + div/curl v, AV switches, momentum-energy).  FP64 form (every hydro
field double) is the headline value; the mixed form (reference default types, FP32 pair
arithmetic) is measured on the same workload and reported beside it with its error against
the FP64 results of the same run.

  python bench.py [--steps 20] [--warmup 3] [--impl reference]

Synthetic inputs are seeded lattices (no dataset downloads); every input array (~1.6 GB) is
larger than the 129 MB L2, so no flush is needed between steps.
"""

from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "SPH sweep particles/s on 1 GB300: mixed-FP32 vs FP64 at stated err; adjoint/fwd"
UNIT = "particles/s"

# Algorithmic FLOPs per neighbour pair of each pass on the jittered Sedov lattice: the reference
# j-loops instantiated on a counting scalar (+ - * / sqrt and each transcendental call 1 flop,
# an FMA 2), workload mean sum(flops) / sum(pairs); oracle/flop_table.json, workload sedov_jit_20.
VE_FLOPS_PER_PAIR = {"xmass": 20.2, "gradh": 34.4, "iad_divv": 37.6 + 59.3, "av": 55.3, "me": 136.2}
STD_FLOPS_PER_PAIR = {"density": 20.2, "iad": 37.6, "me": 117.3}
# DRAM bytes per particle of one launch, from ncu captures at 1 M particles (dram__bytes_read.sum +
# dram__bytes_write.sum, profiles/*_sedov100_jit_1M.md); traffic grows with the particle count.
# The pair-once kernels of the default FP64 mode inside a sweep: most of it is the stream of the
# sweep's pair-geometry cache (80 bytes per owned entry), read instead of recomputed.
NCU_DRAM_BYTES_PER_PARTICLE = {"me": 4808.1, "iad_divv": 4823.9, "av": 4581.1}
STAGES_VE = ["sync", "neighbors", "xmass", "gradh", "eos", "iad_divv", "av", "me"]
STAGES_STD = ["sync", "neighbors", "density", "eos", "iad", "me", "-", "-"]
# FP32 distance test of one search candidate against the target's radius: 3 coordinate differences,
# one multiply and two FMAs (an FMA counts 2)
SEARCH_FLOPS_PER_TEST = 8
# fields compared between the mixed and the FP64 form
CMP_FIELDS = ("xm", "kx", "rho", "ax", "ay", "az", "du", "c11", "c12", "c13", "c22", "c23", "c33", "divv", "curlv",
              "alpha")
# the other configurations measured beside the headline: (timed sweeps, warm-up sweeps)
EXTRA_CONFIGS = {"fourier300": (5, 2), "sphere10M": (5, 2)}


def env_rank():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


class ClockSampler:
    """nvidia-smi clocks/throttle sampling during the timed region (200 ms period)."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines: list[str] = []
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.QUERY}", "--format=csv,noheader,nounits",
                                          "-lms", "200", "-i", str(self.device)], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
        except (OSError, FileNotFoundError):
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)
        sm, smax, reasons, power = [], [], set(), []
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            p = [x.strip() for x in line.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                smax.append(float(p[2]))
                power.append(float(p[3]))
            except ValueError:
                continue
            for k, nm in enumerate(names):
                if p[5 + k].lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm), "power_w_max": max(power) if power else None}


def host_cpu() -> dict:
    """The host cores the CPU baseline runs on: count, model and the OpenMP settings in force."""
    model = None
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.startswith("Model name:"):
                model = line.split(":", 1)[1].strip()
                break
    except (OSError, subprocess.TimeoutExpired):
        pass
    return {"nproc": os.cpu_count(), "cpu_model": model, "OMP_NUM_THREADS": os.environ.get("OMP_NUM_THREADS"),
            "OMP_PROC_BIND": os.environ.get("OMP_PROC_BIND"),
            "build": "oracle/liboracle_o3.so: g++ -std=c++20 -O3 -fopenmp (no -march/-mcpu=native)"}


def set_cpu_threads() -> None:
    """every host core for the OpenMP CPU baseline, threads bound close (set before any OpenMP
    runtime starts)"""
    os.environ.setdefault("OMP_NUM_THREADS", str(os.cpu_count() or 1))
    os.environ.setdefault("OMP_PROC_BIND", "close")


def measured_peaks() -> dict:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        return json.loads(p.read_text())
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "fallback": True}


# name -> (description used verbatim as config.workload by both arms, constructor)
WORKLOADS = {
    "sedov200_jit": ("sedov200_jit: 8000000 particles, periodic [-0.5,0.5]^3, jitter +-0.25 spacing (seed 2), "
                     "Sedov u, v = 0, frozen h",
                     lambda W: W.sedov(200, jitter=0.25, seed=2)),
    "sedov100_jit": ("sedov100_jit: 1000000 particles, periodic [-0.5,0.5]^3, jitter +-0.25 spacing (seed 2), "
                     "Sedov u, v = 0, frozen h",
                     lambda W: W.sedov(100, jitter=0.25, seed=2)),
    "fourier300": ("fourier300: 27000000 particles, periodic unit box, jitter +-0.3 spacing (seed 3), Fourier "
                   "density field in the masses (seed 33), v ~ N(0, 0.1^2) (seed 333), u = 1",
                   lambda W: W.fourier(300)),
    "sphere10M": ("sphere10M: 10000000 particles in the unit sphere, open boundaries, r = sqrt(U) (seed 4), "
                  "u = 0.05, v = 0, h from the local number density",
                  lambda W: W.sphere(10_000_000)),
    # the same Sedov set at 30^3 = 27,000 particles: a case both arms finish in seconds on any host
    "sedov30_jit": ("sedov30_jit: 27000 particles, periodic [-0.5,0.5]^3, jitter +-0.25 spacing (seed 2), "
                    "Sedov u, v = 0, frozen h",
                    lambda W: W.sedov(30, jitter=0.25, seed=2)),
}


def make_workload(name: str):
    from sphexa_gb300 import workloads as W
    if name not in WORKLOADS:
        raise SystemExit(f"unknown workload {name}")
    return WORKLOADS[name][1](W)


def bench_config(args, world: int) -> dict:
    """config object shared by the GPU arm and the reference arm (same workload string)."""
    return {"workload": WORKLOADS[args.workload][0] + f"; one full {args.variant.upper()} sweep per step",
            "variant": args.variant, "precision": "fp64",
            "l2": "inputs larger than L2 (no flush)", "parallelism": f"replicas x{world}"}


def structure_report(ctx, d, stats: dict, ngmax: int) -> dict:
    """Octree depth, neighbour-count histogram, capped count and per-group (32 SFC-consecutive
    targets) pair load of the last sweep."""
    lr = [int(v) for v in stats["level_range"]]
    depth = max(k for k in range(len(lr) - 1) if lr[k + 1] > lr[k]) if any(lr) else 0
    nc = d.nc.cpu().numpy().astype(np.int64)
    pairs = np.minimum(nc - 1, ngmax)
    edges = [0, 25, 50, 75, 100, 125, 150, 151, 10 ** 9]
    hist = np.histogram(nc, bins=edges)[0]
    g = pairs[: (len(pairs) // 32) * 32].reshape(-1, 32).sum(1)
    return {"octree_depth": depth, "num_leaves": stats["num_leaves"], "num_nodes": stats["num_nodes"],
            "nc_hist": {f"[{edges[k]},{edges[k + 1]})": int(hist[k]) for k in range(len(hist))},
            "nc_min": int(nc.min()), "nc_max": int(nc.max()), "capped": stats["capped"],
            "h_iterations": stats["h_iterations"],
            "group_pairs": {"mean": float(g.mean()), "p99": float(np.percentile(g, 99)), "max": int(g.max()),
                            "max_over_mean": float(g.max() / g.mean())}}


def cpu_baseline(wl, workload: str, variant: str = "ve", sweeps: int = 1) -> dict:
    """The oracle (my CPU restatement of the reference's OpenMP path, release flags) on the same
    workload as the GPU arm: `sweeps` full sweeps, all host cores."""
    from oracle import oracle as O
    port = O.port_timed()
    times, r = [], None
    for _ in range(sweeps):
        t0 = time.perf_counter()
        r = port.sweep(wl, variant, False, want_nbr=False, want_tree=False)
        times.append(time.perf_counter() - t0)
    dt = statistics.median(times)
    return {"value": wl.n / dt, "unit": UNIT, "cores": int(r["threads"]), "kind": "port",
            "sample": f"{sweeps} full {variant.upper()} sweep(s) of the {workload} workload ({wl.n} particles, "
                      f"median {dt:.2f} s; stages keys {r['times']['keys']:.2f} tree {r['times']['tree']:.2f} "
                      f"nbr {r['times']['nbr']:.2f} hydro {r['times']['hydro']:.2f} s)",
            "host": host_cpu()}


def adjoint_timing(ctx, dev: str, side: int, steps: int, warmup: int, chain: str = "std",
                   precision: str = "fp64"):
    """Forward chain on frozen lists against its adjoint for the loss sum (rho - rho_target)^2 +
    sum |a|^2, CUDA events on the default stream.  chain "std": density, EOS, IAD, momentum-energy;
    "ve": xmass, gradh, EOS, IAD + divv/curlv, AV switches, momentum-energy.  precision "mixed"
    (std chain): the mixed forward and the FP32-arithmetic adjoint.  Returns the timing record
    and the first backward's gradients (x y z vx vy vz h u, FP64 on the host)."""
    import torch
    from sphexa_gb300 import autograd as AG, sph, workloads as W
    wl = W.fourier(side, seed=5, rho_seed=55, v_seed=555, target_seed=5555)
    d = sph.ParticlesData.from_workload(wl, precision, dev)
    box = sph.Box(wl.box.copy(), wl.bc.copy())
    sw = AG.FrozenStdSweep(ctx, d, box) if chain == "std" else AG.FrozenVeSweep(ctx, d, box)
    sw.freeze()
    order = sph.Domain(ctx, box).order(wl.n)
    rho_t = torch.tensor(wl.fields["rho_target"][order], dtype=torch.float64, device=dev)
    vals = sw.inputs()

    def timed(fn, k):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record()
        for _ in range(k):
            fn()
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / k

    outs = sw.forward(*vals)
    rho, ax, ay, az, du = outs
    seeds = (2.0 * (rho - rho_t), 2.0 * ax, 2.0 * ay, 2.0 * az, None)
    t0 = time.perf_counter()
    grads = sw.backward(*seeds)  # first call also builds the incoming (transposed) lists
    torch.cuda.synchronize()
    first_ms = (time.perf_counter() - t0) * 1e3
    grads = [g.to(torch.float64).cpu().numpy() for g in grads]
    for _ in range(max(1, warmup)):
        sw.forward(*vals)
        sw.backward(*seeds)
    k = max(3, steps // 2)
    fwd = timed(lambda: sw.forward(*vals), k)
    adj = timed(lambda: sw.backward(*seeds), k)
    return {"workload": f"adjoint config: jittered Fourier lattice {side}^3 = {wl.n} particles, frozen lists",
            "form": f"{precision} {chain} chain", "forward_ms": fwd, "adjoint_ms": adj, "ratio": adj / fwd,
            "first_adjoint_ms_incl_transpose": first_ms, "steps": k}, grads


def run_reference(args) -> None:
    """The reference arm: the reference's CPU OpenMP path for this sweep (restated in oracle/, built
    with release flags) on the GPU arm's workload, one full sweep per step, all host cores."""
    rank, world, _ = env_rank()
    if rank != 0:
        return
    set_cpu_threads()
    from oracle import oracle as O
    wl = make_workload(args.workload)
    port = O.port_timed()
    for _ in range(args.warmup):  # untimed, the same work as a timed step
        port.sweep(wl, args.variant, False, want_nbr=False, want_tree=False)
    times, r = [], None
    t_all = time.perf_counter()
    for _ in range(args.steps):
        t0 = time.perf_counter()
        r = port.sweep(wl, args.variant, False, want_nbr=False, want_tree=False)
        times.append(time.perf_counter() - t0)
    wall = time.perf_counter() - t_all
    v = wl.n * args.steps / wall
    line = {"metric": METRIC, "value": v, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": wall * 1e3 / max(1, args.steps), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic: seeded generator of the named configuration (no dataset)", "impl": "reference",
            "config": bench_config(args, world),
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": int(r["threads"]), "kind": "port",
                             "sample": f"every step one full {args.variant.upper()} sweep of the workload "
                                       f"({wl.n} particles; step median {statistics.median(times):.2f} s, "
                                       f"min {min(times):.2f} s)",
                             "host": host_cpu()},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def pair_roofline(stages: np.ndarray, names: list, pairs: int, flops: dict, peak: float, bound: str) -> dict:
    """the pair pass with the largest share of the sweep against a pipe peak: counted reference flops
    of its j-loop per neighbour pair x pairs, over its CUDA-event time"""
    cand = [k for k in range(len(names)) if names[k] in flops]
    k = max(cand, key=lambda q: stages[q])
    achieved = pairs * flops[names[k]] / (stages[k] * 1e-3)
    return {"bound": bound, "kernel": names[k], "achieved": achieved / 1e12, "peak": peak / 1e12, "unit": "TFLOP/s",
            "frac": achieved / peak, "ms": float(stages[k]),
            "algorithmic": f"{pairs} pairs x {flops[names[k]]} flop/pair per launch",
            "peak_source": f"{bound.upper()} FMA probe measured in this run (MEASURED_PEAKS.json has no "
                           f"{bound.upper()} figure)"}


def search_roofline(stats: dict, ms: float, n: int, fp32_peak: float, hbm_gbs: float) -> dict:
    """the neighbour search: FP32 distance tests against the FP32 pipe, list bytes against HBM"""
    tests = int(stats["candidates"])
    list_bytes = 4 * int(stats["nc_sum"]) + 4 * n  # transposed list entries + counts
    tf = tests * SEARCH_FLOPS_PER_TEST / (ms * 1e-3)
    gbs = list_bytes / (ms * 1e-3) / 1e9
    return {"bound": "issue (instructions per candidate test; profiles/nbrGroupKernel_*: sm__inst_issued, "
                     "ALU pipe busiest)",
            "ms": ms, "candidate_tests": tests, "tests_per_particle": tests / n,
            "flop_per_test": SEARCH_FLOPS_PER_TEST, "fp32_tflops": tf / 1e12, "fp32_frac": tf / fp32_peak,
            "list_bytes": list_bytes, "list_gbs": gbs, "hbm_frac": gbs / hbm_gbs if hbm_gbs else None}


def mixed_errors(ref64: dict, r32: dict) -> dict:
    """errors of the mixed form against the FP64 form of the same run, per output field (device
    tensors; rho and xm max relative per particle, the rest max abs over the field's max or normwise)"""
    import torch

    def mx(t):
        return float(t.abs().max().item())

    a64 = torch.stack([ref64["ax"], ref64["ay"], ref64["az"]], 1)
    a32 = torch.stack([r32["ax"], r32["ay"], r32["az"]], 1)
    err = {"rho_max_rel": mx((r32["rho"] - ref64["rho"]) / ref64["rho"]),
           "xm_max_rel": mx((r32["xm"] - ref64["xm"]) / ref64["xm"]),
           "a_normwise": float((torch.linalg.norm(a32 - a64) / torch.linalg.norm(a64).clamp_min(1e-300)).item()),
           "du_normwise": float((torch.linalg.norm(r32["du"] - ref64["du"]) /
                                 torch.linalg.norm(ref64["du"]).clamp_min(1e-300)).item())}
    cij = [f"c{a}{b}" for a, b in ("11", "12", "13", "22", "23", "33")]
    cmag = max(mx(ref64[k]) for k in cij)
    err["cij_max_over_tensor_max"] = max(mx(r32[k] - ref64[k]) for k in cij) / cmag
    for k in ("divv", "curlv", "alpha", "du"):
        scale = mx(ref64[k])
        err[f"{k}_max_over_field_max"] = mx(r32[k] - ref64[k]) / scale if scale > 0 else mx(r32[k] - ref64[k])
    return err


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="sedov200_jit")
    ap.add_argument("--variant", default="ve", choices=["ve", "std"])
    ap.add_argument("--no-configs", action="store_true", help="skip the Fourier 27M and sphere 10M blocks")
    ap.add_argument("--no-mixed", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-adjoint", action="store_true")
    ap.add_argument("--no-integration", action="store_true")
    ap.add_argument("--adjoint-side", type=int, default=100)
    args = ap.parse_args()
    set_cpu_threads()

    if args.impl == "reference":
        run_reference(args)
        return

    import torch
    import torch.distributed as dist
    from sphexa_gb300 import sph

    rank, world, local = env_rank()
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl")
    dev = f"cuda:{local}"

    wl = make_workload(args.workload)
    n = wl.n
    ctx = sph.Context(local)
    ctx.set_params(ng0=wl.params["ng0"], ngmax=wl.params["ngmax"], minDt=wl.params["minDt"])
    peaks = measured_peaks()
    fp64_peak = ctx.fma_peak(True)
    fp32_peak = ctx.fma_peak(False)

    from sphexa_gb300 import replicas as R

    def barrier():
        R.barrier(world)

    def timed_sweeps(d, box, steps, warmup):
        for _ in range(warmup):
            sph.sweep(ctx, d, box, args.variant, False)
        torch.cuda.synchronize()
        barrier()
        torch.cuda.synchronize()
        l0 = ctx.launches()
        stage_sum = np.zeros(8)
        clocks = ClockSampler(local)
        clocks.start()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(steps):
            sph.sweep(ctx, d, box, args.variant, False)
            stage_sum += np.array(ctx.timings())
        e1.record()
        torch.cuda.synchronize()
        barrier()
        ck = clocks.stop()
        ms = R.max_over_ranks(e0.elapsed_time(e1), world, dev)
        return ms, stage_sum / steps, ctx.launches() - l0, ck

    names = STAGES_VE if args.variant == "ve" else STAGES_STD
    flops = VE_FLOPS_PER_PAIR if args.variant == "ve" else STD_FLOPS_PER_PAIR

    def run_form(w, precision, steps, warmup):
        """timed sweeps of one form on workload w; returns the record, the particle set and stats"""
        d = sph.ParticlesData.from_workload(w, precision, dev)
        b = sph.Box(w.box.copy(), w.bc.copy())
        ms, st, nl, ck = timed_sweeps(d, b, steps, warmup)
        stats = ctx.stats()
        rec = {"value": R.job_throughput(w.n, steps, world, ms), "unit": UNIT, "ms_per_step": ms / steps,
               "stages_ms": {names[k]: round(float(st[k]), 3) for k in range(len(names)) if names[k] != "-"}}
        return rec, d, stats, st, nl, ck

    def mixed_vs_fp64(w, rec64, d64, steps, warmup):
        """the mixed form on workload w against the FP64 results of this run (d64 is released)"""
        ref64 = {k: d64.f[k].double().clone() for k in CMP_FIELDS}
        d64 = None
        torch.cuda.empty_cache()
        rec32, d32, stats32, st32, _, _ = run_form(w, "mixed", steps, warmup)
        r32 = {k: d32.f[k].double() for k in CMP_FIELDS}
        rec32["speedup_vs_fp64"] = rec32["value"] / rec64["value"]
        rec32["errors_vs_fp64"] = mixed_errors(ref64, r32)
        rec32["roofline"] = pair_roofline(st32, names, int(stats32["nc_sum"]), flops, fp32_peak, "fp32")
        # every pair pass against the FP32 probe peak: counted flop/pair x pairs / stage time
        rec32["pair_pass_fp32_frac"] = {
            names[k]: round(int(stats32["nc_sum"]) * flops[names[k]] / (float(st32[k]) * 1e-3) / fp32_peak, 4)
            for k in range(len(names)) if names[k] in flops and st32[k] > 0}
        rec32["neighbors_roofline"] = search_roofline(stats32, float(st32[1]), w.n, fp32_peak,
                                                      peaks.get("hbm_gbs"))
        rec32["dominant_stage"] = names[int(np.argmax(st32))]
        rec32["dominant_fp32_frac"] = rec32["roofline"]["frac"]
        del ref64, r32, d32
        torch.cuda.empty_cache()
        return rec32

    # ---------------- FP64 form (headline)
    rec64, d64, stats, st64, launches, clocks = run_form(wl, "fp64", args.steps, args.warmup)
    ms64 = rec64["ms_per_step"] * args.steps
    pairs = stats["nc_sum"]
    value = rec64["value"]

    # dominant kernel: the pair pass with the largest share of the FP64 sweep (the FP64 pipe bounds it)
    roofline = pair_roofline(st64, names, pairs, flops, fp64_peak, "fp64")
    traffic = NCU_DRAM_BYTES_PER_PARTICLE.get(roofline["kernel"])
    roofline["traffic"] = traffic * n if traffic else None
    roofline["traffic_source"] = ("ncu dram bytes of the same kernel at 1M particles, scaled by particles; most of it "
                                  "is the sweep's pair-geometry cache (80 B per owned pair), read instead of recomputed")
    roofline["hbm_peak_gbs"] = peaks.get("hbm_gbs")
    if traffic and peaks.get("hbm_gbs"):  # the same kernel against HBM: DRAM bytes over its time
        gbs = float(traffic * n / (roofline["ms"] * 1e-3) / 1e9)
        roofline["hbm_achieved_gbs"] = gbs
        roofline["hbm_frac"] = gbs / peaks["hbm_gbs"]

    out = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": ms64 / args.steps, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f64",
           "data": "synthetic: seeded generator of the named configuration (no dataset)",
           "config": bench_config(args, world), "n_particles": n,
           "roofline": roofline, "gpu_launches": launches // max(1, args.steps) * args.steps,
           "clocks": clocks,
           "stages_ms": rec64["stages_ms"],
           "neighbors": {"pairs": pairs, "mean": pairs / n, "max_nc": stats["nc_max"], "capped": stats["capped"],
                         "candidates": stats["candidates"], "fp64_rechecks": stats["fp64_rechecks"],
                         "roofline": search_roofline(stats, float(st64[1]), n, fp32_peak, peaks.get("hbm_gbs"))},
           "fp32_peak_tflops": fp32_peak / 1e12, "fp64_peak_tflops": fp64_peak / 1e12}
    if args.workload in ("fourier300", "sphere10M"):
        out["structure"] = structure_report(ctx, d64, stats, int(wl.params["ngmax"]))

    # ---------------- end to end through the C ABI with host buffers (pinned), FP64 form, right after
    # the device-timed sweeps so that both run under the same conditions.  Every step copies its
    # inputs host -> device, sweeps, and copies ax ay az du device -> host, on one stream.  (Copies of
    # neighbouring steps on a second stream do not overlap the sweep: its own host read-backs and
    # field moves use the same copy engines, measured equal to the serial form.)
    if not args.no_e2e:
        d = sph.ParticlesData.from_workload(wl, "fp64", dev)
        host_in = {k: torch.from_numpy(np.ascontiguousarray(wl.fields[k], dtype=np.float64)).pin_memory()
                   for k in sph.INPUTS}
        outs = ("ax", "ay", "az", "du")
        host_out = {k: torch.empty(n, dtype=torch.float64).pin_memory() for k in outs}
        h2d = sum(t.numel() * t.element_size() for t in host_in.values())
        d2h = sum(t.numel() * t.element_size() for t in host_out.values())
        boxe = sph.Box(wl.box.copy(), wl.bc.copy())

        evs = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
        phases = []  # per step: H2D, sweep, D2H milliseconds (CUDA events on the launching stream)

        def e2e_step():
            evs[0].record()
            for k, t in host_in.items():
                d.f[k].copy_(t, non_blocking=True)
            evs[1].record()
            sph.sweep(ctx, d, boxe, args.variant, False)
            evs[2].record()
            for k in outs:
                host_out[k].copy_(d.f[k], non_blocking=True)
            evs[3].record()
            torch.cuda.synchronize()
            phases.append([evs[q].elapsed_time(evs[q + 1]) for q in range(3)])

        for _ in range(max(1, args.warmup)):
            e2e_step()
        phases.clear()
        barrier()
        t0 = time.perf_counter()
        k_e2e = max(3, args.steps // 2)
        for _ in range(k_e2e):
            e2e_step()
        barrier()
        wall_ms = R.max_over_ranks((time.perf_counter() - t0) * 1e3, world, dev)
        med = np.median(np.array(phases), axis=0)
        finite = all(bool(torch.isfinite(host_out[f]).all()) for f in outs)  # the host reads the result
        out["e2e"] = {"value": R.job_throughput(n, k_e2e, world, wall_ms), "unit": UNIT, "h2d_bytes_per_step": h2d,
                      "d2h_bytes_per_step": d2h, "steps": k_e2e, "ms_per_step": wall_ms / k_e2e,
                      "phases_ms_median": {"h2d": float(med[0]), "sweep": float(med[1]), "d2h": float(med[2])},
                      "h2d_gbs": h2d / (float(med[0]) * 1e6), "d2h_gbs": d2h / (float(med[2]) * 1e6),
                      "outputs_finite": finite,
                      "path": "pinned host inputs -> sphgb_sweep (C ABI) -> pinned host ax ay az du"}
        del d

    # ---------------- mixed form on the same workload, errors against this run's FP64 results
    if not args.no_mixed:
        out["mixed"] = mixed_vs_fp64(wl, rec64, d64, args.steps, args.warmup)
    d64 = None
    torch.cuda.empty_cache()

    # ---------------- the other configurations: Fourier 27M (the mixed form's own, v != 0) and the
    # clustered 10M sphere, FP64 and mixed, with structure and per-field errors
    if not args.no_configs and args.workload == "sedov200_jit":
        out["configs"] = {}
        for cname, (csteps, cwarm) in EXTRA_CONFIGS.items():
            cw = make_workload(cname)
            c64, cd, cstats, cst, _, _ = run_form(cw, "fp64", csteps, cwarm)
            c64["roofline"] = pair_roofline(cst, names, int(cstats["nc_sum"]), flops, fp64_peak, "fp64")
            blk = {"workload": WORKLOADS[cname][0], "n_particles": cw.n, "steps": csteps, "warmup": cwarm,
                   "fp64": c64, "structure": structure_report(ctx, cd, cstats, int(cw.params["ngmax"]))}
            blk["mixed"] = mixed_vs_fp64(cw, c64, cd, csteps, cwarm)
            cd = None
            out["configs"][cname] = blk
            del cw
            torch.cuda.empty_cache()

    # ---------------- integration step on the same particles (FP64): time step, positions, h, sums
    if not args.no_integration:
        d = sph.ParticlesData.from_workload(wl, "fp64", dev)
        boxi = sph.Box(wl.box.copy(), wl.bc.copy())
        sph.sweep(ctx, d, boxi, args.variant, False)
        m1 = {k: torch.zeros(n, dtype=torch.float64, device=dev) for k in ("x", "y", "z", "du")}
        ts = sph.Timestep(minDt=1e-7, minDt_m1=1e-7, minDtCourant=d.minDtCourant)

        def integrate():
            sph.compute_timestep(ctx, d, ts)
            sph.compute_positions(ctx, d, boxi, m1["x"], m1["y"], m1["z"], m1["du"], ts)
            sph.update_smoothing_length(ctx, d)
            return sph.conserved_quantities(ctx, d)

        for _ in range(max(1, args.warmup)):
            integrate()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        k_int = max(3, args.steps)
        t0 = time.perf_counter()
        pos_ms = 0.0
        for _ in range(k_int):
            sph.compute_timestep(ctx, d, ts)
            e0.record()
            sph.compute_positions(ctx, d, boxi, m1["x"], m1["y"], m1["z"], m1["du"], ts)
            e1.record()
            sph.update_smoothing_length(ctx, d)
            sph.conserved_quantities(ctx, d)
            torch.cuda.synchronize()
            pos_ms += e0.elapsed_time(e1)
        wall = (time.perf_counter() - t0) * 1e3 / k_int
        pos_ms /= k_int
        # algorithmic bytes of the position + energy update per particle: reads x y z v a x_m1 u du
        # du_m1 (15 doubles), writes x y z v x_m1 u du_m1 (11 doubles)
        bytes_pp = 8 * (15 + 11)
        out["integration"] = {"step_ms": wall, "positions_ms": pos_ms,
                              "positions_gbs": n * bytes_pp / (pos_ms * 1e-3) / 1e9,
                              "positions_hbm_frac": n * bytes_pp / (pos_ms * 1e-3) / 1e9 / peaks.get("hbm_gbs", 6800.0),
                              "bytes_per_particle": bytes_pp,
                              "what": "computeTimestep + computePositions + updateSmoothingLength + conserved sums"}
        del d, m1
        torch.cuda.empty_cache()

    # ---------------- adjoint / forward on the adjoint configuration (1M particles, FP64 std chain)
    if not args.no_adjoint:
        out["adjoint"], g64 = adjoint_timing(ctx, dev, args.adjoint_side, args.steps, args.warmup)
        out["adjoint"]["ve"], _ = adjoint_timing(ctx, dev, args.adjoint_side, args.steps, args.warmup, chain="ve")
        mixed, g32 = adjoint_timing(ctx, dev, args.adjoint_side, args.steps, args.warmup, precision="mixed")
        mixed["grad_error_vs_fp64"] = {f: float(np.linalg.norm(b - a) / np.linalg.norm(a))
                                       for f, a, b in zip(("x", "y", "z", "vx", "vy", "vz", "h", "u"), g64, g32)}
        out["adjoint"]["mixed"] = mixed

    if rank == 0 and not args.no_cpu:
        out["cpu_baseline"] = cpu_baseline(wl, args.workload, variant=args.variant)
    ctx.close()
    if rank == 0:
        print(json.dumps(out), flush=True)
    if world > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
