"""The flops-per-pair figures the bench's roofline uses are the counted ones.

oracle/flop_table.json is written by oracle/flop_table.py from the reference j-loops instantiated
on a counting scalar; where the reference sources are present the count is redone and must match
the committed table exactly.
"""

import json
import os
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
TABLE = ROOT / "oracle" / "flop_table.json"


def _bench_module():
    import importlib.util
    spec = importlib.util.spec_from_file_location("bench_for_flops", ROOT / "bench.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_bench_constants_are_the_counted_table():
    t = json.loads(TABLE.read_text())["workloads"]["sedov_jit_20"]
    b = _bench_module()
    want_ve = {"xmass": t["xmass"], "gradh": t["gradh"], "av": t["av"], "me": t["me_ve"]}
    for k, r in want_ve.items():
        assert b.VE_FLOPS_PER_PAIR[k] == pytest.approx(round(r["flop_per_pair_mean"], 1), abs=1e-9), k
    assert b.VE_FLOPS_PER_PAIR["iad_divv"] == pytest.approx(
        round(t["iad_ve"]["flop_per_pair_mean"], 1) + round(t["divv_curlv"]["flop_per_pair_mean"], 1), abs=1e-9)
    for k, name in (("density", "density_std"), ("iad", "iad_std"), ("me", "me_std")):
        assert b.STD_FLOPS_PER_PAIR[k] == pytest.approx(round(t[name]["flop_per_pair_mean"], 1), abs=1e-9), k


def test_flop_table_reproduces_from_the_reference(tmp_path):
    ref = Path(os.environ.get("SPHGB_REFERENCE", ROOT.parent / "reference"))
    if not (ref / "sph" / "include" / "sph" / "hydro_ve" / "momentum_energy_kern.hpp").exists():
        pytest.skip("reference sources not present")
    import ctypes as C
    import sys
    sys.path.insert(0, str(ROOT))
    from oracle import flop_table as FT
    from oracle import oracle as O
    from sphexa_gb300 import workloads as W
    lib = C.CDLL(str(FT.build()))
    got = FT.count_workload(lib, O.port(), W.sedov(20, jitter=0.25, seed=2))
    want = json.loads(TABLE.read_text())["workloads"]["sedov_jit_20"]
    for name, r in want.items():
        assert got[name]["pairs"] == r["pairs"], name
        assert got[name]["flop_per_pair_mean"] == pytest.approx(r["flop_per_pair_mean"], rel=1e-12), name
