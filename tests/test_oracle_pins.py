"""The oracle (my CPU restatement) pinned against the reference.

1. Known-answer tests: the numbers the reference's own GTest suites assert
   (sph/test/std.cpp:98-127, sph/test/ve.cpp:112-233, sph/test/table_creation.cpp:26-39),
   with the reference's tolerances.
2. Golden fixtures: outputs of the reference's CPU code compiled from its headers
   (tests/golden/make_golden.py), compared bit-exactly for integer data and to 1e-13 for fields.
3. Live: where the reference-compiled oracle exists on this machine, random cases side by side.
"""

import ctypes as C
import math

import numpy as np
import pytest

from conftest import load_golden, workload_from_golden

pytestmark = []


def _jloop(port, fields, neighbors, loop, K, box, **kw):
    import importlib.util
    from pathlib import Path
    spec = importlib.util.spec_from_file_location("mg", Path(__file__).parent / "golden" / "make_golden.py")
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    return mg.run_jloop(port.lib, fields, neighbors, loop, K, box, **kw)


def _inputs(g):
    return {k[3:]: g[k] for k in g if k.startswith("in_")}


def test_kernel_normalisation(port):
    # sph/test/table_creation.cpp: K of sinc^6 by Simpson; value printed by the reference build
    assert port.kernel_K(6.0) == pytest.approx(0.79044958943230337, rel=1e-15)


def test_std_known_answers(port):
    g = load_golden("kat_std.npz")
    f, K = _inputs(g), float(g["K"])
    box = (0, 6, 0, 6, 0, 6)
    iad = _jloop(port, f, [1, 2, 3, 4], "iad_std", K, box)
    # sph/test/std.cpp:98-109
    expect = [0.68826690779384281, -0.12963692768970825, -0.20435302538490346, 0.39616100688793993,
              -0.16797800827029263, 1.9055087813473524]
    np.testing.assert_allclose(iad[:6], expect, rtol=0, atol=1e-8)
    np.testing.assert_array_equal(iad[:6], g["out_iad_std"])
    me = _jloop(port, f, [1, 2, 3, 4], "me_std", K, box)
    # sph/test/std.cpp:111-127: grad_P x y z, du, maxvsignal
    assert me[0] == pytest.approx(14.407211846688075, abs=1.3e-7)
    assert me[1] == pytest.approx(-1.2396802157028355, abs=1.4e-7)
    assert me[2] == pytest.approx(15.596554152643426, abs=2.15e-7)
    assert me[3] == pytest.approx(-0.40541191600274296, abs=1e-8)
    assert me[4] == pytest.approx(1.4112466828564341, abs=1e-10)
    np.testing.assert_array_equal(me[:5], g["out_me_std"])


def test_ve_known_answers(port):
    g = load_golden("kat_ve.npz")
    f, K = _inputs(g), float(g["K"])
    nb = np.arange(1, 99)
    box = (-1e9, 1e9) * 3
    av = _jloop(port, f, nb, "av", K, box, dt=0.3)
    assert av[0] == pytest.approx(0.93941905320351171, abs=2e-9)  # ve.cpp:115-123
    dv = _jloop(port, f, nb, "divv", K, box)
    expect = [3.3760353440920682e-2, 3.7836647734377962e-2, 0.0013578323369918166, 0.02465266861727711,
              -0.0046604174274769167, 0.022556438947324862, 0.0097704904179710741, 0.0098460821566040066]
    np.testing.assert_allclose(dv[:8], expect, rtol=0, atol=2e-9)  # ve.cpp:125-143
    iad = _jloop(port, f, nb, "iad_ve", K, box)
    expect = [1.9296619855715329e-18, -1.7838691836843698e-20, -1.2892885646884301e-20, 1.9482845913025683e-18,
              1.635410357476855e-20, 1.9246939006338132e-18]
    np.testing.assert_allclose(iad[:6], expect, rtol=0, atol=1e-10)  # ve.cpp:145-160
    mec = _jloop(port, f, nb, "me_ve", K, box, avclean=True)  # ve.cpp:176-195
    assert mec[0] == pytest.approx(-505548.68073726865, abs=0.023)
    assert mec[1] == pytest.approx(303384.91384746187, abs=0.053)
    assert mec[2] == pytest.approx(-1767463.9739728321, abs=0.043)
    assert mec[3] == pytest.approx(8.5525242525359648e12, abs=7.1e5)
    assert mec[4] == pytest.approx(26490876.319252387, abs=1e-6)
    me = _jloop(port, f, nb, "me_ve", K, box, avclean=False)  # ve.cpp:196-214
    assert me[0] == pytest.approx(-521261.07791667967, abs=0.022)
    assert me[1] == pytest.approx(-74471.016515749841, abs=0.064)
    assert me[2] == pytest.approx(-1730426.827721074, abs=0.042)
    assert me[3] == pytest.approx(7.1838438980436924e12, abs=3.1e5)
    assert me[4] == pytest.approx(26490876.319252387, abs=1e-6)
    gh = _jloop(port, f, nb, "gradh", K, box)  # ve.cpp:217-226
    assert gh[0] * f["m"][0] / f["xm"][0] == pytest.approx(3.4662283566584293e1, abs=8e-7)
    assert gh[1] == pytest.approx(0.98699067585409861, abs=5e-7)
    assert gh[0] == pytest.approx(1.0042661134076782, abs=3e-7)
    xm = _jloop(port, f, nb, "xmass", K, box)  # ve.cpp:228-237
    assert f["m"][0] / xm[0] == pytest.approx(34.515038498081417, abs=7.33e-7)
    # and bit-identical to the reference's own j-loops on the same inputs
    for name, got in [("av", av[:1]), ("divv", dv[:8]), ("iad_ve", iad[:6]), ("me_ve_clean", mec[:5]),
                      ("me_ve", me[:5]), ("gradh", gh[:2]), ("xmass", xm[:1])]:
        np.testing.assert_allclose(got, g["out_" + name], rtol=2e-15, atol=0, err_msg=name)


GOLDEN_SWEEPS = ["sweep_sedov10_std.npz", "sweep_random2000_ve_clean.npz", "sweep_sphere2000_ve.npz",
                 "sweep_fourier10_ve.npz"]


def compare_sweep(res: dict, g: dict, ngmax: int, field_rtol: float = 1e-13, fields=True):
    from oracle import oracle as O
    np.testing.assert_array_equal(res["keys"], g["keys"])
    np.testing.assert_array_equal(res["order"], g["order"])
    np.testing.assert_array_equal(res["leaves"], g["leaves"])
    np.testing.assert_array_equal(res["counts"], g["counts"])
    np.testing.assert_array_equal(res["prefixes"], g["prefixes"])
    np.testing.assert_array_equal(res["child_offsets"], g["child_offsets"])
    np.testing.assert_array_equal(res["internal_to_leaf"], g["internal_to_leaf"])
    np.testing.assert_array_equal(res["level_range"], g["level_range"])
    np.testing.assert_array_equal(res["nc"], g["nc"])
    sets = O.sorted_sets(res["nbr"], res["nc"], ngmax)
    cnt = np.minimum(res["nc"].astype(np.int64) - 1, ngmax)
    flat = np.concatenate([sets[i, :cnt[i]] for i in range(len(cnt))]).astype(np.uint32)
    np.testing.assert_array_equal(flat, g["nbr_flat"])
    if fields:
        for k in [k for k in g if k.startswith("out_")]:
            name = k[4:]
            scale = np.max(np.abs(g[k])) + 1e-300
            err = np.max(np.abs(res[name] - g[k])) / scale
            assert err <= field_rtol, f"{name}: {err}"


@pytest.mark.parametrize("name", GOLDEN_SWEEPS)
def test_port_matches_reference_golden(port, name):
    g = load_golden(name)
    wl = workload_from_golden(g)
    res = port.sweep(wl, str(g["variant"]), bool(g["avclean"]))
    compare_sweep(res, g, wl.params["ngmax"])
    assert res["minDtCourant"] == pytest.approx(float(g["minDtCourant"]), rel=1e-14)


@pytest.mark.parametrize("case", ["periodic", "open", "gauss"])
def test_port_matches_reference_live(port, ref_oracle, case):
    from sphexa_gb300 import workloads as W
    wl = {"periodic": lambda: W.random_cube(4000, seed=101),
          "open": lambda: W.random_cube(4000, seed=102, periodic=False),
          "gauss": lambda: W.random_cube(4000, seed=103, gaussian=True)}[case]()
    for variant, avc in (("std", False), ("ve", True)):
        a = port.sweep(wl, variant, avc)
        b = ref_oracle.sweep(wl, variant, avc)
        g = {k: b[k] for k in ("keys", "order", "leaves", "counts", "prefixes", "child_offsets",
                               "internal_to_leaf", "level_range", "nc")}
        from oracle import oracle as O
        ng = wl.params["ngmax"]
        sets = O.sorted_sets(b["nbr"], b["nc"], ng)
        cnt = np.minimum(b["nc"].astype(np.int64) - 1, ng)
        g["nbr_flat"] = np.concatenate([sets[i, :cnt[i]] for i in range(wl.n)]).astype(np.uint32)
        for k in O.FIELDS:
            if np.any(b[k] != 0):
                g["out_" + k] = b[k]
        compare_sweep(a, g, ng, field_rtol=1e-14)


def test_hilbert_curve_properties(port):
    """Curve continuity on a 2-level grid, as domain/test/unit/sfc/hilbert.cpp:114-188 checks:
    consecutive keys of the sorted 4^3 lattice are face neighbours."""
    from sphexa_gb300 import workloads as W
    wl = W.random_cube(64)
    side = 4
    c = (np.arange(side) + 0.5) / side
    z, y, x = np.meshgrid(c, c, c, indexing="ij")
    wl.fields.update(x=x.ravel(), y=y.ravel(), z=z.ravel())
    res = port.sweep(wl, "std", stages=1, want_tree=False, want_nbr=False)
    xs = np.stack([res["x"], res["y"], res["z"]], 1)
    steps = np.abs(np.diff(xs, axis=0)).sum(1)
    np.testing.assert_allclose(steps, 1.0 / side, rtol=1e-12)


def test_port_node_centers_equal_reference(port, ref_oracle):
    """nodeFpCenters (focus/source_center.hpp:129-141) with centerAndSize (sfc/box.hpp:317-334):
    the port's geometric node centers and half sizes equal the reference's bit for bit"""
    from oracle import oracle as O
    from sphexa_gb300 import workloads as W
    wls = [W.sedov(20, jitter=0.25, seed=2), W.sphere(5000, seed=4), W.random_cube(3000, seed=66, periodic=False)]
    for wl in wls:
        a = port.sweep(wl, "ve", stages=O.OS_KEYS | O.OS_TREE, want_nbr=False)
        b = ref_oracle.sweep(wl, "ve", stages=O.OS_KEYS | O.OS_TREE, want_nbr=False)
        np.testing.assert_array_equal(a["centers"], b["centers"])
        np.testing.assert_array_equal(a["sizes"], b["sizes"])
