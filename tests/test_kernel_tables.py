"""The mixed passes' kernel function (cubic pieces, sphexa_gb300/csrc/kernel_tables.hpp) on the
CPU: evaluated in FP32 as the device lookup does, it agrees with the closed form of sinc^n and its
derivative to FP32 rounding, and with the FP64 linear interpolant of the reference's 20000-point
table (which the FP64 passes use) to about 1e-7 of the function's scale."""

import ctypes as C
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


@pytest.fixture(scope="module")
def lib(tmp_path_factory):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    so = tmp_path_factory.mktemp("kt") / "libkt.so"
    cmd = [gxx, "-O2", "-std=c++17", "-ffp-contract=off", "-shared", "-fPIC", "-I",
           str(ROOT / "sphexa_gb300" / "csrc"), str(ROOT / "tests" / "kernel_tables" / "kernel_tables_host.cpp"),
           "-o", str(so)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    L = C.CDLL(str(so))
    L.kt_errors.argtypes = [C.c_double, C.c_int, C.c_int, C.POINTER(C.c_double)]
    return L


@pytest.mark.parametrize("n", [4.0, 6.0, 8.0])
def test_cubic_pieces_match_closed_form_and_linear_table(lib, n):
    out = (C.c_double * 4)()
    assert lib.kt_errors(n, 512, 400_000, out) == 0
    w_exact, w_lin, dw_exact, dw_lin = list(out)
    print(f"n={n}: W vs closed form {w_exact:.2e}, vs linear table {w_lin:.2e}; "
          f"dW vs closed form {dw_exact:.2e}, vs linear table {dw_lin:.2e}")
    assert w_exact <= 3e-7 and dw_exact <= 3e-7     # FP32 rounding of the coefficients and Horner
    assert w_lin <= 3e-7 and dw_lin <= 3e-7         # plus the reference interpolant's own error
