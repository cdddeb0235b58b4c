"""The C ABI library loads and exports every symbol include/sphgb.h declares (no GPU needed)."""

import ctypes as C
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def declared_functions() -> list[str]:
    text = (ROOT / "include" / "sphgb.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(sphgb_[A-Za-z0-9_]+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib():
    from sphexa_gb300 import _lib
    from sphexa_gb300.build import build
    build()
    return _lib.load()


def test_every_declared_symbol_is_exported(lib):
    names = declared_functions()
    assert len(names) >= 25
    for n in names:
        assert hasattr(lib, n), n


def test_python_signatures_cover_the_header(lib):
    from sphexa_gb300 import _lib
    assert set(declared_functions()) == set(_lib.SIGNATURES)


def test_status_strings_and_version(lib):
    assert lib.sphgb_version() >= 100
    assert lib.sphgb_status_string(0) == b"ok"
    assert b"converge" in lib.sphgb_status_string(6)
    assert lib.sphgb_status_string(99) == b"unknown status"


def test_default_params_match_reference_constants(lib):
    from sphexa_gb300 import _lib
    p = _lib.SphgbParams()
    assert lib.sphgb_default_params(C.byref(p)) == 0
    # sph/include/sph/particles_data.hpp:90-146
    assert (p.ng0, p.ngmax, p.bucket) == (100, 150, 64)
    assert p.gamma == pytest.approx(5 / 3)
    assert (p.Kcour, p.sincIndex, p.alphamin, p.alphamax, p.decay_constant) == (0.2, 6.0, 0.05, 1.0, 0.2)


def test_null_arguments_are_rejected(lib):
    assert lib.sphgb_create(None, 0) == 1
    assert lib.sphgb_destroy(None) == 1
    assert lib.sphgb_default_params(None) == 1
    assert lib.sphgb_get_stats(None, None) == 1


def test_create_without_device_fails_cleanly(lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a device is present")
    h = C.c_void_p()
    assert lib.sphgb_create(C.byref(h), 0) == 7  # SPHGB_ERR_NOTFOUND
    assert not h.value


def test_struct_layouts_match_header_sizes():
    """The ctypes mirrors have the C layout (x86-64 / aarch64 LP64 ABI)."""
    from sphexa_gb300 import _lib
    assert C.sizeof(_lib.SphgbBox) == 56
    assert C.sizeof(_lib.SphgbParams) == 72
    assert C.sizeof(_lib.SphgbParticles) == 8 + 8 + 8 + 8 * (5 + 30) + 8
    assert C.sizeof(_lib.SphgbStats) == 24 + 92 + 4 + 8 + 8 + 8 * 7
