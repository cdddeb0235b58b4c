"""The one-sweep radix sort behind every sync (sphgb_sort_by_key) against numpy's stable argsort.

Integer bar: keys and values bit-exact, equal keys in input order.  The cases run back to back on
one context, so each sort also meets the look-back words and tickets the previous one left
(epochs), and the look-back buffer grows between them: sizes around the 4096-key tile, random
63-bit keys, heavy duplicates (16 distinct keys: stability), all keys equal (every pass skipped
but one copy), keys already sorted and reversed, keys whose upper bytes are zero (their passes are
skipped), an end bit below 64 (bits above it do not take part), and keys without values."""

import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _sort(lib, ctx, keys, vals, end_bit):
    import torch
    from sphexa_gb300 import _lib
    kin = torch.from_numpy(keys.view(np.int64).copy()).cuda()
    kout = torch.empty_like(kin)
    if vals is not None:
        vin = torch.from_numpy(vals.view(np.int32).copy()).cuda()
        vout = torch.empty_like(vin)
        vp_in, vp_out = vin.data_ptr(), vout.data_ptr()
    else:
        vin = vout = None
        vp_in = vp_out = None
    rc = lib.sphgb_sort_by_key(ctx.h, kin.data_ptr(), kout.data_ptr(), vp_in, vp_out, len(keys), end_bit)
    assert rc == 0, lib.sphgb_status_string(rc)
    # the input stays as it was
    assert np.array_equal(kin.cpu().numpy().view(np.uint64), keys)
    ko = kout.cpu().numpy().view(np.uint64)
    vo = vout.cpu().numpy().view(np.uint32) if vout is not None else None
    return ko, vo


def _expect(keys, vals, end_bit):
    mask = np.uint64((1 << end_bit) - 1) if end_bit < 64 else np.uint64(0xFFFFFFFFFFFFFFFF)
    order = np.argsort(keys & mask, kind="stable")
    return keys[order], (vals[order] if vals is not None else None)


def _cases():
    rng = np.random.default_rng(71)
    r63 = lambda n: rng.integers(0, 1 << 63, size=n, dtype=np.uint64)
    out = []
    for n in (2, 3, 4095, 4096, 4097, 8191, 100_003):
        out.append((f"random63 n={n}", r63(n), 63))
    out.append(("16 distinct keys", rng.integers(0, 16, size=300_000).astype(np.uint64) << np.uint64(40), 63))
    out.append(("all equal", np.full(50_000, 0x123456789, dtype=np.uint64), 63))
    s = np.sort(r63(200_000))
    out.append(("sorted", s, 63))
    out.append(("reversed", s[::-1].copy(), 63))
    out.append(("20-bit keys", rng.integers(0, 1 << 20, size=250_000).astype(np.uint64), 63))
    out.append(("end bit 40", r63(150_000), 40))
    out.append(("64-bit keys", rng.integers(0, np.iinfo(np.uint64).max, size=70_000, dtype=np.uint64,
                                            endpoint=True), 64))
    out.append(("random63 n=3M", r63(3_000_000), 63))
    out.append(("random63 n=5000 after 3M", r63(5000), 63))
    return out


def test_sort_by_key_matches_stable_argsort():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from sphexa_gb300 import _lib, sph
    lib = _lib.load()
    ctx = sph.Context(0)
    rng = np.random.default_rng(72)
    for name, keys, end_bit in _cases():
        for with_vals in (True, False):
            vals = rng.integers(0, 1 << 32, size=len(keys), dtype=np.uint64).astype(np.uint32) if with_vals else None
            ko, vo = _sort(lib, ctx, keys, vals, end_bit)
            ek, ev = _expect(keys, vals, end_bit)
            assert np.array_equal(ko, ek), f"{name}: keys differ"
            if with_vals:
                assert np.array_equal(vo, ev), f"{name}: values differ (stability)"
    ctx.close()


def test_sort_by_key_argument_checks():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from sphexa_gb300 import _lib, sph
    lib = _lib.load()
    ctx = sph.Context(0)
    k = torch.zeros(8, dtype=torch.int64, device="cuda:0")
    v = torch.zeros(8, dtype=torch.int32, device="cuda:0")
    ko = torch.empty_like(k)
    assert lib.sphgb_sort_by_key(ctx.h, k.data_ptr(), ko.data_ptr(), v.data_ptr(), None, 8, 63) == _lib.SPHGB_ERR_ARG
    assert lib.sphgb_sort_by_key(ctx.h, k.data_ptr(), ko.data_ptr(), None, None, 8, 0) == _lib.SPHGB_ERR_ARG
    assert lib.sphgb_sort_by_key(ctx.h, k.data_ptr(), ko.data_ptr(), None, None, 8, 65) == _lib.SPHGB_ERR_ARG
    assert lib.sphgb_sort_by_key(ctx.h, k.data_ptr(), k.data_ptr(), None, None, 8, 63) == _lib.SPHGB_ERR_ARG
    assert lib.sphgb_sort_by_key(ctx.h, k.data_ptr(), ko.data_ptr(), None, None, 0, 63) == 0
    ctx.close()
