"""The CPU oracle against the reference's golden vectors (CPU only).

The golden fixtures were produced by the reference library compiled from its
own sources (tests/golden/make_golden.py).  Fixed-point outputs, every sample
type's twiddle tables and the fast-FIR output must match bit for bit; this
pins the oracle that the GPU parity tests compare against.
"""
import hashlib
import os

import numpy as np
import pytest

import inputs
from oracle import kfo


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def _sel(cases, maxn=20000):
    return [c for c in cases if c.get("n", 0) <= maxn and not c.get("ref_rejects")]


def test_factor_matches_reference_examples():
    # kf_factor radix lists (reference kiss_fft.c:306-328)
    assert kfo.factor(480) == [4, 4, 2, 3, 5]
    assert kfo.factor(1000) == [4, 2, 5, 5, 5]
    assert kfo.factor(1024) == [4] * 5
    assert kfo.factor(3003) == [3, 7, 11, 13]
    assert kfo.factor(65536) == [4] * 8
    assert kfo.factor(131072) == [4] * 8 + [2]
    assert kfo.factor(17017) == [7, 11, 13, 17]
    assert kfo.factor(1) == [1]
    assert kfo.factor(2) == [2]
    assert kfo.factor(97) == [97]


def test_next_fast_size():
    assert kfo.next_fast_size(7) == 8
    assert kfo.next_fast_size(1001) == 1024
    assert kfo.next_fast_size(121) == 125


@pytest.mark.parametrize("dtype", ["float", "double", "int16_t", "int32_t"])
def test_twiddle_tables_bit_exact(golden, dtype):
    for c in golden["twiddles"]:
        if c["dtype"] == dtype:
            assert sha(kfo.twiddles(c["n"], c["inverse"], dtype)) == c["sha256"], c
    for c in golden["super_twiddles"]:
        if c["dtype"] == dtype:
            assert sha(kfo.super_twiddles(c["nfft"], c["inverse"], dtype)) == c["sha256"], c


@pytest.mark.parametrize("dtype", ["float", "double", "int16_t", "int32_t"])
def test_c2c_golden(golden, dtype):
    for c in _sel(golden["c2c"], 140000):
        if c["dtype"] != dtype:
            continue
        x = inputs.cpx((c["batch"], c["n"]), dtype, c["seed"])
        assert sha(kfo.fft(x, c["inverse"], dtype)) == c["sha256"], c


@pytest.mark.parametrize("dtype", ["float", "double", "int16_t", "int32_t"])
def test_real_golden(golden, dtype):
    for c in golden["r2c"]:
        if c["dtype"] == dtype:
            t = inputs.real((c["batch"], c["n"]), dtype, c["seed"])
            assert sha(kfo.fftr(t, dtype)) == c["sha256"], c
    for c in golden["c2r"]:
        if c["dtype"] == dtype:
            f = inputs.cpx((c["batch"], c["n"] // 2 + 1), dtype, c["seed"])
            assert sha(kfo.fftri(f, c["n"], dtype)) == c["sha256"], c


@pytest.mark.parametrize("dtype", ["float", "double", "int16_t", "int32_t"])
def test_nd_golden(golden, dtype):
    for c in golden["nd"]:
        if c["dtype"] == dtype:
            x = inputs.cpx(tuple(c["dims"]), dtype, c["seed"])
            assert sha(kfo.fftnd(x, c["dims"], c["inverse"], dtype)) == c["sha256"], c
    for c in golden["ndr"]:
        if c["dtype"] == dtype and not c.get("ref_rejects"):
            t = inputs.real(tuple(c["dims"]), dtype, c["seed"])
            assert sha(kfo.fftndr(t, c["dims"], dtype)) == c["sha256"], c
    for c in golden["ndri"]:
        if c["dtype"] == dtype:
            d = c["dims"]
            f = inputs.cpx(tuple(d[:-1]) + (d[-1] // 2 + 1,), dtype, c["seed"])
            assert sha(kfo.fftndri(f, d, dtype)) == c["sha256"], c


def test_small_arrays(small):
    for key in small.files:
        if not key.endswith("_in"):
            continue
        kind, rest = key.split("_", 1)
        if kind == "fir":
            continue
        dtype = next(d for d in ("int16_t", "int32_t", "float", "double") if rest.startswith(d + "_"))
        parts = [kind, dtype] + rest[len(dtype) + 1:].split("_")
        n = int(parts[2])
        x = small[key]
        y = small[key[:-3] + "_out"]
        if kind == "c2c":
            got = kfo.fft(x, int(parts[3]), dtype)
        elif kind == "r2c":
            got = kfo.fftr(x, dtype)
        else:
            got = kfo.fftri(x, n, dtype)
        assert np.array_equal(got, y), key


def test_fastfir_golden(golden):
    import numpy as np
    for c in golden["fastfir"]:
        rng = np.random.default_rng(c["seed"])
        h = rng.standard_normal(c["L"]).astype(np.float32)
        x = rng.standard_normal(c["Ns"]).astype(np.float32)
        y = kfo.fastfir(h, x)
        assert y.size == c["nout"] == c["Ns"] - c["L"] + 1
        assert sha(y) == c["sha256"], c
        exact = np.convolve(x.astype(np.float64), h.astype(np.float64), "valid")
        assert np.linalg.norm(y - exact) / np.linalg.norm(exact) < 1e-6


def test_float_error_within_bound(golden):
    """The oracle float build's error equals the reference's (same bits) and
    is inside the float bound 2e-7*log2(N)."""
    for c in golden["c2c"]:
        if c["dtype"] != "float" or c["n"] < 2 or c["n"] > 20000:
            continue
        bound = 2e-7 * max(1.0, np.log2(c["n"]))
        assert c["ref_relerr"] <= bound, c


@pytest.mark.parametrize("dtype", ["float", "double", "int16_t", "int32_t"])
def test_openmp_leg_split_same_bits(dtype):
    """The reference's KISSFFT_OPENMP form (top-level legs in parallel,
    kiss_fft.c:250-272) gives the sequential recursion's results bit for bit,
    including plans whose legs run generic butterflies (3003 = 3*7*11*13) and
    plans it does not split (p > 5 or a single stage)."""
    import inputs
    for n in (2, 4, 7, 12, 480, 1000, 1024, 3003, 17017, 4099):
        for inv in (0, 1):
            x = inputs.cpx((3, n), dtype, n + inv)
            a = kfo.fft(x, inv, dtype)
            b = kfo.fft_legs(x, inv, dtype, nthreads=4)
            assert np.array_equal(a, b), (dtype, n, inv)


def _overflow_cases():
    import json
    with open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "overflow.json")) as f:
        return json.load(f)["cases"]


def test_overflow_counts_match_reference():
    """The oracle's CHECK_OVERFLOW build counts exactly the warnings the
    reference built with -DCHECK_OVERFLOW printed (tests/golden/overflow.json),
    and its outputs hash to the reference's."""
    import inputs
    cases = _overflow_cases()
    assert sum(1 for c in cases if c["overflows"]) >= 40
    for c in cases:
        dt, n, b = c["dtype"], c["n"], c["batch"]
        if c["kind"] == "c2c":
            x = inputs.named(c["gen"], (b, n), dt, c["seed"], True)
            y, cnt = kfo.overflows(kfo.fft, x, c["inverse"], dt)
        elif c["kind"] == "r2c":
            x = inputs.named(c["gen"], (b, n), dt, c["seed"], False)
            y, cnt = kfo.overflows(kfo.fftr, x, dt)
        else:
            x = inputs.named(c["gen"], (b, n // 2 + 1), dt, c["seed"], True)
            y, cnt = kfo.overflows(kfo.fftri, x, n, dt)
        assert cnt == c["overflows"], c
        assert hashlib.sha256(np.ascontiguousarray(y).tobytes()).hexdigest() == c["sha"], c
    # the plain build never counts
    assert kfo.lib().kfo_checks_overflow() == 0 and kfo.lib_ovf().kfo_checks_overflow() == 1
