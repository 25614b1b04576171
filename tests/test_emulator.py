"""The GPU engine's code run by the CPU emulator, against the oracle (CPU only).

tests/emu/kf_emu.cpp executes the library's launch schedules with the very
functions the CUDA kernels run (kissfft_gb300/csrc/kf_engine.cuh), one
thread index at a time.  This checks the plan tables, pass grouping,
digit-reversal addressing, two-pass splits (forced with small tile limits),
real split/merge, N-D axis passes and the fast FIR without a GPU.  Fixed
point must match the oracle bit for bit; float/double within the bound
2e-7*log2(N) / 1e-15*log2(N) (the IEEE generic-radix butterfly regroups
its sums).
"""
import ctypes
import os
import subprocess

import numpy as np
import pytest

import inputs
from oracle import kfo

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
EMU = os.path.join(ROOT, "tests", "emu", "_build", "libkfemu.so")
DT = {"float": 0, "double": 1, "int16_t": 2, "int32_t": 3}
L = ctypes.c_longlong


@pytest.fixture(scope="module")
def emu():
    csrc = os.path.join(ROOT, "kissfft_gb300", "csrc")
    src = os.path.join(ROOT, "tests", "emu", "kf_emu.cpp")
    deps = [src] + [os.path.join(csrc, f) for f in os.listdir(csrc)]
    if not os.path.exists(EMU) or os.path.getmtime(EMU) < max(os.path.getmtime(d) for d in deps):
        os.makedirs(os.path.dirname(EMU), exist_ok=True)
        subprocess.run(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-Wno-unknown-pragmas", "-shared", "-fPIC",
                        "-I", csrc, src, os.path.join(csrc, "kf_plan.cpp"), "-o", EMU], check=True)
    return ctypes.CDLL(EMU)


@pytest.fixture(autouse=True)
def in_bounds(emu):
    """Every test: no shared-tile, global or table access of the engine fell
    outside the memory its run owns (KF_MEM_CHECK hooks, counted by the
    emulator)."""
    emu.emu_oob_take.restype = ctypes.c_longlong
    emu.emu_oob_take()
    yield
    assert emu.emu_oob_take() == 0, "out-of-bounds accesses"


def p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def fixed(dt):
    return dt in ("int16_t", "int32_t")


def check(got, ref_fn, x, dt, n, inv=0):
    if fixed(dt):
        assert np.array_equal(got, ref_fn()), (dt, n, inv)
    else:
        z = inputs.to_complex128(x, dt)
        ex = np.fft.ifft(z, axis=-1) * n if inv else np.fft.fft(z, axis=-1)
        e = np.max(np.linalg.norm(inputs.to_complex128(got, dt) - ex, axis=-1) / np.linalg.norm(ex, axis=-1))
        bound = (2e-7 if dt == "float" else 1e-15) * max(1.0, np.log2(n))
        assert e <= bound, (dt, n, inv, e)


# (n, lmax): lmax > 0 forces the two-pass split through a small tile
C2C_CASES = [(1, 0), (2, 0), (3, 0), (7, 0), (8, 0), (12, 0), (30, 0), (97, 0), (120, 0), (480, 0), (1000, 0),
             (1024, 0), (3003, 0), (4099, 0), (16384, 0), (17017, 0), (65536, 0), (4096, 64), (17017, 256),
             (65536, 256), (131072, 512), (480, 32), (1000, 40), (961, 31), (8198, 4099)]


@pytest.mark.parametrize("dtype", ["int16_t", "int32_t", "float", "double"])
def test_c2c(emu, dtype):
    for n, lmax in C2C_CASES:
        for inv in (0, 1):
            x = inputs.cpx((2, n), dtype, n * 7 + inv)
            y = np.zeros_like(x)
            rc = emu.emu_c2c(DT[dtype], n, inv, lmax, p(x), p(y), L(2), L(n), L(1), L(n))
            assert rc == 0, (dtype, n, lmax, rc)
            check(y, lambda: kfo.fft(x, inv, dtype), x, dtype, n, inv)


@pytest.mark.parametrize("dtype", ["int16_t", "int32_t", "float"])
def test_stride(emu, dtype):
    for n, lmax, st in [(480, 0, 3), (1024, 64, 2), (3003, 0, 5)]:
        x = inputs.cpx((n * st,), dtype, 5)
        y = kfo.empty_cpx((n,), dtype)
        assert emu.emu_c2c(DT[dtype], n, 0, lmax, p(x), p(y), L(1), L(n * st), L(st), L(n)) == 0
        ref = kfo.fft_stride(x, n, st, 0, dtype)
        if fixed(dtype):
            assert np.array_equal(y, ref)
        else:
            assert np.max(np.abs(y - ref)) <= 1e-3 * np.max(np.abs(ref))


@pytest.mark.parametrize("dtype", ["int16_t", "int32_t", "float", "double"])
def test_real(emu, dtype):
    for nfft, lmax in [(2, 0), (4, 0), (6, 0), (10, 0), (30, 0), (120, 0), (480, 0), (1000, 0), (4096, 0),
                       (6006, 0), (34034, 0), (34034, 256), (131072, 0)]:
        t = inputs.real((3, nfft), dtype, nfft)
        f = kfo.empty_cpx((3, nfft // 2 + 1), dtype)
        assert emu.emu_r2c(DT[dtype], nfft, lmax, p(t), p(f), L(3)) == 0
        g = inputs.cpx((3, nfft // 2 + 1), dtype, nfft + 1)
        t2 = np.zeros((3, nfft), kfo.SCALAR[dtype])
        assert emu.emu_c2r(DT[dtype], nfft, lmax, p(g), p(t2), L(3)) == 0
        if fixed(dtype):
            assert np.array_equal(f, kfo.fftr(t, dtype)), (dtype, nfft, lmax)
            assert np.array_equal(t2, kfo.fftri(g, nfft, dtype)), (dtype, nfft, lmax)
        else:
            ex = np.fft.rfft(t.astype(np.float64), axis=-1)
            e = np.max(np.linalg.norm(f - ex, axis=-1) / np.linalg.norm(ex, axis=-1))
            assert e <= (2e-7 if dtype == "float" else 1e-15) * max(1.0, np.log2(nfft)), (dtype, nfft, e)
            ref2 = kfo.fftri(g, nfft, dtype)
            e2 = np.max(np.linalg.norm(t2 - ref2, axis=-1) / np.linalg.norm(ref2, axis=-1))
            assert e2 <= (8e-7 if dtype == "float" else 4e-15) * max(1.0, np.log2(nfft)), (dtype, nfft, e2)


@pytest.mark.parametrize("dtype", ["int16_t", "int32_t", "float"])
def test_nd_axes(emu, dtype):
    for dims in [[2, 3], [4, 4], [3, 5, 7], [8, 6], [2, 3, 4, 6], [64, 64], [5, 7, 11], [1024, 3], [3, 1024],
                 [17, 19, 23], [1, 480], [37, 2]]:
        for inv in (0, 1):
            x = inputs.cpx(tuple(dims), dtype, 11)
            buf = x.copy()
            d = (ctypes.c_int * len(dims))(*dims)
            for ax in range(len(dims)):
                assert emu.emu_axis(DT[dtype], d, len(dims), ax, inv, p(buf)) == 0
            ref = kfo.fftnd(x, dims, inv, dtype)
            if fixed(dtype):
                assert np.array_equal(buf, ref), (dtype, dims, inv)
            else:
                assert np.linalg.norm(buf - ref) / np.linalg.norm(ref) < 1e-5


@pytest.mark.parametrize("dtype", ["int16_t", "int32_t", "float"])
def test_nd_axes_two_pass(emu, dtype):
    """Axes longer than one tile (forced by small tile caps) run as two HBM
    passes over strided fibers: first, middle and last axes, generic radices
    included, bit-exact in fixed point (kiss_fftnd.c:156-188)."""
    for dims, lmax in [([64, 6], 16), ([6, 128], 16), ([3, 256, 5], 32), ([3003, 3], 256), ([2, 480, 7], 64),
                       ([1000, 1], 64)]:
        for inv in (0, 1):
            x = inputs.cpx(tuple(dims), dtype, 12 + inv)
            buf = x.copy()
            d = (ctypes.c_int * len(dims))(*dims)
            for ax in range(len(dims)):
                long_axis = dims[ax] > lmax
                rc = emu.emu_axis_lmax(DT[dtype], d, len(dims), ax, inv, lmax if long_axis else 0, p(buf))
                assert rc == 0, (dims, ax, rc)
            ref = kfo.fftnd(x, dims, inv, dtype)
            if fixed(dtype):
                assert np.array_equal(buf, ref), (dtype, dims, inv)
            else:
                assert np.linalg.norm(buf - ref) / np.linalg.norm(ref) < 1e-5, (dims, inv)


def test_fastfir(emu):
    rng = np.random.default_rng(4)
    for Lh, Ns in [(255, 20000), (1000, 50000), (17, 5000), (255, 2301), (255, 254), (2, 3000), (4095, 30000),
                   (4095, 4095), (1, 100)]:
        h = rng.standard_normal(Lh).astype(np.float32)
        x = rng.standard_normal(Ns).astype(np.float32)
        nfft = kfo.fastfir_nfft(Lh)
        H = np.zeros(nfft // 2 + 1, np.complex64)
        kfo.lib().kfo_fastfir_response_f32(p(h), L(Lh), L(nfft), p(H))
        y = np.zeros(max(Ns - Lh + 1, 1), np.float32)
        assert emu.emu_fastfir(p(H), L(nfft), L(Lh), p(x), L(Ns), p(y)) == 0
        ref = kfo.fastfir(h, x)
        # the power-of-two blocks run the exact kf_bfly sequence: same bits
        assert np.array_equal(y[:ref.size], ref)


def test_forced_tile_shapes(emu):
    """Other jobs-per-tile choices (all tiles partially filled) give the same bits."""
    for J, T in [(1, 32), (2, 64), (8, 96), (16, 512)]:
        emu.emu_force(J, T)
        try:
            for n in (120, 1000, 3003):
                x = inputs.cpx((5, n), "int16_t", n)
                y = np.zeros_like(x)
                assert emu.emu_c2c(2, n, 0, 0, p(x), p(y), L(5), L(n), L(1), L(n)) == 0
                assert np.array_equal(y, kfo.fft(x, 0, "int16_t")), (J, T, n)
        finally:
            emu.emu_force(0, 0)


@pytest.mark.parametrize("dtype", ["int16_t", "int32_t"])
def test_narrow_tiles_real_and_nd(emu, dtype):
    """Tiles of 1, 2 and 4 jobs (the narrower shapes the autotuner also times
    for launches with few tiles per SM) on real rows, both directions, and
    on every axis of N-D arrays, including the 128^3-style real-row shape:
    bit-exact against the oracle."""
    for J in (1, 2, 4):
        emu.emu_force(J, 0)
        try:
            for nfft in (128, 480, 4096):
                t = inputs.real((5, nfft), dtype, nfft + J)
                f = kfo.empty_cpx((5, nfft // 2 + 1), dtype)
                assert emu.emu_r2c(DT[dtype], nfft, 0, p(t), p(f), L(5)) == 0
                assert np.array_equal(f, kfo.fftr(t, dtype)), (J, nfft)
                g = inputs.cpx((5, nfft // 2 + 1), dtype, nfft + J + 1)
                t2 = np.zeros((5, nfft), kfo.SCALAR[dtype])
                assert emu.emu_c2r(DT[dtype], nfft, 0, p(g), p(t2), L(5)) == 0
                assert np.array_equal(t2, kfo.fftri(g, nfft, dtype)), (J, nfft)
            for dims in ([16, 65], [128, 6], [3, 64, 5]):
                for inv in (0, 1):
                    x = inputs.cpx(tuple(dims), dtype, 20 + J + inv)
                    buf = x.copy()
                    d = (ctypes.c_int * len(dims))(*dims)
                    for ax in range(len(dims)):
                        assert emu.emu_axis(DT[dtype], d, len(dims), ax, inv, p(buf)) == 0
                    assert np.array_equal(buf, kfo.fftnd(x, dims, inv, dtype)), (J, dims, inv)
        finally:
            emu.emu_force(0, 0)


@pytest.mark.parametrize("mode", [0, 1, 2])
@pytest.mark.parametrize("dtype", ["int16_t", "int32_t", "float"])
def test_shared_index_maps(emu, dtype, mode):
    """Every shared-tile index map (XOR fold, identity, one-level XOR) on row
    and column tiles, real transforms included, gives the oracle's bits."""
    emu.emu_force_swz(mode)
    try:
        for col in (0, 1):
            emu.emu_force_col(col)
            for n in (30, 480, 1000, 3003, 1024, 65536):
                x = inputs.cpx((6, n), dtype, n + mode)
                y = np.zeros_like(x)
                assert emu.emu_c2c(DT[dtype], n, 0, 0, p(x), p(y), L(6), L(n), L(1), L(n)) == 0
                check(y, lambda: kfo.fft(x, 0, dtype), x, dtype, n, 0)
            for nfft in (480, 4096, 6006):
                t = inputs.real((3, nfft), dtype, nfft)
                f = kfo.empty_cpx((3, nfft // 2 + 1), dtype)
                assert emu.emu_r2c(DT[dtype], nfft, 0, p(t), p(f), L(3)) == 0
                if fixed(dtype):
                    assert np.array_equal(f, kfo.fftr(t, dtype)), (mode, col, nfft)
                else:
                    ex = np.fft.rfft(t.astype(np.float64), axis=-1)
                    e = np.max(np.linalg.norm(f - ex, axis=-1) / np.linalg.norm(ex, axis=-1))
                    assert e <= 2e-7 * np.log2(nfft), (mode, col, nfft, e)
    finally:
        emu.emu_force_col(0)
        emu.emu_force_swz(-1)


@pytest.mark.parametrize("dtype", ["int16_t", "int32_t", "float"])
def test_column_tiles_on_row_batches(emu, dtype):
    """Column-layout tiles (jobs fastest in shared memory) on row-major
    batches give the same results as row-layout tiles."""
    emu.emu_force_col(1)
    try:
        for J in (2, 8):
            emu.emu_force(J, 0)
            for n in (30, 480, 1000, 3003, 1024, 65536):
                for inv in (0, 1):
                    x = inputs.cpx((11, n), dtype, n + J + inv)
                    y = np.zeros_like(x)
                    rc = emu.emu_c2c(DT[dtype], n, inv, 0, p(x), p(y), L(11), L(n), L(1), L(n))
                    assert rc == 0
                    check(y, lambda: kfo.fft(x, inv, dtype), x, dtype, n, inv)
            for nfft in (480, 4096, 6006):
                t = inputs.real((5, nfft), dtype, nfft)
                f = kfo.empty_cpx((5, nfft // 2 + 1), dtype)
                assert emu.emu_r2c(DT[dtype], nfft, 0, p(t), p(f), L(5)) == 0
                g = inputs.cpx((5, nfft // 2 + 1), dtype, nfft + 1)
                t2 = np.zeros((5, nfft), kfo.SCALAR[dtype])
                assert emu.emu_c2r(DT[dtype], nfft, 0, p(g), p(t2), L(5)) == 0
                if fixed(dtype):
                    assert np.array_equal(f, kfo.fftr(t, dtype)), (J, nfft)
                    assert np.array_equal(t2, kfo.fftri(g, nfft, dtype)), (J, nfft)
                else:
                    ex = np.fft.rfft(t.astype(np.float64), axis=-1)
                    e = np.max(np.linalg.norm(f - ex, axis=-1) / np.linalg.norm(ex, axis=-1))
                    assert e <= 2e-7 * np.log2(nfft), (J, nfft, e)
    finally:
        emu.emu_force_col(0)
        emu.emu_force(0, 0)


def _largest_prime(n):
    big, q = 1, 2
    while q * q <= n:
        while n % q == 0:
            big, n = q, n // q
        q += 1
    return max(big, n) if n > 1 else big


def test_uneven_mix_sizes(emu):
    """A seeded sample of the 20,000-request uneven mix (seed 3): up to 12
    sizes of every generic-prime class 7..31 and 40 smooth sizes, each run
    as its own request kind and sample type against the oracle, and every
    sampled size also as a Q15 complex transform, bit for bit."""
    mix = inputs.uneven_mix(20000, seed=3)
    rng = np.random.default_rng(30)
    classes = {}
    for k, d, n in mix:
        big = _largest_prime(n)
        classes.setdefault(big if big > 5 else 0, []).append((k, d, n))
    assert sorted(c for c in classes if c) == [7, 11, 13, 17, 19, 23, 29, 31]
    sample = []
    for c, reqs in sorted(classes.items()):
        pick = rng.choice(len(reqs), size=min(len(reqs), 40 if c == 0 else 12), replace=False)
        sample += [reqs[i] for i in pick]
    for k, d, n in sample:
        x = inputs.cpx((1, n), "int16_t", n + 3)
        y = np.zeros_like(x)
        assert emu.emu_c2c(DT["int16_t"], n, 0, 0, p(x), p(y), L(1), L(n), L(1), L(n)) == 0
        assert np.array_equal(y, kfo.fft(x, 0, "int16_t")), n
        if k == "c2c" and d != "int16_t":
            x = inputs.cpx((1, n), d, n)
            y = np.zeros_like(x)
            assert emu.emu_c2c(DT[d], n, 0, 0, p(x), p(y), L(1), L(n), L(1), L(n)) == 0
            check(y, lambda: kfo.fft(x, 0, d), x, d, n)
        elif k == "r2c":
            t = inputs.real((1, n), d, n)
            f = kfo.empty_cpx((1, n // 2 + 1), d)
            assert emu.emu_r2c(DT[d], n, 0, p(t), p(f), L(1)) == 0
            ex = np.fft.rfft(t.astype(np.float64), axis=-1)
            e = np.linalg.norm(f - ex) / np.linalg.norm(ex)
            assert e <= 2e-7 * max(1.0, np.log2(n)), (n, e)


def test_overflow_counts_match_reference(emu):
    """The GPU engine's code performs the reference's overflow-checked
    operations one for one: run by the emulator with the engine's overflow
    hook counting (KF_OVF_CHECK, kissfft_gb300/csrc/kf_arith.cuh), every case
    of tests/golden/overflow.json gives the reference's CHECK_OVERFLOW warning
    count and output, also through two-pass splits and column tiles."""
    import hashlib
    import json
    emu.emu_overflows_take.restype = ctypes.c_longlong
    with open(os.path.join(ROOT, "tests", "golden", "overflow.json")) as f:
        cases = json.load(f)["cases"]
    sha = lambda a: hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()
    # tile limits that force two HBM passes (for real cases: of the half-size transform)
    split = {480: 32, 961: 31, 1000: 40, 4096: 64, 17017: 256, 34034: 256, 65536: 256}
    ran = 0
    for two_pass, col in ((0, 0), (1, 0), (0, 1)):
        emu.emu_force_col(col)
        try:
            for c in cases:
                dt, n, b = c["dtype"], c["n"], c["batch"]
                if two_pass and n not in split:
                    continue
                lmax = split[n] if two_pass else 0
                emu.emu_overflows_take()
                ran += 1
                if c["kind"] == "c2c":
                    x = inputs.named(c["gen"], (b, n), dt, c["seed"], True)
                    y = np.zeros_like(x)
                    assert emu.emu_c2c(DT[dt], n, c["inverse"], lmax, p(x), p(y), L(b), L(n), L(1), L(n)) == 0
                elif c["kind"] == "r2c":
                    x = inputs.named(c["gen"], (b, n), dt, c["seed"], False)
                    y = kfo.empty_cpx((b, n // 2 + 1), dt)
                    assert emu.emu_r2c(DT[dt], n, lmax, p(x), p(y), L(b)) == 0
                else:
                    x = inputs.named(c["gen"], (b, n // 2 + 1), dt, c["seed"], True)
                    y = np.zeros((b, n), kfo.SCALAR[dt])
                    assert emu.emu_c2r(DT[dt], n, lmax, p(x), p(y), L(b)) == 0
                assert emu.emu_overflows_take() == c["overflows"], (lmax, col, c)
                assert sha(y) == c["sha"], (lmax, col, c)
        finally:
            emu.emu_force_col(0)
    assert ran > 2 * len(cases)


def test_bounds_check_catches_short_regions(emu):
    """The bounds check fires: with the output region or the shared tile
    declared 8 bytes short of the real buffers (which keep their full size),
    the engine's last accesses are counted as out of bounds."""
    x = inputs.cpx((2, 480), "int16_t", 1)
    y = np.zeros_like(x)
    for which in (1, 2):
        emu.emu_trim(which, L(8))
        try:
            assert emu.emu_c2c(DT["int16_t"], 480, 0, 0, p(x), p(y), L(2), L(480), L(1), L(480)) == 0
        finally:
            emu.emu_trim(which, L(0))
        assert emu.emu_oob_take() > 0, which
    assert emu.emu_c2c(DT["int16_t"], 480, 0, 0, p(x), p(y), L(2), L(480), L(1), L(480)) == 0
    assert np.array_equal(y, kfo.fft(x, 0, "int16_t"))


@pytest.mark.parametrize("dtype", ["int16_t", "int32_t"])
def test_every_small_size(emu, dtype):
    """Exhaustive small sizes: every complex nfft 1..1100 in both directions
    (every generic prime up to 1097 included) and every even real nfft
    2..1100 forward and inverse, bit for bit against the oracle (and in
    bounds, as every emulator test)."""
    for n in range(1, 1101):
        for inv in (0, 1):
            x = inputs.cpx((3, n), dtype, 7 * n + inv)
            y = np.zeros_like(x)
            assert emu.emu_c2c(DT[dtype], n, inv, 0, p(x), p(y), L(3), L(n), L(1), L(n)) == 0, n
            assert np.array_equal(y, kfo.fft(x, inv, dtype)), (n, inv)
    for nfft in range(2, 1101, 2):
        t = inputs.real((3, nfft), dtype, nfft)
        f = kfo.empty_cpx((3, nfft // 2 + 1), dtype)
        assert emu.emu_r2c(DT[dtype], nfft, 0, p(t), p(f), L(3)) == 0, nfft
        assert np.array_equal(f, kfo.fftr(t, dtype)), nfft
        g = inputs.cpx((3, nfft // 2 + 1), dtype, nfft + 1)
        t2 = np.zeros((3, nfft), kfo.SCALAR[dtype])
        assert emu.emu_c2r(DT[dtype], nfft, 0, p(g), p(t2), L(3)) == 0, nfft
        assert np.array_equal(t2, kfo.fftri(g, nfft, dtype)), nfft


def test_refuses_offsets_beyond_32_bits(emu):
    """Strides whose in-transform offsets would pass 2^31 - 1 elements (a
    huge kiss_fft_stride stride, an N-D axis over 2^30 other elements) are
    refused when the schedule is built, before any memory is touched (the
    buffers passed here are tiny and never read)."""
    x = np.zeros((1, 2), np.int16)
    y = np.zeros((1, 2), np.int16)
    st = 3_000_000  # 999 * 3e6 > 2^31
    assert emu.emu_c2c(DT["int16_t"], 1000, 0, 0, p(x), p(y), L(1), L(1000 * st), L(st), L(1000)) == -3
    st = 2_150_000  # just over: 999 * 2.15e6 > 2^31 - 1 (2_149_634 is the first stride that does not fit)
    assert emu.emu_c2c(DT["int16_t"], 1000, 0, 0, p(x), p(y), L(1), L(1000 * st), L(st), L(1000)) == -3
    dims = (ctypes.c_int * 2)(3, 1 << 30)
    assert emu.emu_axis(DT["float"], dims, 2, 0, 0, p(x)) == -3

