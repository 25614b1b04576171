"""GPU parity tests: the sm_103a kernels through the drop-in C ABI
(libkissfft_cuda-<type>.so) against the reference's golden vectors and the
oracle.

Fixed point (Q15/Q31) must match the reference bit for bit (SHA-256 of the
output bytes).  Float and double must stay within the relative L2 bound
2e-7*log2(N) (float) / 1e-15*log2(N) (double) of an FP64 transform, per
transform.
"""
import numpy as np
import pytest

import inputs
from gpu_util import bound, c128, empty_dev, from_dev, relerr_rows, sha, to_dev
from oracle import kfo

pytestmark = pytest.mark.gpu

DTYPES = ["float", "double", "int16_t", "int32_t"]


@pytest.fixture(scope="module")
def kf():
    import torch
    if not torch.cuda.is_available():
        pytest.fail("GPU tests need a CUDA device")
    import kissfft_gb300
    return kissfft_gb300


def fixed(dt):
    return dt in ("int16_t", "int32_t")


@pytest.mark.parametrize("dtype", DTYPES)
def test_c2c_golden(kf, golden, dtype):
    """Every golden complex case, batched on device buffers."""
    for c in golden["c2c"]:
        if c["dtype"] != dtype:
            continue
        n, b, inv = c["n"], c["batch"], c["inverse"]
        x = inputs.cpx((b, n), dtype, c["seed"])
        cfg = kf.kiss_fft_alloc(n, inv, dtype)
        assert cfg is not None, (n, kf.last_error(dtype))
        xd = to_dev(x)
        yd = empty_dev(x)
        kf.kiss_fft_batch(cfg, xd, yd, b)
        y = from_dev(yd, x)
        if fixed(dtype):
            assert sha(y) == c["sha256"], c
        else:
            z = c128(x, dtype)
            exact = np.fft.ifft(z, axis=-1) * n if inv else np.fft.fft(z, axis=-1)
            err = relerr_rows(c128(y, dtype), exact)
            assert err <= bound(dtype, n), (c, err)
        cfg.free()


def test_device_plan_tables_match_the_reference(kf, golden):
    """The twiddle tables the kernels read, copied back from the device plan,
    hash-match the reference's cfg->twiddles (kiss_fft.c:361-367) and the
    real plans' super twiddles (kiss_fftr.c:53-59), for all four sample
    types and both directions."""
    import ctypes
    L = kf.core()
    code = {"float": 0, "double": 1, "int16_t": 2, "int32_t": 3}
    for key, make, which, nkey in (("twiddles", L.kfg_plan_c2c, 0, "n"),
                                   ("super_twiddles", L.kfg_plan_real, 1, "nfft")):
        for c in golden[key]:
            p = make(code[c["dtype"]], c[nkey], c["inverse"])
            assert p, (c, L.kfg_last_error())
            try:
                nb = L.kfg_plan_table(p, which, None, 0)
                assert nb > 0, (c, L.kfg_last_error())
                buf = (ctypes.c_uint8 * nb)()
                assert L.kfg_plan_table(p, which, buf, nb) == nb
                assert sha(np.frombuffer(buf, np.uint8)) == c["sha256"], c
            finally:
                L.kfg_plan_free(p)


@pytest.mark.parametrize("dtype", DTYPES)
def test_c2c_host_pointers_single_calls(kf, dtype):
    """kiss_fft with host buffers, one transform per call (the reference's own
    calling convention), against the oracle."""
    for n in [1, 7, 64, 480, 1000, 3003, 4099, 65536]:
        cfg = kf.kiss_fft_alloc(n, 0, dtype)
        x = inputs.cpx((n,), dtype, n)
        y = kfo.empty_cpx((n,), dtype)
        kf.kiss_fft(cfg, x, y)
        ref = kfo.fft(x, 0, dtype)
        if fixed(dtype):
            assert np.array_equal(y, ref), n
        else:
            assert relerr_rows(c128(y, dtype)[None], c128(ref, dtype)[None]) <= 2 * bound(dtype, n)


@pytest.mark.parametrize("dtype", DTYPES)
def test_cfg_in_caller_memory(kf, dtype):
    """kiss_fft_alloc's placement protocol (reference kiss_fft.h:94-115): a
    size query, then the cfg placed in the caller's buffer (the returned
    pointer is that buffer), a correct transform through it, and a free that
    releases the device plan but leaves the buffer to the caller."""
    import ctypes
    L = kf.load(dtype)
    n = 480
    need = ctypes.c_size_t(0)
    assert not L.kiss_fft_cuda_alloc(n, 0, None, ctypes.byref(need))
    buf = ctypes.create_string_buffer(need.value + 64)
    got = ctypes.c_size_t(len(buf))
    cfg = L.kiss_fft_cuda_alloc(n, 0, buf, ctypes.byref(got))
    assert cfg == ctypes.addressof(buf), kf.last_error(dtype)
    assert got.value == need.value
    x = inputs.cpx((n,), dtype, 94)
    y = kfo.empty_cpx((n,), dtype)
    L.kiss_fft_cuda(ctypes.c_void_p(cfg), x.ctypes.data_as(ctypes.c_void_p), y.ctypes.data_as(ctypes.c_void_p))
    assert L.kiss_fft_cuda_status() == 0
    ref = kfo.fft(x, 0, dtype)
    if fixed(dtype):
        assert np.array_equal(y, ref)
    else:
        assert relerr_rows(c128(y, dtype)[None], c128(ref, dtype)[None]) <= 2 * bound(dtype, n)
    L.kiss_fft_cuda_free(ctypes.c_void_p(cfg))
    del buf


@pytest.mark.parametrize("dtype", DTYPES)
def test_kfc_plan_cache(kf, dtype):
    """kfc_fft / kfc_ifft / kfc_cleanup (reference kfc.c:24-83): the cache
    sizes of the reference's KFC_TEST sequence (kfc.c:85-109), and results
    against the oracle on host buffers, bit-identical on device buffers."""
    n = 512
    kf.kfc_cleanup(dtype)
    assert kf.kfc_ncached(dtype) == 0
    x = inputs.cpx((n,), dtype, 85)
    y = kfo.empty_cpx((n,), dtype)
    kf.kfc_fft(n, x, y, dtype)
    assert kf.kfc_ncached(dtype) == 1
    y2 = kfo.empty_cpx((n,), dtype)
    kf.kfc_fft(n, x, y2, dtype)
    assert kf.kfc_ncached(dtype) == 1
    z = kfo.empty_cpx((n,), dtype)
    kf.kfc_ifft(n, x, z, dtype)
    assert kf.kfc_ncached(dtype) == 2
    for got, inv in ((y, 0), (y2, 0), (z, 1)):
        ref = kfo.fft(x, inv, dtype)
        if fixed(dtype):
            assert np.array_equal(got, ref), inv
        else:
            assert relerr_rows(c128(got, dtype)[None], c128(ref, dtype)[None]) <= 2 * bound(dtype, n), inv
    yd = empty_dev(y)
    kf.kfc_fft(n, to_dev(x), yd, dtype)
    assert np.array_equal(from_dev(yd, y), y)
    assert kf.kfc_ncached(dtype) == 2
    kf.kfc_cleanup(dtype)
    assert kf.kfc_ncached(dtype) == 0


@pytest.mark.parametrize("dtype", DTYPES)
def test_stride(kf, dtype):
    for n, st in [(480, 3), (1024, 2), (3003, 5), (65536, 2)]:
        cfg = kf.kiss_fft_alloc(n, 0, dtype)
        x = inputs.cpx((n * st,), dtype, 99)
        y = empty_dev(kfo.empty_cpx((n,), dtype))
        kf.kiss_fft_stride(cfg, to_dev(x), y, st)
        got = from_dev(y, kfo.empty_cpx((n,), dtype))
        ref = kfo.fft_stride(x, n, st, 0, dtype)
        if fixed(dtype):
            assert np.array_equal(got, ref), (n, st)
        else:
            assert relerr_rows(c128(got, dtype)[None], c128(ref, dtype)[None]) <= 2 * bound(dtype, n)


@pytest.mark.parametrize("dtype", DTYPES)
def test_real_golden(kf, golden, dtype):
    for c in golden["r2c"]:
        if c["dtype"] != dtype:
            continue
        n, b = c["n"], c["batch"]
        t = inputs.real((b, n), dtype, c["seed"])
        cfg = kf.kiss_fftr_alloc(n, 0, dtype)
        out = kfo.empty_cpx((b, n // 2 + 1), dtype)
        od = empty_dev(out)
        kf.kiss_fftr_batch(cfg, to_dev(t), od, b)
        f = from_dev(od, out)
        if fixed(dtype):
            assert sha(f) == c["sha256"], c
        else:
            exact = np.fft.rfft(t.astype(np.float64), axis=-1)
            assert relerr_rows(c128(f, dtype), exact) <= bound(dtype, n), c
    for c in golden["c2r"]:
        if c["dtype"] != dtype:
            continue
        n, b = c["n"], c["batch"]
        f = inputs.cpx((b, n // 2 + 1), dtype, c["seed"])
        cfg = kf.kiss_fftr_alloc(n, 1, dtype)
        out = np.zeros((b, n), kfo.SCALAR[dtype])
        od = empty_dev(out)
        kf.kiss_fftri_batch(cfg, to_dev(f), od, b)
        t = from_dev(od, out)
        if fixed(dtype):
            assert sha(t) == c["sha256"], c
        else:
            ref = kfo.fftri(f, n, dtype)
            e = np.linalg.norm(t - ref, axis=1) / np.maximum(np.linalg.norm(ref, axis=1), 1e-30)
            assert float(np.max(e)) <= 4 * bound(dtype, n), c


@pytest.mark.parametrize("dtype", DTYPES)
def test_nd_golden(kf, golden, dtype):
    for c in golden["nd"]:
        if c["dtype"] != dtype:
            continue
        dims, inv = c["dims"], c["inverse"]
        x = inputs.cpx(tuple(dims), dtype, c["seed"])
        cfg = kf.kiss_fftnd_alloc(dims, inv, dtype)
        od = empty_dev(x)
        kf.kiss_fftnd(cfg, to_dev(x), od)
        y = from_dev(od, x)
        if fixed(dtype):
            assert sha(y) == c["sha256"], c
        else:
            z = c128(x, dtype)
            exact = np.fft.ifftn(z) * z.size if inv else np.fft.fftn(z)
            assert relerr_rows(c128(y, dtype)[None], exact[None]) <= bound(dtype, z.size), c


@pytest.mark.parametrize("dtype", DTYPES)
def test_ndr_golden(kf, golden, dtype):
    for c in golden["ndr"]:
        if c["dtype"] != dtype or c.get("ref_rejects"):
            continue
        dims = c["dims"]
        t = inputs.real(tuple(dims), dtype, c["seed"])
        cfg = kf.kiss_fftndr_alloc(dims, 0, dtype)
        out = kfo.empty_cpx(tuple(dims[:-1]) + (dims[-1] // 2 + 1,), dtype)
        od = empty_dev(out)
        kf.kiss_fftndr(cfg, to_dev(t), od)
        f = from_dev(od, out)
        if fixed(dtype):
            assert sha(f) == c["sha256"], c
        else:
            exact = np.fft.rfftn(t.astype(np.float64))
            assert relerr_rows(c128(f, dtype)[None], exact[None]) <= bound(dtype, t.size), c
    for c in golden["ndri"]:
        if c["dtype"] != dtype:
            continue
        dims = c["dims"]
        f = inputs.cpx(tuple(dims[:-1]) + (dims[-1] // 2 + 1,), dtype, c["seed"])
        cfg = kf.kiss_fftndr_alloc(dims, 1, dtype)
        out = np.zeros(tuple(dims), kfo.SCALAR[dtype])
        od = empty_dev(out)
        kf.kiss_fftndri(cfg, to_dev(f), od)
        t = from_dev(od, out)
        if fixed(dtype):
            assert sha(t) == c["sha256"], c
        else:
            ref = kfo.fftndri(f, dims, dtype)
            assert np.linalg.norm(t - ref) / np.linalg.norm(ref) <= 4 * bound(dtype, t.size), c


@pytest.mark.parametrize("dtype", ["float", "int16_t"])
def test_nd_autotuned_and_specialised(kf, dtype):
    """N-D transforms after the autotuner has picked their launch shapes and
    with plan-specialised kernels: complex 2-D (one axis longer than a tile),
    real 3-D forward and inverse, against the oracle (Q15 bit for bit)."""
    kf.set_specialize(True)
    try:
        for dims in ([48, 20000], [24, 40, 16]):
            x = inputs.cpx(tuple(dims), dtype, 77)
            cfg = kf.kiss_fftnd_alloc(dims, 0, dtype)
            kf.autotune(cfg, 1)
            kf.prepare(cfg, 1)
            od = empty_dev(x)
            kf.kiss_fftnd(cfg, to_dev(x), od)
            y = from_dev(od, x)
            ref = kfo.fftnd(x, dims, 0, dtype)
            if fixed(dtype):
                assert np.array_equal(y, ref), dims
            else:
                assert relerr_rows(c128(y, dtype)[None], c128(ref, dtype)[None]) <= bound(dtype, x.size), dims
            cfg.free()
        dims = [32, 24, 40]
        t = inputs.real(tuple(dims), dtype, 78)
        fcfg, icfg = kf.kiss_fftndr_alloc(dims, 0, dtype), kf.kiss_fftndr_alloc(dims, 1, dtype)
        for c in (fcfg, icfg):
            kf.autotune(c, 1)
            kf.prepare(c, 1)
        out = kfo.empty_cpx((32, 24, 21), dtype)
        od = empty_dev(out)
        kf.kiss_fftndr(fcfg, to_dev(t), od)
        f = from_dev(od, out)
        back = np.zeros(tuple(dims), kfo.SCALAR[dtype])
        bd = empty_dev(back)
        kf.kiss_fftndri(icfg, to_dev(f), bd)
        tb = from_dev(bd, back)
        if fixed(dtype):
            assert np.array_equal(f, kfo.fftndr(t, dims, dtype))
            assert np.array_equal(tb, kfo.fftndri(f, dims, dtype))
        else:
            assert relerr_rows(c128(f, dtype)[None], c128(kfo.fftndr(t, dims, dtype), dtype)[None]) <= bound(dtype, t.size)
            ref = kfo.fftndri(f, dims, dtype)
            assert np.linalg.norm(tb - ref) / np.linalg.norm(ref) <= 4 * bound(dtype, t.size)
        fcfg.free()
        icfg.free()
    finally:
        kf.set_specialize(False)


def test_fastfir_golden(kf, golden):
    for c in golden["fastfir"]:
        rng = np.random.default_rng(c["seed"])
        h = rng.standard_normal(c["L"]).astype(np.float32)
        x = rng.standard_normal(c["Ns"]).astype(np.float32)
        cfg = kf.kiss_fastfir_alloc(h)
        assert cfg is not None and cfg.nfft == kfo.fastfir_nfft(c["L"])
        y = np.zeros(c["nout"], np.float32)
        yd = empty_dev(y)
        n = kf.kiss_fastfir_filter(cfg, to_dev(x), yd)
        assert n == c["nout"]
        got = from_dev(yd, y)
        exact = np.convolve(x.astype(np.float64), h.astype(np.float64), "valid")
        err = np.linalg.norm(got - exact) / np.linalg.norm(exact)
        # the reference's own fast FIR error on this case, with headroom
        assert err <= max(4 * c["ref_relerr"], 1e-6), (c, err)


def test_fastfir_streaming_matches_whole_signal(kf):
    """kiss_fastfir's chunked calls plus the flush give the whole-signal result
    (tools/kiss_fastfir.c:222-239 as driven by do_file_filter)."""
    rng = np.random.default_rng(7)
    h = rng.standard_normal(255).astype(np.float32)
    x = rng.standard_normal(50000).astype(np.float32)
    cfg = kf.kiss_fastfir_alloc(h)
    whole = np.zeros(x.size - h.size + 1, np.float32)
    kf.kiss_fastfir_filter(cfg, x, whole)
    nbuf = cfg.nfft + 4 * (cfg.nfft - h.size + 1)
    inbuf = np.zeros(nbuf, np.float32)
    outbuf = np.zeros(nbuf, np.float32)
    off = [0]
    got = []
    pos = 0
    while True:
        nread = min(nbuf - off[0], x.size - pos)
        inbuf[off[0]:off[0] + nread] = x[pos:pos + nread]
        pos += nread
        n = kf.kiss_fastfir(cfg, inbuf, outbuf, nread, off)
        got.append(outbuf[:n].copy())
        if nread == 0:
            break
    got = np.concatenate(got)
    assert got.size == whole.size
    assert np.allclose(got, whole, rtol=0, atol=1e-5)


def test_round_trip_1024_on_4096(kf):
    """4096 x 1024-point complex float forward then inverse: N*x back."""
    import torch
    n, b = 1024, 4096
    x = inputs.cpx((b, n), "float", 0)
    fw, iv = kf.kiss_fft_alloc(n, 0), kf.kiss_fft_alloc(n, 1)
    xd = to_dev(x)
    yd, zd = torch.empty_like(xd), torch.empty_like(xd)
    kf.kiss_fft_batch(fw, xd, yd, b)
    kf.kiss_fft_batch(iv, yd, zd, b)
    y, z = from_dev(yd, x), from_dev(zd, x)
    exact = np.fft.fft(x.astype(np.complex128), axis=-1)
    assert relerr_rows(y.astype(np.complex128), exact) <= bound("float", n)
    assert relerr_rows(z.astype(np.complex128) / n, x.astype(np.complex128)) <= 2 * bound("float", n)


@pytest.mark.parametrize("dtype", ["int16_t", "int32_t"])
def test_fixed_point_bench_batches(kf, dtype):
    """The mixed-radix sizes at larger batches, bit-exact against the oracle."""
    for n, b in [(480, 512), (1000, 256), (3003, 64), (65536, 8)]:
        x = inputs.cpx((b, n), dtype, 1)
        cfg = kf.kiss_fft_alloc(n, 0, dtype)
        yd = empty_dev(x)
        kf.kiss_fft_batch(cfg, to_dev(x), yd, b)
        y = from_dev(yd, x)
        ref = kfo.fft(x, 0, dtype, nthreads=kfo.max_threads())
        assert np.array_equal(y, ref), (dtype, n)


def test_real_4096_round_trip(kf):
    """kiss_fftr / kiss_fftri at 4096 on sinusoids plus noise: ri(r(x)) = N*x."""
    import torch
    n, b = 4096, 512
    t = inputs.sinusoids(b, n, 2)
    fw, iv = kf.kiss_fftr_alloc(n, 0), kf.kiss_fftr_alloc(n, 1)
    td = to_dev(t)
    fd = torch.zeros((b, n // 2 + 1, 2), dtype=torch.float32, device="cuda")
    rd = torch.zeros_like(td)
    kf.kiss_fftr_batch(fw, td, fd, b)
    kf.kiss_fftri_batch(iv, fd, rd, b)
    f = fd.cpu().numpy().view(np.complex64)[..., 0]
    r = from_dev(rd, t)
    exact = np.fft.rfft(t.astype(np.float64), axis=-1)
    assert relerr_rows(f.astype(np.complex128), exact) <= bound("float", n)
    assert relerr_rows(r.astype(np.float64) / n, t.astype(np.float64)) <= 4 * bound("float", n)


def test_nd_2048_square_and_128_cube(kf):
    """2048 x 2048 complex and 128^3 real N-D transforms against numpy."""
    x = inputs.cpx((2048, 2048), "float", 2)
    cfg = kf.kiss_fftnd_alloc([2048, 2048], 0)
    od = empty_dev(x)
    kf.kiss_fftnd(cfg, to_dev(x), od)
    y = from_dev(od, x)
    exact = np.fft.fft2(x.astype(np.complex128))
    assert relerr_rows(y.astype(np.complex128)[None], exact[None]) <= bound("float", x.size)
    rng = np.random.default_rng(2)
    t = rng.standard_normal((128, 128, 128)).astype(np.float32)
    cfg = kf.kiss_fftndr_alloc([128, 128, 128], 0)
    out = np.zeros((128, 128, 65), np.complex64)
    od = empty_dev(out)
    kf.kiss_fftndr(cfg, to_dev(t), od)
    f = from_dev(od, out)
    exact = np.fft.rfftn(t.astype(np.float64))
    assert relerr_rows(f.astype(np.complex128)[None], exact[None]) <= bound("float", t.size)


def test_error_behaviour(kf):
    assert kf.kiss_fftr_alloc(1001, 0) is None          # kiss_fftr.c:29-32
    assert kf.kiss_fastfir_alloc.__doc__
    fw = kf.kiss_fftr_alloc(64, 0)
    t = np.zeros(64, np.float32)
    f = np.zeros(33, np.complex64)
    with pytest.raises(kf.KissFFTError):
        kf.kiss_fftri(fw, f, t)                         # improper alloc, kiss_fftr.c:124-127
    assert kf.kiss_fft_alloc(0, 0) is None
    assert kf.kiss_fftndr_alloc([4, 5], 0) is None       # odd real axis


@pytest.mark.parametrize("dtype", ["int16_t", "int32_t"])
def test_fixed_point_most_negative_samples(kf, dtype):
    """Inputs with the most negative sample (-32768 / -2^31) at 5% of the
    positions: negations and sums that wrap must truncate exactly as the
    reference's stores do (a device compile once turned -(-32768) into
    32768).  c2c over radices 2..5 and generic, real forward and inverse,
    and N-D, all bit for bit against the oracle."""
    import torch
    rng = np.random.default_rng(11)
    lo = np.iinfo(np.int16 if dtype == "int16_t" else np.int32).min

    def spiked(a):
        a = a.copy()
        a[rng.random(a.shape) < 0.05] = lo
        return a

    for n in (480, 1000, 3003, 4096, 65536):
        b = 8
        x = spiked(inputs.cpx((b, n), dtype, n + 3))
        for inv in (0, 1):
            cfg = kf.kiss_fft_alloc(n, inv, dtype)
            yd = empty_dev(x)
            kf.kiss_fft_batch(cfg, to_dev(x), yd, b)
            assert sha(from_dev(yd, x)) == sha(kfo.fft(x, inv, dtype)), (n, inv)
            cfg.free()
    for nfft in (1024, 6006):
        b = 16
        t = spiked(inputs.real((b, nfft), dtype, nfft))
        f = spiked(inputs.cpx((b, nfft // 2 + 1), dtype, nfft + 1))
        fw = kf.kiss_fftr_alloc(nfft, 0, dtype)
        iv = kf.kiss_fftr_alloc(nfft, 1, dtype)
        fd = empty_dev(kfo.empty_cpx((b, nfft // 2 + 1), dtype))
        kf.kiss_fftr_batch(fw, to_dev(t), fd, b)
        assert sha(from_dev(fd, kfo.empty_cpx((b, nfft // 2 + 1), dtype))) == sha(kfo.fftr(t, dtype)), nfft
        td = torch.zeros((b, nfft), dtype=getattr(torch, kfo.SCALAR[dtype].__name__), device="cuda")
        kf.kiss_fftri_batch(iv, to_dev(f), td, b)
        torch.cuda.synchronize()
        assert sha(td.cpu().numpy()) == sha(kfo.fftri(f, nfft, dtype)), nfft
        fw.free()
        iv.free()
    x = spiked(inputs.cpx((24, 40), dtype, 9))
    cfg = kf.kiss_fftnd_alloc([24, 40], 0, dtype)
    yd = empty_dev(x)
    kf.kiss_fftnd(cfg, to_dev(x), yd)
    assert sha(from_dev(yd, x)) == sha(kfo.fftnd(x, [24, 40], 0, dtype))
    cfg.free()
