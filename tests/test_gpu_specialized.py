"""GPU parity of the plan-specialised kernels (NVRTC-compiled for each plan
shape) and of the TMA-staged tile loop, against the golden vectors.

The same golden cases as test_gpu_parity, run with specialisation on; the
fixed-point outputs must still match the reference bit for bit.
"""
import numpy as np
import pytest

import inputs
from gpu_util import bound, c128, empty_dev, from_dev, relerr_rows, sha, to_dev

pytestmark = pytest.mark.gpu

DTYPES = ["float", "double", "int16_t", "int32_t"]
SIZES = [7, 16, 64, 120, 480, 1000, 1024, 2048, 3003, 4096, 16384, 65536, 131072]


@pytest.fixture(scope="module")
def kf():
    import torch
    if not torch.cuda.is_available():
        pytest.fail("GPU tests need a CUDA device")
    import kissfft_gb300
    kissfft_gb300.set_specialize(True)
    yield kissfft_gb300
    kissfft_gb300.set_specialize(False)


@pytest.mark.parametrize("dtype", DTYPES)
def test_c2c_specialized(kf, golden, dtype):
    for c in golden["c2c"]:
        if c["dtype"] != dtype or c["n"] not in SIZES:
            continue
        n, b, inv = c["n"], c["batch"], c["inverse"]
        x = inputs.cpx((b, n), dtype, c["seed"])
        cfg = kf.kiss_fft_alloc(n, inv, dtype)
        kf.prepare(cfg, b)
        yd = empty_dev(x)
        kf.kiss_fft_batch(cfg, to_dev(x), yd, b)
        y = from_dev(yd, x)
        if dtype in ("int16_t", "int32_t"):
            assert sha(y) == c["sha256"], c
        else:
            z = c128(x, dtype)
            exact = np.fft.ifft(z, axis=-1) * n if inv else np.fft.fft(z, axis=-1)
            assert relerr_rows(c128(y, dtype), exact) <= bound(dtype, n), c


@pytest.mark.parametrize("dtype", DTYPES)
def test_real_specialized(kf, golden, dtype):
    for c in golden["r2c"]:
        if c["dtype"] != dtype:
            continue
        n, b = c["n"], c["batch"]
        t = inputs.real((b, n), dtype, c["seed"])
        cfg = kf.kiss_fftr_alloc(n, 0, dtype)
        from oracle import kfo
        out = kfo.empty_cpx((b, n // 2 + 1), dtype)
        od = empty_dev(out)
        kf.kiss_fftr_batch(cfg, to_dev(t), od, b)
        f = from_dev(od, out)
        if dtype in ("int16_t", "int32_t"):
            assert sha(f) == c["sha256"], c
        else:
            exact = np.fft.rfft(t.astype(np.float64), axis=-1)
            assert relerr_rows(c128(f, dtype), exact) <= bound(dtype, n), c


@pytest.mark.parametrize("dtype", ["int16_t", "float"])
def test_large_batches_tma_staged(kf, dtype):
    """Many tiles per persistent CTA (the TMA-staged loop wraps around):
    bit-exact against the oracle (Q15) or within the bound (float), with and
    without staging."""
    from oracle import kfo
    for n, b in [(1024, 20000), (480, 30001), (4096, 3000)]:
        x = inputs.cpx((b, n), dtype, 5)
        cfg = kf.kiss_fft_alloc(n, 0, dtype)
        kf.prepare(cfg, b)
        outs = []
        for tma in (1, 0):
            kf.core().kfg_set_tma(tma)
            yd = empty_dev(x)
            kf.kiss_fft_batch(cfg, to_dev(x), yd, b)
            outs.append(from_dev(yd, x))
        kf.core().kfg_set_tma(1)
        assert np.array_equal(outs[0], outs[1]), (dtype, n)
        if dtype == "int16_t":
            ref = kfo.fft(x[:512], 0, dtype, nthreads=kfo.max_threads())
            assert np.array_equal(outs[0][:512], ref)
        else:
            exact = np.fft.fft(x[:512].astype(np.complex128), axis=-1)
            assert relerr_rows(outs[0][:512].astype(np.complex128), exact) <= bound(dtype, n)
