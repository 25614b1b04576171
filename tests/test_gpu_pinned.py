"""Pinned host buffers through the C ABI.

Page-locked host memory is read and written by the kernels in place over
the host link (no staging copies).  Results must equal the same call on
device buffers bit for bit (the same kernels run), for single- and two-pass
complex plans, real forward/inverse, N-D and the fast FIR.
"""
import numpy as np
import pytest

import inputs

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def kf():
    import torch
    if not torch.cuda.is_available():
        pytest.fail("GPU tests need a CUDA device")
    import kissfft_gb300
    return kissfft_gb300


def pinned(a):
    import torch
    t = torch.from_numpy(np.ascontiguousarray(a).view(np.uint8).reshape(-1).copy()).pin_memory()
    return t


def device(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a).view(np.uint8).reshape(-1).copy()).cuda()


def host(t):
    import torch
    torch.cuda.synchronize()
    return t.cpu().numpy()


@pytest.mark.parametrize("dt,n,b", [("float", 1000, 7), ("float", 65536, 3), ("int16_t", 3003, 5),
                                    ("int32_t", 65536, 2), ("double", 480, 4)])
def test_c2c(kf, dt, n, b):
    import torch
    x = inputs.cpx((b, n), dt, n)
    cfg = kf.kiss_fft_alloc(n, 0, dt)
    xp, yp = pinned(x), torch.zeros(x.nbytes, dtype=torch.uint8).pin_memory()
    xd, yd = device(x), torch.zeros(x.nbytes, dtype=torch.uint8, device="cuda")
    kf.kiss_fft_batch(cfg, xp, yp, b)
    kf.kiss_fft_batch(cfg, xd, yd, b)
    assert np.array_equal(yp.numpy(), host(yd))
    cfg.free()


@pytest.mark.parametrize("nfft,b", [(4096, 9), (131072, 2)])
def test_real_round_trip(kf, nfft, b):
    import torch
    t = inputs.real((b, nfft), "float", nfft)
    fw = kf.kiss_fftr_alloc(nfft, 0, "float")
    iv = kf.kiss_fftr_alloc(nfft, 1, "float")
    nb = nfft // 2 + 1
    tp = pinned(t)
    fp = torch.zeros(b * nb * 8, dtype=torch.uint8).pin_memory()
    td = device(t)
    fd = torch.zeros(b * nb * 8, dtype=torch.uint8, device="cuda")
    kf.kiss_fftr_batch(fw, tp, fp, b)
    kf.kiss_fftr_batch(fw, td, fd, b)
    assert np.array_equal(fp.numpy(), host(fd))
    rp = torch.zeros(t.nbytes, dtype=torch.uint8).pin_memory()
    rd = torch.zeros(t.nbytes, dtype=torch.uint8, device="cuda")
    kf.kiss_fftri_batch(iv, fp, rp, b)
    kf.kiss_fftri_batch(iv, fd, rd, b)
    assert np.array_equal(rp.numpy(), host(rd))
    fw.free()
    iv.free()


def test_nd_and_fir(kf):
    import torch
    x = inputs.cpx((48, 64), "float", 3)
    cfg = kf.kiss_fftnd_alloc([48, 64], 0, "float")
    xp, yp = pinned(x), torch.zeros(x.nbytes, dtype=torch.uint8).pin_memory()
    xd, yd = device(x), torch.zeros(x.nbytes, dtype=torch.uint8, device="cuda")
    kf.kiss_fftnd(cfg, xp, yp)
    kf.kiss_fftnd(cfg, xd, yd)
    assert np.array_equal(yp.numpy(), host(yd))
    cfg.free()
    rng = np.random.default_rng(5)
    h = rng.standard_normal(255).astype(np.float32)
    s = rng.standard_normal(30000).astype(np.float32)
    ff = kf.kiss_fastfir_alloc(h)
    ny = s.size - h.size + 1
    # float tensors: the wrapper takes the signal length from numel()
    sp, op = torch.from_numpy(s.copy()).pin_memory(), torch.zeros(ny, dtype=torch.float32).pin_memory()
    sd, od = torch.from_numpy(s.copy()).cuda(), torch.zeros(ny, dtype=torch.float32, device="cuda")
    assert sp.numel() == s.size and sd.numel() == s.size
    assert kf.kiss_fastfir_filter(ff, sp, op) == ny
    assert kf.kiss_fastfir_filter(ff, sd, od) == ny
    assert np.array_equal(op.numpy(), host(od))
    ff.free()


@pytest.mark.parametrize("dt,n,b", [("float", 4096, 5000), ("int16_t", 1000, 50000), ("float", 65536, 300)])
def test_large_batches_pipelined(kf, dt, n, b):
    """Batches of 128 MiB and more on pinned buffers run as a chunked
    copy-in / kernels / copy-out pipeline: same bits as device buffers."""
    import torch
    x = inputs.cpx((b, n), dt, n + b)
    cfg = kf.kiss_fft_alloc(n, 0, dt)
    xp, yp = pinned(x), torch.zeros(x.nbytes, dtype=torch.uint8).pin_memory()
    xd, yd = device(x), torch.zeros(x.nbytes, dtype=torch.uint8, device="cuda")
    kf.kiss_fft_batch(cfg, xp, yp, b)
    kf.kiss_fft_batch(cfg, xd, yd, b)
    assert np.array_equal(yp.numpy(), host(yd))
    cfg.free()


def test_large_real_batches_pipelined(kf):
    import torch
    nfft, b = 4096, 10000
    t = inputs.real((b, nfft), "float", 8)
    fw = kf.kiss_fftr_alloc(nfft, 0, "float")
    iv = kf.kiss_fftr_alloc(nfft, 1, "float")
    nb = nfft // 2 + 1
    fp = torch.zeros(b * nb * 8, dtype=torch.uint8).pin_memory()
    fd = torch.zeros(b * nb * 8, dtype=torch.uint8, device="cuda")
    kf.kiss_fftr_batch(fw, pinned(t), fp, b)
    kf.kiss_fftr_batch(fw, device(t), fd, b)
    assert np.array_equal(fp.numpy(), host(fd))
    rp = torch.zeros(t.nbytes, dtype=torch.uint8).pin_memory()
    rd = torch.zeros(t.nbytes, dtype=torch.uint8, device="cuda")
    kf.kiss_fftri_batch(iv, fp, rp, b)
    kf.kiss_fftri_batch(iv, fd, rd, b)
    assert np.array_equal(rp.numpy(), host(rd))
    fw.free()
    iv.free()
