"""The serving loop (kfg_server_*) through the C ABI.

Requests of every kind (c2c float and Q15, real forward and inverse, 2-D,
fast FIR), with device, pinned-host and ordinary host buffers, are submitted
from several threads at once.  Each served result is checked against the
oracle (the C restatement of the reference path) on its own input --
kiss_fft (kiss_fft.c:375-404) with Q15 bit for bit, kiss_fftr / kiss_fftri
(kiss_fftr.c:63-155), kiss_fftnd (kiss_fftnd.c:156-188), and for the fast
FIR np.convolve within 4x the error of the reference's own overlap-scrap
filter (tools/kiss_fastfir.c:167-239) -- float within 2e-7*log2(N) relative
L2 (2-D: N = rows*cols).  It must also equal the same request run alone
through the plain API (the same tolerances; fast FIR 1e-6 relative).  A
budget smaller than the mix forces requests to queue for admission; a
request larger than the whole budget fails on its own without disturbing
the others.
"""
import threading

import numpy as np
import pytest

import inputs
from oracle import kfo

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def kf():
    import torch
    if not torch.cuda.is_available():
        pytest.fail("GPU tests need a CUDA device")
    import kissfft_gb300
    return kissfft_gb300


def pinned_like(a):
    import torch
    t = torch.empty(a.nbytes, dtype=torch.uint8).pin_memory()
    v = t.numpy().view(a.dtype).reshape(a.shape)
    v[...] = a
    return t, v


def make_requests(kf, seed):
    rng = np.random.default_rng(seed)
    reqs = []
    k = 0
    for n in (480, 1000, 1024, 3003, 65536, 17):
        reqs.append(("c2c", "float", n, inputs.cpx((n,), "float", seed + k)))
        k += 1
    for n in (480, 1024, 4099):
        reqs.append(("c2c", "int16_t", n, inputs.cpx((n,), "int16_t", seed + k)))
        k += 1
    for n in (512, 4096, 131072):
        reqs.append(("r2c", "float", n, inputs.real((n,), "float", seed + k)))
        k += 1
    for n in (1024, 6006):
        reqs.append(("c2r", "float", n, inputs.cpx((n // 2 + 1,), "float", seed + k)))
        k += 1
    for shape in ((64, 48), (256, 256)):
        reqs.append(("2d", "float", shape, inputs.cpx(shape, "float", seed + k)))
        k += 1
    for L, ns in ((255, 50000), (1000, 20000)):
        h = rng.standard_normal(L).astype(np.float32)
        x = rng.standard_normal(ns).astype(np.float32)
        reqs.append(("fir", "float", (h, ns), x))
    return reqs


def alone(kf, kind, dt, n, x):
    if kind == "c2c":
        cfg = kf.kiss_fft_alloc(n, 0, dt)
        y = np.zeros_like(x)
        kf.kiss_fft(cfg, x, y)
    elif kind == "r2c":
        cfg = kf.kiss_fftr_alloc(n, 0, dt)
        y = np.zeros(n // 2 + 1, np.complex64)
        kf.kiss_fftr(cfg, x, y)
    elif kind == "c2r":
        cfg = kf.kiss_fftr_alloc(n, 1, dt)
        y = np.zeros(n, np.float32)
        kf.kiss_fftri(cfg, x, y)
    elif kind == "2d":
        cfg = kf.kiss_fftnd_alloc(list(n), 0, dt)
        y = np.zeros_like(x)
        kf.kiss_fftnd(cfg, x, y)
    else:
        h, ns = n
        cfg = kf.kiss_fastfir_alloc(h)
        y = np.zeros(ns - h.size + 1, np.float32)
        kf.kiss_fastfir_filter(cfg, x, y)
    cfg.free()
    return y


def out_like(kind, n, x):
    if kind == "r2c":
        return np.zeros(n // 2 + 1, np.complex64)
    if kind == "c2r":
        return np.zeros(n, np.float32)
    if kind == "fir":
        h, ns = n
        return np.zeros(ns - h.size + 1, np.float32)
    return np.zeros_like(x)


def submit(kf, srv, kind, dt, n, x, y):
    K = {"c2c": kf.SERVE_C2C, "r2c": kf.SERVE_R2C, "c2r": kf.SERVE_C2R, "2d": kf.SERVE_C2C_2D, "fir": kf.SERVE_FIR}
    if kind == "2d":
        return srv.submit(K[kind], x, y, n[0], n[1], dtype=dt)
    if kind == "fir":
        h, ns = n
        return srv.submit(K[kind], x, y, h.size, dtype=dt, taps=h, length=ns)
    return srv.submit(K[kind], x, y, n, dtype=dt)


def close(kind, dt, n, got, ref):
    if dt == "int16_t":
        return np.array_equal(got, ref)
    if kind == "fir":
        tol = 1e-6
    else:
        N = n[0] * n[1] if kind == "2d" else n
        tol = 2e-7 * max(1.0, np.log2(N))
    g = np.asarray(got).astype(np.complex128 if np.iscomplexobj(got) else np.float64)
    r = np.asarray(ref).astype(g.dtype)
    return np.linalg.norm(g - r) <= tol * max(np.linalg.norm(r), 1e-30)


def relerr(got, ref):
    g = np.asarray(got).astype(np.complex128 if np.iscomplexobj(got) or np.iscomplexobj(ref) else np.float64)
    r = np.asarray(ref).astype(g.dtype)
    return float(np.linalg.norm(g - r) / max(np.linalg.norm(r), 1e-30))


def oracle_ok(kind, dt, n, x, got):
    """The served result against the oracle on the same input."""
    if kind == "fir":
        h, ns = n
        exact = np.convolve(x.astype(np.float64), h.astype(np.float64), "valid")
        ref_err = relerr(kfo.fastfir(h, x), exact)  # the reference's own overlap-scrap error
        return relerr(got, exact) <= max(4 * ref_err, 1e-6)
    if kind == "c2c":
        ref = kfo.fft(x, 0, dt)
        if dt == "int16_t":
            return np.array_equal(got, ref)
        exact = np.fft.fft(x.astype(np.complex128))
    elif kind == "r2c":
        ref, exact = kfo.fftr(x, dt), np.fft.rfft(x.astype(np.float64))
    elif kind == "c2r":
        ref, exact = kfo.fftri(x, n, dt), n * np.fft.irfft(x.astype(np.complex128), n)
    else:
        ref, exact = kfo.fftnd(x, list(n), 0, dt), np.fft.fft2(x.astype(np.complex128))
    N = n[0] * n[1] if kind == "2d" else n
    tol = 2e-7 * max(1.0, np.log2(N))
    return relerr(got, ref) <= tol and relerr(got, exact) <= tol


def test_mix_from_threads_matches_alone(kf):
    import torch
    reqs = make_requests(kf, 40)
    refs = [alone(kf, *r) for r in reqs]
    srv = kf.Server(hbm_budget=512 << 20, slots=4)
    try:
        bufs = []
        for i, (kind, dt, n, x) in enumerate(reqs):
            mode = i % 3  # 0 pageable numpy, 1 pinned host, 2 device
            y0 = out_like(kind, n, x)
            if mode == 0:
                bufs.append((x.copy(), y0, None))
            elif mode == 1:
                tx, vx = pinned_like(x)
                ty, vy = pinned_like(y0)
                bufs.append((vx, vy, (tx, ty)))
            else:
                xd = torch.from_numpy(np.ascontiguousarray(x).view(np.uint8).copy()).cuda()
                yd = torch.zeros(y0.nbytes, dtype=torch.uint8, device="cuda")
                bufs.append((xd, yd, None))
        ids = [None] * len(reqs)

        def worker(part):
            for i in part:
                kind, dt, n, _ = reqs[i]
                ids[i] = submit(kf, srv, kind, dt, n, bufs[i][0], bufs[i][1])

        th = [threading.Thread(target=worker, args=(list(range(t, len(reqs), 4)),)) for t in range(4)]
        for t in th:
            t.start()
        for t in th:
            t.join()
        for i in range(len(reqs)):
            lat = srv.wait(ids[i], timeout=60.0)
            assert lat is not None and lat > 0
        for i, (kind, dt, n, x) in enumerate(reqs):
            y = bufs[i][1]
            if hasattr(y, "is_cuda"):
                torch.cuda.synchronize()
                y = y.cpu().numpy().view(refs[i].dtype).reshape(refs[i].shape)
            assert close(kind, dt, n, y, refs[i]), (i, kind, dt, n)
            assert oracle_ok(kind, dt, n, x, y), ("oracle", i, kind, dt, n)
        st = srv.stats()
        assert st["completed"] == len(reqs) and st["failed"] == 0
        assert 0 < st["p50_s"] <= st["p99_s"] <= st["max_s"]
    finally:
        srv.close()


def test_admission_under_a_small_budget(kf):
    """64 requests of 1 MiB device footprint under a 4 MiB budget: they queue,
    the budget is never exceeded, all complete correctly; a request larger
    than the budget fails alone."""
    n = 65536  # 512 KiB in + 512 KiB out (+ two-pass scratch)
    srv = kf.Server(hbm_budget=4 << 20, slots=2)
    try:
        xs = [inputs.cpx((n,), "float", 500 + i) for i in range(64)]
        ys = [np.zeros_like(x) for x in xs]
        ids = [srv.submit(kf.SERVE_C2C, x, y, n) for x, y in zip(xs, ys)]
        big_in = inputs.cpx((1 << 20,), "float", 7)
        big_out = np.zeros_like(big_in)
        big = srv.submit(kf.SERVE_C2C, big_in, big_out, 1 << 20)
        with pytest.raises(kf.KissFFTError):
            srv.wait(big, timeout=60.0)
        for rid in ids:
            assert srv.wait(rid, timeout=60.0) is not None
        ref = alone(kf, "c2c", "float", n, xs[5])
        assert close("c2c", "float", n, ys[5], ref)
        for k in range(0, 64, 9):
            assert oracle_ok("c2c", "float", n, xs[k], ys[k]), k
        st = srv.stats()
        assert st["completed"] == 64 and st["failed"] == 1
        assert st["peak_hbm_bytes"] <= 4 << 20
        assert st["batches"] >= 8  # at most 2-3 requests fit per batch
    finally:
        srv.close()


def test_plan_cache_evicts_under_the_budget(kf):
    """Ten plan sizes cycled through a 2 MiB budget: plans (about 0.4 MiB
    each) are evicted least recently used first, never while a request holds
    them, and every result stays right."""
    sizes = [16384, 15625, 16200, 15552, 16000, 15360, 14580, 14400, 13824, 13500]
    srv = kf.Server(hbm_budget=2 << 20, slots=2)
    try:
        xs, ys, ids = [], [], []
        for k in range(30):
            n = sizes[k % len(sizes)]
            x = inputs.cpx((n,), "float", 900 + k)
            y = np.zeros_like(x)
            xs.append(x)
            ys.append(y)
            ids.append(srv.submit(kf.SERVE_C2C, x, y, n))
        for rid in ids:
            assert srv.wait(rid, timeout=60.0) is not None
        for k in (0, 13, 29):
            n = sizes[k % len(sizes)]
            assert close("c2c", "float", n, ys[k], alone(kf, "c2c", "float", n, xs[k]))
            assert oracle_ok("c2c", "float", n, xs[k], ys[k]), k
        st = srv.stats()
        assert st["completed"] == 30 and st["failed"] == 0
        assert st["evictions"] > 0
        assert st["peak_hbm_bytes"] <= 2 << 20
        assert st["plan_bytes"] <= 2 << 20
    finally:
        srv.close()


def test_loadtest_runs(kf):
    """A short Poisson load (2,000 req/s for 0.5 s) completes every request."""
    srv = kf.Server()
    try:
        r = srv.loadtest(rate=2000.0, seconds=0.5, percall_max=50, fir_len_max=1 << 18, d2_max=512,
                         in_pool_mb=64, out_pool_mb=256)
        assert r["offered"] > 500
        assert r["served"]["completed"] == r["offered"] and r["served"]["failed"] == 0
        assert r["percall_count"] == 50
        assert r["served"]["p50_s"] > 0
    finally:
        srv.close()
