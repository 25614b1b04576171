"""The batched uneven-mix API (kfg_batch_*) through the C ABI.

Every request of a mix, in every form (run directly, replayed from a CUDA
graph, and the per-call form), is checked against the oracle -- the C
restatement of the reference path -- on its own input: Q15 complex
requests bit for bit against kiss_fft (kiss_fft.c:375-404), float complex
against kiss_fft and an FP64 DFT, float real forward against kiss_fftr
(kiss_fftr.c:63-117) and np.fft.rfft, float real inverse against
kiss_fftri (kiss_fftr.c:119-155) and n * np.fft.irfft, float within
2e-7*log2(N) relative L2.  Each request must also give the same result in
the batch as alone through kfg_exec_batch.  The mixes cover single- and
two-pass complex and real plans, the real inverse, generic radices and
Q15, at arena offsets that are not packed.
"""
import ctypes

import numpy as np
import pytest

import inputs
from oracle import kfo

pytestmark = pytest.mark.gpu

vp, ll, ci = ctypes.c_void_p, ctypes.c_longlong, ctypes.c_int
ESZ = {0: 8, 2: 4}
DTN = {0: "float", 2: "int16_t"}
KIND = {"c2c": 1, "r2c": 2, "c2r": 3}


@pytest.fixture(scope="module")
def core():
    import torch
    if not torch.cuda.is_available():
        pytest.fail("GPU tests need a CUDA device")
    import kissfft_gb300
    L = kissfft_gb300.core()
    L.kfg_batch_create.restype = vp
    L.kfg_batch_add.argtypes = [vp, ci, ci, ci, ll, ll]
    L.kfg_batch_commit.argtypes = [vp, vp, vp, ci]
    for fn in ("kfg_batch_run", "kfg_batch_capture", "kfg_batch_run_percall"):
        getattr(L, fn).argtypes = [vp, vp]
    L.kfg_batch_info.argtypes = [vp, vp, ci]
    L.kfg_batch_free.argtypes = [vp]
    return L


def layout(mix, gap=0):
    """(kind, dtype, n, in_off, out_off, in_bytes, out_bytes) per request."""
    reqs, io, oo = [], 0, 0
    for kind, dt, n in mix:
        esz = ESZ[dt]
        nb = n // 2 + 1
        ib = {1: n * esz, 2: n * esz // 2, 3: nb * esz}[kind]
        ob = {1: n * esz, 2: nb * esz, 3: n * esz // 2}[kind]
        reqs.append((kind, dt, n, io, oo, ib, ob))
        io = (io + ib + gap + 255) // 256 * 256
        oo = (oo + ob + gap + 255) // 256 * 256
    return reqs, io, oo


def request_input(kind, dt, n, seed):
    d = DTN[dt]
    if kind == 2:
        a = inputs.real((n,), d, seed)
    elif kind == 3:
        a = inputs.cpx((n // 2 + 1,), d, seed)
    else:
        a = inputs.cpx((n,), d, seed)
    return np.ascontiguousarray(a).view(np.uint8).ravel()


def oracle_result(kind, dt, n, raw):
    """The oracle's result(s) for one request's input bytes: the bit pattern
    (uint8) for Q15, else the oracle's float result and an FP64 transform."""
    if dt == 2:
        x = raw.view(np.int16).reshape(n, 2)
        return [np.ascontiguousarray(kfo.fft(x, 0, "int16_t")).view(np.uint8).ravel()]
    if kind == 1:
        x = raw.view(np.complex64)
        return [kfo.fft(x, 0, "float").astype(np.complex128), np.fft.fft(x.astype(np.complex128))]
    if kind == 2:
        t = raw.view(np.float32)
        return [kfo.fftr(t, "float").astype(np.complex128), np.fft.rfft(t.astype(np.float64))]
    f = raw.view(np.complex64)
    return [kfo.fftri(f, n, "float").astype(np.float64), n * np.fft.irfft(f.astype(np.complex128), n)]


def run_mix(L, mix, target_threads=256):
    import torch
    reqs, ib_tot, ob_tot = layout(mix, gap=64)
    host = np.zeros(ib_tot, np.uint8)
    for k, (kind, dt, n, io, oo, ib, ob) in enumerate(reqs):
        host[io:io + ib] = request_input(kind, dt, n, 1000 + k)
    ind = torch.from_numpy(host).cuda()
    st = vp(torch.cuda.current_stream().cuda_stream)
    # alone: one kfg_exec_batch per request
    alone = torch.zeros(ob_tot, dtype=torch.uint8, device="cuda")
    for (kind, dt, n, io, oo, ib, ob) in reqs:
        p = L.kfg_plan_c2c(dt, n, 0) if kind == 1 else L.kfg_plan_real(dt, n, 1 if kind == 3 else 0)
        assert p, L.kfg_last_error()
        rc = L.kfg_exec_batch(p, vp(ind.data_ptr() + io), vp(alone.data_ptr() + oo), ll(1), ll(0), ll(0), st)
        assert rc == 0, L.kfg_last_error()
        torch.cuda.synchronize()
        L.kfg_plan_free(p)
    alone_h = alone.cpu().numpy()
    outd = torch.zeros(ob_tot, dtype=torch.uint8, device="cuda")
    B = L.kfg_batch_create()
    try:
        for (kind, dt, n, io, oo, ib, ob) in reqs:
            assert L.kfg_batch_add(B, kind, dt, n, io, oo) == 0
        assert L.kfg_batch_commit(B, vp(ind.data_ptr()), vp(outd.data_ptr()), target_threads) == 0, L.kfg_last_error()
        results = {}
        assert L.kfg_batch_run(B, st) == 0, L.kfg_last_error()
        torch.cuda.synchronize()
        results["direct"] = outd.cpu().numpy()
        outd.zero_()
        assert L.kfg_batch_capture(B, st) == 0, L.kfg_last_error()
        for rep in range(2):
            assert L.kfg_batch_run(B, st) == 0, L.kfg_last_error()
        torch.cuda.synchronize()
        results["graph"] = outd.cpu().numpy()
        outd.zero_()
        assert L.kfg_batch_run_percall(B, st) == 0, L.kfg_last_error()
        torch.cuda.synchronize()
        results["percall"] = outd.cpu().numpy()
    finally:
        L.kfg_batch_free(B)
    oracle = [oracle_result(kind, dt, n, host[io:io + ib]) for (kind, dt, n, io, oo, ib, ob) in reqs]
    for form, got in results.items():
        for k, (kind, dt, n, io, oo, ib, ob) in enumerate(reqs):
            g, a = got[oo:oo + ob], alone_h[oo:oo + ob]
            if dt == 2:
                assert np.array_equal(g, a), (form, k, kind, n)
                assert np.array_equal(g, oracle[k][0]), ("oracle", form, k, kind, n)
            else:
                gv, av = g.view(np.float32), a.view(np.float32)
                tol = 2e-7 * max(1.0, np.log2(n))
                err = np.linalg.norm(gv - av) / max(np.linalg.norm(av), 1e-30)
                assert err <= tol, (form, k, kind, n, err)
                gc = gv.view(np.complex64) if kind != 3 else gv
                for ref in oracle[k]:
                    e2 = np.linalg.norm(gc.astype(ref.dtype) - ref) / max(np.linalg.norm(ref), 1e-30)
                    assert e2 <= tol, ("oracle", form, k, kind, n, e2)
    return results


EDGE = [(1, 0, 480), (1, 0, 1000), (1, 0, 1024), (1, 0, 3003), (1, 0, 65536), (1, 0, 17), (1, 0, 1), (1, 0, 2),
        (2, 0, 2), (2, 0, 512), (2, 0, 2000), (2, 0, 131072), (2, 0, 34034), (3, 0, 1024), (3, 0, 131072),
        (1, 2, 480), (1, 2, 4099), (1, 2, 65536), (1, 2, 1), (1, 0, 480), (2, 0, 512), (1, 2, 480), (1, 0, 961)]


def test_edge_mix(core):
    run_mix(core, EDGE)


def test_edge_mix_wide_tiles(core):
    run_mix(core, EDGE, target_threads=512)


def test_uneven_mix(core):
    mix = [(KIND[k], 0 if d == "float" else 2, n) for k, d, n in inputs.uneven_mix(600, seed=3)]
    run_mix(core, mix)


def test_batch_info_and_errors(core):
    L = core
    B = L.kfg_batch_create()
    try:
        assert L.kfg_batch_add(B, 2, 0, 1001, 0, 0) == -1  # odd real length (kiss_fftr.c:29-32)
        assert L.kfg_batch_add(B, 9, 0, 64, 0, 0) == -1
        assert L.kfg_batch_run(B, None) == -1  # not committed
        for k in range(5):
            assert L.kfg_batch_add(B, 1, 0, 64, 512 * k, 512 * k) == 0
        import torch
        a = torch.zeros(4096, dtype=torch.uint8, device="cuda")
        assert L.kfg_batch_commit(B, vp(a.data_ptr()), vp(a.data_ptr() + 2048 * 0), 0) == 0
        info = (ctypes.c_longlong * 5)()
        assert L.kfg_batch_info(B, info, 5) == 0
        assert info[0] == 5 and info[2] >= 1 and info[3] >= 1
        assert info[4] == 0  # 64-point requests fit one shared tile: no intermediate traffic
    finally:
        L.kfg_batch_free(B)
    # one 65536-point float request runs two passes through an intermediate
    # of 65536 complex floats: written once, read once
    B = L.kfg_batch_create()
    try:
        n = 65536
        assert L.kfg_batch_add(B, 1, 0, n, 0, 0) == 0
        a = torch.zeros(n * 8, dtype=torch.uint8, device="cuda")
        c = torch.zeros(n * 8, dtype=torch.uint8, device="cuda")
        assert L.kfg_batch_commit(B, vp(a.data_ptr()), vp(c.data_ptr()), 0) == 0
        info = (ctypes.c_longlong * 5)()
        assert L.kfg_batch_info(B, info, 5) == 0
        assert info[4] == 2 * n * 8
    finally:
        L.kfg_batch_free(B)
