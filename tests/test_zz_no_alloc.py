"""kfg_exec_batch_noalloc through the C ABI against kfg_exec_batch.

The no-alloc entry point serves callers that may not allocate device memory
while they transform (code inside an allocator hook, fixed-memory real-time
loops): it runs complex 1-D batches with the scratch of two-pass plans in a
fixed device array instead of a stream-ordered allocation.  Its results
must match kfg_exec_batch on the same inputs (float within 2e-7*log2(N)
relative L2 per transform, Q15 bit for bit), and the oracle (Q15 bit for
bit against kiss_fft, kiss_fft.c:375-404; float against an FP64 DFT), on
two calls in a row (the second call finds the first call's data in the
shared array), in place, with row distances that are not packed, and again
after a device reset (a new CUDA context, where the array has to be looked
up again).  Batches whose scratch exceeds the array are refused before
anything is launched.
"""
import ctypes
import os
import subprocess
import sys
import textwrap

import numpy as np
import pytest

import inputs
from oracle import kfo
from gpu_util import bound, c128, empty_dev, from_dev, relerr_rows, to_dev

pytestmark = pytest.mark.gpu

vp, ll = ctypes.c_void_p, ctypes.c_longlong
DT = {"float": 0, "int16_t": 2}
SCRATCH_BYTES = 64 << 20


@pytest.fixture(scope="module")
def core():
    import torch
    if not torch.cuda.is_available():
        pytest.fail("GPU tests need a CUDA device")
    import kissfft_gb300
    L = kissfft_gb300.core()
    L.kfg_exec_batch_noalloc.argtypes = [vp, vp, vp, ll, ll, ll, vp]
    return L


def stream():
    import torch
    return vp(torch.cuda.current_stream().cuda_stream)


def run(L, fn, plan, x, batch):
    xd = to_dev(x)
    yd = empty_dev(x)
    rc = fn(plan, vp(xd.data_ptr()), vp(yd.data_ptr()), ll(batch), ll(0), ll(0), stream())
    assert rc == 0, L.kfg_last_error().decode()
    return from_dev(yd, x)


@pytest.mark.parametrize("dtype,n,batch", [("float", 65536, 8), ("int16_t", 65536, 4), ("float", 1000, 64),
                                           ("float", 131072, 3)])
def test_matches_exec_batch_twice(core, dtype, n, batch):
    L = core
    plan = L.kfg_plan_c2c(DT[dtype], n, 0)
    assert plan, L.kfg_last_error().decode()
    try:
        info = (ctypes.c_int * 6)()
        L.kfg_plan_info(plan, info, 6)
        if n >= 65536:
            assert info[3] == 2  # two HBM passes: the scratch is used
        for call in range(2):
            x = inputs.cpx((batch, n), dtype, 100 * n + call)
            got = run(L, L.kfg_exec_batch_noalloc, plan, x, batch)
            ref = run(L, L.kfg_exec_batch, plan, x, batch)
            if dtype == "int16_t":
                assert np.array_equal(got, ref), (n, call)
                assert np.array_equal(got, kfo.fft(x, 0, "int16_t")), ("oracle", n, call)
            else:
                err = relerr_rows(c128(got, dtype), c128(ref, dtype))
                assert err <= bound(dtype, n), (n, call, err)
                exact = np.fft.fft(c128(x, dtype), axis=-1)
                assert relerr_rows(c128(got, dtype), exact) <= bound(dtype, n)
    finally:
        L.kfg_plan_free(plan)


@pytest.mark.parametrize("dtype", ["float", "int16_t"])
def test_in_place_and_strided_rows(core, dtype):
    """A two-pass size in place (in == out) and with row distances larger
    than nfft on both sides; the gaps between rows stay untouched."""
    import torch
    L = core
    n, batch = 65536, 3
    plan = L.kfg_plan_c2c(DT[dtype], n, 0)
    assert plan, L.kfg_last_error().decode()
    try:
        x = inputs.cpx((batch, n), dtype, 4242)
        exact = kfo.fft(x, 0, dtype)
        # in place: noalloc twice in a row on fresh copies, against kfg_exec_batch in place
        outs = []
        for fn in (L.kfg_exec_batch_noalloc, L.kfg_exec_batch_noalloc, L.kfg_exec_batch):
            xd = to_dev(x)
            rc = fn(plan, vp(xd.data_ptr()), vp(xd.data_ptr()), ll(batch), ll(0), ll(0), stream())
            assert rc == 0, L.kfg_last_error().decode()
            outs.append(from_dev(xd, x))
        # strided rows: in_dist = n + 64, out_dist = n + 160 complex elements
        di, do = n + 64, n + 160
        xs = np.zeros((batch, di) + x.shape[2:], x.dtype)
        xs[:, :n] = x
        for fn in (L.kfg_exec_batch_noalloc, L.kfg_exec_batch):
            xd = to_dev(xs)
            y0 = np.zeros((batch, do) + x.shape[2:], x.dtype)
            yd = to_dev(y0)
            rc = fn(plan, vp(xd.data_ptr()), vp(yd.data_ptr()), ll(batch), ll(di), ll(do), stream())
            assert rc == 0, L.kfg_last_error().decode()
            y = from_dev(yd, y0)
            assert not np.any(y[:, n:]), "a gap between output rows was written"
            outs.append(np.ascontiguousarray(y[:, :n]))
        for k, got in enumerate(outs):
            if dtype == "int16_t":
                assert np.array_equal(got, exact), k
            else:
                assert relerr_rows(c128(got, dtype), c128(exact, dtype)) <= bound(dtype, n), k
                assert relerr_rows(c128(got, dtype), np.fft.fft(c128(x, dtype), axis=-1)) <= bound(dtype, n), k
    finally:
        L.kfg_plan_free(plan)


# Run in a child process without torch: allocate with the CUDA runtime the
# library itself uses, compare noalloc with kfg_exec_batch, reset the device
# (this process's own context only), and compare again with a new plan.
_RESET_CHILD = textwrap.dedent("""
    import ctypes, sys
    import numpy as np
    sys.path.insert(0, sys.argv[1])
    import kissfft_gb300
    L = kissfft_gb300.core()
    vp, ll = ctypes.c_void_p, ctypes.c_longlong
    L.kfg_exec_batch_noalloc.argtypes = [vp, vp, vp, ll, ll, ll, vp]
    rt = ctypes.CDLL("libcudart.so.13")
    n, batch = 65536, 4
    rng = np.random.default_rng(77)
    def once(tag):
        x = (rng.uniform(-1, 1, (batch, n)) + 1j * rng.uniform(-1, 1, (batch, n))).astype(np.complex64)
        plan = L.kfg_plan_c2c(0, n, 0)
        assert plan, (tag, L.kfg_last_error())
        bufs = [ctypes.c_void_p() for _ in range(4)]
        for b in bufs:
            assert rt.cudaMalloc(ctypes.byref(b), ctypes.c_size_t(x.nbytes)) == 0, tag
        assert rt.cudaMemcpy(bufs[0], x.ctypes.data_as(vp), ctypes.c_size_t(x.nbytes), 1) == 0, tag
        # two no-alloc calls in a row, then the allocating entry point
        for k, fn in ((1, L.kfg_exec_batch_noalloc), (2, L.kfg_exec_batch_noalloc), (3, L.kfg_exec_batch)):
            rc = fn(plan, bufs[0], bufs[k], ll(batch), ll(0), ll(0), None)
            assert rc == 0, (tag, L.kfg_last_error())
        assert rt.cudaDeviceSynchronize() == 0, tag
        ys = []
        for k in (1, 2, 3):
            y = np.empty_like(x)
            assert rt.cudaMemcpy(y.ctypes.data_as(vp), bufs[k], ctypes.c_size_t(x.nbytes), 2) == 0, tag
            ys.append(y.astype(np.complex128))
        exact = np.fft.fft(x.astype(np.complex128), axis=-1)
        tol = 2e-7 * np.log2(n)
        for y in ys:
            err = np.max(np.linalg.norm(y - exact, axis=1) / np.linalg.norm(exact, axis=1))
            assert err <= tol, (tag, err)
        for y in ys[:2]:
            err = np.max(np.linalg.norm(y - ys[2], axis=1) / np.linalg.norm(ys[2], axis=1))
            assert err <= tol, (tag, "vs kfg_exec_batch", err)
        for b in bufs:
            rt.cudaFree(b)
        L.kfg_plan_free(plan)
    once("before reset")
    assert rt.cudaDeviceReset() == 0
    once("after reset")
    print("reset ok")
""")


def test_after_device_reset_in_a_fresh_process():
    """Two no-alloc calls in a row and kfg_exec_batch agree with each other
    and with an FP64 DFT before and after cudaDeviceReset: the array's
    address is looked up again in the new context."""
    import torch
    if not torch.cuda.is_available():
        pytest.fail("GPU tests need a CUDA device")
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    env = dict(os.environ)
    r = subprocess.run([sys.executable, "-c", _RESET_CHILD, root], capture_output=True, text=True, timeout=300,
                       env=env)
    assert r.returncode == 0 and "reset ok" in r.stdout, r.stdout + r.stderr


def test_refuses_batches_beyond_the_array(core):
    import torch
    L = core
    n = 65536
    plan = L.kfg_plan_c2c(0, n, 0)
    assert plan
    try:
        batch = SCRATCH_BYTES // (n * 8) + 1  # one transform more than fits
        xd = torch.zeros((batch, 2 * n), dtype=torch.float32, device="cuda")
        yd = torch.zeros_like(xd)
        rc = L.kfg_exec_batch_noalloc(plan, vp(xd.data_ptr()), vp(yd.data_ptr()), ll(batch), ll(0), ll(0), stream())
        assert rc == -1
        assert b"scratch" in L.kfg_last_error()
        # exactly the array's size is accepted
        rc = L.kfg_exec_batch_noalloc(plan, vp(xd.data_ptr()), vp(yd.data_ptr()), ll(batch - 1), ll(0), ll(0),
                                      stream())
        assert rc == 0, L.kfg_last_error().decode()
        torch.cuda.synchronize()
    finally:
        L.kfg_plan_free(plan)


def test_refuses_host_pointers_and_other_plans(core):
    L = core
    x = inputs.cpx((1, 1024), "float", 1)
    y = np.zeros_like(x)
    plan = L.kfg_plan_c2c(0, 1024, 0)
    try:
        assert L.kfg_exec_batch_noalloc(plan, vp(x.ctypes.data), vp(y.ctypes.data), ll(1), ll(0), ll(0), None) == -1
    finally:
        L.kfg_plan_free(plan)
    rplan = L.kfg_plan_real(0, 1024, 0)
    try:
        xd = to_dev(inputs.real((1, 1024), "float", 2))
        yd = empty_dev(np.zeros((1, 513), np.complex64))
        assert L.kfg_exec_batch_noalloc(rplan, vp(xd.data_ptr()), vp(yd.data_ptr()), ll(1), ll(0), ll(0), None) == -1
    finally:
        L.kfg_plan_free(rplan)
