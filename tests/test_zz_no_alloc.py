"""kfg_exec_batch_noalloc through the C ABI against kfg_exec_batch.

The no-alloc entry point runs complex 1-D batches with the scratch of
two-pass plans in a fixed device array instead of a stream-ordered
allocation.  Its results must match kfg_exec_batch on the same inputs
(float within 2e-7*log2(N) relative L2 per transform, Q15 bit for bit),
on two calls in a row (the second call finds the first call's data in the
shared array), and batches whose scratch exceeds the array are refused
before anything is launched.
"""
import ctypes

import numpy as np
import pytest

import inputs
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
            else:
                err = relerr_rows(c128(got, dtype), c128(ref, dtype))
                assert err <= bound(dtype, n), (n, call, err)
                exact = np.fft.fft(c128(x, dtype), axis=-1)
                assert relerr_rows(c128(got, dtype), exact) <= bound(dtype, n)
    finally:
        L.kfg_plan_free(plan)


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
