"""The C ABI without a GPU: the built libraries load, export every function
include/*.h declares, fail loudly (no CPU fallback) when no GPU is present,
and the run-time specialisation compiles its kernels from the embedded
sources (NVRTC needs no GPU)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INC = os.path.join(ROOT, "include")


@pytest.fixture(scope="module")
def libs():
    from kissfft_gb300 import build
    if not os.path.exists(build.core_lib()) or any(not os.path.exists(build.dropin_lib(d)) for d in build.DTYPES):
        build.build()
    core = ctypes.CDLL(build.core_lib(), mode=ctypes.RTLD_GLOBAL)
    drop = {d: ctypes.CDLL(build.dropin_lib(d)) for d in build.DTYPES}
    return core, drop


def declared(header):
    txt = open(os.path.join(INC, header)).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    names = re.findall(r"\b(k(?:iss|fg|fc)_[a-z0-9_]+)\s*\(", txt)
    return sorted(set(names))


def test_core_exports(libs):
    core, _ = libs
    names = declared("kissfft_gb300.h")
    assert len(names) >= 15
    for n in names:
        assert hasattr(core, n), n


def test_dropin_exports(libs):
    _, drop = libs
    names = declared("kiss_fft_cuda.h")
    assert "kiss_fft_cuda_alloc" in names and "kiss_fftndri_cuda" in names and "kiss_fastfir_cuda" in names
    assert "kfc_cuda_fft" in names and "kfc_cuda_cleanup" in names
    for d, L in drop.items():
        for n in names:
            assert hasattr(L, n), (d, n)


def test_no_cpu_fallback_without_gpu(libs):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    core, drop = libs
    L = drop["float"]
    L.kiss_fft_cuda_alloc.restype = ctypes.c_void_p
    assert not L.kiss_fft_cuda_alloc(1024, 0, None, None)   # NULL like a failed kiss_fft_alloc
    assert L.kiss_fft_cuda_status() != 0


def test_kfc_fails_loudly_without_gpu(libs):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    import numpy as np
    _, drop = libs
    L = drop["float"]
    x = np.zeros(512, np.complex64)
    y = np.zeros(512, np.complex64)
    L.kfc_cuda_fft(512, x.ctypes.data_as(ctypes.c_void_p), y.ctypes.data_as(ctypes.c_void_p))
    assert L.kiss_fft_cuda_status() != 0   # no plan, no CPU fallback
    assert L.kfc_cuda_ncached() == 0
    L.kfc_cuda_cleanup()


def test_reference_size_rules(libs):
    core, drop = libs
    L = drop["float"]
    L.kiss_fftr_cuda_alloc.restype = ctypes.c_void_p
    assert not L.kiss_fftr_cuda_alloc(1001, 0, None, None)  # odd real size (kiss_fftr.c:29-32)
    assert core.kfg_next_fast_size(1001) == 1024
    assert core.kfg_next_fast_size(7) == 8
    drop["int16_t"].kiss_fastfir_cuda_alloc.restype = ctypes.c_void_p
    import numpy as np
    h = np.ones(16, np.int16)
    assert not drop["int16_t"].kiss_fastfir_cuda_alloc(h.ctypes.data, 16, None, None, None)


@pytest.mark.parametrize("dt,real,n", [(0, 0, 1024), (0, 0, 1000), (2, 0, 3003), (0, 1, 4096), (3, 0, 65536),
                                       (1, 0, 480), (0, 0, 4099), (2, 1, 6006)])
def test_specialised_kernels_compile(libs, dt, real, n):
    core, _ = libs
    core.kfg_last_error.restype = ctypes.c_char_p
    rc = core.kfg_specialize_check(dt, real, n, 0, ctypes.c_longlong(4096))
    assert rc == 0, core.kfg_last_error().decode()


def test_every_kernel_part_linked(libs):
    """The per-(type, family, mode) kernel units all reach the core library:
    every launcher the mode dispatchers call is defined there, and nothing of
    the library's own namespace is left undefined for the loader."""
    import shutil
    import subprocess
    from kissfft_gb300 import build
    if not shutil.which("nm"):
        pytest.skip("nm not available")
    out = subprocess.run(["nm", "-C", build.core_lib()], capture_output=True, text=True, check=True).stdout
    defined = set(re.findall(r"^\S+ [Tt] kf::(launch_(?:engine|multi)_dt\d_fam\d_m\d)\(", out, flags=re.M))
    want = set()
    for dt, fam, mode in build.INST_PARTS:
        want.add("launch_engine_dt%d_fam%d_m%d" % (dt, fam, mode))
        if mode < 3:
            want.add("launch_multi_dt%d_fam%d_m%d" % (dt, fam, mode))
    assert want <= defined, sorted(want - defined)
    assert len(build.INST_PARTS) == 4 * 3 * 3 + 2   # every type, family and mode, plus the float fast-FIR parts
    undef = subprocess.run(["nm", "-C", "-u", build.core_lib()], capture_output=True, text=True, check=True).stdout
    assert "kf::" not in undef


def test_mem_lenmem_protocol(libs):
    """The placement protocol of kiss_fft_alloc (reference kiss_fft.h:94-115,
    kiss_fft.c:349-355) on every alloc of every sample type: with mem NULL
    the call returns NULL and writes the size it needs to *lenmem; a buffer
    one byte short is refused the same way.  (Placing the cfg in a large
    enough buffer needs a GPU: tests/test_gpu_parity.py.)"""
    import numpy as np
    _, drop = libs
    dims = (ctypes.c_int * 2)(8, 6)
    taps = np.ones(31, np.float32)
    for dt, L in drop.items():
        calls = {
            "kiss_fft_cuda_alloc": lambda m, ln: L.kiss_fft_cuda_alloc(480, 0, m, ln),
            "kiss_fftr_cuda_alloc": lambda m, ln: L.kiss_fftr_cuda_alloc(480, 0, m, ln),
            "kiss_fftnd_cuda_alloc": lambda m, ln: L.kiss_fftnd_cuda_alloc(dims, 2, 0, m, ln),
            "kiss_fftndr_cuda_alloc": lambda m, ln: L.kiss_fftndr_cuda_alloc(dims, 2, 0, m, ln),
        }
        if dt == "float":
            calls["kiss_fastfir_cuda_alloc"] = lambda m, ln: L.kiss_fastfir_cuda_alloc(
                taps.ctypes.data_as(ctypes.c_void_p), 31, None, m, ln)
        sizes = set()
        for name, call in calls.items():
            getattr(L, name).restype = ctypes.c_void_p
            need = ctypes.c_size_t(0)
            assert not call(None, ctypes.byref(need)), (dt, name)
            assert need.value > 0, (dt, name)
            sizes.add(need.value)
            short = ctypes.create_string_buffer(need.value - 1)
            got = ctypes.c_size_t(need.value - 1)
            assert not call(short, ctypes.byref(got)), (dt, name)
            assert got.value == need.value, (dt, name)
        assert len(sizes) == 1  # one host handle layout for every kind
