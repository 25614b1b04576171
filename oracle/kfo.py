"""numpy front end of the C oracle (oracle/kfo.c) -- test infrastructure only.

Sample types follow the reference's compile-time choice of
``kiss_fft_scalar`` (reference kiss_fft.h:73-85): ``"float"``, ``"double"``,
``"int16_t"`` (Q15) and ``"int32_t"`` (Q31).  Complex arrays are numpy
complex64/complex128 for the IEEE types and ``(..., 2)`` integer arrays for
the fixed-point ones (interleaved re/im, reference kiss_fft.h:87-90).
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libkfo.so")

SFX = {"float": "f32", "double": "f64", "int16_t": "q15", "int32_t": "q31"}
SCALAR = {"float": np.float32, "double": np.float64, "int16_t": np.int16, "int32_t": np.int32}
CPLX = {"float": np.complex64, "double": np.complex128}

# the CHECK_OVERFLOW build (-DKFO_CHECK_OVERFLOW): same results, and it
# counts the fixed-point overflows the reference's CHECK_OVERFLOW warns about
LIB_OVF_PATH = os.path.join(HERE, "_build", "libkfo_ovf.so")

# the same restatement compiled at the reference's release flags
# (-O3 -ffast-math -fomit-frame-pointer, CMakeLists.txt:98-102): used only to
# time the CPU baseline, never as the checker
LIB_REL_PATH = os.path.join(HERE, "_build", "libkfo_rel.so")

_lib = None
_lib_ovf = None
_lib_rel = None
_override = None  # set by overflows() while it runs


def build():
    """Compile the oracle libraries with their Makefile (gcc)."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)


def _load(path):
    if not os.path.exists(path):
        build()
    L = ctypes.CDLL(path)
    L.kfo_fastfir_f32.restype = ctypes.c_long
    L.kfo_direct_fir_f32.restype = ctypes.c_long
    L.kfo_fastfir_nfft.restype = ctypes.c_long
    L.kfo_overflows_take.restype = ctypes.c_long
    for s in SFX.values():
        getattr(L, "kfo_fftr_batch_" + s).restype = ctypes.c_int
    return L


def lib():
    global _lib
    if _override is not None:
        return _override
    if _lib is None:
        _lib = _load(LIB_PATH)
    return _lib


def lib_ovf():
    global _lib_ovf
    if _lib_ovf is None:
        _lib_ovf = _load(LIB_OVF_PATH)
    return _lib_ovf


def lib_rel():
    global _lib_rel
    if _lib_rel is None:
        _lib_rel = _load(LIB_REL_PATH)
    return _lib_rel


def overflows(fn, *args, **kwargs):
    """Run ``fn`` (fft, fftr, fftri, fftnd, ...) of this module on the
    CHECK_OVERFLOW build of the oracle; returns (result, overflow count).

    The count is the number of warnings the reference built with
    -DCHECK_OVERFLOW prints (_kiss_fft_guts.h:57-61): one per component of a
    C_ADD / C_SUB / C_ADDTO / C_SUBFROM whose exact sum leaves
    [SAMP_MIN, SAMP_MAX], plus kiss_fftr's two DC checks (kiss_fftr.c:94-95).
    Float and double never count (the reference checks fixed point only)."""
    global _override
    L = lib_ovf()
    L.kfo_overflows_take()
    _override = L
    try:
        out = fn(*args, **kwargs)
    finally:
        _override = None
    return out, int(L.kfo_overflows_take())


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def is_fixed(dtype):
    return dtype in ("int16_t", "int32_t")


def empty_cpx(shape, dtype):
    if is_fixed(dtype):
        return np.zeros(tuple(shape) + (2,), SCALAR[dtype])
    return np.zeros(tuple(shape), CPLX[dtype])


def as_cpx(x, dtype):
    """Contiguous complex array in the oracle's layout for ``dtype``."""
    if is_fixed(dtype):
        x = np.ascontiguousarray(x, dtype=SCALAR[dtype])
        assert x.shape[-1] == 2
        return x
    return np.ascontiguousarray(x, dtype=CPLX[dtype])


def factor(n):
    """kf_factor's radix list (reference kiss_fft.c:306-328)."""
    fac = (ctypes.c_int * 64)()
    k = lib().kfo_factor(int(n), fac)
    return [fac[2 * i] for i in range(k)]


def next_fast_size(n):
    return lib().kfo_next_fast_size(int(n))


def max_threads():
    return lib().kfo_max_threads()


def twiddles(nfft, inverse, dtype):
    out = empty_cpx((nfft,), dtype)
    getattr(lib(), "kfo_twiddles_" + SFX[dtype])(int(nfft), int(inverse), _p(out))
    return out


def super_twiddles(nfft, inverse, dtype):
    """Super twiddles of a real plan of size nfft (ncfft = nfft/2)."""
    ncfft = nfft // 2
    out = empty_cpx((ncfft // 2,), dtype)
    getattr(lib(), "kfo_super_twiddles_" + SFX[dtype])(int(ncfft), int(inverse), _p(out))
    return out


def fft(x, inverse=False, dtype="float", nthreads=1, release=False):
    """Batched complex transform along the last (complex) axis.  release=True
    runs the release-flags build (timing only)."""
    x = as_cpx(x, dtype)
    n = x.shape[-2] if is_fixed(dtype) else x.shape[-1]
    batch = x.size // (2 * n if is_fixed(dtype) else n)
    out = np.empty_like(x)
    getattr(lib_rel() if release else lib(), "kfo_fft_batch_" + SFX[dtype])(int(n), int(bool(inverse)), _p(x), _p(out),
                                                   ctypes.c_long(batch), int(nthreads))
    return out


def fft_legs(x, inverse=False, dtype="float", nthreads=1, release=False):
    """Batched complex transform with the reference's KISSFFT_OPENMP split:
    transforms one after the other, the top-level legs of each in parallel
    (kiss_fft.c:250-272).  Same results as fft()."""
    x = as_cpx(x, dtype)
    n = x.shape[-2] if is_fixed(dtype) else x.shape[-1]
    batch = x.size // (2 * n if is_fixed(dtype) else n)
    out = np.empty_like(x)
    rc = getattr(lib_rel() if release else lib(), "kfo_fft_batch_legs_" + SFX[dtype])(int(n), int(bool(inverse)), _p(x), _p(out),
                                                             ctypes.c_long(batch), int(nthreads))
    if rc != 0:
        raise MemoryError("kfo_fft_batch_legs: scratch allocation failed")
    return out


def fft_stride(x, nfft, stride, inverse=False, dtype="float"):
    """One kiss_fft_stride call: input read at every ``stride``-th element."""
    x = as_cpx(x, dtype)
    out = empty_cpx((nfft,), dtype)
    getattr(lib(), "kfo_fft_" + SFX[dtype])(int(nfft), int(bool(inverse)), _p(x), int(stride), _p(out))
    return out


def fftr(t, dtype="float", nthreads=1):
    """Batched real forward transform along the last axis: n reals -> n/2+1 bins."""
    t = np.ascontiguousarray(t, dtype=SCALAR[dtype])
    n = t.shape[-1]
    batch = t.size // n
    out = empty_cpx(t.shape[:-1] + (n // 2 + 1,), dtype)
    rc = getattr(lib(), "kfo_fftr_batch_" + SFX[dtype])(int(n), _p(t), _p(out), ctypes.c_long(batch), int(nthreads))
    if rc:
        raise ValueError("real transform size must be even")
    return out


def fftri(f, nfft, dtype="float", nthreads=1):
    """Batched real inverse transform: nfft/2+1 bins -> nfft reals."""
    f = as_cpx(f, dtype)
    nb = nfft // 2 + 1
    batch = f.size // (2 * nb if is_fixed(dtype) else nb)
    lead = f.shape[:-2] if is_fixed(dtype) else f.shape[:-1]
    out = np.zeros(lead + (nfft,), SCALAR[dtype])
    rc = getattr(lib(), "kfo_fftri_batch_" + SFX[dtype])(int(nfft), _p(f), _p(out), ctypes.c_long(batch), int(nthreads))
    if rc:
        raise ValueError("real transform size must be even")
    return out


def fftnd(x, dims, inverse=False, dtype="float"):
    x = as_cpx(x, dtype)
    d = (ctypes.c_int * len(dims))(*dims)
    out = np.empty_like(x)
    getattr(lib(), "kfo_fftnd_" + SFX[dtype])(d, len(dims), int(bool(inverse)), _p(x), _p(out))
    return out


def fftndr(t, dims, dtype="float"):
    t = np.ascontiguousarray(t, dtype=SCALAR[dtype])
    d = (ctypes.c_int * len(dims))(*dims)
    out = empty_cpx(tuple(dims[:-1]) + (dims[-1] // 2 + 1,), dtype)
    getattr(lib(), "kfo_fftndr_" + SFX[dtype])(d, len(dims), _p(t), _p(out))
    return out


def fftndri(f, dims, dtype="float"):
    f = as_cpx(f, dtype)
    d = (ctypes.c_int * len(dims))(*dims)
    out = np.zeros(tuple(dims), SCALAR[dtype])
    getattr(lib(), "kfo_fftndri_" + SFX[dtype])(d, len(dims), _p(f), _p(out))
    return out


def fastfir_nfft(L):
    return int(lib().kfo_fastfir_nfft(ctypes.c_long(L)))


def fastfir(h, x, nfft=0, nthreads=1):
    """Real overlap-scrap FIR of the whole signal (valid convolution, Ns-L+1 outputs)."""
    h = np.ascontiguousarray(h, np.float32)
    x = np.ascontiguousarray(x, np.float32)
    L, Ns = h.size, x.size
    y = np.zeros(max(Ns - L + 1, 1), np.float32)
    n = lib().kfo_fastfir_f32(_p(h), ctypes.c_long(L), ctypes.c_long(nfft), _p(x), ctypes.c_long(Ns), _p(y),
                              int(nthreads))
    if n < 0:
        raise ValueError("bad fast FIR arguments")
    return y[:n]


def direct_fir(h, x):
    h = np.ascontiguousarray(h, np.float32)
    x = np.ascontiguousarray(x, np.float32)
    y = np.zeros(max(x.size - h.size + 1, 1), np.float32)
    n = lib().kfo_direct_fir_f32(_p(h), ctypes.c_long(h.size), _p(x), ctypes.c_long(x.size), _p(y))
    return y[:n]
