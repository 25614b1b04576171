"""ctypes binding of the reference library compiled from its own sources into
oracle/_ref/ (see oracle/Makefile, target ``ref``) -- test infrastructure only.

Used to pin the C oracle against the reference and to generate the golden
fixtures under tests/golden/.  Present only where the reference tree exists.
"""
import ctypes
import os
import subprocess

import numpy as np

from . import kfo

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(HERE, "_ref")
REF_SRC = os.environ.get("KISSFFT_REF_SRC", "/root/reference")

_libc = ctypes.CDLL(None)
_libc.free.argtypes = [ctypes.c_void_p]
_libs = {}


def available():
    return os.path.exists(os.path.join(REF_DIR, "libkissfft-float.so")) or os.path.isdir(REF_SRC)


def build():
    subprocess.run(["make", "-s", "-C", HERE, "ref", "REF=" + REF_SRC], check=True)


def lib(dtype, variant=""):
    key = dtype + variant
    if key not in _libs:
        path = os.path.join(REF_DIR, "libkissfft-%s%s.so" % (dtype, variant))
        if not os.path.exists(path):
            build()
        L = ctypes.CDLL(path)
        for fn in ("kiss_fft_alloc", "kiss_fftr_alloc", "kiss_fftnd_alloc", "kiss_fftndr_alloc"):
            getattr(L, fn).restype = ctypes.c_void_p
        L.kiss_fft_alloc.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
        L.kiss_fftr_alloc.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
        L.kiss_fftnd_alloc.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
        L.kiss_fftndr_alloc.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
        for fn in ("kiss_fft", "kiss_fftr", "kiss_fftri", "kiss_fftnd", "kiss_fftndr", "kiss_fftndri"):
            getattr(L, fn).argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
        L.kiss_fft_stride.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]
        _libs[key] = L
    return _libs[key]


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def fft(x, inverse=False, dtype="float", variant=""):
    x = kfo.as_cpx(x, dtype)
    fixed = kfo.is_fixed(dtype)
    n = x.shape[-2] if fixed else x.shape[-1]
    L = lib(dtype, variant)
    cfg = L.kiss_fft_alloc(n, int(bool(inverse)), None, None)
    out = np.empty_like(x)
    xf = x.reshape((-1, n, 2) if fixed else (-1, n))
    of = out.reshape(xf.shape)
    for b in range(xf.shape[0]):
        L.kiss_fft(cfg, _p(xf[b]), _p(of[b]))
    _libc.free(cfg)
    return out


def fftr(t, dtype="float", variant=""):
    t = np.ascontiguousarray(t, dtype=kfo.SCALAR[dtype])
    n = t.shape[-1]
    L = lib(dtype, variant)
    cfg = L.kiss_fftr_alloc(n, 0, None, None)
    out = kfo.empty_cpx(t.shape[:-1] + (n // 2 + 1,), dtype)
    tf = t.reshape(-1, n)
    of = out.reshape((tf.shape[0], n // 2 + 1) + ((2,) if kfo.is_fixed(dtype) else ()))
    for b in range(tf.shape[0]):
        L.kiss_fftr(cfg, _p(tf[b]), _p(of[b]))
    _libc.free(cfg)
    return out


def fftri(f, nfft, dtype="float", variant=""):
    f = kfo.as_cpx(f, dtype)
    nb = nfft // 2 + 1
    fixed = kfo.is_fixed(dtype)
    L = lib(dtype, variant)
    cfg = L.kiss_fftr_alloc(nfft, 1, None, None)
    ff = f.reshape((-1, nb, 2) if fixed else (-1, nb))
    out = np.zeros((ff.shape[0], nfft), kfo.SCALAR[dtype])
    for b in range(ff.shape[0]):
        L.kiss_fftri(cfg, _p(ff[b]), _p(out[b]))
    _libc.free(cfg)
    lead = f.shape[:-2] if fixed else f.shape[:-1]
    return out.reshape(lead + (nfft,))


def fftnd(x, dims, inverse=False, dtype="float"):
    x = kfo.as_cpx(x, dtype)
    L = lib(dtype)
    d = (ctypes.c_int * len(dims))(*dims)
    cfg = L.kiss_fftnd_alloc(d, len(dims), int(bool(inverse)), None, None)
    out = np.empty_like(x)
    L.kiss_fftnd(cfg, _p(x), _p(out))
    _libc.free(cfg)
    return out


def fftndr(t, dims, dtype="float"):
    t = np.ascontiguousarray(t, dtype=kfo.SCALAR[dtype])
    L = lib(dtype)
    d = (ctypes.c_int * len(dims))(*dims)
    cfg = L.kiss_fftndr_alloc(d, len(dims), 0, None, None)
    if not cfg:
        raise MemoryError("reference kiss_fftndr_alloc returned NULL for dims %r" % (dims,))
    out = kfo.empty_cpx(tuple(dims[:-1]) + (dims[-1] // 2 + 1,), dtype)
    L.kiss_fftndr(cfg, _p(t), _p(out))
    _libc.free(cfg)
    return out


def fftndri(f, dims, dtype="float"):
    f = kfo.as_cpx(f, dtype)
    L = lib(dtype)
    d = (ctypes.c_int * len(dims))(*dims)
    cfg = L.kiss_fftndr_alloc(d, len(dims), 1, None, None)
    if not cfg:
        raise MemoryError("reference kiss_fftndr_alloc returned NULL for dims %r" % (dims,))
    out = np.zeros(tuple(dims), kfo.SCALAR[dtype])
    L.kiss_fftndri(cfg, _p(f), _p(out))
    _libc.free(cfg)
    return out


def overflow_warnings(fn, *args, **kwargs):
    """Run ``fn`` (fft, fftr or fftri of this module with variant="-ovf": the
    reference built with -DCHECK_OVERFLOW) and count the overflow warnings it
    prints on stderr (_kiss_fft_guts.h:57-61).  Returns (result, count)."""
    import tempfile
    _libc.fflush(None)
    saved = os.dup(2)
    with tempfile.TemporaryFile() as tf:
        os.dup2(tf.fileno(), 2)
        try:
            out = fn(*args, **kwargs)
        finally:
            _libc.fflush(None)
            os.dup2(saved, 2)
            os.close(saved)
        tf.seek(0)
        count = sum(1 for line in tf if b"overflow" in line)
    return out, count


def fastconvr(h, x, tmpdir):
    """Run the reference's fastconvr tool on float32 taps/signal."""
    hp = os.path.join(tmpdir, "h.f32")
    xp = os.path.join(tmpdir, "x.f32")
    yp = os.path.join(tmpdir, "y.f32")
    np.asarray(h, np.float32).tofile(hp)
    np.asarray(x, np.float32).tofile(xp)
    subprocess.run([os.path.join(REF_DIR, "fastconvr"), "-h", hp, "-i", xp, "-o", yp], check=True)
    return np.fromfile(yp, np.float32)
