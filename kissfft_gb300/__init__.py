"""kissfft_gb300 -- KISS FFT on NVIDIA GB300 (sm_103a), driven through its C ABI.

The functions of this module carry the reference's names and argument
meaning (mborgerding/kissfft: kiss_fft.h, kiss_fftr.h, kiss_fftnd.h,
kiss_fftndr.h, tools/kiss_fastfir.c) and call the drop-in libraries
``libkissfft_cuda-<type>.so`` (include/kiss_fft_cuda.h) through ctypes::

    import kissfft_gb300 as kf
    cfg = kf.kiss_fft_alloc(1024, 0, dtype="float")
    kf.kiss_fft(cfg, fin, fout)

Buffers are numpy arrays (host memory: the call stages them and returns
when done) or torch tensors on the GPU (the call is enqueued on torch's
current stream).  Complex buffers use the reference layout: complex64 /
complex128 for float / double, ``(..., 2)`` int16 / int32 arrays for Q15 /
Q31.  As in the reference an alloc that fails returns None; a transform
that fails prints the reference-style message on stderr and, here, also
raises ``KissFFTError``.

There is no CPU fallback: without the built libraries and a GPU every call
fails loudly.
"""
import ctypes
import os

from . import build as _build

DTYPES = ("float", "double", "int16_t", "int32_t")
DTYPE_CODE = {"float": 0, "double": 1, "int16_t": 2, "int32_t": 3}
_SCALAR_NP = {"float": "float32", "double": "float64", "int16_t": "int16", "int32_t": "int32"}

_libs = {}
_core = None


class KissFFTError(RuntimeError):
    pass


def lib_dir():
    return _build.LIB


def _check_built():
    if not os.path.exists(_build.core_lib()):
        raise KissFFTError("kissfft_gb300 is not built: run `python -m kissfft_gb300.build` "
                           "(no CPU fallback exists)")


def core():
    """The core library (include/kissfft_gb300.h)."""
    global _core
    if _core is None:
        _check_built()
        L = ctypes.CDLL(_build.core_lib(), mode=ctypes.RTLD_GLOBAL)
        vp, i, ll = ctypes.c_void_p, ctypes.c_int, ctypes.c_longlong
        for fn in ("kfg_plan_c2c", "kfg_plan_real"):
            getattr(L, fn).restype = vp
            getattr(L, fn).argtypes = [i, i, i]
        for fn in ("kfg_plan_nd", "kfg_plan_ndr"):
            getattr(L, fn).restype = vp
            getattr(L, fn).argtypes = [i, vp, i, i]
        L.kfg_plan_fir.restype = vp
        L.kfg_plan_fir.argtypes = [vp, ctypes.c_size_t, ctypes.c_size_t, vp]
        L.kfg_plan_free.argtypes = [vp]
        L.kfg_exec.argtypes = [vp, vp, vp, vp]
        L.kfg_exec_stride.argtypes = [vp, vp, vp, i, vp]
        L.kfg_exec_batch.argtypes = [vp, vp, vp, ll, ll, ll, vp]
        L.kfg_fir_filter.argtypes = [vp, vp, ctypes.c_size_t, vp, vp, vp]
        L.kfg_set_stream.argtypes = [vp]
        L.kfg_get_stream.restype = vp
        L.kfg_last_error.restype = ctypes.c_char_p
        L.kfg_plan_info.argtypes = [vp, vp, i]
        L.kfg_plan_table.restype = ll
        L.kfg_plan_table.argtypes = [vp, i, vp, ctypes.c_size_t]
        _core = L
    return _core


def load(dtype="float"):
    """The drop-in library of one sample type (include/kiss_fft_cuda.h)."""
    if dtype not in DTYPE_CODE:
        raise ValueError("dtype must be one of %s" % (DTYPES,))
    if dtype not in _libs:
        core()
        L = ctypes.CDLL(_build.dropin_lib(dtype))
        vp, i, ll, sz = ctypes.c_void_p, ctypes.c_int, ctypes.c_longlong, ctypes.c_size_t
        for fn in ("kiss_fft_cuda_alloc", "kiss_fftr_cuda_alloc"):
            getattr(L, fn).restype = vp
            getattr(L, fn).argtypes = [i, i, vp, vp]
        for fn in ("kiss_fftnd_cuda_alloc", "kiss_fftndr_cuda_alloc"):
            getattr(L, fn).restype = vp
            getattr(L, fn).argtypes = [vp, i, i, vp, vp]
        L.kiss_fastfir_cuda_alloc.restype = vp
        L.kiss_fastfir_cuda_alloc.argtypes = [vp, sz, vp, vp, vp]
        for fn in ("kiss_fft_cuda", "kiss_fftr_cuda", "kiss_fftri_cuda", "kiss_fftnd_cuda", "kiss_fftndr_cuda",
                   "kiss_fftndri_cuda"):
            getattr(L, fn).argtypes = [vp, vp, vp]
        L.kiss_fft_cuda_stride.argtypes = [vp, vp, vp, i]
        for fn in ("kiss_fft_cuda_batch", "kiss_fftr_cuda_batch", "kiss_fftri_cuda_batch"):
            getattr(L, fn).argtypes = [vp, vp, vp, ll, ll, ll]
        for fn in ("kiss_fft_cuda_free", "kiss_fftr_cuda_free", "kiss_fftnd_cuda_free", "kiss_fftndr_cuda_free",
                   "kiss_fastfir_cuda_free"):
            getattr(L, fn).argtypes = [vp]
        L.kiss_fastfir_cuda.restype = sz
        L.kiss_fastfir_cuda.argtypes = [vp, vp, vp, sz, vp]
        L.kiss_fastfir_cuda_filter.restype = sz
        L.kiss_fastfir_cuda_filter.argtypes = [vp, vp, sz, vp]
        L.kiss_fft_cuda_set_stream.argtypes = [vp]
        L.kiss_fft_cuda_prepare.argtypes = [vp, ll]
        L.kiss_fft_cuda_autotune.argtypes = [vp, ll]
        L.kiss_fft_cuda_last_error.restype = ctypes.c_char_p
        L.kfc_cuda_fft.argtypes = [i, vp, vp]
        L.kfc_cuda_ifft.argtypes = [i, vp, vp]
        _libs[dtype] = L
    return _libs[dtype]


# ---------------------------------------------------------------- buffers
def _ptr(buf):
    """(pointer, is_torch_cuda) for a numpy array, a torch tensor or an int."""
    if buf is None:
        return None, False
    if isinstance(buf, int):
        return buf, False
    if hasattr(buf, "data_ptr"):
        if not buf.is_contiguous():
            raise ValueError("tensor must be contiguous")
        return buf.data_ptr(), bool(buf.is_cuda)
    if hasattr(buf, "ctypes"):
        if not buf.flags["C_CONTIGUOUS"]:
            raise ValueError("array must be C-contiguous")
        return buf.ctypes.data, False
    raise TypeError("unsupported buffer type %r" % type(buf))


_CPX_BYTES = {"float": 8, "double": 16, "int16_t": 4, "int32_t": 8}


def _nbytes(buf):
    """Byte size of a numpy array or torch tensor (None for a raw address)."""
    if buf is None or isinstance(buf, int):
        return None
    if hasattr(buf, "element_size") and hasattr(buf, "numel"):
        return int(buf.element_size() * buf.numel())
    if hasattr(buf, "nbytes"):
        return int(buf.nbytes)
    return None


def _need(buf, nbytes, what):
    """Refuse a buffer smaller than the bytes the call reads or writes (the
    library takes plain pointers and cannot check)."""
    have = _nbytes(buf)
    if have is not None and have < nbytes:
        raise ValueError("%s holds %d bytes; the call reads or writes %d" % (what, have, nbytes))


def _span(batch, dist, frame):
    """Elements a batch touches: (batch - 1) * dist + frame (dist 0 = packed)."""
    return (int(batch) - 1) * (int(dist) or frame) + frame if batch > 0 else 0


def _use_torch_stream(L, *bufs):
    for b in bufs:
        if hasattr(b, "is_cuda") and b.is_cuda:
            import torch
            L.kiss_fft_cuda_set_stream(ctypes.c_void_p(torch.cuda.current_stream(b.device).cuda_stream))
            return


def _raise_on_status(L, where):
    rc = L.kiss_fft_cuda_status()
    if rc != 0:
        msg = L.kiss_fft_cuda_last_error()
        raise KissFFTError("%s failed (%d): %s" % (where, rc, msg.decode() if msg else ""))


class Cfg(object):
    """A drop-in cfg: the pointer returned by a kiss_*_cuda_alloc call.

    Released by ``free()`` or when garbage-collected (the reference frees
    with free(); a GPU cfg must go through kiss_*_cuda_free)."""

    def __init__(self, lib, ptr, kind, dtype, **meta):
        self.lib, self.ptr, self.kind, self.dtype = lib, ptr, kind, dtype
        self.__dict__.update(meta)

    def free(self):
        if self.ptr:
            self.lib.kiss_fft_cuda_free(ctypes.c_void_p(self.ptr))
            self.ptr = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


def _mk(L, ptr, kind, dtype, **meta):
    return Cfg(L, ptr, kind, dtype, **meta) if ptr else None


# ---------------------------------------------------------------- kiss_fft.h
def kiss_fft_alloc(nfft, inverse_fft=0, dtype="float"):
    """kiss_fft_alloc (reference kiss_fft.h:117)."""
    L = load(dtype)
    return _mk(L, L.kiss_fft_cuda_alloc(int(nfft), int(inverse_fft), None, None), "c2c", dtype, nfft=int(nfft),
               inverse=int(inverse_fft))


def kiss_fft(cfg, fin, fout):
    """kiss_fft (reference kiss_fft.h:129)."""
    kiss_fft_stride(cfg, fin, fout, 1)


def kiss_fft_stride(cfg, fin, fout, fin_stride):
    """kiss_fft_stride (reference kiss_fft.h:134)."""
    ce, n = _CPX_BYTES[cfg.dtype], cfg.nfft
    _need(fin, ((n - 1) * int(fin_stride) + 1) * ce, "fin")
    _need(fout, n * ce, "fout")
    L = cfg.lib
    _use_torch_stream(L, fin, fout)
    L.kiss_fft_cuda_stride(ctypes.c_void_p(cfg.ptr), _ptr(fin)[0], _ptr(fout)[0], int(fin_stride))
    _raise_on_status(L, "kiss_fft_stride")


def kiss_fft_batch(cfg, fin, fout, batch, in_dist=0, out_dist=0):
    """A batch of kiss_fft calls in one launch (distances in complex elements)."""
    ce, n = _CPX_BYTES[cfg.dtype], cfg.nfft
    _need(fin, _span(batch, in_dist, n) * ce, "fin")
    _need(fout, _span(batch, out_dist, n) * ce, "fout")
    L = cfg.lib
    _use_torch_stream(L, fin, fout)
    rc = L.kiss_fft_cuda_batch(ctypes.c_void_p(cfg.ptr), _ptr(fin)[0], _ptr(fout)[0], int(batch), int(in_dist),
                               int(out_dist))
    if rc:
        _raise_on_status(L, "kiss_fft_batch")


def kiss_fft_free(cfg):
    cfg.free()


def kiss_fft_cleanup():
    pass


# ---------------------------------------------------------------- kfc.h
def _kfc(fn, nfft, fin, fout, dtype):
    ce = _CPX_BYTES[dtype]
    _need(fin, int(nfft) * ce, "fin")
    _need(fout, int(nfft) * ce, "fout")
    L = load(dtype)
    _use_torch_stream(L, fin, fout)
    getattr(L, fn)(int(nfft), _ptr(fin)[0], _ptr(fout)[0])
    _raise_on_status(L, fn)


def kfc_fft(nfft, fin, fout, dtype="float"):
    """kfc_fft (reference kfc.h:43): forward transform with a cached plan."""
    _kfc("kfc_cuda_fft", nfft, fin, fout, dtype)


def kfc_ifft(nfft, fin, fout, dtype="float"):
    """kfc_ifft (reference kfc.h:45): inverse transform with a cached plan."""
    _kfc("kfc_cuda_ifft", nfft, fin, fout, dtype)


def kfc_cleanup(dtype="float"):
    """kfc_cleanup (reference kfc.h:48): frees the cached plans of one sample type."""
    load(dtype).kfc_cuda_cleanup()


def kfc_ncached(dtype="float"):
    """Number of cached plans of one sample type (the reference's ncached, kfc.c:22)."""
    return int(load(dtype).kfc_cuda_ncached())


def kiss_fft_next_fast_size(n):
    """kiss_fft_next_fast_size (reference kiss_fft.h:150)."""
    return int(core().kfg_next_fast_size(int(n)))


def kiss_fftr_next_fast_size_real(n):
    """kiss_fftr_next_fast_size_real (reference kiss_fft.h:153-154)."""
    return kiss_fft_next_fast_size((int(n) + 1) >> 1) << 1


# ---------------------------------------------------------------- kiss_fftr.h
def kiss_fftr_alloc(nfft, inverse_fft=0, dtype="float"):
    """kiss_fftr_alloc (reference kiss_fftr.h:29); None for odd nfft."""
    L = load(dtype)
    return _mk(L, L.kiss_fftr_cuda_alloc(int(nfft), int(inverse_fft), None, None), "real", dtype, nfft=int(nfft),
               inverse=int(inverse_fft))


def kiss_fftr(cfg, timedata, freqdata):
    """kiss_fftr (reference kiss_fftr.h:37)."""
    ce, n = _CPX_BYTES[cfg.dtype], cfg.nfft
    _need(timedata, n * ce // 2, "timedata")
    _need(freqdata, (n // 2 + 1) * ce, "freqdata")
    L = cfg.lib
    _use_torch_stream(L, timedata, freqdata)
    L.kiss_fftr_cuda(ctypes.c_void_p(cfg.ptr), _ptr(timedata)[0], _ptr(freqdata)[0])
    _raise_on_status(L, "kiss_fftr")


def kiss_fftri(cfg, freqdata, timedata):
    """kiss_fftri (reference kiss_fftr.h:43)."""
    ce, n = _CPX_BYTES[cfg.dtype], cfg.nfft
    _need(freqdata, (n // 2 + 1) * ce, "freqdata")
    _need(timedata, n * ce // 2, "timedata")
    L = cfg.lib
    _use_torch_stream(L, timedata, freqdata)
    L.kiss_fftri_cuda(ctypes.c_void_p(cfg.ptr), _ptr(freqdata)[0], _ptr(timedata)[0])
    _raise_on_status(L, "kiss_fftri")


def kiss_fftr_batch(cfg, timedata, freqdata, batch, in_dist=0, out_dist=0):
    """A batch of kiss_fftr calls (distances in reals / bins, 0 = packed)."""
    ce, n = _CPX_BYTES[cfg.dtype], cfg.nfft
    _need(timedata, _span(batch, in_dist, n) * ce // 2, "timedata")
    _need(freqdata, _span(batch, out_dist, n // 2 + 1) * ce, "freqdata")
    L = cfg.lib
    _use_torch_stream(L, timedata, freqdata)
    rc = L.kiss_fftr_cuda_batch(ctypes.c_void_p(cfg.ptr), _ptr(timedata)[0], _ptr(freqdata)[0], int(batch),
                                int(in_dist), int(out_dist))
    if rc:
        _raise_on_status(L, "kiss_fftr_batch")


def kiss_fftri_batch(cfg, freqdata, timedata, batch, in_dist=0, out_dist=0):
    """A batch of kiss_fftri calls (distances in bins / reals, 0 = packed)."""
    ce, n = _CPX_BYTES[cfg.dtype], cfg.nfft
    _need(freqdata, _span(batch, in_dist, n // 2 + 1) * ce, "freqdata")
    _need(timedata, _span(batch, out_dist, n) * ce // 2, "timedata")
    L = cfg.lib
    _use_torch_stream(L, timedata, freqdata)
    rc = L.kiss_fftri_cuda_batch(ctypes.c_void_p(cfg.ptr), _ptr(freqdata)[0], _ptr(timedata)[0], int(batch),
                                 int(in_dist), int(out_dist))
    if rc:
        _raise_on_status(L, "kiss_fftri_batch")


# ---------------------------------------------------------------- kiss_fftnd.h / kiss_fftndr.h
def kiss_fftnd_alloc(dims, inverse_fft=0, dtype="float"):
    """kiss_fftnd_alloc (reference kiss_fftnd.h:20)."""
    L = load(dtype)
    d = (ctypes.c_int * len(dims))(*[int(x) for x in dims])
    return _mk(L, L.kiss_fftnd_cuda_alloc(d, len(dims), int(inverse_fft), None, None), "nd", dtype, dims=list(dims),
               inverse=int(inverse_fft))


def kiss_fftnd(cfg, fin, fout):
    """kiss_fftnd (reference kiss_fftnd.h:21)."""
    prod = 1
    for d in cfg.dims:
        prod *= int(d)
    _need(fin, prod * _CPX_BYTES[cfg.dtype], "fin")
    _need(fout, prod * _CPX_BYTES[cfg.dtype], "fout")
    L = cfg.lib
    _use_torch_stream(L, fin, fout)
    L.kiss_fftnd_cuda(ctypes.c_void_p(cfg.ptr), _ptr(fin)[0], _ptr(fout)[0])
    _raise_on_status(L, "kiss_fftnd")


def kiss_fftndr_alloc(dims, inverse_fft=0, dtype="float"):
    """kiss_fftndr_alloc (reference kiss_fftndr.h:23); the last axis is the real one."""
    L = load(dtype)
    d = (ctypes.c_int * len(dims))(*[int(x) for x in dims])
    return _mk(L, L.kiss_fftndr_cuda_alloc(d, len(dims), int(inverse_fft), None, None), "ndr", dtype,
               dims=list(dims), inverse=int(inverse_fft))


def _ndr_need(cfg, timedata, freqdata):
    ce = _CPX_BYTES[cfg.dtype]
    prod = 1
    for d in cfg.dims:
        prod *= int(d)
    last = int(cfg.dims[-1])
    _need(timedata, prod * ce // 2, "timedata")
    _need(freqdata, prod // last * (last // 2 + 1) * ce, "freqdata")


def kiss_fftndr(cfg, timedata, freqdata):
    """kiss_fftndr (reference kiss_fftndr.h:31)."""
    _ndr_need(cfg, timedata, freqdata)
    L = cfg.lib
    _use_torch_stream(L, timedata, freqdata)
    L.kiss_fftndr_cuda(ctypes.c_void_p(cfg.ptr), _ptr(timedata)[0], _ptr(freqdata)[0])
    _raise_on_status(L, "kiss_fftndr")


def kiss_fftndri(cfg, freqdata, timedata):
    """kiss_fftndri (reference kiss_fftndr.h:40)."""
    _ndr_need(cfg, timedata, freqdata)
    L = cfg.lib
    _use_torch_stream(L, timedata, freqdata)
    L.kiss_fftndri_cuda(ctypes.c_void_p(cfg.ptr), _ptr(freqdata)[0], _ptr(timedata)[0])
    _raise_on_status(L, "kiss_fftndri")


# ---------------------------------------------------------------- tools/kiss_fastfir.c
def kiss_fastfir_alloc(imp_resp, nfft=0):
    """kiss_fastfir_alloc (reference tools/kiss_fastfir.c:36, REAL_FASTFIR, float).

    imp_resp: host float32 array of taps.  Returns the cfg (its ``nfft``
    attribute holds the chosen block size) or None."""
    import numpy as np
    L = load("float")
    h = np.ascontiguousarray(imp_resp, dtype=np.float32)
    n = ctypes.c_size_t(int(nfft))
    p = L.kiss_fastfir_cuda_alloc(h.ctypes.data, h.size, ctypes.byref(n), None, None)
    return _mk(L, p, "fir", "float", nfft=int(n.value), ntaps=int(h.size))


def kiss_fastfir(cfg, inbuf, outbuf, n_new, offset):
    """kiss_fastfir (reference tools/kiss_fastfir.c:40).

    ``offset`` is a one-element list (the in/out ``size_t *offset``).
    Returns the number of output samples written."""
    _need(inbuf, (int(offset[0]) + int(n_new)) * 4, "inbuf")
    L = cfg.lib
    _use_torch_stream(L, inbuf, outbuf)
    off = ctypes.c_size_t(int(offset[0]))
    n = L.kiss_fastfir_cuda(ctypes.c_void_p(cfg.ptr), _ptr(inbuf)[0], _ptr(outbuf)[0], int(n_new), ctypes.byref(off))
    _raise_on_status(L, "kiss_fastfir")
    offset[0] = int(off.value)
    return int(n)


def _float32_count(buf, what):
    """Element count of a float32 numpy array or torch tensor (anything else is refused,
    so a byte view can never be taken for samples)."""
    if hasattr(buf, "numel"):
        import torch
        if buf.dtype != torch.float32:
            raise ValueError("%s must be a float32 tensor" % what)
        return buf.numel()
    import numpy as np
    if getattr(buf, "dtype", None) != np.float32:
        raise ValueError("%s must be a float32 array" % what)
    return buf.size


def kiss_fastfir_filter(cfg, x, y):
    """Whole-signal fast FIR: y[:nx-ntaps+1] = valid convolution of x with the taps."""
    L = cfg.lib
    nx = _float32_count(x, "x")
    ny = _float32_count(y, "y")
    ntaps = getattr(cfg, "ntaps", 1)
    if ny < nx - ntaps + 1:
        raise ValueError("y holds %d samples; the valid convolution has %d" % (ny, nx - ntaps + 1))
    _use_torch_stream(L, x, y)
    n = L.kiss_fastfir_cuda_filter(ctypes.c_void_p(cfg.ptr), _ptr(x)[0], int(nx), _ptr(y)[0])
    _raise_on_status(L, "kiss_fastfir_filter")
    return int(n)


# ---------------------------------------------------------------- specialised kernels
def set_specialize(on=True):
    """Use kernels compiled (NVRTC, cached on disk) for each plan's exact shape."""
    core().kfg_set_specialize(int(bool(on)))


def autotune(cfg, batch):
    """Time candidate launch shapes for batched calls of this size; keep the fastest."""
    rc = cfg.lib.kiss_fft_cuda_autotune(ctypes.c_void_p(cfg.ptr), int(batch))
    if rc:
        _raise_on_status(cfg.lib, "autotune")


def prepare(cfg, batch):
    """Compile the specialised kernels a batched call on cfg will use."""
    rc = cfg.lib.kiss_fft_cuda_prepare(ctypes.c_void_p(cfg.ptr), int(batch))
    if rc:
        _raise_on_status(cfg.lib, "prepare")


# ---------------------------------------------------------------- misc
def last_error(dtype="float"):
    msg = load(dtype).kiss_fft_cuda_last_error()
    return msg.decode() if msg else ""


def plan_info(cfg):
    """(kind, dtype, length, hbm_passes, family, tile) of a cfg's device plan."""
    c = core()
    out = (ctypes.c_int * 6)()
    # the cfg's first field after the header is the core plan pointer
    plan_ptr = ctypes.c_void_p.from_address(cfg.ptr + 40).value
    c.kfg_plan_info(ctypes.c_void_p(plan_ptr), out, 6)
    return tuple(int(v) for v in out)


# ---------------------------------------------------------------- serving loop
SERVE_C2C, SERVE_R2C, SERVE_C2R, SERVE_C2C_2D, SERVE_FIR = 1, 2, 3, 4, 5


class ServeReq(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int), ("dtype", ctypes.c_int), ("inverse", ctypes.c_int), ("n0", ctypes.c_int),
                ("n1", ctypes.c_int), ("len", ctypes.c_longlong), ("taps", ctypes.c_void_p),
                ("in_", ctypes.c_void_p), ("out", ctypes.c_void_p)]


class ServeStats(ctypes.Structure):
    _fields_ = [(n, ctypes.c_longlong) for n in ("completed", "failed", "batches", "max_batch", "peak_hbm_bytes")] + \
               [(n, ctypes.c_double) for n in ("p50_s", "p99_s", "max_s", "mean_s", "req_per_s", "gbs", "bytes",
                                               "host_s")] + \
               [(n, ctypes.c_longlong) for n in ("plans", "plan_bytes", "evictions")]

    def as_dict(self):
        return {n: getattr(self, n) for n, _ in self._fields_}


class LoadTest(ctypes.Structure):
    _fields_ = [("rate", ctypes.c_double), ("seconds", ctypes.c_double), ("count", ctypes.c_longlong),
                ("seed", ctypes.c_ulonglong), ("mix", ctypes.c_double * 4)] + \
               [(n, ctypes.c_int) for n in ("c2c_min", "c2c_max", "d2_min", "d2_max", "fir_taps_min",
                                            "fir_taps_max")] + \
               [("fir_len_min", ctypes.c_longlong), ("fir_len_max", ctypes.c_longlong),
                ("percall_max", ctypes.c_longlong), ("in_pool_mb", ctypes.c_int), ("out_pool_mb", ctypes.c_int)]


class LoadTestResult(ctypes.Structure):
    _fields_ = [("offered", ctypes.c_longlong), ("submit_s", ctypes.c_double), ("served", ServeStats),
                ("percall_count", ctypes.c_longlong)] + \
               [(n, ctypes.c_double) for n in ("percall_req_per_s", "percall_gbs", "percall_p50_s", "percall_p99_s")]


def _serve_lib():
    L = core()
    if not getattr(L, "_serve_ready", False):
        vp, ll = ctypes.c_void_p, ctypes.c_longlong
        L.kfg_server_create.restype = vp
        L.kfg_server_create.argtypes = [ctypes.c_size_t, ctypes.c_int]
        L.kfg_server_submit.restype = ll
        L.kfg_server_submit.argtypes = [vp, ctypes.POINTER(ServeReq)]
        L.kfg_server_wait.argtypes = [vp, ll, ctypes.c_double, ctypes.POINTER(ctypes.c_double)]
        L.kfg_server_drain.argtypes = [vp]
        L.kfg_server_stats.argtypes = [vp, ctypes.POINTER(ServeStats)]
        L.kfg_server_reset_stats.argtypes = [vp]
        L.kfg_server_free.argtypes = [vp]
        L.kfg_server_loadtest.argtypes = [vp, ctypes.POINTER(LoadTest), ctypes.POINTER(LoadTestResult)]
        L._serve_ready = True
    return L


class Server(object):
    """The serving loop (kfg_server_*): submit requests from any thread, wait
    for them, read p50/p99 latency and throughput.  Buffers (numpy arrays,
    torch tensors or raw addresses) must stay alive until waited for."""

    def __init__(self, hbm_budget=0, slots=0):
        self.L = _serve_lib()
        self.ptr = self.L.kfg_server_create(int(hbm_budget), int(slots))
        if not self.ptr:
            raise KissFFTError("kfg_server_create: " + (self.L.kfg_last_error() or b"").decode())
        self._keep = {}

    def submit(self, kind, inp, out, n0, n1=0, dtype="float", inverse=0, taps=None, length=0):
        r = ServeReq()
        r.kind, r.dtype, r.inverse, r.n0, r.n1, r.len = kind, DTYPE_CODE[dtype], int(inverse), int(n0), int(n1), \
            int(length)
        r.taps = _ptr(taps)[0] if taps is not None else None
        r.in_ = _ptr(inp)[0]
        r.out = _ptr(out)[0]
        rid = self.L.kfg_server_submit(ctypes.c_void_p(self.ptr), ctypes.byref(r))
        if rid <= 0:
            raise KissFFTError("kfg_server_submit: " + (self.L.kfg_last_error() or b"").decode())
        self._keep[rid] = (inp, out, taps)
        return rid

    def wait(self, rid, timeout=-1.0):
        lat = ctypes.c_double(0)
        rc = self.L.kfg_server_wait(ctypes.c_void_p(self.ptr), ctypes.c_longlong(rid), float(timeout),
                                    ctypes.byref(lat))
        if rc == 1:
            return None
        self._keep.pop(rid, None)
        if rc != 0:
            raise KissFFTError("request %d failed (%d): %s" % (rid, rc, (self.L.kfg_last_error() or b"").decode()))
        return lat.value

    def drain(self):
        self.L.kfg_server_drain(ctypes.c_void_p(self.ptr))

    def stats(self):
        st = ServeStats()
        self.L.kfg_server_stats(ctypes.c_void_p(self.ptr), ctypes.byref(st))
        return st.as_dict()

    def loadtest(self, **kw):
        cfg = LoadTest()
        defaults = dict(rate=50000.0, seconds=5.0, count=0, seed=4, mix=(0.25, 0.25, 0.25, 0.25), c2c_min=64,
                        c2c_max=65536, d2_min=256, d2_max=1024, fir_taps_min=255, fir_taps_max=4095,
                        fir_len_min=1 << 16, fir_len_max=1 << 22, percall_max=2000, in_pool_mb=256,
                        out_pool_mb=2048)
        defaults.update(kw)
        for k, v in defaults.items():
            if k == "mix":
                for i in range(4):
                    cfg.mix[i] = v[i]
            else:
                setattr(cfg, k, v)
        res = LoadTestResult()
        rc = self.L.kfg_server_loadtest(ctypes.c_void_p(self.ptr), ctypes.byref(cfg), ctypes.byref(res))
        if rc:
            raise KissFFTError("loadtest: " + (self.L.kfg_last_error() or b"").decode())
        out = {n: getattr(res, n) for n, _ in res._fields_ if n != "served"}
        out["served"] = res.served.as_dict()
        return out

    def close(self):
        if self.ptr:
            self.L.kfg_server_free(ctypes.c_void_p(self.ptr))
            self.ptr = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ---------------------------------------------------------------- tools/psdpng.c
def psd(samples, nfft, navg, stereo=False, remove_dc=False):
    """Power spectrogram of psdpng (tools/psdpng.c:116-175): 16-bit samples
    (interleaved pairs summed when stereo), frames of nfft (mean removed when
    remove_dc), rows of navg frames, 10*log10(mean |X|^2 + 1) per frequency.
    Returns a (rows, nfft/2+1) float32 array."""
    import numpy as np
    L = core()
    L.kfg_psd.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_longlong, ctypes.c_int, ctypes.c_int,
                          ctypes.c_int, ctypes.c_void_p, ctypes.POINTER(ctypes.c_longlong), ctypes.c_void_p]
    x = np.ascontiguousarray(samples, dtype=np.int16)
    per_channel = x.size // 2 if stereo else x.size
    nrows = per_channel // nfft // navg
    rows = np.zeros((nrows, nfft // 2 + 1), np.float32)
    plan = L.kfg_plan_real(DTYPE_CODE["float"], int(nfft), 0)
    if not plan:
        raise KissFFTError("kfg_plan_real: " + L.kfg_last_error().decode())
    try:
        got = ctypes.c_longlong(0)
        rc = L.kfg_psd(ctypes.c_void_p(plan), x.ctypes.data, per_channel, int(bool(stereo)), int(bool(remove_dc)),
                       int(navg), rows.ctypes.data if nrows else None, ctypes.byref(got), None)
        if rc:
            raise KissFFTError("kfg_psd: " + L.kfg_last_error().decode())
        assert got.value == nrows
    finally:
        L.kfg_plan_free(ctypes.c_void_p(plan))
    return rows
