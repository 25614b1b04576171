"""The Python mirror refuses buffers smaller than what a call reads or
writes (the C ABI takes plain pointers and cannot check), before any
library call -- so these run without a GPU."""
import numpy as np
import pytest

import kissfft_gb300 as kf


class FakeCfg(object):
    lib = None
    ptr = 0

    def __init__(self, **kw):
        self.__dict__.update(kw)


def test_complex_calls():
    c = FakeCfg(kind="c2c", dtype="float", nfft=1024)
    with pytest.raises(ValueError):
        kf.kiss_fft(c, np.zeros(1000, np.complex64), np.zeros(1024, np.complex64))
    with pytest.raises(ValueError):
        kf.kiss_fft(c, np.zeros(1024, np.complex64), np.zeros(1023, np.complex64))
    with pytest.raises(ValueError):
        kf.kiss_fft_stride(c, np.zeros(2 * 1024 - 2, np.complex64), np.zeros(1024, np.complex64), 2)
    with pytest.raises(ValueError):
        kf.kiss_fft_batch(c, np.zeros((4, 1024), np.complex64), np.zeros((4, 1024), np.complex64), 5)
    with pytest.raises(ValueError):  # out_dist larger than the frame
        kf.kiss_fft_batch(c, np.zeros((4, 1024), np.complex64), np.zeros((4, 1024), np.complex64), 4, 0, 2048)
    q = FakeCfg(kind="c2c", dtype="int16_t", nfft=480)
    with pytest.raises(ValueError):
        kf.kiss_fft(q, np.zeros((480, 2), np.int16), np.zeros((479, 2), np.int16))


def test_real_nd_and_fir_calls():
    r = FakeCfg(kind="real", dtype="float", nfft=4096)
    with pytest.raises(ValueError):
        kf.kiss_fftr(r, np.zeros(4096, np.float32), np.zeros(2048, np.complex64))
    with pytest.raises(ValueError):
        kf.kiss_fftri(r, np.zeros(2049, np.complex64), np.zeros(4095, np.float32))
    with pytest.raises(ValueError):
        kf.kiss_fftr_batch(r, np.zeros((3, 4096), np.float32), np.zeros((3, 2049), np.complex64), 4)
    with pytest.raises(ValueError):
        kf.kiss_fftri_batch(r, np.zeros((2, 2049), np.complex64), np.zeros((1, 4096), np.float32), 2)
    nd = FakeCfg(kind="nd", dtype="double", dims=[8, 16])
    with pytest.raises(ValueError):
        kf.kiss_fftnd(nd, np.zeros((8, 15), np.complex128), np.zeros((8, 16), np.complex128))
    ndr = FakeCfg(kind="ndr", dtype="float", dims=[8, 16])
    with pytest.raises(ValueError):
        kf.kiss_fftndr(ndr, np.zeros((8, 16), np.float32), np.zeros((8, 8), np.complex64))
    with pytest.raises(ValueError):
        kf.kiss_fftndri(ndr, np.zeros((8, 9), np.complex64), np.zeros((8, 15), np.float32))
    fir = FakeCfg(kind="fir", dtype="float", nfft=2048, ntaps=255)
    with pytest.raises(ValueError):
        kf.kiss_fastfir(fir, np.zeros(100, np.float32), np.zeros(100, np.float32), 90, [20])
    with pytest.raises(ValueError):
        kf.kiss_fastfir_filter(fir, np.zeros(1000, np.float32), np.zeros(745, np.float32))
