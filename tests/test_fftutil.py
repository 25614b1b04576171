"""fftutil_cuda-<type>: the tools/fftutil.c stream front end on the GPU.

Frames of random samples go through the tool as raw binary files, the way
test/testkiss.py drives the reference's tool, and come out equal to the
oracle: Q15/Q31 bit for bit, float within 2e-7*log2(N) relative L2 per
frame.  Covered: 1-D complex forward/inverse, real forward/inverse (-R),
N-D complex and N-D real (-n d1,d2,...), a trailing partial frame (ignored,
as in the reference) and many frames per batched call.
"""
import os
import subprocess

import numpy as np
import pytest

import inputs
from oracle import kfo

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def tool(dtype):
    from kissfft_gb300 import build
    path = build.fftutil_bin(dtype)
    if not os.path.exists(path):
        build.build()
    return path


def test_usage_without_gpu():
    """A bad option prints the reference's usage text and exits 1 before any GPU call."""
    r = subprocess.run([tool("float"), "-x"], capture_output=True, text=True)
    assert r.returncode == 1
    assert "-n d1[,d2,d3...]: fft dimension(s)" in r.stderr


def run(dtype, args, data, tmp_path):
    fin = tmp_path / "in.bin"
    fout = tmp_path / "out.bin"
    fin.write_bytes(data)
    r = subprocess.run([tool(dtype)] + args + [str(fin), str(fout)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    return fout.read_bytes()


def frames_close(got, ref, dtype, n):
    if dtype in ("int16_t", "int32_t"):
        return got.tobytes() == ref.tobytes()
    g = inputs.to_complex128(got, dtype) if np.iscomplexobj(got) else got.astype(np.float64)
    r = inputs.to_complex128(ref, dtype) if np.iscomplexobj(ref) else ref.astype(np.float64)
    g = g.reshape(g.shape[0], -1)
    r = r.reshape(r.shape[0], -1)
    err = np.linalg.norm(g - r, axis=1) / np.maximum(np.linalg.norm(r, axis=1), 1e-30)
    return float(err.max()) <= 2e-7 * max(1.0, np.log2(n))


@pytest.mark.gpu
@pytest.mark.parametrize("dtype", ["float", "int16_t", "int32_t"])
@pytest.mark.parametrize("inv", [0, 1])
def test_complex_frames(dtype, inv, tmp_path):
    n, frames = 480, 300
    x = inputs.cpx((frames, n), dtype, 10 + inv)
    data = np.ascontiguousarray(x).tobytes() + b"\x01" * 7  # partial frame at the end
    out = run(dtype, ["-n", str(n)] + (["-i"] if inv else []), data, tmp_path)
    got = np.frombuffer(out, dtype=x.dtype).reshape(x.shape)
    assert frames_close(got, kfo.fft(x, inv, dtype), dtype, n)


@pytest.mark.gpu
@pytest.mark.parametrize("dtype", ["float", "int16_t"])
def test_real_frames(dtype, tmp_path):
    n, frames = 1024, 200
    t = inputs.real((frames, n), dtype, 3)
    out = run(dtype, ["-n", str(n), "-R"], t.tobytes(), tmp_path)
    ref = kfo.fftr(t, dtype)
    got = np.frombuffer(out, dtype=ref.dtype).reshape(ref.shape)
    assert frames_close(got, ref, dtype, n)
    f = inputs.cpx((frames, n // 2 + 1), dtype, 4)
    out = run(dtype, ["-n", str(n), "-R", "-i"], np.ascontiguousarray(f).tobytes(), tmp_path)
    ref = kfo.fftri(f, n, dtype)
    got = np.frombuffer(out, dtype=ref.dtype).reshape(ref.shape)
    if dtype == "int16_t":
        assert got.tobytes() == ref.tobytes()
    else:
        err = np.linalg.norm(got - ref, axis=1) / np.linalg.norm(ref, axis=1)
        assert err.max() <= 8e-7 * np.log2(n)


@pytest.mark.gpu
@pytest.mark.parametrize("dtype", ["float", "int32_t"])
def test_nd_frames(dtype, tmp_path):
    dims = [12, 20]
    x = inputs.cpx((3, 12, 20), dtype, 5)
    out = run(dtype, ["-n", "12,20"], np.ascontiguousarray(x).tobytes(), tmp_path)
    got = np.frombuffer(out, dtype=x.dtype).reshape(x.shape)
    ref = np.stack([kfo.fftnd(x[k], dims, 0, dtype) for k in range(3)])
    assert frames_close(got, ref, dtype, 240)
    t = inputs.real((2, 8, 16), dtype, 6)
    out = run(dtype, ["-n", "8,16", "-R"], t.tobytes(), tmp_path)
    ref = np.stack([kfo.fftndr(t[k], [8, 16], dtype) for k in range(2)])
    got = np.frombuffer(out, dtype=ref.dtype).reshape(ref.shape)
    assert frames_close(got, ref, dtype, 128)
