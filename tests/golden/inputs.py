"""Seeded synthetic inputs shared by the golden-fixture generator and the tests.

numpy's PCG64 ``default_rng`` streams are identical on every platform, so
the same (kind, dtype, shape, seed) reproduces the same bytes here and on the
GPU host.  Value distributions follow the workload descriptions:
complex IEEE inputs have re/im i.i.d. uniform[-1, 1); fixed-point inputs are
uniform over the full integer range.
"""
import numpy as np

SCALAR = {"float": np.float32, "double": np.float64, "int16_t": np.int16, "int32_t": np.int32}
CPLX = {"float": np.complex64, "double": np.complex128}
IMAX = {"int16_t": 2 ** 15, "int32_t": 2 ** 31}


def is_fixed(dtype):
    return dtype in IMAX


def cpx(shape, dtype, seed):
    """Complex samples: shape (...) complex for IEEE, (..., 2) integers for fixed point."""
    rng = np.random.default_rng(seed)
    shape = tuple(shape)
    if is_fixed(dtype):
        m = IMAX[dtype]
        return rng.integers(-m, m, size=shape + (2,), dtype=np.int64).astype(SCALAR[dtype])
    re = rng.uniform(-1.0, 1.0, shape)
    im = rng.uniform(-1.0, 1.0, shape)
    return (re + 1j * im).astype(CPLX[dtype])


def real(shape, dtype, seed):
    rng = np.random.default_rng(seed)
    shape = tuple(shape)
    if is_fixed(dtype):
        m = IMAX[dtype]
        return rng.integers(-m, m, size=shape, dtype=np.int64).astype(SCALAR[dtype])
    return rng.uniform(-1.0, 1.0, shape).astype(SCALAR[dtype])


def sinusoids(batch, n, seed, noise=0.1):
    """Rows of 3 unit sinusoids (random frequency and phase) plus N(0, noise^2)."""
    rng = np.random.default_rng(seed)
    t = np.arange(n)
    freq = rng.uniform(0, n / 2, (batch, 3, 1))
    ph = rng.uniform(0, 2 * np.pi, (batch, 3, 1))
    x = np.cos(2 * np.pi * freq * t / n + ph).sum(axis=1)
    x += rng.normal(0, noise, (batch, n))
    return x.astype(np.float32)


def to_complex128(a, dtype):
    """Exact float64 complex view of an oracle-layout complex array."""
    if is_fixed(dtype):
        return a[..., 0].astype(np.float64) + 1j * a[..., 1].astype(np.float64)
    return a.astype(np.complex128)
