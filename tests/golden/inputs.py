"""Seeded synthetic inputs shared by the golden-fixture generator and the tests.

numpy's PCG64 ``default_rng`` streams are identical on every platform, so
the same (kind, dtype, shape, seed) reproduces the same bytes on every
machine (x86-64 and aarch64 alike).  Value distributions follow the workload descriptions:
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


def extremes(shape, dtype, seed):
    """Fixed-point samples drawn from the two ends of the range only (SAMP_MIN
    or SAMP_MAX, each with probability 1/2): the inputs that drive the
    butterflies' sums out of range, for the overflow-count checks.  ``shape``
    is the complex shape for (..., 2) arrays or the real shape."""
    rng = np.random.default_rng(seed)
    m = IMAX[dtype]
    return rng.choice(np.array([-m, m - 1], np.int64), size=tuple(shape)).astype(SCALAR[dtype])


def named(gen, shape, dtype, seed, complex_):
    """The input a golden case names: inputs.<gen>(shape, dtype, seed), where
    ``extremes`` takes the (..., 2) shape for complex data."""
    if gen == "extremes" and complex_:
        shape = tuple(shape) + (2,)
    return globals()[gen](shape, dtype, seed)


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


# ------------------------------------------------------------ uneven mix
MIX_KINDS = ((0.6, "c2c", "float"), (0.9, "r2c", "float"), (1.0, "c2c", "int16_t"))


def _smooth(lo, hi, primes):
    out = {1}
    for p in primes:
        grown = set()
        for v in out:
            while v <= hi:
                grown.add(v)
                v *= p
        out = grown
    return sorted(v for v in out if lo <= v <= hi)


def uneven_mix(count, seed=3, lo=16, hi=131072):
    """Requests (kind, dtype, nfft) of the batched uneven-size mix.

    nfft is drawn log-uniform on [lo, hi] and moved to the nearest (in log)
    length of its class: 80% 2^a*3^b*5^c, 20% with at least one prime factor
    7..31 (and none above 31).  Kinds: 60% complex float32, 30% real float32
    (even nfft), 10% complex Q15.
    """
    rng = np.random.default_rng(seed)
    smooth = np.array(_smooth(lo, hi, (2, 3, 5)))
    s31 = set(_smooth(lo, hi, (2, 3, 5, 7, 11, 13, 17, 19, 23, 29, 31)))
    rough = np.array(sorted(s31 - set(smooth.tolist())))
    pools = {}
    for name, arr in (("smooth", smooth), ("rough", rough)):
        pools[(name, False)] = arr
        pools[(name, True)] = arr[arr % 2 == 0]
    logs = {k: np.log(v) for k, v in pools.items()}
    out = []
    for _ in range(count):
        u = rng.random()
        kind, dtype = next((k, d) for c, k, d in MIX_KINDS if u < c)
        target = np.log(lo) + rng.random() * (np.log(hi) - np.log(lo))
        cls = "smooth" if rng.random() < 0.8 else "rough"
        key = (cls, kind == "r2c")
        n = int(pools[key][int(np.argmin(np.abs(logs[key] - target)))])
        out.append((kind, dtype, n))
    return out
