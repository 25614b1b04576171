"""Generate the golden fixtures from the reference library built from source.

Run where the reference tree is present (the tests read the files it writes
anywhere, with or without the reference):

    python tests/golden/make_golden.py

It builds oracle/_ref/ (oracle/Makefile target ``ref``: the reference's own
kiss_fft.c, kiss_fftr.c, kiss_fftnd.c, kiss_fftndr.c and tools/kiss_fastfir.c
compiled per sample type with -O2 -ffp-contract=off) and writes

* golden.json -- for every case: the seeded input recipe and the SHA-256 of
  the reference's output bytes (fixed point must match bit for bit), the
  SHA-256 of the reference plan's twiddle tables, and for float/double the
  reference build's own worst relative L2 error against an FP64 transform;
* small.npz  -- full input/output arrays of the small cases.

Inputs come from tests/golden/inputs.py (numpy PCG64 streams, identical on
every platform), so only hashes need to travel for the large cases.
"""
import ctypes
import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)

from oracle import kfo, ref  # noqa: E402
import inputs  # noqa: E402

DTYPES = ["float", "double", "int16_t", "int32_t"]
C2C_SIZES = [1, 2, 3, 4, 5, 6, 7, 8, 9, 12, 16, 25, 30, 32, 49, 64, 97, 112, 120, 121, 136, 169, 257, 480,
             961, 1000, 1024, 2048, 3003, 4096, 4099, 16384, 17017, 34034, 65536, 131072]
R_SIZES = [2, 4, 6, 8, 10, 12, 30, 64, 120, 480, 1000, 2048, 4096, 6006, 34034]
ND_DIMS = [[2, 3], [4, 4], [3, 5, 7], [8, 6], [2, 3, 4, 6], [16, 32], [64, 64], [5, 7, 11], [128, 96],
           # axes longer than one shared-memory tile (two HBM passes on the GPU)
           [32768, 3], [2, 65536], [3, 40000, 2]]
NDR_DIMS = [[2, 4], [4, 4], [3, 5, 8], [8, 6], [2, 3, 4, 6], [16, 32], [32, 64], [8, 16, 16], [6, 10],
            [40000, 4], [3, 65536]]
TW_SIZES = [480, 1000, 1024, 2048, 3003, 4096, 17017, 65536, 131072]
FIR_CASES = [(255, 20000), (1000, 50000), (4095, 70000), (17, 5000)]
SMALL = 64


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def seed_of(*parts):
    return int.from_bytes(hashlib.sha256(repr(parts).encode()).digest()[:4], "little")


def batch_for(n):
    return 2 if n <= 65536 else 1


def ref_twiddle_bytes(dtype, n, inverse):
    """Bytes of cfg->twiddles of a reference kiss_fft_alloc plan
    (struct kiss_fft_state: int nfft, int inverse, int factors[64], twiddles)."""
    L = ref.lib(dtype)
    cfg = L.kiss_fft_alloc(n, inverse, None, None)
    esz = 2 * np.dtype(inputs.SCALAR[dtype]).itemsize
    off = 8 + 64 * 4
    raw = ctypes.string_at(cfg + off, n * esz)
    ref._libc.free(cfg)
    return raw


def ref_super_twiddle_bytes(dtype, nfft, inverse):
    """Bytes of the super twiddles of a reference kiss_fftr_alloc plan
    (struct kiss_fftr_state: substate, tmpbuf, super_twiddles pointers)."""
    L = ref.lib(dtype)
    cfg = L.kiss_fftr_alloc(nfft, inverse, None, None)
    ptrs = (ctypes.c_void_p * 3).from_address(cfg)
    esz = 2 * np.dtype(inputs.SCALAR[dtype]).itemsize
    raw = ctypes.string_at(ptrs[2], (nfft // 4) * esz)
    ref._libc.free(cfg)
    return raw


def relerr_fp64(out, x, dtype, axis_fn):
    """Worst per-transform relative L2 error of ``out`` vs an FP64 transform."""
    exact = axis_fn(inputs.to_complex128(x, dtype))
    got = inputs.to_complex128(out, dtype)
    e = np.linalg.norm((got - exact).reshape(exact.shape[0], -1), axis=1)
    s = np.linalg.norm(exact.reshape(exact.shape[0], -1), axis=1)
    return float(np.max(e / s))


def main():
    ref.build()
    gold = {"c2c": [], "r2c": [], "c2r": [], "nd": [], "ndr": [], "ndri": [], "twiddles": [], "super_twiddles": [],
            "fastfir": []}
    small = {}
    for dt in DTYPES:
        for n in C2C_SIZES:
            for inv in (0, 1):
                b = batch_for(n)
                seed = seed_of("c2c", dt, n, inv)
                x = inputs.cpx((b, n), dt, seed)
                y = ref.fft(x, inv, dt)
                rec = {"dtype": dt, "n": n, "inverse": inv, "batch": b, "seed": seed, "sha256": sha(y)}
                if not kfo.is_fixed(dt):
                    fn = (lambda z: np.fft.ifft(z, axis=-1) * z.shape[-1]) if inv else (lambda z: np.fft.fft(z, axis=-1))
                    rec["ref_relerr"] = relerr_fp64(y, x, dt, fn)
                gold["c2c"].append(rec)
                if n <= SMALL:
                    small["c2c_%s_%d_%d_in" % (dt, n, inv)] = x
                    small["c2c_%s_%d_%d_out" % (dt, n, inv)] = y
        for n in R_SIZES:
            b = batch_for(n)
            seed = seed_of("r2c", dt, n)
            t = inputs.real((b, n), dt, seed)
            f = ref.fftr(t, dt)
            rec = {"dtype": dt, "n": n, "batch": b, "seed": seed, "sha256": sha(f)}
            if not kfo.is_fixed(dt):
                exact = np.fft.rfft(t.astype(np.float64), axis=-1)
                got = inputs.to_complex128(f, dt)
                rec["ref_relerr"] = float(np.max(np.linalg.norm(got - exact, axis=1) / np.linalg.norm(exact, axis=1)))
            gold["r2c"].append(rec)
            # inverse: seeded random bins (not necessarily Hermitian; the
            # reference's merge is defined for any input)
            seed2 = seed_of("c2r", dt, n)
            fi = inputs.cpx((b, n // 2 + 1), dt, seed2)
            ti = ref.fftri(fi, n, dt)
            gold["c2r"].append({"dtype": dt, "n": n, "batch": b, "seed": seed2, "sha256": sha(ti)})
            if n <= SMALL:
                small["r2c_%s_%d_in" % (dt, n)] = t
                small["r2c_%s_%d_out" % (dt, n)] = f
                small["c2r_%s_%d_in" % (dt, n)] = fi
                small["c2r_%s_%d_out" % (dt, n)] = ti
        for dims in ND_DIMS:
            for inv in (0, 1):
                seed = seed_of("nd", dt, tuple(dims), inv)
                x = inputs.cpx(tuple(dims), dt, seed)
                y = ref.fftnd(x, dims, inv, dt)
                gold["nd"].append({"dtype": dt, "dims": dims, "inverse": inv, "seed": seed, "sha256": sha(y)})
        for dims in NDR_DIMS:
            seed = seed_of("ndr", dt, tuple(dims))
            t = inputs.real(tuple(dims), dt, seed)
            try:
                f = ref.fftndr(t, dims, dt)
            except MemoryError:
                # kiss_fftndr_alloc's size heuristic (kiss_fftndr.c:50-59)
                # rejects some small fixed-point shapes; record that.
                gold["ndr"].append({"dtype": dt, "dims": dims, "seed": seed, "ref_rejects": True})
                continue
            gold["ndr"].append({"dtype": dt, "dims": dims, "seed": seed, "sha256": sha(f)})
            seed2 = seed_of("ndri", dt, tuple(dims))
            fi = inputs.cpx(tuple(dims[:-1]) + (dims[-1] // 2 + 1,), dt, seed2)
            ti = ref.fftndri(fi, dims, dt)
            gold["ndri"].append({"dtype": dt, "dims": dims, "seed": seed2, "sha256": sha(ti)})
        for n in TW_SIZES:
            for inv in (0, 1):
                gold["twiddles"].append({"dtype": dt, "n": n, "inverse": inv,
                                         "sha256": hashlib.sha256(ref_twiddle_bytes(dt, n, inv)).hexdigest()})
                if n % 4 == 0:
                    gold["super_twiddles"].append({"dtype": dt, "nfft": n, "inverse": inv,
                                                   "sha256": hashlib.sha256(
                                                       ref_super_twiddle_bytes(dt, n, inv)).hexdigest()})
    import tempfile
    for L, Ns in FIR_CASES:
        seed = seed_of("fir", L, Ns)
        rng = np.random.default_rng(seed)
        h = rng.standard_normal(L).astype(np.float32)
        x = rng.standard_normal(Ns).astype(np.float32)
        with tempfile.TemporaryDirectory() as d:
            y = ref.fastconvr(h, x, d)
        exact = np.convolve(x.astype(np.float64), h.astype(np.float64), "valid")
        gold["fastfir"].append({"L": L, "Ns": Ns, "seed": seed, "nout": int(y.size), "sha256": sha(y),
                                "ref_relerr": float(np.linalg.norm(y - exact) / np.linalg.norm(exact))})
        if Ns <= 20000:
            small["fir_%d_%d_out" % (L, Ns)] = y
    with open(os.path.join(HERE, "golden.json"), "w") as f:
        json.dump(gold, f, indent=0, sort_keys=True)
    np.savez_compressed(os.path.join(HERE, "small.npz"), **small)
    print("wrote", sum(len(v) for v in gold.values()), "cases,", len(small), "small arrays")


if __name__ == "__main__":
    main()
