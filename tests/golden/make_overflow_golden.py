"""Generate tests/golden/overflow.json from the reference built with its
overflow warnings on.

Run where the reference tree is present (the tests read the file it writes
anywhere, with or without the reference):

    python tests/golden/make_overflow_golden.py

oracle/Makefile target ``ref`` compiles the reference's kiss_fft.c,
kiss_fftr.c, kiss_fftnd.c and kiss_fftndr.c with -DFIXED_POINT=16/32
-DCHECK_OVERFLOW into oracle/_ref/libkissfft-<type>-ovf.so.  Every C_ADD /
C_SUB / C_ADDTO / C_SUBFROM component and kiss_fftr DC sum whose exact value
leaves [SAMP_MIN, SAMP_MAX] prints one warning on stderr
(_kiss_fft_guts.h:57-61, kiss_fftr.c:94-95); this script counts those lines
per case.  Inputs are inputs.extremes (seeded; samples at the two ends of
the range, the inputs that overflow) and inputs.cpx / inputs.real (uniform
over the range, which rarely do).  Each case records the input recipe, the
warning count and the SHA-256 of the reference output.
"""
import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)

from oracle import ref  # noqa: E402
import inputs  # noqa: E402

C2C = [2, 3, 4, 5, 7, 8, 12, 30, 37, 74, 120, 480, 961, 1000, 1024, 3003, 4099, 17017, 65536]
REAL = [6, 30, 120, 480, 1000, 4096, 6006, 34034]
BATCH = 3


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def make(gen, dtype, shape, seed, complex_):
    return inputs.named(gen, shape, dtype, seed, complex_)


def main():
    ref.build()
    cases = []
    for dt in ("int16_t", "int32_t"):
        for gen in ("extremes", "cpx"):
            for n in C2C:
                for inv in (0, 1):
                    seed = 1000 * inv + n
                    x = make(gen, dt, (BATCH, n), seed, True)
                    y, cnt = ref.overflow_warnings(ref.fft, x, inv, dt, variant="-ovf")
                    cases.append({"kind": "c2c", "dtype": dt, "n": n, "inverse": inv, "batch": BATCH,
                                  "gen": gen, "seed": seed, "overflows": cnt, "sha": sha(y)})
        for gen_r, gen_c in (("extremes", "extremes"), ("real", "cpx")):
            for n in REAL:
                seed = 7 * n
                t = make(gen_r, dt, (BATCH, n), seed, False)
                f, cnt = ref.overflow_warnings(ref.fftr, t, dt, variant="-ovf")
                cases.append({"kind": "r2c", "dtype": dt, "n": n, "inverse": 0, "batch": BATCH, "gen": gen_r,
                              "seed": seed, "overflows": cnt, "sha": sha(f)})
                g = make(gen_c, dt, (BATCH, n // 2 + 1), seed + 1, True)
                t2, cnt = ref.overflow_warnings(ref.fftri, g, n, dt, variant="-ovf")
                cases.append({"kind": "c2r", "dtype": dt, "n": n, "inverse": 1, "batch": BATCH, "gen": gen_c,
                              "seed": seed + 1, "overflows": cnt, "sha": sha(t2)})
    out = os.path.join(HERE, "overflow.json")
    with open(out, "w") as f:
        json.dump({"source": "reference built with -DCHECK_OVERFLOW, warnings counted per call", "cases": cases},
                  f, indent=0)
    print("wrote %s: %d cases, %d with overflows" % (out, len(cases), sum(1 for c in cases if c["overflows"])))


if __name__ == "__main__":
    main()
