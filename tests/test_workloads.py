"""The seeded synthetic workloads (tests/golden/inputs.py) keep the shapes
and shares their descriptions state, and every size they draw builds a plan
(checked with the library's own plan builder through the CPU emulator)."""
import ctypes
import os

import numpy as np

import inputs

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def prime_factors(n):
    out, p = set(), 2
    while p * p <= n:
        while n % p == 0:
            out.add(p)
            n //= p
        p += 1
    if n > 1:
        out.add(n)
    return out


def test_uneven_mix_shares_and_sizes():
    mix = inputs.uneven_mix(4000, seed=3)
    assert mix == inputs.uneven_mix(4000, seed=3)  # seeded
    kinds = [(k, d) for k, d, _ in mix]
    share = lambda kd: kinds.count(kd) / len(kinds)
    assert abs(share(("c2c", "float")) - 0.6) < 0.03
    assert abs(share(("r2c", "float")) - 0.3) < 0.03
    assert abs(share(("c2c", "int16_t")) - 0.1) < 0.02
    smooth = 0
    for k, d, n in mix:
        assert 16 <= n <= 131072
        if k == "r2c":
            assert n % 2 == 0
        f = prime_factors(n)
        assert max(f) <= 31
        smooth += f <= {2, 3, 5}
    assert abs(smooth / len(mix) - 0.8) < 0.03
    ns = np.array([n for _, _, n in mix])
    # log-uniform on [16, 131072]: about half the draws below the geometric mean
    assert abs(np.mean(ns < np.sqrt(16 * 131072)) - 0.5) < 0.05


def test_uneven_mix_sizes_build_plans():
    lib = os.path.join(ROOT, "tests", "emu", "_build", "libkfemu.so")
    if not os.path.exists(lib):
        import subprocess
        csrc = os.path.join(ROOT, "kissfft_gb300", "csrc")
        os.makedirs(os.path.dirname(lib), exist_ok=True)
        subprocess.run(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-Wno-unknown-pragmas", "-shared", "-fPIC",
                        "-I", csrc, os.path.join(ROOT, "tests", "emu", "kf_emu.cpp"), os.path.join(csrc, "kf_plan.cpp"),
                        "-o", lib], check=True)
    E = ctypes.CDLL(lib)
    out = (ctypes.c_int * 4)()
    for k, d, n in set(inputs.uneven_mix(20000, seed=3)):
        dt = 0 if d == "float" else 2
        assert E.emu_plan_info(dt, n // 2 if k == "r2c" else n, 0, out) == 0, (k, d, n)


def test_bench_operation_count():
    """bench.py's GFLOP/s figures count 5*N*log2(N) per complex transform."""
    import bench
    assert bench.c2c_flops(1024, 2) == 2 * 5 * 1024 * 10
    assert bench.c2c_flops(480, 1) == 5 * 480 * np.log2(480)
    assert bench.c2c_flops(1, 7) == 0


def test_bench_accuracy_helpers():
    """bench.py's accuracy fields: the device-buffer row view, the float error
    beside the reference float build's, fixed-point bit-exactness, and the
    summary (run here on CPU tensors laid out as the bench uploads them)."""
    import torch

    import bench
    rows = []
    for dt, n in (("float", 480), ("int16_t", 1000), ("int32_t", 3003)):
        x = inputs.cpx((5, n), dt, n)
        xv = x.view(np.float32) if dt == "float" else x
        t = torch.from_numpy(np.ascontiguousarray(xv))
        back = bench.device_rows(t, dt, n, 3)
        assert np.array_equal(back, x[:3])
        from oracle import kfo
        y = kfo.fft(x[:3], 0, dt)
        a = bench.accuracy(dt, n, x[:3], y)
        if dt == "float":
            assert a["relerr"] == a["ref_relerr"] and a["relerr"] <= a["bound"]
        else:
            assert a["bit_exact"]
            y2 = y.copy()
            y2[0, 0, 0] ^= 1
            assert not bench.accuracy(dt, n, x[:3], y2)["bit_exact"]
        rows.append({"accuracy": a})
    s = bench.accuracy_summary(rows)
    assert s["fixed_bit_exact"] and s["float_within_bound"] and s["rows_per_unit"] == 3


def test_bench_reference_arm_line():
    """bench.py --impl reference (CPU only) prints one JSON line with the
    keys the benchmark contract names, on a tiny sample of the workload."""
    import json
    import subprocess
    import sys
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "3", "--cpu-frac", "0.002"], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads(r.stdout.strip().splitlines()[-1])
    for k in ("impl", "metric", "value", "unit", "n_gpus", "steps", "warmup", "higher_is_better", "scaling",
              "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert k in line, k
    assert line["impl"] == "reference" and line["warmup"] >= 3 and line["value"] > 0
    cb = line["cpu_baseline"]
    for k in ("value", "unit", "cores", "kind", "sample"):
        assert k in cb, k
    assert cb["openmp_build"]["value"] > 0
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["d2h_bytes_per_step"] == 0
    assert "workload" in line["config"]
