"""bench.py's GPU arm end to end on the CPU, with the CUDA calls faked.

The GPU arm only runs on a GB300, so its bookkeeping (per-unit timing rows,
accuracy against the oracle, GFLOP/s, roofline, the e2e host-buffer leg,
both CPU baselines and the JSON line) is exercised here with CUDA events,
device moves and pinned memory replaced by CPU stand-ins and the library's
transforms computed by the oracle.  The numbers are meaningless; the test
checks that the arm runs through and fills every field.  It runs in a
subprocess so the stand-ins never reach other tests.
"""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

SCRIPT = r'''
import contextlib, io, json, sys, time, types
sys.path.insert(0, ROOT)
import numpy as np
import torch

class Ev:
    def __init__(self, enable_timing=False):
        self.t = None
    def record(self, s=None):
        self.t = time.perf_counter()
    def elapsed_time(self, other):
        return (other.t - self.t) * 1e3

torch.cuda.set_device = lambda d: None
torch.cuda.current_stream = lambda *a: types.SimpleNamespace(cuda_stream=0)
torch.cuda.Event = Ev
torch.cuda.synchronize = lambda *a: None
_to = torch.Tensor.to
def to(self, *a, **k):
    if a and isinstance(a[0], torch.device) and a[0].type == "cuda":
        return self.clone()
    return _to(self, *a, **k)
torch.Tensor.to = to
torch.Tensor.pin_memory = lambda self: self.clone()

import kissfft_gb300 as kf
from oracle import kfo

class Cfg:
    def __init__(self, n, inv, dt):
        self.nfft, self.inverse, self.dtype = n, inv, dt

def batch(cfg, x, y, b):
    xn = x.numpy()
    if cfg.dtype == "float":
        r = kfo.fft(xn.view(np.complex64).reshape(b, cfg.nfft), cfg.inverse, "float").view(np.float32)
    else:
        r = kfo.fft(xn.reshape(b, cfg.nfft, 2), cfg.inverse, cfg.dtype)
    y.copy_(torch.from_numpy(np.ascontiguousarray(r).reshape(y.shape)))

kf.kiss_fft_alloc = lambda n, inv, dt: Cfg(n, inv, dt)
kf.plan_info = lambda c: [0, 0, 0, 1]
kf.set_specialize = lambda on: None
kf.autotune = lambda c, b: None
kf.prepare = lambda c, b: None
kf.kiss_fft_batch = batch

import bench
bench.link_peak = lambda *a, **k: {"h2d_gbs": 1.0, "d2h_gbs": 1.0, "bidir_gbs": 2.0, "how": "stand-in"}
bench._CASES = [("float", 480, 32), ("int16_t", 1000, 16), ("int32_t", 3003, 8), ("float", 65536, 2)]
args = types.SimpleNamespace(steps=2, warmup=3, specialize=1, autotune=1, no_e2e=False, no_cpu=False, no_mix=True,
                             no_serve=True, no_configs=True, cpu_seconds=0.2, traffic=None, case=[])
r = bench.run_gpu(args)
sys.argv = ["bench.py", "--case", "float:480:32", "--case", "int16_t:1000:16", "--steps", "2"]
out = io.StringIO()
with contextlib.redirect_stdout(out):
    bench.main()
print(json.dumps({"run": {k: r[k] for k in ("units", "cpu", "e2e", "roofline", "gflops", "gpu_launches")},
                  "line": json.loads(out.getvalue().strip().splitlines()[-1])}))
'''


def test_gpu_arm_runs_through_on_cpu_stand_ins():
    code = "ROOT = %r\n" % ROOT + SCRIPT
    p = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=900, cwd=ROOT)
    assert p.returncode == 0, p.stderr[-3000:]
    res = json.loads(p.stdout.strip().splitlines()[-1])
    run, line = res["run"], res["line"]
    assert len(run["units"]) == 4
    for u in run["units"]:
        # stand-in timings of a busy host can round the rates to 0.0
        assert u["ms"] > 0 and u["gbs"] >= 0 and u["gflops_5nlog2n"] >= 0
        a = u["accuracy"]
        if u["dtype"] == "float":
            # the stand-in is the oracle itself: its error is the reference float build's
            assert a["relerr"] == a["ref_relerr"] <= a["bound"]
        else:
            assert a["bit_exact"]
    assert run["cpu"]["value"] > 0 and run["cpu"]["openmp_build"]["value"] > 0
    assert run["e2e"]["h2d_bytes_per_step"] > 0 and run["e2e"]["d2h_bytes_per_step"] > 0
    assert run["e2e"]["link"]["bidir_gbs"] > 0 and run["e2e"]["link"]["frac"] > 0
    assert run["roofline"]["bound"] == "hbm" and run["roofline"]["peak"] > 0
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
              "vs_baseline", "dtype", "data", "config", "roofline", "cpu_baseline", "e2e", "clocks", "gpu_launches",
              "units", "accuracy", "gflops_5nlog2n"):
        assert k in line, k
    assert line["accuracy"]["fixed_bit_exact"] and line["accuracy"]["float_within_bound"]
