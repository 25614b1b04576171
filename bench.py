"""Benchmark of the GPU KISS FFT path on one GB300.

Workload (default, "mixed-radix"): complex forward transforms at
nfft in {480, 1000, 3003, 65536} -- the kf_factor plans [4,4,2,3,5],
[4,2,5,5,5], [3,7,11,13] (generic radix) and [4]*8 (two HBM passes) -- each
with a batch of 256 MiB of input, for float32, Q15 and Q31 samples
(float inputs uniform[-1,1), fixed-point inputs uniform over the full
integer range, seed 1; synthetic, generated on the host).  One step runs
all 12 (type, size) batches once.  Every input batch is larger than the
129 MB L2, so no L2 flush is needed between steps.

Printed JSON line (one, on rank 0):
  value   whole-job HBM throughput, GB/s of compulsory bytes
          (2*N*sizeof(complex) per transform), inputs resident in HBM;
          gflops_5nlog2n gives the same run (and each unit) as
          5*N*log2(N) operations per transform
  accuracy  the outputs of the timed launches, first 64 transforms of every
          unit: float worst relative L2 error against FP64 beside the
          reference float build's own error on the same rows; Q15/Q31
          bit-exactness against the reference's fixed-point arithmetic
  e2e     the same through the drop-in C ABI with host (pinned) buffers,
          host<->device copies inside the timed region; its "link" entry is
          the measured copy-engine peak of the host link and the step's
          fraction of it
  roofline  the dominant kernel's achieved GB/s (its compulsory bytes per
          launch / its CUDA-event launch time) against the measured HBM peak
  cpu_baseline  the CPU restatement of the reference path (oracle/, OpenMP
          over transforms) on this host's cores, on a bounded sample; its
          "openmp_build" entry times the reference's own OpenMP form
          (KISSFFT_OPENMP=1: top-level radix legs of each transform in
          parallel) on a 1/64 sample
  batched_mix  the uneven-size mix (20,000 requests) as one batch replayed
          from a CUDA graph against the plain per-call form
  serving  the serving loop under Poisson arrivals offered at 50k..500k
          requests/s and held at 50k for 60 s: p50/p99 latency, throughput,
          host-link GB/s, saturated throughput, and the per-call form
  other_configs  the 1024-point round trip, real 4096 x 65536 forward and
          inverse, 2-D 2048^2 and real 3-D 128^3, each timed alone

--impl reference times that CPU path on the same workload instead.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))

SIZES = [480, 1000, 3003, 65536]
DTYPES = ["float", "int16_t", "int32_t"]
ESZ = {"float": 8, "double": 16, "int16_t": 4, "int32_t": 8}
BATCH_BYTES = 256 * 1024 * 1024
# DRAM bytes (read + write) per launch measured by ncu on these exact
# launches (profiles/ncu_q15_3003_generic_radix.md, profiles/ncu_dram_traffic_3003.md,
# profiles/ncu_fixed_point_bench_sizes.md); the write figure misses the
# dirty lines still in L2 when the capture ends
NCU_TRAFFIC = {("int16_t", 3003, 22347): 485.3e6, ("int32_t", 3003, 11173): 483.2e6,
               ("int16_t", 1000, 67108): 483.1e6, ("int32_t", 65536, 512): 486.7e6}


def c2c_flops(n, b):
    """Nominal operations of b complex transforms of n points: 5*n*log2(n)
    each, the usual FFT operation count (for Q15/Q31 these are integer
    operations counted the same way)."""
    return 5.0 * n * float(np.log2(n)) * b if n > 1 else 0.0


def device_rows(t, dt, n, k):
    """The first k transforms of a bench buffer (a torch tensor laid out as
    the bench uploads it: float32 (b, 2n) for float, (b, n, 2) integers for
    Q15/Q31) as a numpy array in the oracle's layout."""
    a = t[:k].cpu().numpy()
    if dt == "float":
        return a.view(np.complex64).reshape(k, n)
    return a.reshape(k, n, 2)


def accuracy(dt, n, x, y):
    """Accuracy of forward transforms y of the rows x: for float the worst
    per-row relative L2 error against an FP64 transform, beside the same for
    the reference float build's own output (the oracle, bit-identical to
    it) and the bound 2e-7*log2(n); for Q15/Q31 bit-exactness against the
    oracle (the reference's fixed-point build)."""
    from oracle import kfo
    ref = kfo.fft(x, 0, dt)
    if dt in ("int16_t", "int32_t"):
        return {"rows": int(x.shape[0]), "bit_exact": bool(np.array_equal(y, ref))}
    exact = np.fft.fft(x.astype(np.complex128), axis=-1)
    scale = np.linalg.norm(exact, axis=-1)
    scale[scale == 0] = 1

    def worst(a):
        return float(np.max(np.linalg.norm(a.astype(np.complex128) - exact, axis=-1) / scale))
    return {"rows": int(x.shape[0]), "relerr": worst(y), "ref_relerr": worst(ref),
            "bound": 2e-7 * max(1.0, float(np.log2(n)))}


def accuracy_summary(unit_rows):
    """The worst float error (and the reference float build's on the same
    rows) and whether every Q15/Q31 unit was bit-exact."""
    fl = [u["accuracy"] for u in unit_rows if "relerr" in u.get("accuracy", {})]
    fx = [u["accuracy"] for u in unit_rows if "bit_exact" in u.get("accuracy", {})]
    out = {"rows_per_unit": max([a["rows"] for a in fl + fx] or [0])}
    if fl:
        out["float_worst_relerr"] = max(a["relerr"] for a in fl)
        out["float_ref_worst_relerr"] = max(a["ref_relerr"] for a in fl)
        out["float_within_bound"] = all(a["relerr"] <= a["bound"] for a in fl)
    if fx:
        out["fixed_bit_exact"] = all(a["bit_exact"] for a in fx)
    return out


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d.get("hbm_gbs", 6800.0)), "measured"
    return 6800.0, "fallback"


_CASES = None


def units():
    if _CASES:
        return list(_CASES)
    out = []
    for dt in DTYPES:
        for n in SIZES:
            b = BATCH_BYTES // (n * ESZ[dt])
            out.append((dt, n, b))
    return out


def make_input(dt, n, b, seed=1):
    import inputs
    return inputs.cpx((b, n), dt, seed + n)


class ClockSampler(object):
    """nvidia-smi clock/throttle samples while the timed region runs."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index=0):
        self.rows = []
        self.proc = None
        self.gpu = gpu_index

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
        sm = [float(r[1]) for r in self.rows if len(r) > 8 and r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if len(r) > 8 and r[2].replace(".", "").isdigit()]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            if len(r) > 8:
                for k, nm in enumerate(names):
                    if r[5 + k].lower().startswith("active"):
                        reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ------------------------------------------------------------------ GPU arm
def run_gpu(args):
    import torch

    import kissfft_gb300 as kf

    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    stream = torch.cuda.current_stream()
    us = units()
    cfgs, xs, ys, host_in = [], [], [], []
    for dt, n, b in us:
        x = make_input(dt, n, b)
        host_in.append(x)
        xv = x.view(np.float32) if dt == "float" else x
        xt = torch.from_numpy(np.ascontiguousarray(xv)).to(dev)
        xs.append(xt)
        ys.append(torch.empty_like(xt))
        cfgs.append(kf.kiss_fft_alloc(n, 0, dt))
    launches_per_unit = [kf.plan_info(c)[3] for c in cfgs]  # HBM passes = kernel launches
    kf.set_specialize(args.specialize)
    t_prep = time.perf_counter()
    for c, (dt, n, b) in zip(cfgs, us):
        if args.autotune:
            kf.autotune(c, b)
        kf.prepare(c, b)
    t_prep = time.perf_counter() - t_prep

    def step(events=None):
        for i, (dt, n, b) in enumerate(us):
            if events is not None:
                events[i][0].record(stream)
            kf.kiss_fft_batch(cfgs[i], xs[i], ys[i], b)
            if events is not None:
                events[i][1].record(stream)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    # timed region: whole steps, device time
    clk = ClockSampler()
    clk.start()
    time.sleep(0.3)
    t0 = torch.cuda.Event(enable_timing=True)
    t1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    t0.record(stream)
    for _ in range(args.steps):
        step()
    t1.record(stream)
    torch.cuda.synchronize()
    clocks = clk.stop()
    ms = t0.elapsed_time(t1) / args.steps
    alg_bytes = sum(2 * n * ESZ[dt] * b for dt, n, b in us)
    value = alg_bytes / (ms * 1e-3) / 1e9
    # per-unit launch times: each unit launched back to back between two
    # events (the device never waits for the host inside the bracket), every
    # launch re-reading its >L2 input from HBM
    per = [0.0] * len(us)
    reps = max(3, args.steps)
    for i, (dt, n, b) in enumerate(us):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        kf.kiss_fft_batch(cfgs[i], xs[i], ys[i], b)  # keeps the device busy while the bracket is queued
        e0.record(stream)
        for _ in range(reps):
            kf.kiss_fft_batch(cfgs[i], xs[i], ys[i], b)
        e1.record(stream)
        torch.cuda.synchronize()
        per[i] = e0.elapsed_time(e1) / reps
    unit_rows = []
    for i, (dt, n, b) in enumerate(us):
        byts = 2 * n * ESZ[dt] * b
        unit_rows.append({"dtype": dt, "nfft": n, "batch": b, "ms": round(per[i], 4),
                          "gbs": round(byts / (per[i] * 1e-3) / 1e9, 1),
                          "gflops_5nlog2n": round(c2c_flops(n, b) / (per[i] * 1e-3) / 1e9, 1),
                          "launches": launches_per_unit[i]})
    # accuracy of the outputs just timed, on the first 64 transforms of every unit
    for i, (dt, n, b) in enumerate(us):
        k = min(b, 64)
        unit_rows[i]["accuracy"] = accuracy(dt, n, host_in[i][:k], device_rows(ys[i], dt, n, k))
    dom = max(range(len(us)), key=lambda i: per[i])
    peak, peak_kind = peaks()
    dt_, n_, b_ = us[dom]
    dom_bytes = 2 * n_ * ESZ[dt_] * b_
    achieved = dom_bytes / (per[dom] * 1e-3) / 1e9
    roof = {"bound": "hbm", "kernel": "engine kernel %s nfft=%d batch=%d (%d launch%s)" % (
        dt_, n_, b_, launches_per_unit[dom], "es" if launches_per_unit[dom] > 1 else ""),
        "achieved": round(achieved, 1), "peak": peak, "peak_source": peak_kind, "unit": "GB/s",
        "frac": round(achieved / peak, 4),
        "traffic": args.traffic if args.traffic is not None else NCU_TRAFFIC.get((dt_, n_, b_)),
        "traffic_unit": "DRAM bytes per launch (ncu)", "algorithmic_bytes": dom_bytes}
    # e2e: host pinned buffers through the C ABI (H2D + D2H inside the timed region)
    e2e = None
    if not args.no_e2e:
        hin = [torch.from_numpy(np.ascontiguousarray(x.view(np.float32) if dt == "float" else x)).pin_memory()
               for x, (dt, n, b) in zip(host_in, us)]
        hout = [torch.empty_like(h).pin_memory() for h in hin]
        for _ in range(args.warmup):  # W warm-up steps of the host path too
            for i, (dt, n, b) in enumerate(us):
                kf.kiss_fft_batch(cfgs[i], hin[i], hout[i], b)
        e_steps = max(3, min(args.steps, 5))
        torch.cuda.synchronize()
        ts = time.perf_counter()
        for _ in range(e_steps):
            for i, (dt, n, b) in enumerate(us):
                kf.kiss_fft_batch(cfgs[i], hin[i], hout[i], b)
        torch.cuda.synchronize()
        e_ms = (time.perf_counter() - ts) * 1e3 / e_steps
        h2d = sum(h.numel() * h.element_size() for h in hin)
        # per unit, the same calls one unit at a time
        e_units = []
        for i, (dt, n, b) in enumerate(us):
            torch.cuda.synchronize()
            tu = time.perf_counter()
            for _ in range(e_steps):
                kf.kiss_fft_batch(cfgs[i], hin[i], hout[i], b)
            torch.cuda.synchronize()
            u_ms = (time.perf_counter() - tu) * 1e3 / e_steps
            e_units.append({"dtype": dt, "nfft": n, "ms": round(u_ms, 3),
                            "gbs": round(2 * n * ESZ[dt] * b / (u_ms * 1e-3) / 1e9, 1)})
        e2e = {"value": round(alg_bytes / (e_ms * 1e-3) / 1e9, 2), "unit": "GB/s", "h2d_bytes_per_step": h2d,
               "d2h_bytes_per_step": h2d, "ms_per_step": round(e_ms, 3),
               "path": "pinned host buffers: single-step row-tile schedules read and write them in place over the "
                       "host link; two-pass and column-tile schedules run a chunked copy-in / kernels / copy-out "
                       "pipeline on three streams",
               "units": e_units}
        link = link_peak()
        moved = (h2d + h2d) / (e_ms * 1e-3) / 1e9  # host-link bytes of a step, both directions
        e2e["link"] = dict(link, step_link_gbs=round(moved, 1),
                           frac=round(moved / link["bidir_gbs"], 3) if link["bidir_gbs"] > 0 else None)
        # the e2e output must equal the device-resident output
        for i in range(len(us)):
            if not torch.equal(hout[i], ys[i].cpu()):
                raise RuntimeError("e2e output differs from device output for %s" % (us[i],))
    mix = None
    if not args.no_mix:
        mix = run_mix(args)
    serving = None
    if not args.no_serve:
        serving = run_serving(args)
    others = None
    if not args.no_configs:
        others = run_configs(args)
    cpu = None
    if not args.no_cpu:
        from oracle import kfo
        nth = kfo.max_threads()
        g, secs, passes = run_cpu(host_in, nth, args.cpu_seconds)
        gp, secs_p, passes_p = run_cpu(host_in, nth, min(5.0, args.cpu_seconds), release=False)
        cpu = {"value": round(g, 3), "unit": "GB/s", "cores": nth, "kind": "port",
               "sample": "the whole workload (all 12 batches) %d time(s), %.1f s of CPU work" % (passes, secs),
               "form": "OpenMP over the transforms of each batch (one plan per thread)", "build": REL_BUILD,
               "parity_build": {"value": round(gp, 3), "build": PARITY_BUILD,
                                "sample": "the whole workload %d time(s), %.1f s" % (passes_p, secs_p)}}
        cpu["openmp_build"] = legs_entry(host_in, nth, min(3.0, args.cpu_seconds), 1.0 / 64)
    gflops = sum(c2c_flops(n, b) for dt, n, b in us) / (ms * 1e-3) / 1e9
    return {"value": value, "gflops": gflops, "ms": ms, "units": unit_rows, "roofline": roof, "e2e": e2e,
            "clocks": clocks, "cpu": cpu,
            "gpu_launches": args.steps * sum(launches_per_unit), "alg_bytes": alg_bytes,
            "prepare_s": round(t_prep, 2), "mix": mix, "serving": serving, "others": others}


# ------------------------------------------------------------------ uneven mix
MIX_COUNT = 20000


def run_mix(args, count=MIX_COUNT):
    """Batched uneven-size mix (20,000 requests, seed 3; uneven_mix in
    tests/golden/inputs.py): one kfg_batch of all requests in two arenas, its launch shape
    (threads per tile) picked by timing the candidates, captured in a CUDA
    graph and replayed, against the plain per-call form (one kfg_exec_batch
    per request, precompiled kernels) on the same arenas.  Returns GB/s of
    compulsory bytes (input + output of every request) for both forms."""
    import ctypes

    import torch

    import inputs
    import kissfft_gb300 as kf

    L = kf.core()
    vp, ll, ci = ctypes.c_void_p, ctypes.c_longlong, ctypes.c_int
    L.kfg_batch_create.restype = vp
    L.kfg_batch_add.argtypes = [vp, ci, ci, ci, ll, ll]
    L.kfg_batch_commit.argtypes = [vp, vp, vp, ci]
    for fn in ("kfg_batch_run", "kfg_batch_capture", "kfg_batch_run_percall"):
        getattr(L, fn).argtypes = [vp, vp]
    L.kfg_batch_info.argtypes = [vp, vp, ci]
    L.kfg_batch_free.argtypes = [vp]
    kf.set_specialize(False)  # thousands of distinct plans: precompiled kernels in both forms
    mix = inputs.uneven_mix(count, seed=3)
    kinds = {"c2c": 1, "r2c": 2}
    dts = {"float": 0, "int16_t": 2}
    reqs, io, oo = [], 0, 0
    for kind, d, n in mix:
        esz = ESZ[d]
        ib = n * esz if kind == "c2c" else n * 4
        ob = n * esz if kind == "c2c" else (n // 2 + 1) * 8
        reqs.append((kinds[kind], dts[d], n, io, oo, ib, ob))
        io = (io + ib + 255) // 256 * 256
        oo = (oo + ob + 255) // 256 * 256
    alg = sum(r[5] + r[6] for r in reqs)
    gen = torch.Generator(device="cuda")
    gen.manual_seed(3)
    ind = (torch.rand(io // 4, device="cuda", generator=gen) * 2 - 1).view(torch.uint8)  # uniform[-1, 1)
    q15 = torch.zeros(io, dtype=torch.bool, device="cuda")
    for r in reqs:
        if r[1] == 2:
            q15[r[3]:r[3] + r[5]] = True
    ind[q15] = torch.randint(0, 256, (int(q15.sum()),), dtype=torch.uint8, device="cuda", generator=gen)
    outd = torch.zeros(oo, dtype=torch.uint8, device="cuda")
    st = vp(torch.cuda.current_stream().cuda_stream)
    stream = torch.cuda.current_stream()

    def commit(target):
        B = L.kfg_batch_create()
        for r in reqs:
            if L.kfg_batch_add(B, r[0], r[1], r[2], r[3], r[4]) != 0:
                raise RuntimeError(L.kfg_last_error().decode())
        if L.kfg_batch_commit(B, vp(ind.data_ptr()), vp(outd.data_ptr()), target) != 0:
            raise RuntimeError(L.kfg_last_error().decode())
        return B

    def timed(fn, steps):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(steps):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / steps

    t_commit = time.perf_counter()
    best = None
    for target in (128, 256, 512):  # autotune: threads per tile the launches are widened towards
        B = commit(target)
        L.kfg_batch_run(B, st)
        ms = timed(lambda: L.kfg_batch_run(B, st), 3)
        if best is None or ms < best[1]:
            if best is not None:
                L.kfg_batch_free(best[0])
            best = (B, ms, target)
        else:
            L.kfg_batch_free(B)
    B, _, target = best
    t_commit = time.perf_counter() - t_commit
    info = (ctypes.c_longlong * 5)()
    L.kfg_batch_info(B, info, 5)
    direct_ms = timed(lambda: L.kfg_batch_run(B, st), max(3, args.steps // 3))
    if L.kfg_batch_capture(B, st) != 0:
        raise RuntimeError(L.kfg_last_error().decode())
    for _ in range(args.warmup):
        L.kfg_batch_run(B, st)
    graph_ms = timed(lambda: L.kfg_batch_run(B, st), max(3, args.steps))
    got = outd.clone()
    L.kfg_batch_run_percall(B, st)  # warm-up
    percall_ms = timed(lambda: L.kfg_batch_run_percall(B, st), 3)
    ref = outd
    # equal accuracy: both forms give the same transforms (Q15 bit for bit)
    worst = 0.0
    for r in reqs:
        a, b = got[r[4]:r[4] + r[6]], ref[r[4]:r[4] + r[6]]
        if r[1] == 2:
            if not torch.equal(a, b):
                raise RuntimeError("batched Q15 result differs from the per-call form (nfft %d)" % r[2])
        else:
            av, bv = a.view(torch.float32).double(), b.view(torch.float32).double()
            worst = max(worst, float((av - bv).norm() / bv.norm().clamp_min(1e-30)))
    L.kfg_batch_free(B)
    single = percall_single(L, st)
    distinct = len(set((r[0], r[1], r[2]) for r in reqs))
    peak, _ = peaks()
    # the mix's own ceiling: compulsory bytes plus the intermediate round
    # trip of every request longer than one shared tile (written, read back)
    ceil_bytes = alg + int(info[4])
    return {"workload": "uneven mix: %d requests, nfft log-uniform [16, 131072], 80%% 2^a3^b5^c / 20%% with a "
                        "prime 7..31; 60%% c2c f32, 30%% r2c f32, 10%% c2c Q15; seed 3" % count,
            "requests": count, "distinct_plans": distinct, "compulsory_bytes": alg,
            "intermediate_bytes": int(info[4]),
            "graph": {"ms": round(graph_ms, 3), "gbs": round(alg / graph_ms / 1e6, 1),
                      "frac_compulsory": round(alg / graph_ms / 1e6 / peak, 3),
                      "hbm_gbs_with_intermediates": round(ceil_bytes / graph_ms / 1e6, 1),
                      "frac_of_own_ceiling": round(ceil_bytes / graph_ms / 1e6 / peak, 3)},
            "direct": {"ms": round(direct_ms, 3), "gbs": round(alg / direct_ms / 1e6, 1)},
            "percall": {"ms": round(percall_ms, 3), "gbs": round(alg / percall_ms / 1e6, 1),
                        "us_per_request": round(percall_ms * 1e3 / count, 2)},
            "percall_us": single,
            "speedup_vs_percall": round(percall_ms / graph_ms, 2),
            "autotuned_target_threads": target, "launches": int(info[2]), "tiles": int(info[3]),
            "max_rel_diff_vs_percall": worst, "commit_and_tune_s": round(t_commit, 2)}


def run_mix_runs(args):
    """Profiling form of the uneven mix: one kfg_batch of the 20,000 requests
    (256 threads per tile), run --steps times back to back (no per-call form)."""
    import ctypes

    import torch

    import inputs
    import kissfft_gb300 as kf

    L = kf.core()
    vp, ll, ci = ctypes.c_void_p, ctypes.c_longlong, ctypes.c_int
    L.kfg_batch_create.restype = vp
    L.kfg_batch_add.argtypes = [vp, ci, ci, ci, ll, ll]
    L.kfg_batch_commit.argtypes = [vp, vp, vp, ci]
    L.kfg_batch_run.argtypes = [vp, vp]
    L.kfg_batch_free.argtypes = [vp]
    kf.set_specialize(False)
    kinds, dts = {"c2c": 1, "r2c": 2}, {"float": 0, "int16_t": 2}
    B = L.kfg_batch_create()
    io = oo = 0
    for kind, d, n in inputs.uneven_mix(MIX_COUNT, seed=3):
        ib = n * ESZ[d] if kind == "c2c" else n * 4
        ob = n * ESZ[d] if kind == "c2c" else (n // 2 + 1) * 8
        L.kfg_batch_add(B, kinds[kind], dts[d], n, io, oo)
        io = (io + ib + 255) // 256 * 256
        oo = (oo + ob + 255) // 256 * 256
    ind = torch.zeros(io, dtype=torch.uint8, device="cuda")
    outd = torch.zeros(oo, dtype=torch.uint8, device="cuda")
    if L.kfg_batch_commit(B, vp(ind.data_ptr()), vp(outd.data_ptr()), 256) != 0:
        raise RuntimeError(L.kfg_last_error().decode())
    st = vp(torch.cuda.current_stream().cuda_stream)
    times = []
    for _ in range(max(1, args.steps)):
        torch.cuda.synchronize()
        t = time.perf_counter()
        L.kfg_batch_run(B, st)
        torch.cuda.synchronize()
        times.append((time.perf_counter() - t) * 1e3)
    L.kfg_batch_free(B)
    return {"runs_ms": [round(x, 3) for x in times]}


def run_serve_burst(args):
    """Profiling form of the serving loop: 3,000 requests of the serving mix
    submitted at once (seed 5), 40 GB budget, 4 slots."""
    import kissfft_gb300 as kf

    kf.set_specialize(False)
    srv = kf.Server(hbm_budget=40 << 30, slots=4)
    try:
        r = srv.loadtest(rate=0.0, count=3000, seed=5, percall_max=0)
    finally:
        srv.close()
    return r


# ------------------------------------------------------------------ other workloads
def _configs_1d(args, kf, inputs, dev, timed, row):
    """The 1024-point forward + inverse round trip on 4096 transforms and the
    real 4096-point forward / inverse pair on 65536 rows, for run_configs."""
    import torch

    out = {}
    x = torch.from_numpy(inputs.cpx((4096, 1024), "float", 0).view(np.float32).copy()).to(dev)
    y = torch.empty_like(x)
    z = torch.empty_like(x)
    fw, iv = kf.kiss_fft_alloc(1024, 0), kf.kiss_fft_alloc(1024, 1)
    for c in (fw, iv):
        kf.autotune(c, 4096)
        kf.prepare(c, 4096)
    fn = lambda: (kf.kiss_fft_batch(fw, x, y, 4096), kf.kiss_fft_batch(iv, y, z, 4096))  # noqa: E731
    out["c2c_1024_fwd_inv_4096"] = row(2 * 2 * 1024 * 8 * 4096, timed(fn), "32 MiB each way: L2-resident", fn)
    del x, y, z
    # real 4096-point rows x 65536 (1 GiB of reals)
    B, N = 65536, 4096
    g = torch.Generator(device=dev)
    g.manual_seed(2)
    t = torch.arange(N, device=dev, dtype=torch.float32)
    tr = torch.empty((B, N), device=dev, dtype=torch.float32)
    for r0 in range(0, B, 8192):
        f = torch.rand((8192, 3, 1), device=dev, generator=g) * (N / 2)
        ph = torch.rand((8192, 3, 1), device=dev, generator=g) * 6.283185307179586
        tr[r0:r0 + 8192] = torch.cos(6.283185307179586 * f * t / N + ph).sum(1) + \
            0.1 * torch.randn((8192, N), device=dev, generator=g)
    fr = torch.empty((B, N // 2 + 1, 2), device=dev, dtype=torch.float32)
    back = torch.empty_like(tr)
    rf, ri = kf.kiss_fftr_alloc(N, 0), kf.kiss_fftr_alloc(N, 1)
    for c in (rf, ri):
        kf.autotune(c, B)
        kf.prepare(c, B)
    rbytes = (4 * N + 8 * (N // 2 + 1)) * B
    fn = lambda: kf.kiss_fftr_batch(rf, tr, fr, B)  # noqa: E731
    out["r2c_4096_65536"] = row(rbytes, timed(fn), "1 GiB in", fn)
    fn = lambda: kf.kiss_fftri_batch(ri, fr, back, B)  # noqa: E731
    out["c2r_4096_65536"] = row(rbytes, timed(fn), "1 GiB out", fn)
    del tr, fr, back
    return out


def run_configs(args):
    """The reference's other workloads, each timed alone (back-to-back
    launches between two events, after a warm launch): the 1024-point
    forward+inverse round trip on 4096 transforms (seed 0); kiss_fftr and
    kiss_fftri at nfft 4096 on 65536 rows of 3 unit sinusoids + N(0, 0.1^2)
    noise (generated on the device, seed 2); kiss_fftnd on a 2048x2048
    complex array; kiss_fftndr / kiss_fftndri on a 128^3 real array (every
    plan autotuned and its specialised kernels compiled first).  GB/s of
    compulsory bytes (c2c 2*N*8, r2c 4N + 8(N/2+1), nd 2*prod*8, ndr
    4*prod + 8*prod/N*(N/2+1) per transform).  Each row also carries
    `graph`: ten of the same calls captured in one CUDA graph and replayed,
    the device time without the per-call host work and launch gaps."""
    import torch

    import inputs
    import kissfft_gb300 as kf

    dev = torch.device("cuda", 0)
    stream = torch.cuda.current_stream()
    peak, _ = peaks()
    reps = max(3, args.steps // 2)
    kf.set_specialize(args.specialize)

    def timed(fn):
        torch.cuda.synchronize()
        fn()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / reps

    def graph_timed(fn, calls=10):
        # the same calls captured once in a CUDA graph and replayed: device
        # time without the host's per-call work and launch gaps
        g = torch.cuda.CUDAGraph()
        cs = torch.cuda.Stream()
        cs.wait_stream(stream)
        with torch.cuda.graph(g, stream=cs, capture_error_mode="thread_local"):
            for _ in range(calls):
                fn()
        stream.wait_stream(cs)
        g.replay()
        ms = timed(g.replay) / calls
        del g
        return ms

    def row(byts, ms, note, fn=None):
        r = {"ms": round(ms, 4), "gbs": round(byts / ms / 1e6, 1), "frac_of_measured_peak": round(byts / ms / 1e6 / peak, 3),
             "note": note}
        if fn is not None:
            gms = graph_timed(fn)
            r["graph"] = {"ms": round(gms, 4), "gbs": round(byts / gms / 1e6, 1),
                          "frac_of_measured_peak": round(byts / gms / 1e6 / peak, 3)}
        return r

    out = {}
    nd_only = args.only == "nd"  # the N-D workloads alone (small: 32 MiB and 8 MiB arrays)
    if not nd_only:
        out.update(_configs_1d(args, kf, inputs, dev, timed, row))
    # 2-D complex 2048^2 and 3-D real 128^3
    a = torch.from_numpy(inputs.cpx((2048, 2048), "float", 2).view(np.float32).copy()).to(dev)
    b = torch.empty_like(a)
    nd = kf.kiss_fftnd_alloc([2048, 2048], 0)
    kf.autotune(nd, 1)
    kf.prepare(nd, 1)
    fn = lambda: kf.kiss_fftnd(nd, a, b)  # noqa: E731
    out["nd_2048x2048"] = row(2 * 2048 * 2048 * 8, timed(fn), "32 MiB: L2-resident", fn)
    rng = np.random.default_rng(2)
    v = torch.from_numpy(rng.standard_normal((128, 128, 128)).astype(np.float32)).to(dev)
    w = torch.empty((128, 128, 65, 2), device=dev, dtype=torch.float32)
    v2 = torch.empty_like(v)
    ndr, ndri = kf.kiss_fftndr_alloc([128, 128, 128], 0), kf.kiss_fftndr_alloc([128, 128, 128], 1)
    for c in (ndr, ndri):
        kf.autotune(c, 1)
        kf.prepare(c, 1)
    nbytes = 4 * 128 ** 3 + 8 * 128 * 128 * 65
    fn = lambda: kf.kiss_fftndr(ndr, v, w)  # noqa: E731
    out["ndr_128^3"] = row(nbytes, timed(fn), "8 MiB: L2-resident", fn)
    fn = lambda: kf.kiss_fftndri(ndri, w, v2)  # noqa: E731
    out["ndri_128^3"] = row(nbytes, timed(fn), "8 MiB: L2-resident", fn)
    return out


# ------------------------------------------------------------------ serving loop
def run_serving(args):
    """Serving loop (kfg_server, 40 GB HBM budget) on a mix of c2c (N
    log-uniform 64..65536), r2c, 2-D (256..1024 per side) and fast-FIR
    (255..4095 taps, 2^16..2^22 samples) requests in equal shares (seed 4),
    inputs and outputs in pinned host memory: Poisson arrivals offered at
    50k, 100k, 200k and 500k requests/s (each for at most 3 s and 150,000
    requests), then held at 50,000 requests/s for --serve-hold seconds
    (default 60); then the same mix submitted all at once (the loop's
    saturated throughput); then the first 2,000 requests of the held run
    through the plain per-call form.  Latency is submit to completion,
    p50/p99; link_gbs counts the requests' bytes over the host link."""
    import kissfft_gb300 as kf

    kf.set_specialize(False)
    srv = kf.Server(hbm_budget=40 << 30, slots=4)
    try:
        # warm the device plan cache with the mix's sizes (a burst of the same seed)
        srv.loadtest(rate=0.0, count=5000, seed=4, percall_max=0)
        sweep = []
        for rate in (50000.0, 100000.0, 200000.0, 500000.0):
            # offered for at most 3 s and 150,000 requests; the loop drains what it admitted
            secs = min(3.0, 150000.0 / rate)
            r = srv.loadtest(rate=rate, seconds=secs, seed=4, percall_max=0)
            sweep.append(serve_row(rate, secs, r))
        poisson = srv.loadtest(rate=50000.0, seconds=args.serve_hold, seed=4, percall_max=2000)
        sat = srv.loadtest(rate=0.0, count=20000, seed=5, percall_max=0)
    finally:
        srv.close()
    ps, ss = poisson["served"], sat["served"]
    return {"workload": "Poisson arrivals; c2c/r2c N 64..65536, 2-D 256..1024 per side, fast FIR 255..4095 "
                        "taps on 2^16..2^22 samples, equal shares, float32, pinned host buffers; seed 4; "
                        "HBM budget 40 GB",
            "held": dict(serve_row(50000.0, args.serve_hold, poisson), batches=ps["batches"],
                         peak_hbm_gb=round(ps["peak_hbm_bytes"] / 1e9, 3)),
            "sweep": sweep,
            "saturated": {"requests": sat["offered"], "req_per_s": round(ss["req_per_s"], 1),
                          "gbs": round(ss["gbs"], 2), "p50_ms": round(ss["p50_s"] * 1e3, 3),
                          "p99_ms": round(ss["p99_s"] * 1e3, 3), "host_busy_s": round(ss["host_s"], 3)},
            "percall": {"requests": poisson["percall_count"], "req_per_s": round(poisson["percall_req_per_s"], 1),
                        "gbs": round(poisson["percall_gbs"], 2), "p50_ms": round(poisson["percall_p50_s"] * 1e3, 3),
                        "p99_ms": round(poisson["percall_p99_s"] * 1e3, 3)},
            "saturated_vs_percall": round(ss["req_per_s"] / max(poisson["percall_req_per_s"], 1e-9), 2)}


def serve_row(rate, secs, r):
    """One offered rate of the serving loop: latency, what completed, host
    time, host-link bytes."""
    sv = r["served"]
    return {"offered_req_per_s": rate, "seconds": round(secs, 3), "offered": r["offered"],
            "completed": sv["completed"], "failed": sv["failed"], "req_per_s": round(sv["req_per_s"], 1),
            "p50_ms": round(sv["p50_s"] * 1e3, 3), "p99_ms": round(sv["p99_s"] * 1e3, 3),
            "link_gbs": round(sv["gbs"], 2), "host_busy_s": round(sv["host_s"], 3)}


def link_peak(mib=512, reps=3):
    """Measured copy-engine bandwidth of the host link on page-locked
    buffers (cudaMemcpyAsync through torch copies, CUDA events, best of
    reps): host to device, device to host, and both at once on two streams
    (GB/s of bytes moved)."""
    import torch
    nb = mib << 20
    h1 = torch.empty(nb, dtype=torch.uint8).pin_memory()
    h2 = torch.empty(nb, dtype=torch.uint8).pin_memory()
    d1 = torch.empty(nb, dtype=torch.uint8, device="cuda")
    d2 = torch.empty(nb, dtype=torch.uint8, device="cuda")
    s1, s2 = torch.cuda.Stream(), torch.cuda.Stream()

    def best(fn):
        b = None
        for _ in range(reps + 1):
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            fn()
            e1.record()
            torch.cuda.synchronize()
            ms = e0.elapsed_time(e1)
            b = ms if b is None else min(b, ms)
        return b

    def both():
        ev = torch.cuda.Event()
        ev.record()
        for st, f in ((s1, lambda: d1.copy_(h1, non_blocking=True)), (s2, lambda: h2.copy_(d2, non_blocking=True))):
            st.wait_event(ev)
            with torch.cuda.stream(st):
                f()
        cur = torch.cuda.current_stream()
        cur.wait_stream(s1)
        cur.wait_stream(s2)

    t_h2d = best(lambda: d1.copy_(h1, non_blocking=True))
    t_d2h = best(lambda: h2.copy_(d2, non_blocking=True))
    t_bi = best(both)
    del h1, h2, d1, d2
    return {"h2d_gbs": round(nb / (t_h2d * 1e-3) / 1e9, 1), "d2h_gbs": round(nb / (t_d2h * 1e-3) / 1e9, 1),
            "bidir_gbs": round(2 * nb / (t_bi * 1e-3) / 1e9, 1),
            "how": "cudaMemcpyAsync of %d MiB page-locked buffers, CUDA events, best of %d" % (mib, reps)}


def percall_single(L, st, n=1024, calls=5000):
    """Host cost of one plain drop-in call: a 1024-point float forward
    transform on device buffers (kfg_exec, enqueued on the stream), timed
    over `calls` back-to-back calls from Python (ctypes), with the
    plan-specialised kernels and with the precompiled family kernels, and
    the cost of a ctypes call that does nothing beside them."""
    import ctypes
    import torch

    import kissfft_gb300 as kf
    vp = ctypes.c_void_p
    p = L.kfg_plan_c2c(0, n, 0)
    x = torch.randn(2 * n, device="cuda")
    y = torch.empty_like(x)
    xa, ya = vp(x.data_ptr()), vp(y.data_ptr())

    def per_call(spec):
        kf.set_specialize(spec)
        for _ in range(200):
            L.kfg_exec(p, xa, ya, st)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(calls):
            L.kfg_exec(p, xa, ya, st)
        t1 = time.perf_counter()
        torch.cuda.synchronize()
        return (t1 - t0) / calls * 1e6

    us_spec = per_call(True)
    us_fam = per_call(False)
    t1 = time.perf_counter()
    for _ in range(calls):
        L.kfg_get_stream()
    t2 = time.perf_counter()
    L.kfg_plan_free(p)
    return {"nfft": n, "us": round(us_spec, 2), "us_precompiled": round(us_fam, 2),
            "python_ctypes_us": round((t2 - t1) / calls * 1e6, 2), "calls": calls,
            "what": "kfg_exec on device buffers, host time per call including the Python call; us: plan-specialised "
                    "kernels, us_precompiled: the precompiled family kernels"}


# ------------------------------------------------------------------ CPU arm
REL_BUILD = "-O3 -ffast-math -fomit-frame-pointer (the reference's CMake release flags, CMakeLists.txt:98-102)"
PARITY_BUILD = "-O2 -ffp-contract=off (the parity build the tests check against)"


def run_cpu(host_in, nthreads, min_seconds, release=True):
    """The oracle (CPU restatement of the reference path, OpenMP over the
    transforms of a batch) on the bench's own input batches, whole passes
    repeated until at least min_seconds of wall time; returns GB/s of
    compulsory bytes, the seconds and the passes.  release: the build at the
    reference's release flags (else the -O2 parity build)."""
    from oracle import kfo
    us = units()
    tot_bytes, tot_s, passes = 0, 0.0, 0
    while tot_s < min_seconds or passes == 0:
        for x, (dt, n, b) in zip(host_in, us):
            ts = time.perf_counter()
            kfo.fft(x, 0, dt, nthreads=nthreads, release=release)
            tot_s += time.perf_counter() - ts
            tot_bytes += 2 * n * ESZ[dt] * b
        passes += 1
    return tot_bytes / tot_s / 1e9, tot_s, passes


def run_cpu_legs(host_in, nthreads, min_seconds, frac=1.0 / 64):
    """The reference's own OpenMP build as configured (KISSFFT_OPENMP=1):
    transforms one after the other, the top-level radix legs of each split
    over OpenMP threads (kiss_fft.c:250-272), on the first ``frac`` of every
    input batch, whole passes repeated until at least min_seconds; returns
    the same fields as run_cpu plus the sample's transform count."""
    from oracle import kfo
    us = units()
    parts = [(x[:max(1, int(b * frac))], dt, n, max(1, int(b * frac))) for x, (dt, n, b) in zip(host_in, us)]
    tot_bytes, tot_s, passes = 0, 0.0, 0
    while tot_s < min_seconds or passes == 0:
        for x, dt, n, k in parts:
            ts = time.perf_counter()
            kfo.fft_legs(x, 0, dt, nthreads=nthreads, release=True)
            tot_s += time.perf_counter() - ts
            tot_bytes += 2 * n * ESZ[dt] * k
        passes += 1
    return tot_bytes / tot_s / 1e9, tot_s, passes, sum(k for _, _, _, k in parts)


def legs_entry(host_in, nthreads, min_seconds, frac, base_frac=1.0):
    """run_cpu_legs as a JSON object; host_in holds base_frac of every full batch."""
    g, secs, passes, count = run_cpu_legs(host_in, nthreads, min_seconds, frac)
    return {"value": round(g, 3), "unit": "GB/s", "cores": nthreads, "kind": "port",
            "sample": "1/%d of every batch (%d transforms), %d pass(es), %.1f s" % (round(1 / (frac * base_frac)),
                                                                                      count, passes, secs),
            "form": "KISSFFT_OPENMP=1: transforms in sequence, top-level radix legs (p <= 5) in parallel"}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=30)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cpu-frac", type=float, default=1.0 / 8,
                    help="reference arm: fraction of every batch one step runs on the CPU")
    ap.add_argument("--cpu-seconds", type=float, default=10.0,
                    help="CPU baseline of the GPU arm: minimum seconds of CPU work")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-mix", action="store_true", help="skip the batched uneven-mix measurement")
    ap.add_argument("--no-serve", action="store_true", help="skip the serving-loop measurement")
    ap.add_argument("--serve-hold", type=float, default=60.0,
                    help="seconds the serving loop is held at 50,000 requests/s")
    ap.add_argument("--no-configs", action="store_true", help="skip the real / N-D / round-trip workloads")
    ap.add_argument("--only", choices=["mix", "serve", "configs", "nd", "mix-runs", "serve-burst"], default=None,
                    help="run only one measurement and print it: the uneven mix, serving, the other workloads "
                         "(configs) or their N-D part (nd), the mix's launch runs, a serving burst")
    ap.add_argument("--traffic", type=float, default=None,
                    help="dram bytes per launch of the dominant kernel from an ncu capture")
    ap.add_argument("--specialize", type=int, default=1,
                    help="1: plan-specialised kernels (compiled before warm-up); 0: precompiled family kernels")
    ap.add_argument("--autotune", type=int, default=1,
                    help="1: time candidate tile shapes per batch before warm-up (cached on disk)")
    ap.add_argument("--case", action="append", default=[],
                    help="run only these units, TYPE:NFFT:BATCH (profiling runs)")
    args = ap.parse_args()
    args.warmup = max(3, args.warmup)
    global _CASES
    if args.case:
        _CASES = []
        for c in args.case:
            dt, n, b = c.split(":")
            _CASES.append((dt, int(n), int(b)))
        args.no_e2e = args.no_cpu = args.no_mix = args.no_serve = args.no_configs = True
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    config = {"workload": "mixed-radix complex forward: nfft 480,1000,3003,65536 x float32,Q15,Q31, "
                          "256 MiB input per batch", "sizes": SIZES, "dtypes": DTYPES,
              "batches": [b for _, _, b in units()], "l2": "inputs larger than L2 (256 MiB per batch)"}
    if args.impl == "reference":
        if rank != 0:
            return
        from oracle import kfo
        nth = kfo.max_threads()
        host_in = [make_input(dt, n, max(1, int(b * args.cpu_frac))) for dt, n, b in units()]
        _CASES = [(dt, n, max(1, int(b * args.cpu_frac))) for dt, n, b in units()]
        for _ in range(args.warmup):
            run_cpu(host_in, nth, 0)
        per = []
        for _ in range(args.steps):
            g, s, _p = run_cpu(host_in, nth, 0)
            per.append(g)
        v = statistics.median(per)
        gp, _s, _p = run_cpu(host_in, nth, 0, release=False)
        sample = "each step: one pass over %s of every batch (%d transforms)" % (
            "all" if args.cpu_frac >= 1 else "1/%d" % round(1 / args.cpu_frac), sum(b for _, _, b in _CASES))
        line = {"impl": "reference", "metric": "HBM GB/s (compulsory bytes), batched FFT", "value": round(v, 3),
                "unit": "GB/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32+q15+q31",
                "data": "synthetic", "config": config,
                "cpu_baseline": {"value": round(v, 3), "unit": "GB/s", "cores": nth, "kind": "port",
                                 "sample": sample,
                                 "form": "OpenMP over the transforms of each batch (one plan per thread)",
                                 "build": REL_BUILD,
                                 "parity_build": {"value": round(gp, 3), "build": PARITY_BUILD,
                                                  "sample": "one pass of the same sample"},
                                 "openmp_build": legs_entry(host_in, nth, 3.0, 1.0 / 8, args.cpu_frac)},
                "e2e": {"value": round(v, 3), "unit": "GB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return
    if rank != 0:
        # one GPU per run: transforms are independent units, so more GPUs
        # would be replicas; this bench measures the one on rank 0
        return
    if args.only:
        import torch
        torch.cuda.set_device(0)
        fn = {"mix": run_mix, "serve": run_serving, "configs": run_configs, "nd": run_configs, "mix-runs": run_mix_runs,
              "serve-burst": run_serve_burst}[args.only]
        print(json.dumps(fn(args)))
        return
    r = run_gpu(args)
    cpu = r["cpu"]
    if rank == 0:
        line = {"metric": "HBM GB/s (compulsory bytes), batched FFT", "value": round(r["value"], 1), "unit": "GB/s",
                "gflops_5nlog2n": round(r["gflops"], 1),
                "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(r["ms"], 3),
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32+q15+q31",
                "data": "synthetic", "config": config, "roofline": r["roofline"], "cpu_baseline": cpu,
                "accuracy": accuracy_summary(r["units"]),
                "e2e": r["e2e"], "clocks": r["clocks"], "gpu_launches": r["gpu_launches"], "units": r["units"],
                "batched_mix": r["mix"], "serving": r["serving"], "other_configs": r["others"],
                "kernels": ("plan-specialised (NVRTC)" if args.specialize else "precompiled families") +
                ("; autotuned" if args.autotune else "") + "; set-up before warm-up %.1f s" % r["prepare_s"]}
        print(json.dumps(line))


if __name__ == "__main__":
    main()
