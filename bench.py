#!/usr/bin/env python3
"""Benchmark of the FFT family on GB300 (one JSON line on stdout).

Default workload: realft-based convolution and correlation of an N = 2^20
real f64 signal (i.i.d. N(0,1)) with a 257-tap response (Gaussian window,
sigma = m/6, times N(0,1)) stored in wrap-around order in a length-N buffer.
One step = one convlv(isign=+1) call and one correl call.  The nominal work
is 3 real FFTs per call, 2.5 N log2 N flops each.

  value     GFLOP/s with inputs resident in HBM (device tensors through the
            C ABI), CUDA events on the launching stream, L2 flushed (256 MiB
            write) before every timed step
  e2e       the same steps through the C ABI with pinned host buffers, the
            host->device and device->host copies inside the timed region
  roofline  the Stockham pass kernel: algorithmic bytes / its event-timed
            duration against the measured HBM copy bandwidth
  cpu_baseline  the CPU oracle (a C++ restatement of the crate's routines)
            on the host cores for a bounded sample of the same workload

--impl reference times the CPU oracle alone (the reference crate itself
cannot be built: no Rust toolchain, and its FFT modules are not compiled).
Other workloads (--workload four1|large|batch|fourn|rlft3|c1|convbatch) exercise the other
configurations; with no flags the convolution/correlation workload runs.
"""
import argparse
import json
import math
import os
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "FFT GFLOP/s (5N·log2N) & HBM GB/s vs peak; TC-split vs FP64 at rel-L2≤1e-6"
FP64_PEAK_TFLOPS = 1.20  # DFMA-loop throughput measured on GB300 (2 DFMA lanes per SM per cycle)

# DRAM bytes (read + write) per launch of the dominant kernel, from one ncu
# capture of the same workload (dram__bytes_read.sum + dram__bytes_write.sum),
# keyed by (workload, form).  The summaries under profiles/ give the commands.
MEASURED_TRAFFIC = {
    # 40 k_pass launches of the device-resident steps: forward 16.93 MB, inverse 8.54 MB
    ("convlv", "fp64"): (12.74e6, "profiles/k_pass_f64_convlv_correl_n2p20.md"),
    # the three passes of one 2^24-point transform: 367.1, 218.5, 346.0 MB
    ("four1_24", "fp32"): (310.5e6, "profiles/k_pass_fp32_fused_four1_n2p24.md"),
    # one persistent launch over the 20,000 transforms
    ("batch", "fp32"): (3.2058e9, "profiles/k_batch_c3_20000_transforms.md"),
    ("batch", "tc32"): (3.2069e9, "profiles/k_batch_c3_20000_transforms.md"),
}


def traffic_of(workload, form):
    t = MEASURED_TRAFFIC.get((workload, form))
    return (t[0], t[1]) if t else (None, None)


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=400)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="convlv",
                    choices=["convlv", "four1", "batch", "fourn", "rlft3", "large", "c1", "convbatch"])
    ap.add_argument("--form", default="fp64", choices=["fp64", "df64", "fp32", "tc32"])
    ap.add_argument("--no-forms", action="store_true", help="skip the extra precision forms")
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--log2n", type=int, default=0, help="four1 workload size (default 2^24)")
    return ap.parse_args()


def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


# ---------------------------------------------------------------------------
# clocks during the timed region
# ---------------------------------------------------------------------------
class Clocks:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=self.fh, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.fh.close()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        with open(self.path) as f:
            for line in f:
                p = [x.strip() for x in line.split(",")]
                if len(p) < 9:
                    continue
                try:
                    sm.append(float(p[1]))
                    smax.append(float(p[2]))
                except ValueError:
                    continue
                for nm, v in zip(names, p[5:9]):
                    if v.lower() == "active":
                        reasons.add(nm)
        os.unlink(self.path)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": max(smax), "samples": len(sm),
                "reasons": sorted(reasons)}


# ---------------------------------------------------------------------------
# distributed bookkeeping (one process per GPU; replicas of the workload)
# ---------------------------------------------------------------------------
def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def max_over_ranks(x, world):
    """Maximum of a per-rank scalar (timings) over the ranks: the job's time is
    its slowest rank's.  Works on the NCCL (CUDA tensor) and gloo (CPU tensor)
    backends."""
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    dev = "cpu" if dist.get_backend() == "gloo" else "cuda"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


# ---------------------------------------------------------------------------
# workloads
# ---------------------------------------------------------------------------
def convlv_inputs():
    from numrs_gb300 import workloads as W
    x, r = W.convlv_c2()
    y = W.normal(W.BASE_SEED + 21, x.size)
    return x, r, y


CONV_N = 1 << 20
CONV_FLOPS = 2 * 3 * 2.5 * CONV_N * 20  # two calls, three real FFTs each


def cpu_convlv_step(x, r, y):
    import oracle as O
    st, a = O.convlv(x, r, 1)
    st2, b = O.correl(x, y)
    assert st == 0 and st2 == 0
    return a, b


def cpu_baseline(seconds, x, r, y):
    """Time the CPU oracle on whole steps for about `seconds` of work.  Returns
    the baseline record and the oracle's outputs of the step, which the GPU
    results are checked against."""
    import oracle as O
    threads = os.cpu_count() or 1
    O.set_threads(threads)
    outs = cpu_convlv_step(x, r, y)  # warm-up
    n, t0 = 0, time.perf_counter()
    while True:
        cpu_convlv_step(x, r, y)
        n += 1
        el = time.perf_counter() - t0
        if el >= seconds or n >= 1000:
            break
    O.set_threads(1)
    return outs, {
        "value": CONV_FLOPS * n / el / 1e9, "unit": "GFLOP/s", "cores": min(2, threads),
        "kind": "port",
        "sample": "%d whole steps (convlv + correl, N=2^20) in %.1f s; the two forward "
                  "transforms of each call run on 2 threads as the reference's rayon::join "
                  "does, the transforms themselves are serial as in the crate" % (n, el),
    }


def run_reference_arm(args, world, rank):
    if rank != 0:
        return
    x, r, y = convlv_inputs()
    import oracle as O
    threads = os.cpu_count() or 1
    O.set_threads(threads)
    for _ in range(max(0, min(args.warmup, 2))):
        cpu_convlv_step(x, r, y)
    t1 = time.perf_counter()
    cpu_convlv_step(x, r, y)
    per = time.perf_counter() - t1
    budget = 90.0
    steps = max(1, min(args.steps, int(budget / max(per, 1e-6))))
    t0 = time.perf_counter()
    for _ in range(steps):
        cpu_convlv_step(x, r, y)
    el = time.perf_counter() - t0
    val = CONV_FLOPS * steps / el / 1e9
    line = {
        "impl": "reference", "metric": METRIC, "value": val, "unit": "GFLOP/s", "n_gpus": args.gpus,
        "steps": steps, "warmup": args.warmup, "ms_per_step": 1e3 * el / steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded N(0,1) signal, Gaussian-window response)",
        "config": {"workload": "realft convlv + correl, N=2^20 real f64, m=257 taps in a "
                               "length-N wrap-around buffer", "form": "fp64 (CPU)",
                   "sampled_steps": steps, "requested_steps": args.steps},
        "cpu_baseline": {"value": val, "unit": "GFLOP/s", "cores": min(2, threads), "kind": "port",
                         "sample": "%d of %d requested steps, CPU oracle (C++ restatement of "
                                   "Convolve.rs/Correlation.rs/Real_FT.rs)" % (steps, args.steps)},
        "e2e": {"value": val, "unit": "GFLOP/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    O.set_threads(1)
    print(json.dumps(line), flush=True)


def run_convlv(args, world, rank, local):
    import torch
    import numrs_gb300 as nr
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    x, r, y = convlv_inputs()
    xd = torch.from_numpy(x).to(dev)
    rd = torch.from_numpy(r).to(dev)
    yd = torch.from_numpy(y).to(dev)
    outa = torch.empty_like(xd)
    outb = torch.empty_like(xd)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    form = args.form

    def step(f=form):
        nr.convlv(xd, rd, 1, form=f, out=outa)
        nr.correl(xd, yd, form=f, out=outb)

    nr.set_async(True)
    for _ in range(max(args.warmup, 3)):
        step()
    torch.cuda.synchronize()

    # ---- device-resident timed region ----
    stream = torch.cuda.current_stream()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(args.steps)]
    clocks = Clocks(local)
    barrier(world)
    torch.cuda.synchronize()
    clocks.start()
    time.sleep(0.3)
    nr.launch_count(reset=True)
    for i in range(args.steps):
        flush.zero_()
        ev[i][0].record(stream)
        step()
        ev[i][1].record(stream)
    torch.cuda.synchronize()
    launches = nr.launch_count()
    clk = clocks.stop()
    barrier(world)
    total_ms = sum(a.elapsed_time(b) for a, b in ev)
    total_ms = max_over_ranks(total_ms, world)
    value = CONV_FLOPS * args.steps * world / (total_ms / 1e3) / 1e9

    # outputs of the timed run, checked against the CPU baseline's at the end
    outputs = {form: (outa.cpu().numpy().copy(), outb.cpu().numpy().copy())} if rank == 0 else {}

    # ---- per-kernel event timing (a separate profiled repetition) ----
    nprof = min(args.steps, 50)
    nr.profile(True)
    for i in range(nprof):
        flush.zero_()
        step()
    torch.cuda.synchronize()
    pass_ms, pass_n, pass_bytes, pass_flops = nr.profile_read("pass")
    tw_ms, tw_n, _, _ = nr.profile_read("twist")
    sp_ms, sp_n, sp_bytes, _ = nr.profile_read("spectral")
    nr.profile(False)

    # ---- other precision forms, same step ----
    forms = {}
    if not args.no_forms and rank == 0:
        for f in ("df64", "fp32", "tc32"):
            if f == form:
                continue
            for _ in range(3):
                step(f)
            torch.cuda.synchronize()
            evs = []
            for i in range(min(args.steps, 200)):
                a0, b0 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                flush.zero_()
                a0.record(stream)
                step(f)
                b0.record(stream)
                evs.append((a0, b0))
            torch.cuda.synchronize()
            ms = sum(a.elapsed_time(b) for a, b in evs)
            outputs[f] = (outa.cpu().numpy().copy(), outb.cpu().numpy().copy())
            forms[f] = {"value": CONV_FLOPS * len(evs) / (ms / 1e3) / 1e9, "unit": "GFLOP/s",
                        "ms_per_step": ms / len(evs)}
    nr.set_async(False)

    # ---- end to end through the C ABI with pinned host buffers ----
    xh = torch.from_numpy(x).pin_memory().numpy()
    rh = torch.from_numpy(r).pin_memory().numpy()
    yh = torch.from_numpy(y).pin_memory().numpy()
    oa = torch.empty(CONV_N, dtype=torch.float64).pin_memory().numpy()
    ob = torch.empty(CONV_N, dtype=torch.float64).pin_memory().numpy()

    def host_step():
        nr.convlv(xh, rh, 1, form=form, out=oa)
        nr.correl(xh, yh, form=form, out=ob)

    for _ in range(3):
        host_step()
    e2e_steps = max(10, min(args.steps, 200))
    barrier(world)
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        host_step()
    e2e_s = max_over_ranks(time.perf_counter() - t0, world)
    e2e_val = CONV_FLOPS * e2e_steps * world / e2e_s / 1e9

    if rank != 0:
        return
    # ---- CPU baseline (rank 0, after every GPU leg); its outputs check the
    # accuracy of each form's run ----
    (ra, rb), cpu = cpu_baseline(args.cpu_seconds, x, r, y)
    acc = {}
    for f, (ga, gb) in outputs.items():
        e = max(np.linalg.norm(ga - ra) / np.linalg.norm(ra),
                np.linalg.norm(gb - rb) / np.linalg.norm(rb))
        if f == form:
            acc[f] = e
        else:
            forms[f]["rel_l2_vs_fp64_oracle"] = e
    hbm, hbm_kind = peaks()
    pass_avg_ms = pass_ms / max(pass_n, 1)
    achieved = (pass_bytes / max(pass_n, 1)) / (pass_avg_ms / 1e3) / 1e9 if pass_n else 0.0
    line = {
        "metric": METRIC, "value": value, "unit": "GFLOP/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64" if form == "fp64" else form,
        "data": "synthetic (seeded N(0,1) signal, Gaussian-window response)",
        "config": {"workload": "realft convlv + correl, N=2^20 real f64, m=257 taps in a "
                               "length-N wrap-around buffer; one step = one convlv and one correl",
                   "form": form, "l2": "flushed between timed steps (256 MiB write)",
                   "nominal_flops_per_step": CONV_FLOPS},
        "e2e": {"value": e2e_val, "unit": "GFLOP/s", "steps": e2e_steps,
                "h2d_bytes_per_step": 4 * CONV_N * 8, "d2h_bytes_per_step": 2 * CONV_N * 8,
                "host_buffers": "pinned"},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s",
                     "frac": achieved / hbm, "traffic": traffic_of("convlv", form)[0],
                     "traffic_source": traffic_of("convlv", form)[1],
                     "kernel": "k_pass (Stockham pass)",
                     "peak_source": "%s MEASURED_PEAKS.json hbm_gbs" % hbm_kind if hbm_kind == "measured"
                     else "fallback 6.8 TB/s",
                     "launches": pass_n, "avg_launch_ms": pass_avg_ms,
                     "bytes_per_launch": pass_bytes / max(pass_n, 1)},
        "compute_roofline": {"bound": "fp64" if form == "fp64" else "fp32",
                             "achieved_tflops": pass_flops / (pass_ms / 1e3) / 1e12 if pass_ms else 0.0,
                             "peak_tflops": FP64_PEAK_TFLOPS if form == "fp64" else 73.3,
                             "note": "nominal 5 N log2 R per pass over the pass-kernel time; peaks "
                                     "from the DFMA / FFMA probes"},
        "kernels": {"pass": {"ms": pass_ms, "launches": pass_n},
                    "twist": {"ms": tw_ms, "launches": tw_n},
                    "spectral": {"ms": sp_ms, "launches": sp_n}, "profiled_steps": nprof},
        "accuracy": {"rel_l2_vs_cpu_oracle": acc},
        "forms": forms,
        "cpu_baseline": cpu,
        "clocks": clk,
        "gpu_launches": launches,
    }
    if hbm_kind == "measured":
        line["roofline"]["peak_source"] = "of measured (MEASURED_PEAKS.json hbm_gbs)"
    print(json.dumps(line), flush=True)


def run_four1(args, world, rank, local):
    """One in-place complex FFT of 2^log2n points per step (device resident)."""
    import torch
    import numrs_gb300 as nr
    from numrs_gb300 import workloads as W
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    log2n = args.log2n or (28 if args.workload == "large" else 24)
    nn = 1 << log2n
    x = W.normal(W.BASE_SEED + 5, 2 * nn) if log2n <= 24 else None
    d = torch.from_numpy(x).to(dev) if x is not None else torch.randn(2 * nn, dtype=torch.float64, device=dev)
    acc = _accuracy_vs_fp64(args.form, d, lambda t, form: nr.four1(t, nn, 1, form=form))
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    nr.set_async(True)
    sign = [1]

    def step():
        nr.four1(d, nn, sign[0], form=args.form)
        sign[0] = -sign[0]

    for _ in range(max(args.warmup, 3)):
        step()
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(args.steps)]
    clocks = Clocks(local)
    clocks.start()
    time.sleep(0.3)
    nr.launch_count(reset=True)
    for i in range(args.steps):
        if nn * 16 < (256 << 20):
            flush.zero_()
        ev[i][0].record(stream)
        step()
        ev[i][1].record(stream)
    torch.cuda.synchronize()
    launches = nr.launch_count()
    clk = clocks.stop()
    total_ms = max_over_ranks(sum(a.elapsed_time(b) for a, b in ev), world)
    flops = 5.0 * nn * log2n
    nr.profile(True)
    for i in range(min(args.steps, 20)):
        step()
    torch.cuda.synchronize()
    pass_ms, pass_n, pass_bytes, pass_flops = nr.profile_read("pass")
    nr.profile(False)
    nr.set_async(False)
    if rank != 0:
        return None
    hbm, hbm_kind = peaks()
    achieved = pass_bytes / (pass_ms / 1e3) / 1e9 if pass_ms else 0.0
    return {
        "metric": METRIC, "value": flops * args.steps * world / (total_ms / 1e3) / 1e9,
        "unit": "GFLOP/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": total_ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64" if args.form == "fp64" else args.form,
        "data": "synthetic N(0,1) complex",
        "config": {"workload": "four1 complex in-place FFT, N=2^%d (%d MiB), alternating isign"
                               % (log2n, (16 * nn) >> 20), "form": args.form,
                   "l2": "input larger than L2" if nn * 16 >= (256 << 20) else "flushed between steps"},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s",
                     "frac": achieved / hbm, "traffic": traffic_of("four1_%d" % log2n, args.form)[0],
                     "traffic_source": traffic_of("four1_%d" % log2n, args.form)[1],
                     "kernel": "k_pass (Stockham pass)", "launches": pass_n, "avg_launch_ms": pass_ms / max(pass_n, 1),
                     "bytes_per_launch": pass_bytes / max(pass_n, 1)},
        "compute_roofline": {"bound": "fp64" if args.form == "fp64" else "fp32",
                             "achieved_tflops": pass_flops / (pass_ms / 1e3) / 1e12 if pass_ms else 0.0,
                             "peak_tflops": FP64_PEAK_TFLOPS if args.form == "fp64" else 73.3},
        "accuracy": acc, "clocks": clk, "gpu_launches": launches,
    }


def _accuracy_vs_fp64(form, data, forward):
    """rel-L2 of one forward transform in `form` against the same transform in
    the FP64 form, on copies of `data` (the FP64 form itself is held to the CPU
    oracle at 1e-12 by the parity tests).  For the FP64 form: None."""
    if form == "fp64":
        return None
    import torch
    ref = data.clone()
    forward(ref, "fp64")
    got = data.clone()
    forward(got, form)
    torch.cuda.synchronize()
    e = float((got - ref).norm() / ref.norm())
    del ref, got
    return {"rel_l2_vs_fp64_form": e}


def run_batch(args, world, rank, local):
    """20,000 complex transforms of sizes 2^k, k uniform in 6..14, amplitudes
    10^u (u uniform in [-3, 3]); one step = one batched call over all of them."""
    import torch
    import numrs_gb300 as nr
    from numrs_gb300 import workloads as W
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    sizes, u = W.batch_c3()
    host = W.batch_c3_data(sizes, u)
    total = int(sum(2 * s for s in sizes))
    buf = torch.empty(total, dtype=torch.float64, device=dev)
    views, off = [], 0
    for a in host:
        v = buf[off:off + a.size]
        v.copy_(torch.from_numpy(a))
        views.append(v)
        off += a.size
    orig = buf.clone()
    flops = float(sum(5.0 * s * math.log2(s) for s in sizes))
    nbytes = 2.0 * 8 * total
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    stream = torch.cuda.current_stream()
    nr.set_async(True)
    results = {}
    sample = list(range(0, len(sizes), max(1, len(sizes) // 200)))
    # CPU baseline (rank 0): the oracle's FFTProcessor::fft_batch (one task per
    # transform on all host threads) over the sampled transforms; its outputs
    # check every form's accuracy
    cpu, refs = None, {}
    if rank == 0:
        import oracle as O
        threads = os.cpu_count() or 1
        O.set_threads(threads)
        arrs = [host[t].copy() for t in sample]
        O.fft_batch(arrs, 1)  # warm-up
        arrs = [host[t].copy() for t in sample]
        t0 = time.perf_counter()
        O.fft_batch(arrs, 1)
        el = time.perf_counter() - t0
        O.set_threads(1)
        refs = dict(zip(sample, arrs))
        sflops = float(sum(5.0 * sizes[t] * math.log2(sizes[t]) for t in sample))
        cpu = {"value": sflops / el / 1e9, "unit": "GFLOP/s", "cores": threads, "kind": "port",
               "sample": "%d of the 20,000 transforms (every %d-th), one fft_batch call of the "
                         "CPU oracle, %.3f s" % (len(sample), max(1, len(sizes) // 200), el)}
    for form in [args.form] + ([f for f in ("fp64", "df64", "fp32", "tc32") if f != args.form]
                               if not args.no_forms else []):
        b = nr.FFTBatch(views, form=form)
        buf.copy_(orig)
        b.run(1)
        torch.cuda.synchronize()
        # accuracy on the sampled transforms, against the CPU baseline's outputs
        errs = []
        got = buf.cpu().numpy()
        offs = np.concatenate([[0], np.cumsum(2 * sizes)])
        for t in (sample if rank == 0 else []):
            ref = refs[t]
            g = got[offs[t]:offs[t + 1]]
            errs.append(np.linalg.norm(g - ref) / np.linalg.norm(ref))
        for _ in range(max(args.warmup, 3)):
            b.run(1)
        torch.cuda.synchronize()
        steps = args.steps if form == args.form else min(args.steps, 50)
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
              for _ in range(steps)]
        clocks = Clocks(local)
        if form == args.form:
            clocks.start()
            time.sleep(0.3)
        nr.launch_count(reset=True)
        for i in range(steps):
            flush.zero_()
            ev[i][0].record(stream)
            b.run(1)
            ev[i][1].record(stream)
        torch.cuda.synchronize()
        launches = nr.launch_count()
        clk = clocks.stop() if form == args.form else None
        ms = max_over_ranks(sum(a.elapsed_time(c) for a, c in ev), world)
        results[form] = {"value": flops * steps * world / (ms / 1e3) / 1e9, "unit": "GFLOP/s",
                         "transforms_per_s": len(sizes) * steps * world / (ms / 1e3),
                         "ms_per_step": ms / steps, "hbm_gbs": nbytes * steps / (ms / 1e3) / 1e9,
                         "rel_l2_max": float(max(errs)) if errs else None,
                         "rel_l2_median": float(np.median(errs)) if errs else None,
                         "launches": launches, "clocks": clk}
    nr.set_async(False)
    # end to end with host arrays: FFTBatch marshals the 20,000 pointers once,
    # and each run is one library call on the caller's numpy arrays
    hb = [a.copy() for a in host]
    hbatch = nr.FFTBatch(hb, form=args.form)
    hbatch.run(1)
    e2e_steps = max(3, min(args.steps, 10))
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        hbatch.run(1)
    e2e_s = max_over_ranks(time.perf_counter() - t0, world)
    if rank != 0:
        return None
    hbm, hbm_kind = peaks()
    main_r = results[args.form]
    line = {
        "metric": METRIC, "value": main_r["value"], "unit": "GFLOP/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": main_r["ms_per_step"],
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64" if args.form == "fp64" else args.form,
        "data": "synthetic complex N(0,1) x 10^u",
        "config": {"workload": "batched uneven four1: 20000 transforms, sizes 2^k, k uniform "
                               "in 6..14, one persistent launch (CUDA graph)", "form": args.form,
                   "l2": "inputs (%.2f GB) larger than L2; L2 also flushed" % (nbytes / 2e9)},
        "e2e": {"value": flops * e2e_steps * world / e2e_s / 1e9, "unit": "GFLOP/s",
                "h2d_bytes_per_step": total * 8, "d2h_bytes_per_step": total * 8,
                "host_buffers": "pageable numpy arrays through FFTBatch.run; the persistent "
                                "kernel reads and writes them in place over the host link when "
                                "they are 16-byte aligned (otherwise one packed staging copy "
                                "each way)"},
        "roofline": {"bound": "hbm", "achieved": main_r["hbm_gbs"], "peak": hbm, "unit": "GB/s",
                     "frac": main_r["hbm_gbs"] / hbm, "traffic": traffic_of("batch", args.form)[0],
                     "traffic_source": traffic_of("batch", args.form)[1],
                     "kernel": "k_batch (persistent)"},
        "forms": results, "cpu_baseline": cpu, "clocks": main_r["clocks"],
        "gpu_launches": main_r["launches"],
    }
    return line


def _simple_line(args, world, workload, flops, total_ms, steps, launches, clk, extra=None):
    hbm, hbm_kind = peaks()
    line = {
        "metric": METRIC, "value": flops * steps * world / (total_ms / 1e3) / 1e9,
        "unit": "GFLOP/s", "n_gpus": world, "steps": steps, "warmup": args.warmup,
        "ms_per_step": total_ms / steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64" if args.form == "fp64" else args.form,
        "data": "synthetic", "config": {"workload": workload, "form": args.form},
        "clocks": clk, "gpu_launches": launches,
    }
    if extra:
        line.update(extra)
    return line


def _timed(args, local, step, flush, steps):
    import torch
    import numrs_gb300 as nr
    stream = torch.cuda.current_stream()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(steps)]
    clocks = Clocks(local)
    clocks.start()
    time.sleep(0.3)
    nr.launch_count(reset=True)
    for i in range(steps):
        if flush is not None:
            flush.zero_()
        ev[i][0].record(stream)
        step()
        ev[i][1].record(stream)
    torch.cuda.synchronize()
    launches = nr.launch_count()
    clk = clocks.stop()
    return sum(a.elapsed_time(b) for a, b in ev), launches, clk


def _pass_roofline():
    import numrs_gb300 as nr
    hbm, _ = peaks()
    ms, n, by, fl = nr.profile_read("pass")
    ach = by / (ms / 1e3) / 1e9 if ms else 0.0
    return {"bound": "hbm", "achieved": ach, "peak": hbm, "unit": "GB/s", "frac": ach / hbm,
            "traffic": None, "kernel": "k_pass (Stockham pass)", "launches": n,
            "avg_launch_ms": ms / max(n, 1), "bytes_per_launch": by / max(n, 1),
            "fp64_tflops_nominal": fl / (ms / 1e3) / 1e12 if ms else 0.0}


def _plane_wave_field(shape, dev, seed=0x6B3A2026 + 4, count=32):
    """uniform[-1,1) plus `count` unit plane waves with integer wave vectors and
    random phases, generated on the device (same construction as
    numrs_gb300.workloads.plane_waves)."""
    import torch
    g = torch.Generator(device=dev)
    g.manual_seed(seed)
    x = torch.rand(shape, generator=g, device=dev, dtype=torch.float64) * 2 - 1
    kv = (torch.rand((count, len(shape)), generator=g, device=dev, dtype=torch.float64) *
          torch.tensor(shape, device=dev, dtype=torch.float64)).floor()
    ph = 2 * math.pi * torch.rand(count, generator=g, device=dev, dtype=torch.float64)
    grids = torch.meshgrid(*[torch.arange(s, device=dev, dtype=torch.float64) / s for s in shape],
                           indexing="ij")
    for c in range(count):
        arg = sum(kv[c, d] * grids[d] for d in range(len(shape)))
        x += torch.cos(2 * math.pi * arg + ph[c])
    return x.contiguous()


def run_nd(args, world, rank, local):
    """fourn 256 x 256 x 512 complex, or rlft3 512^3 real; forward + inverse per step."""
    import torch
    import numrs_gb300 as nr
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    nr.set_async(True)
    if args.workload == "fourn":
        shape = (256, 256, 512)
        n = int(np.prod(shape))
        re = _plane_wave_field(shape, dev).reshape(-1)
        im = _plane_wave_field(shape, dev, seed=0x6B3A2026 + 40).reshape(-1)
        d = torch.stack([re, im], dim=1).reshape(-1).contiguous()
        del re, im
        orig = d.clone()

        def step():
            nr.fourn(d, shape, 3, 1, form=args.form)
            nr.fourn(d, shape, 3, -1, form=args.form)
            d.mul_(1.0 / n)
        flops = 2 * 5.0 * n * math.log2(n)
        wl = "fourn 256x256x512 complex f64 (512 MiB), forward + inverse (scaled 1/N) per step"
    else:
        shape = (512, 512, 512)
        n = int(np.prod(shape))
        d = _plane_wave_field(shape, dev).reshape(-1)
        orig = d.clone()
        sp = torch.zeros(512 * 2 * 512, dtype=torch.float64, device=dev)

        def step():
            nr.rlft3(d, sp, 512, 512, 512, 1, form=args.form)
            nr.rlft3(d, sp, 512, 512, 512, -1, form=args.form)
            d.mul_(2.0 / n)
        flops = 2 * 2.5 * n * math.log2(n)
        wl = "rlft3 512^3 real f64 (1 GiB) + speq, forward + inverse (scaled 2/N) per step"
    if args.workload == "fourn":
        fwd = (lambda t, form: nr.fourn(t, shape, 3, 1, form=form))
    else:
        spw = torch.zeros_like(sp)
        fwd = (lambda t, form: nr.rlft3(t, spw, 512, 512, 512, 1, form=form))
    acc = _accuracy_vs_fp64(args.form, d, fwd) or {}
    for _ in range(max(args.warmup, 3)):
        step()
    torch.cuda.synchronize()
    err = float((d - orig).norm() / orig.norm())
    steps = min(args.steps, 20)
    total_ms, launches, clk = _timed(args, local, step, None, steps)
    nr.profile(True)
    step()
    torch.cuda.synchronize()
    roof = _pass_roofline()
    nr.profile(False)
    nr.set_async(False)
    if rank != 0:
        return None
    acc["roundtrip_rel_l2"] = err
    return _simple_line(args, world, wl, flops, total_ms, steps, launches, clk,
                        {"roofline": roof, "accuracy": acc})


def run_c1(args, world, rank, local):
    """four1 N=4096 round trip (+1, -1, x 1/N): latency of one small transform."""
    import torch
    import numrs_gb300 as nr
    from numrs_gb300 import workloads as W
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    x = W.four1_c1()
    d = torch.from_numpy(x).to(dev)
    nr.set_async(True)

    def step():
        nr.four1(d, 4096, 1, form=args.form)
        nr.four1(d, 4096, -1, form=args.form)
        d.mul_(1.0 / 4096)
    step()
    torch.cuda.synchronize()
    # accuracy of one round trip (repeated round trips accumulate their errors)
    err = float(np.linalg.norm(d.cpu().numpy() - x) / np.linalg.norm(x))
    for _ in range(max(args.warmup, 3)):
        step()
    torch.cuda.synchronize()
    steps = max(args.steps, 100)
    total_ms, launches, clk = _timed(args, local, step, None, steps)
    nr.set_async(False)
    if rank != 0:
        return None
    return _simple_line(args, world, "four1 N=4096 round trip (+1, -1, x1/N), one transform",
                        2 * 5.0 * 4096 * 12, total_ms, steps, launches, clk,
                        {"us_per_roundtrip": 1e3 * total_ms / steps,
                         "accuracy": {"roundtrip_rel_l2": err}})


def run_convbatch(args, world, rank, local):
    """convlv_batch: 64 convolutions of N=2^16 reals with one 257-tap response
    (the C2 response construction at N=2^16), one library call per step; the
    same 64 convolutions as 64 convlv calls are timed beside it."""
    import torch
    import numrs_gb300 as nr
    from numrs_gb300 import workloads as W
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    count, n = 64, 1 << 16
    _, r = W.convlv_c2(n=n)
    items = [torch.from_numpy(W.normal(W.BASE_SEED + 100 + i, n)).to(dev) for i in range(count)]
    rd = torch.from_numpy(r).to(dev)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    nr.set_async(True)
    flops = count * 3 * 2.5 * n * math.log2(n)  # the crate's work: 3 real FFTs per item
    outs = [None]

    def step_batch():
        outs[0] = nr.convlv_batch(items, rd, 1, form=args.form)

    def step_single():
        outs[0] = [nr.convlv(x, rd, 1, form=args.form) for x in items]

    for _ in range(max(args.warmup, 3)):
        step_batch()
        step_single()
    torch.cuda.synchronize()
    steps = min(args.steps, 50)
    ms_b, launches, clk = _timed(args, local, step_batch, flush, steps)
    ms_s, _, _ = _timed(args, local, step_single, flush, steps)
    step_batch()
    torch.cuda.synchronize()
    nr.set_async(False)
    if rank != 0:
        return None
    # CPU baseline: the oracle's convlv on items 0 and 63; its outputs check
    # the GPU results
    import oracle as O
    errs = []
    t0 = time.perf_counter()
    refs = [O.convlv(items[i].cpu().numpy(), r, 1)[1] for i in (0, count - 1)]
    el = time.perf_counter() - t0
    for i, ref in zip((0, count - 1), refs):
        got = outs[0][i].cpu().numpy()
        errs.append(float(np.linalg.norm(got - ref) / np.linalg.norm(ref)))
    cpu = {"value": 2 * 3 * 2.5 * n * math.log2(n) / el / 1e9, "unit": "GFLOP/s", "cores": 2,
           "kind": "port", "sample": "2 of the 64 convolutions (items 0 and 63), %.3f s" % el}
    return _simple_line(
        args, world, "convlv_batch: 64 convolutions of N=2^16 reals, one 257-tap response "
        "(Gaussian window x N(0,1)), device resident, one call per step", flops, ms_b, steps,
        launches, clk,
        {"single_calls": {"ms_per_step": ms_s / steps,
                          "value": flops * steps / (ms_s / 1e3) / 1e9, "unit": "GFLOP/s",
                          "note": "the same 64 convolutions as 64 convlv calls"},
         "accuracy": {"rel_l2_vs_cpu_oracle_items_0_and_63": errs},
         "cpu_baseline": cpu, "l2": "flushed between timed steps (256 MiB write)"})


def main():
    args = parse()
    world, rank, local = dist_setup()
    if args.impl == "reference":
        run_reference_arm(args, world, rank)
        return
    import torch
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    if args.workload in ("four1", "large", "batch"):
        fn = run_batch if args.workload == "batch" else run_four1
        line = fn(args, world, rank, local)
        if line:
            print(json.dumps(line), flush=True)
    elif args.workload in ("fourn", "rlft3", "c1", "convbatch"):
        fn = {"c1": run_c1, "convbatch": run_convbatch}.get(args.workload, run_nd)
        line = fn(args, world, rank, local)
        if line:
            print(json.dumps(line), flush=True)
    else:
        run_convlv(args, world, rank, local)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
