#!/usr/bin/env python3
"""Benchmark of the FFT family on GB300 (one JSON line on stdout).

Default workload (the largest configuration that runs on one GPU): one
complex four1 of nn = 2^28 points (4 GiB of interleaved f64), i.i.d. N(0,1)
from the seeded generator, FP64 arithmetic.  One step = one in-place forward
transform; the nominal work is 5 nn log2 nn flops.

  value     GFLOP/s with the input resident in HBM (device tensor through the
            C ABI), CUDA events on the launching stream around each transform;
            the input is restored from a device copy between steps, outside
            the events.  The 4 GiB input is larger than L2.
  e2e       the same transform through the C ABI on a pinned host array: the
            host->device copy, the transform and the device->host copy are
            inside each timed call
  roofline  the Stockham pass kernel: algorithmic bytes per launch over its
            event-timed duration, against the measured HBM copy bandwidth;
            compute_roofline gives the same kernel against the FP64 pipe
  forms     the double-float, FP32 and tensor-core forms on the same step,
            with their rel-L2 against the FP64 form
  batch_target  the batched configuration (20,000 transforms of 2^6..2^14
            points, amplitudes 10^u): transforms/s of every form and the
            tensor-core form's per-transform rel-L2 against FP64
  cpu_baseline  the CPU oracle (a C++ restatement of the crate's routines) on
            the host cores, on a bounded sample of the workload

--impl reference times the CPU oracle alone on the same configuration (the
crate itself cannot be built: no Rust toolchain, and its FFT modules are not
compiled).  Other workloads (--workload convlv|four1|batch|fourn|rlft3|c1|convbatch)
exercise the other configurations.
"""
import argparse
import json
import math
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "FFT GFLOP/s (5N·log2N) & HBM GB/s vs peak; TC-split vs FP64 at rel-L2≤1e-6"
FP64_PEAK_TFLOPS = 1.20  # DFMA-loop throughput measured on GB300 (2 DFMA lanes per SM per cycle)
FP32_PEAK_TFLOPS = 73.3  # FFMA-loop throughput measured on GB300

LARGE_LOG2N = 28

# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) per launch of the
# dominant kernel from one ncu capture of the same kernel on the same
# workload, keyed by (workload, form).  Fixed numbers from an earlier capture,
# not measured by this run.
NCU_TRAFFIC = {
    ("convlv", "fp64"): 12.74e6,
    ("four1_24", "fp32"): 310.5e6,
    ("batch", "fp32"): 3.2058e9,
    ("batch", "tc32"): 3.2069e9,
}


# FP64 pipe activity (sm__pipe_fp64_cycles_active, % of active cycles) of the
# FP64 pass kernel, passes 1-3 of four1 2^26, from one ncu capture: fixed,
# not measured by this run.
NCU_FP64_PIPE_BUSY = [0.841, 0.839, 0.835]


def traffic_of(workload, form):
    t = NCU_TRAFFIC.get((workload, form))
    if t is None:
        return None, None
    return t, "ncu capture of this kernel and workload (fixed, not measured in this run)"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="large",
                    choices=["large", "convlv", "four1", "batch", "fourn", "rlft3", "c1", "convbatch",
                             "peaks", "sharded", "link"])
    ap.add_argument("--form", default="fp64", choices=["fp64", "df64", "fp32", "tc32"])
    ap.add_argument("--no-forms", action="store_true", help="skip the extra precision forms")
    ap.add_argument("--no-batch", action="store_true", help="skip the batched target in the default line")
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--log2n", type=int, default=0, help="four1 workload size (default 2^24; large: 2^28)")
    ap.add_argument("--shares", type=int, default=0,
                    help="sharded workload in one process: P shares on this GPU (exchanges as copies)")
    return ap.parse_args()


def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def host_cores():
    return os.cpu_count() or 1


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
# distributed bookkeeping (one process per GPU)
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


def _events(n):
    import torch
    return [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
            for _ in range(n)]


def _rel_l2_dev(a, b):
    return float((a - b).norm() / b.norm())


# ---------------------------------------------------------------------------
# the default workload: four1, nn = 2^28
# ---------------------------------------------------------------------------
def large_config(log2n, form):
    nn = 1 << log2n
    return {"workload": "four1 complex FFT, nn=2^%d (%d MiB of interleaved f64), i.i.d. N(0,1) "
                        "from the seeded generator; one step = one in-place forward transform"
                        % (log2n, (16 * nn) >> 20),
            "form": form,
            "l2": "input (%d MiB) larger than L2 (129 MB); no flush needed" % ((16 * nn) >> 20)}


def large_input(log2n):
    from numrs_gb300 import workloads as W
    return W.normal(W.BASE_SEED + 5, 2 * (1 << log2n))


def cpu_four1_sample(log2n, threads):
    """One oracle four1 of 2^log2n points on `threads` threads; GFLOP/s."""
    import oracle as O
    from numrs_gb300 import workloads as W
    nn = 1 << log2n
    x = W.normal(W.BASE_SEED + 6, 2 * nn)
    O.set_threads(threads)
    w = W.normal(W.BASE_SEED + 7, 2 * 4096)
    O.four1(w, 4096, 1)  # warm-up (pool threads, code)
    t0 = time.perf_counter()
    O.four1(x, nn, 1)
    el = time.perf_counter() - t0
    O.set_threads(1)
    return 5.0 * nn * log2n / el / 1e9, el


def run_large(args, world, rank, local):
    import torch
    import numrs_gb300 as nr
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    log2n = args.log2n or LARGE_LOG2N
    nn = 1 << log2n
    form = args.form
    flops = 5.0 * nn * log2n
    x = large_input(log2n)
    x0 = torch.from_numpy(x).to(dev)  # the input, kept to restore between steps
    d = torch.empty_like(x0)
    stream = torch.cuda.current_stream()
    nr.set_async(True)

    def step(f):
        nr.four1(d, nn, 1, form=f)

    def timed(f, steps):
        ev = _events(steps)
        for i in range(steps):
            d.copy_(x0)
            ev[i][0].record(stream)
            step(f)
            ev[i][1].record(stream)
        torch.cuda.synchronize()
        return sum(a.elapsed_time(b) for a, b in ev)

    # the FP64 form's output: the yardstick of the other forms (the FP64 form
    # itself is held to the CPU oracle at 1e-12 by the parity tests)
    d.copy_(x0)
    step("fp64")
    torch.cuda.synchronize()
    ref64 = d.clone()
    for _ in range(max(args.warmup, 3)):
        d.copy_(x0)
        step(form)
    torch.cuda.synchronize()

    # ---- device-resident timed region ----
    clocks = Clocks(local)
    barrier(world)
    torch.cuda.synchronize()
    clocks.start()
    time.sleep(0.3)
    nr.launch_count(reset=True)
    total_ms = timed(form, args.steps)
    launches = nr.launch_count()
    clk = clocks.stop()
    barrier(world)
    total_ms = max_over_ranks(total_ms, world)
    value = flops * args.steps * world / (total_ms / 1e3) / 1e9
    acc_main = None if form == "fp64" else _rel_l2_dev(d, ref64)

    # ---- per-kernel event timing (a separate profiled repetition) ----
    nr.profile(True)
    for _ in range(min(args.steps, 10)):
        d.copy_(x0)
        step(form)
    torch.cuda.synchronize()
    pass_ms, pass_n, pass_bytes, pass_flops = nr.profile_read("pass")
    nr.profile(False)

    # ---- the other arithmetic forms on the same step ----
    forms = {}
    if not args.no_forms and rank == 0:
        for f in ("fp64", "df64", "fp32", "tc32"):
            if f == form:
                continue
            for _ in range(3):
                d.copy_(x0)
                step(f)
            k = min(args.steps, 10)
            ms = timed(f, k)
            forms[f] = {"value": flops * k / (ms / 1e3) / 1e9, "unit": "GFLOP/s",
                        "ms_per_step": ms / k,
                        "rel_l2_vs_fp64_form": None if f == "fp64" else _rel_l2_dev(d, ref64)}
    nr.set_async(False)
    del d
    torch.cuda.empty_cache()

    # ---- end to end through the C ABI on a pinned host array ----
    xh = torch.from_numpy(x).pin_memory()
    xn = xh.numpy()
    e2e_steps = max(3, min(args.steps, 5))
    nr.four1(xn, nn, 1, form=form)  # warm-up (staging buffers)
    e2e_s = 0.0
    barrier(world)
    for _ in range(e2e_steps):
        xh.copy_(torch.from_numpy(x))
        t0 = time.perf_counter()
        nr.four1(xn, nn, 1, form=form)
        e2e_s += time.perf_counter() - t0
    e2e_s = max_over_ranks(e2e_s, world)
    e2e_val = flops * e2e_steps * world / e2e_s / 1e9
    e2e_acc = _rel_l2_dev(torch.from_numpy(xn).to(dev), ref64)
    del xh, xn, x0
    torch.cuda.empty_cache()

    # ---- the batched target (20,000 uneven transforms) ----
    batch = None
    if not args.no_batch:
        batch = batch_target(args, dev, rank, world)
    if rank != 0:
        return None

    # ---- CPU baseline: the oracle on a bounded sample (2^26 points) ----
    cores = host_cores()
    cpu_all, el_all = cpu_four1_sample(26, cores)
    cpu_one, el_one = cpu_four1_sample(26, 1)

    hbm, hbm_kind = peaks()
    pass_avg_ms = pass_ms / max(pass_n, 1)
    per_launch = pass_bytes / max(pass_n, 1)
    achieved = per_launch / (pass_avg_ms / 1e3) / 1e9 if pass_n else 0.0
    traffic, traffic_note = traffic_of("large", form)
    cfg = large_config(log2n, form)
    line = {
        "metric": METRIC, "value": value, "unit": "GFLOP/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64" if form == "fp64" else form,
        "data": "synthetic (seeded N(0,1) complex)",
        "config": cfg,
        "e2e": {"value": e2e_val, "unit": "GFLOP/s", "steps": e2e_steps,
                "h2d_bytes_per_step": 16 * nn, "d2h_bytes_per_step": 16 * nn,
                "host_buffers": "pinned", "rel_l2_vs_device_fp64": e2e_acc},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s",
                     "frac": achieved / hbm, "traffic": traffic, "traffic_note": traffic_note,
                     "kernel": "k_pass (Stockham pass)",
                     "peak_source": ("of measured (MEASURED_PEAKS.json hbm_gbs)" if hbm_kind == "measured"
                                     else "of fallback 6.8 TB/s"),
                     "launches": pass_n, "avg_launch_ms": pass_avg_ms,
                     "bytes_per_launch": per_launch,
                     "bytes_rule": "32 B per point per pass (16 B read + 16 B written, f64 I/O; "
                                   "8 B per side for FP32 scratch)"},
        "compute_roofline": {"bound": "fp64" if form in ("fp64",) else "fp32",
                             "achieved_tflops": pass_flops / (pass_ms / 1e3) / 1e12 if pass_ms else 0.0,
                             "peak_tflops": FP64_PEAK_TFLOPS if form == "fp64" else FP32_PEAK_TFLOPS,
                             "frac": ((pass_flops / (pass_ms / 1e3) / 1e12) /
                                      (FP64_PEAK_TFLOPS if form == "fp64" else FP32_PEAK_TFLOPS))
                             if pass_ms else 0.0,
                             "note": "nominal 5 N log2 R per radix-R pass over the pass kernel's "
                                     "event time; peaks from the DFMA / FFMA loop probes",
                             "fp64_pipe_busy": NCU_FP64_PIPE_BUSY if form == "fp64" else None,
                             "fp64_pipe_busy_note": "ncu sm__pipe_fp64_cycles_active of the same "
                             "pass kernel on four1 2^26 (fixed capture, not measured in this "
                             "run); nominal flops undercount the pipe because most FP64 "
                             "instructions are DADD/DMUL, not DFMA" if form == "fp64" else None},
        "kernels": {"pass": {"ms": pass_ms, "launches": pass_n}},
        "accuracy": {"rel_l2_vs_fp64_form": acc_main},
        "forms": forms,
        "batch_target": batch,
        "cpu_baseline": {"value": cpu_all, "unit": "GFLOP/s", "cores": cores, "kind": "port",
                         "sample": "one oracle four1 of 2^26 points (a quarter of the 2^28 "
                                   "workload) on all %d host threads: %.1f s; GFLOP/s by "
                                   "5 N log2 N" % (cores, el_all),
                         "one_core": {"value": cpu_one, "seconds": el_one},
                         "host_cores": cores,
                         "build": "g++ -O3 -ffp-contract=off (portable flags, no -march)"},
        "clocks": clk,
        "gpu_launches": launches,
    }
    return line


# ---------------------------------------------------------------------------
# the batched configuration: 20,000 transforms, 2^6..2^14 points
# ---------------------------------------------------------------------------
def batch_inputs():
    from numrs_gb300 import workloads as W
    sizes, u = W.batch_c3()
    return sizes, W.batch_c3_data(sizes, u)


def batch_target(args, dev, rank, world):
    """Every form on the 20,000-transform batch: one persistent launch (a
    CUDA-graph replay) per step, inputs restored between steps outside the
    timed events.  Per-transform rel-L2 of every form against the FP64 form,
    whose own per-transform error against the CPU oracle is reported too."""
    import torch
    import numrs_gb300 as nr
    import oracle as O
    sizes, host = batch_inputs()
    flat = np.concatenate(host)
    buf = torch.from_numpy(flat).to(dev)
    orig = buf.clone()
    starts = np.concatenate([[0], np.cumsum(2 * sizes)[:-1]])
    views = [buf[int(s):int(s) + 2 * int(n)] for s, n in zip(starts, sizes)]
    seg = torch.repeat_interleave(torch.arange(len(sizes), device=dev),
                                  torch.from_numpy(2 * sizes).to(dev))
    flops = float(sum(5.0 * s * math.log2(s) for s in sizes))
    stream = torch.cuda.current_stream()

    def seg_norms(v):
        return torch.zeros(len(sizes), dtype=torch.float64, device=dev).index_add_(0, seg, v * v).sqrt()

    nr.set_async(True)
    res, outs = {}, {}
    for f in ("fp64", "tc32", "fp32", "df64"):
        b = nr.FFTBatch(views, form=f)
        buf.copy_(orig)
        b.run(1)
        torch.cuda.synchronize()
        outs[f] = buf.clone()
        for _ in range(max(args.warmup, 3)):
            buf.copy_(orig)
            b.run(1)
        steps = min(args.steps, 30)
        ev = _events(steps)
        nr.launch_count(reset=True)
        for i in range(steps):
            buf.copy_(orig)
            ev[i][0].record(stream)
            b.run(1)
            ev[i][1].record(stream)
        torch.cuda.synchronize()
        launches = nr.launch_count()
        ms = max_over_ranks(sum(a.elapsed_time(c) for a, c in ev), world)
        res[f] = {"ms_per_step": ms / steps, "transforms_per_s": len(sizes) * steps * world / (ms / 1e3),
                  "value": flops * steps * world / (ms / 1e3) / 1e9, "unit": "GFLOP/s",
                  "launches_per_step": launches / steps}
    nr.set_async(False)
    ref_n = seg_norms(outs["fp64"])
    for f in ("tc32", "fp32", "df64"):
        rel = (seg_norms(outs[f] - outs["fp64"]) / ref_n).cpu().numpy()
        res[f]["rel_l2_vs_fp64_max"] = float(rel.max())
        res[f]["rel_l2_vs_fp64_median"] = float(np.median(rel))
    got64 = outs["fp64"].cpu().numpy()
    del outs, buf, orig, seg
    torch.cuda.empty_cache()
    if rank != 0:
        return None
    # CPU oracle over all 20,000 transforms on every host thread: the batch's
    # CPU baseline and the FP64 form's per-transform error against the oracle
    threads = host_cores()
    O.set_threads(threads)
    refs = [a.copy() for a in host]
    t0 = time.perf_counter()
    O.fft_batch(refs, 1)
    el = time.perf_counter() - t0
    O.set_threads(1)
    ref = np.concatenate(refs)
    rel64 = np.sqrt(np.add.reduceat((got64 - ref) ** 2, starts)) / np.sqrt(np.add.reduceat(ref ** 2, starts))
    res["fp64"]["rel_l2_vs_oracle_max"] = float(rel64.max())
    ratio = res["tc32"]["transforms_per_s"] / res["fp64"]["transforms_per_s"]
    return {
        "workload": "batched uneven four1: 20,000 transforms, sizes 2^k with k uniform in 6..14, "
                    "complex N(0,1) x 10^u, u ~ U[-3,3]; one persistent launch (CUDA graph) per step",
        "forms": res,
        "tc32_over_fp64_transforms_per_s": ratio,
        "fp32_over_fp64_transforms_per_s": res["fp32"]["transforms_per_s"] / res["fp64"]["transforms_per_s"],
        "target": "tensor-core form >= 3x the FP64 form's transforms/s at rel-L2 <= 1e-6 per transform",
        "target_met": bool(ratio >= 3.0 and res["tc32"]["rel_l2_vs_fp64_max"] <= 1e-6),
        "cpu_baseline": {"transforms_per_s": len(sizes) / el, "value": flops / el / 1e9,
                         "unit": "GFLOP/s", "cores": threads, "kind": "port",
                         "sample": "all 20,000 transforms, one fft_batch call of the CPU oracle, "
                                   "%.2f s" % el},
    }


# ---------------------------------------------------------------------------
# reference arm: the CPU oracle on the same configuration
# ---------------------------------------------------------------------------
def run_reference_arm(args, world, rank):
    if rank != 0:
        return
    if args.workload == "convlv":
        return run_reference_convlv(args)
    if args.workload not in ("large",):
        print(json.dumps({"impl": "reference", "unavailable":
                          "the reference arm is provided for the large and convlv workloads"}))
        return
    import oracle as O
    log2n = args.log2n or LARGE_LOG2N
    nn = 1 << log2n
    flops = 5.0 * nn * log2n
    x = large_input(log2n)
    threads = host_cores()
    O.set_threads(threads)
    from numrs_gb300 import workloads as W
    w = W.normal(W.BASE_SEED + 7, 2 * (1 << 20))
    for _ in range(max(0, min(args.warmup, 2))):
        O.four1(w, 1 << 20, 1)  # warm-up on a 2^20 sample (pool threads, code)
    budget = 150.0
    steps, el = 0, 0.0
    d = np.empty_like(x)
    while steps < args.steps:
        d[:] = x
        t0 = time.perf_counter()
        O.four1(d, nn, 1)
        el += time.perf_counter() - t0
        steps += 1
        if el + el / steps > budget:
            break
    O.set_threads(1)
    val = flops * steps / el / 1e9
    line = {
        "impl": "reference", "metric": METRIC, "value": val, "unit": "GFLOP/s", "n_gpus": args.gpus,
        "steps": steps, "warmup": args.warmup, "ms_per_step": 1e3 * el / steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded N(0,1) complex)",
        "config": large_config(log2n, "fp64"),
        "requested_steps": args.steps,
        "cpu_baseline": {"value": val, "unit": "GFLOP/s", "cores": threads, "kind": "port",
                         "sample": "%d of %d requested steps, each one whole 2^%d-point four1 of "
                                   "the CPU oracle (C++ restatement of FFT_1.rs:5-107), all %d "
                                   "host threads; steps bounded by a %.0f s budget; warm-up on "
                                   "2^20-point transforms" % (steps, args.steps, log2n, threads,
                                                              budget)},
        "e2e": {"value": val, "unit": "GFLOP/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
# convolution / correlation, N = 2^20
# ---------------------------------------------------------------------------
def convlv_inputs():
    from numrs_gb300 import workloads as W
    x, r = W.convlv_c2()
    y = W.normal(W.BASE_SEED + 21, x.size)
    return x, r, y


CONV_N = 1 << 20
CONV_FLOPS = 2 * 3 * 2.5 * CONV_N * 20  # two calls, three real FFTs each


def convlv_config(form):
    return {"workload": "realft convlv + correl, N=2^20 real f64, m=257 taps in a length-N "
                        "wrap-around buffer; one step = one convlv and one correl",
            "form": form, "l2": "flushed between timed steps (256 MiB write)"}


def cpu_convlv_step(x, r, y):
    import oracle as O
    st, a = O.convlv(x, r, 1)
    st2, b = O.correl(x, y)
    assert st == 0 and st2 == 0
    return a, b


def cpu_baseline_convlv(seconds, x, r, y):
    """Time the CPU oracle on whole steps for about `seconds` of work.  Returns
    the baseline record and the oracle's outputs of the step, which the GPU
    results are checked against."""
    import oracle as O
    threads = host_cores()
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
        "kind": "port", "host_cores": threads,
        "sample": "%d whole steps (convlv + correl, N=2^20) in %.1f s; the two forward "
                  "transforms of each call run on 2 threads as the reference's rayon::join "
                  "does, the transforms themselves are serial as in the crate" % (n, el),
    }


def run_reference_convlv(args):
    x, r, y = convlv_inputs()
    import oracle as O
    threads = host_cores()
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
        "config": convlv_config("fp64"), "requested_steps": args.steps,
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
    (ra, rb), cpu = cpu_baseline_convlv(args.cpu_seconds, x, r, y)
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
        "config": convlv_config(form), "nominal_flops_per_step": CONV_FLOPS,
        "e2e": {"value": e2e_val, "unit": "GFLOP/s", "steps": e2e_steps,
                "h2d_bytes_per_step": 4 * CONV_N * 8, "d2h_bytes_per_step": 2 * CONV_N * 8,
                "host_buffers": "pinned"},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s",
                     "frac": achieved / hbm, "traffic": traffic_of("convlv", form)[0],
                     "traffic_note": traffic_of("convlv", form)[1],
                     "kernel": "k_pass (Stockham pass)",
                     "peak_source": "%s MEASURED_PEAKS.json hbm_gbs" % hbm_kind if hbm_kind == "measured"
                     else "fallback 6.8 TB/s",
                     "launches": pass_n, "avg_launch_ms": pass_avg_ms,
                     "bytes_per_launch": pass_bytes / max(pass_n, 1)},
        "compute_roofline": {"bound": "fp64" if form == "fp64" else "fp32",
                             "achieved_tflops": pass_flops / (pass_ms / 1e3) / 1e12 if pass_ms else 0.0,
                             "peak_tflops": FP64_PEAK_TFLOPS if form == "fp64" else FP32_PEAK_TFLOPS,
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
    """One in-place complex FFT of 2^log2n points per step (device resident,
    input restored between steps outside the timed events)."""
    import torch
    import numrs_gb300 as nr
    from numrs_gb300 import workloads as W
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    log2n = args.log2n or 24
    nn = 1 << log2n
    x0 = torch.from_numpy(W.normal(W.BASE_SEED + 5, 2 * nn)).to(dev)
    d = x0.clone()
    acc = _accuracy_vs_fp64(args.form, x0, lambda t, form: nr.four1(t, nn, 1, form=form))
    big = nn * 16 >= (256 << 20)
    flush = None if big else torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    nr.set_async(True)

    def step():
        d.copy_(x0)
        if flush is not None:
            flush.zero_()

    for _ in range(max(args.warmup, 3)):
        step()
        nr.four1(d, nn, 1, form=args.form)
    torch.cuda.synchronize()
    total_ms, launches, clk = _timed_pre(args, local, step,
                                         lambda: nr.four1(d, nn, 1, form=args.form), args.steps)
    total_ms = max_over_ranks(total_ms, world)
    flops = 5.0 * nn * log2n
    nr.profile(True)
    for _ in range(min(args.steps, 20)):
        step()
        nr.four1(d, nn, 1, form=args.form)
    torch.cuda.synchronize()
    roof = _pass_roofline()
    nr.profile(False)
    nr.set_async(False)
    if rank != 0:
        return None
    t, note = traffic_of("four1_%d" % log2n, args.form)
    roof["traffic"], roof["traffic_note"] = t, note
    return _simple_line(args, world,
                        "four1 complex in-place FFT, nn=2^%d (%d MiB), i.i.d. N(0,1)" % (log2n, (16 * nn) >> 20),
                        flops, total_ms, args.steps, launches, clk,
                        {"roofline": roof, "accuracy": acc,
                         "l2": "input larger than L2" if big else "flushed between steps (256 MiB write)"})


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
    """The 20,000-transform batch (sizes 2^k, k uniform in 6..14, amplitudes
    10^u); one step = one batched call.  With several ranks the transforms are
    partitioned by work (numrs_gb300.shard) and every rank runs its share:
    the total work is fixed, so the scaling is strong."""
    import torch
    import numrs_gb300 as nr
    from numrs_gb300 import shard
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    sizes_all, host_all = batch_inputs()
    mine = shard.partition_by_work(sizes_all, world)[rank]
    sizes = sizes_all[mine]
    host = [host_all[i] for i in mine]
    buf = torch.from_numpy(np.concatenate(host)).to(dev)
    orig = buf.clone()
    starts = np.concatenate([[0], np.cumsum(2 * sizes)[:-1]])
    views = [buf[int(s):int(s) + 2 * int(n)] for s, n in zip(starts, sizes)]
    flops_all = float(sum(shard.transform_work(s) for s in sizes_all))
    nbytes = 2.0 * 8 * float(sum(2 * s for s in sizes_all))
    stream = torch.cuda.current_stream()
    nr.set_async(True)
    b = nr.FFTBatch(views, form=args.form)
    for _ in range(max(args.warmup, 3)):
        buf.copy_(orig)
        b.run(1)
    torch.cuda.synchronize()
    steps = args.steps
    ev = _events(steps)
    clocks = Clocks(local)
    barrier(world)
    clocks.start()
    time.sleep(0.3)
    nr.launch_count(reset=True)
    for i in range(steps):
        buf.copy_(orig)
        ev[i][0].record(stream)
        b.run(1)
        ev[i][1].record(stream)
    torch.cuda.synchronize()
    launches = nr.launch_count()
    clk = clocks.stop()
    ms = max_over_ranks(sum(a.elapsed_time(c) for a, c in ev), world)
    nr.set_async(False)
    if rank != 0:
        return None
    hbm, hbm_kind = peaks()
    gbs = nbytes * steps / (ms / 1e3) / 1e9
    t, note = traffic_of("batch", args.form)
    return _simple_line(
        args, world, "batched uneven four1: 20000 transforms, sizes 2^k, k uniform in 6..14, "
        "one persistent launch (CUDA graph) per rank", flops_all, ms, steps, launches, clk,
        {"transforms_per_s": len(sizes_all) * steps / (ms / 1e3),
         "scaling": "strong",
         "partition": "longest-processing-time by 5 nn log2 nn over %d rank(s); rank 0 holds "
                      "%d transforms" % (world, len(mine)),
         "roofline": {"bound": "hbm", "achieved": gbs, "peak": hbm, "unit": "GB/s",
                      "frac": gbs / hbm, "traffic": t, "traffic_note": note,
                      "kernel": "k_batch (persistent)"},
         "l2": "inputs (2.33 GB) larger than L2"})


def _simple_line(args, world, workload, flops, total_ms, steps, launches, clk, extra=None):
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


def _timed_pre(args, local, pre, step, steps):
    """As _timed, with pre() run before each step outside the timed events."""
    import torch
    import numrs_gb300 as nr
    stream = torch.cuda.current_stream()
    ev = _events(steps)
    clocks = Clocks(local)
    clocks.start()
    time.sleep(0.3)
    nr.launch_count(reset=True)
    for i in range(steps):
        pre()
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


def run_nd(args, world, rank, local):
    """fourn 256 x 256 x 512 complex, or rlft3 512^3 real; forward + inverse per step."""
    import torch
    import numrs_gb300 as nr
    from numrs_gb300 import workloads as W
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    nr.set_async(True)
    if args.workload == "fourn":
        shape = (256, 256, 512)
        n = int(np.prod(shape))
        re = W.plane_waves_torch(shape, dev).reshape(-1)
        im = W.plane_waves_torch(shape, dev, seed=W.BASE_SEED + 40).reshape(-1)
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
        d = W.plane_waves_torch(shape, dev).reshape(-1)
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
    # the same round trip captured once in a CUDA graph and replayed: the
    # device-side latency without the per-call host work (the library
    # launches on the caller's current stream)
    graph = {"us_per_roundtrip": None}
    try:
        g = torch.cuda.CUDAGraph()
        side = torch.cuda.Stream()
        side.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(side):
            step()
        torch.cuda.current_stream().wait_stream(side)
        torch.cuda.synchronize()
        with torch.cuda.graph(g):
            step()
        for _ in range(10):
            g.replay()
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        reps = 1000
        e0.record()
        for _ in range(reps):
            g.replay()
        e1.record()
        torch.cuda.synchronize()
        graph["us_per_roundtrip"] = 1e3 * e0.elapsed_time(e1) / reps
    except Exception as ex:  # capture refused: report why
        graph["note"] = str(ex).splitlines()[0][:200]
    nr.set_async(False)
    if rank != 0:
        return None
    # CPU baseline: the oracle's round trip on one core, about a second of work
    import oracle as O
    xs = x.copy()
    n_rt = 0
    t0 = time.perf_counter()
    while time.perf_counter() - t0 < 1.0:
        O.four1(xs, 4096, 1)
        O.four1(xs, 4096, -1)
        xs *= 1.0 / 4096
        n_rt += 1
    cpu_s = (time.perf_counter() - t0) / n_rt
    flops = 2 * 5.0 * 4096 * 12
    return _simple_line(args, world, "four1 N=4096 round trip (+1, -1, x1/N), one transform",
                        flops, total_ms, steps, launches, clk,
                        {"us_per_roundtrip": 1e3 * total_ms / steps,
                         "graph_replay": graph,
                         "accuracy": {"roundtrip_rel_l2": err},
                         "cpu_baseline": {"value": flops / cpu_s / 1e9, "unit": "GFLOP/s",
                                          "us_per_roundtrip": cpu_s * 1e6, "cores": 1,
                                          "kind": "port",
                                          "sample": "%d oracle round trips of 4096 points on one "
                                                    "host thread" % n_rt}})


def run_peaks(args, world, rank, local):
    """Arithmetic ceilings behind `compute_roofline`: FP64 and FP32 (TF32 off)
    GEMM throughput through torch's cuBLAS call, timed with CUDA events.  A
    DGEMM keeps the FP64 pipe at its DFMA rate; an SGEMM without TF32 keeps
    the FP32 pipe at its FFMA rate.  Not an FFT workload."""
    import torch
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    prev = torch.backends.cuda.matmul.allow_tf32
    torch.backends.cuda.matmul.allow_tf32 = False
    res = {}
    try:
        for name, dt, n, steps in (("fp64", torch.float64, 4096, 10), ("fp32", torch.float32, 8192, 20)):
            g = torch.Generator(device=dev)
            g.manual_seed(7)
            a = torch.randn(n, n, dtype=dt, device=dev, generator=g)
            b = torch.randn(n, n, dtype=dt, device=dev, generator=g)
            c = torch.empty_like(a)
            for _ in range(max(args.warmup, 3)):
                torch.matmul(a, b, out=c)
            torch.cuda.synchronize()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record()
            for _ in range(steps):
                torch.matmul(a, b, out=c)
            e1.record()
            torch.cuda.synchronize()
            ms = e0.elapsed_time(e1) / steps
            res[name] = {"tflops": 2.0 * n ** 3 / ms / 1e9, "ms_per_gemm": ms, "n": n, "gemms": steps}
            del a, b, c
    finally:
        torch.backends.cuda.matmul.allow_tf32 = prev
    if rank != 0:
        return None
    return {"metric": "GEMM TFLOP/s (FP64 and FP32 pipe ceilings)", "value": res["fp64"]["tflops"],
            "unit": "TFLOP/s", "n_gpus": world, "higher_is_better": True, "dtype": "f64",
            "data": "synthetic (seeded N(0,1) matrices)",
            "config": {"workload": "torch.matmul square GEMMs: f64 4096^3 and f32 8192^3, TF32 off"},
            "gemm": res, "used_in_bench": {"fp64_peak_tflops": FP64_PEAK_TFLOPS,
                                            "fp32_peak_tflops": FP32_PEAK_TFLOPS}}


def run_sharded(args, world, rank, local):
    """four1 of 2^log2n points (default 2^28, FP64) split over the ranks with
    the four-step schedule of numrs_gb300.dist: local column transforms, the
    twiddle kernel, one all-to-all, local row transforms, natural-order block
    input and output (two more all-to-alls).  Total work is fixed (strong
    scaling).  With --shares P in one process, the P shares live on this GPU
    and the exchanges are device copies: the whole transform's local work and
    data movement on one GPU."""
    import torch
    import numrs_gb300 as nr
    from numrs_gb300 import dist as D
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    log2n = args.log2n or LARGE_LOG2N
    N = 1 << log2n
    emulate = args.shares > 0
    P = args.shares if emulate else world
    x = large_input(log2n)
    parts = D.to_layout(x, N, P, "block")
    if emulate:
        src = [torch.from_numpy(p).to(dev) for p in parts]
        run = lambda: D.four1_sharded_local(src, N, 1, "block", "block", form=args.form)
    else:
        src = torch.from_numpy(parts[rank]).to(dev)
        run = lambda: D.four1_sharded(src, N, 1, "block", "block", form=args.form)
    del parts
    nr.set_async(True)
    out = run()
    torch.cuda.synchronize()
    # accuracy of this rank's (or the shares') output against the single-GPU transform
    ref = torch.from_numpy(x).to(dev)
    nr.four1(ref, N, 1, form=args.form)
    got = torch.cat(out) if emulate else out
    lo = 0 if emulate else rank * (2 * N // P)
    want = ref[lo:lo + got.numel()]
    err = float(torch.linalg.vector_norm(got - want) / torch.linalg.vector_norm(want))
    del ref, got, want, out
    torch.cuda.empty_cache()
    for _ in range(max(args.warmup, 3)):
        run()
    torch.cuda.synchronize()
    barrier(world)
    total_ms, launches, clk = _timed(args, local, run, None, args.steps)
    total_ms = max_over_ranks(total_ms, world)
    nr.set_async(False)
    if rank != 0:
        return None
    flops = 5.0 * N * log2n
    line = _simple_line(args, world, "four1 complex FFT, nn=2^%d split over %d %s with the four-step "
                        "schedule (one transform per step)" % (log2n, P, "shares on one GPU" if emulate else "ranks"),
                        flops, total_ms, args.steps, launches, clk,
                        {"accuracy": {"rel_l2_vs_single_gpu_four1": err}})
    # one transform per step whatever the rank count: total work is fixed
    line["value"] = flops * args.steps / (total_ms / 1e3) / 1e9
    line["scaling"] = "strong"
    line["config"]["shares"] = P
    line["config"]["exchange"] = "device copies (one process)" if emulate else "torch.distributed all_to_all_single"
    return line


def run_link(args, world, rank, local):
    """CPU-GPU link bandwidth through torch copies of a 4 GiB pinned host
    tensor (cudaMemcpyAsync), timed with CUDA events: host to device, device
    to host, and both at once on two streams.  The first and last passes of
    a transform of host data move its bytes over this link.  Not an FFT
    workload."""
    import torch
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    nbytes = 4 << 30
    h = torch.empty(nbytes, dtype=torch.uint8).pin_memory()
    h2 = torch.empty(nbytes, dtype=torch.uint8).pin_memory()
    d = torch.empty(nbytes, dtype=torch.uint8, device=dev)
    d2 = torch.empty(nbytes, dtype=torch.uint8, device=dev)
    s1, s2 = torch.cuda.Stream(), torch.cuda.Stream()

    def timed(fn, reps=3):
        best = None
        for _ in range(reps):
            torch.cuda.synchronize()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record()
            fn()
            torch.cuda.synchronize()
            e1.record()
            torch.cuda.synchronize()
            ms = e0.elapsed_time(e1)
            best = ms if best is None else min(best, ms)
        return best

    def both():
        with torch.cuda.stream(s1):
            d.copy_(h, non_blocking=True)
        with torch.cuda.stream(s2):
            h2.copy_(d2, non_blocking=True)

    for _ in range(max(args.warmup, 1)):
        d.copy_(h, non_blocking=True)
    res = {"h2d_gbs": nbytes / timed(lambda: d.copy_(h, non_blocking=True)) / 1e6,
           "d2h_gbs": nbytes / timed(lambda: h.copy_(d, non_blocking=True)) / 1e6,
           "both_at_once_gbs_each_way": nbytes / timed(both) / 1e6}
    if rank != 0:
        return None
    return {"metric": "CPU-GPU link GB/s (pinned host memory)", "value": res["h2d_gbs"],
            "unit": "GB/s", "n_gpus": world, "higher_is_better": True, "dtype": "u8",
            "data": "4 GiB pinned host tensors", "config": {"workload": "torch copies host <-> device"},
            "link": res}


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
    fn = {"large": run_large, "four1": run_four1, "batch": run_batch, "fourn": run_nd,
          "rlft3": run_nd, "c1": run_c1, "convbatch": run_convbatch,
          "peaks": run_peaks, "sharded": run_sharded, "link": run_link}.get(args.workload)
    if fn is None:
        run_convlv(args, world, rank, local)
    else:
        line = fn(args, world, rank, local)
        if line:
            print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
