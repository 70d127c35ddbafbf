#!/usr/bin/env python3
"""Benchmark of the GB300 FFT path on fyFFT's precision-sweep workload.

Workload (one "step"): one forward pass over complex<float> transforms of lengths
N in {2520, 59049, 117649, 2^20, 1009, 65537, 999983, 131074}, batch 64 each (7-smooth mixed
radix, pure radix 3 / 7, power of two, Rader primes, Bluestein prime and 2*65537), inputs
i.i.d. N(0,1) re/im from seed 1.  Metric: GFLOP/s with the fixed count 5 N log2 N per
transform; GB/s with 2 N sizeof(complex) bytes per transform; fraction of the measured HBM
roofline.  Inputs (1.24 GB per step) are larger than L2, so no flush is needed.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                  [--workload sweep|c1|c5|uneven]

N > 1 runs one independent replica per GPU (the path does not shard): value is the total
over ranks divided by the max time over ranks.  --impl reference times the CPU restatement of
the reference's algorithm (oracle/, FP64) on the host cores on a bounded sample of the same
workload (the reference's own AVX2 code is x86-only).
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "FFT GFLOP/s (5N log2N/t) & %HBM roofline, batched vs plain, rel-L2<=2e-6 vs FP64"
SWEEP_SIZES = [2520, 59049, 117649, 1 << 20, 1009, 65537, 999983, 131074]
SWEEP_BATCH = 64
SEED = 1


def flops(n: int) -> float:
    return 5.0 * n * math.log2(n) if n > 1 else 0.0


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


# ----------------------------------------------------------------------------------------------
# clocks during the timed region
# ----------------------------------------------------------------------------------------------

class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200", "-i", str(self.device)],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
            time.sleep(0.6)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        rows = []
        for line in open(self.path):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                rows.append((float(parts[1]), float(parts[2]), float(parts[3]), parts[5:9]))
            except ValueError:
                continue
        os.unlink(self.path)
        if not rows:
            return None
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[3][i].lower().startswith("active")})
        return {"sm_mhz": statistics.median(r[0] for r in rows), "sm_max_mhz": max(r[1] for r in rows),
                "power_w_max": max(r[2] for r in rows), "samples": len(rows), "reasons": reasons}


# ----------------------------------------------------------------------------------------------
# workloads
# ----------------------------------------------------------------------------------------------

def workload(name: str, sizes=None, batch=None):
    """[(n, batch, dtype, dist, seed)] and a description."""
    if name == "sweep" and (sizes or batch):
        sz = sizes or SWEEP_SIZES
        b = batch or SWEEP_BATCH
        return ([(n, b, "complex64", "normal", SEED) for n in sz],
                f"sweep subset: complex<float> N in {sz} x batch {b}, N(0,1) seed 1")
    if name == "sweep":
        return ([(n, SWEEP_BATCH, "complex64", "normal", SEED) for n in SWEEP_SIZES],
                "precision sweep: complex<float> N in {2520, 59049, 117649, 2^20, 1009, 65537, "
                "999983, 131074} x batch 64, N(0,1) seed 1, one forward pass over all sizes per step")
    if name == "c1":
        return ([(4096, 256, "complex128", "uniform", 0)],
                "plain forward complex<double> N=4096 x batch 256, uniform[-1,1] seed 0")
    if name == "c5":
        return ([(1 << 27, 1, "complex64", "uniform", 4), (1 << 24, 8, "complex64", "uniform", 4)],
                "large: complex<float> N=2^27 x 1 and N=2^24 x 8, uniform[-1,1] seed 4")
    raise ValueError(name)


def run_ours(args, rank: int, world: int):
    import torch
    import fyfft_gb300 as fg

    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    stream = torch.cuda.current_stream()
    items, desc = workload(args.workload, args.sizes, args.batch)
    hbm_peak, peak_src = peaks()

    # schedule choice measured on this device before anything is timed (cached in a temp file)
    if not args.no_autotune:
        cache = args.autotune_cache or os.path.join(tempfile.gettempdir(),
                                                    f"fyfft_gb300_bench_autotune_{os.getpid()}.json")
        os.environ["FYG_AUTOTUNE_CACHE"] = cache
        have = set()
        if args.autotune_cache and os.path.exists(cache):
            with open(cache) as f:
                have = set(json.load(f).get("entries", {}))
        for (n, batch, dt, *_ ) in items:
            if f"{'c32' if dt == 'complex64' else 'c64'}:{n}" not in have:
                fg.autotune(n, dt, batch, cache_path=cache)
    plan_flags = 0 if args.no_autotune else fg.FYG_FLAG_AUTOTUNED

    plans, xin, yout, host_in, host_out = [], [], [], [], []
    for (n, batch, dt, dist, seed) in items:
        npdt = np.complex64 if dt == "complex64" else np.complex128
        tdt = torch.complex64 if dt == "complex64" else torch.complex128
        x = fg.fill_random(seed, n * batch, npdt, dist)
        hx = torch.from_numpy(x).pin_memory()
        host_in.append(hx)
        host_out.append(torch.empty_like(hx).pin_memory())
        xin.append(hx.to(f"cuda:{dev}"))
        yout.append(torch.empty(n * batch, dtype=tdt, device=f"cuda:{dev}"))
        plans.append(fg.FFT1D_C2C_invoker(n, dt, batch, flags=plan_flags))
    eb = [8 if dt == "complex64" else 16 for (_, _, dt, _, _) in items]
    step_flops = sum(flops(n) * b for (n, b, *_ ) in items)
    step_bytes = sum(2 * n * b * e for (n, b, *_), e in zip(items, eb))
    launches_per_step = sum(p.launches() for p in plans)

    def step():
        for p, x, y in zip(plans, xin, yout):
            p.dispatch(False, x, y, stream)

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()

    # per-size device times (outside the headline region, for the breakdown)
    per_size = {}
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    for (n, b, *_ ), p, x, y, e in zip(items, plans, xin, yout, eb):
        reps = 5
        ev0.record(stream)
        for _ in range(reps):
            p.dispatch(False, x, y, stream)
        ev1.record(stream)
        torch.cuda.synchronize()
        ms = ev0.elapsed_time(ev1) / reps
        gbs = 2 * n * b * e / (ms * 1e-3) / 1e9
        per_size[str(n)] = {"ms": round(ms, 4), "gflops": round(flops(n) * b / (ms * 1e-3) / 1e9, 1),
                            "gbs": round(gbs, 1), "hbm_frac": round(gbs / hbm_peak, 3),
                            "gpu_strategy": int(fg.FFT1D_C2C_invoker.gpu_execution_strategy(n)),
                            "kernels": p.launches(), "conv_length": p.info()["conv_length"],
                            "passes": p.info()["passes"]}

    # headline: K steps, events on the launching stream, per-pass events for the roofline
    for p in plans:
        p.profile(True)
    clocks = ClockSampler(dev)
    clocks.start()
    barrier()
    torch.cuda.synchronize()
    t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    t0.record(stream)
    for _ in range(args.steps):
        step()
    t1.record(stream)
    torch.cuda.synchronize()
    barrier()
    clk = clocks.stop()
    ms_total = t0.elapsed_time(t1)
    if world > 1:
        tt = torch.tensor([ms_total], device=f"cuda:{dev}")
        torch.distributed.all_reduce(tt, op=torch.distributed.ReduceOp.MAX)
        ms_total = float(tt.item())
    ms_step = ms_total / args.steps
    value = step_flops * world / (ms_step * 1e-3) / 1e9

    # dominant kernel: the pass with the largest accumulated time
    best = None
    for (n, b, *_ ), p in zip(items, plans):
        for i, (tms, nl, bpl) in enumerate(p.profile_read()):
            if nl and (best is None or tms > best[0]):
                best = (tms, nl, bpl, n, i, len(p.profile_read()), p.describe()[i])
        p.profile(False)
    roof = None
    if best:
        tms, nl, bpl, n, i, npass, pdesc = best
        kind = "k_fast" if "kernel=fast" in pdesc else "k_pass"
        shape = " ".join(w for w in pdesc.split() if w.startswith(("R=", "C=")))
        avg_ms = tms / nl
        achieved = bpl / (avg_ms * 1e-3) / 1e9
        share = tms / (ms_total if ms_total > 0 else 1)
        roof = {"bound": "hbm", "achieved": round(achieved, 1), "peak": hbm_peak, "unit": "GB/s",
                "frac": round(achieved / hbm_peak, 3), "traffic": read_traffic(n, i),
                "peak_source": f"{peak_src} (MEASURED_PEAKS.json hbm_gbs)" if peak_src == "measured" else peak_src,
                "kernel": f"{kind} {shape} (N={n} pass {i + 1}/{npass}{', mid' if ' mid' in pdesc else ''})",
                "bytes_per_launch": int(bpl),
                "avg_launch_ms": round(avg_ms, 4), "share_of_step": round(share, 3)}

    # end to end through the public API with pinned host buffers (H2D + compute + D2H per step)
    # each step timed on its own; the value uses the median step (host-side copy bandwidth on a
    # shared machine fluctuates), every step time is reported
    e2e_steps = max(1, min(args.steps, args.e2e_steps))
    hx_np = [h.numpy() for h in host_in]
    hy_np = [h.numpy() for h in host_out]
    for _ in range(2):
        for p, x, y in zip(plans, hx_np, hy_np):
            p.dispatch(False, x, y)
    barrier()
    step_times = []
    for _ in range(e2e_steps):
        ts = time.perf_counter()
        for p, x, y in zip(plans, hx_np, hy_np):
            p.dispatch(False, x, y)
        step_times.append(time.perf_counter() - ts)
    te = statistics.median(step_times)
    if world > 1:
        tt = torch.tensor([te], device=f"cuda:{dev}")
        torch.distributed.all_reduce(tt, op=torch.distributed.ReduceOp.MAX)
        te = float(tt.item())
    e2e_value = step_flops * world / te / 1e9
    in_bytes = sum(n * b * e for (n, b, *_), e in zip(items, eb))
    # this box's pinned copy bandwidth (the e2e path is bound by it): one direction at a time
    # and both directions at once, 256 MB per copy
    cb = 256 << 20
    hb = torch.empty(cb, dtype=torch.uint8).pin_memory()
    hb2 = torch.empty(cb, dtype=torch.uint8).pin_memory()
    db = torch.empty(cb, dtype=torch.uint8, device=f"cuda:{dev}")
    db2 = torch.empty(cb, dtype=torch.uint8, device=f"cuda:{dev}")
    s_a, s_b = torch.cuda.Stream(), torch.cuda.Stream()

    def copy_time(fn, reps=3):
        fn()
        torch.cuda.synchronize()
        ta = time.perf_counter()
        for _ in range(reps):
            fn()
        torch.cuda.synchronize()
        return (time.perf_counter() - ta) / reps

    def both():
        with torch.cuda.stream(s_a):
            db.copy_(hb, non_blocking=True)
        with torch.cuda.stream(s_b):
            hb2.copy_(db2, non_blocking=True)
    h2d_gbs = cb / copy_time(lambda: db.copy_(hb, non_blocking=True)) / 1e9
    d2h_gbs = cb / copy_time(lambda: hb.copy_(db, non_blocking=True)) / 1e9
    bidir_gbs = cb / copy_time(both) / 1e9
    copy_floor_ms = in_bytes / (bidir_gbs * 1e9) * 1e3
    del hb, hb2, db, db2

    out = {
        "metric": METRIC, "value": round(value, 1), "unit": "GFLOP/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms_step, 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32" if all(it[2] == "complex64" for it in items) else "f64",
        "data": "synthetic (seeded counter-based generator, fyg_fill_random)",
        "config": {"workload": desc, "sizes": [it[0] for it in items], "batch": [it[1] for it in items],
                   "l2": f"inputs larger than L2 ({in_bytes / 1e9:.2f} GB per step), no flush",
                   "parallelism": "replicas" if world > 1 else "single GPU",
                   "schedules": "planner defaults" if args.no_autotune else
                   "autotuned on this device before timing (fyg_autotune; conv length, pass radix, cols)"},
        "gbs": round(step_bytes * world / (ms_step * 1e-3) / 1e9, 1),
        "hbm_frac_step": round(step_bytes / (ms_step * 1e-3) / 1e9 / hbm_peak, 3),
        "roofline": roof,
        "e2e": {"value": round(e2e_value, 1), "unit": "GFLOP/s", "h2d_bytes_per_step": int(in_bytes),
                "d2h_bytes_per_step": int(in_bytes), "steps": e2e_steps,
                "path": "fyg_execute on pinned host buffers (chunked H2D / kernels / D2H on three streams, "
                        "returns when the result is in host memory)",
                "ms_per_step": round(te * 1e3, 3), "step_ms": [round(t * 1e3, 3) for t in step_times],
                "box_copy_gbs": {"h2d": round(h2d_gbs, 1), "d2h": round(d2h_gbs, 1),
                                 "each_way_concurrent": round(bidir_gbs, 1)},
                "copy_floor_ms_per_step": round(copy_floor_ms, 3)},
        "gpu_launches": int(launches_per_step * args.steps),
        "clocks": clk,
        "per_size": per_size,
    }
    if not args.no_uneven:
        out["batched_vs_plain"] = uneven_batch(dev, stream, no_autotune=args.no_autotune)
    if rank == 0 and not args.no_cpu_baseline:
        out["cpu_baseline"] = cpu_baseline(items, args, check=(plans, yout))
    return out


def uneven_batch(dev: int, stream, reps: int = 10, no_autotune: bool = False):
    """The mixed-length batch (4096 lengths in [16, 65536], 7-smooth / prime / other, seed 2):
    one persistent launch (CUDA graph) against one launch sequence per transform."""
    import torch
    import fyfft_gb300 as fg
    from fyfft_gb300.workloads import uneven_lengths
    lengths = uneven_lengths(4096, 2)
    t0 = time.perf_counter()
    tuned = None
    if not no_autotune:
        # option sets of the persistent launch timed on this device, cached (FYG_AUTOTUNE_CACHE)
        fg.autotune_batch(lengths, cache_path=os.environ.get("FYG_AUTOTUNE_CACHE"))
        tuned = round(time.perf_counter() - t0, 2)
    t1 = time.perf_counter()
    b = fg.UnevenBatch(lengths, flags=0 if no_autotune else fg.FYG_FLAG_AUTOTUNED)
    create_s = time.perf_counter() - t1
    x = torch.from_numpy(fg.fill_random(2, sum(lengths), np.complex64, "uniform")).to(f"cuda:{dev}")
    y = torch.empty_like(x)
    fl = sum(flops(n) for n in lengths)
    res = {"workload": "4096 complex<float> transforms, lengths log-uniform in [16, 65536] "
                       "(0.70 7-smooth / 0.15 prime / 0.15 other), uniform[-1,1] seed 2, packed back to back",
           "points": int(sum(lengths)), "distinct_lengths": len(set(lengths)), "create_s": round(create_s, 2),
           "autotune_s": tuned}
    for name, f in (("batched", lambda: b.execute(x, y, stream=stream)),
                    ("plain", lambda: b.execute_plain(x, y, stream=stream))):
        for _ in range(3):
            f()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            f()
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / reps
        res[f"{name}_ms"] = round(ms, 4)
        res[f"{name}_gflops"] = round(fl / (ms * 1e-3) / 1e9, 1)
    res["status"] = b.status(stream)
    if not no_autotune:
        cache = os.environ.get("FYG_AUTOTUNE_CACHE")
        if cache and os.path.exists(cache):
            with open(cache) as f:
                ent = [v for k, v in json.load(f).get("entries", {}).items() if k.startswith("batch32:4096:")]
            if ent:
                res["autotuned"] = {"stage_radix_cap": ent[0]["max_pass_radix"], "single_tile_kb": ent[0]["cols"],
                                    "tuner_ms": ent[0]["ms"]}
    res["speedup"] = round(res["plain_ms"] / res["batched_ms"], 2)
    return res


def read_traffic(n: int, pass_index: int):
    """DRAM bytes per launch from the committed ncu summary (profiles/traffic.txt), or None."""
    path = os.path.join(ROOT, "profiles", "traffic.txt")
    if not os.path.exists(path):
        return None
    for line in open(path):
        parts = line.split()
        if len(parts) >= 3 and not line.startswith("#") and parts[0] == f"N={n}" and parts[1] == f"pass={pass_index + 1}":
            return float(parts[2])
    return None


# ----------------------------------------------------------------------------------------------
# CPU baseline (oracle port, FP64, all host threads, bounded sample)
# ----------------------------------------------------------------------------------------------

def cpu_baseline(items, args, check=None):
    from oracle import oracle as O
    import fyfft_gb300 as fg
    threads = os.cpu_count() or 1
    tot_flops, tot_s, sample, errs = 0.0, 0.0, [], {}
    for idx, (n, batch, dt, dist, seed) in enumerate(items):
        cnt = min(batch, threads) if n < (1 << 24) else 1
        npdt = np.complex64 if dt == "complex64" else np.complex128
        x = fg.fill_random(seed, n * cnt, npdt, dist).reshape(cnt, n)
        t = time.perf_counter()
        y = O.fft_batch(x, inverse=False, threads=threads)
        dt_s = time.perf_counter() - t
        tot_flops += flops(n) * cnt
        tot_s += dt_s
        sample.append(f"{cnt}x{n}")
        if check is not None:
            plans, youts = check
            g = youts[idx][: n * cnt].reshape(cnt, n).cpu().numpy()
            errs[str(n)] = float(f"{O.rel_l2(g, y):.3e}")
    res = {"value": round(tot_flops / tot_s / 1e9, 3), "unit": "GFLOP/s", "cores": threads, "kind": "port",
           "sample": "first transforms of each size (" + ", ".join(sample) + "), FP64 oracle restating the "
                     "reference's radix/Rader/Bluestein algorithm, one transform per thread",
           "seconds": round(tot_s, 2)}
    if errs:
        res["gpu_rel_l2_vs_fp64_oracle"] = errs
    return res


def run_reference(args, rank: int, world: int):
    items, desc = workload(args.workload, args.sizes, args.batch)
    if rank != 0:
        return None
    from oracle import oracle as O
    import fyfft_gb300 as fg
    threads = os.cpu_count() or 1
    # bounded sample: per step, `threads` transforms of each size below 2^24 (one of larger ones)
    xs = []
    for (n, batch, dt, dist, seed) in items:
        cnt = min(batch, threads) if n < (1 << 24) else 1
        npdt = np.complex64 if dt == "complex64" else np.complex128
        xs.append((n, fg.fill_random(seed, n * cnt, npdt, dist).reshape(cnt, n)))
    step_flops = sum(flops(n) * x.shape[0] for n, x in xs)
    # keep the whole run within a few minutes: time one step first, then cap the step count
    def step():
        for n, x in xs:
            O.fft_batch(x, inverse=False, threads=threads)
    t = time.perf_counter()
    step()
    one = time.perf_counter() - t
    budget = 150.0
    steps = max(1, min(args.steps, int(budget / max(one, 1e-3)) - args.warmup))
    warm = min(args.warmup, max(0, int(budget / max(one, 1e-3)) - steps))
    for _ in range(warm):
        step()
    t = time.perf_counter()
    for _ in range(steps):
        step()
    el = time.perf_counter() - t
    value = step_flops / (el / steps) / 1e9
    sample = ", ".join(f"{x.shape[0]}x{n}" for n, x in xs)
    return {
        "impl": "reference", "metric": METRIC, "value": round(value, 3), "unit": "GFLOP/s", "n_gpus": world,
        "steps": steps, "warmup": warm, "ms_per_step": round(el / steps * 1e3, 2), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64 (oracle port of the reference's algorithm)",
        "data": "synthetic (seeded counter-based generator, fyg_fill_random)",
        "config": {"workload": desc, "sizes": [it[0] for it in items], "batch": [it[1] for it in items],
                   "sample_per_step": sample},
        "cpu_baseline": {"value": round(value, 3), "unit": "GFLOP/s", "cores": threads, "kind": "port",
                         "sample": f"per step: {sample}; the reference's own AVX2 C++ is x86-only and "
                                   f"does not build on this {os.uname().machine} host"},
        "e2e": {"value": round(value, 3), "unit": "GFLOP/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=300)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="sweep", choices=["sweep", "c1", "c5"])
    ap.add_argument("--e2e-steps", type=int, default=7)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--sizes", type=lambda v: [int(t) for t in v.split(",")], default=None,
                    help="sweep subset (comma-separated lengths), for small profiling cases")
    ap.add_argument("--batch", type=int, default=None, help="sweep batch override")
    ap.add_argument("--autotune-cache", default=None,
                    help="autotune cache file; tuning is skipped when it already holds every size")
    ap.add_argument("--no-autotune", action="store_true", help="planner defaults instead of measured schedules")
    ap.add_argument("--no-uneven", action="store_true", help="skip the mixed-length batch comparison")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if args.impl == "reference":
        out = run_reference(args, rank, world)
        if rank == 0:
            print(json.dumps(out))
        return
    if world > 1:
        import torch
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        torch.distributed.init_process_group("nccl")
    out = run_ours(args, rank, world)
    if rank == 0:
        print(json.dumps(out))
    if world > 1:
        import torch
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
