#!/usr/bin/env python3
"""Benchmark of the GB300 FFT path on fyFFT's precision-sweep workload.

Workload (one "step"): one forward pass over complex<float> transforms of lengths
N in {2520, 59049, 117649, 2^20, 1009, 65537, 999983, 131074}, batch 64 each (7-smooth mixed
radix, pure radix 3 / 7, power of two, Rader primes, Bluestein prime and 2*65537), inputs
i.i.d. N(0,1) re/im from seed 1.  Metric: GFLOP/s with the fixed count 5 N log2 N per
transform; GB/s with 2 N sizeof(complex) bytes per transform; fraction of the measured HBM
roofline.  Inputs (1.24 GB per step) are larger than L2, so no flush is needed.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                  [--workload sweep|c1|c5]

The default run also reports, as extra keys of the same JSON line: the same figure over the
lengths the reference can run (ref_runnable_subset), the other configurations timed on their
own (configs: C1 complex<double> 4096 x 256, C4 forward + adjoint, C5 2^27 x 1 and 2^24 x 8, each
with its dominant pass's roofline), the mixed-length batch in one persistent launch against one
launch sequence per plan (batched_vs_plain), and the CPU baseline with the GPU's rel-L2 against
the reference and the FP64 oracle.

N > 1 (torchrun, one rank per GPU) shards a global batch of batch x N transforms per length
with the library's partition (fyg_partition): each rank runs its contiguous shard of the
seeded stream, no collective on the data path; value is the units all ranks processed divided
by the max time over ranks (weak scaling).  --impl reference times the reference's own
C++ FFT (oracle/_ref/libfyref.so: the unmodified reference, built natively with AVX2 on x86-64
and against oracle/ref/portable_intrin.h on the aarch64 GPU hosts) on all host cores, one plan
per thread, over the whole batch of every workload length it can run.
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

    # schedule choice measured on this device before anything is timed (cached in a temp file,
    # seeded from the committed choices for this device type when its signature matches, so
    # that repeated runs use the same schedules)
    if not args.no_autotune:
        cache = args.autotune_cache or os.path.join(tempfile.gettempdir(),
                                                    f"fyfft_gb300_bench_autotune_{os.getpid()}.json")
        os.environ["FYG_AUTOTUNE_CACHE"] = cache
        seed = os.path.join(ROOT, "fyfft_gb300", "tuned", "gb300_autotune.json")
        if not os.path.exists(cache) and os.path.exists(seed) and not args.retune:
            import shutil
            shutil.copyfile(seed, cache)
        have = set()
        if os.path.exists(cache):
            with open(cache) as f:
                doc = json.load(f)
            if fg.device_signature() == doc.get("device"):
                have = set(doc.get("entries", {}))
        for (n, batch, dt, *_ ) in items:
            if f"{'c32' if dt == 'complex64' else 'c64'}:{n}" not in have:
                fg.autotune(n, dt, batch, cache_path=cache)
    plan_flags = (0 if args.no_autotune else fg.FYG_FLAG_AUTOTUNED) | args.plan_flags

    # N > 1: the global batch of every length is batch x N transforms, sharded by the library's
    # partition (fyg_partition); this rank runs its contiguous shard of the seeded stream, so
    # per-GPU work stays fixed as N grows (weak scaling) and no rank repeats another's work
    shards = []
    for i, (n, batch, dt, dist, seed) in enumerate(items):
        b = fg.partition(batch * world, world)
        shards.append(b[rank])
        items[i] = (n, b[rank + 1] - b[rank], dt, dist, seed)
    plans, xin, yout, host_in, host_out = [], [], [], [], []
    for (n, batch, dt, dist, seed), first in zip(items, shards):
        npdt = np.complex64 if dt == "complex64" else np.complex128
        tdt = torch.complex64 if dt == "complex64" else torch.complex128
        x = fg.fill_random(seed, n * batch, npdt, dist, first=first * n)
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
        reps = 5 if n * b >= (1 << 22) else 20
        # a spin kernel first, so that the host has enqueued every repetition before the first
        # starts: the events then bracket device time, not host launch latency (small sizes)
        torch.cuda._sleep(100_000_000)
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
    roof = dominant_pass([(n, p) for (n, *_ ), p in zip(items, plans)], ms_total, hbm_peak)
    if roof:
        roof["peak_source"] = f"{peak_src} (MEASURED_PEAKS.json hbm_gbs)" if peak_src == "measured" else peak_src
        roof["share_of_step"] = roof.pop("share")

    # end to end through the public API with pinned host buffers (H2D + compute + D2H per step)
    # each step timed on its own; the value uses the median step (host-side copy bandwidth on a
    # shared machine fluctuates), every step time is reported
    e2e_steps = max(1, min(args.steps, args.e2e_steps))
    # every size enqueued without blocking (fyg_execute_async): a size's copies overlap the
    # kernels of its neighbours; the step ends when the stream has every output in host memory
    hx_np = [h.numpy() for h in host_in]
    hy_np = [h.numpy() for h in host_out]

    def e2e_step():
        for p, x, y in zip(plans, hx_np, hy_np):
            p.dispatch(False, x, y, stream, blocking=False)
        for p in plans:
            p.join(stream)
        stream.synchronize()
    for _ in range(2):
        e2e_step()
    barrier()
    step_times = []
    for _ in range(e2e_steps):
        ts = time.perf_counter()
        e2e_step()
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
                   "parallelism": (f"batch sharded over {world} GPUs (fyg_partition, no collective; "
                                   f"global batch = per-GPU batch x {world})") if world > 1 else "single GPU",
                   "schedules": "planner defaults" if args.no_autotune else
                   "autotuned on this device type (fyg_autotune: conv length, pass radix and order, columns and "
                   "threads per transform, tile width; missing lengths tuned before timing)"},
        "gbs": round(step_bytes * world / (ms_step * 1e-3) / 1e9, 1),
        "hbm_frac_step": round(step_bytes / (ms_step * 1e-3) / 1e9 / hbm_peak, 3),
        "roofline": roof,
        "e2e": {"value": round(e2e_value, 1), "unit": "GFLOP/s", "h2d_bytes_per_step": int(in_bytes),
                "d2h_bytes_per_step": int(in_bytes), "steps": e2e_steps,
                "path": "fyg_execute_async on pinned host buffers (per size: chunked H2D / kernels / D2H on "
                        "three streams; sizes pipeline; timed until every output is in host memory)",
                "ms_per_step": round(te * 1e3, 3), "step_ms": [round(t * 1e3, 3) for t in step_times],
                "box_copy_gbs": {"h2d": round(h2d_gbs, 1), "d2h": round(d2h_gbs, 1),
                                 "each_way_concurrent": round(bidir_gbs, 1)},
                "copy_floor_ms_per_step": round(copy_floor_ms, 3)},
        "gpu_launches": int(launches_per_step * args.steps),
        "clocks": clk,
        "per_size": per_size,
    }
    # the same figure over the lengths the reference can run (the reference arm's value is
    # taken over those; 65537, 999983 and 131074 fall to its O(N^2) DFT)
    sub = [(n, b) for (n, b, *_ ) in items if n in REF_RUNNABLE]
    if sub:
        sub_ms = sum(per_size[str(n)]["ms"] for n, _ in sub)
        out["ref_runnable_subset"] = {
            "sizes": [n for n, _ in sub],
            "value": round(sum(flops(n) * b for n, b in sub) / (sub_ms * 1e-3) / 1e9, 1), "unit": "GFLOP/s",
            "ms_per_step": round(sub_ms, 4), "from": "per_size device times (events around back-to-back repetitions)"}
    uneven = None
    if not args.no_uneven:
        out["batched_vs_plain"], uneven = uneven_batch(dev, stream, no_autotune=args.no_autotune, rank=rank,
                                                       world=world)
    if not args.no_configs and args.workload == "sweep" and not args.sizes:
        del xin, host_in, host_out
        out["configs"] = measure_configs(dev, stream, hbm_peak, plan_flags)
    if rank == 0 and not args.no_cpu_baseline:
        out["cpu_baseline"] = cpu_baseline(items, args, check=(plans, yout), uneven=uneven)
    return out


REF_RUNNABLE = (2520, 59049, 117649, 1 << 20, 1009)
FP64_PEAK_TFLOPS = 1.25     # nominal dense FP64 rate of a GB300 (no measured figure exists)


def dominant_pass(plans_items, total_ms, hbm_peak):
    """Roofline entry of the pass with the largest accumulated event time."""
    best = None
    for n, p in plans_items:
        prof = p.profile_read()
        for i, (tms, nl, bpl) in enumerate(prof):
            if nl and (best is None or tms > best[0]):
                best = (tms, nl, bpl, n, i, len(prof), p.describe()[i])
        p.profile(False)
    if not best:
        return None
    tms, nl, bpl, n, i, npass, pdesc = best
    kind = "k_fast" if "kernel=fast" in pdesc else "k_split" if "kernel=split" in pdesc else "k_pass"
    shape = " ".join(w for w in pdesc.split() if w.startswith(("R=", "C=")))
    avg_ms = tms / nl
    achieved = bpl / (avg_ms * 1e-3) / 1e9
    return {"bound": "hbm", "achieved": round(achieved, 1), "peak": hbm_peak, "unit": "GB/s",
            "frac": round(achieved / hbm_peak, 3), "traffic": read_traffic(n, i),
            "kernel": f"{kind} {shape} (N={n} pass {i + 1}/{npass}{', mid' if ' mid' in pdesc else ''})",
            "bytes_per_launch": int(bpl), "avg_launch_ms": round(avg_ms, 4),
            "share": round(tms / total_ms, 3) if total_ms > 0 else None}


def measure_configs(dev: int, stream, hbm_peak: float, plan_flags: int, reps: int = 10):
    """The other configurations, each timed on its own (events on the launching stream, inputs
    resident, larger than L2 except C1's 33.5 MB, which is re-read from L2 between repetitions
    unless flushed: C1 flushes L2 with a 256 MB write before every repetition)."""
    import torch
    import fyfft_gb300 as fg
    res = {}
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=f"cuda:{dev}")

    def timed(fn, reps, flush_l2=False):
        for _ in range(3):
            fn()
        torch.cuda.synchronize()
        tot = 0.0
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        for _ in range(reps):
            if flush_l2:
                flush.zero_()
            e0.record(stream)
            fn()
            e1.record(stream)
            torch.cuda.synchronize()
            tot += e0.elapsed_time(e1)
        return tot / reps

    def case(n, batch, dt, dist, seed, what="forward"):
        npdt = np.complex64 if dt == "complex64" else np.complex128
        esz = 8 if dt == "complex64" else 16
        x = torch.empty(n * batch, dtype=torch.complex64 if dt == "complex64" else torch.complex128,
                        device=f"cuda:{dev}")
        fg.fill_random_device(seed, x, dist, stream)
        y = torch.empty_like(x)
        p = fg.FFT1D_C2C_invoker(n, dt, batch, flags=plan_flags)
        if what == "forward":
            fn = lambda: p.dispatch(False, x, y, stream)  # noqa: E731
            nt = 1
        else:
            g = torch.empty_like(x)
            fg.fill_random_device(3, g, "normal", stream)
            gx = torch.empty_like(x)

            def fn():
                p.dispatch(False, x, y, stream)
                p.adjoint(g, gx, 1.0, stream)
            nt = 2
        small = 2 * n * batch * esz < (128 << 20)
        ms = timed(fn, reps, flush_l2=small)
        p.profile(True)
        fn()
        torch.cuda.synchronize()
        roof = dominant_pass([(n, p)], ms, hbm_peak)
        gbs = nt * 2 * n * batch * esz / (ms * 1e-3) / 1e9
        gfl = nt * flops(n) * batch / (ms * 1e-3) / 1e9
        r = {"n": n, "batch": batch, "dtype": dt, "ms": round(ms, 4), "gflops": round(gfl, 1),
             "gbs": round(gbs, 1), "hbm_frac": round(gbs / hbm_peak, 3), "passes": p.info()["passes"],
             "conv_length": p.info()["conv_length"], "roofline": roof,
             "l2": "flushed (256 MB write) before each repetition" if small else "inputs larger than L2"}
        if dt == "complex128":
            r["fp64_frac_of_nominal"] = round(gfl / (FP64_PEAK_TFLOPS * 1e3), 3)
        del x, y
        return r

    res["c1"] = {"workload": "plain forward complex<double> N=4096 x 256, uniform[-1,1] seed 0",
                 **case(4096, 256, "complex128", "uniform", 0)}
    res["c4"] = {"workload": "forward + adjoint (F^H g), complex<float>, N(0,1) seed 3 / g seed 3",
                 "cases": [case(1 << 20, 16, "complex64", "normal", 3, "grad"),
                           case(100003, 32, "complex64", "normal", 3, "grad")]}
    res["c5"] = {"workload": "large HBM-bound: complex<float> N=2^27 x 1 and 2^24 x 8, uniform[-1,1] seed 4",
                 "cases": [case(1 << 27, 1, "complex64", "uniform", 4),
                           case(1 << 24, 8, "complex64", "uniform", 4)]}
    del flush
    torch.cuda.empty_cache()
    return res


def uneven_batch(dev: int, stream, reps: int = 10, no_autotune: bool = False, rank: int = 0, world: int = 1):
    """The mixed-length batch (4096 lengths in [16, 65536], 7-smooth / prime / other, seed 2):
    one persistent launch (CUDA graph) against one launch sequence per transform.  With N > 1
    ranks each runs its cost-balanced contiguous shard of the 4096 (fyg_partition)."""
    import torch
    import fyfft_gb300 as fg
    from fyfft_gb300.workloads import uneven_lengths
    lengths = uneven_lengths(4096, 2)
    bounds = fg.partition(lengths, world)
    first = int(sum(lengths[:bounds[rank]]))
    lengths = lengths[bounds[rank]:bounds[rank + 1]]
    t0 = time.perf_counter()
    tuned = None
    if not no_autotune:
        # execution forms and option sets timed on this device, cached (FYG_AUTOTUNE_CACHE);
        # skipped when the cache already holds this length sequence for this device
        cache = os.environ.get("FYG_AUTOTUNE_CACHE")
        have = False
        if cache and os.path.exists(cache):
            with open(cache) as f:
                doc = json.load(f)
            have = doc.get("device") == fg.device_signature() and any(
                k.startswith(f"batch32:{len(lengths)}:") for k in doc.get("entries", {}))
        if not have:
            fg.autotune_batch(lengths, cache_path=cache)
        tuned = round(time.perf_counter() - t0, 2)
    t1 = time.perf_counter()
    b = fg.UnevenBatch(lengths, flags=0 if no_autotune else fg.FYG_FLAG_AUTOTUNED)
    create_s = time.perf_counter() - t1
    x = torch.from_numpy(fg.fill_random(2, sum(lengths), np.complex64, "uniform", first=first)).to(f"cuda:{dev}")
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
                form = {0: "persistent kernel", 1: "graph branches (one plan per length)",
                        2: f"persistent kernel up to length {ent[0]['conv_length']}, graph branches above"}
                res["autotuned"] = {"form": form.get(ent[0]["order"], "?"), "stage_radix_cap": ent[0]["max_pass_radix"],
                                    "single_tile_kb": ent[0]["cols"], "tuner_ms": ent[0]["ms"]}
    res["speedup"] = round(res["plain_ms"] / res["batched_ms"], 2)
    b.execute(x, y, stream=stream)
    torch.cuda.synchronize()
    return res, (lengths, x.cpu().numpy(), y.cpu().numpy())


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
# The reference's own C++ FFT on the host cores (CPU baseline and the reference arm)
# ----------------------------------------------------------------------------------------------

def cpu_model() -> str:
    try:
        for line in open("/proc/cpuinfo"):
            if line.lower().startswith(("model name", "cpu model")):
                return line.split(":", 1)[1].strip()
    except OSError:
        pass
    return os.uname().machine


def reference_handle():
    """(oracle.Reference, None) when oracle/_ref/libfyref.so was built, else (None, why)."""
    from oracle import oracle as O
    if not O.Reference.available():
        return None, ("oracle/_ref/libfyref.so was not built: the reference's sources were not staged "
                      "(oracle/ref/build_ref.sh needs the reference checkout once)")
    return O.Reference(), None


def reference_steps(items, steps: int, warmup: int, budget_s: float = 150.0, threads: int | None = None):
    """Times the reference's FFT1D_C2C_invoker over every item it can run, the whole batch per
    step, one plan per host thread (oracle/ref/ref_capi.cpp pools).  Inputs come from the
    oracle's restatement of the seeded generator, never from the GPU library.  Returns a dict
    with the GFLOP/s, the timing details and the outputs of the last step."""
    from oracle import oracle as O
    ref, why = reference_handle()
    if ref is None:
        return {"unavailable": why}
    threads = threads or os.cpu_count() or 1
    run, unsupported, pools, bufs = [], {}, [], []
    plan_s = 0.0
    for (n, batch, dt, dist, seed) in items:
        if not ref.runnable(n):
            unsupported[str(n)] = ("the reference falls back to its O(N^2) DFT (src/foye_FFT_dft.hpp), whose "
                                   f"16 N^2-byte tables ({16 * n * n / 1e9:.0f} GB) cannot be allocated")
            continue
        x = O.fill_random(seed, n * batch, np.complex64, dist).reshape(batch, n)
        y = np.empty_like(x)
        pool = O.ReferencePool(ref, n, min(threads, batch))
        plan_s += pool.plan_seconds
        run.append((n, batch))
        pools.append(pool)
        bufs.append((x, y))
    if not run:
        return {"unavailable": "the reference can run none of this workload's lengths"}

    def step():
        return [pool.run(x, y) for pool, (x, y) in zip(pools, bufs)]
    t = time.perf_counter()
    step()
    one = time.perf_counter() - t
    steps = max(1, min(steps, int(budget_s / max(one, 1e-3))))
    warm = max(0, min(warmup - 1, int(budget_s / max(one, 1e-3)) - steps))
    for _ in range(warm):
        step()
    per = np.zeros(len(run))
    t = time.perf_counter()
    for _ in range(steps):
        per += np.array(step())
    el = time.perf_counter() - t
    step_flops = sum(flops(n) * b for n, b in run)
    for pool in pools:
        pool.close()
    return {"value": step_flops / (el / steps) / 1e9, "steps": steps, "warmup": warm + 1, "seconds": el,
            "ms_per_step": el / steps * 1e3, "threads": threads, "run": run, "unsupported": unsupported,
            "plan_s": plan_s, "build": ref.build_info(), "cpu": cpu_model(),
            "per_size_gflops": {str(n): round(flops(n) * b * steps / per[i] / 1e9, 2) for i, (n, b) in enumerate(run)},
            "outputs": {n: y for (n, _), (_, y) in zip(run, bufs)}}


def reference_kind(build: str) -> str:
    return ("reference's AVX2 C++ (FFT1D_C2C_invoker), native AVX2 build" if build.startswith("native")
            else f"reference's AVX2 C++ (FFT1D_C2C_invoker), emulated on {cpu_model()} "
                 f"(oracle/ref/portable_intrin.h, bit-identical to the native build on x86-64)")


def cpu_baseline(items, args, check=None, uneven=None):
    """The reference's own code on this host's cores (kind "reference"), a bounded run of the
    same workload; where the GPU outputs are passed, their rel-L2 against the reference's
    outputs and against the FP64 oracle (the checker)."""
    from oracle import oracle as O
    r = reference_steps(items, steps=3, warmup=1, budget_s=30.0)
    if "unavailable" in r:
        res = {"value": None, "unit": "GFLOP/s", "cores": os.cpu_count() or 1, "kind": "reference",
               "unavailable": r["unavailable"]}
    else:
        res = {"value": round(r["value"], 3), "unit": "GFLOP/s", "cores": r["threads"], "kind": "reference",
               "build": reference_kind(r["build"]),
               "sample": (f"{r['steps']} step(s) of the whole batch of every length the reference runs "
                          f"({', '.join(f'{b}x{n}' for n, b in r['run'])}), one plan per thread; "
                          f"unsupported: {', '.join(r['unsupported']) or 'none'}"),
               "seconds": round(r["seconds"], 2), "plan_s": round(r["plan_s"], 2),
               "per_size_gflops": r["per_size_gflops"], "machine": os.uname().machine, "cpu": r["cpu"]}
        # the same code on one thread (the reference itself is single-threaded; the value above
        # spreads the batch over every core, one plan per thread)
        r1 = reference_steps(items, steps=1, warmup=1, budget_s=15.0, threads=1)
        if "unavailable" not in r1:
            res["single_thread"] = {"value": round(r1["value"], 3), "unit": "GFLOP/s", "cores": 1,
                                    "steps": r1["steps"], "seconds": round(r1["seconds"], 2)}
    if check is not None:
        plans, youts = check
        vs_ref, vs_oracle, max_abs = {}, {}, {}
        threads = os.cpu_count() or 1
        for (n, batch, dt, dist, seed), y in zip(items, youts):
            g = y.view(batch, n)
            rows = [0, batch - 1] if batch > 1 else [0]
            gr = g[rows].cpu().numpy()
            x = O.fill_random(seed, n * batch, np.complex128 if dt == "complex128" else np.complex64,
                              dist).reshape(batch, n)
            ref = O.fft_batch(x[rows].astype(np.complex128), threads=threads)
            vs_oracle[str(n)] = float(f"{O.rel_l2(gr, ref):.3e}")
            max_abs[str(n)] = float(f"{np.max(np.abs(gr.astype(np.complex128) - ref)):.3e}")
            if "outputs" in r and n in r["outputs"]:
                vs_ref[str(n)] = float(f"{O.rel_l2(g.cpu().numpy(), r['outputs'][n]):.3e}")
        res["gpu_rel_l2_vs_reference"] = vs_ref
        res["gpu_rel_l2_vs_fp64_oracle"] = vs_oracle
        res["gpu_max_abs_vs_fp64_oracle"] = max_abs
        res["rel_l2_rows"] = ("vs reference: whole batch; vs FP64 oracle (rel-L2 and max abs): first and last "
                              "transform")
    if uneven is not None:
        import concurrent.futures as cf
        lengths, xh, yh = uneven
        offs = np.concatenate([[0], np.cumsum(lengths)])

        def err(i):
            a, b = offs[i], offs[i + 1]
            return O.rel_l2(yh[a:b], O.fft(xh[a:b]))
        with cf.ThreadPoolExecutor(os.cpu_count() or 4) as ex:
            errs = list(ex.map(err, range(len(lengths))))
        res["mixed_batch_rel_l2_vs_fp64_oracle"] = {"max": float(f"{max(errs):.3e}"),
                                                    "median": float(f"{statistics.median(errs):.3e}"),
                                                    "transforms": len(errs)}
    return res


def run_reference(args, rank: int, world: int):
    """--impl reference: the reference's own FFT on the host cores, rank 0 only."""
    items, desc = workload(args.workload, args.sizes, args.batch)
    if rank != 0:
        return None
    r = reference_steps(items, args.steps, args.warmup)
    if "unavailable" in r:
        return {"impl": "reference", "unavailable": r["unavailable"]}
    value = round(r["value"], 3)
    sample = ", ".join(f"{b}x{n}" for n, b in r["run"])
    return {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "GFLOP/s", "n_gpus": world,
        "steps": r["steps"], "warmup": r["warmup"], "ms_per_step": round(r["ms_per_step"], 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded counter-based generator, oracle restatement)",
        "config": {"workload": desc, "sizes": [it[0] for it in items], "batch": [it[1] for it in items],
                   "reference_runs": sample, "reference_unsupported": r["unsupported"],
                   "value_over": "the lengths the reference runs (unsupported lengths excluded)"},
        "cpu_baseline": {"value": value, "unit": "GFLOP/s", "cores": r["threads"], "kind": "reference",
                         "build": reference_kind(r["build"]), "cpu": r["cpu"],
                         "sample": f"per step the whole batch: {sample}; one plan per thread",
                         "plan_s": round(r["plan_s"], 2), "per_size_gflops": r["per_size_gflops"]},
        "e2e": {"value": value, "unit": "GFLOP/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
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
    ap.add_argument("--no-configs", action="store_true", help="skip the C1 / C4 / C5 configuration lines")
    ap.add_argument("--plan-flags", type=int, default=0,
                    help="extra FYG_FLAG_* bits for the sweep's plans (comparisons, e.g. 256 = no TMA loads)")
    ap.add_argument("--retune", action="store_true", help="ignore the committed schedule choices and tune anew")
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
