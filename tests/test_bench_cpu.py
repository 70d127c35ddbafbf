"""bench.py on the CPU (no GPU involved).  The reference arm: the reference's own FFT over the
lengths it runs, one JSON line with the keys of the benchmark contract, lengths it cannot run
listed with the reason, and ranks above 0 printing nothing.  The CPU-baseline report: rel-L2 and
max-abs errors of given outputs against the reference and the FP64 oracle."""
import json
import os
import subprocess
import sys

import numpy as np
import pytest

from oracle import oracle as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

pytestmark = pytest.mark.skipif(not O.Reference.available(), reason="oracle/_ref not built")


def run_bench(*args, env=None):
    e = dict(os.environ)
    e.update(env or {})
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), *args], capture_output=True, text=True,
                       cwd=ROOT, env=e, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    return [json.loads(ln) for ln in r.stdout.splitlines() if ln.startswith("{")]


def test_reference_arm_prints_the_contract_line():
    lines = run_bench("--impl", "reference", "--steps", "3", "--warmup", "3", "--sizes", "2520,1009,65537")
    assert len(lines) == 1
    d = lines[0]
    assert d["impl"] == "reference" and d["unit"] == "GFLOP/s" and d["higher_is_better"] is True
    assert d["value"] > 0 and d["steps"] >= 1 and d["warmup"] >= 1 and d["n_gpus"] == 1
    assert d["config"]["sizes"] == [2520, 1009, 65537] and d["config"]["batch"] == [64, 64, 64]
    # 65537 is a DFT length for the reference (its N^2 tables cannot be allocated)
    assert list(d["config"]["reference_unsupported"]) == ["65537"]
    cb = d["cpu_baseline"]
    assert cb["kind"] == "reference" and cb["cores"] >= 1 and cb["value"] == d["value"]
    assert set(cb["per_size_gflops"]) == {"2520", "1009"}
    assert d["e2e"] == {"value": d["value"], "unit": "GFLOP/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}


def test_reference_arm_runs_on_rank_zero_only():
    assert run_bench("--impl", "reference", "--steps", "3", "--warmup", "3", "--sizes", "2520",
                     env={"RANK": "1", "WORLD_SIZE": "2"}) == []


def test_reference_arm_reports_a_workload_it_cannot_run():
    lines = run_bench("--impl", "reference", "--steps", "3", "--warmup", "3", "--sizes", "65537")
    assert lines == [{"impl": "reference", "unavailable": "the reference can run none of this workload's lengths"}]


def test_cpu_baseline_reports_errors_against_reference_and_oracle():
    """The benchmark's error report on outputs held in CPU tensors: here the oracle's own FP64
    results rounded to complex<float>, so every error is at FP32 rounding level."""
    torch = pytest.importorskip("torch")
    sys.path.insert(0, ROOT)
    import bench
    items = [(2520, 4, "complex64", "normal", 1), (1009, 3, "complex64", "normal", 1),
             (65537, 2, "complex64", "normal", 1)]
    youts = []
    for n, b, _, dist, seed in items:
        x = O.fill_random(seed, n * b, np.complex64, dist).reshape(b, n)
        youts.append(torch.from_numpy(O.fft_batch(x.astype(np.complex128)).astype(np.complex64).reshape(-1)))
    res = bench.cpu_baseline(items, None, check=(None, youts))
    assert res["kind"] == "reference" and res["value"] > 0 and res["machine"]
    assert res["single_thread"]["cores"] == 1 and res["single_thread"]["value"] > 0
    assert set(res["gpu_rel_l2_vs_fp64_oracle"]) == {"2520", "1009", "65537"}
    assert set(res["gpu_rel_l2_vs_reference"]) == {"2520", "1009"}          # 65537: not runnable there
    for n, e in res["gpu_rel_l2_vs_fp64_oracle"].items():
        assert e <= 1e-7, (n, e)
        assert 0 < res["gpu_max_abs_vs_fp64_oracle"][n] <= 1e-4 * np.sqrt(int(n)), n
    for n, e in res["gpu_rel_l2_vs_reference"].items():
        assert e <= 4 * np.log2(int(n)) * float(np.finfo(np.float32).eps), (n, e)
