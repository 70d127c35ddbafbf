"""bench.py's reference arm on the CPU (no GPU involved): the reference's own FFT over the lengths
it runs, one JSON line with the keys of the benchmark contract, lengths it cannot run listed
with the reason, and ranks above 0 printing nothing."""
import json
import os
import subprocess
import sys

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
