"""Autotuned schedules: the measured choice is cached per device, reused by FYG_FLAG_AUTOTUNED
plans, and every candidate the tuner may pick stays within the precision bound."""
import json
import os

import numpy as np
import pytest

torch = pytest.importorskip("torch")

import fyfft_gb300 as fg  # noqa: E402
from oracle import oracle as O  # noqa: E402

pytestmark = pytest.mark.gpu

# single-pass (cols), multi-pass (pass-radix cap), Rader with N-1 smooth, Rader padded,
# Bluestein (convolution length)
LENGTHS = [4096, 2520, 1 << 20, 1009, 65537, 999983, 131074]


def run(n, batch, flags=0, inverse=False, seed=3, **kw):
    x = fg.fill_random(seed, n * batch, np.complex64, "normal")
    t = torch.from_numpy(x).cuda()
    y = torch.empty_like(t)
    fg.FFT1D_C2C_invoker(n, "complex64", batch, flags=flags, **kw).dispatch(inverse, t, y)
    torch.cuda.synchronize()
    return x.reshape(batch, n), y.cpu().numpy().reshape(batch, n)


@pytest.fixture(scope="module")
def cache(tmp_path_factory):
    path = str(tmp_path_factory.mktemp("tune") / "autotune.json")
    for n in LENGTHS:
        ms = fg.autotune(n, "complex64", 16 if n < 500000 else 4, cache_path=path)
        assert ms > 0
    return path


def test_cache_file_lists_every_length(cache):
    doc = json.load(open(cache))
    assert doc["device"] and torch.cuda.get_device_name(0) in doc["device"]
    for n in LENGTHS:
        e = doc["entries"][f"c32:{n}"]
        assert e["ms"] > 0 and set(e) == {"max_pass_radix", "conv_length", "cols", "order", "threads", "wide", "ms"}
        assert e["threads"] in (0, 1) and e["wide"] in (0, 1)


@pytest.mark.parametrize("n", LENGTHS)
def test_autotuned_plan_matches_oracle(cache, n):
    batch = 8 if n < 500000 else 2
    x, y = run(n, batch, flags=fg.FYG_FLAG_AUTOTUNED)
    for b in range(batch):
        assert O.rel_l2(y[b], O.fft(x[b])) <= 2e-6
    _, yi = run(n, batch, flags=fg.FYG_FLAG_AUTOTUNED, inverse=True)
    xi = fg.fill_random(3, n * batch, np.complex64, "normal").reshape(batch, n)
    assert O.rel_l2(yi[0], O.fft(xi[0], inverse=True)) <= 2e-6


def test_autotuned_convolution_length_is_used(cache):
    doc = json.load(open(cache))
    for n in (999983, 131074, 65537):
        m = doc["entries"][f"c32:{n}"]["conv_length"]
        tuned = fg.FFT1D_C2C_invoker(n, "complex64", 1, flags=fg.FYG_FLAG_AUTOTUNED).info()["conv_length"]
        default = fg.FFT1D_C2C_invoker(n, "complex64", 1).info()["conv_length"]
        assert tuned == (m if m else default)
        # Rader of N, Rader of p for the split N = 2 p (131074 = 2 x 65537), or Bluestein
        assert tuned in (n - 1, n // 2 - 1) or tuned >= 2 * n - 3


@pytest.mark.parametrize("n,m", [(999983, 2000000), (999983, 2016000), (131074, 263424), (65537, 131220)])
def test_every_convolution_candidate_is_accurate(n, m):
    x, y = run(n, 2, conv_length=m)
    assert O.rel_l2(y[1], O.fft(x[1])) <= 2e-6


@pytest.mark.parametrize("r", [128, 256, 512])
def test_pass_radix_caps_are_accurate(r):
    n = 1 << 20
    x, y = run(n, 2, max_pass_radix=r)
    assert O.rel_l2(y[0], O.fft(x[0])) <= 2e-6


def test_cache_for_another_device_is_ignored(tmp_path):
    path = str(tmp_path / "other.json")
    with open(path, "w") as f:
        f.write('{\n  "device": "some other GPU|1|1.0|1",\n  "entries": {\n'
                '    "c32:1009": {"max_pass_radix": 0, "conv_length": 5000, "cols": 0, "order": 0, "threads": 0, '
                '"wide": 0, "ms": 1.0}\n  }\n}\n')
    # tuning another length into that file replaces the foreign entries
    fg.autotune(2520, "complex64", 4, cache_path=path)
    doc = json.load(open(path))
    assert "c32:1009" not in doc["entries"] and "c32:2520" in doc["entries"]
    assert os.path.getsize(path) > 0
