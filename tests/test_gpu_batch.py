"""Uneven-length batch: one persistent launch over a device work queue (CUDA graph) against the
FP64 oracle, the one-plan-per-launch path, custom offsets, and the bounded dependency wait."""
import time

import numpy as np
import pytest

torch = pytest.importorskip("torch")

import fyfft_gb300 as fg  # noqa: E402
from fyfft_gb300.workloads import uneven_lengths  # noqa: E402
from oracle import oracle as O  # noqa: E402

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def batch():
    lengths = uneven_lengths(count=192, seed=2)
    b = fg.UnevenBatch(lengths)
    x = fg.fill_random(2, sum(lengths), np.complex64, "uniform")
    return lengths, b, x


def split(v, lengths):
    out, o = [], 0
    for n in lengths:
        out.append(v[o:o + n])
        o += n
    return out


@pytest.mark.parametrize("inverse", [False, True])
def test_persistent_batch_matches_oracle_and_plain_path(batch, inverse):
    lengths, b, x = batch
    xd = torch.from_numpy(x).cuda()
    y = torch.empty_like(xd)
    b.execute(xd, y, invert=inverse)
    assert b.status() == 0
    y2 = torch.empty_like(xd)
    b.execute_plain(xd, y2, invert=inverse)
    torch.cuda.synchronize()
    ys, y2s = split(y.cpu().numpy(), lengths), split(y2.cpu().numpy(), lengths)
    for n, xi, yi, y2i in zip(lengths, split(x, lengths), ys, y2s):
        ref = O.fft(xi, inverse=inverse)
        assert O.rel_l2(yi, ref) <= 2e-6, n
        assert O.rel_l2(yi, y2i) <= 2e-6, n


def test_graph_replay_is_repeatable(batch):
    lengths, b, x = batch
    xd = torch.from_numpy(x).cuda()
    y1, y2 = torch.empty_like(xd), torch.empty_like(xd)
    b.execute(xd, y1)
    b.execute(xd, y2)
    assert b.status() == 0
    assert torch.equal(y1, y2)


def test_custom_offsets(batch):
    lengths, b, x = batch
    # pack the transforms in reverse order
    offs, o = [0] * len(lengths), 0
    for i in reversed(range(len(lengths))):
        offs[i] = o
        o += lengths[i]
    xr = np.empty_like(x)
    for i, xi in enumerate(split(x, lengths)):
        xr[offs[i]:offs[i] + lengths[i]] = xi
    xd = torch.from_numpy(xr).cuda()
    y = torch.empty_like(xd)
    off_d = torch.tensor(offs, dtype=torch.int64, device="cuda")
    b.execute(xd, y, offsets_dev=off_d)
    assert b.status() == 0
    yh = y.cpu().numpy()
    for i, xi in enumerate(split(x, lengths)):
        assert O.rel_l2(yh[offs[i]:offs[i] + lengths[i]], O.fft(xi)) <= 2e-6


def test_stalled_dependency_times_out_and_context_recovers(batch):
    lengths, b, x = batch
    xd = torch.from_numpy(x).cuda()
    y = torch.empty_like(xd)
    b.inject_stall(True, timeout_ms=200)
    t0 = time.time()
    b.execute(xd, y)
    assert b.status() == 6          # FYG_ERR_TIMEOUT
    assert time.time() - t0 < 10
    b.inject_stall(False)
    b.execute(xd, y)
    assert b.status() == 0
    ys = split(y.cpu().numpy(), lengths)
    for n, xi, yi in zip(lengths[:32], split(x, lengths), ys):
        assert O.rel_l2(yi, O.fft(xi)) <= 2e-6, n


def test_batch_autotune_caches_a_choice_and_the_tuned_batch_is_exact(tmp_path):
    import json
    lengths = uneven_lengths(count=160, seed=7)
    path = str(tmp_path / "batch_tune.json")
    ms = fg.autotune_batch(lengths, cache_path=path)
    assert ms > 0
    doc = json.load(open(path))
    keys = [k for k in doc["entries"] if k.startswith("batch32:160:")]
    assert len(keys) == 1
    e = doc["entries"][keys[0]]
    # form 0: persistent kernel (stage radix cap, single-pass tile KB); 1: branches; 2: both,
    # split at the length in conv_length
    assert e["order"] in (0, 1, 2)
    if e["order"] != 1:
        assert e["max_pass_radix"] in (16, 32) and e["cols"] in (48, 100, 160)
    if e["order"] == 2:
        assert e["conv_length"] in (4096, 16384)
    b = fg.UnevenBatch(lengths, flags=fg.FYG_FLAG_AUTOTUNED)
    x = fg.fill_random(8, sum(lengths), np.complex64, "uniform")
    xd = torch.from_numpy(x).cuda()
    y = torch.empty_like(xd)
    b.execute(xd, y)
    assert b.status() == 0
    torch.cuda.synchronize()
    for n, xi, yi in zip(lengths, split(x, lengths), split(y.cpu().numpy(), lengths)):
        assert O.rel_l2(yi, O.fft(xi)) <= 2e-6, n


def test_full_mixed_length_configuration_vs_oracle():
    """The benchmark's own batch: all 4096 lengths (seed 2, 0.70 7-smooth / 0.15 prime / 0.15
    other) in one persistent launch, every transform within 2e-6 (and 4 log2 N eps32) of the
    FP64 oracle."""
    import concurrent.futures as cf
    import os
    lengths = uneven_lengths(4096, 2)
    b = fg.UnevenBatch(lengths)
    x = fg.fill_random(2, sum(lengths), np.complex64, "uniform")
    xd = torch.from_numpy(x).cuda()
    y = torch.empty_like(xd)
    b.execute(xd, y)
    assert b.status() == 0
    ys = split(y.cpu().numpy(), lengths)
    xs = split(x, lengths)

    def err(i):
        return O.rel_l2(ys[i], O.fft(xs[i]))
    with cf.ThreadPoolExecutor(os.cpu_count() or 4) as ex:
        errs = list(ex.map(err, range(len(lengths))))
    worst = max(range(len(lengths)), key=lambda i: errs[i])
    assert errs[worst] <= 2e-6, (lengths[worst], errs[worst])
    assert all(e <= 4 * np.log2(n) * float(np.finfo(np.float32).eps) for e, n in zip(errs, lengths))


@pytest.mark.parametrize("inverse", [False, True])
def test_branch_form_matches_persistent_form_and_oracle(batch, inverse):
    """FYG_FLAG_BATCH_BRANCHES: one plan per distinct length as parallel chains of one graph."""
    lengths, b, x = batch
    bb = fg.UnevenBatch(lengths, flags=fg.FYG_FLAG_BATCH_BRANCHES)
    xd = torch.from_numpy(x).cuda()
    y, yp = torch.empty_like(xd), torch.empty_like(xd)
    bb.execute(xd, y, invert=inverse)
    bb.execute(xd, y, invert=inverse)     # graph replay
    assert bb.status() == 0
    b.execute(xd, yp, invert=inverse)
    torch.cuda.synchronize()
    for n, xi, yi, ypi in zip(lengths, split(x, lengths), split(y.cpu().numpy(), lengths), split(yp.cpu().numpy(), lengths)):
        assert O.rel_l2(yi, O.fft(xi, inverse=inverse)) <= 2e-6, n
        assert O.rel_l2(yi, ypi) <= 2e-6, n


def test_branch_form_custom_offsets(batch):
    lengths, _, x = batch
    bb = fg.UnevenBatch(lengths, flags=fg.FYG_FLAG_BATCH_BRANCHES)
    offs, o = [0] * len(lengths), 0
    for i in reversed(range(len(lengths))):
        offs[i] = o
        o += lengths[i]
    xr = np.empty_like(x)
    for i, xi in enumerate(split(x, lengths)):
        xr[offs[i]:offs[i] + lengths[i]] = xi
    xd = torch.from_numpy(xr).cuda()
    y = torch.empty_like(xd)
    bb.execute(xd, y, offsets_dev=torch.tensor(offs, dtype=torch.int64, device="cuda"))
    assert bb.status() == 0
    yh = y.cpu().numpy()
    for i, xi in enumerate(split(x, lengths)):
        assert O.rel_l2(yh[offs[i]:offs[i] + lengths[i]], O.fft(xi)) <= 2e-6


@pytest.mark.parametrize("split", [4096, 16384])
def test_hybrid_form_matches_oracle(split):
    """Lengths up to `split` in the persistent kernel, longer ones as graph branches, concurrently."""
    lengths = uneven_lengths(count=200, seed=9)
    b = fg.UnevenBatch(lengths, form=2, split=split, radix_cap=16, single_tile_kb=100)
    x = fg.fill_random(10, sum(lengths), np.complex64, "uniform")
    xd = torch.from_numpy(x).cuda()
    y = torch.empty_like(xd)
    for inverse in (False, True):
        b.execute(xd, y, invert=inverse)
        assert b.status() == 0
        torch.cuda.synchronize()
        for n, xi, yi in zip(lengths, split_(x, lengths), split_(y.cpu().numpy(), lengths)):
            assert O.rel_l2(yi, O.fft(xi, inverse=inverse)) <= 2e-6, (n, inverse)


split_ = split
