"""The process-wide table cache: a second plan of the same length reuses every read-only table
(no new entries, only hits), computes bit-identical results, and fyg_plan_cache_clear frees
what no live plan holds while the tables of live plans stay valid."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

import fyfft_gb300 as fg  # noqa: E402
from oracle import oracle as O  # noqa: E402

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n", [999983, 65537, 1 << 20, 2520, 1009])
def test_second_plan_hits_the_cache(n):
    batch = 3
    x = torch.from_numpy(fg.fill_random(5, n * batch, np.complex64, "normal")).cuda()
    a = fg.FFT1D_C2C_invoker(n, "complex64", batch)
    s1 = fg.plan_cache_stats()
    b = fg.FFT1D_C2C_invoker(n, "complex64", batch + 1)
    s2 = fg.plan_cache_stats()
    assert s2["entries"] == s1["entries"]
    assert s2["misses"] == s1["misses"]
    assert s2["hits"] > s1["hits"]
    ya, yb = torch.empty_like(x), torch.empty(n * (batch + 1), dtype=torch.complex64, device="cuda")
    a.dispatch(False, x, ya)
    b.dispatch(False, torch.cat([x, x[:n]]), yb)
    torch.cuda.synchronize()
    assert torch.equal(ya, yb[: n * batch])
    ref = O.fft(x.cpu().numpy().reshape(batch, n)[:1])
    assert O.rel_l2(ya.cpu().numpy()[:n], ref[0]) <= 2e-6


def test_clear_keeps_live_plans_valid():
    n, batch = 131074, 2
    x = torch.from_numpy(fg.fill_random(6, n * batch, np.complex64, "normal")).cuda()
    keep = fg.FFT1D_C2C_invoker(n, "complex64", batch)
    tmp = fg.FFT1D_C2C_invoker(40009, "complex64", batch)
    tmp.close()
    before = fg.plan_cache_stats()
    fg.plan_cache_clear()
    after = fg.plan_cache_stats()
    assert after["entries"] < before["entries"]
    y = torch.empty_like(x)
    keep.dispatch(False, x, y)
    torch.cuda.synchronize()
    ref = O.fft(x.cpu().numpy().reshape(batch, n))
    assert O.rel_l2(y.cpu().numpy().reshape(batch, n), ref) <= 2e-6
