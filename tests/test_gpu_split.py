"""N = m p split (p prime, p - 1 13-smooth, m <= 8): a pass of length-m DFTs and twiddles, then m
Rader transforms of length p whose scatter store interleaves them.  Every form of execution
(forward, inverse, adjoint, FP64, strided and in-place layouts, host buffers, uneven batches)
against the FP64 oracle, and against the Bluestein plan of the same length."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

import fyfft_gb300 as fg  # noqa: E402
from oracle import oracle as O  # noqa: E402

pytestmark = pytest.mark.gpu

SENTINEL = np.complex64(123.0 - 45.0j)
EPS64 = float(np.finfo(np.float64).eps)

# (N, m, p): register-resident Rader passes (65537), single-pass Rader tiles (12289, 7681, 3457),
# every m from 2 to 8
CASES = [(131074, 2, 65537), (196611, 3, 65537), (24578, 2, 12289), (73734, 6, 12289), (98312, 8, 12289),
         (53767, 7, 7681), (17285, 5, 3457), (13828, 4, 3457)]


def kernels(p):
    return [ln.split("kernel=")[1].split()[0] for ln in p.describe()]


def run(n, batch, inverse=False, dtype="complex64", seed=41, **kw):
    npdt = np.complex64 if dtype == "complex64" else np.complex128
    x = fg.fill_random(seed, n * batch, npdt, "normal")
    t = torch.from_numpy(x).cuda()
    y = torch.empty_like(t)
    p = fg.FFT1D_C2C_invoker(n, dtype, batch, **kw)
    p.dispatch(inverse, t, y)
    torch.cuda.synchronize()
    return p, x.reshape(batch, n), y.cpu().numpy().reshape(batch, n)


@pytest.mark.parametrize("n,m,prime", CASES)
@pytest.mark.parametrize("inverse", [False, True])
def test_split_matches_oracle(n, m, prime, inverse):
    batch = 3
    p, x, y = run(n, batch, inverse)
    info = p.info()
    assert info["gpu_strategy"] == 5 and info["conv_length"] == prime - 1, (info, p.describe())
    ks = kernels(p)
    assert ks[0] == "split" and f"R={m} " in p.describe()[0]
    assert "gather" in p.describe()[1] and "scatter" in p.describe()[-1]
    assert fg.FFT1D_C2C_invoker.gpu_execution_strategy(n) == fg.FFT_execution_strategy.rader
    for b in range(batch):
        assert O.rel_l2(y[b], O.fft(x[b], inverse=inverse)) <= 2e-6, (n, b)


@pytest.mark.parametrize("n", [131074, 73734])
def test_split_agrees_with_bluestein_plan(n):
    _, x, ys = run(n, 2)
    L = 1
    while L < 2 * n - 1:
        L *= 2
    pb, _, yb = run(n, 2, conv_length=L)
    assert pb.info()["gpu_strategy"] == 3
    for b in range(2):
        assert O.rel_l2(ys[b], yb[b]) <= 2e-6


@pytest.mark.parametrize("n", [131074, 24578])
def test_split_fp64(n):
    for inverse in (False, True):
        _, x, y = run(n, 2, inverse, dtype="complex128")
        for b in range(2):
            assert O.rel_l2(y[b], O.fft(x[b], inverse=inverse)) <= 4 * np.log2(n) * EPS64


def test_split_round_trip_and_adjoint():
    n, batch = 131074, 2
    x = fg.fill_random(43, n * batch, np.complex64, "normal")
    t = torch.from_numpy(x).cuda()
    y, back, adj = torch.empty_like(t), torch.empty_like(t), torch.empty_like(t)
    p = fg.FFT1D_C2C_invoker(n, "complex64", batch)
    p.dispatch(False, t, y)
    p.dispatch(True, y, back)
    p.adjoint(t, adj)
    torch.cuda.synchronize()
    assert O.rel_l2(back.cpu().numpy(), x) <= 2e-6
    xr = x.reshape(batch, n)
    # F^H g = N * IFFT(g)
    assert O.rel_l2(adj.cpu().numpy().reshape(batch, n)[1], n * O.fft(xr[1], inverse=True)) <= 2e-6


def test_split_in_place():
    n, batch = 73734, 3
    x = fg.fill_random(44, n * batch, np.complex64, "normal")
    t = torch.from_numpy(x.copy()).cuda()
    p = fg.FFT1D_C2C_invoker(n, "complex64", batch)
    p.dispatch(False, t, t)
    torch.cuda.synchronize()
    y = t.cpu().numpy().reshape(batch, n)
    for b in range(batch):
        assert O.rel_l2(y[b], O.fft(x.reshape(batch, n)[b])) <= 2e-6


@pytest.mark.parametrize("where", ["device", "host"])
def test_split_strided_layout(where):
    n, batch, idist, odist = 131074, 3, 131074 + 37, 131074 + 101
    x = fg.fill_random(45, n * batch, np.complex64, "normal").reshape(batch, n)
    xin = np.full((batch - 1) * idist + n, SENTINEL, dtype=np.complex64)
    for b in range(batch):
        xin[b * idist:b * idist + n] = x[b]
    yout = np.full((batch - 1) * odist + n, SENTINEL, dtype=np.complex64)
    p = fg.FFT1D_C2C_invoker(n, "complex64", batch, idist=idist, odist=odist)
    if where == "device":
        yd = torch.from_numpy(yout).cuda()
        p.dispatch(False, torch.from_numpy(xin).cuda(), yd)
        torch.cuda.synchronize()
        yout = yd.cpu().numpy()
    else:
        p.dispatch(False, xin, yout)
    mask = np.ones(yout.size, dtype=bool)
    for b in range(batch):
        mask[b * odist:b * odist + n] = False
        assert O.rel_l2(yout[b * odist:b * odist + n], O.fft(x[b])) <= 2e-6
    assert np.all(yout[mask] == SENTINEL)


def test_split_host_buffers_overlapped_staging():
    """8 MB and more of host buffers: chunked copies overlapping the split pass and Rader passes."""
    n, batch = 131074, 16
    x = fg.fill_random(46, n * batch, np.complex64, "normal")
    y = np.empty_like(x)
    p = fg.FFT1D_C2C_invoker(n, "complex64", batch)
    p.dispatch(False, x, y)
    yd = torch.empty(n * batch, dtype=torch.complex64, device="cuda")
    p.dispatch(False, torch.from_numpy(x).cuda(), yd)
    torch.cuda.synchronize()
    assert np.array_equal(y, yd.cpu().numpy())
    xr, yr = x.reshape(batch, n), y.reshape(batch, n)
    for b in (0, batch - 1):
        assert O.rel_l2(yr[b], O.fft(xr[b])) <= 2e-6


def test_split_lengths_in_uneven_batch():
    """Split lengths in an uneven batch: graph branches (offset tables) and the persistent kernel
    (which runs them as Bluestein convolutions)."""
    lengths = [131074, 3000, 24578, 131074, 4096, 73734, 24578, 1009]
    x = fg.fill_random(47, sum(lengths), np.complex64, "normal")
    xd = torch.from_numpy(x).cuda()
    for kw in ({"flags": fg.FYG_FLAG_BATCH_BRANCHES}, {}):
        b = fg.UnevenBatch(lengths, **kw)
        y = torch.empty_like(xd)
        for inverse in (False, True):
            b.execute(xd, y, invert=inverse)
            assert b.status() == 0
            yh = y.cpu().numpy()
            o = 0
            for n in lengths:
                assert O.rel_l2(yh[o:o + n], O.fft(x[o:o + n], inverse=inverse)) <= 2e-6, (n, kw, inverse)
                o += n
