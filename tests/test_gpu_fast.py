"""Register-resident power-of-two pass kernels: every tile shape, every fusion they take
(inter-pass twiddle, Bluestein chirp load / store, convolution mid pass, Rader gather / DC
capture / scatter), both directions, against the FP64 oracle and against the generic kernel on
the same inputs."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

import fyfft_gb300 as fg  # noqa: E402
from oracle import oracle as O  # noqa: E402

pytestmark = pytest.mark.gpu

EPS32 = float(np.finfo(np.float32).eps)


def run(n, batch, inverse=False, flags=0, seed=5, **kw):
    x = fg.fill_random(seed, n * batch, np.complex64, "normal")
    t = torch.from_numpy(x).cuda()
    y = torch.empty_like(t)
    p = fg.FFT1D_C2C_invoker(n, "complex64", batch, flags=flags, **kw)
    p.dispatch(inverse, t, y)
    torch.cuda.synchronize()
    return p, x.reshape(batch, n), y.cpu().numpy().reshape(batch, n)


def kernels(p):
    return [ln.split("kernel=")[1].split()[0] for ln in p.describe()]


# tile lengths 256, 512, 1024 and 2048 (two and three passes; the planner schedules no 4096-point
# pass, whose generic-kernel tile does not fit shared memory)
@pytest.mark.parametrize("n,batch", [(1 << 16, 8), (1 << 18, 4), (1 << 20, 2), (1 << 21, 2), (1 << 22, 1),
                                     (1 << 24, 1), (512 * 2048, 2)])
@pytest.mark.parametrize("inverse", [False, True])
def test_power_of_two_passes(n, batch, inverse):
    p, x, y = run(n, batch, inverse)
    assert set(kernels(p)) == {"fast"}, p.describe()
    for b in (0, batch - 1):
        assert O.rel_l2(y[b], O.fft(x[b], inverse=inverse)) <= 4 * np.log2(n) * EPS32


@pytest.mark.parametrize("n", [1 << 16, 1 << 20])
def test_fast_equals_generic(n):
    _, _, yf = run(n, 4)
    pg, _, yg = run(n, 4, flags=fg.FYG_FLAG_GENERIC_KERNELS)
    assert set(kernels(pg)) == {"generic"}
    assert O.rel_l2(yf, yg) <= 2e-7


# 131078 = 2 x 65539 (65538 is not 13-smooth: no N = m p split)
@pytest.mark.parametrize("n", [40009, 131078, 999983])
@pytest.mark.parametrize("inverse", [False, True])
def test_bluestein_power_of_two_convolution(n, inverse):
    p, x, y = run(n, 2, inverse)
    L = p.info()["conv_length"]
    assert L & (L - 1) == 0 and L >= 2 * n - 1
    assert "fast" in kernels(p)
    for b in range(2):
        assert O.rel_l2(y[b], O.fft(x[b], inverse=inverse)) <= 2e-6


def test_rader_passes():
    n = 65537                      # prime, N-1 = 2^16: cyclic convolution over 256 x 256
    p, x, y = run(n, 3)
    ks = kernels(p)
    # gather load (x0 saved), mid pass (DC captured), scatter store: all register-resident
    assert ks == ["fast"] * 3 and "mid" in p.describe()[1] and "gather" in p.describe()[0], p.describe()
    for b in range(3):
        assert O.rel_l2(y[b], O.fft(x[b])) <= 2e-6
    _, xi, yi = run(n, 3, inverse=True)
    assert O.rel_l2(yi[2], O.fft(xi[2], inverse=True)) <= 2e-6


def test_round_trip_and_adjoint_on_fast_plan():
    n, batch = 1 << 20, 2
    x = fg.fill_random(9, n * batch, np.complex64, "normal")
    t = torch.from_numpy(x).cuda()
    y = torch.empty_like(t)
    z = torch.empty_like(t)
    p = fg.FFT1D_C2C_invoker(n, "complex64", batch)
    p.dispatch(False, t, y)
    p.dispatch(True, y, z)
    torch.cuda.synchronize()
    assert O.rel_l2(z.cpu().numpy(), x) <= 4e-7
    a = torch.empty_like(t)
    p.adjoint(t, a, scale=1.0)
    torch.cuda.synchronize()
    # adjoint of the unnormalized DFT = N * inverse
    ref = O.fft(x.reshape(batch, n)[1], inverse=True) * n
    assert O.rel_l2(a.cpu().numpy().reshape(batch, n)[1], ref) <= 4 * np.log2(n) * EPS32


# tile lengths 243 = 27 * 9 and 343 = 7 * 7 * 7 (columns per tile 27 and 7, not powers of two)
@pytest.mark.parametrize("n,batch,fast", [(59049, 8, 2), (117649, 4, 2), (16807, 16, 1), (177147, 2, 1)])
@pytest.mark.parametrize("inverse", [False, True])
def test_power_of_three_and_seven_passes(n, batch, fast, inverse):
    p, x, y = run(n, batch, inverse)
    assert kernels(p).count("fast") >= fast, p.describe()
    for b in (0, batch - 1):
        assert O.rel_l2(y[b], O.fft(x[b], inverse=inverse)) <= 4 * np.log2(n) * EPS32


@pytest.mark.parametrize("inverse", [False, True])
def test_bluestein_on_243_tiles(inverse):
    n = 29000                      # 2^3 5^3 29: Bluestein, convolution 59049 = 243 * 243
    p, x, y = run(n, 3, inverse, conv_length=59049)
    assert kernels(p) == ["fast"] * 3, p.describe()
    for b in range(3):
        assert O.rel_l2(y[b], O.fft(x[b], inverse=inverse)) <= 2e-6


# wide tiles (FYG_FLAG_WIDE_TILES): 512-thread CTAs with twice the columns, every fusion
@pytest.mark.parametrize("n,batch", [(1 << 16, 8), (1 << 18, 4), (1 << 20, 2), (1 << 21, 2), (65537, 3),
                                     (131074, 2), (999983, 2)])
@pytest.mark.parametrize("inverse", [False, True])
def test_wide_tiles(n, batch, inverse):
    p, x, y = run(n, batch, inverse, flags=fg.FYG_FLAG_WIDE_TILES)
    desc = p.describe()
    assert "fast" in kernels(p)
    # at least one pass runs a wide shape (C of 8 at 2048, 16 at 1024, 32 at 512 and 256)
    wide_c = {"2048": "8", "1024": "16", "512": "32", "256": "32"}
    assert any(f"R={r} C={c} " in ln for ln in desc for r, c in wide_c.items()), desc
    _, _, yn = run(n, batch, inverse)
    for b in (0, batch - 1):
        ref = O.fft(x[b], inverse=inverse)
        assert O.rel_l2(y[b], ref) <= 2e-6 and O.rel_l2(y[b], ref) <= 4 * np.log2(n) * EPS32
        assert O.rel_l2(y[b], yn[b]) <= 2e-7


# TMA tile loads (FYG_FLAG_TMA_LOADS): the same values arrive by tensor copies, so the outputs are
# identical to the per-thread-load path, and no bounded wait expired
@pytest.mark.parametrize("n,batch", [(1 << 16, 8), (1 << 20, 3), (1 << 21, 2), (65537, 3), (131074, 2),
                                     (999983, 2), (1 << 24, 1)])
@pytest.mark.parametrize("inverse", [False, True])
def test_tma_loads_match_per_thread_loads(n, batch, inverse):
    x = fg.fill_random(21, n * batch, np.complex64, "normal")
    t = torch.from_numpy(x).cuda()
    pt = fg.FFT1D_C2C_invoker(n, "complex64", batch, flags=fg.FYG_FLAG_TMA_LOADS)
    pn = fg.FFT1D_C2C_invoker(n, "complex64", batch, flags=fg.FYG_FLAG_NO_TMA_LOADS)
    yt, yn = torch.empty_like(t), torch.empty_like(t)
    pt.dispatch(inverse, t, yt)
    pn.dispatch(inverse, t, yn)
    torch.cuda.synchronize()
    assert pt.status() == 0
    assert torch.equal(yt, yn)
    # the default plan (TMA on 4-column tiles only) computes the same values too
    pd = fg.FFT1D_C2C_invoker(n, "complex64", batch)
    yd = torch.empty_like(t)
    pd.dispatch(inverse, t, yd)
    torch.cuda.synchronize()
    assert pd.status() == 0 and torch.equal(yd, yn)
    ref = O.fft(x.reshape(batch, n)[batch - 1], inverse=inverse)
    assert O.rel_l2(yt.view(batch, n)[batch - 1].cpu().numpy(), ref) <= 2e-6
