"""Strided batch layout (fyg_plan_create_layout): transforms idist / odist elements apart in the
user buffers; every transform matches the FP64 oracle and the gaps between transforms keep
their contents, for device buffers and for host buffers (plain and overlapped staging)."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

import fyfft_gb300 as fg  # noqa: E402
from oracle import oracle as O  # noqa: E402

pytestmark = pytest.mark.gpu

SENTINEL = np.complex64(123.0 - 45.0j)


def strided(x, n, batch, dist):
    buf = np.full((batch - 1) * dist + n, SENTINEL, dtype=np.complex64)
    for b in range(batch):
        buf[b * dist:b * dist + n] = x[b]
    return buf


def rows(buf, n, batch, dist):
    return np.stack([buf[b * dist:b * dist + n] for b in range(batch)])


def gaps_intact(buf, n, batch, dist):
    mask = np.ones(buf.size, dtype=bool)
    for b in range(batch):
        mask[b * dist:b * dist + n] = False
    return np.all(buf[mask] == SENTINEL)


# single-pass tile (4096), Rader single pass (1009), generic multi-pass (10000 = 100 x 100),
# register-resident passes (2^16, Rader 65537, Bluestein 40009 on 2^17)
@pytest.mark.parametrize("n", [4096, 1009, 10000, 1 << 16, 65537, 40009])
@pytest.mark.parametrize("where", ["device", "host"])
@pytest.mark.parametrize("inverse", [False, True])
def test_strided_layout(n, where, inverse):
    batch, idist, odist = 3, n + 37, n + 101
    x = fg.fill_random(17, n * batch, np.complex64, "normal").reshape(batch, n)
    xin = strided(x, n, batch, idist)
    yout = np.full((batch - 1) * odist + n, SENTINEL, dtype=np.complex64)
    plan = fg.FFT1D_C2C_invoker(n, "complex64", batch, idist=idist, odist=odist)
    if where == "device":
        xd = torch.from_numpy(xin).cuda()
        yd = torch.from_numpy(yout).cuda()
        plan.dispatch(inverse, xd, yd)
        torch.cuda.synchronize()
        y = yd.cpu().numpy()
        assert np.array_equal(xd.cpu().numpy(), xin)      # the input is not modified
    else:
        plan.dispatch(inverse, xin, yout)
        y = yout
    assert gaps_intact(y, n, batch, odist)
    for b, yb in enumerate(rows(y, n, batch, odist)):
        assert O.rel_l2(yb, O.fft(x[b], inverse=inverse)) <= 2e-6, (n, b)


def test_strided_layout_overlapped_host_staging():
    # 3 x 2^20 complex<float> = 25 MB: host buffers go through the chunked copy/compute pipeline
    n, batch, idist, odist = 1 << 20, 3, (1 << 20) + 64, (1 << 20) + 96
    x = fg.fill_random(19, n * batch, np.complex64, "normal").reshape(batch, n)
    xin = strided(x, n, batch, idist)
    yout = np.full((batch - 1) * odist + n, SENTINEL, dtype=np.complex64)
    plan = fg.FFT1D_C2C_invoker(n, "complex64", batch, idist=idist, odist=odist)
    plan.dispatch(False, xin, yout)
    assert gaps_intact(yout, n, batch, odist)
    ys = rows(yout, n, batch, odist)
    for b in (0, batch - 1):
        assert O.rel_l2(ys[b], O.fft(x[b])) <= 2e-6


def test_layout_in_place_needs_equal_distances():
    n, batch = 4096, 2
    plan = fg.FFT1D_C2C_invoker(n, "complex64", batch, idist=n + 8, odist=n + 16)
    buf = torch.zeros((batch - 1) * (n + 16) + n, dtype=torch.complex64, device="cuda")
    with pytest.raises(fg.FygError):
        plan.dispatch(False, buf, buf)
    same = fg.FFT1D_C2C_invoker(n, "complex64", batch, idist=n + 8, odist=n + 8)
    x = fg.fill_random(3, n * batch, np.complex64, "normal").reshape(batch, n)
    b2 = torch.from_numpy(strided(x, n, batch, n + 8)).cuda()
    same.dispatch(False, b2, b2)
    torch.cuda.synchronize()
    y = b2.cpu().numpy()
    assert gaps_intact(y, n, batch, n + 8)
    for b, yb in enumerate(rows(y, n, batch, n + 8)):
        assert O.rel_l2(yb, O.fft(x[b])) <= 2e-6


def test_layout_rejects_short_distances():
    with pytest.raises(fg.FygError):
        fg.FFT1D_C2C_invoker(4096, "complex64", 2, idist=4000)


@pytest.mark.parametrize("n,batch", [(1 << 16, 64), (999983, 4), (2520, 8)])
def test_async_host_execution_pipelines_and_matches(n, batch):
    """fyg_execute_async on pinned host buffers: two plans enqueued back to back without
    blocking, then one stream synchronize; outputs equal the blocking path's."""
    x1 = torch.from_numpy(fg.fill_random(31, n * batch, np.complex64, "normal")).pin_memory()
    x2 = torch.from_numpy(fg.fill_random(32, n * batch, np.complex64, "normal")).pin_memory()
    y1, y2 = torch.empty_like(x1).pin_memory(), torch.empty_like(x2).pin_memory()
    p1 = fg.FFT1D_C2C_invoker(n, "complex64", batch)
    p2 = fg.FFT1D_C2C_invoker(n, "complex64", batch)
    s = torch.cuda.current_stream()
    for _ in range(2):
        p1.dispatch(False, x1.numpy(), y1.numpy(), s, blocking=False)
        p2.dispatch(True, x2.numpy(), y2.numpy(), s, blocking=False)
        p1.dispatch(False, x1.numpy(), y1.numpy(), s, blocking=False)   # same plan again: staging reuse
    p1.join(s)
    p2.join(s)
    s.synchronize()
    r1, r2 = np.empty_like(x1.numpy()), np.empty_like(x2.numpy())
    p1.dispatch(False, x1.numpy(), r1)
    p2.dispatch(True, x2.numpy(), r2)
    assert np.array_equal(y1.numpy(), r1) and np.array_equal(y2.numpy(), r2)
    assert O.rel_l2(r1.reshape(batch, n)[-1], O.fft(x1.numpy().reshape(batch, n)[-1])) <= 2e-6
