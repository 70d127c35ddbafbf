"""Multi-device plan on the one GPU a test gets: the device list repeats device 0, so every
shard runs its own plan and stream on it (no shard waits on another).  Sharded results equal
the single-plan results bit for bit and the FP64 oracle within 2e-6."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

import fyfft_gb300 as fg  # noqa: E402
from oracle import oracle as O  # noqa: E402

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n,batch,devices", [(4096, 10, (0, 0)), (1 << 20, 5, (0, 0, 0)), (999983, 3, (0, 0)),
                                             (1009, 7, (0, 0, 0, 0)), (65537, 2, (0, 0, 0))])
def test_host_buffers_sharded(n, batch, devices):
    m = fg.MultiDevicePlan(n, "complex64", batch, devices)
    assert m.bounds[0] == 0 and m.bounds[-1] == batch
    x = fg.fill_random(11, n * batch, np.complex64, "normal")
    y = np.empty_like(x)
    m.execute(x, y)
    single = fg.FFT1D_C2C_invoker(n, "complex64", batch)
    y1 = np.empty_like(x)
    single.dispatch(False, x, y1)
    assert np.array_equal(y, y1)
    for b in (0, batch - 1):
        assert O.rel_l2(y[b * n:(b + 1) * n], O.fft(x[b * n:(b + 1) * n])) <= 2e-6
    z = np.empty_like(x)
    m.execute(y, z, invert=True)
    assert O.rel_l2(z, x) <= 2e-6


def test_device_buffers_sharded():
    n, batch, devices = 131074, 5, (0, 0)
    m = fg.MultiDevicePlan(n, "complex64", batch, devices)
    x = fg.fill_random(12, n * batch, np.complex64, "normal")
    xs, ys = [], []
    for i in range(len(devices)):
        a, b = m.bounds[i], m.bounds[i + 1]
        xs.append(torch.from_numpy(x[a * n:b * n]).cuda())
        ys.append(torch.empty_like(xs[-1]))
    m.execute_device(xs, ys)
    m.synchronize()
    y = np.concatenate([t.cpu().numpy() for t in ys])
    ref = O.fft(x.reshape(batch, n)[[0, batch - 1]])
    assert O.rel_l2(y.reshape(batch, n)[[0, batch - 1]], ref) <= 2e-6


def test_rejects_missing_device():
    with pytest.raises(fg.FygError):
        fg.MultiDevicePlan(1024, "complex64", 4, (0, 4096))
