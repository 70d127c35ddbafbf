"""The benchmark configurations as parity tests (seeded synthetic inputs with their shapes).

C1  complex<double> N=4096 x 256: vs the FP64 oracle (4 log2 N eps64) and, on the reference's
    own float input/output pair, vs the reference at the float bound.
C2  complex<float> precision sweep, batch 64: rel-L2 <= 2e-6 vs the FP64 oracle on sampled
    transforms of every size (every transform of the batch is computed on the GPU).
C5  complex<float> N=2^27 x 1 and 2^24 x 8: rel-L2 on 1,048,576 sampled outputs vs a full FP64
    oracle FFT, plus round trip."""
import os

import numpy as np
import pytest

torch = pytest.importorskip("torch")

import fyfft_gb300 as fg  # noqa: E402
from oracle import oracle as O  # noqa: E402

pytestmark = pytest.mark.gpu

EPS32 = float(np.finfo(np.float32).eps)
EPS64 = float(np.finfo(np.float64).eps)
GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "reference_vectors.npz")


def run(x, n, batch, dtype, inverse=False):
    t = torch.from_numpy(x).cuda()
    y = torch.empty_like(t)
    fg.FFT1D_C2C_invoker(n, dtype, batch).dispatch(inverse, t, y)
    torch.cuda.synchronize()
    return y.cpu().numpy().reshape(batch, n)


def test_c1_double_4096x256():
    n, batch = 4096, 256
    x = fg.fill_random(0, n * batch, np.complex128, "uniform")
    y = run(x, n, batch, "complex128")
    ref = O.fft(x.reshape(batch, n))
    assert O.rel_l2(y, ref) <= 4 * np.log2(n) * EPS64
    # the reference's own float pair, computed in FP64 on the GPU
    d = np.load(GOLDEN)
    xr = d["in_4096"].astype(np.complex128)
    yr = run(xr, n, 1, "complex128")
    assert O.rel_l2(yr[0], d["fwd_4096"]) <= 4 * np.log2(n) * EPS32


@pytest.mark.parametrize("n", [2520, 59049, 117649, 1 << 20, 1009, 65537, 999983, 131074])
def test_c2_precision_sweep(n):
    batch = 64
    x = fg.fill_random(1, n * batch, np.complex64, "normal")
    y = run(x, n, batch, "complex64")
    xs = x.reshape(batch, n)
    for b in ((0, 37, 63) if n < 500000 else (37,)):
        err = O.rel_l2(y[b], O.fft(xs[b]))
        assert err <= 2e-6, (n, b, err)
        assert err <= 4 * np.log2(n) * EPS32


@pytest.mark.parametrize("n,batch", [(1 << 27, 1), (1 << 24, 8)])
def test_c5_large(n, batch):
    x = fg.fill_random(4, n * batch, np.complex64, "uniform")
    t = torch.from_numpy(x).cuda()
    y = torch.empty_like(t)
    plan = fg.FFT1D_C2C_invoker(n, "complex64", batch)
    plan.dispatch(False, t, y)
    z = torch.empty_like(t)
    plan.dispatch(True, y, z)
    torch.cuda.synchronize()
    rt = (torch.linalg.vector_norm(z - t) / torch.linalg.vector_norm(t)).item()
    assert rt <= 2e-6
    rng = np.random.default_rng(4)
    idx = rng.integers(0, n, 1 << 20)
    b = batch - 1
    ref = O.fft(x[b * n:(b + 1) * n])
    got = y[b * n:(b + 1) * n].cpu().numpy()
    err = O.rel_l2(got[idx], ref[idx])
    assert err <= 2e-6, err
