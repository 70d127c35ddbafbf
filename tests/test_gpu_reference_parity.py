"""GPU outputs against the reference's own outputs on the benchmark configurations' inputs.

tests/golden/config_vectors.npz holds what the reference's FFT1D_C2C_invoker computed
(tests/golden/make_golden.py) on the seeded inputs of every configuration it can run: C1
(4096 x 256, the float twin of the complex<double> configuration), the C2 sizes 2520, 59049,
117649, 2^20 and 1009, the C4 reference gradient n * dispatch<true>(g) at 2^20, and C5 (2^24 x 8,
2^27 x 1).  The parity bound of the plain form is rel-L2 <= 4 log2(N) eps32 against the
reference (the reference computes in float); the same outputs are also within 2e-6 of the FP64
oracle (tests/test_gpu_configs.py).  The whole batch of each configuration runs on the GPU; the
recorded rows are compared at the recorded output indices."""
import os

import numpy as np
import pytest

torch = pytest.importorskip("torch")

import fyfft_gb300 as fg  # noqa: E402

pytestmark = pytest.mark.gpu

EPS32 = float(np.finfo(np.float32).eps)
CONFIG = os.path.join(os.path.dirname(__file__), "golden", "config_vectors.npz")


@pytest.fixture(scope="module")
def g():
    return np.load(CONFIG)


def rel_l2(a, b):
    a = np.asarray(a, dtype=np.complex128)
    b = np.asarray(b, dtype=np.complex128)
    return float(np.linalg.norm((a - b).ravel()) / np.linalg.norm(b.ravel()))


def gpu_case(g, key, dtype="complex64"):
    n, batch = int(g[f"{key}_n"]), int(g[f"{key}_batch"])
    npdt = np.complex64 if dtype == "complex64" else np.complex128
    x = fg.fill_random(int(g[f"{key}_seed"]), n * batch, npdt, str(g[f"{key}_dist"]))
    assert np.array_equal(x[:8].astype(np.complex64), g[f"{key}_head"])
    xd = torch.from_numpy(x).cuda()
    yd = torch.empty_like(xd)
    plan = fg.FFT1D_C2C_invoker(n, dtype, batch)
    if int(g[f"{key}_inverse"]):
        plan.adjoint(xd, yd, 1.0)           # F^H g = n * IFFT(g), the reference gradient
    else:
        plan.dispatch(False, xd, yd)
    torch.cuda.synchronize()
    rows = torch.as_tensor(g[f"{key}_rows"], device="cuda")
    idx = torch.as_tensor(g[f"{key}_idx"], device="cuda")
    got = yd.view(batch, n).index_select(0, rows).index_select(1, idx).cpu().numpy()
    return n, got


def test_c1_complex_double_vs_reference_float():
    gg = np.load(CONFIG)
    n, got = gpu_case(gg, "c1", "complex128")
    assert rel_l2(got, gg["c1_out"]) <= 4 * np.log2(n) * EPS32


@pytest.mark.parametrize("key", ["c2_2520", "c2_59049", "c2_117649", "c2_1048576", "c2_1009", "c4",
                                 "c5_16777216", "c5_134217728"])
def test_config_vs_reference(g, key):
    n, got = gpu_case(g, key)
    err = rel_l2(got, g[f"{key}_out"])
    assert err <= 4 * np.log2(n) * EPS32, (key, err)
