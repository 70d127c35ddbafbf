"""GPU parity: the CUDA path (through the C ABI) against the FP64 oracle and against the
reference's own outputs (tests/golden).  Bounds: rel-L2 <= 4 log2(N) eps(dtype) (the plain
form's parity rule), and <= 2e-6 against the FP64 oracle for FP32."""
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


def bound(n, eps):
    return 4 * max(np.log2(n), 1.0) * eps


def gpu_fft(x, inverse=False, dtype="complex64", flags=0):
    """x: (batch, n) numpy complex array -> GPU result as numpy."""
    batch, n = x.shape
    t = torch.from_numpy(np.ascontiguousarray(x)).cuda()
    y = torch.empty_like(t)
    plan = fg.FFT1D_C2C_invoker(n, dtype, batch, flags)
    plan.dispatch(inverse, t, y)
    torch.cuda.synchronize()
    return y.cpu().numpy()


def rand(n, batch, seed, dtype=np.complex64, dist="normal"):
    return fg.fill_random(seed, n * batch, dtype, dist).reshape(batch, n)


SWEEP = list(range(1, 130)) + [
    243, 256, 343, 512, 625, 729, 1000, 1024, 2048, 2187, 2401, 2520, 3125, 4096, 5040, 6561, 8192,
    10000, 12288, 13720, 14000, 15625, 16384, 16807, 19683, 32768, 40000, 59049, 65536, 78125,
    117649, 1 << 17, 1 << 18,
    # primes: Rader (cyclic when N-1 is 13-smooth, else zero-padded up to 39064)
    131, 257, 1009, 4099, 7681, 12289, 65537, 47, 59, 83, 107, 1019, 39043,
    # Bluestein
    999, 1001, 2050, 4097, 9999, 39062, 39063, 65535, 100003, 131074,
]


@pytest.mark.parametrize("n", SWEEP)
def test_fp32_forward_inverse_vs_oracle(n):
    batch = 3 if n < 50000 else 1
    x = rand(n, batch, n)
    ref = O.fft(x)
    y = gpu_fft(x)
    err = O.rel_l2(y, ref)
    assert err <= min(bound(n, EPS32), 2e-6) or err <= bound(n, EPS32), (n, err)
    assert err <= 2e-6, (n, err)
    yi = gpu_fft(x, inverse=True)
    erri = O.rel_l2(yi, O.fft(x, inverse=True))
    assert erri <= 2e-6, (n, erri)


@pytest.mark.parametrize("n", [2, 3, 7, 16, 60, 97, 243, 1000, 1009, 2520, 4096, 8192, 999, 39043,
                               65536, 65537, 117649, 131074])
def test_fp64_vs_oracle(n):
    batch = 2
    x = rand(n, batch, 7 * n, np.complex128)
    y = gpu_fft(x, dtype="complex128")
    err = O.rel_l2(y, O.fft(x))
    assert err <= bound(n, EPS64), (n, err)
    yi = gpu_fft(x, inverse=True, dtype="complex128")
    assert O.rel_l2(yi, O.fft(x, inverse=True)) <= bound(n, EPS64)


def test_fp32_vs_reference_golden_vectors():
    d = np.load(GOLDEN)
    for n in d["lengths"]:
        n = int(n)
        x = d[f"in_{n}"].reshape(1, n)
        for inv, key in ((False, "fwd"), (True, "inv")):
            y = gpu_fft(x, inverse=inv)
            err = O.rel_l2(y[0], d[f"{key}_{n}"])
            assert err <= bound(n, EPS32), (n, key, err)


def test_strategy_matches_reference_table():
    d = np.load(GOLDEN)
    s = d["strategy"]
    for n in list(range(2, 5000)) + list(range(38000, 40000)) + [65536, 65537, 78125, 79999, 80000]:
        assert int(fg.FFT1D_C2C_invoker.acquired_execution_strategy(n)) == int(s[n]), n


@pytest.mark.parametrize("n", [64, 1009, 4096, 65536, 999])
def test_in_place(n):
    x = rand(n, 2, 11)
    t = torch.from_numpy(x).cuda()
    plan = fg.FFT1D_C2C_invoker(n, "complex64", 2)
    plan.dispatch(False, t, t)
    torch.cuda.synchronize()
    assert O.rel_l2(t.cpu().numpy(), O.fft(x)) <= 2e-6


@pytest.mark.parametrize("n", [128, 2520, 65537])
def test_host_pointers_are_staged(n):
    x = rand(n, 2, 12)
    y = np.zeros_like(x)
    plan = fg.FFT1D_C2C_invoker(n, "complex64", 2)
    plan.dispatch(False, x, y)
    assert O.rel_l2(y, O.fft(x)) <= 2e-6


@pytest.mark.parametrize("n", [256, 1009, 999, 1 << 16])
def test_adjoint_is_scaled_conjugate_transpose(n):
    x = rand(n, 2, 13)
    t = torch.from_numpy(x).cuda()
    y = torch.empty_like(t)
    plan = fg.FFT1D_C2C_invoker(n, "complex64", 2)
    plan.adjoint(t, y, 0.5)
    torch.cuda.synchronize()
    ref = 0.5 * n * O.fft(x, inverse=True)
    assert O.rel_l2(y.cpu().numpy(), ref) <= 2e-6


def test_round_trip_and_linearity_large():
    n = 1 << 20
    x = rand(n, 2, 21)
    t = torch.from_numpy(x).cuda()
    plan = fg.FFT1D_C2C_invoker(n, "complex64", 2)
    y = torch.empty_like(t)
    z = torch.empty_like(t)
    plan.dispatch(False, t, y)
    plan.dispatch(True, y, z)
    torch.cuda.synchronize()
    assert O.rel_l2(z.cpu().numpy(), x) < 1e-6
    # linearity: F(a x0 + b x1) = a F(x0) + b F(x1)
    a, b = 0.75 - 0.25j, -1.5 + 2.0j
    u = (a * t[0] + b * t[1]).reshape(1, n).contiguous()
    fu = torch.empty_like(u)
    fg.FFT1D_C2C_invoker(n, "complex64", 1).dispatch(False, u, fu)
    torch.cuda.synchronize()
    assert O.rel_l2(fu.cpu().numpy()[0], (a * y[0] + b * y[1]).cpu().numpy()) < 2e-6


@pytest.mark.parametrize("n,batch,inverse", [(1 << 20, 9, False), (1 << 20, 9, True), (40009, 64, False),
                                             (2520, 4096, True)])
def test_host_pointers_overlapped_chunks(n, batch, inverse):
    # batches of 8 MB and more from host memory run as copy-in / kernels / copy-out chunks on
    # three streams; the result must equal the device-resident execution of the same plan
    x = rand(n, batch, 21)
    y = np.zeros_like(x)
    plan = fg.FFT1D_C2C_invoker(n, "complex64", batch)
    plan.dispatch(inverse, x, y)
    t = torch.from_numpy(x).cuda()
    yd = torch.empty_like(t)
    plan.dispatch(inverse, t, yd)
    torch.cuda.synchronize()
    assert np.array_equal(y, yd.cpu().numpy().reshape(y.shape))
    for b in (0, batch // 2, batch - 1):
        assert O.rel_l2(y[b], O.fft(x[b], inverse=inverse)) <= 2e-6
