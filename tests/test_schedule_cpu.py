"""The planner's schedules on the CPU.  fyg_plan_schedule computes, without a GPU, the strategy,
convolution length, split factor and pass radices that fyg_plan_create chooses.  These tests
(1) pin the schedules of the benchmark's configurations to the ones the GPU runs record, and
(2) run each schedule through the algorithms' index maps in numpy, in FP64, against the FP64
oracle.  Covered: the multi-pass Stockham algebra of fyg_pass.cuh (column j, k = j mod Ns,
inputs x[j + m Rr], twiddle exp(-2 pi i m k / (Ns R)), outputs (j / Ns) Ns R + k + m' Ns); Rader
with a cyclic and a zero-padded convolution; Bluestein; and the N = m p split.  The length-R DFT
inside a pass is the oracle's; the kernels themselves are checked on the GPU."""
import numpy as np
import pytest

import fyfft_gb300 as fg
from oracle import oracle as O

TOL = 1e-12


def stockham(x, radices, inverse=False):
    """The multi-pass Stockham transform of x (length prod(radices)) with these pass radices."""
    x = np.asarray(x, dtype=np.complex128)
    if inverse:
        return np.conj(stockham(np.conj(x), radices)) / x.size
    L = x.size
    assert int(np.prod(radices)) == L
    ns = 1
    for R in radices:
        rr = L // R
        j = np.arange(rr)
        k = j % ns
        X = x.reshape(R, rr) * np.exp(-2j * np.pi * np.outer(np.arange(R), k) / (ns * R))
        Y = O.fft_batch(np.ascontiguousarray(X.T)).T          # Y[m', j] = DFT_R over m
        y = np.empty(L, dtype=np.complex128)
        y[((j // ns) * ns * R + k)[None, :] + (np.arange(R) * ns)[:, None]] = Y
        x, ns = y, ns * R
    return x


def conv(a, b, radices):
    """Cyclic convolution through the schedule's forward and inverse transforms."""
    return stockham(stockham(a, radices) * stockham(b, radices), radices, inverse=True)


def rader(x, L, radices):
    n = x.size
    g = O.primitive_root(n)
    lc = n - 1
    ginv = pow(g, n - 2, n)
    gp = np.array([pow(g, q, n) for q in range(lc)])
    gi = np.array([pow(ginv, q, n) for q in range(lc)])
    a = np.zeros(L, dtype=np.complex128)
    a[:lc] = x[gi]
    kt = np.exp(-2j * np.pi * gp[np.arange(L) % lc] / n)      # periodic for the zero-padded form
    c = conv(a, kt, radices)
    y = np.empty(n, dtype=np.complex128)
    y[0] = x[0] + x[1:].sum()
    if L == lc:
        y[gp] = x[0] + c
    else:
        q = np.arange(lc - 1, 2 * lc - 1)                    # outputs that carry the cyclic result
        y[gp[q % lc]] = x[0] + c[q]
    return y


def bluestein(x, M, radices):
    n = x.size
    k = np.arange(n, dtype=np.int64)
    w = np.exp(1j * np.pi * ((k * k) % (2 * n)) / n)
    a = np.zeros(M, dtype=np.complex128)
    a[:n] = x * np.conj(w)
    b = np.zeros(M, dtype=np.complex128)
    b[:n] = w
    b[M - n + 1:] = w[1:][::-1]
    return np.conj(w) * conv(a, b, radices)[:n]


def split(x, m, radices):
    n = x.size
    p = n // m
    k1, n2 = np.arange(m), np.arange(p)
    z = (np.exp(-2j * np.pi * np.outer(k1, k1) / m) @ x.reshape(m, p)) * np.exp(-2j * np.pi * np.outer(k1, n2) / n)
    y = np.empty(n, dtype=np.complex128)
    for j in range(m):
        y[j::m] = rader(z[j], p - 1, radices)
    return y


def run_schedule(x, dtype="complex64"):
    s = fg.plan_schedule(x.size, dtype)
    st, L, m, rad = s["gpu_strategy"], s["conv_length"], s["split_m"], s["pass_radices"]
    if st in (0, 1):
        return stockham(x, rad), s
    if st == 2:
        return rader(x, L, rad), s
    if st == 3:
        return bluestein(x, L, rad), s
    if st == 5:
        return split(x, m, rad), s
    raise AssertionError(s)


# (n, dtype) -> (strategy, conv length, split m, pass radices) as the GPU runs record them
# (plan info and kernel names of the benchmark and configuration runs)
RECORDED = {
    (2520, "complex64"): (0, 2520, 1, [2520]),
    (59049, "complex64"): (1, 59049, 1, [243, 243]),
    (117649, "complex64"): (1, 117649, 1, [343, 343]),
    (1 << 20, "complex64"): (1, 1 << 20, 1, [1024, 1024]),
    (1009, "complex64"): (2, 1008, 1, [1008]),
    (65537, "complex64"): (2, 65536, 1, [256, 256]),
    (999983, "complex64"): (3, 1 << 21, 1, [1024, 2048]),
    (131074, "complex64"): (5, 65536, 2, [256, 256]),
    (100003, "complex64"): (3, 1 << 18, 1, [512, 512]),
    (1 << 24, "complex64"): (1, 1 << 24, 1, [256, 256, 256]),
    (1 << 27, "complex64"): (1, 1 << 27, 1, [512, 512, 512]),
    (4096, "complex128"): (0, 4096, 1, [4096]),
}


@pytest.mark.parametrize("key", list(RECORDED))
def test_benchmark_schedules_match_the_gpu_records(key):
    n, dt = key
    s = fg.plan_schedule(n, dt)
    assert (s["gpu_strategy"], s["conv_length"], s["split_m"], s["pass_radices"]) == RECORDED[key]


def test_schedule_needs_no_gpu_and_validates():
    assert fg.plan_schedule(1)["gpu_strategy"] == 4
    with pytest.raises(fg.FygError):
        fg.plan_schedule(0)
    with pytest.raises(fg.FygError):
        fg.plan_schedule(1 << 31)
    # Bluestein lengths are 7-smooth or powers of two; the split leaves p - 1 as the length
    for n in (40009, 999983, 131078, 100003):
        L = fg.plan_schedule(n)["conv_length"]
        assert L >= 2 * n - 1 and int(np.prod(fg.plan_schedule(n)["pass_radices"])) == L


@pytest.mark.parametrize("n", [4096, 10000, 59049, 78125, 60060, 73216, 117649, 1 << 17, 1 << 20, 3 << 20])
@pytest.mark.parametrize("dtype", ["complex64", "complex128"])
def test_stockham_schedules_reproduce_the_dft(n, dtype):
    x = O.fill_random(n % 1000 + 1, n, np.complex128, "normal")
    y, s = run_schedule(x, dtype)
    assert s["gpu_strategy"] in (0, 1)
    assert O.rel_l2(y, O.fft(x)) <= TOL, s


def test_three_pass_schedule_reproduces_the_dft():
    n = 1 << 23                      # three passes, 32 x 512 x 512
    x = O.fill_random(23, n, np.complex128, "normal")
    y, s = run_schedule(x)
    assert len(s["pass_radices"]) == 3
    assert O.rel_l2(y, O.fft(x)) <= TOL, s


@pytest.mark.parametrize("n", [1009, 65537, 12289, 1031, 39043, 999983, 100003, 40009, 131078, 131074, 24578,
                               73734])
@pytest.mark.parametrize("dtype", ["complex64", "complex128"])
def test_convolution_schedules_reproduce_the_dft(n, dtype):
    x = O.fill_random(n % 1000 + 2, n, np.complex128, "normal")
    y, s = run_schedule(x, dtype)
    assert s["gpu_strategy"] in (2, 3, 5)
    assert O.rel_l2(y, O.fft(x)) <= TOL, s
