"""Differentiation through the hand-written adjoint: loss = Re<g, FFT(x)>, so dL/dx = F^H g.
Checked against central finite differences (h = 1e-3, FP64 replay of the loss with the FP64
GPU transform) on 64 random coordinates, against N * (the reference's inverse transform) from
the golden vectors, against N * (FP64 oracle inverse), and with torch.autograd.gradcheck."""
import os

import numpy as np
import pytest

torch = pytest.importorskip("torch")

import fyfft_gb300 as fg  # noqa: E402
from fyfft_gb300.autograd import FFTFunction, fft, ifft  # noqa: E402
from oracle import oracle as O  # noqa: E402

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "reference_vectors.npz")
EPS32 = float(np.finfo(np.float32).eps)


def loss_fp64(x64_row, g64_row, plan64):
    X = torch.empty_like(x64_row)
    plan64.dispatch(False, x64_row, X)
    return float(torch.sum(torch.conj(g64_row) * X).real)


@pytest.mark.parametrize("n,batch", [(1 << 20, 16), (100003, 32)])
def test_adjoint_gradient_vs_finite_differences_and_oracle(n, batch):
    x = torch.from_numpy(fg.fill_random(3, n * batch, np.complex64, "normal")).cuda().reshape(batch, n)
    g = torch.from_numpy(fg.fill_random(103, n * batch, np.complex64, "normal")).cuda().reshape(batch, n)
    x.requires_grad_(True)
    y = fft(x)
    L = torch.sum(torch.conj(g) * y).real
    L.backward()
    grad = x.grad.detach()
    torch.cuda.synchronize()
    # central differences in FP64 on 64 coordinates (real and imaginary parts)
    rng = np.random.default_rng(3)
    plan64 = fg.FFT1D_C2C_invoker(n, "complex128", 1)
    x64, g64 = x.detach().to(torch.complex128), g.to(torch.complex128)
    h = 1e-3
    for _ in range(64):
        b, i = int(rng.integers(batch)), int(rng.integers(n))
        for unit, part in ((1.0, "re"), (1j, "im")):
            xp = x64[b].clone(); xp[i] += h * unit
            xm = x64[b].clone(); xm[i] -= h * unit
            fd = (loss_fp64(xp, g64[b], plan64) - loss_fp64(xm, g64[b], plan64)) / (2 * h)
            an = float(grad[b, i].real if part == "re" else grad[b, i].imag)
            assert abs(fd - an) <= 1e-4 * max(1.0, abs(fd)), (n, b, i, part, fd, an)
    # the whole gradient against N * inverse (FP64 oracle) on two rows
    for b in (0, batch - 1):
        ref = n * O.fft(g[b].cpu().numpy(), inverse=True)
        assert O.rel_l2(grad[b].cpu().numpy(), ref) <= 2e-6


def test_adjoint_equals_n_times_reference_inverse_on_golden_vectors():
    d = np.load(GOLDEN)
    for n in d["lengths"]:
        n = int(n)
        gvec = torch.from_numpy(d[f"in_{n}"]).cuda()
        out = torch.empty_like(gvec)
        fg.FFT1D_C2C_invoker(n, "complex64", 1).adjoint(gvec, out, 1.0)
        torch.cuda.synchronize()
        ref = n * d[f"inv_{n}"].astype(np.complex128)
        assert O.rel_l2(out.cpu().numpy(), ref) <= 4 * max(np.log2(n), 1) * EPS32, n


@pytest.mark.parametrize("n", [16, 60, 97, 999])
def test_gradcheck_fp64(n):
    x = torch.randn(2, n, dtype=torch.complex128, device="cuda", requires_grad=True)
    assert torch.autograd.gradcheck(lambda t: FFTFunction.apply(t, False), (x,), eps=1e-6, atol=1e-7, rtol=1e-6)
    assert torch.autograd.gradcheck(lambda t: FFTFunction.apply(t, True), (x,), eps=1e-6, atol=1e-7, rtol=1e-6)


def test_inverse_backward_and_round_trip_gradient():
    n = 4096
    x = torch.from_numpy(fg.fill_random(9, 4 * n, np.complex64, "normal")).cuda().reshape(4, n)
    x.requires_grad_(True)
    y = ifft(fft(x))
    L = torch.sum(y.real * 2.0 + y.imag)
    L.backward()
    # d/dx of Re-linear functional through the identity
    expected = torch.full_like(x, 2.0 + 1.0j)
    assert torch.allclose(x.grad, expected, atol=1e-5)
