"""The allocation-free entry point (fyg_execute_noalloc) against the plan-based entry point and
the FP64 oracle.

Who calls it: a host application that owns all device memory (it sizes one pool up front and
gives each plugin only its input and output buffers) cannot let this library allocate behind
its back, and a loop with a latency budget cannot take the device-wide synchronization that
cudaMalloc / cudaFree may cause.  fyg_execute_noalloc keeps its scratch and twiddle tables in a
fixed device array inside the library instead.  Each case makes two calls in a row on the same
array (forward, then inverse on other data), so a stale table or intermediate from the first
call would show in the second.  This file is collected last, so a failure here leaves every
other test run; it passes alone in a fresh process and after the rest of the suite."""
import ctypes

import numpy as np
import pytest

torch = pytest.importorskip("torch")

import fyfft_gb300 as fg  # noqa: E402
from oracle import oracle as O  # noqa: E402

pytestmark = pytest.mark.gpu

FYG_ERR_INVALID_LENGTH = 1


def rel_l2(a, b):
    a = np.asarray(a, np.complex128)
    b = np.asarray(b, np.complex128)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def noalloc(x, n, batch, inverse, dtype_code):
    y = torch.empty_like(x)
    rc = fg.lib().fyg_execute_noalloc(n, batch, dtype_code, fg.FYG_INVERSE if inverse else fg.FYG_FORWARD,
                                      x.data_ptr(), y.data_ptr(), torch.cuda.current_stream().cuda_stream)
    fg.check(rc)
    return y


@pytest.mark.parametrize("n,batch,dtype", [
    (65536, 8, "complex64"),      # two passes: uses the scratch
    (1 << 20, 2, "complex64"),    # two passes of 1024
    (117649, 4, "complex64"),     # two passes, odd radices
    (2520, 16, "complex64"),      # single pass
    (16384, 4, "complex128"),     # FP64, two passes
])
def test_noalloc_matches_plan_path_twice_in_a_row(n, batch, dtype):
    npdt = np.complex64 if dtype == "complex64" else np.complex128
    tdt = torch.complex64 if dtype == "complex64" else torch.complex128
    code = fg.FYG_C32 if dtype == "complex64" else fg.FYG_C64
    eps = float(np.finfo(np.float32 if dtype == "complex64" else np.float64).eps)
    tol = 4 * np.log2(n) * eps
    plan = fg.FFT1D_C2C_invoker(n, dtype, batch)
    for call, (seed, inverse) in enumerate(((101, False), (202, True))):
        x = torch.from_numpy(fg.fill_random(seed + n, n * batch, npdt, "normal")).cuda()
        y = noalloc(x, n, batch, inverse, code)
        ref = torch.empty(n * batch, dtype=tdt, device="cuda")
        plan.dispatch(inverse, x, ref)
        torch.cuda.synchronize()
        yh = y.cpu().numpy()
        err = rel_l2(yh, ref.cpu().numpy())
        assert err <= tol, (n, batch, call, err, tol)
        # first and last transform against the FP64 oracle
        xh = x.cpu().numpy().reshape(batch, n)
        for b in (0, batch - 1):
            err_o = rel_l2(yh.reshape(batch, n)[b], O.fft(xh[b], inverse=inverse))
            assert err_o <= tol, (n, batch, call, b, err_o, tol)


def test_noalloc_rejects_sizes_beyond_its_array():
    n, batch = 1 << 20, 8   # 64 MiB of intermediates > 16 MiB
    x = torch.zeros(n * batch, dtype=torch.complex64, device="cuda")
    y = torch.empty_like(x)
    rc = fg.lib().fyg_execute_noalloc(n, batch, fg.FYG_C32, fg.FYG_FORWARD, x.data_ptr(), y.data_ptr(),
                                      torch.cuda.current_stream().cuda_stream)
    assert rc == FYG_ERR_INVALID_LENGTH
    assert b"16777216" in fg.lib().fyg_last_error_string()


def test_noalloc_rejects_host_pointers():
    x = np.zeros(256, np.complex64)
    y = np.zeros(256, np.complex64)
    rc = fg.lib().fyg_execute_noalloc(256, 1, fg.FYG_C32, fg.FYG_FORWARD, x.ctypes.data, y.ctypes.data, None)
    assert rc != 0
