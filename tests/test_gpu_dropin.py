"""The drop-in C++ header (include/foye_FFT_gpu.hpp) compiled into a program that uses the
reference's API, run on the GPU; and the FP64-convolution variant of FP32 plans."""
import os
import subprocess

import numpy as np
import pytest

torch = pytest.importorskip("torch")

import fyfft_gb300 as fg  # noqa: E402
from oracle import oracle as O  # noqa: E402

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_cpp_dropin_example(tmp_path):
    exe = tmp_path / "dropin"
    libdir = os.path.dirname(fg.LIB_PATH)
    subprocess.run(["g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", "dropin_example.cpp"), "-L", libdir, "-lfygpu",
                    f"-Wl,-rpath,{libdir}", "-o", str(exe)], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    print(r.stdout)
    assert r.returncode == 0, r.stdout + r.stderr


@pytest.mark.parametrize("n", [999, 1009, 65537, 131074, 39043])
def test_fp64_convolution_variant(n):
    batch = 2
    x = fg.fill_random(n + 5, n * batch, np.complex64, "normal")
    t = torch.from_numpy(x).cuda()
    y = torch.empty_like(t)
    plan = fg.FFT1D_C2C_invoker(n, "complex64", batch, fg.FYG_FLAG_CONV_FP64)
    for inv in (False, True):
        plan.dispatch(inv, t, y)
        torch.cuda.synchronize()
        err = O.rel_l2(y.cpu().numpy().reshape(batch, n), O.fft(x.reshape(batch, n), inverse=inv))
        assert err <= 1e-6, (n, inv, err)
