"""The oracle's restatement of the seeded input generator equals the GPU library's host
generator (fyg_fill_random) bit for bit, so that fixtures and the CPU baseline can make every
configuration's inputs without loading the product library.  No GPU needed."""
import numpy as np
import pytest

from oracle import oracle as O

fg = pytest.importorskip("fyfft_gb300")


def _lib_or_skip():
    try:
        fg.lib()
    except RuntimeError as e:       # the library is built by __graft_entry__.build()
        pytest.skip(str(e))


@pytest.mark.parametrize("dtype", [np.complex64, np.complex128])
@pytest.mark.parametrize("dist", ["uniform", "normal"])
@pytest.mark.parametrize("seed,n", [(0, 1), (0, 4096 * 3), (1, 300001), (2, 65536), (4, 1 << 17)])
def test_generator_matches_library(dtype, dist, seed, n):
    _lib_or_skip()
    a = O.fill_random(seed, n, dtype, dist)
    b = fg.fill_random(seed, n, dtype, dist)
    assert np.array_equal(a.view(np.uint8), b.view(np.uint8))


def test_generator_is_independent_of_thread_count():
    a = O.fill_random(9, 200003, np.complex64, "normal", threads=1)
    b = O.fill_random(9, 200003, np.complex64, "normal", threads=7)
    assert np.array_equal(a.view(np.uint8), b.view(np.uint8))


def test_generator_distributions():
    u = O.fill_random(3, 1 << 18, np.complex128, "uniform")
    assert u.real.min() >= -1 and u.real.max() < 1 and abs(u.real.mean()) < 0.01
    z = O.fill_random(3, 1 << 18, np.complex128, "normal")
    assert abs(z.real.std() - 1) < 0.01 and abs(z.imag.std() - 1) < 0.01
