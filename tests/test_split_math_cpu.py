"""The index map of the N = m p split, restated in numpy on the CPU: length-m DFTs over the
p-strided input and the twiddles w_N^(n2 k1) (what fyg_split.cu computes), then length-p DFTs
whose outputs land at k1 + m k2 (what the Rader scatter store with stride m writes), equal the
FP64 oracle's DFT of length N in both directions."""
import numpy as np
import pytest

from oracle import oracle as O


def split_dft(x, m, inverse=False):
    n = x.size
    p = n // m
    sgn = 1.0 if inverse else -1.0
    n2 = np.arange(p)
    k1 = np.arange(m)
    xs = x.reshape(m, p)                                         # xs[n1, n2] = x[n2 + p n1]
    wm = np.exp(sgn * 2j * np.pi * np.outer(k1, k1) / m)         # w_m^(n1 k1)
    z = (wm @ xs) * np.exp(sgn * 2j * np.pi * np.outer(k1, n2) / n)   # z[k1, n2]
    y = np.empty(n, dtype=np.complex128)
    for j in range(m):
        y[j::m] = O.fft(z[j], inverse=inverse) * (1.0 / m if inverse else 1.0)
    return y


@pytest.mark.parametrize("m,p", [(2, 3457), (3, 1031), (5, 257), (7, 97), (8, 193), (6, 12289)])
@pytest.mark.parametrize("inverse", [False, True])
def test_split_index_map_equals_dft(m, p, inverse):
    x = O.fill_random(50 + m, m * p, np.complex128, "normal")
    assert O.rel_l2(split_dft(x, m, inverse), O.fft(x, inverse=inverse)) <= 1e-13
