"""Seeded synthetic workloads with the shapes of the benchmark configurations.

uneven_lengths: the mixed-length batch (4096 lengths in [16, 65536]): each length first picks a
category -- 7-smooth (0.70), prime (0.15), or with a prime factor > 7 (0.15) -- then draws a
log-uniform value in [16, 65536] and snaps to the nearest member of that category.  The
uniforms come from the library's counter-based generator, so the lengths are identical on
every machine.
"""
from __future__ import annotations

import bisect
import functools

import numpy as np

LO, HI = 16, 65536


def _max_prime_factor(n: int) -> int:
    best, p = 1, 2
    while p * p <= n:
        while n % p == 0:
            best, n = p, n // p
        p += 1
    return max(best, n) if n > 1 else best


@functools.lru_cache(maxsize=None)
def _categories():
    smooth, primes, awkward = [], [], []
    for n in range(LO, HI + 1):
        m = _max_prime_factor(n)
        if m <= 7:
            smooth.append(n)
        elif m == n:
            primes.append(n)
        else:
            awkward.append(n)
    return smooth, primes, awkward


def _snap(sorted_vals, x: float) -> int:
    i = bisect.bisect_left(sorted_vals, x)
    cands = [sorted_vals[j] for j in (i - 1, i) if 0 <= j < len(sorted_vals)]
    return min(cands, key=lambda v: abs(np.log(v) - np.log(x)))


def uneven_lengths(count: int = 4096, seed: int = 2):
    from . import fill_random
    u = fill_random(seed, count, np.complex128, "uniform")
    cat_u = (u.real + 1.0) / 2.0          # category draw in [0, 1)
    len_u = (u.imag + 1.0) / 2.0          # log-uniform draw in [0, 1)
    smooth, primes, awkward = _categories()
    out = []
    for cu, lu in zip(cat_u, len_u):
        x = float(np.exp(np.log(LO) + lu * (np.log(HI) - np.log(LO))))
        cat = smooth if cu < 0.70 else (primes if cu < 0.85 else awkward)
        out.append(_snap(cat, x))
    return out
