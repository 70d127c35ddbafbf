"""Pins the CPU oracle against the reference's own outputs (tests/golden, made by
tests/golden/make_golden.py from the compiled reference) and against a long-double DFT."""
import os

import numpy as np
import pytest

from oracle import oracle as O

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "reference_vectors.npz")
EPS32 = float(np.finfo(np.float32).eps)


@pytest.fixture(scope="module")
def golden():
    return np.load(GOLDEN)


def test_golden_lengths_cover_every_reference_strategy(golden):
    strat = golden["strategy"]
    seen = {int(strat[n]) for n in golden["lengths"]}
    assert {0, 1, 2, 3} <= seen


def test_oracle_matches_reference_outputs(golden):
    # parity bound of the plain form: rel-L2 <= 4 log2(N) eps(float)
    for n in golden["lengths"]:
        n = int(n)
        x = golden[f"in_{n}"]
        tol = 4 * np.log2(n) * EPS32
        for inv, key in ((False, "fwd"), (True, "inv")):
            err = O.rel_l2(golden[f"{key}_{n}"], O.fft(x, inverse=inv))
            assert err <= tol, (n, key, err, tol)


def test_strategy_restatement_matches_reference_for_all_lengths(golden):
    strat = golden["strategy"]
    lib = O.lib()
    mism = [n for n in range(2, 80001) if lib.orc_strategy(n) != strat[n]]
    assert mism == []


@pytest.mark.parametrize("n", list(range(1, 130)) + [243, 256, 343, 625, 997, 1000, 1009, 2310])
def test_oracle_fft_equals_long_double_dft(n):
    rng = np.random.default_rng(n)
    x = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    for inv in (False, True):
        assert O.rel_l2(O.fft(x, inv), O.dft(x, inv)) < 2e-15


@pytest.mark.parametrize("n", [65537, 131074, 100003, 117649, 59049])
def test_oracle_large_lengths_against_sampled_dft(n):
    rng = np.random.default_rng(7)
    x = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    y = O.fft(x)
    idx = rng.integers(0, n, 16)
    assert O.rel_l2(y[idx], O.dft_sampled(x, idx)) < 1e-13
    # numpy's pocketfft (FP64) as an independent cross-check
    assert O.rel_l2(y, np.fft.fft(x)) < 1e-14


def test_oracle_number_theory():
    assert O.primitive_root(1009) == 11
    assert O.primitive_root(65537) == 3
    assert O.next_smooth(2 * 1008 - 1) == 2048
    assert O.next_smooth(78126) == 0
    assert O.next_7smooth(2 * 999983 - 1) == 2000000


def test_reference_batch_threads_if_built():
    if not O.Reference.available():
        pytest.skip("reference not built on this host")
    ref = O.Reference()
    rng = np.random.default_rng(3)
    x = (rng.standard_normal((8, 1024)) + 1j * rng.standard_normal((8, 1024))).astype(np.complex64)
    y, t, _ = ref.batch(x, threads=2)
    assert t > 0
    assert O.rel_l2(y, O.fft(x)) < 4 * 10 * EPS32


CONFIG = os.path.join(os.path.dirname(__file__), "golden", "config_vectors.npz")


@pytest.fixture(scope="module")
def config_golden():
    return np.load(CONFIG)


def config_case(g, key):
    n, batch = int(g[f"{key}_n"]), int(g[f"{key}_batch"])
    x = O.fill_random(int(g[f"{key}_seed"]), n * batch, np.complex64, str(g[f"{key}_dist"])).reshape(batch, n)
    return n, x


def test_config_inputs_come_from_the_seeded_generator(config_golden):
    for key in config_golden["keys"]:
        key = str(key)
        n, batch = int(config_golden[f"{key}_n"]), int(config_golden[f"{key}_batch"])
        head = O.fill_random(int(config_golden[f"{key}_seed"]), 8, np.complex64, str(config_golden[f"{key}_dist"]))
        assert np.array_equal(head, config_golden[f"{key}_head"]), key


# the 2^27 transform takes about a minute in the FP64 oracle; its GPU output is compared with
# the reference's directly in tests/test_gpu_reference_parity.py
@pytest.mark.parametrize("key", ["c1", "c2_2520", "c2_59049", "c2_117649", "c2_1048576", "c2_1009", "c4",
                                 "c5_16777216"])
def test_oracle_matches_reference_on_config_inputs(config_golden, key):
    g = config_golden
    n, x = config_case(g, key)
    rows, idx = g[f"{key}_rows"], g[f"{key}_idx"]
    inverse = bool(int(g[f"{key}_inverse"]))
    y = O.fft_batch(x[rows].astype(np.complex128), inverse=inverse, threads=os.cpu_count() or 1)
    if inverse:
        y = y * n        # the reference gradient n * IFFT(g)
    err = O.rel_l2(y[:, idx], g[f"{key}_out"])
    assert err <= 4 * np.log2(n) * EPS32, (key, err)
