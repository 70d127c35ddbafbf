"""The reference's own code built against the portable intrinsics (oracle/ref/portable_intrin.h),
as it runs on the aarch64 GPU host for the CPU baseline, reproduces the native AVX2 build.

On x86-64 both builds exist (oracle/_ref/libfyref.so native, libfyref_emu.so emulated) and must
agree bit for bit.  On any host, whichever build oracle/_ref/libfyref.so is must reproduce the
committed golden outputs (made by the native build): bit for bit where the host's libm gives
the same table entries, and always within the plan bound 4 log2(N) eps32."""
import os

import numpy as np
import pytest

from oracle import oracle as O

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(os.path.dirname(HERE), "oracle", "_ref")
NATIVE = os.path.join(REF_DIR, "libfyref.so")
EMULATED = os.path.join(REF_DIR, "libfyref_emu.so")
EPS32 = float(np.finfo(np.float32).eps)


def _ref(path):
    if not os.path.exists(path):
        pytest.skip(f"{os.path.basename(path)} not built on this host")
    return O.Reference(path)


@pytest.fixture(scope="module")
def both():
    nat, emu = _ref(NATIVE), _ref(EMULATED)
    if nat.build_info() != "native x86_64":
        pytest.skip("no native AVX2 build on this host")
    return nat, emu


LENGTHS = list(range(2, 130)) + [243, 256, 343, 625, 999, 1009, 2048, 2520, 4096, 6000, 8191, 16807, 39043, 39062,
                                 59049, 65536, 78125, 117649]


@pytest.mark.parametrize("inverse", [False, True])
def test_emulated_build_is_bit_identical_to_native(both, inverse):
    nat, emu = both
    rng = np.random.default_rng(11)
    for n in LENGTHS:
        if not nat.runnable(n):
            continue
        x = (rng.standard_normal((2, n)) + 1j * rng.standard_normal((2, n))).astype(np.complex64)
        a, b = nat.fft(x, inverse), emu.fft(x, inverse)
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32)), n


def test_built_reference_reproduces_golden_vectors():
    ref = _ref(NATIVE)
    g = np.load(os.path.join(HERE, "golden", "reference_vectors.npz"))
    exact = 0
    for n in g["lengths"]:
        n = int(n)
        for key, inv in (("fwd", False), ("inv", True)):
            y = ref.fft(g[f"in_{n}"], inverse=inv)
            exact += int(np.array_equal(y.view(np.uint32), g[f"{key}_{n}"].view(np.uint32)))
            assert O.rel_l2(y, g[f"{key}_{n}"]) <= 4 * np.log2(n) * EPS32, (n, key)
    if ref.build_info() == "native x86_64":
        assert exact == 2 * len(g["lengths"])


@pytest.mark.parametrize("key", ["c1", "c2_2520", "c2_59049", "c2_117649", "c2_1009"])
def test_built_reference_reproduces_config_fixtures(key):
    ref = _ref(NATIVE)
    g = np.load(os.path.join(HERE, "golden", "config_vectors.npz"))
    n, batch = int(g[f"{key}_n"]), int(g[f"{key}_batch"])
    x = O.fill_random(int(g[f"{key}_seed"]), n * batch, np.complex64, str(g[f"{key}_dist"])).reshape(batch, n)
    rows, idx = g[f"{key}_rows"], g[f"{key}_idx"]
    xr = np.ascontiguousarray(x[rows])
    y = np.empty_like(xr)
    pool = O.ReferencePool(ref, n, 4)
    pool.run(xr, y)
    pool.close()
    assert O.rel_l2(y[:, idx], g[f"{key}_out"]) <= 4 * np.log2(n) * EPS32
    if ref.build_info() == "native x86_64":
        assert np.array_equal(np.ascontiguousarray(y[:, idx]).view(np.uint32), g[f"{key}_out"].view(np.uint32))
