"""Generate the golden fixtures of tests/golden/ from the reference's own C++ FFT.

Runs where the reference checkout is available (it builds oracle/_ref/libfyref.so with
oracle/ref/build_ref.sh, which locates the checkout itself; pass a directory to override):

    python tests/golden/make_golden.py [REFERENCE_DIR]

reference_vectors.npz -- small lengths covering every strategy (complex64, interleaved like the
reference's float* buffers):
  in_<n>   input, numpy default_rng(1000+n), re/im i.i.d. uniform[-1, 1]
  fwd_<n>  FFT1D_C2C_invoker{n}.dispatch<false>(in)   (foye_FFT.hpp:128-151)
  inv_<n>  FFT1D_C2C_invoker{n}.dispatch<true>(in)    (scaled by 1/n)
  strategy uint8[80001]: FFT1D_C2C_invoker::acquired_execution_strategy(n) for n in [0, 80000]
           (foye_FFT.hpp:162-184; entries 0 and 1 are outside the reference's range and hold 255)
  lengths  the n values above

config_vectors.npz -- the reference's outputs on the benchmark configurations' own inputs (the
seeded generator, oracle.fill_random), for every configuration the reference can run:
  <key>_n, <key>_batch, <key>_seed, <key>_dist   the configuration
  <key>_rows   transforms (batch rows) recorded
  <key>_idx    output indices recorded per row (all of them for short lengths)
  <key>_out    complex64 [rows, idx]: the reference's output there
  <key>_head   complex64: the first 8 input values (detects a change of the generator)
  <key>_inverse 1 when the recorded output is n * dispatch<true>(in) (the reference gradient)
keys: c1 (4096 x 256, uniform seed 0; float twin of the complex<double> configuration),
c2_<n> (n in 2520, 59049, 117649, 2^20, 1009; batch 64, normal seed 1), c4 (2^20 x 16, normal
seed 3: the reference gradient n * IFFT(g)), c5_<n> (2^24 x 8 and 2^27 x 1, uniform seed 4).
The other configuration lengths (65537, 999983, 131074, 100003, and the mixed batch's primes
and awkward lengths above 39062) fall to the reference's O(N^2) DFT and cannot be run.
"""
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402

# Every strategy of the reference is represented: directly supported radix-2/3/4/5/7 lengths
# (including every micro-kernel size), mixed radix, Rader primes, Bluestein lengths and the
# small-n DFT fallback is not reachable below 39063, so it has no entry.
LENGTHS = sorted(set(
    [2, 3, 4, 5, 7, 8, 9, 16, 25, 27, 32, 49, 64, 81, 125, 128, 243, 256, 343, 512, 625, 729,
     1024, 2048, 2187, 2401, 3125, 4096, 6561, 8192]
    + [6, 10, 12, 14, 15, 18, 20, 21, 24, 28, 30, 35, 36, 40, 42, 45, 48, 60, 63, 70, 72, 96,
       100, 105, 120, 210, 360, 420, 1000, 1260, 2520, 5040, 6000]
    + [11, 13, 17, 19, 23, 29, 31, 37, 97, 101, 257, 509, 1009, 2003, 4001, 8191]
    + [22, 26, 33, 34, 38, 39, 51, 55, 77, 121, 143, 187, 999, 1001, 1234, 2050, 4097]))

# (key, n, batch, seed, dist, rows, samples per row (0 = all), reference gradient)
CONFIGS = [
    ("c1", 4096, 256, 0, "uniform", list(range(256)), 64, False),
    ("c2_2520", 2520, 64, 1, "normal", [0, 1, 63], 0, False),
    ("c2_59049", 59049, 64, 1, "normal", [0, 63], 2048, False),
    ("c2_117649", 117649, 64, 1, "normal", [0, 63], 2048, False),
    ("c2_1048576", 1 << 20, 64, 1, "normal", [0, 63], 2048, False),
    ("c2_1009", 1009, 64, 1, "normal", [0, 1, 63], 0, False),
    ("c4", 1 << 20, 16, 3, "normal", [0, 15], 2048, True),
    ("c5_16777216", 1 << 24, 8, 4, "uniform", [0, 7], 2048, False),
    ("c5_134217728", 1 << 27, 1, 4, "uniform", [0], 2048, False),
]


def sample_indices(n: int, count: int) -> np.ndarray:
    if count == 0 or count >= n:
        return np.arange(n, dtype=np.int64)
    return np.sort(np.random.default_rng(n).choice(n, count, replace=False)).astype(np.int64)


def make_reference_vectors(ref):
    out = {"lengths": np.array(LENGTHS, dtype=np.int64)}
    strat = np.full(80001, 255, dtype=np.uint8)
    for n in range(2, 80001):
        strat[n] = ref.strategy(n)
    out["strategy"] = strat
    for n in LENGTHS:
        rng = np.random.default_rng(1000 + n)
        x = (rng.uniform(-1, 1, n) + 1j * rng.uniform(-1, 1, n)).astype(np.complex64)
        out[f"in_{n}"] = x
        out[f"fwd_{n}"] = ref.fft(x, inverse=False)
        out[f"inv_{n}"] = ref.fft(x, inverse=True)
    path = os.path.join(HERE, "reference_vectors.npz")
    np.savez_compressed(path, **out)
    print(f"wrote {path} ({os.path.getsize(path) / 1e6:.2f} MB, {len(LENGTHS)} lengths)")


def make_config_vectors(ref):
    out = {}
    threads = os.cpu_count() or 1
    for key, n, batch, seed, dist, rows, samples, grad in CONFIGS:
        x = O.fill_random(seed, n * batch, np.complex64, dist).reshape(batch, n)
        xr = np.ascontiguousarray(x[rows])
        yr = np.empty_like(xr)
        pool = O.ReferencePool(ref, n, min(threads, len(rows)))
        pool.run(xr, yr, inverse=grad)
        pool.close()
        if grad:
            yr = (yr.astype(np.complex128) * n).astype(np.complex64)
        idx = sample_indices(n, samples)
        out.update({f"{key}_n": np.int64(n), f"{key}_batch": np.int64(batch), f"{key}_seed": np.int64(seed),
                    f"{key}_dist": np.array(dist), f"{key}_rows": np.array(rows, dtype=np.int64),
                    f"{key}_idx": idx, f"{key}_out": np.ascontiguousarray(yr[:, idx]),
                    f"{key}_head": x.reshape(-1)[:8].copy(), f"{key}_inverse": np.int64(int(grad))})
        print(f"{key}: n={n} rows={len(rows)} samples={len(idx)}")
    out["keys"] = np.array([c[0] for c in CONFIGS])
    out["reference_build"] = np.array(ref.build_info())
    path = os.path.join(HERE, "config_vectors.npz")
    np.savez_compressed(path, **out)
    print(f"wrote {path} ({os.path.getsize(path) / 1e6:.2f} MB)")


def main():
    cmd = [os.path.join(ROOT, "oracle", "ref", "build_ref.sh")] + sys.argv[1:2]
    subprocess.run(cmd, check=True)
    ref = O.Reference()
    if ref.build_info() != "native x86_64":
        raise SystemExit("golden fixtures are generated from the native AVX2 build (x86-64)")
    make_reference_vectors(ref)
    make_config_vectors(ref)


if __name__ == "__main__":
    main()
