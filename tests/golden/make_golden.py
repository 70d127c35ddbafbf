"""Generate tests/golden/reference_vectors.npz from the reference's own C++ FFT.

Runs only where the reference checkout and an x86-64 AVX2 host are available (it builds
oracle/_ref/libfyref.so with oracle/ref/build_ref.sh).  The committed .npz is what the tests
read; this script is how it was made:

    python tests/golden/make_golden.py [REFERENCE_DIR]

Contents (complex64 arrays, interleaved like the reference's float* buffers):
  in_<n>   input, seed 1000+n, re/im i.i.d. uniform[-1, 1]
  fwd_<n>  FFT1D_C2C_invoker{n}.dispatch<false>(in)   (foye_FFT.hpp:128-151)
  inv_<n>  FFT1D_C2C_invoker{n}.dispatch<true>(in)    (scaled by 1/n)
  strategy uint8[80001]: FFT1D_C2C_invoker::acquired_execution_strategy(n) for n in [0, 80000]
           (foye_FFT.hpp:162-184; entries 0 and 1 are outside the reference's range and hold 255)
  lengths  the n values above
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


def main():
    ref_dir = sys.argv[1] if len(sys.argv) > 1 else "/root/reference"
    subprocess.run([os.path.join(ROOT, "oracle", "ref", "build_ref.sh"), ref_dir], check=True)
    ref = O.Reference()
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


if __name__ == "__main__":
    main()
