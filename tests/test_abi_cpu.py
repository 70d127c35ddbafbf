"""CPU-side checks of the C ABI: the library loads, exports every symbol include/fygpu.h
declares, and its host logic (strategy selection, seeded generator, argument validation)
behaves.  No GPU compute calls."""
import ctypes
import os
import re
import shutil
import subprocess

import numpy as np
import pytest

import fyfft_gb300 as fg
from oracle import oracle as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HERE = os.path.join(ROOT, "tests")
INCLUDE = os.path.join(ROOT, "include")


@pytest.fixture(scope="module", autouse=True)
def built():
    fg.build.build()


def declared_symbols():
    src = open(os.path.join(ROOT, "include", "fygpu.h")).read()
    return sorted(set(re.findall(r"\b(fyg_[a-z_0-9]+)\s*\(", src)))


def test_header_declarations_match_python_list():
    assert declared_symbols() == sorted(fg.EXPORTED_SYMBOLS)


def test_library_exports_every_declared_symbol():
    L = fg.lib()
    for name in declared_symbols():
        assert hasattr(L, name), name


def test_strategy_parity_with_reference_everywhere():
    d = np.load(os.path.join(ROOT, "tests", "golden", "reference_vectors.npz"))
    s = d["strategy"]
    L = fg.lib()
    mism = [n for n in range(2, 80001) if L.fyg_strategy(n) != s[n]]
    assert mism == []
    assert L.fyg_strategy(1) == -1


def test_gpu_strategy_never_dft():
    L = fg.lib()
    for n in list(range(2, 3000)) + [39063, 65537, 100003, 131074, 999983]:
        assert L.fyg_gpu_strategy(n) in (0, 1, 2, 3)
    assert L.fyg_gpu_strategy(999983) == 3 and L.fyg_gpu_strategy(65537) == 2
    assert L.fyg_gpu_strategy(1009) == 2 and L.fyg_gpu_strategy(2520) == 1


def test_split_lengths_report_rader():
    """N = m p (m <= 8, p prime with p - 1 13-smooth, N > 8192) runs m Rader transforms; other
    composites stay Bluestein."""
    L = fg.lib()
    for n in (131074, 196611, 24578, 73734, 98312, 53767, 17285, 13828):
        assert L.fyg_gpu_strategy(n) == 2, n
    # 131078 = 2 x 65539 (65538 not 13-smooth), 6914 = 2 x 3457 (<= 8192), 9 x 12289 (m > 8)
    for n in (131078, 6914, 9 * 12289):
        assert L.fyg_gpu_strategy(n) == 3, n


def test_generator_is_counter_based_and_distributed():
    a = fg.fill_random(5, 1 << 18, np.complex64, "uniform")
    b = fg.fill_random(5, 1 << 10, np.complex64, "uniform")
    assert np.array_equal(a[: 1 << 10], b)
    assert -1 <= a.real.min() and a.real.max() < 1 and abs(a.real.mean()) < 1e-2
    c = fg.fill_random(6, 1 << 18, np.complex128, "normal")
    assert abs(c.real.std() - 1) < 1e-2 and abs(c.imag.mean()) < 1e-2
    assert not np.array_equal(fg.fill_random(7, 16), fg.fill_random(8, 16))


def test_plan_create_rejects_bad_arguments_without_gpu():
    L = fg.lib()
    h = ctypes.c_void_p()
    assert L.fyg_plan_create(0, 0, 1, 0, ctypes.byref(h)) == 1        # invalid length
    assert L.fyg_plan_create(16, 5, 1, 0, ctypes.byref(h)) == 7        # bad dtype
    assert L.fyg_plan_create(16, 0, 0, 0, ctypes.byref(h)) == 7        # zero batch
    assert b"length" in L.fyg_last_error_string() or b"batch" in L.fyg_last_error_string()
    assert L.fyg_execute(None, None, None, 1, None) == 2


def test_oracle_and_library_agree_on_reference_strategy_samples():
    for n in (4096, 2520, 59049, 117649, 1009, 39062, 39063, 65537):
        assert fg.lib().fyg_strategy(n) == O.strategy(n)


@pytest.mark.skipif(shutil.which("gcc") is None, reason="needs gcc")
def test_c_abi_header_is_plain_c99(tmp_path):
    # the boundary header uses only C types: it compiles as strict C99
    src = tmp_path / "h.c"
    src.write_text('#include "fygpu.h"\nint main(void) { return FYG_OK; }\n')
    r = subprocess.run(["gcc", "-std=c99", "-Wall", "-Wextra", "-pedantic", "-Werror", "-I", INCLUDE,
                        "-fsyntax-only", str(src)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


@pytest.mark.skipif(shutil.which("g++") is None, reason="needs g++")
def test_dropin_header_example_links(tmp_path):
    # the reference-API example program compiles against foye_FFT_gpu.hpp and links the library
    exe = tmp_path / "dropin"
    r = subprocess.run(["g++", "-std=c++17", "-I", INCLUDE, os.path.join(HERE, "cpp", "dropin_example.cpp"),
                        "-L", os.path.dirname(fg.LIB_PATH), "-lfygpu", f"-Wl,-rpath,{os.path.dirname(fg.LIB_PATH)}",
                        "-o", str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
