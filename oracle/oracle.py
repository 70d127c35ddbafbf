"""ctypes front end of the CPU oracle (fft_oracle.c) and of the compiled reference.

TEST INFRASTRUCTURE.  Only tests/, ``__graft_entry__.smoke()`` and the cpu_baseline /
reference legs of ``bench.py`` import this module, and only as the checker or as the timed
CPU baseline; the GPU library never does.

``fft`` / ``dft`` restate the reference's transform (foye_FFT.hpp:128-151: forward
exp(-2 pi i kn/N), inverse exp(+2 pi i kn/N) scaled by 1/N) in FP64 with long-double
twiddles.  ``fill_random`` generates the seeded inputs of every configuration without the GPU
library.  ``Reference`` wraps the reference's own C++ code when oracle/_ref/libfyref.so was
built by oracle/ref/build_ref.sh (natively with AVX2 on x86-64; elsewhere against the
portable intrinsics of oracle/ref/portable_intrin.h).
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")
REF_PATH = os.path.join(HERE, "_ref", "libfyref.so")

STRATEGY_NAMES = ("kernel_direct", "mix_radix", "rader", "bluestein", "DFT")

_lib = None


def build() -> str:
    """Compile fft_oracle.c (idempotent)."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB_PATH


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < os.path.getmtime(
                os.path.join(HERE, "fft_oracle.c")):
            build()
        L = ctypes.CDLL(LIB_PATH)
        sz, vp, i = ctypes.c_size_t, ctypes.c_void_p, ctypes.c_int
        for name in ("orc_is_directly_supported", "orc_mixed_is_processable", "orc_is_prime",
                     "orc_rader_is_processable", "orc_bluestein_is_processable", "orc_strategy"):
            getattr(L, name).argtypes = [sz]
            getattr(L, name).restype = i
        for name in ("orc_next_smooth", "orc_next_7smooth", "orc_find_primitive_root"):
            getattr(L, name).argtypes = [sz]
            getattr(L, name).restype = sz
        L.orc_power_mod.argtypes = [sz, sz, sz]
        L.orc_power_mod.restype = sz
        L.orc_fft.argtypes = [sz, i, vp, vp]
        L.orc_dft.argtypes = [sz, i, vp, vp]
        L.orc_dft_sampled.argtypes = [sz, i, vp, vp, sz, vp]
        L.orc_fft_batch.argtypes = [sz, sz, i, vp, vp, i, i]
        L.orc_fill_random.argtypes = [ctypes.c_uint64, i, i, sz, vp, i]
        L.orc_fill_random.restype = i
        for f in (L.orc_fft, L.orc_dft, L.orc_dft_sampled, L.orc_fft_batch):
            f.restype = i
        _lib = L
    return _lib


def strategy(n: int) -> int:
    return lib().orc_strategy(n)


def next_smooth(n: int) -> int:
    return lib().orc_next_smooth(n)


def next_7smooth(n: int) -> int:
    return lib().orc_next_7smooth(n)


def primitive_root(n: int) -> int:
    return lib().orc_find_primitive_root(n)


def _as_c128(x) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(x, dtype=np.complex128))


def fft(x, inverse: bool = False) -> np.ndarray:
    """FP64 transform along the last axis of x (any leading shape)."""
    x = _as_c128(x)
    n = x.shape[-1]
    y = np.empty_like(x)
    xf, yf = x.reshape(-1, n), y.reshape(-1, n)
    for b in range(xf.shape[0]):
        rc = lib().orc_fft(n, int(inverse), xf[b].ctypes.data, yf[b].ctypes.data)
        if rc:
            raise RuntimeError(f"orc_fft({n}) failed: {rc}")
    return y


def fft_batch(x, inverse: bool = False, threads: int = 1) -> np.ndarray:
    """Threaded FP64 transform of a (batch, n) complex128 or complex64 array."""
    x = np.ascontiguousarray(x)
    f32 = x.dtype == np.complex64
    if not f32:
        x = _as_c128(x)
    batch, n = x.shape
    y = np.empty_like(x)
    rc = lib().orc_fft_batch(n, batch, int(inverse), x.ctypes.data, y.ctypes.data, threads, int(f32))
    if rc:
        raise RuntimeError(f"orc_fft_batch({n}) failed: {rc}")
    return y


def dft(x, inverse: bool = False) -> np.ndarray:
    """Naive long-double DFT along the last axis (O(N^2): small N only)."""
    x = _as_c128(x)
    n = x.shape[-1]
    y = np.empty_like(x)
    xf, yf = x.reshape(-1, n), y.reshape(-1, n)
    for b in range(xf.shape[0]):
        lib().orc_dft(n, int(inverse), xf[b].ctypes.data, yf[b].ctypes.data)
    return y


def dft_sampled(x, idx, inverse: bool = False) -> np.ndarray:
    """Long-double DFT of one transform x at output indices idx (O(N * len(idx)))."""
    x = _as_c128(x)
    idx = np.ascontiguousarray(np.asarray(idx, dtype=np.int64))
    out = np.empty(idx.shape[0], dtype=np.complex128)
    lib().orc_dft_sampled(x.shape[-1], int(inverse), x.ctypes.data, idx.ctypes.data, idx.shape[0],
                          out.ctypes.data)
    return out


def fill_random(seed: int, n: int, dtype=np.complex64, dist: str = "normal", threads: int | None = None) -> np.ndarray:
    """n seeded complex values (dist "uniform": re, im in [-1, 1); "normal": N(0, 1) each),
    identical to the GPU library's fyg_fill_random for the same (seed, dist, dtype)."""
    dtype = np.dtype(dtype)
    if dtype not in (np.complex64, np.complex128):
        raise ValueError("dtype must be complex64 or complex128")
    if dist not in ("uniform", "normal"):
        raise ValueError("dist must be 'uniform' or 'normal'")
    out = np.empty(int(n), dtype=dtype)
    rc = lib().orc_fill_random(int(seed), 0 if dist == "uniform" else 1, int(dtype == np.complex64), int(n),
                               out.ctypes.data, int(threads or os.cpu_count() or 1))
    if rc:
        raise RuntimeError("orc_fill_random failed")
    return out


def rel_l2(a, b) -> float:
    a = np.asarray(a, dtype=np.complex128)
    b = np.asarray(b, dtype=np.complex128)
    d = np.linalg.norm((a - b).ravel())
    r = np.linalg.norm(b.ravel())
    return float(d / r) if r else float(d)


class Reference:
    """The reference's own FFT1D_C2C_invoker (foye_FFT.hpp:89-185) from oracle/_ref/libfyref.so."""

    def __init__(self, path: str = REF_PATH):
        L = ctypes.CDLL(path)
        sz, vp, i = ctypes.c_size_t, ctypes.c_void_p, ctypes.c_int
        L.fyref_strategy.argtypes = [sz]
        L.fyref_runnable.argtypes = [sz]
        L.fyref_fft.argtypes = [sz, i, vp, vp]
        L.fyref_plan_create.argtypes = [sz]
        L.fyref_plan_create.restype = vp
        L.fyref_plan_destroy.argtypes = [vp]
        L.fyref_plan_execute.argtypes = [vp, i, vp, vp]
        L.fyref_batch.argtypes = [sz, sz, i, vp, vp, i, ctypes.POINTER(ctypes.c_double),
                                  ctypes.POINTER(ctypes.c_double)]
        L.fyref_pool_create.argtypes = [sz, i, ctypes.POINTER(ctypes.c_double)]
        L.fyref_pool_create.restype = vp
        L.fyref_pool_run.argtypes = [vp, sz, i, vp, vp, ctypes.POINTER(ctypes.c_double)]
        L.fyref_pool_destroy.argtypes = [vp]
        L.fyref_build_info.restype = ctypes.c_char_p
        self.L = L
        self.path = path

    def build_info(self) -> str:
        """'native x86_64', 'emulated aarch64' or 'emulated x86_64'."""
        return self.L.fyref_build_info().decode()

    @staticmethod
    def available(path: str = REF_PATH) -> bool:
        return os.path.exists(path)

    def strategy(self, n: int) -> int:
        return self.L.fyref_strategy(n)

    def runnable(self, n: int) -> bool:
        return bool(self.L.fyref_runnable(n))

    def fft(self, x, inverse: bool = False) -> np.ndarray:
        x = np.ascontiguousarray(np.asarray(x, dtype=np.complex64))
        n = x.shape[-1]
        y = np.zeros_like(x)
        xf, yf = x.reshape(-1, n), y.reshape(-1, n)
        for b in range(xf.shape[0]):
            if self.L.fyref_fft(n, int(inverse), xf[b].ctypes.data, yf[b].ctypes.data):
                raise RuntimeError(f"reference cannot run length {n}")
        return y

    def batch(self, x, inverse: bool = False, threads: int = 1):
        """Threaded batch; returns (output, exec_seconds, plan_seconds)."""
        x = np.ascontiguousarray(np.asarray(x, dtype=np.complex64))
        batch, n = x.shape
        y = np.zeros_like(x)
        t, tp = ctypes.c_double(), ctypes.c_double()
        if self.L.fyref_batch(n, batch, int(inverse), x.ctypes.data, y.ctypes.data, threads,
                              ctypes.byref(t), ctypes.byref(tp)):
            raise RuntimeError(f"reference cannot run length {n}")
        return y, t.value, tp.value


class ReferencePool:
    """`threads` worker threads with one reference plan of length n each (plans hold mutable
    workspace and are never shared); ``run`` splits a contiguous batch over them."""

    def __init__(self, ref: Reference, n: int, threads: int):
        t = ctypes.c_double()
        self.ref, self.n = ref, int(n)
        self.h = ref.L.fyref_pool_create(self.n, int(threads), ctypes.byref(t))
        if not self.h:
            raise RuntimeError(f"reference cannot run length {n}")
        self.plan_seconds = t.value

    def run(self, x: np.ndarray, y: np.ndarray, inverse: bool = False) -> float:
        """y = transform of x ((batch, n) complex64, C-contiguous); returns the wall seconds."""
        assert x.dtype == np.complex64 and y.dtype == np.complex64 and x.flags.c_contiguous and y.flags.c_contiguous
        assert x.shape[-1] == self.n and x.size == y.size
        t = ctypes.c_double()
        self.ref.L.fyref_pool_run(self.h, x.size // self.n, int(inverse), x.ctypes.data, y.ctypes.data,
                                  ctypes.byref(t))
        return t.value

    def close(self):
        if self.h:
            self.ref.L.fyref_pool_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
