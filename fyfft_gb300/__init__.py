"""fyfft_gb300 -- GB300-native (sm_103a) 1D complex FFT with fyFFT's plan/execute interface.

The Python surface mirrors the reference's C++ class ``fy::fft::FFT1D_C2C_invoker``
(foye_FFT.hpp:89-185):

    inv = FFT1D_C2C_invoker(N)                   # plan (strategy, tables, scratch) once
    inv.dispatch(False, x, y)                   # forward  exp(-2 pi i kn/N)
    inv.dispatch(True, x, y)                    # inverse  exp(+2 pi i kn/N) / N
    FFT1D_C2C_invoker.acquired_execution_strategy(N)   # the reference's strategy for N

and adds batching, complex128, an adjoint entry point and an uneven-length batch.  Every call
goes through the C ABI of libfygpu.so (include/fygpu.h) into hand-written CUDA kernels; there
is no CPU fallback: without the built library (``fyfft_gb300.build.build()``) importing the
ABI raises.
"""
from __future__ import annotations

import ctypes
import enum
import os

import numpy as np

from . import build as _build_mod

LIB_PATH = _build_mod.LIB

FYG_OK = 0
FYG_C32, FYG_C64 = 0, 1
FYG_FORWARD, FYG_INVERSE = 1, -1
FYG_FLAG_CONV_FP64, FYG_FLAG_CONV_FP32, FYG_FLAG_NO_L2_CHUNK = 1, 2, 4
FYG_FLAG_SMALL_TILES, FYG_FLAG_AUTOTUNED, FYG_FLAG_GENERIC_KERNELS = 8, 16, 32
FYG_FLAG_WIDE_TILES, FYG_FLAG_TMA_LOADS, FYG_FLAG_NO_TMA_LOADS = 64, 128, 256
FYG_FLAG_BATCH_BRANCHES = 512

# every symbol include/fygpu.h declares
EXPORTED_SYMBOLS = (
    "fyg_plan_create", "fyg_plan_create_ex", "fyg_plan_create_layout", "fyg_autotune", "fyg_plan_destroy", "fyg_execute", "fyg_execute_adjoint", "fyg_strategy",
    "fyg_gpu_strategy", "fyg_plan_info", "fyg_plan_launches", "fyg_plan_describe", "fyg_plan_profile",
    "fyg_plan_profile_read", "fyg_batch_create", "fyg_batch_autotune", "fyg_batch_destroy",
    "fyg_batch_execute", "fyg_batch_execute_plain", "fyg_batch_status", "fyg_batch_inject_stall",
    "fyg_execute_noalloc", "fyg_last_error_string",
    "fyg_fill_random",
    "fyg_fill_random_device", "fyg_version", "fyg_plan_cache_stats", "fyg_plan_cache_clear",
    "fyg_partition", "fyg_multi_create", "fyg_multi_shards", "fyg_multi_execute", "fyg_multi_execute_device",
    "fyg_multi_synchronize", "fyg_multi_destroy", "fyg_fill_random_at", "fyg_fill_random_device_at",
    "fyg_plan_status", "fyg_execute_async", "fyg_batch_create_ex", "fyg_plan_join", "fyg_device_signature",
    "fyg_plan_schedule",
)


class FFT_execution_strategy(enum.IntEnum):
    """foye_FFT.hpp:153-160"""
    kernel_direct = 0
    mix_radix = 1
    rader = 2
    bluestein = 3
    DFT = 4


class FygError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"fygpu error {code}: {msg}")
        self.code = code


_lib = None


def lib() -> ctypes.CDLL:
    """The loaded libfygpu.so (raises if it was not built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is missing: build it with fyfft_gb300.build.build()")
        L = ctypes.CDLL(LIB_PATH)
        sz, vp, i, d, u64 = ctypes.c_size_t, ctypes.c_void_p, ctypes.c_int, ctypes.c_double, ctypes.c_uint64
        L.fyg_plan_create.argtypes = [sz, i, sz, i, ctypes.POINTER(vp)]
        L.fyg_plan_create_ex.argtypes = [sz, i, sz, i, sz, sz, ctypes.POINTER(vp)]
        L.fyg_plan_create_layout.argtypes = [sz, i, sz, sz, sz, i, ctypes.POINTER(vp)]
        L.fyg_autotune.argtypes = [sz, i, sz, ctypes.c_char_p, ctypes.POINTER(d)]
        L.fyg_plan_destroy.argtypes = [vp]
        L.fyg_execute.argtypes = [vp, vp, vp, i, vp]
        L.fyg_execute_async.argtypes = [vp, vp, vp, i, vp]
        L.fyg_plan_join.argtypes = [vp, vp]
        L.fyg_device_signature.argtypes = [ctypes.c_char_p, sz]
        L.fyg_execute_adjoint.argtypes = [vp, vp, vp, d, vp]
        L.fyg_strategy.argtypes = [sz]
        L.fyg_gpu_strategy.argtypes = [sz]
        L.fyg_plan_info.argtypes = [vp, ctypes.POINTER(sz), ctypes.POINTER(i), ctypes.POINTER(i)]
        L.fyg_plan_schedule.argtypes = [sz, i, i, ctypes.POINTER(i), ctypes.POINTER(sz), ctypes.POINTER(i),
                                        ctypes.POINTER(i), i, ctypes.POINTER(i)]
        L.fyg_plan_launches.argtypes = [vp, ctypes.POINTER(i)]
        L.fyg_plan_describe.argtypes = [vp, ctypes.c_char_p, sz]
        L.fyg_plan_profile.argtypes = [vp, i]
        L.fyg_plan_profile_read.argtypes = [vp, ctypes.POINTER(d), ctypes.POINTER(ctypes.c_int64),
                                            ctypes.POINTER(ctypes.c_int64), i, ctypes.POINTER(i)]
        L.fyg_batch_create.argtypes = [ctypes.POINTER(sz), sz, i, i, ctypes.POINTER(vp)]
        L.fyg_batch_create_ex.argtypes = [ctypes.POINTER(sz), sz, i, i, i, sz, i, i, ctypes.POINTER(vp)]
        L.fyg_batch_autotune.argtypes = [ctypes.POINTER(sz), sz, i, ctypes.c_char_p, ctypes.POINTER(d)]
        L.fyg_batch_destroy.argtypes = [vp]
        L.fyg_batch_execute.argtypes = [vp, vp, vp, vp, i, vp]
        L.fyg_batch_execute_plain.argtypes = [vp, vp, vp, i, vp]
        L.fyg_batch_status.argtypes = [vp, vp]
        L.fyg_batch_inject_stall.argtypes = [vp, i, i]
        L.fyg_execute_noalloc.argtypes = [sz, sz, i, i, vp, vp, vp]
        L.fyg_last_error_string.restype = ctypes.c_char_p
        L.fyg_fill_random.argtypes = [u64, i, i, sz, vp]
        L.fyg_fill_random_device.argtypes = [u64, i, i, sz, vp, vp]
        L.fyg_fill_random_at.argtypes = [u64, i, i, sz, sz, vp]
        L.fyg_fill_random_device_at.argtypes = [u64, i, i, sz, sz, vp, vp]
        L.fyg_version.restype = ctypes.c_char_p
        L.fyg_plan_cache_stats.argtypes = [ctypes.POINTER(sz), ctypes.POINTER(sz), ctypes.POINTER(u64),
                                           ctypes.POINTER(u64)]
        L.fyg_partition.argtypes = [ctypes.POINTER(sz), sz, i, ctypes.POINTER(sz)]
        L.fyg_plan_status.argtypes = [vp, vp, ctypes.POINTER(i)]
        L.fyg_multi_create.argtypes = [sz, i, sz, i, ctypes.POINTER(i), i, ctypes.POINTER(vp)]
        L.fyg_multi_shards.argtypes = [vp, ctypes.POINTER(i), ctypes.POINTER(sz)]
        L.fyg_multi_execute.argtypes = [vp, vp, vp, i]
        L.fyg_multi_execute_device.argtypes = [vp, ctypes.POINTER(vp), ctypes.POINTER(vp), i]
        L.fyg_multi_synchronize.argtypes = [vp]
        L.fyg_multi_destroy.argtypes = [vp]
        _lib = L
    return _lib


def autotune(length: int, dtype="complex64", batch: int = 1, cache_path: str | None = None) -> float:
    """Time the schedule candidates of one length on the current device and cache the fastest.

    Plans created afterwards with flags=FYG_FLAG_AUTOTUNED use it.  Returns the winner's
    milliseconds per forward batch."""
    code = FYG_C32 if str(dtype).endswith("complex64") else FYG_C64
    ms = ctypes.c_double()
    path = cache_path.encode() if cache_path else None
    check(lib().fyg_autotune(int(length), code, int(batch), path, ctypes.byref(ms)))
    return ms.value


def autotune_batch(lengths, dtype="complex64", cache_path: str | None = None) -> float:
    """Time the uneven-batch option sets for this length sequence and cache the fastest; create
    the batch with flags=FYG_FLAG_AUTOTUNED to use it.  Returns the winner's milliseconds."""
    lens = [int(n) for n in lengths]
    arr = (ctypes.c_size_t * len(lens))(*lens)
    code = FYG_C32 if str(dtype).endswith("complex64") else FYG_C64
    ms = ctypes.c_double()
    path = cache_path.encode() if cache_path else None
    check(lib().fyg_batch_autotune(arr, len(lens), code, path, ctypes.byref(ms)))
    return ms.value


def device_signature() -> str:
    """The current device's key in autotune caches: name|SMs|compute capability|driver."""
    buf = ctypes.create_string_buffer(512)
    check(lib().fyg_device_signature(buf, len(buf)))
    return buf.value.decode()


def plan_cache_stats() -> dict:
    """Entries and device bytes of the process-wide table cache, and its hit / miss counts."""
    e, b, h, m = ctypes.c_size_t(), ctypes.c_size_t(), ctypes.c_uint64(), ctypes.c_uint64()
    check(lib().fyg_plan_cache_stats(ctypes.byref(e), ctypes.byref(b), ctypes.byref(h), ctypes.byref(m)))
    return {"entries": e.value, "bytes": b.value, "hits": h.value, "misses": m.value}


def plan_schedule(length: int, dtype="complex64", flags: int = 0) -> dict:
    """The schedule a plan of `length` gets, computed on the host (no GPU needed): GPU strategy
    (as FFT1D_C2C_invoker.info() reports it), algorithm length L, split factor m and the pass
    radices of the length-L transform."""
    code = {"complex64": 0, "complex128": 1}[str(np.dtype(dtype))]
    st, L, m, npass = ctypes.c_int(), ctypes.c_size_t(), ctypes.c_int(), ctypes.c_int()
    rad = (ctypes.c_int * 16)()
    check(lib().fyg_plan_schedule(int(length), code, int(flags), ctypes.byref(st), ctypes.byref(L), ctypes.byref(m),
                                  rad, 16, ctypes.byref(npass)))
    return {"gpu_strategy": st.value, "conv_length": L.value, "split_m": m.value,
            "pass_radices": list(rad[:min(npass.value, 16)])}


def plan_cache_clear() -> None:
    """Free the cached tables that no live plan uses."""
    check(lib().fyg_plan_cache_clear())


def check(rc: int) -> None:
    if rc != FYG_OK:
        raise FygError(rc, lib().fyg_last_error_string().decode())


def _stream_handle(stream) -> int | None:
    if stream is None:
        try:
            import torch
            if torch.cuda.is_available():
                return torch.cuda.current_stream().cuda_stream
        except ImportError:
            pass
        return None
    return getattr(stream, "cuda_stream", stream)


def _buffer_ptr(x):
    """(pointer, n_complex, dtype code, on_device) of a torch tensor or numpy array."""
    if isinstance(x, np.ndarray):
        if not x.flags.c_contiguous:
            raise ValueError("arrays must be C-contiguous")
        if x.dtype == np.complex64:
            return x.ctypes.data, x.size, FYG_C32, False
        if x.dtype == np.complex128:
            return x.ctypes.data, x.size, FYG_C64, False
        if x.dtype == np.float32:
            return x.ctypes.data, x.size // 2, FYG_C32, False
        if x.dtype == np.float64:
            return x.ctypes.data, x.size // 2, FYG_C64, False
        raise TypeError(f"unsupported dtype {x.dtype}")
    import torch
    if not x.is_contiguous():
        raise ValueError("tensors must be contiguous")
    dt = {torch.complex64: (FYG_C32, 1), torch.complex128: (FYG_C64, 1),
          torch.float32: (FYG_C32, 2), torch.float64: (FYG_C64, 2)}.get(x.dtype)
    if dt is None:
        raise TypeError(f"unsupported dtype {x.dtype}")
    return x.data_ptr(), x.numel() // dt[1], dt[0], x.is_cuda


def fill_random(seed: int, n_complex: int, dtype=np.complex64, dist: str = "uniform", first: int = 0) -> np.ndarray:
    """Seeded synthetic data on the host (uniform re/im in [-1, 1) or standard normal):
    elements [first, first + n_complex) of stream `seed`."""
    out = np.empty(n_complex, dtype=dtype)
    code = FYG_C32 if np.dtype(dtype) == np.complex64 else FYG_C64
    check(lib().fyg_fill_random_at(seed, 0 if dist == "uniform" else 1, code, int(first), n_complex, out.ctypes.data))
    return out


def fill_random_device(seed: int, out, dist: str = "uniform", stream=None, first: int = 0) -> None:
    """Same stream as fill_random, generated on the GPU into a CUDA tensor."""
    ptr, n, code, _ = _buffer_ptr(out)
    check(lib().fyg_fill_random_device_at(seed, 0 if dist == "uniform" else 1, code, int(first), n, ptr,
                                          _stream_handle(stream)))


class FFT1D_C2C_invoker:
    """GPU plan for `batch` contiguous transforms of length N (foye_FFT.hpp:89-185).

    dtype: "complex64" (the reference's float buffers) or "complex128".
    """

    FFT_execution_strategy = FFT_execution_strategy

    def __init__(self, length: int, dtype="complex64", batch: int = 1, flags: int = 0,
                 max_pass_radix: int = 0, conv_length: int = 0, idist: int = 0, odist: int = 0):
        self.N = int(length)
        self.batch = int(batch)
        self.idist = int(idist) or self.N
        self.odist = int(odist) or self.N
        self.dtype_code = FYG_C32 if str(dtype).endswith("complex64") else FYG_C64
        h = ctypes.c_void_p()
        if idist or odist:
            check(lib().fyg_plan_create_layout(self.N, self.dtype_code, self.batch, int(idist), int(odist), flags,
                                               ctypes.byref(h)))
        elif max_pass_radix or conv_length:
            check(lib().fyg_plan_create_ex(self.N, self.dtype_code, self.batch, flags, int(max_pass_radix),
                                           int(conv_length), ctypes.byref(h)))
        else:
            check(lib().fyg_plan_create(self.N, self.dtype_code, self.batch, flags, ctypes.byref(h)))
        self._h = h

    def close(self):
        if getattr(self, "_h", None):
            lib().fyg_plan_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _io(self, x, y):
        px, nx, dx, _ = _buffer_ptr(x)
        py, ny, dy, _ = _buffer_ptr(y)
        need_x = (self.batch - 1) * self.idist + self.N
        need_y = (self.batch - 1) * self.odist + self.N
        if dx != self.dtype_code or dy != self.dtype_code:
            raise TypeError("buffer dtype does not match the plan")
        if nx < need_x or ny < need_y:
            raise ValueError(f"buffers hold {nx}/{ny} complex elements, plan needs {need_x}/{need_y}")
        return px, py

    def dispatch(self, invert: bool, input, output, stream=None, blocking: bool = True) -> None:
        """foye_FFT.hpp:128-151: dispatch<invert>(input, output).  blocking=False with host
        buffers returns after enqueueing (fyg_execute_async): call join(stream) and synchronize
        `stream` (or the device) before reading `output`."""
        px, py = self._io(input, output)
        fn = lib().fyg_execute if blocking else lib().fyg_execute_async
        check(fn(self._h, px, py, FYG_INVERSE if invert else FYG_FORWARD, _stream_handle(stream)))

    def join(self, stream=None) -> None:
        """Make `stream` wait for the copy-outs of asynchronous host dispatches."""
        check(lib().fyg_plan_join(self._h, _stream_handle(stream)))

    def forward(self, input, output, stream=None) -> None:
        self.dispatch(False, input, output, stream)

    def backward(self, input, output, stream=None) -> None:
        self.dispatch(True, input, output, stream)

    def adjoint(self, g, output, scale: float = 1.0, stream=None) -> None:
        """output = scale * F^H g (= scale * N * backward(g))."""
        px, py = self._io(g, output)
        check(lib().fyg_execute_adjoint(self._h, px, py, float(scale), _stream_handle(stream)))

    def status(self, stream=None) -> int:
        """Device error bits recorded by the plan's kernels since the last call (0 = none)."""
        st = ctypes.c_int()
        check(lib().fyg_plan_status(self._h, _stream_handle(stream), ctypes.byref(st)))
        return st.value

    def info(self):
        L, P, S = ctypes.c_size_t(), ctypes.c_int(), ctypes.c_int()
        check(lib().fyg_plan_info(self._h, ctypes.byref(L), ctypes.byref(P), ctypes.byref(S)))
        return {"conv_length": L.value, "passes": P.value, "gpu_strategy": S.value}

    def describe(self) -> list[str]:
        """One line per forward pass: kernel kind, tile shape and fusions."""
        buf = ctypes.create_string_buffer(8192)
        check(lib().fyg_plan_describe(self._h, buf, len(buf)))
        return buf.value.decode().splitlines()

    def launches(self) -> int:
        n = ctypes.c_int()
        check(lib().fyg_plan_launches(self._h, ctypes.byref(n)))
        return n.value

    def profile(self, enable: bool = True) -> None:
        check(lib().fyg_plan_profile(self._h, int(enable)))

    def profile_read(self):
        """[(total_ms, launches, bytes_per_launch)] per forward pass (synchronizes)."""
        m = 32
        ms = (ctypes.c_double * m)()
        ln = (ctypes.c_int64 * m)()
        by = (ctypes.c_int64 * m)()
        n = ctypes.c_int()
        check(lib().fyg_plan_profile_read(self._h, ms, ln, by, m, ctypes.byref(n)))
        return [(ms[i], ln[i], by[i]) for i in range(min(n.value, m))]

    @staticmethod
    def acquired_execution_strategy(length: int) -> FFT_execution_strategy:
        """foye_FFT.hpp:162-184 (the reference's choice, reported unchanged)."""
        s = lib().fyg_strategy(int(length))
        if s < 0:
            raise ValueError("length must be >= 2")
        return FFT_execution_strategy(s)

    @staticmethod
    def gpu_execution_strategy(length: int) -> FFT_execution_strategy:
        """The strategy this library runs (never DFT)."""
        return FFT_execution_strategy(lib().fyg_gpu_strategy(int(length)))


class UnevenBatch:
    """Many transforms of different lengths packed back to back, run by one persistent kernel."""

    def __init__(self, lengths, dtype="complex64", flags: int = 0, form=None, split: int = 0, radix_cap: int = 0,
                 single_tile_kb: int = 0):
        """form None: by flags (the tuner's choice with FYG_FLAG_AUTOTUNED); 0 persistent kernel,
        1 graph branches, 2 persistent up to `split` and branches above (fyg_batch_create_ex)."""
        self.lengths = [int(n) for n in lengths]
        self.dtype_code = FYG_C32 if str(dtype).endswith("complex64") else FYG_C64
        arr = (ctypes.c_size_t * len(self.lengths))(*self.lengths)
        h = ctypes.c_void_p()
        if form is None:
            check(lib().fyg_batch_create(arr, len(self.lengths), self.dtype_code, flags, ctypes.byref(h)))
        else:
            check(lib().fyg_batch_create_ex(arr, len(self.lengths), self.dtype_code, flags, int(form), int(split),
                                            int(radix_cap), int(single_tile_kb), ctypes.byref(h)))
        self._h = h
        self.offsets = np.concatenate([[0], np.cumsum(self.lengths)[:-1]]).astype(np.int64)
        self.total = int(sum(self.lengths))

    def close(self):
        if getattr(self, "_h", None):
            lib().fyg_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def execute(self, x, y, invert: bool = False, offsets_dev=None, stream=None) -> None:
        px, _, _, _ = _buffer_ptr(x)
        py, _, _, _ = _buffer_ptr(y)
        po = None
        if offsets_dev is not None:
            po = offsets_dev.data_ptr() if hasattr(offsets_dev, "data_ptr") else int(offsets_dev)
        check(lib().fyg_batch_execute(self._h, px, py, po, FYG_INVERSE if invert else FYG_FORWARD,
                                      _stream_handle(stream)))

    def status(self, stream=None) -> int:
        """Synchronizes and returns the device status of the last execute (0 = OK)."""
        return lib().fyg_batch_status(self._h, _stream_handle(stream))

    def inject_stall(self, enable: bool = True, timeout_ms: int = 200) -> None:
        """Test hook: make a pass dependency unreachable so the next execute times out."""
        check(lib().fyg_batch_inject_stall(self._h, int(enable), timeout_ms))

    def execute_plain(self, x, y, invert: bool = False, stream=None) -> None:
        px, _, _, _ = _buffer_ptr(x)
        py, _, _, _ = _buffer_ptr(y)
        check(lib().fyg_batch_execute_plain(self._h, px, py, FYG_INVERSE if invert else FYG_FORWARD,
                                            _stream_handle(stream)))


def partition(batch, parts: int) -> list[int]:
    """Contiguous shards of near-equal cost: bounds[0..parts] (fyg_partition).  `batch` is a
    count (uniform batch) or a sequence of transform lengths (cost n log2 n each)."""
    bounds = (ctypes.c_size_t * (parts + 1))()
    if isinstance(batch, int):
        check(lib().fyg_partition(None, batch, int(parts), bounds))
    else:
        lens = [int(n) for n in batch]
        arr = (ctypes.c_size_t * max(len(lens), 1))(*lens)
        check(lib().fyg_partition(arr, len(lens), int(parts), bounds))
    return list(bounds)


class MultiDevicePlan:
    """`batch` transforms of length N sharded over `devices` (a device may repeat): one plan and
    stream per shard, no collective (fyg_multi_*)."""

    def __init__(self, length: int, dtype="complex64", batch: int = 1, devices=(0,), flags: int = 0):
        self.N, self.batch = int(length), int(batch)
        self.dtype_code = FYG_C32 if str(dtype).endswith("complex64") else FYG_C64
        devs = (ctypes.c_int * len(devices))(*[int(d) for d in devices])
        h = ctypes.c_void_p()
        check(lib().fyg_multi_create(self.N, self.dtype_code, self.batch, flags, devs, len(devices), ctypes.byref(h)))
        self._h = h
        nd = ctypes.c_int()
        b = (ctypes.c_size_t * (len(devices) + 1))()
        check(lib().fyg_multi_shards(h, ctypes.byref(nd), b))
        self.devices = list(devices)
        self.bounds = list(b)

    def close(self):
        if getattr(self, "_h", None):
            lib().fyg_multi_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def execute(self, x: np.ndarray, y: np.ndarray, invert: bool = False) -> None:
        """Host arrays holding the whole batch; returns when y is complete."""
        px, nx, dx, _ = _buffer_ptr(x)
        py, ny, dy, _ = _buffer_ptr(y)
        if dx != self.dtype_code or dy != self.dtype_code or nx < self.N * self.batch or ny < self.N * self.batch:
            raise ValueError("buffers do not match the plan")
        check(lib().fyg_multi_execute(self._h, px, py, FYG_INVERSE if invert else FYG_FORWARD))

    def execute_device(self, xs, ys, invert: bool = False) -> None:
        """Per-shard device tensors (shard i on devices[i]); asynchronous."""
        ins = (ctypes.c_void_p * len(xs))(*[_buffer_ptr(t)[0] for t in xs])
        outs = (ctypes.c_void_p * len(ys))(*[_buffer_ptr(t)[0] for t in ys])
        check(lib().fyg_multi_execute_device(self._h, ins, outs, FYG_INVERSE if invert else FYG_FORWARD))

    def synchronize(self) -> None:
        check(lib().fyg_multi_synchronize(self._h))


_plan_cache: dict = {}


def fft(x, inverse: bool = False, stream=None):
    """Transform along the last axis of a contiguous CUDA tensor (complex64 or complex128)."""
    import torch
    n = x.shape[-1]
    batch = x.numel() // n
    key = (n, batch, x.dtype, x.device)
    plan = _plan_cache.get(key)
    if plan is None:
        plan = FFT1D_C2C_invoker(n, "complex64" if x.dtype == torch.complex64 else "complex128", batch)
        _plan_cache[key] = plan
    y = torch.empty_like(x)
    plan.dispatch(inverse, x.contiguous(), y, stream)
    return y
