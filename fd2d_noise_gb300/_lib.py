"""ctypes binding of libfd2d.so (include/fd2d.h).

The library is built in-tree by :mod:`fd2d_noise_gb300.build`.  There is no
fallback: if the shared library is missing or fails to load, importing the
solvers raises, and every solve runs on the GPU through this library.
"""
from __future__ import annotations

import ctypes
import os
import threading

from .config import FD2DConfig, FD2DSizes

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libfd2d.so")

FD2D_OK = 0
STATUS_NAMES = {
    0: "FD2D_OK", 1: "FD2D_ERR_ARG", 2: "FD2D_ERR_SHAPE", 3: "FD2D_ERR_ORDER",
    4: "FD2D_ERR_OOM", 5: "FD2D_ERR_CUDA", 6: "FD2D_ERR_TIMEOUT", 7: "FD2D_ERR_INDEX",
    8: "FD2D_ERR_NO_DEVICE", 9: "FD2D_ERR_UNSUPPORTED",
}
PREC_FP64, PREC_FP32 = 0, 1
MEM_HOST, MEM_DEVICE = 0, 1

# Every symbol include/fd2d.h declares (checked by the CPU test suite).
EXPORTED = [
    "fd2d_abi_version", "fd2d_ctx_create", "fd2d_ctx_destroy", "fd2d_ctx_set_stream",
    "fd2d_ctx_set_memspace", "fd2d_ctx_set_precision", "fd2d_ctx_synchronize",
    "fd2d_ctx_kernel_launches", "fd2d_last_error", "fd2d_query_sizes",
    "fd2d_forward1_green", "fd2d_forward2_correlation", "fd2d_noise_adjoint",
    "fd2d_ctx_set_timing", "fd2d_ctx_timing", "fd2d_contract_f32",
    "fd2d_forward1_seismograms_noalloc", "fd2d_correlation_batch", "fd2d_ctx_set_memory_budget",
    "fd2d_make_adjoint_sources", "fd2d_ctx_last_batch", "fd2d_ctx_release", "fd2d_ctx_workspace_bytes",
    "fd2d_gaussblur2d", "fd2d_imfilter_circular", "fd2d_ctx_set_chunks", "fd2d_ctx_set_tile_rows", "fd2d_ctx_last_tile_rows",
    "fd2d_ctx_set_shared_gpu", "fd2d_device_free_bytes", "fd2d_ctx_set_time_depth", "fd2d_ctx_last_time_depth",
    "fd2d_check_bounded_wait",
]
TILE_ROWS_AUTO = 0
TILE_ROWS_RULE = -1
MEAS_WAVEFORM_DIFFERENCE = 0
MEAS_LOG_AMPLITUDE_RATIO = 1
MEAS_CC_TIME_SHIFT = 2
MEAS_AMPLITUDE_DIFFERENCE = 3


class FD2DJob(ctypes.Structure):
    """ctypes mirror of ``fd2d_job``."""

    _fields_ = [
        ("cfg", ctypes.POINTER(FD2DConfig)), ("mu", ctypes.c_void_p), ("rho", ctypes.c_void_p),
        ("spectrum", ctypes.c_void_p), ("n_noise_sources", ctypes.c_int32),
        ("source_dist", ctypes.c_void_p), ("n_dist", ctypes.c_int32),
        ("src", ctypes.c_void_p), ("rec", ctypes.c_void_p), ("nr", ctypes.c_int32),
        ("correlations", ctypes.c_void_p),
    ]
TIMER_STEP_V, TIMER_STEP_VU, TIMER_CONTRACT, TIMER_COUNT = 0, 1, 2, 3

_vp = ctypes.c_void_p
_i32 = ctypes.c_int32
_i64 = ctypes.c_int64
_cfgp = ctypes.POINTER(FD2DConfig)


class FD2DError(RuntimeError):
    def __init__(self, status: int, msg: str):
        self.status = status
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {msg}")


_lib = None
_lock = threading.Lock()


def load(path: str = LIB_PATH):
    """Load libfd2d.so and declare the C prototypes (raises if it is missing)."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(path):
            raise ImportError(
                f"{path} is not built; run `python -c 'import __graft_entry__ as g; g.build()'` "
                "(the GPU path has no CPU fallback)")
        L = ctypes.CDLL(path)
        L.fd2d_abi_version.restype = _i32
        L.fd2d_ctx_create.argtypes = [_i32, _i32, ctypes.POINTER(_vp)]
        L.fd2d_ctx_destroy.argtypes = [_vp]
        L.fd2d_ctx_set_stream.argtypes = [_vp, _vp]
        L.fd2d_ctx_set_memspace.argtypes = [_vp, _i32]
        L.fd2d_ctx_set_precision.argtypes = [_vp, _i32]
        L.fd2d_ctx_synchronize.argtypes = [_vp]
        L.fd2d_ctx_kernel_launches.argtypes = [_vp]
        L.fd2d_ctx_kernel_launches.restype = _i64
        L.fd2d_ctx_last_batch.argtypes = [_vp, ctypes.POINTER(ctypes.c_int32), _i32]
        L.fd2d_ctx_last_batch.restype = _i32
        L.fd2d_ctx_set_tile_rows.argtypes = [_vp, _i32]
        L.fd2d_ctx_set_shared_gpu.argtypes = [_vp, _i32]
        L.fd2d_ctx_last_tile_rows.argtypes = [_vp]
        L.fd2d_ctx_set_time_depth.argtypes = [_vp, _i32]
        L.fd2d_check_bounded_wait.argtypes = [_vp, _i64]
        L.fd2d_ctx_last_time_depth.argtypes = [_vp]
        L.fd2d_ctx_workspace_bytes.argtypes = [_vp]
        L.fd2d_ctx_workspace_bytes.restype = _i64
        L.fd2d_ctx_release.argtypes = [_vp, ctypes.POINTER(_i64)]
        L.fd2d_device_free_bytes.argtypes = [_i32, ctypes.POINTER(_i64), ctypes.POINTER(_i64)]
        L.fd2d_gaussblur2d.argtypes = [_vp, _vp, _i32, _i32, _vp, _vp, ctypes.c_double, ctypes.c_double, _vp]
        L.fd2d_imfilter_circular.argtypes = [_vp, _vp, _i32, _i32, _vp, _i32, _i32, _vp]
        L.fd2d_last_error.argtypes = [_vp]
        L.fd2d_last_error.restype = ctypes.c_char_p
        L.fd2d_query_sizes.argtypes = [_cfgp, _i32, ctypes.POINTER(FD2DSizes)]
        L.fd2d_contract_f32.argtypes = [_vp, _vp, _i64, _vp, _i64, _i32, _i32, _i32, _vp, _i64]
        L.fd2d_forward1_seismograms_noalloc.argtypes = [_cfgp, _vp, _vp, _vp, _i32, _vp, _i32, _vp, _vp]
        L.fd2d_correlation_batch.argtypes = [_vp, ctypes.POINTER(FD2DJob), _i32]
        L.fd2d_ctx_set_memory_budget.argtypes = [_vp, _i64]
        L.fd2d_ctx_set_timing.argtypes = [_vp, _i32]
        L.fd2d_ctx_timing.argtypes = [_vp, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(_i64),
                                      ctypes.POINTER(_i64)]
        L.fd2d_forward1_green.argtypes = [
            _vp, _cfgp, _vp, _vp, _vp, _i32, _vp, _i32, _i32, _vp, _vp, _i32, _vp, _vp, _vp, _vp]
        L.fd2d_forward2_correlation.argtypes = [
            _vp, _cfgp, _vp, _vp, _vp, _vp, _i32, _vp, _i32, _vp, _i32, _vp, _i32, _i32, _vp,
            _vp, _i32, _vp, _vp]
        L.fd2d_noise_adjoint.argtypes = [
            _vp, _cfgp, _vp, _vp, _vp, _i32, _vp, _vp, ctypes.POINTER(_i64), _vp, _i32, _vp, _i32,
            _vp, _i32, _vp, _i32, _vp, _vp, _i32, _i32, _vp, _vp, _i32, _vp, _vp, _vp, _vp, _vp]
        for name in EXPORTED:
            if name not in ("fd2d_abi_version", "fd2d_ctx_kernel_launches", "fd2d_last_error",
                            "fd2d_ctx_last_batch", "fd2d_ctx_workspace_bytes", "fd2d_ctx_last_tile_rows"):
                getattr(L, name).restype = _i32
        _lib = L
        return L


def check(status: int, ctx=None):
    if status != FD2D_OK:
        L = load()
        msg = L.fd2d_last_error(ctx).decode(errors="replace")
        raise FD2DError(status, msg)


class Context:
    """Owns an ``fd2d_ctx`` (one CUDA device, one stream, cached workspace)."""

    def __init__(self, device: int = 0, precision: int = PREC_FP32):
        self.L = load()
        h = _vp()
        check(self.L.fd2d_ctx_create(int(device), int(precision), ctypes.byref(h)))
        self.h = h
        self.device = device
        self.precision = precision
        self.memspace = MEM_HOST

    def close(self):
        if getattr(self, "h", None):
            self.L.fd2d_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_precision(self, precision: int):
        if precision != self.precision:
            check(self.L.fd2d_ctx_set_precision(self.h, int(precision)), self.h)
            self.precision = precision

    def set_memspace(self, memspace: int):
        if memspace != self.memspace:
            check(self.L.fd2d_ctx_set_memspace(self.h, int(memspace)), self.h)
            self.memspace = memspace

    def set_stream(self, stream_ptr: int):
        check(self.L.fd2d_ctx_set_stream(self.h, _vp(stream_ptr or None)), self.h)

    def synchronize(self):
        check(self.L.fd2d_ctx_synchronize(self.h), self.h)

    @property
    def kernel_launches(self) -> int:
        return int(self.L.fd2d_ctx_kernel_launches(self.h))

    def release(self) -> int:
        """Frees the workspace and cached graphs; returns the bytes freed."""
        b = _i64(0)
        check(self.L.fd2d_ctx_release(self.h, ctypes.byref(b)), self.h)
        return int(b.value)

    @property
    def workspace_bytes(self) -> int:
        return int(self.L.fd2d_ctx_workspace_bytes(self.h))

    def set_tile_rows(self, rows: int):
        """Step-kernel tile rows: 16, 30, 32 or 40 forced, TILE_ROWS_AUTO (0)
        timed per grid when the stream is idle, TILE_ROWS_RULE (-1) by grid size
        only."""
        check(self.L.fd2d_ctx_set_tile_rows(self.h, int(rows)), self.h)

    def set_shared_gpu(self, shared: bool):
        """Other work shares the GPU: no programmatic early launch of steps,
        tile shapes by the size rule."""
        check(self.L.fd2d_ctx_set_shared_gpu(self.h, 1 if shared else 0), self.h)

    def last_tile_rows(self) -> int:
        return int(self.L.fd2d_ctx_last_tile_rows(self.h))

    def set_time_depth(self, depth: int):
        """Steps per launch of the FP32 Green and correlation loops at orders 2
        and 4: 1 or 2 forced, 0 timed per grid when the stream is idle."""
        check(self.L.fd2d_ctx_set_time_depth(self.h, int(depth)), self.h)

    def last_time_depth(self) -> int:
        return int(self.L.fd2d_ctx_last_time_depth(self.h))

    def last_batch(self):
        """Lane counts of the launch groups of the last batch."""
        cap = 4096
        buf = (ctypes.c_int32 * cap)()
        n = int(self.L.fd2d_ctx_last_batch(self.h, buf, cap))
        return [int(buf[i]) for i in range(min(n, cap))]

    def set_timing(self, enable: bool):
        check(self.L.fd2d_ctx_set_timing(self.h, 1 if enable else 0), self.h)

    def timing(self):
        """Per timer class: (milliseconds, launches, units); resets the counters."""
        ms = (ctypes.c_double * TIMER_COUNT)()
        n = (_i64 * TIMER_COUNT)()
        u = (_i64 * TIMER_COUNT)()
        check(self.L.fd2d_ctx_timing(self.h, ms, n, u), self.h)
        return [(float(ms[c]), int(n[c]), int(u[c])) for c in range(TIMER_COUNT)]


def device_free_bytes(device: int = 0) -> int:
    """Device memory libfd2d can still allocate (free memory plus the unused
    part of the device's stream-ordered pool)."""
    L = load()
    f, t = _i64(0), _i64(0)
    check(L.fd2d_device_free_bytes(int(device), ctypes.byref(f), ctypes.byref(t)))
    return int(f.value)


def query_sizes(cfg, nr: int) -> FD2DSizes:
    L = load()
    out = FD2DSizes()
    c = cfg.to_c()
    check(L.fd2d_query_sizes(ctypes.byref(c), int(nr), ctypes.byref(out)))
    return out
