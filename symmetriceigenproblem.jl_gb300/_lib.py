"""ctypes binding of libsymeig.so (the C ABI declared in include/symeig.h).

There is no CPU fallback: if the library is missing or cannot be loaded, every call raises.
"""
from __future__ import annotations

import ctypes
import threading
from pathlib import Path

from . import build as _build

c_i64 = ctypes.c_int64
c_i32 = ctypes.c_int32
c_dbl = ctypes.c_double
c_vp = ctypes.c_void_p
P_i32 = ctypes.POINTER(c_i32)
P_i64 = ctypes.POINTER(c_i64)

SYMEIG_OK = 0
STATUS_NAMES = {
    0: "SYMEIG_OK", 1: "SYMEIG_ERR_NULL", 2: "SYMEIG_ERR_SIZE", 3: "SYMEIG_ERR_LD",
    4: "SYMEIG_ERR_LAYERS", 5: "SYMEIG_ERR_HANDLE", -1: "SYMEIG_ERR_CUDA", -2: "SYMEIG_ERR_NOMEM",
    -3: "SYMEIG_ERR_TIMEOUT", -4: "SYMEIG_ERR_DEVICE",
}

# name -> (restype, argtypes); mirrors include/symeig.h
SIGNATURES = {
    "symeig_create": (ctypes.c_int, [ctypes.POINTER(c_vp), ctypes.c_int]),
    "symeig_destroy": (ctypes.c_int, [c_vp]),
    "symeig_set_stream": (ctypes.c_int, [c_vp, c_vp]),
    "symeig_get_stream": (ctypes.c_int, [c_vp, ctypes.POINTER(c_vp)]),
    "symeig_get_stats": (ctypes.c_int, [c_vp, c_vp]),
    "symeig_set_exact_order": (ctypes.c_int, [c_vp, c_i32]),
    "symeig_set_chase_mode": (ctypes.c_int, [c_vp, c_i32]),
    "symeig_set_multishift": (ctypes.c_int, [c_vp, c_i32, c_i32, c_i32]),
    "symeig_set_multishift_min": (ctypes.c_int, [c_vp, c_i32]),
    "symeig_set_apply_form": (ctypes.c_int, [c_vp, c_i32]),
    "symeig_set_test_stall": (ctypes.c_int, [c_vp, c_i32]),
    "symeig_get_rotation_f64": (ctypes.c_int, [c_vp, c_i64, c_vp, c_vp, c_vp, c_vp, c_vp]),
    "symeig_sytrd_f64": (ctypes.c_int, [c_vp, c_i64, c_vp, c_i64, c_vp, c_vp, c_vp]),
    "symeig_sytrd_f64_dev": (ctypes.c_int, [c_vp, c_i64, c_vp, c_i64, c_vp, c_vp, c_vp]),
    "symeig_orgtr_f64": (ctypes.c_int, [c_vp, c_i64, c_vp, c_i64, c_vp, c_vp, c_i64]),
    "symeig_orgtr_f64_dev": (ctypes.c_int, [c_vp, c_i64, c_vp, c_i64, c_vp, c_vp, c_i64]),
    "symeig_syev_f64": (ctypes.c_int, [c_vp, c_i64, c_vp, c_i64, c_vp, c_vp, c_i64, c_vp, c_vp]),
    "symeig_syev_f64_dev": (ctypes.c_int, [c_vp, c_i64, c_vp, c_i64, c_vp, c_vp, c_i64, c_vp, c_vp]),
    "symeig_get_rotation_f64_dev": (ctypes.c_int, [c_vp, c_i64, c_vp, c_vp, c_vp, c_vp, c_vp]),
    "symeig_mul_rn_f64_dev": (ctypes.c_int, [c_vp, c_i64, c_vp, c_vp, c_vp, c_i32]),
    "symeig_set_kernel_timing": (ctypes.c_int, [c_vp, c_i32]),
    "symeig_measure_fma_peak": (ctypes.c_int, [ctypes.c_int, c_i32, ctypes.POINTER(c_dbl)]),
    "symeig_measure_dmma_peak": (ctypes.c_int, [ctypes.c_int, ctypes.POINTER(c_dbl)]),
    "symeig_status_string": (ctypes.c_char_p, [ctypes.c_int]),
    "symeig_device_info": (ctypes.c_int, [c_vp, P_i32, P_i32, P_i32]),
    "symeig_qr_f64": (ctypes.c_int, [c_vp, c_vp, c_vp, c_i64, c_vp, c_i64, c_i64, c_i32, c_dbl, c_i64, P_i32, P_i64]),
    "symeig_qr_f64_dev": (ctypes.c_int, [c_vp, c_vp, c_vp, c_i64, c_vp, c_i64, c_i64, c_i32, c_dbl, c_i64, P_i32, P_i64]),
    "symeig_qr_f64_q32": (ctypes.c_int, [c_vp, c_vp, c_vp, c_i64, c_vp, c_i64, c_i64, c_i32, c_dbl, c_i64, P_i32, P_i64]),
    "symeig_qr_f64_q32_dev": (ctypes.c_int, [c_vp, c_vp, c_vp, c_i64, c_vp, c_i64, c_i64, c_i32, c_dbl, c_i64, P_i32, P_i64]),
    "symeig_apply_givens_f64": (ctypes.c_int, [c_vp, c_vp, c_i64, c_i64, c_i64, c_vp, c_i64]),
    "symeig_apply_givens_f32": (ctypes.c_int, [c_vp, c_vp, c_i64, c_i64, c_i64, c_vp, c_i64]),
    "symeig_apply_givens_f64_dev": (ctypes.c_int, [c_vp, c_vp, c_i64, c_i64, c_i64, c_vp, c_i64]),
    "symeig_apply_givens_f32_dev": (ctypes.c_int, [c_vp, c_vp, c_i64, c_i64, c_i64, c_vp, c_i64]),
    "symeig_apply_givens_left_f64": (ctypes.c_int, [c_vp, c_vp, c_i64, c_i64, c_i64, c_vp, c_i64]),
    "symeig_apply_givens_left_f32": (ctypes.c_int, [c_vp, c_vp, c_i64, c_i64, c_i64, c_vp, c_i64]),
    "symeig_apply_givens_left_f64_dev": (ctypes.c_int, [c_vp, c_vp, c_i64, c_i64, c_i64, c_vp, c_i64]),
    "symeig_apply_givens_left_f32_dev": (ctypes.c_int, [c_vp, c_vp, c_i64, c_i64, c_i64, c_vp, c_i64]),
    "symeig_apply_givens_f64_noalloc": (ctypes.c_int, [c_vp, c_i64, c_i64, c_i64, c_vp, c_i64, c_vp]),
    "symeig_noalloc_init": (ctypes.c_int, []),
    "symeig_noalloc_status": (ctypes.c_int, [c_vp]),
    "symeig_qr_batched_f64": (ctypes.c_int, [c_vp, c_i64, c_vp, c_vp, c_vp, c_vp, c_i32, c_dbl, c_i64, c_vp, c_vp]),
    "symeig_qr_batched_f64_dev": (ctypes.c_int, [c_vp, c_i64, c_vp, c_vp, c_vp, c_vp, c_i32, c_dbl, c_i64, c_vp, c_vp]),
    "symeig_batched_autotune": (ctypes.c_int, [c_vp, c_vp]),
    "symeig_batched_autotune_sizes": (ctypes.c_int, [c_vp, c_i64, c_vp, c_vp]),
    "symeig_batched_tuning": (ctypes.c_int, [P_i64, P_i32, P_i32, c_i32]),
    "symeig_batched_tuning_dtype": (ctypes.c_int, [c_i32, P_i64, P_i32, P_i32, c_i32]),
    "symeig_qr_batched_f64_q32": (ctypes.c_int, [c_vp, c_i64, c_vp, c_vp, c_vp, c_vp, c_i32, c_dbl, c_i64, c_vp, c_vp]),
    "symeig_qr_batched_f64_q32_dev": (ctypes.c_int, [c_vp, c_i64, c_vp, c_vp, c_vp, c_vp, c_i32, c_dbl, c_i64, c_vp, c_vp]),
    "symeig_apply_tuning": (ctypes.c_int, [c_i32, P_i32, c_i32]),
    "symeig_eig_adjoint_f64": (ctypes.c_int, [c_vp, c_i64, c_i64, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp]),
    "symeig_eig_adjoint_f64_dev": (ctypes.c_int, [c_vp, c_i64, c_i64, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp]),
    "symeig_eigen_decomp_f64": (ctypes.c_int, [c_vp, c_vp, c_vp, c_i64, c_vp, c_i64, P_i32, P_i64]),
}


class Stats(ctypes.Structure):
    _fields_ = [("iterations", c_i64), ("flushes", c_i64), ("rotations", c_i64),
                ("applied_rotation_rows", c_i64), ("chase_ms", c_dbl), ("apply_ms", c_dbl),
                ("total_ms", c_dbl), ("early_flushes", c_i64), ("wave_launches", c_i64),
                ("wave_kernel_ms", c_dbl), ("device_errors", c_i64), ("redone_sweeps", c_i64),
                ("bulge_batches", c_i64)]

    def as_dict(self) -> dict:
        return {f: getattr(self, f) for f, _ in self._fields_}


class SymeigError(RuntimeError):
    def __init__(self, fn: str, status: int):
        self.status = status
        super().__init__(f"{fn} returned {STATUS_NAMES.get(status, status)}: {status_string(status)}")


_lib = None
_lock = threading.Lock()


def lib_path() -> Path:
    return _build.LIB


def load(build_if_missing: bool = True):
    """Load libsymeig.so (building it first when missing and nvcc is present)."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = _build.LIB
        if not path.exists() or _build._stale():
            if not build_if_missing:
                raise RuntimeError(f"libsymeig.so is not built ({path})")
            _build.build()
        L = ctypes.CDLL(str(path))
        for name, (res, args) in SIGNATURES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
        return L


def load_checked():
    """The checked build (libsymeig_checked.so, built on first use): the same ABI, with every
    global access of the wave tiles checked against its pass's extent (see build.build_checked).
    A separate library instance: its handles are created with its own symeig_create."""
    path = _build.build_checked()
    L = ctypes.CDLL(str(path))
    for name, (res, args) in SIGNATURES.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    return L


def status_string(status: int) -> str:
    return load().symeig_status_string(status).decode()


def check(fn: str, status: int):
    if status != SYMEIG_OK:
        raise SymeigError(fn, status)


class Handle:
    """One libsymeig context (device, stream, scratch buffers)."""

    def __init__(self, device: int = 0):
        self._lib = load()
        h = c_vp()
        check("symeig_create", self._lib.symeig_create(ctypes.byref(h), device))
        self.ptr = h
        self.device = device

    def close(self):
        if self.ptr:
            self._lib.symeig_destroy(self.ptr)
            self.ptr = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def stats(self) -> dict:
        s = Stats()
        check("symeig_get_stats", self._lib.symeig_get_stats(self.ptr, ctypes.byref(s)))
        return s.as_dict()

    def set_kernel_timing(self, on: bool):
        check("symeig_set_kernel_timing", self._lib.symeig_set_kernel_timing(self.ptr, int(bool(on))))

    def set_exact_order(self, exact: bool):
        check("symeig_set_exact_order", self._lib.symeig_set_exact_order(self.ptr, int(bool(exact))))

    def set_apply_form(self, form):
        """0: canonical rotations (default); 1: the scaled form for FP64 applies."""
        check("symeig_set_apply_form", self._lib.symeig_set_apply_form(self.ptr, int(form)))

    def set_multishift(self, max_bulges: int = 64, rows_per_bulge: int = 16, release_every: int = 4):
        """Batch shape of chase mode 3 (symeig_set_multishift)."""
        check("symeig_set_multishift", self._lib.symeig_set_multishift(
            self.ptr, int(max_bulges), int(rows_per_bulge), int(release_every)))

    def set_multishift_min(self, min_bulges: int = 2):
        """Fewest bulges of a chase-mode-3 batch (symeig_set_multishift_min)."""
        check("symeig_set_multishift_min", self._lib.symeig_set_multishift_min(self.ptr, int(min_bulges)))

    def set_chase_mode(self, mode):
        """0: Newton-form two-warp chase (default); 1: reference form; 2: Newton form with
        every sweep redone in the reference form -- these give the reference's bits; 3: the
        multishift chase (within the reference's error bounds)."""
        check("symeig_set_chase_mode", self._lib.symeig_set_chase_mode(self.ptr, int(mode)))

    def set_stream(self, stream_ptr: int | None):
        """Run *_dev calls on this cudaStream_t (0/None = the legacy default stream)."""
        check("symeig_set_stream", self._lib.symeig_set_stream(self.ptr, stream_ptr))

    def get_stream(self) -> int | None:
        s = c_vp()
        check("symeig_get_stream", self._lib.symeig_get_stream(self.ptr, ctypes.byref(s)))
        return s.value

    def on_stream(self, stream_ptr: int | None):
        """Context manager: run on `stream_ptr`, then restore the previous stream."""
        import contextlib

        @contextlib.contextmanager
        def cm():
            old = self.get_stream()
            self.set_stream(stream_ptr)
            try:
                yield self
            finally:
                self.set_stream(old)
        return cm()

    def call(self, name: str, *args):
        check(name, getattr(self._lib, name)(self.ptr, *args))


def measure_fma_peak(device: int = 0, fp64: bool = True) -> float:
    """FMA throughput of the device now, TFLOP/s (FMA = 2 flops)."""
    v = c_dbl()
    check("symeig_measure_fma_peak", load().symeig_measure_fma_peak(device, int(fp64), ctypes.byref(v)))
    return v.value


def measure_dmma_peak(device: int = 0) -> float:
    """FP64 tensor-core (mma.sync .f64) throughput of the device now, TFLOP/s."""
    v = c_dbl()
    check("symeig_measure_dmma_peak", load().symeig_measure_dmma_peak(device, ctypes.byref(v)))
    return v.value


_tls = threading.local()


def default_handle(device: int = 0) -> Handle:
    """Per-thread, per-device handle (handles are not shared across threads)."""
    hs = getattr(_tls, "handles", None)
    if hs is None:
        hs = _tls.handles = {}
    if device not in hs:
        hs[device] = Handle(device)
    return hs[device]
