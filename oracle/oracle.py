"""ctypes front end of the CPU oracle (oracle/symeig_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, by ``__graft_entry__.smoke()`` and by the
CPU-baseline leg of ``bench.py`` -- never by the product package.  Each function names the
reference routine it restates (paths inside the SymmetricEigenProblem.jl project).
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "_build" / "liboracle.so"
# the same source built for timing only (contraction allowed, tuned for the host's cores):
# the CPU baselines run it; the checks never do
FAST_LIB_PATH = HERE / "_build" / "liboracle_fast.so"

_lib = None
_fast = None

c_i64 = ctypes.c_int64
c_i32 = ctypes.c_int32
c_dbl = ctypes.c_double
c_vp = ctypes.c_void_p


def build(force: bool = False) -> Path:
    """Compile the oracle with its Makefile (gcc; a second or two)."""
    src = HERE / "symeig_oracle.c"
    deps = [src, HERE / "Makefile"]
    stale = any(not p.exists() or any(p.stat().st_mtime < d.stat().st_mtime for d in deps)
                for p in (LIB_PATH, FAST_LIB_PATH))
    if force or stale:
        subprocess.run(["make", "-s", "-C", str(HERE)], check=True)
    return LIB_PATH


def lib(fast: bool = False):
    """The checker library, or with fast=True the timing build of the same source."""
    global _lib, _fast
    if fast:
        if _fast is None:
            build()
            _fast = _bind(ctypes.CDLL(str(FAST_LIB_PATH)))
        return _fast
    if _lib is None:
        build()
        _lib = _bind(ctypes.CDLL(str(LIB_PATH)))
    return _lib


def _bind(L):
    if True:
        L.oracle_givens.argtypes = [c_dbl, c_dbl, ctypes.POINTER(c_dbl), ctypes.POINTER(c_dbl), ctypes.POINTER(c_dbl)]
        L.oracle_givens.restype = None
        for name in ("oracle_apply_seq_f64", "oracle_apply_seq_f32"):
            f = getattr(L, name)
            f.argtypes = [c_vp, c_i64, c_i64, c_i64, c_vp, c_i64]
            f.restype = None
        for name in ("oracle_apply_wave_f64", "oracle_apply_wave_f32"):
            f = getattr(L, name)
            f.argtypes = [c_vp, c_i64, c_i64, c_i64, c_vp, c_i64, ctypes.c_int]
            f.restype = ctypes.c_int
        L.oracle_wilkinson_shift.argtypes = [c_dbl, c_dbl, c_dbl]
        L.oracle_wilkinson_shift.restype = c_dbl
        L.oracle_qr.argtypes = [c_vp, c_vp, c_i64, c_vp, c_i64, c_i64, ctypes.c_int, c_i32, c_dbl, c_i64,
                                c_i32, ctypes.POINTER(c_i32), ctypes.POINTER(c_i64),
                                ctypes.POINTER(c_i64), ctypes.POINTER(c_i64)]
        L.oracle_qr.restype = ctypes.c_int
        L.oracle_qr_form.argtypes = [c_vp, c_vp, c_i64, c_vp, c_i64, c_i64, ctypes.c_int, c_i32, c_dbl, c_i64,
                                     c_i32, c_i32, ctypes.POINTER(c_i32), ctypes.POINTER(c_i64),
                                     ctypes.POINTER(c_i64), ctypes.POINTER(c_i64)]
        L.oracle_qr_form.restype = ctypes.c_int
        L.oracle_qr_multishift.argtypes = [c_vp, c_vp, c_i64, c_vp, c_i64, c_i64, c_i32, c_dbl, c_i64, c_i32,
                                           c_i32, c_i32, c_i32, c_i32, ctypes.POINTER(c_i32), ctypes.POINTER(c_i64),
                                           ctypes.POINTER(c_i64), ctypes.POINTER(c_i64), ctypes.POINTER(c_i64)]
        L.oracle_qr_multishift.restype = ctypes.c_int
        L.oracle_apply_scaled_f64.argtypes = [c_vp, c_i64, c_i64, c_i64, c_vp, c_i64]
        L.oracle_apply_scaled_f64.restype = ctypes.c_int
        L.oracle_qr_init.argtypes = [c_vp, c_i64, c_i32, c_dbl, c_i64, c_i32]
        L.oracle_qr_init.restype = None
        L.oracle_qr_flush.argtypes = [c_vp, c_vp, c_vp, c_vp, c_vp, c_vp]
        L.oracle_qr_flush.restype = ctypes.c_int
        L.oracle_qr_timeorder.argtypes = [c_vp, c_vp, c_i64, c_vp, c_i64, c_i64, c_i32, c_dbl, c_i64,
                                          ctypes.POINTER(c_i32), ctypes.POINTER(c_i64), ctypes.POINTER(c_i64)]
        L.oracle_qr_timeorder.restype = ctypes.c_int
        L.oracle_qr_reference_path.argtypes = [c_vp, c_vp, c_i64, c_vp, c_i64, c_i64, c_i32, c_dbl, c_i64,
                                               ctypes.c_int, c_i32, ctypes.POINTER(c_i32), ctypes.POINTER(c_i64),
                                               ctypes.POINTER(c_i64), ctypes.POINTER(c_dbl),
                                               ctypes.POINTER(c_dbl), ctypes.POINTER(c_i64),
                                               ctypes.POINTER(c_i64)]
        L.oracle_qr_reference_path.restype = ctypes.c_int
    return L


def _ptr(a: np.ndarray) -> int:
    return a.ctypes.data


def givens(f: float, g: float):
    """LinearAlgebra.givensAlgorithm(f, g) -> (c, s, r)  (src/simple_givens.jl:20-23)."""
    c, s, r = c_dbl(), c_dbl(), c_dbl()
    lib().oracle_givens(f, g, ctypes.byref(c), ctypes.byref(s), ctypes.byref(r))
    return c.value, s.value, r.value


def wilkinson_shift(a: float, b: float, c: float) -> float:
    """Shift of src/bulge_chasing.jl:239-265 for the trailing block [a c; c b]."""
    return lib().oracle_wilkinson_shift(a, b, c)


def _check_q(Q: np.ndarray):
    if Q.ndim != 2 or not Q.flags.f_contiguous:
        raise ValueError("Q must be a 2-D column-major (Fortran-ordered) array")


def apply_seq(Q: np.ndarray, cs: np.ndarray) -> None:
    """Layer-major rmul! of every rotation in cs ((n-1) x k x 2, Julia tuple layout) to Q,
    in place: the semantics of bulk_wave_order_2x2_rmul! (src/wave.jl:62-162)."""
    _check_q(Q)
    m, n = Q.shape
    cs = np.asfortranarray(cs)
    k = cs.shape[1] if cs.ndim == 3 else 0
    if Q.dtype not in (np.float64, np.float32):
        raise TypeError(Q.dtype)
    # keep the converted buffer referenced for the duration of the call
    flat = np.ascontiguousarray(np.transpose(cs, (1, 0, 2)).reshape(-1), dtype=Q.dtype) if k else np.zeros(2, Q.dtype)
    ld = Q.strides[1] // Q.itemsize if n > 1 else max(m, 1)
    fn = lib().oracle_apply_seq_f64 if Q.dtype == np.float64 else lib().oracle_apply_seq_f32
    fn(_ptr(Q), ld, m, n, _ptr(flat), k)


def apply_scaled(Q: np.ndarray, cs: np.ndarray) -> None:
    """The device's scaled (fast-Givens) form of the bulk apply, in place on FP64 Q: passes of
    64 layers with per-column scale factors (see oracle_apply_scaled_pass_f64)."""
    _check_q(Q)
    if Q.dtype != np.float64:
        raise TypeError("the scaled form is FP64 only")
    m, n = Q.shape
    k = cs.shape[1] if cs.ndim == 3 else 0
    flat = np.ascontiguousarray(np.transpose(cs, (1, 0, 2)).reshape(-1), dtype=np.float64) if k else np.zeros(2)
    ld = Q.strides[1] // Q.itemsize if n > 1 else max(m, 1)
    rc = lib().oracle_apply_scaled_f64(_ptr(Q), ld, m, n, _ptr(flat), k)
    if rc != 0:
        raise RuntimeError(f"oracle_apply_scaled_f64 failed with status {rc}")


def apply_wave(Q: np.ndarray, cs: np.ndarray, nthreads: int = 1, fast: bool = False) -> None:
    """The wave-order fused apply itself (src/wave.jl:36-162, src/bulk_givens.jl), with the
    reference's row-slab threading.  Requires odd n-1 and even k, as the reference asserts.
    fast=True runs the timing build (contracted arithmetic: for CPU baselines only)."""
    _check_q(Q)
    m, n = Q.shape
    k = cs.shape[1]
    flat = np.ascontiguousarray(np.transpose(cs, (1, 0, 2)).reshape(-1), dtype=Q.dtype)
    ld = Q.strides[1] // Q.itemsize if n > 1 else max(m, 1)
    L = lib(fast)
    fn = L.oracle_apply_wave_f64 if Q.dtype == np.float64 else L.oracle_apply_wave_f32
    rc = fn(_ptr(Q), ld, m, n, _ptr(flat), k, nthreads)
    if rc != 0:
        raise AssertionError("wave order needs n-1 odd and k even (src/wave.jl:65-66)")


class QRState(ctypes.Structure):
    _fields_ = [("n", c_i64), ("max_layers", c_i32), ("tol", c_dbl), ("maxiter", c_i64),
                ("start", c_i64), ("last_block_ends_at", c_i64), ("iter", c_i64),
                ("exact_order", c_i32), ("grid_layers", c_i32),
                ("flush_count", c_i64), ("rotations", c_i64), ("total_rotations", c_i64),
                ("early_flushes", c_i64), ("max_place", c_i64)]


def qr_flushes(d: np.ndarray, e: np.ndarray, max_layers: int = 128, tol: float | None = None,
               maxiter: int | None = None, exact_order: bool = True):
    """Generator over the flushes of qr_algorithm! (src/bulge_chasing.jl:166-279): yields
    (status, grid ((n-1) x grid_layers x 2), thickness (n,), placement (n,), iter) per flush,
    with d/e updated in place.  status 1 = rotations recorded, 0 = converged, -1 = maxiter."""
    n = d.shape[0]
    tol = np.finfo(np.float64).eps if tol is None else tol
    maxiter = 100 * n if maxiter is None else maxiter
    st = QRState()
    lib().oracle_qr_init(ctypes.byref(st), n, max_layers, tol, maxiter, int(exact_order))
    GL = st.grid_layers
    rows = max(n - 1, 1)
    g = np.empty(2 * rows * GL)
    th = np.zeros(n, dtype=np.int64)
    pl = np.zeros(n, dtype=np.int64)
    while True:
        rc = lib().oracle_qr_flush(ctypes.byref(st), _ptr(d), _ptr(e), _ptr(g), _ptr(th), _ptr(pl))
        grid = g.reshape(GL, rows, 2).transpose(1, 0, 2).copy()
        yield rc, grid, th.copy(), pl.copy(), st.iter
        if rc != 1:
            return


def qr_timeorder(d: np.ndarray, e: np.ndarray, Q: np.ndarray, max_layers: int = 128,
                 tol: float | None = None, maxiter: int | None = None):
    """The same solve with every rotation applied to Q as soon as the chase makes it
    (the mathematical order).  Returns (converged, iter, uneven_sweeps)."""
    n = d.shape[0]
    tol = np.finfo(np.float64).eps if tol is None else tol
    maxiter = 100 * n if maxiter is None else maxiter
    _check_q(Q)
    conv, it, un = c_i32(), c_i64(), c_i64()
    ebuf = e if e.size else np.zeros(1)
    rc = lib().oracle_qr_timeorder(_ptr(d), _ptr(ebuf), n, _ptr(Q), Q.strides[1] // Q.itemsize, Q.shape[0],
                                   max_layers, tol, maxiter, ctypes.byref(conv), ctypes.byref(it), ctypes.byref(un))
    if rc != 0:
        raise RuntimeError(rc)
    return bool(conv.value), it.value, un.value


def qr_algorithm(d: np.ndarray, e: np.ndarray, Q: np.ndarray | None, max_layers: int = 128,
                 tol: float | None = None, maxiter: int | None = None, exact_order: bool = True,
                 apply_form: int = 0, fast: bool = False):
    """qr_algorithm!(SymTridiagonal(d, e), Q, max_layers, tol, maxiter)
    (src/bulge_chasing.jl:146-288): d, e and Q updated in place.  exact_order=False keeps the
    reference's grid placement (rotation i of a sweep at layer ++thickness[i]); True (default)
    places each sweep at one layer so the grid's layer-major order is the chase's order.
    apply_form=1 applies each flush in the device's scaled form (FP64 Q only).  fast=True runs
    the timing build (CPU baselines only: its contracted arithmetic is not the reference's).
    Returns (converged, iter, flushes, rotations)."""
    n = d.shape[0]
    assert d.dtype == np.float64 and e.dtype == np.float64 and e.shape[0] == max(n - 1, 0)
    tol = np.finfo(np.float64).eps if tol is None else tol
    maxiter = 100 * n if maxiter is None else maxiter
    conv, it, fl, rot = c_i32(), c_i64(), c_i64(), c_i64()
    if Q is not None:
        _check_q(Q)
        m = Q.shape[0]
        ld = Q.strides[1] // Q.itemsize
        qp, is32 = _ptr(Q), int(Q.dtype == np.float32)
    else:
        m, ld, qp, is32 = 0, 1, None, 0
    ebuf = e if e.size else np.zeros(1)
    rc = lib(fast).oracle_qr_form(_ptr(d), _ptr(ebuf), n, qp, ld, m, is32, max_layers, tol, maxiter, int(exact_order),
                              int(apply_form), ctypes.byref(conv), ctypes.byref(it), ctypes.byref(fl),
                              ctypes.byref(rot))
    if rc != 0:
        raise RuntimeError(f"oracle_qr failed with status {rc}")
    return bool(conv.value), it.value, fl.value, rot.value


# The device's default fewest bulges of a multishift batch (symeig_set_multishift_min).
MS_MIN_DEFAULT = 2


def qr_multishift(d: np.ndarray, e: np.ndarray, Q: np.ndarray | None, max_layers: int = 128,
                  tol: float | None = None, maxiter: int | None = None, exact_order: bool = True,
                  ms_bulges: int = 64, ms_rows: int = 16, ms_window: int = 2, ms_min: int = MS_MIN_DEFAULT):
    """The device's multishift chase (chase mode 3) restated: batches of up to ms_bulges
    sweeps whose shifts are eigenvalues of the block's trailing window of ms_window times the
    batch's size (ranked about the bottom entry), run in sequence with the reference's
    rotations (oracle_qr_multishift); a block with room for fewer than ms_min bulges takes a
    single sweep with the reference's shift.  Not the reference's algorithm; its results are judged
    by the reference's error bounds.  FP64 Q or None.
    Returns (converged, iter, flushes, rotations, batches)."""
    n = d.shape[0]
    assert d.dtype == np.float64 and e.dtype == np.float64 and e.shape[0] == max(n - 1, 0)
    tol = np.finfo(np.float64).eps if tol is None else tol
    maxiter = 100 * n if maxiter is None else maxiter
    conv, it, fl, rot, bat = c_i32(), c_i64(), c_i64(), c_i64(), c_i64()
    if Q is not None:
        _check_q(Q)
        assert Q.dtype == np.float64
        m, ld, qp = Q.shape[0], Q.strides[1] // Q.itemsize, _ptr(Q)
    else:
        m, ld, qp = 0, 1, None
    ebuf = e if e.size else np.zeros(1)
    rc = lib().oracle_qr_multishift(_ptr(d), _ptr(ebuf), n, qp, ld, m, max_layers, tol, maxiter,
                                    int(exact_order), int(ms_bulges), int(ms_rows), int(ms_window), int(ms_min),
                                    ctypes.byref(conv),
                                    ctypes.byref(it), ctypes.byref(fl), ctypes.byref(rot), ctypes.byref(bat))
    if rc != 0:
        raise RuntimeError(f"oracle_qr_multishift failed with status {rc}")
    return bool(conv.value), it.value, fl.value, rot.value, bat.value


def qr_reference_path(d: np.ndarray, e: np.ndarray, Q: np.ndarray | None, max_layers: int = 128,
                      nthreads: int = 1, fast: bool = True, apply_every: int = 1):
    """The reference's solve path on the host, timed (oracle_qr_reference_path): its chase and
    grid placement, and every flush's whole (n-1) x max_layers grid applied by the row-slab
    threaded wave kernel (src/bulge_chasing.jl:146-288 -> src/wave.jl:36-60).  Even n only,
    as the reference.  d, e, Q updated in place.  fast=True (default) uses the timing build.
    apply_every > 1 applies only every apply_every-th flush (a timing sample; Q is then not
    the solve's Q).  Returns (converged, iter, flushes, chase_seconds, apply_seconds,
    rotations_of_applied_flushes, rotations_of_all_flushes)."""
    n = d.shape[0]
    assert d.dtype == np.float64 and e.dtype == np.float64 and e.shape[0] == n - 1
    conv, it, fl = c_i32(), c_i64(), c_i64()
    tc, ta = c_dbl(), c_dbl()
    ra, rt = c_i64(), c_i64()
    if Q is not None:
        _check_q(Q)
        assert Q.dtype == np.float64
        m, ld, qp = Q.shape[0], Q.strides[1] // Q.itemsize, _ptr(Q)
    else:
        m, ld, qp = 0, 1, None
    rc = lib(fast).oracle_qr_reference_path(_ptr(d), _ptr(e), n, qp, ld, m, int(max_layers),
                                            float(np.finfo(np.float64).eps), 100 * n, int(nthreads),
                                            int(apply_every), ctypes.byref(conv), ctypes.byref(it),
                                            ctypes.byref(fl), ctypes.byref(tc), ctypes.byref(ta),
                                            ctypes.byref(ra), ctypes.byref(rt))
    if rc != 0:
        raise ValueError(f"oracle_qr_reference_path: status {rc} (even n and even max_layers needed)")
    return bool(conv.value), it.value, fl.value, tc.value, ta.value, ra.value, rt.value
