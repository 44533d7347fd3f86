"""Failure detection without a GPU fault: every wait of the wave kernels is bounded (about
2 s of SM clock).  symeig_set_test_stall makes those waits run out on purpose -- the kernels'
thread 0 stops copying the rotation table, nothing else changes -- and the host must see
SYMEIG_ERR_TIMEOUT and device_errors = 1, after which the same handle and context must give
correct results again."""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

from conftest import rotation_grid

pytestmark = pytest.mark.gpu

SYMEIG_ERR_TIMEOUT = -3


def test_bounded_wait_timeout_is_reported_and_recoverable(cuda, pkg, oracle):
    lib = pkg.load_library()
    h = pkg.Handle(0)
    rng = np.random.default_rng(21)
    m, n, k = 64, 200, 8
    Q0 = np.asfortranarray(rng.uniform(-1, 1, (m, n)))
    cs = rotation_grid(pkg, rng, n, k)
    flat = np.ascontiguousarray(np.transpose(cs, (1, 0, 2)).reshape(-1))
    A = Q0.copy(order="F")
    assert lib.symeig_set_test_stall(h.ptr, 1) == 0
    rc = lib.symeig_apply_givens_f64(h.ptr, A.ctypes.data, m, m, n, flat.ctypes.data, k)
    assert rc == SYMEIG_ERR_TIMEOUT
    assert h.stats()["device_errors"] == 1
    # the qr driver reports it too
    d, e = rng.random(40), rng.random(39)
    Qe = np.asfortranarray(np.eye(40))
    conv, it = ctypes.c_int32(), ctypes.c_int64()
    rc = lib.symeig_qr_f64(h.ptr, d.ctypes.data, e.ctypes.data, 40, Qe.ctypes.data, 40, 40, 128,
                           np.finfo(np.float64).eps, 4000, ctypes.byref(conv), ctypes.byref(it))
    assert rc == SYMEIG_ERR_TIMEOUT
    # switched off: the same handle works and is exact again
    assert lib.symeig_set_test_stall(h.ptr, 0) == 0
    A = Q0.copy(order="F")
    pkg.bulk_wave_order_2x2_rmul_(A, cs, handle=h)
    ref = Q0.copy(order="F")
    oracle.apply_seq(ref, cs)
    assert np.array_equal(A, ref)
    assert h.stats()["device_errors"] == 0


def test_multishift_bulge_wait_timeout_is_reported_and_recoverable(cuda, pkg):
    """Chase mode 3: with the stall hook on, bulge 0 of each batch never releases its progress;
    the next bulge's bounded wait runs out (~2 s), sets the error word, and every later wait
    gives up at once, so the call ends (here at maxiter = 50) and reports SYMEIG_ERR_TIMEOUT.
    No GPU fault: every index is independent of the values read.  The same handle then
    solves correctly."""
    from scipy.linalg import eigh_tridiagonal
    lib = pkg.load_library()
    h = pkg.Handle(0)
    try:
        rng = np.random.default_rng(5)
        n = 600
        d, e = rng.standard_normal(n), rng.random(n - 1)
        eps = np.finfo(np.float64).eps
        conv, it = ctypes.c_int32(), ctypes.c_int64()
        h.set_chase_mode(3)
        assert lib.symeig_set_test_stall(h.ptr, 1) == 0
        dd, ee = d.copy(), e.copy()
        rc = lib.symeig_qr_f64(h.ptr, dd.ctypes.data, ee.ctypes.data, n, None, 1, 0, 128, eps, 50,
                               ctypes.byref(conv), ctypes.byref(it))
        assert rc == SYMEIG_ERR_TIMEOUT
        assert h.stats()["device_errors"] == 1 and h.stats()["bulge_batches"] > 0
        assert lib.symeig_set_test_stall(h.ptr, 0) == 0
        dd, ee = d.copy(), e.copy()
        rc = lib.symeig_qr_f64(h.ptr, dd.ctypes.data, ee.ctypes.data, n, None, 1, 0, 128, eps, 100 * n,
                               ctypes.byref(conv), ctypes.byref(it))
        assert rc == 0 and conv.value == 1 and h.stats()["device_errors"] == 0
        ref = eigh_tridiagonal(d, e, eigvals_only=True)
        assert np.max(np.abs(np.sort(dd) - ref)) <= 10 * n * eps * np.max(np.abs(ref))
    finally:
        h.set_chase_mode(0)
        h.close()
