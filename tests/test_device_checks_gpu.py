"""The checked build (libsymeig_checked.so, -DSYMEIG_DEVICE_CHECKS): every global access of a
wave tile to Q is checked against its pass's extent before it is made, and a failed check is
counted in the call's error word and reported as SYMEIG_ERR_DEVICE.  On the shapes and paths
below, which cover partial tiles and warps, edge chunks, the column segments of the host-pointer
path, both precisions, the 27- and 14-warp CTAs and the batched tiles, no check fires and the
results are the oracle's bits."""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

from conftest import rotation_grid
from test_batched_gpu import make_batch, pack

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def checked(cuda, pkg):
    L = pkg.load_checked()
    h = ctypes.c_void_p()
    assert L.symeig_create(ctypes.byref(h), 0) == 0
    yield L, h
    L.symeig_destroy(h)


def device_errors(pkg, L, h):
    from importlib import import_module
    stats_t = import_module(pkg.__name__ + "._lib").Stats
    s = stats_t()
    assert L.symeig_get_stats(h, ctypes.byref(s)) == 0
    return s.device_errors


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
@pytest.mark.parametrize("m,n,k,ld", [(33, 70, 64, 33), (100, 129, 130, 103), (7, 20, 5, 7),
                                      (4100, 300, 64, 4100), (4099, 129, 40, 4111), (15360, 90, 64, 15363),
                                      (16417, 40, 64, 16417), (2000, 600, 128, 2000)])
def test_checked_apply(checked, pkg, oracle, m, n, k, ld, dtype):
    L, h = checked
    rng = np.random.default_rng(m + n + k)
    big = np.asfortranarray((rng.random((ld, n)) * 2 - 1).astype(dtype))
    A = big[:m, :]
    g = rotation_grid(pkg, rng, n, k, dtype)
    ref = np.asfortranarray(A.copy())
    oracle.apply_seq(ref, g)
    fn = L.symeig_apply_givens_f64 if dtype == np.float64 else L.symeig_apply_givens_f32
    gg = np.ascontiguousarray(g.transpose(1, 0, 2))   # pair (i, L) at 2 (i + L (n - 1)): the C ABI's layout
    st = fn(h, ctypes.c_void_p(big.ctypes.data), ld, m, n, ctypes.c_void_p(gg.ctypes.data), k)
    assert st == 0, st
    assert device_errors(pkg, L, h) == 0
    assert np.array_equal(A, ref)


def test_checked_batched(checked, pkg, oracle):
    L, h = checked
    sizes = [2, 9, 40, 64, 65, 119, 257, 333, 17, 1, 600]
    ds, es = make_batch(41, sizes)
    d, e, Q = pack(ds, es)
    n = np.asarray(sizes, dtype=np.int64)
    conv = np.zeros(len(sizes), dtype=np.int32)
    iters = np.zeros(len(sizes), dtype=np.int64)
    st = L.symeig_qr_batched_f64(h, len(sizes), ctypes.c_void_p(n.ctypes.data), ctypes.c_void_p(d.ctypes.data),
                                 ctypes.c_void_p(e.ctypes.data), ctypes.c_void_p(Q.ctypes.data), 128,
                                 float(np.finfo(np.float64).eps), 100, ctypes.c_void_p(conv.ctypes.data),
                                 ctypes.c_void_p(iters.ctypes.data))
    assert st == 0, st
    qo = 0
    for k, nk in enumerate(sizes):
        oQ = np.asfortranarray(np.eye(nk))
        od, oe = ds[k].copy(), es[k].copy()
        oracle.qr_algorithm(od, oe, oQ)
        assert np.array_equal(Q[qo:qo + nk * nk].reshape(nk, nk, order="F"), oQ), (k, nk)
        qo += nk * nk
