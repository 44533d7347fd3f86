"""The scaled ("fast Givens") form of the FP64 bulk apply (symeig_set_apply_form(h, 1)): two
FMAs per rotation and row with per-column scale factors within each pass of 64 layers.  It
must reproduce the oracle's restatement of the same form bit for bit (both tile shapes, several
passes, odd and tiny shapes, lda > m), stay within a few ulps per rotation of the canonical
form, and inside qr_algorithm! give the oracle's scaled-form Q bit for bit with the usual
residual and orthogonality bounds."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import rotation_grid, to_device_colmajor

pytestmark = pytest.mark.gpu

EPS = np.finfo(np.float64).eps


def _set_shape(pkg, shape):
    import ctypes
    lib = pkg.load_library()
    s = ctypes.c_int32(shape)
    lib.symeig_apply_tuning(1, ctypes.byref(s), 1)


@pytest.mark.parametrize("shape", [0, 1])
@pytest.mark.parametrize("m,n,k", [(97, 41, 12), (64, 65, 64), (130, 301, 150), (33, 2, 5), (1, 100, 70),
                                   (257, 129, 128)])
def test_scaled_apply_matches_oracle(cuda, pkg, oracle, shape, m, n, k):
    rng = np.random.default_rng(m * 1000 + n + k)
    Q0 = np.asfortranarray(rng.uniform(-1, 1, (m, n)))
    cs = rotation_grid(pkg, rng, n, k)
    ref = Q0.copy(order="F")
    oracle.apply_scaled(ref, cs)
    _set_shape(pkg, shape)
    try:
        A = Q0.copy(order="F")
        pkg.bulk_wave_order_2x2_rmul_(A, cs, form=1)
        dA = to_device_colmajor(cuda, Q0)
        pkg.bulk_wave_order_2x2_rmul_(dA, cuda.from_numpy(cs).cuda(), form=1)
    finally:
        _set_shape(pkg, -1)
    assert np.array_equal(A, ref)
    assert np.array_equal(dA.cpu().numpy(), ref)
    canon = Q0.copy(order="F")
    oracle.apply_seq(canon, cs)
    # a few ulps per rotation a column takes part in (2 per layer)
    assert np.max(np.abs(A - canon)) <= 8 * (2 * k) * EPS * max(np.max(np.abs(canon)), 1.0)


def test_scaled_apply_leading_dimension(cuda, pkg, oracle):
    rng = np.random.default_rng(5)
    m, n, k = 50, 77, 40
    big = np.asfortranarray(rng.uniform(-1, 1, (m + 7, n)))
    cs = rotation_grid(pkg, rng, n, k)
    ref = np.asfortranarray(big[:m].copy())
    oracle.apply_scaled(ref, cs)
    view = big[:m]
    pkg.bulk_wave_order_2x2_rmul_(view, cs, form=1)
    assert np.array_equal(np.asarray(view), ref)


@pytest.mark.parametrize("exact", [True, False])
@pytest.mark.parametrize("n,seed", [(64, 1), (129, 2), (300, 3)])
def test_qr_scaled_apply_matches_oracle(cuda, pkg, oracle, exact, n, seed):
    rng = np.random.default_rng(seed)
    d, e = rng.random(n), rng.random(n - 1)
    od, oe, oQ = d.copy(), e.copy(), np.asfortranarray(np.eye(n))
    conv_o, it_o, _, _ = oracle.qr_algorithm(od, oe, oQ, exact_order=exact, apply_form=1)
    H = pkg.SymTridiagonal(d.copy(), e.copy())
    Q = np.asfortranarray(np.eye(n))
    _, conv, it = pkg.qr_algorithm_(H, Q, exact_order=exact, apply_form=1)
    assert (conv, it) == (conv_o, it_o)
    assert np.array_equal(H.dv, od) and np.array_equal(H.ev, oe)
    assert np.array_equal(Q, oQ)
    if exact:
        T = np.diag(d) + np.diag(e, 1) + np.diag(e, -1)
        assert np.linalg.norm(T @ Q - Q * H.dv) / np.linalg.norm(T) <= 10 * n * EPS
        assert np.linalg.norm(Q.T @ Q - np.eye(n)) <= 10 * n * EPS


@pytest.mark.parametrize("m,n,k", [(4096, 300, 64), (4100, 77, 33)])
def test_scaled_apply_host_pipelined(cuda, pkg, oracle, m, n, k):
    """The scaled form through the host-pointer entry point, which streams Q by column segments
    (m >= 4096, k <= 64): the oracle's restatement of the form, bit for bit."""
    rng = np.random.default_rng(m + n + k)
    g = rotation_grid(pkg, rng, n, k)
    A = np.asfortranarray(rng.random((m, n)) * 2 - 1)
    ref = A.copy(order="F")
    oracle.apply_scaled(ref, g)
    pkg.bulk_wave_order_2x2_rmul_(A, g, form=1)
    assert np.array_equal(A, ref)
