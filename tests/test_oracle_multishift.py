"""The oracle's restatement of the multishift chase (chase mode 3, oracle_qr_multishift), on
the CPU: batches of sweeps whose shifts are the eigenvalues of the block's trailing square, on
the reference's deflation, capacity and placement rules.  It is not the reference's sweep
sequence, so it is held to the reference's error bounds (eigenvalues within 10 n eps ||T|| of
LAPACK, residual and orthogonality within 10 n eps), and to the reference's own bits where
no block is long enough for a batch."""
from __future__ import annotations

import numpy as np
import pytest
from scipy.linalg import eigh_tridiagonal

EPS = np.finfo(np.float64).eps


def tridiag(kind, n, seed):
    rng = np.random.default_rng(seed)
    if kind == "A":
        return np.arange(1, n + 1, dtype=np.float64), rng.random(n - 1)
    if kind == "B":
        return rng.standard_normal(n), 0.5 * rng.standard_normal(n - 1)
    if kind == "C":
        return rng.standard_normal(n), rng.random(n - 1) * 0.9 + 0.1
    if kind == "split":
        d, e = rng.standard_normal(n), rng.random(n - 1)
        e[n // 3] = 0.0
        e[(2 * n) // 3] = 0.0
        return d, e
    if kind == "graded":
        return 10.0 ** np.linspace(0, -8, n), rng.random(n - 1) * 10.0 ** np.linspace(0, -8, n - 1)
    raise ValueError(kind)


def bounds(d, e, lam, Q):
    """(eigenvalue error, residual, orthogonality), each over its 10 n eps bound."""
    n = d.size
    ref = eigh_tridiagonal(d, e, eigvals_only=True)
    eig = np.max(np.abs(np.sort(lam) - ref)) / (10 * n * EPS * np.max(np.abs(ref)))
    TQ = d[:, None] * Q
    TQ[:-1] += e[:, None] * Q[1:]
    TQ[1:] += e[:, None] * Q[:-1]
    res = np.linalg.norm(TQ - Q * lam[None, :]) / np.sqrt((d * d).sum() + 2 * (e * e).sum()) / (10 * n * EPS)
    orth = np.linalg.norm(Q.T @ Q - np.eye(n)) / (10 * n * EPS)
    return eig, res, orth


@pytest.mark.parametrize("kind,n", [("C", 150), ("A", 200), ("split", 180)])
def test_no_batch_is_the_reference(oracle, kind, n):
    """With more rows per bulge than any block has, every decision is a Wilkinson single
    sweep: the reference's bits."""
    d, e = tridiag(kind, n, n)
    rd, re_, rQ = d.copy(), e.copy(), np.asfortranarray(np.eye(n))
    r_ref = oracle.qr_algorithm(rd, re_, rQ)
    md, me, mQ = d.copy(), e.copy(), np.asfortranarray(np.eye(n))
    r_ms = oracle.qr_multishift(md, me, mQ, ms_rows=10 * n)
    assert r_ms[4] == 0
    assert r_ms[:4] == r_ref
    assert np.array_equal(md, rd) and np.array_equal(me, re_) and np.array_equal(mQ, rQ)


@pytest.mark.parametrize("kind,n", [("A", 600), ("B", 500), ("C", 300), ("split", 400), ("graded", 300)])
@pytest.mark.parametrize("exact_order", [True, False])
def test_multishift_within_the_bounds(oracle, kind, n, exact_order):
    d, e = tridiag(kind, n, n)
    lam, ee, Q = d.copy(), e.copy(), np.asfortranarray(np.eye(n))
    conv, it, flushes, rot, batches = oracle.qr_multishift(lam, ee, Q, exact_order=exact_order)
    assert conv and batches > 0
    eig, res, orth = bounds(d, e, lam, Q)
    assert eig <= 1.0 and orth <= 1.0, (eig, orth)
    if exact_order:
        # the reference's placement misses the residual bound in the reference's own
        # sequence too once split blocks re-merge; the exact-order placement meets it
        assert res <= 1.0, res
    # about as many sweeps as the reference's sequence: the shifts of the window twice the
    # batch's size lose little against the Wilkinson shift (case A: fewer rotations)
    r0 = oracle.qr_algorithm(d.copy(), e.copy(), None)
    assert 0.7 <= rot / r0[3] <= 2.5, rot / r0[3]


@pytest.mark.parametrize("kind,n", [("A", 1500), ("B", 1500)])
def test_multishift_window_costs_fewer_sweeps(oracle, kind, n):
    """The shift window of twice the batch's size (the device's rule) makes fewer sweeps than
    the square of the batch's size, and both stay within the bounds."""
    d, e = tridiag(kind, n, 7)
    rots = {}
    for w in (1, 2):
        lam, ee, Q = d.copy(), e.copy(), np.asfortranarray(np.eye(n))
        conv, _, _, rots[w], batches = oracle.qr_multishift(lam, ee, Q, ms_window=w)
        assert conv and batches > 0
        eig, res, orth = bounds(d, e, lam, Q)
        assert eig <= 1.0 and res <= 1.0 and orth <= 1.0, (w, eig, res, orth)
    assert rots[2] < rots[1], rots


def test_multishift_eigenvalues_do_not_depend_on_q(oracle):
    d, e = tridiag("B", 400, 9)
    a, ea = d.copy(), e.copy()
    b, eb = d.copy(), e.copy()
    Q = np.asfortranarray(np.eye(400))
    ra = oracle.qr_multishift(a, ea, None)
    rb = oracle.qr_multishift(b, eb, Q)
    assert ra[:2] == rb[:2] and ra[3:] == rb[3:]
    assert np.array_equal(a, b)


@pytest.mark.parametrize("max_layers", [2, 3, 8])
def test_multishift_layer_room_caps_the_batches(oracle, max_layers):
    d, e = tridiag("C", 350, 4)
    lam, ee, Q = d.copy(), e.copy(), np.asfortranarray(np.eye(350))
    conv, it, flushes, rot, batches = oracle.qr_multishift(lam, ee, Q, max_layers=max_layers)
    assert conv and batches > 0
    eig, res, orth = bounds(d, e, lam, Q)
    assert eig <= 1.0 and res <= 1.0 and orth <= 1.0, (eig, res, orth)


def test_multishift_maxiter(oracle):
    d, e = tridiag("A", 500, 2)
    conv, it, _, _, batches = oracle.qr_multishift(d.copy(), e.copy(), None, maxiter=10)
    assert not conv and it <= 11 and batches >= 1


def test_multishift_arguments_are_checked(oracle):
    d, e = tridiag("C", 50, 1)
    for bad in (dict(ms_bulges=1), dict(ms_bulges=129), dict(ms_rows=3), dict(ms_window=0), dict(ms_window=5),
                dict(ms_min=1), dict(ms_min=65)):
        with pytest.raises(RuntimeError):
            oracle.qr_multishift(d.copy(), e.copy(), None, **bad)


def test_multishift_min_bulges_trades_batches_for_sweeps(oracle):
    """A minimum batch size sends short blocks to single sweeps with the reference's shift:
    fewer batches, the same eigenvalues within the bounds, and with a minimum above every
    block's room no batch at all (then the chase is the reference's)."""
    from scipy.linalg import eigh_tridiagonal
    n = 800
    d = np.arange(1, n + 1, dtype=np.float64)
    e = np.random.default_rng(0).random(n - 1)
    ref = eigh_tridiagonal(d, e, eigvals_only=True)
    batches = {}
    for mn in (2, 8, 64):
        dd, ee = d.copy(), e.copy()
        conv, it, _, rot, bat = oracle.qr_multishift(dd, ee, None, ms_min=mn)
        assert conv
        assert np.max(np.abs(np.sort(dd) - ref)) < 10 * n * np.finfo(float).eps * np.max(np.abs(ref))
        batches[mn] = bat
    assert batches[2] > batches[8] > batches[64] == 0
    dd, ee = d.copy(), e.copy()
    c0, it0, _, _ = oracle.qr_algorithm(dd, ee, None)
    d64, e64 = d.copy(), e.copy()
    conv, it, _, _, _ = oracle.qr_multishift(d64, e64, None, ms_min=64)
    assert c0 and conv and it == it0 and np.array_equal(d64, dd)
