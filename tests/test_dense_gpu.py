"""Dense symmetric -> tridiagonal (sytrd_ / orgtr) and the dense eigensolve (syev): the step
before qr_algorithm!, which the reference leaves to its callers.  Checked against LAPACK
(scipy dsytrd / dorgtr, numpy eigvalsh), which it follows (Householder reflectors, lower):
d, e, tau and Q agree within rounding; A = Q T Q^T and Q^T Q = I within 10 n eps; eigenpairs
within the eigensolve's bounds.  Sizes cross the 64-column panel boundaries."""
from __future__ import annotations

import numpy as np
import pytest
from scipy.linalg import lapack

pytestmark = pytest.mark.gpu

EPS = np.finfo(np.float64).eps


def sym(n, seed, kind="normal"):
    rng = np.random.default_rng(seed)
    if kind == "normal":
        A = rng.standard_normal((n, n))
    elif kind == "graded":
        A = rng.standard_normal((n, n)) * np.logspace(0, -6, n)[None, :]
    elif kind == "lowrank":
        B = rng.standard_normal((n, 3))
        A = B @ B.T
    else:
        raise ValueError(kind)
    return np.asfortranarray((A + A.T) / 2)


def tri(d, e):
    return np.diag(d) + np.diag(e, 1) + np.diag(e, -1)


def lapack_orgtr(c, tau):
    """LAPACK dorgtr (lower): dorgqr on the reflectors shifted by one row (the vector of column j
    has its implicit 1 in row j+1), Q = diag(1, Q2)."""
    n = c.shape[0]
    Q = np.eye(n)
    if n > 1:
        q2, _, info = lapack.dorgqr(np.asfortranarray(c[1:, : n - 1]), tau)
        assert info == 0
        Q[1:, 1:] = q2
    return Q


@pytest.mark.parametrize("n", [1, 2, 3, 5, 63, 64, 65, 66, 128, 129, 200, 301])
def test_sytrd_orgtr_match_lapack(cuda, pkg, n):
    A = sym(n, n)
    A0 = A.copy()
    Ar = A.copy(order="F")
    d, e, tau = pkg.sytrd_(Ar)
    c, dl, el, taul, info = lapack.dsytrd(A0, lower=1)
    assert info == 0
    nrm = np.linalg.norm(A0)
    tol = 100 * n * EPS * max(nrm, 1.0)
    assert np.max(np.abs(d - dl)) <= tol
    if n > 1:
        assert np.max(np.abs(e - el)) <= tol
        assert np.max(np.abs(tau - taul)) <= 100 * n * EPS
        # A's diagonal / subdiagonal hold T, as in LAPACK
        assert np.array_equal(np.diag(Ar), d) and np.array_equal(np.diag(Ar, -1), e)
    Q = pkg.orgtr(Ar, tau)
    if n > 1:
        ql = lapack_orgtr(c, taul)
        assert np.max(np.abs(Q - ql)) <= 100 * n * EPS
    T = tri(d, e)
    assert np.linalg.norm(A0 - Q @ T @ Q.T) / max(nrm, 1e-300) <= 10 * n * EPS
    assert np.linalg.norm(Q.T @ Q - np.eye(n)) <= 10 * n * EPS


@pytest.mark.parametrize("n,kind", [(1, "normal"), (2, "normal"), (50, "normal"), (64, "graded"),
                                    (130, "normal"), (97, "lowrank"), (257, "normal")])
def test_syev_host(cuda, pkg, n, kind):
    A = sym(n, 7 + n, kind)
    A0 = A.copy()
    lam, V, conv, it = pkg.syev(A)
    assert conv
    assert np.array_equal(A, A0)          # the host entry point leaves A unchanged
    ref = np.linalg.eigvalsh(A0)
    nrm = max(np.max(np.abs(ref)), 1e-300)
    assert np.max(np.abs(np.sort(lam) - ref)) <= 10 * n * EPS * nrm
    assert np.linalg.norm(A0 @ V - V * lam[None, :]) / max(np.linalg.norm(A0), 1e-300) <= 10 * n * EPS
    assert np.linalg.norm(V.T @ V - np.eye(n)) <= 10 * n * EPS


def test_syev_device_matches_host(cuda, pkg):
    torch = cuda
    n = 190
    A = sym(n, 3)
    lam_h, V_h, conv_h, it_h = pkg.syev(A)
    tA = torch.from_numpy(A.T.copy()).cuda().T        # column-major view
    lam_d, V_d, conv_d, it_d = pkg.syev(tA)
    assert conv_h and conv_d and it_h == it_d
    assert np.array_equal(lam_d.cpu().numpy(), lam_h)
    assert np.array_equal(V_d.cpu().numpy(), V_h)


def test_sytrd_power_of_two_scaling_is_exact(cuda, pkg):
    """The entry points rescale A by a power of two around its largest entry, so A * 2^k gives
    exactly 2^k times the tridiagonal of A and the same reflectors (also for k = +-600,
    where the unscaled sums of squares would overflow or underflow)."""
    n = 90
    A = sym(n, 11)
    d0, e0, t0 = pkg.sytrd_(A.copy(order="F"))
    for k in (600, -600, 3, -7):
        As = np.asfortranarray(np.ldexp(A, k))
        d, e, t = pkg.sytrd_(As)
        assert np.array_equal(d, np.ldexp(d0, k))
        assert np.array_equal(e, np.ldexp(e0, k))
        assert np.array_equal(t, t0)


def test_sytrd_diagonal_and_zero_columns(cuda, pkg):
    """Columns whose below-subdiagonal part is zero give tau = 0 (H = I), as dlarfg."""
    n = 70
    A = np.asfortranarray(np.diag(np.arange(1.0, n + 1)))
    A[5, 40] = A[40, 5] = 0.5
    d, e, tau = pkg.sytrd_(A.copy(order="F"))
    c, dl, el, taul, info = lapack.dsytrd(A, lower=1)
    assert np.max(np.abs(d - dl)) <= 1e-12 and np.max(np.abs(e - el)) <= 1e-12
    assert np.max(np.abs(tau - taul)) <= 1e-12
    assert np.sum(tau != 0) == np.sum(taul != 0)
