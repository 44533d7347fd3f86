"""The adjoint (symeig_eig_adjoint_f64*): dL/d(d, e) of the eigensolve, checked against an
independent FP64 reference gradient (LAPACK eigenpairs + the closed-form pullback, numpy) and
central finite differences (h = 1e-6), with the loss of the batched/adjoint workload:
L = sum_i w_i lam_(i) + sum_{i <= K} q_(i)^T B q_(i) over eigenpairs sorted by ascending lam."""
from __future__ import annotations

import numpy as np
import pytest
from scipy.linalg import eigh_tridiagonal

pytestmark = pytest.mark.gpu


def problem(n, seed, K):
    rng = np.random.default_rng(seed)
    d = rng.standard_normal(n)
    e = rng.random(n - 1) * 0.9 + 0.1
    w = rng.standard_normal(n)
    Bm = rng.standard_normal((n, n)) / np.sqrt(n)
    Bm = (Bm + Bm.T) / 2
    return d, e, w, Bm, K


def reference_grad(d, e, w, Bm, K):
    """FP64 reference: eigenpairs from LAPACK, pullback in numpy."""
    lam, V = eigh_tridiagonal(d, e)          # ascending
    n = d.size
    glam = w.copy()
    gV = np.zeros((n, n))
    gV[:, :K] = 2 * Bm @ V[:, :K]
    F = lam[None, :] - lam[:, None]
    np.fill_diagonal(F, 1.0)
    F = 1.0 / F
    np.fill_diagonal(F, 0.0)
    M = np.diag(glam) + F * (V.T @ gV)
    A = V @ M @ V.T
    return np.diag(A).copy(), np.diag(A, 1) + np.diag(A, -1)


def loss_np(d, e, w, Bm, K):
    lam, V = eigh_tridiagonal(d, e)
    return float(w @ lam + np.sum(V[:, :K] * (Bm @ V[:, :K])))


def torch_loss(torch, lam, Q, w, Bm, K):
    order = torch.argsort(lam)
    lam_s = lam[order]
    Q_s = Q[:, order]
    QK = Q_s[:, :K]
    return (w * lam_s).sum() + (QK * (Bm @ QK)).sum()


@pytest.mark.parametrize("n,K", [(8, 3), (40, 10), (129, 64), (300, 64)])
def test_adjoint_matches_reference_gradient(cuda, pkg, n, K):
    torch = cuda
    d, e, w, Bm, K = problem(n, n, K)
    gd_ref, ge_ref = reference_grad(d, e, w, Bm, K)
    td = torch.tensor(d, device="cuda", requires_grad=True)
    te = torch.tensor(e, device="cuda", requires_grad=True)
    lam, Q = pkg.TridiagEigh.apply(td, te)
    L = torch_loss(torch, lam, Q, torch.tensor(w, device="cuda"), torch.tensor(Bm, device="cuda"), K)
    L.backward()
    gd, ge = td.grad.cpu().numpy(), te.grad.cpu().numpy()
    scale = np.linalg.norm(np.concatenate([gd_ref, ge_ref]))
    err = np.linalg.norm(np.concatenate([gd - gd_ref, ge - ge_ref]))
    assert err <= 1e-9 * max(scale, 1.0), (err, scale)


def test_adjoint_central_differences(cuda, pkg):
    torch = cuda
    n, K = 48, 12
    d, e, w, Bm, K = problem(n, 4, K)
    td = torch.tensor(d, device="cuda", requires_grad=True)
    te = torch.tensor(e, device="cuda", requires_grad=True)
    lam, Q = pkg.TridiagEigh.apply(td, te)
    L = torch_loss(torch, lam, Q, torch.tensor(w, device="cuda"), torch.tensor(Bm, device="cuda"), K)
    L.backward()
    g = np.concatenate([td.grad.cpu().numpy(), te.grad.cpu().numpy()])
    rng = np.random.default_rng(9)
    coords = rng.choice(2 * n - 1, 32, replace=False)
    h = 1e-6
    for c in coords:
        x = np.concatenate([d, e])
        xp, xm = x.copy(), x.copy()
        xp[c] += h
        xm[c] -= h
        fd = (loss_np(xp[:n], xp[n:], w, Bm, K) - loss_np(xm[:n], xm[n:], w, Bm, K)) / (2 * h)
        assert abs(fd - g[c]) <= 1e-5 * max(1.0, abs(fd)), (c, fd, g[c])


def test_adjoint_eigenvalue_only_and_host_entry(cuda, pkg):
    torch = cuda
    n = 77
    d, e, w, Bm, _ = problem(n, 12, 1)
    td = torch.tensor(d, device="cuda", requires_grad=True)
    te = torch.tensor(e, device="cuda", requires_grad=True)
    lam, Q = pkg.TridiagEigh.apply(td, te)
    (torch.tensor(w, device="cuda") * torch.sort(lam).values).sum().backward()
    gd_ref, ge_ref = reference_grad(d, e, w, Bm, 0)
    assert np.allclose(td.grad.cpu().numpy(), gd_ref, rtol=0, atol=1e-12)
    assert np.allclose(te.grad.cpu().numpy(), ge_ref, rtol=0, atol=1e-12)
    # host-buffer entry point gives the same numbers as the device one
    lam_h, Q_h = lam.detach().cpu().numpy(), Q.detach().cpu().numpy()
    glam = np.random.default_rng(1).standard_normal(n)
    gQ = np.random.default_rng(2).standard_normal((n, n))
    gd1, ge1 = pkg.eig_adjoint(lam_h, Q_h, glam, gQ)
    gd2, ge2 = pkg.eig_adjoint(lam.detach(), Q.detach(), torch.tensor(glam, device="cuda"),
                               torch.tensor(gQ, device="cuda"))
    assert np.array_equal(gd1, gd2.cpu().numpy()) and np.array_equal(ge1, ge2.cpu().numpy())


def test_adjoint_batched_matches_single(cuda, pkg):
    torch = cuda
    B, n, K = 5, 60, 8
    rng = np.random.default_rng(21)
    d = rng.standard_normal((B, n))
    e = rng.random((B, n - 1)) * 0.9 + 0.1
    w = torch.tensor(rng.standard_normal(n), device="cuda")
    Bm = torch.tensor(rng.standard_normal((n, n)) / np.sqrt(n), device="cuda")
    Bm = (Bm + Bm.T) / 2
    td = torch.tensor(d, device="cuda", requires_grad=True)
    te = torch.tensor(e, device="cuda", requires_grad=True)
    lam, Q = pkg.TridiagEighBatched.apply(td, te)
    L = sum(torch_loss(torch, lam[b], Q[b], w, Bm, K) for b in range(B))
    L.backward()
    for b in range(B):
        sd = torch.tensor(d[b], device="cuda", requires_grad=True)
        se = torch.tensor(e[b], device="cuda", requires_grad=True)
        l1, q1 = pkg.TridiagEigh.apply(sd, se)
        torch_loss(torch, l1, q1, w, Bm, K).backward()
        assert torch.equal(l1, lam[b].detach())
        assert torch.allclose(sd.grad, td.grad[b], rtol=1e-12, atol=1e-13)
        assert torch.allclose(se.grad, te.grad[b], rtol=1e-12, atol=1e-13)


def test_adjoint_central_differences_n4096(cuda, pkg):
    """The adjoint workload at its own size: n = 4096, d ~ N(0,1), e ~ U[0.1,1) (seed 4),
    L = sum_i w_i lam_(i) + sum_{i <= 64} q_(i)^T B q_(i); dL/d(d, e) from the device (forward
    with the multishift chase, backward symeig_eig_adjoint_f64_dev) against central differences
    (h = 1e-6) on 32 random coordinates, each loss evaluated by LAPACK (all eigenvalues, and
    the 64 lowest eigenvectors)."""
    torch = cuda
    n, K = 4096, 64
    d, e, w, Bm, K = problem(n, 4, K)
    td = torch.tensor(d, device="cuda", requires_grad=True)
    te = torch.tensor(e, device="cuda", requires_grad=True)
    lam, Q = pkg.TridiagEigh.apply(td, te, 3)
    L = torch_loss(torch, lam, Q, torch.tensor(w, device="cuda"), torch.tensor(Bm, device="cuda"), K)
    L.backward()
    g = np.concatenate([td.grad.cpu().numpy(), te.grad.cpu().numpy()])

    def loss(dd, ee):
        lam_all = eigh_tridiagonal(dd, ee, eigvals_only=True)
        _, V = eigh_tridiagonal(dd, ee, select="i", select_range=(0, K - 1))
        return float(w @ lam_all + np.sum(V * (Bm @ V)))

    rng = np.random.default_rng(9)
    coords = rng.choice(2 * n - 1, 32, replace=False)
    h = 1e-6
    x = np.concatenate([d, e])
    for c in coords:
        xp, xm = x.copy(), x.copy()
        xp[c] += h
        xm[c] -= h
        fd = (loss(xp[:n], xp[n:]) - loss(xm[:n], xm[n:])) / (2 * h)
        assert abs(fd - g[c]) <= 1e-5 * max(1.0, abs(fd)), (c, fd, g[c])
