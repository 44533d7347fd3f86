"""The benchmark configurations of this project, each checked on the device:

  C1  qr_algorithm! on the README example (src/bulge_chasing.jl:146-288, README.md:65-77):
      n = 2000, d = 1..n, e ~ U[0,1) (seed 0), Q = I, in the reference's sweep sequence
      (chase mode 0): eigenvalues, off-diagonal, iteration count and flush count equal the
      oracle's bit for bit, and Q equals the oracle's on a sample of rows (rows of Q are
      independent under column rotations, so the oracle runs on those rows of I only).
      The multishift chase (mode 3) on the same matrix within the reference's error bounds.
  C2  the bulk apply microbenchmark (src/wave.jl:36-162, benchmark/benchmark.jl:4-30):
      Q 16384 x 16384 ~ U[-1,1), k = 64 layers of (cos t, sin t), FP64 and FP32, at full
      size on the device; 256 rows (the first and last rows, CTA boundaries, random ones)
      equal the oracle's layer-major application bit for bit.
  C3  the full eigensolve at n = 16384 (case A, d = 1..n, e ~ U[0,1), seed 1) and
      n = 16383 (case B, d ~ N(0,1), e ~ 0.5 N(0,1), seed 2): in mode 0 the eigenvalues
      equal the oracle's chase bit for bit (eigenvalues only: the chase alone is the
      reference's bits); the multishift solve with Q within 10 n eps ||T|| (eigenvalues vs
      LAPACK), residual and orthogonality within 10 n eps.
  C4  4096 tridiagonals n ~ U{32..1024} (seed 3) in one batched call: every matrix's
      eigenvalues within the bound, a sample bit for bit against the oracle.
  eigen_decomp! (src/bulge_chasing.jl:290-299) through its C entry point.

Tolerances: bit for bit (np.array_equal) where the reference's sweep sequence runs; the
spec bounds (eigenvalues 10 n eps ||T||, residual and orthogonality 10 n eps) for the
multishift sequence, which is not the reference's.
"""
from __future__ import annotations

import math

import numpy as np
import pytest
from scipy.linalg import eigh_tridiagonal

pytestmark = pytest.mark.gpu

EPS = float(np.finfo(np.float64).eps)


def readme_example():
    n = 2000
    rng = np.random.default_rng(0)
    return np.arange(1, n + 1, dtype=np.float64), rng.random(n - 1)


def case_inputs(n, case):
    if case == "A":
        rng = np.random.default_rng(1)
        return np.arange(1, n + 1, dtype=np.float64), rng.random(n - 1)
    rng = np.random.default_rng(2)
    return rng.standard_normal(n), 0.5 * rng.standard_normal(n - 1)


def row_sample(m, count, seed, block=108):
    """Rows of an m-row Q to compare: the first and last 32, rows on both sides of CTA
    boundaries (every `block` rows), and random ones; sorted, unique, `count` at most."""
    rng = np.random.default_rng(seed)
    rows = set(range(min(32, m))) | set(range(max(m - 32, 0), m))
    for b in range(block, m, block * 17):
        rows |= {b - 1, b}
    while len(rows) < min(count, m):
        rows.add(int(rng.integers(0, m)))
    return np.array(sorted(rows)[:count], dtype=np.int64)


def tq_errors(torch, d, e, lam, Q):
    """(||TQ - Q diag(lam)||_F / ||T||_F, ||Q^T Q - I||_F) in FP64 on the device."""
    dev = Q.device
    dT, eT = torch.from_numpy(d).to(dev), torch.from_numpy(e).to(dev)
    TQ = dT[:, None] * Q
    TQ[:-1] += eT[:, None] * Q[1:]
    TQ[1:] += eT[:, None] * Q[:-1]
    normT = math.sqrt(float((d * d).sum() + 2 * (e * e).sum()))
    resid = float(torch.linalg.norm(TQ - Q * lam[None, :])) / normT
    del TQ
    G = Q.T @ Q
    G.diagonal().sub_(1.0)
    return resid, float(torch.linalg.norm(G))


# ---- C1 -------------------------------------------------------------------------------
def test_c1_readme_example_mode0_bit_exact(cuda, pkg, oracle):
    torch = cuda
    d, e = readme_example()
    n = d.size
    od, oe = d.copy(), e.copy()
    rows = row_sample(n, 96, seed=1, block=16)
    oQ = np.asfortranarray(np.eye(n)[rows, :])          # the sampled rows of Q = I
    conv_o, it_o, fl_o, rot_o = oracle.qr_algorithm(od, oe, oQ)
    h = pkg.Handle(0)
    try:
        H = pkg.SymTridiagonal(d.copy(), e.copy())
        Q = np.asfortranarray(np.eye(n))
        _, conv, it = pkg.qr_algorithm_(H, Q, handle=h)
        st = h.stats()
    finally:
        h.close()
    assert conv and conv_o and it == it_o
    assert st["flushes"] == fl_o == 18
    assert st["rotations"] == rot_o
    assert np.array_equal(H.dv, od)
    assert np.array_equal(H.ev, oe)
    assert np.array_equal(Q[rows, :], oQ)
    # the README's own check: ||A Q - Q D||_F of the README's magnitude (2.86e-10)
    tQ = torch.from_numpy(np.ascontiguousarray(Q.T)).cuda().T
    resid, orth = tq_errors(torch, d, e, torch.from_numpy(H.dv).cuda(), tQ)
    normT = math.sqrt(float((d * d).sum() + 2 * (e * e).sum()))
    assert 2.86e-10 / 2 <= resid * normT <= 2.86e-10 * 2
    assert resid <= 10 * n * EPS and orth <= 10 * n * EPS


def test_c1_readme_example_multishift_within_bounds(cuda, pkg):
    torch = cuda
    d, e = readme_example()
    n = d.size
    H = pkg.SymTridiagonal(torch.from_numpy(d.copy()).cuda(), torch.from_numpy(e.copy()).cuda())
    Q = torch.eye(n, dtype=torch.float64, device="cuda").T
    h = pkg.Handle(0)
    try:
        _, conv, _ = pkg.qr_algorithm_(H, Q, handle=h, chase_mode=3)
        assert h.stats()["bulge_batches"] > 0
    finally:
        h.close()
    assert conv
    lam = eigh_tridiagonal(d, e, eigvals_only=True)
    assert np.max(np.abs(np.sort(H.dv.cpu().numpy()) - lam)) <= 10 * n * EPS * np.max(np.abs(lam))
    resid, orth = tq_errors(torch, d, e, H.dv, Q)
    assert resid <= 10 * n * EPS and orth <= 10 * n * EPS


# ---- C2 -------------------------------------------------------------------------------
@pytest.mark.parametrize("dtype", ["f64", "f32"])
def test_c2_apply_16384_row_sample_bit_exact(cuda, pkg, oracle, dtype):
    torch = cuda
    m = n = 16384
    k = 64
    tdt = torch.float64 if dtype == "f64" else torch.float32
    g = torch.Generator(device="cuda").manual_seed(1234)
    Qt = (torch.rand(n, m, generator=g, dtype=torch.float64, device="cuda") * 2 - 1).to(tdt)
    th = torch.rand(k, n - 1, generator=g, dtype=torch.float64, device="cuda") * (2 * np.pi)
    cs = torch.stack([torch.cos(th), torch.sin(th)], -1).to(tdt).contiguous()   # Julia layout
    del th
    rows = row_sample(m, 256, seed=2)
    sample = np.asfortranarray(Qt[:, torch.from_numpy(rows).cuda()].T.cpu().numpy())
    Q = Qt.T                                       # column-major 16384 x 16384 view
    pkg.bulk_wave_order_2x2_rmul_(Q, cs.view(k, n - 1, 2).permute(1, 0, 2))
    got = Q[torch.from_numpy(rows).cuda(), :].cpu().numpy()
    grid = cs.cpu().numpy().transpose(1, 0, 2)     # (n-1, k, 2) view of the Julia layout
    oracle.apply_seq(sample, grid)
    assert np.array_equal(got, sample), float(np.max(np.abs(got - sample)))


# ---- C3 -------------------------------------------------------------------------------
def test_c3_n16384_case_a_mode0_eigenvalues_bit_equal(cuda, pkg, oracle):
    """The reference's sweep sequence at n = 16384: the device chase reproduces the oracle's
    eigenvalues bit for bit (about two minutes of device chase: 0.9 us per rotation)."""
    torch = cuda
    n = 16384
    d, e = case_inputs(n, "A")
    od, oe = d.copy(), e.copy()
    conv_o, it_o, fl_o, _ = oracle.qr_algorithm(od, oe, None)
    H = pkg.SymTridiagonal(torch.from_numpy(d.copy()).cuda(), torch.from_numpy(e.copy()).cuda())
    _, conv, it = pkg.qr_algorithm_(H, None)
    assert conv and conv_o and it == it_o
    assert np.array_equal(H.dv.cpu().numpy(), od)


@pytest.mark.parametrize("n,case,form", [(16384, "A", 1), (16383, "B", 0)])
def test_c3_full_solve_multishift_within_bounds(cuda, pkg, n, case, form):
    torch = cuda
    d, e = case_inputs(n, case)
    H = pkg.SymTridiagonal(torch.from_numpy(d.copy()).cuda(), torch.from_numpy(e.copy()).cuda())
    Q = torch.eye(n, dtype=torch.float64, device="cuda").T
    _, conv, _ = pkg.qr_algorithm_(H, Q, chase_mode=3, apply_form=form)
    assert conv
    lam = eigh_tridiagonal(d, e, eigvals_only=True)
    err = np.max(np.abs(np.sort(H.dv.cpu().numpy()) - lam))
    assert err <= 10 * n * EPS * np.max(np.abs(lam)), err
    resid, orth = tq_errors(torch, d, e, H.dv, Q)
    assert resid <= 10 * n * EPS, resid
    assert orth <= 10 * n * EPS, orth


# ---- C4 -------------------------------------------------------------------------------
def test_c4_batched_4096_uneven(cuda, pkg, oracle):
    torch = cuda
    rng = np.random.default_rng(3)
    count = 4096
    sizes = rng.integers(32, 1025, size=count)
    d = rng.standard_normal(int(sizes.sum()))
    e = rng.random(int((sizes - 1).sum())) * 0.9 + 0.1
    td, te = torch.from_numpy(d.copy()).cuda(), torch.from_numpy(e.copy()).cuda()
    tQ = torch.zeros(int((sizes * sizes).sum()), dtype=torch.float64, device="cuda")
    off = 0
    for n in sizes:
        tQ[off:off + n * n].view(n, n).fill_diagonal_(1.0)
        off += n * n
    conv, iters = pkg.qr_algorithm_batched_(td, te, sizes, tQ)
    assert conv.all()
    lam_all = td.cpu().numpy()
    check = set(rng.choice(count, 3, replace=False).tolist())
    do = eo = qo = 0
    for j, n in enumerate(sizes):
        n = int(n)
        dj, ej = d[do:do + n], e[eo:eo + n - 1]
        ref = eigh_tridiagonal(dj, ej, eigvals_only=True)
        assert np.max(np.abs(np.sort(lam_all[do:do + n]) - ref)) <= 10 * n * EPS * np.max(np.abs(ref)), j
        if j in check:      # the reference's sweep sequence: the oracle's bits
            od, oe, oQ = dj.copy(), ej.copy(), np.asfortranarray(np.eye(n))
            c_o, it_o, _, _ = oracle.qr_algorithm(od, oe, oQ)
            assert c_o and int(iters[j]) == it_o
            assert np.array_equal(lam_all[do:do + n], od)
            got = tQ[qo:qo + n * n].cpu().numpy().reshape(n, n, order="F")
            assert np.array_equal(got, oQ)
        do += n
        eo += n - 1
        qo += n * n


# ---- eigen_decomp! ---------------------------------------------------------------------
@pytest.mark.parametrize("n,seed", [(1, 0), (2, 1), (300, 2), (513, 3)])
def test_eigen_decomp_c_entry_matches_oracle(cuda, pkg, oracle, n, seed):
    rng = np.random.default_rng(seed)
    d, e = rng.standard_normal(n), rng.random(n - 1) * 0.9 + 0.1
    od, oe, oQ = d.copy(), e.copy(), np.asfortranarray(np.eye(n))
    conv_o, _, _, _ = oracle.qr_algorithm(od, oe, oQ)
    H = pkg.SymTridiagonal(d.copy(), e.copy())
    lam, Q = pkg.eigen_decomp_(H)            # host arrays: symeig_eigen_decomp_f64
    assert conv_o
    assert np.array_equal(lam, od) and np.array_equal(H.ev, oe)
    assert np.array_equal(Q, oQ)
    # device tensors take the qr_algorithm_ route with Q = I: the same bits
    torch = cuda
    Hd = pkg.SymTridiagonal(torch.from_numpy(d.copy()).cuda(), torch.from_numpy(e.copy()).cuda())
    lam_d, Q_d = pkg.eigen_decomp_(Hd)
    assert np.array_equal(lam_d.cpu().numpy(), od) and np.array_equal(Q_d.cpu().numpy(), oQ)


def test_eigen_decomp_rejects_bad_arguments(cuda, pkg):
    lib = pkg.load_library()
    h = pkg.Handle(0)
    try:
        import ctypes
        d = np.ones(4)
        e = np.ones(3)
        conv, it = ctypes.c_int32(), ctypes.c_int64()
        assert lib.symeig_eigen_decomp_f64(h.ptr, d.ctypes.data, e.ctypes.data, 4, None, 4,
                                           ctypes.byref(conv), ctypes.byref(it)) == 1   # NULL Q
        Q = np.zeros((4, 4), order="F")
        assert lib.symeig_eigen_decomp_f64(h.ptr, d.ctypes.data, e.ctypes.data, 4, Q.ctypes.data, 3,
                                           ctypes.byref(conv), ctypes.byref(it)) == 3   # ldq < n
        assert lib.symeig_eigen_decomp_f64(h.ptr, d.ctypes.data, e.ctypes.data, 0, Q.ctypes.data, 4,
                                           ctypes.byref(conv), ctypes.byref(it)) == 2   # n < 1
    finally:
        h.close()
