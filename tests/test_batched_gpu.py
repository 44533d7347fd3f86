"""Batched eigensolves (symeig_qr_batched_f64): every matrix of a batch must give exactly what
a separate qr_algorithm! gives (the oracle, and the single-matrix device path), bit for bit."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def make_batch(seed, sizes):
    rng = np.random.default_rng(seed)
    ds, es = [], []
    for k, n in enumerate(sizes):
        if k % 3 == 0:
            d, e = rng.standard_normal(n), rng.random(n - 1) * 0.9 + 0.1
        elif k % 3 == 1:
            d, e = rng.random(n), rng.random(n - 1)
        else:
            d, e = np.arange(1, n + 1, dtype=np.float64), rng.random(n - 1)
        ds.append(d)
        es.append(e)
    return ds, es


def pack(ds, es, with_q=True):
    d = np.concatenate(ds)
    e = np.concatenate(es) if sum(x.size for x in es) else np.zeros(0)
    Q = np.concatenate([np.eye(x.size).ravel(order="F") for x in ds]) if with_q else None
    return d, e, Q


@pytest.mark.parametrize("with_q", [True, False])
def test_batched_matches_oracle(cuda, pkg, oracle, with_q):
    sizes = [2, 3, 5, 8, 17, 33, 64, 65, 100, 130, 200, 257, 300, 31, 7, 150, 96, 1, 4, 90]
    ds, es = make_batch(3, sizes)
    d, e, Q = pack(ds, es, with_q)
    conv, iters = pkg.qr_algorithm_batched_(d, e, sizes, Q)
    do, eo, qo = 0, 0, 0
    for k, n in enumerate(sizes):
        od, oe = ds[k].copy(), es[k].copy()
        oQ = np.asfortranarray(np.eye(n)) if with_q else None
        c_o, it_o, _, _ = oracle.qr_algorithm(od, oe, oQ)
        assert conv[k] == c_o and iters[k] == it_o, (k, n)
        assert np.array_equal(d[do:do + n], od), (k, n)
        assert np.array_equal(e[eo:eo + n - 1], oe), (k, n)
        if with_q:
            got = Q[qo:qo + n * n].reshape(n, n, order="F")
            assert np.array_equal(got, oQ), (k, n)
        do += n
        eo += n - 1
        qo += n * n


def test_batched_device_buffers_and_autotune(cuda, pkg, oracle):
    torch = cuda
    tuning, ms = pkg.batched_autotune()
    assert tuning["shape_small"] in (0, 1) and tuning["shape_large"] in (0, 1)
    assert all(t > 0 for row in ms for t in row)
    sizes = list(np.random.default_rng(7).integers(32, 400, size=70))
    ds, es = make_batch(5, sizes)
    d, e, Q = pack(ds, es)
    td, te, tQ = (torch.from_numpy(x.copy()).cuda() for x in (d, e, Q))
    conv, iters = pkg.qr_algorithm_batched_(td, te, sizes, tQ)
    d2, e2, Q2 = td.cpu().numpy(), te.cpu().numpy(), tQ.cpu().numpy()
    do, qo = 0, 0
    for k, n in enumerate(sizes):
        od, oe = ds[k].copy(), es[k].copy()
        oQ = np.asfortranarray(np.eye(n))
        c_o, it_o, _, _ = oracle.qr_algorithm(od, oe, oQ)
        assert conv[k] == c_o and iters[k] == it_o
        assert np.array_equal(d2[do:do + n], od)
        assert np.array_equal(Q2[qo:qo + n * n].reshape(n, n, order="F"), oQ)
        do += n
        qo += n * n


def test_batched_maxiter_per_matrix(cuda, pkg, oracle):
    sizes = [40, 60, 80]
    ds, es = make_batch(11, sizes)
    d, e, Q = pack(ds, es)
    conv, iters = pkg.qr_algorithm_batched_(d, e, sizes, Q, maxiter_factor=1)
    qo = 0
    for k, n in enumerate(sizes):
        od, oe, oQ = ds[k].copy(), es[k].copy(), np.asfortranarray(np.eye(n))
        c_o, it_o, _, _ = oracle.qr_algorithm(od, oe, oQ, maxiter=n)
        assert (bool(conv[k]), int(iters[k])) == (c_o, it_o)
        assert np.array_equal(Q[qo:qo + n * n].reshape(n, n, order="F"), oQ)
        qo += n * n
