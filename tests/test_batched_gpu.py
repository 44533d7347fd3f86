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


def check_against_oracle(oracle, sizes, ds, es, d, e, Q, conv, iters, qdtype):
    do, eo, qo = 0, 0, 0
    for k, n in enumerate(sizes):
        od, oe = ds[k].copy(), es[k].copy()
        oQ = np.asfortranarray(np.eye(n, dtype=qdtype))
        c_o, it_o, _, _ = oracle.qr_algorithm(od, oe, oQ)
        assert conv[k] == c_o and iters[k] == it_o, (k, n)
        assert np.array_equal(d[do:do + n], od), (k, n)
        assert np.array_equal(e[eo:eo + n - 1], oe), (k, n)
        assert np.array_equal(Q[qo:qo + n * n].reshape(n, n, order="F"), oQ), (k, n)
        do += n
        eo += n - 1
        qo += n * n


def test_batched_q32_matches_oracle(cuda, pkg, oracle):
    """FP32 Q: the chase is FP64 (the same d, e, iterations as the FP64 solve) and every
    matrix's Q is the oracle's FP32-Q qr_algorithm! bit for bit, host and device buffers."""
    torch = cuda
    sizes = [2, 3, 5, 8, 17, 33, 64, 65, 100, 130, 200, 257, 300, 31, 7, 150, 96, 1, 4, 90]
    ds, es = make_batch(23, sizes)
    d, e, _ = pack(ds, es, False)
    Q = np.concatenate([np.eye(n, dtype=np.float32).ravel(order="F") for n in sizes])
    conv, iters = pkg.qr_algorithm_batched_(d, e, sizes, Q)
    check_against_oracle(oracle, sizes, ds, es, d, e, Q, conv, iters, np.float32)
    d, e, _ = pack(ds, es, False)
    Q = np.concatenate([np.eye(n, dtype=np.float32).ravel(order="F") for n in sizes])
    td, te, tQ = (torch.from_numpy(x.copy()).cuda() for x in (d, e, Q))
    conv, iters = pkg.qr_algorithm_batched_(td, te, sizes, tQ)
    check_against_oracle(oracle, sizes, ds, es, td.cpu().numpy(), te.cpu().numpy(), tQ.cpu().numpy(),
                         conv, iters, np.float32)


@pytest.mark.parametrize("qdtype", [np.float64, np.float32])
@pytest.mark.parametrize("small,large", [(0, 2), (2, 1), (1, 0), (2, 2)])
def test_batched_every_tile(cuda, pkg, oracle, qdtype, small, large):
    """Every batched tile (0: 16 rows x 64 layers, 1: 32 rows x 64 layers, 2: 8 rows x 128
    layers per pass) in either size class gives the oracle's bits; exact-order flushes of up to
    256 layers take four passes of the 64-layer tiles and two of the 128-layer tile."""
    fp64 = qdtype == np.float64
    old = pkg.batched_tuning(fp64=fp64)
    pkg.batched_tuning(fp64=fp64, split=120, shape_small=small, shape_large=large)
    try:
        assert pkg.batched_tuning(fp64=fp64) == {"split": 120, "shape_small": small, "shape_large": large}
        sizes = [2, 9, 40, 64, 65, 119, 120, 121, 130, 200, 257, 333, 17, 1, 600]
        ds, es = make_batch(31 + small * 3 + large, sizes)
        d, e, _ = pack(ds, es, False)
        Q = np.concatenate([np.eye(n, dtype=qdtype).ravel(order="F") for n in sizes])
        conv, iters = pkg.qr_algorithm_batched_(d, e, sizes, Q)
        check_against_oracle(oracle, sizes, ds, es, d, e, Q, conv, iters, qdtype)
    finally:
        pkg.batched_tuning(fp64=fp64, **old)


@pytest.mark.parametrize("sizes", [None, [40, 70, 300, 900, 2, 1, 257]])
def test_batched_autotune(cuda, pkg, sizes):
    """The autotuner times every tile per size class and precision of Q and keeps the fastest;
    with the batch's own orders (a class may be empty, orders 1 are left out) as with the
    default spread."""
    tuning, ms = pkg.batched_autotune(sizes=sizes)
    for name in ("f64", "f32"):
        assert tuning[name]["shape_small"] in (0, 1, 2) and tuning[name]["shape_large"] in (0, 1, 2)
        assert len(ms[name]) == 2 and all(len(row) == 3 for row in ms[name])
        assert all(0 < t < 1e4 for row in ms[name] for t in row)
        for c, key in ((0, "shape_small"), (1, "shape_large")):
            assert ms[name][c][tuning[name][key]] == min(ms[name][c])


def test_batched_device_buffers_and_autotune(cuda, pkg, oracle):
    torch = cuda
    tuning, ms = pkg.batched_autotune()
    for name in ("f64", "f32"):
        assert tuning[name]["shape_small"] in (0, 1, 2) and tuning[name]["shape_large"] in (0, 1, 2)
        assert len(ms[name]) == 2 and all(len(row) == 3 for row in ms[name])
        assert all(0 < t < 1e4 for row in ms[name] for t in row)
        for c, key in ((0, "shape_small"), (1, "shape_large")):
            assert ms[name][c][tuning[name][key]] == min(ms[name][c])
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
