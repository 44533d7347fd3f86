"""Golden fixtures (tests/golden/, made by tests/golden/make_golden.py): an independent
pure-Python restatement of the reference's path with exactly rounded FMAs, and LAPACK
eigenvalues.  The C oracle must reproduce the former bit for bit and the latter within
10 n eps ||T||; the device path (gpu-marked) must reproduce the former bit for bit."""
from __future__ import annotations

import json
from pathlib import Path

import numpy as np
import pytest

GOLDEN = Path(__file__).resolve().parent / "golden"


def unhex(xs):
    return np.array([float.fromhex(x) for x in xs])


def test_oracle_givens_matches_golden(oracle):
    cases = json.loads((GOLDEN / "golden_givens.json").read_text())
    assert len(cases) > 200
    for cse in cases:
        f, g = float.fromhex(cse["f"]), float.fromhex(cse["g"])
        want = [float.fromhex(x) for x in cse["csr"]]
        got = oracle.givens(f, g)
        assert [x.hex() for x in got] == [x.hex() for x in want], (cse["f"], cse["g"])


@pytest.mark.parametrize("idx", range(12))
def test_oracle_qr_matches_golden(oracle, idx):
    cse = json.loads((GOLDEN / "golden_qr.json").read_text())[idx]
    n = cse["n"]
    d, e = unhex(cse["d"]), unhex(cse["e"])
    Q = np.asfortranarray(np.eye(n))
    conv, it, _, _ = oracle.qr_algorithm(d, e, Q, max_layers=cse["max_layers"])
    assert (conv, it) == (cse["conv"], cse["iter"])
    assert np.array_equal(d, unhex(cse["d_out"]))
    assert np.array_equal(e, unhex(cse["e_out"]))
    assert np.array_equal(Q.ravel(order="F"), unhex(cse["Q_out_colmajor"]))


def test_oracle_matches_lapack_golden(oracle):
    eps = np.finfo(np.float64).eps
    for cse in json.loads((GOLDEN / "golden_lapack.json").read_text()):
        n = cse["n"]
        d, e = unhex(cse["d"]), unhex(cse["e"])
        T = np.diag(d) + np.diag(e, 1) + np.diag(e, -1)
        dd, ee = d.copy(), e.copy()
        conv, _, _, _ = oracle.qr_algorithm(dd, ee, None)
        assert conv
        lam = unhex(cse["eigvals"])
        assert np.max(np.abs(np.sort(dd) - lam)) <= 10 * n * eps * np.linalg.norm(T, 2)


@pytest.mark.gpu
@pytest.mark.parametrize("idx", range(12))
def test_device_qr_matches_golden(cuda, pkg, idx):
    cse = json.loads((GOLDEN / "golden_qr.json").read_text())[idx]
    n = cse["n"]
    H = pkg.SymTridiagonal(unhex(cse["d"]), unhex(cse["e"]))
    Q = np.asfortranarray(np.eye(n))
    _, conv, it = pkg.qr_algorithm_(H, Q, max_layers=cse["max_layers"])
    assert (conv, it) == (cse["conv"], cse["iter"])
    assert np.array_equal(H.dv, unhex(cse["d_out"]))
    assert np.array_equal(Q.ravel(order="F"), unhex(cse["Q_out_colmajor"]))


@pytest.mark.gpu
@pytest.mark.parametrize("form", [0, 1])
def test_device_get_rotation_matches_golden(cuda, pkg, form):
    """The device's rotation generator (form 0: the chase's proved Newton form; form 1: the
    reference form) reproduces the independent restatement's (c, s, r) bits."""
    cases = json.loads((GOLDEN / "golden_givens.json").read_text())
    f = np.array([float.fromhex(c["f"]) for c in cases])
    g = np.array([float.fromhex(c["g"]) for c in cases])
    c, s, r = pkg.get_rotation(f, g, form=form)
    want = np.array([[float.fromhex(x) for x in cse["csr"]] for cse in cases])
    got = np.stack([c, s, r], axis=1)
    assert np.array_equal(got.view(np.uint64), want.view(np.uint64))


@pytest.mark.gpu
def test_device_get_rotation_random_matches_oracle(cuda, pkg, oracle):
    """2^20 random pairs with chase-like and wide exponents: Newton form == reference form ==
    the C oracle's givensAlgorithm, bit for bit (signed zeros included)."""
    rng = np.random.default_rng(77)
    m = 1 << 20
    e1 = np.where(rng.random(m) < 0.8, rng.integers(-30, 31, m), rng.integers(-1000, 1001, m))
    e2 = np.where(rng.random(m) < 0.8, e1 + rng.integers(-30, 31, m), rng.integers(-1000, 1001, m))
    f = rng.standard_normal(m) * np.ldexp(1.0, e1)
    g = rng.standard_normal(m) * np.ldexp(1.0, np.clip(e2, -1070, 1000))
    f[::97] = 0.0
    g[::89] = 0.0
    import torch
    tf, tg = torch.from_numpy(f).cuda(), torch.from_numpy(g).cuda()
    c0, s0, r0 = (t.cpu().numpy() for t in pkg.get_rotation(tf, tg, form=0))
    c1, s1, r1 = pkg.get_rotation(f, g, form=1)
    sample = rng.choice(m, 4096, replace=False)
    oc = np.array([oracle.givens(float(f[i]), float(g[i])) for i in sample])
    for a, b in ((c0, c1), (s0, s1), (r0, r1)):
        assert np.array_equal(a.view(np.uint64), b.view(np.uint64))
    got = np.stack([c0[sample], s0[sample], r0[sample]], axis=1)
    assert np.array_equal(got.view(np.uint64), oc.view(np.uint64))
