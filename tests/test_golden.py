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
