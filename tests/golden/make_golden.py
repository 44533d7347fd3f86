"""Generate the golden fixtures of tests/golden/.

The reference (Julia) cannot run in this environment, so the fixtures come from two sources
that do not share code with the C oracle:

1. LAPACK (scipy.linalg.eigh_tridiagonal, i.e. LAPACK stemr), the check the reference's own
   test makes (test/runtests.jl:10): eigenvalues of seeded tridiagonals.
2. A second, pure-Python restatement of the reference's path, written independently of
   oracle/symeig_oracle.c from the reference's source: LinearAlgebra.givensAlgorithm (LAPACK
   3.2 DLARTG, src/simple_givens.jl:20-23), the Wilkinson shift and the flush loop of
   qr_algorithm! (src/bulge_chasing.jl:146-288), single_shift! (:11-144), and rotations
   applied to Q in the order the chase makes them.  Fused multiply-adds are evaluated
   exactly with fractions.Fraction and rounded once, so its floating-point results are fully
   determined and the C oracle must match them bit for bit.

Run:  python tests/golden/make_golden.py   (writes golden_*.json next to this file)
"""
from __future__ import annotations

import json
import math
from fractions import Fraction
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent

SAFMN2 = 2.0 ** -485
SAFMX2 = 2.0 ** 485


def fma(a: float, b: float, c: float) -> float:
    """a*b + c rounded once (exact rational arithmetic, correctly rounded conversion)."""
    if not (math.isfinite(a) and math.isfinite(b) and math.isfinite(c)):
        return a * b + c
    r = Fraction(a) * Fraction(b) + Fraction(c)
    if r == 0:
        # signed zero of an exact zero sum follows IEEE round-to-nearest
        p = a * b
        return p + c
    return float(r)


def jl_max(a: float, b: float) -> float:
    if math.isnan(a) or math.isnan(b):
        return math.nan
    return a if a > b else b


def givens(f: float, g: float):
    """LinearAlgebra.givensAlgorithm(f, g) -> (c, s, r) (LAPACK 3.2 DLARTG)."""
    if g == 0.0:
        return 1.0, 0.0, f
    if f == 0.0:
        return 0.0, 1.0, g
    f1, g1 = f, g
    scale = jl_max(abs(f1), abs(g1))
    if scale >= SAFMX2:
        count = 0
        while True:
            count += 1
            f1 *= SAFMN2
            g1 *= SAFMN2
            scale = jl_max(abs(f1), abs(g1))
            if not (scale >= SAFMX2 and count < 20):
                break
        r = math.sqrt(f1 * f1 + g1 * g1)
        cs, sn = f1 / r, g1 / r
        for _ in range(count):
            r *= SAFMX2
    elif scale <= SAFMN2:
        count = 0
        while True:
            count += 1
            f1 *= SAFMX2
            g1 *= SAFMX2
            scale = jl_max(abs(f1), abs(g1))
            if not scale <= SAFMN2:
                break
        r = math.sqrt(f1 * f1 + g1 * g1)
        cs, sn = f1 / r, g1 / r
        for _ in range(count):
            r *= SAFMN2
    else:
        r = math.sqrt(f1 * f1 + g1 * g1)
        cs, sn = f1 / r, g1 / r
    if abs(f) > abs(g) and cs < 0.0:
        cs, sn, r = -cs, -sn, -r
    return cs, sn, r


def wilkinson(a: float, b: float, c: float) -> float:
    scale = abs(a) + 2.0 * abs(c) + abs(b)
    H11, H12, H22 = a / scale, c / scale, b / scale
    t = (H11 + H22) / 2.0
    d = (H11 - t) * (H22 - t) - H12 * H12
    sq = math.sqrt(abs(d))
    l1, l2 = t + sq, t - sq
    lam = l1 if abs(H22 - l1) < abs(H22 - l2) else l2
    return lam * scale


def is_small(dv, ev, j, tol):  # 1-based j
    return abs(ev[j - 1]) <= tol * (abs(dv[j - 1]) + abs(dv[j]))


def sweep(dv, ev, frm, to, mu):
    """single_shift!: returns the list of (i, c, s) in the order they are made."""
    rots = []

    def update(i, c, s, B11, B21, B22):
        B11p = fma(c, B11, s * B21)
        B21p = fma(c, B21, -(s * B11))
        B12p = fma(c, B21, s * B22)
        B22p = fma(c, B22, -(s * B21))
        return (fma(B11p, c, B12p * s), fma(B12p, c, -(B11p * s)), fma(B22p, c, -(B21p * s)))

    c, s, _ = givens(dv[frm - 1] - mu, ev[frm - 1])
    a, b, d2 = update(frm, c, s, dv[frm - 1], ev[frm - 1], dv[frm])
    dv[frm - 1], ev[frm - 1], dv[frm] = a, b, d2
    bulge = 0.0
    if frm + 2 <= to:
        H23 = ev[frm]
        bulge = s * H23
        ev[frm] = c * H23
    rots.append((frm, c, s))
    for i in range(frm + 1, to):
        c, s, nrm = givens(ev[i - 2], bulge)
        ev[i - 2] = nrm
        a, b, d2 = update(i, c, s, dv[i - 1], ev[i - 1], dv[i])
        dv[i - 1], ev[i - 1], dv[i] = a, b, d2
        if i + 2 <= to:
            B23 = ev[i]
            bulge = s * B23
            ev[i] = c * B23
        rots.append((i, c, s))
    return rots


def qr_algorithm(d, e, max_layers=128, tol=2.0 ** -52, maxiter=None):
    """qr_algorithm! with Q = I, every rotation applied to Q when the chase makes it."""
    n = len(d)
    dv, ev = list(map(float, d)), list(map(float, e))
    Q = [[1.0 if r == c else 0.0 for c in range(n)] for r in range(n)]  # Q[row][col]
    maxiter = 100 * n if maxiter is None else maxiter
    start, it, lbe = 1, 0, n
    while True:
        thick = [0] * n
        did = False
        to = lbe
        while True:
            if it > maxiter:
                return dv, ev, Q, False, it
            frm = to
            while frm > start and not is_small(dv, ev, frm - 1, tol):
                frm -= 1
            if to <= start:
                break
            if frm == to:
                ev[frm - 2] = 0.0
                if to == lbe:
                    lbe -= 1
                to -= 1
            else:
                if max(thick[frm - 1:to]) == max_layers:
                    to = frm - 1
                else:
                    mu = wilkinson(dv[to - 2], dv[to - 1], ev[to - 2])
                    did = True
                    for (i, c, s) in sweep(dv, ev, frm, to, mu):
                        thick[i - 1] += 1
                        for row in Q:
                            x, y = row[i - 1], row[i]
                            row[i - 1] = fma(c, x, s * y)
                            row[i] = fma(c, y, -(s * x))
                    it += 1
            if to <= start:
                break
        if not did:
            return dv, ev, Q, True, it


def hexlist(xs):
    return [float(x).hex() for x in xs]


def main():
    # 1. givensAlgorithm on ordinary, zero, signed, huge and tiny inputs
    rng = np.random.default_rng(2024)
    pairs = [(3.0, 0.0), (0.0, -2.0), (-4.0, 3.0), (-3.0, 4.0), (1e300, 1e300), (1e-310, 3e-310),
             (-0.0, 5.0), (5.0, -0.0), (1e200, -3e205), (-2e-300, 7e-301), (1.0, 1.0), (-1.0, -1.0)]
    for _ in range(200):
        f, g = rng.standard_normal(2) * 10.0 ** rng.integers(-300, 300, 2)
        pairs.append((float(f), float(g)))
    gv = [{"f": f.hex(), "g": g.hex(), "csr": hexlist(givens(f, g))} for f, g in pairs]
    (HERE / "golden_givens.json").write_text(json.dumps(gv, indent=0))

    # 2. full qr_algorithm! runs (eigenvalues, off-diagonal, Q) on small seeded matrices
    cases = []
    specs = [("A", 6, 1), ("B", 9, 2), ("C", 16, 3), ("U", 24, 5), ("A", 13, 4), ("U", 40, 6)]
    for kind, n, seed in specs:
        r = np.random.default_rng(seed)
        if kind == "A":
            d, e = np.arange(1, n + 1, dtype=float), r.random(n - 1)
        elif kind == "B":
            d, e = r.standard_normal(n), 0.5 * r.standard_normal(n - 1)
        elif kind == "C":
            d, e = r.standard_normal(n), r.random(n - 1) * 0.9 + 0.1
        else:
            d, e = r.random(n), r.random(n - 1)
        for max_layers in (128, 3):
            dv, ev, Q, conv, it = qr_algorithm(d, e, max_layers=max_layers)
            cases.append({"kind": kind, "n": n, "seed": seed, "max_layers": max_layers,
                          "d": hexlist(d), "e": hexlist(e), "conv": conv, "iter": it,
                          "d_out": hexlist(dv), "e_out": hexlist(ev),
                          "Q_out_colmajor": hexlist(np.array(Q).T.ravel())})
    (HERE / "golden_qr.json").write_text(json.dumps(cases))

    # 3. LAPACK eigenvalues (the reference test's check)
    from scipy.linalg import eigh_tridiagonal
    lap = []
    for n, seed in [(2, 0), (3, 1), (10, 2), (99, 3), (100, 4), (257, 5), (500, 6)]:
        r = np.random.default_rng(seed)
        d, e = r.random(n), r.random(n - 1)
        lap.append({"n": n, "seed": seed, "d": hexlist(d), "e": hexlist(e),
                    "eigvals": hexlist(eigh_tridiagonal(d, e, eigvals_only=True))})
    (HERE / "golden_lapack.json").write_text(json.dumps(lap))
    print("wrote", [p.name for p in sorted(HERE.glob("golden_*.json"))])


if __name__ == "__main__":
    main()
