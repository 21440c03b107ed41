"""DGESVX on the GPU (SRC/dgesvx.f) against the oracle's restatement.

Exact mode: every output (equilibrated A, AF, IPIV, EQUED, R, C, scaled B,
X, RCOND, FERR, BERR, the reciprocal pivot growth, INFO) bitwise equal to
the oracle's for FACT = 'N', 'E', 'F' and TRANS = 'N', 'T' on the DCHKGE
matrix types and row / column scaled copies (all four EQUED values).
Default mode: DDRVGE's DGESVX checks (TESTING/LIN/ddrvge.f:518-628)."""
import numpy as np
import pytest

import oracle
import oracle.checks as ck

pytestmark = pytest.mark.gpu
THRESH = 30.0

EQUED_CASES = {
    "N": [[2.0, 1.0], [1.0, 3.0]],
    "R": [[1e8, 2e8], [1.0, 3.0]],
    "C": [[1.0, 1e-8], [1.0, 2e-8]],
    "B": [[1e8, 1.0], [1.0, 2e-8]],
}


def _systems(n, imat, seed):
    a, izero = oracle.ge_test_matrix(n, n, imat, seed)
    out = [(a, izero)]
    if n >= 2 and izero == 0:
        g = np.random.default_rng(seed)
        dr = 10.0 ** g.uniform(-6, 6, n)
        dc = 10.0 ** g.uniform(-6, 6, n)
        out += [(dr[:, None] * a, 0), (a * dc[None, :], 0), (dr[:, None] * a * dc[None, :], 0)]
    return out


def _same(g, o, keys):
    for k in keys:
        gv, ov = g[k], o[k]
        if isinstance(ov, np.ndarray):
            assert np.asarray(gv).tobytes() == np.asarray(ov).tobytes(), k
        elif isinstance(ov, float):
            assert np.float64(gv).tobytes() == np.float64(ov).tobytes(), (k, gv, ov)
        else:
            assert gv == ov, (k, gv, ov)


ALL = ["a", "af", "ipiv", "equed", "r", "c", "b", "x", "rcond", "ferr", "berr", "rpvgrw", "info"]


@pytest.mark.parametrize("fact", ["N", "E"])
@pytest.mark.parametrize("trans", ["N", "T"])
@pytest.mark.parametrize("n,imat", [(1, 1), (3, 2), (10, 4), (50, 1), (50, 6), (50, 9), (50, 11), (200, 3)])
def test_gesvx_exact_bitwise(gpu, exact_mode, fact, trans, n, imat):
    for a, izero in _systems(n, imat, 77 + n + imat):
        xact = oracle.random_matrix(n, 3, 5 + n, idist=2)[0]
        b = (a if trans == "N" else a.T) @ xact
        o = oracle.gesvx(a, b, fact, trans)
        g = gpu.gesvx(a, b, fact, trans)
        if o["info"] > 0 and o["info"] <= n:     # singular U: X, FERR, BERR are not produced
            _same(g, o, ["af", "ipiv", "equed", "rcond", "rpvgrw", "info"])
            continue
        _same(g, o, ALL)
        # FACT = 'F' with the returned factors and scalings
        of = oracle.gesvx(o["a"], b, "F", trans, af=o["af"], ipiv=o["ipiv"], equed=o["equed"], r=o["r"], c=o["c"])
        gf = gpu.gesvx(o["a"], b, "F", trans, af=o["af"], ipiv=o["ipiv"], equed=o["equed"], r=o["r"], c=o["c"])
        _same(gf, of, ["x", "rcond", "ferr", "berr", "rpvgrw", "info", "b"])


@pytest.mark.parametrize("equed", "NRCB")
@pytest.mark.parametrize("trans", "NT")
def test_gesvx_equed_cases(gpu, equed, trans):
    a = np.array(EQUED_CASES[equed])
    xact = np.array([[1.0, -2.0], [3.0, 0.5]])
    b = (a if trans == "N" else a.T) @ xact
    g = gpu.gesvx(a, b, "E", trans)
    assert g["equed"] == equed and g["info"] == 0
    assert np.allclose(g["x"], xact, rtol=1e-6)


@pytest.mark.parametrize("imat", range(1, 12))
@pytest.mark.parametrize("fact,trans", [("N", "N"), ("E", "N"), ("E", "T")])
def test_gesvx_ddrvge_ratios(gpu, imat, fact, trans):
    for n in (3, 10, 50, 120):
        if 5 <= imat <= 7 and n < imat - 4:
            continue
        for a, izero in _systems(n, imat, 1995 + 3 * n + imat):
            xact = oracle.random_matrix(n, 2, 9 + n, idist=2)[0]
            b = (a if trans == "N" else a.T) @ xact
            g = gpu.gesvx(a, b, fact, trans)
            if izero:
                assert g["info"] == izero and g["rcond"] == 0.0
                continue
            assert g["info"] in (0, n + 1)
            assert (g["info"] == n + 1) == (g["rcond"] < ck.EPS64)
            assert ck.dget01(g["a"], g["af"], g["ipiv"]) < THRESH
            assert ck.dget02(a, g["x"], b, trans) < THRESH
            p = 1 if trans == "N" else np.inf
            assert ck.dget04(g["x"], xact, 1.0 / np.linalg.cond(a, p)) < THRESH
            r1, r2 = ck.dget07(a, b, g["x"], xact, g["ferr"], g["berr"], trans)
            assert r1 < THRESH and r2 < THRESH, (n, imat, g["equed"], r1, r2)
            assert ck.dget06(g["rcond"], 1.0 / np.linalg.cond(g["a"], p)) < THRESH
