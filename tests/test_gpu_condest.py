"""DGECON on the GPU (SRC/dgecon.f) against the oracle's restatement.

Exact mode: RCOND bitwise equal to the oracle's, through the DTRSV path of
DLATRS and through its careful (scaled) solve.  Default mode: DCHKGE test 8
(TESTING/LIN/dchkge.f:536-579: DGET06 against the condition number of the
explicit inverse below THRESH) and agreement with the oracle's estimate."""
import numpy as np
import pytest

import oracle
import oracle.checks as ck

pytestmark = pytest.mark.gpu
THRESH = 30.0


def _factored(n, imat, seed):
    a, izero = oracle.ge_test_matrix(n, n, imat, seed)
    lu, ipiv, info = oracle.getrf(a)
    return a, lu, izero or info


@pytest.mark.parametrize("norm", ["1", "I"])
@pytest.mark.parametrize("n,imat", [(1, 1), (2, 2), (5, 3), (10, 4), (50, 8), (50, 9), (50, 10), (50, 11),
                                    (300, 1), (600, 6)])
def test_gecon_exact_bitwise(gpu, exact_mode, norm, n, imat):
    a, lu, bad = _factored(n, imat, 17 + n + imat)
    if bad:
        pytest.skip("singular test matrix")
    anorm = np.linalg.norm(a, 1 if norm == "1" else np.inf)
    r_ref, i_ref = oracle.gecon(lu, anorm, norm)
    r_gpu, i_gpu = gpu.gecon(lu, anorm, norm)
    assert i_gpu == i_ref == 0
    assert np.float64(r_gpu).tobytes() == np.float64(r_ref).tobytes(), (r_gpu, r_ref)


@pytest.mark.parametrize("norm", ["1", "I"])
@pytest.mark.parametrize("tiny", [1e-80, 1e-150, 1e-300])
def test_gecon_careful_solve_exact_bitwise(gpu, exact_mode, norm, tiny):
    """Factors whose U has tiny pivots (DLATRS growth bound below SMLNUM, so
    the careful solve with rescaling runs): the same RCOND (or the early
    RCOND = 0 of dgecon.f:236) as the oracle, bit for bit."""
    n = 40
    rng = np.random.default_rng(int(-np.log10(tiny)))
    lu = rng.standard_normal((n, n))
    d = np.ones(n)
    d[::7] = tiny
    lu[np.diag_indices(n)] = d
    anorm = 3.0
    r_ref, i_ref = oracle.gecon(lu, anorm, norm)
    r_gpu, i_gpu = gpu.gecon(lu, anorm, norm)
    assert i_gpu == i_ref
    assert np.float64(r_gpu).tobytes() == np.float64(r_ref).tobytes(), (r_gpu, r_ref)


@pytest.mark.parametrize("imat", range(1, 12))
def test_gecon_dchkge_ratio(gpu, imat):
    for n in (3, 10, 50, 200):
        if 5 <= imat <= 7 and n < imat - 4:
            continue
        a, lu, bad = _factored(n, imat, 1988 + 9 * n)
        if bad:
            continue
        ainv = np.linalg.inv(a)
        for norm, p in (("1", 1), ("I", np.inf)):
            anorm = np.linalg.norm(a, p)
            rcondc = (1.0 / anorm) / np.linalg.norm(ainv, p)
            rcond, info = gpu.gecon(lu, anorm, norm)
            assert info == 0
            assert ck.dget06(rcond, rcondc) < THRESH, (n, imat, norm, rcond, rcondc)
            r_ref, _ = oracle.gecon(lu, anorm, norm)
            assert r_ref / 3 <= rcond <= 3 * r_ref, (rcond, r_ref)   # two runs of an estimator


def test_gecon_device_api_matches_host_abi(gpu):
    a, lu, _ = _factored(400, 2, 5)
    anorm = np.linalg.norm(a, 1)
    rh, ih = gpu.gecon(lu, anorm, "1")
    rd, idev = gpu.gecon_dev(gpu.to_colmajor(lu), anorm, "1")
    assert ih == idev == 0 and rd == rh


def test_gecon_n4096(gpu):
    n = 4096
    rng = np.random.default_rng(21)
    a = rng.standard_normal((n, n))
    lu, ipiv, info = gpu.getrf(a)
    assert info == 0
    ainv = np.linalg.inv(a)
    for norm, p in (("1", 1), ("I", np.inf)):
        anorm = np.linalg.norm(a, p)
        rcond, info = gpu.gecon(lu, anorm, norm)
        assert info == 0
        assert ck.dget06(rcond, (1.0 / anorm) / np.linalg.norm(ainv, p)) < THRESH


COMBOS = [(u, t, d) for u in "UL" for t in "NT" for d in "NU"]


def _triangle(n, uplo, seed, diag_scale=1.0):
    rng = np.random.default_rng(seed)
    t = rng.standard_normal((n, n)) / np.sqrt(n)
    t[np.diag_indices(n)] = diag_scale * (1.5 + rng.random(n))
    return np.triu(t) if uplo == "U" else np.tril(t)


@pytest.mark.parametrize("uplo,trans,diag", COMBOS)
def test_latrs_dtrsv_path_exact_bitwise(gpu, exact_mode, uplo, trans, diag):
    """A well-scaled triangle (the growth bound admits DTRSV): x bitwise the
    oracle's (DTRSV loop order, BLAS/SRC/dtrsv.f), SCALE = 1, CNORM equal;
    then NORMIN = 'Y' with that CNORM gives the same again."""
    n = 300
    t = _triangle(n, uplo, 3 + n)
    b = np.random.default_rng(4).standard_normal(n)
    xr, sr, cr = oracle.latrs(t, b, uplo, trans, diag)
    xg, sg, cg = gpu.latrs(t, b, uplo, trans, diag)
    assert sr == sg == 1.0
    assert xg.tobytes() == xr.tobytes() and cg.tobytes() == cr.tobytes()
    xr2, _, _ = oracle.latrs(t, b, uplo, trans, diag, cnorm=cr)
    xg2, _, _ = gpu.latrs(t, b, uplo, trans, diag, cnorm=cg)
    assert xg2.tobytes() == xr2.tobytes()


@pytest.mark.parametrize("uplo,trans,diag", COMBOS)
@pytest.mark.parametrize("n", [6, 33, 200])
def test_latrs_careful_path_exact_bitwise(gpu, exact_mode, uplo, trans, diag, n):
    """A triangle whose solution would overflow (diagonal 1e-80, or a unit
    triangle with off-diagonal 1e80): the careful solve's x, SCALE < 1 and
    CNORM bitwise the oracle's."""
    rng = np.random.default_rng(n + ord(uplo) + ord(trans) + ord(diag))
    t = rng.standard_normal((n, n))
    if diag == "N":
        t[np.diag_indices(n)] = 1e-80 * (1 + rng.random(n))
    else:
        t *= 1e80
    t = np.triu(t) if uplo == "U" else np.tril(t)
    b = rng.standard_normal(n)
    xr, sr, cr = oracle.latrs(t, b, uplo, trans, diag)
    xg, sg, cg = gpu.latrs(t, b, uplo, trans, diag)
    assert sr < 1.0
    assert np.float64(sg).tobytes() == np.float64(sr).tobytes(), (sg, sr)
    assert xg.tobytes() == xr.tobytes()
    assert cg.tobytes() == cr.tobytes()


@pytest.mark.parametrize("uplo,trans,diag", COMBOS)
def test_latrs_default_mode(gpu, uplo, trans, diag):
    """Default mode: n = 2000 well-scaled, op(T) x = b to working accuracy
    with SCALE = 1; n = 60 on the careful path, a finite x with SCALE < 1
    (zero exactly when the oracle's is)."""
    n = 2000
    t = _triangle(n, uplo, 9)
    b = np.random.default_rng(10).standard_normal(n)
    x, sc, _ = gpu.latrs(t, b, uplo, trans, diag)
    tt = t.copy()
    if diag == "U":
        tt[np.diag_indices(n)] = 1.0
    op = tt if trans == "N" else tt.T
    assert sc == 1.0
    assert np.abs(op @ x - b).max() <= 1e3 * n * ck.EPS64 * np.abs(op).max() * np.abs(x).max()
    n = 60
    rng = np.random.default_rng(12)
    t = rng.standard_normal((n, n))
    t[np.diag_indices(n)] = 1e-80 * (1 + rng.random(n)) if diag == "N" else 1.0
    t = np.triu(t) if uplo == "U" else np.tril(t)
    if diag == "U":
        t = t * 1e80
    b = rng.standard_normal(n)
    x, sc, _ = gpu.latrs(t, b, uplo, trans, diag)
    _, sr, _ = oracle.latrs(t, b, uplo, trans, diag)
    assert np.all(np.isfinite(x)) and 0.0 <= sc < 1.0 and (sc == 0.0) == (sr == 0.0)
