"""The oracle (C restatement of the reference routines) against the
reference's own pins: the DLARUV multiplier table read from SRC/dlaruv.f,
the TESTING/LIN test ratios over the TESTING/dtest.in and dstest.in grids,
the error-exit tables, and an independent LU (OpenBLAS via scipy)."""
import ctypes
import json
import os

import numpy as np
import pytest

import oracle
import oracle.checks as ck

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
INPUTS = json.load(open(os.path.join(GOLDEN, "test_inputs.json")))
THRESH = INPUTS["dtest"]["thresh"]


def test_dlaruv_multipliers_match_reference_table():
    mm = json.load(open(os.path.join(GOLDEN, "dlaruv_mm.json")))["mm"]
    assert len(mm) == 128
    for i, row in enumerate(mm, start=1):
        assert oracle.dlaruv_power(i) == row, f"MM({i},:)"


def test_dlarnv_stream_properties():
    it1 = oracle.seed_to_iseed(7)
    a = oracle.dlarnv(1, it1, 200)
    it2 = oracle.seed_to_iseed(7)
    b = np.concatenate([oracle.dlarnv(1, it2, 64), oracle.dlarnv(1, it2, 136)])
    assert np.array_equal(a, b)                 # chunking does not change the stream
    assert np.all((a > 0) & (a < 1))
    assert np.array_equal(it1, it2)
    u = oracle.dlarnv(2, oracle.seed_to_iseed(1), 100000)
    assert np.all((u > -1) & (u < 1)) and abs(u.mean()) < 0.02
    z = oracle.dlarnv(3, oracle.seed_to_iseed(0), 100000)
    assert abs(z.mean()) < 0.02 and abs(z.std() - 1) < 0.02


@pytest.mark.parametrize("imat", range(1, 12))
@pytest.mark.parametrize("nb", sorted(set(INPUTS["dtest"]["nb"])))
def test_dgetrf_dchkge_ratios(imat, nb):
    """DCHKGE tests 1, 3, 4 (TESTING/LIN/dchkge.f:280-583) on every M x N of
    dtest.in: INFO = IZERO for the zero-column types, DGET01 < THRESH,
    and for square nonsingular systems DGET02 / DGET04 < THRESH."""
    for m in INPUTS["dtest"]["m"]:
        for n in INPUTS["dtest"]["n"]:
            if 5 <= imat <= 7 and n < imat - 4:
                continue
            a, izero = oracle.ge_test_matrix(m, n, imat, 1988 + 7 * m + n)
            lu, ipiv, info = oracle.getrf(a, nb=nb)
            assert info == izero, (m, n, imat, info, izero)
            if m and n:
                assert ck.dget01(a, lu, ipiv) < THRESH, (m, n, imat)
            if m == n and n > 0 and izero == 0:
                for nrhs in INPUTS["dtest"]["nrhs"]:
                    xact = oracle.random_matrix(n, nrhs, 5 + n + nrhs, idist=2)[0]
                    for trans in "NTC":
                        b = (a if trans == "N" else a.T) @ xact
                        x, info = oracle.getrs(lu, ipiv, b, trans)
                        assert info == 0
                        assert ck.dget02(a, x, b, "N" if trans == "N" else "T") < THRESH
                        rcond = 1.0 / np.linalg.cond(a, 1)
                        assert ck.dget04(x, xact, rcond) < THRESH


@pytest.mark.parametrize("nrhs", INPUTS["dstest"]["nrhs"])
def test_dsgesv_ddrvab_ratios(nrhs):
    """DDRVAB (TESTING/LIN/ddrvab.f): DGET08 < sqrt(N) when ITER >= 0, else <
    THRESH, INFO = IZERO, on the dstest.in N list for GE types 1-11."""
    for n in INPUTS["dstest"]["n"]:
        for imat in range(1, 12):
            if 5 <= imat <= 7 and n < imat - 4:
                continue
            a, izero = oracle.ge_test_matrix(n, n, imat, 2006 + n + imat)
            xact = oracle.random_matrix(n, nrhs, 2009 + n, idist=2)[0]
            b = a @ xact
            ao, ip, x, it, info = oracle.dsgesv(a, b)
            assert info == izero, (n, imat, info, izero)
            if n == 0 or izero:
                continue
            r = ck.dget08(a, x, b)
            if it >= 0:
                assert r < np.sqrt(n) or r < 1.0, (n, imat, it, r)
                assert np.array_equal(ao, a)
            else:
                assert r < THRESH, (n, imat, it, r)


@pytest.mark.parametrize("imat", range(1, 12))
def test_dgerfs_dchkge_ratios(imat):
    """DCHKGE tests 5, 6, 7 (TESTING/LIN/dchkge.f:496-520): after DGERFS
    refines the DGETRS solution, DGET04 and both DGET07 ratios (forward error
    bound, componentwise backward error) stay below THRESH, for every square
    nonsingular N of dtest.in, every NRHS and TRANS = N, T, C."""
    for n in INPUTS["dtest"]["n"]:
        if n == 0 or (5 <= imat <= 7 and n < imat - 4):
            continue
        a, izero = oracle.ge_test_matrix(n, n, imat, 1988 + 7 * n + n)
        if izero:
            continue
        lu, ipiv, info = oracle.getrf(a)
        assert info == 0
        for nrhs in INPUTS["dtest"]["nrhs"]:
            xact = oracle.random_matrix(n, nrhs, 5 + n + nrhs, idist=2)[0]
            for trans in "NTC":
                op = a if trans == "N" else a.T
                rcond = 1.0 / np.linalg.cond(op, 1)
                b = op @ xact
                x0, info = oracle.getrs(lu, ipiv, b, trans)
                x, ferr, berr, info = oracle.gerfs(a, lu, ipiv, b, x0, trans)
                assert info == 0
                assert ck.dget04(x, xact, rcond) < THRESH, (n, imat, nrhs, trans)
                r1, r2 = ck.dget07(a, b, x, xact, ferr, berr, "N" if trans == "N" else "T")
                assert r1 < THRESH and r2 < THRESH, (n, imat, nrhs, trans, r1, r2)


@pytest.mark.parametrize("imat", range(1, 12))
def test_dgecon_dchkge_ratios(imat):
    """DCHKGE test 8 (TESTING/LIN/dchkge.f:536-579): DGET06(RCOND, RCONDC) <
    THRESH for NORM = '1' and 'I', RCONDC from the explicit inverse, on every
    square nonsingular N of dtest.in."""
    for n in INPUTS["dtest"]["n"]:
        if n == 0 or (5 <= imat <= 7 and n < imat - 4):
            continue
        a, izero = oracle.ge_test_matrix(n, n, imat, 1988 + 7 * n + n)
        if izero:
            continue
        lu, ipiv, info = oracle.getrf(a)
        ainv = np.linalg.inv(a)
        for norm, p in (("1", 1), ("I", np.inf)):
            anorm = np.linalg.norm(a, p)
            rcondc = (1.0 / anorm) / np.linalg.norm(ainv, p)
            rcond, info = oracle.gecon(lu, anorm, norm)
            assert info == 0
            assert ck.dget06(rcond, rcondc) < THRESH, (n, imat, norm, rcond, rcondc)


@pytest.mark.parametrize("uplo,trans,diag", [("U", "N", "N"), ("L", "N", "U"), ("U", "T", "N"), ("L", "T", "U")])
def test_dlatrs_careful_path(uplo, trans, diag):
    """DLATRS (SRC/dlatrs.f) on a triangle whose growth bound rejects DTRSV
    (n = 6, diagonal 1e-80, off-diagonal O(1), so x would reach ~1e480): the
    careful solve returns a finite x with 0 < SCALE < 1 and op(T) x = SCALE * b
    to working accuracy."""
    n = 6
    rng = np.random.default_rng(3)
    t = rng.standard_normal((n, n))
    t = np.triu(t) if uplo == "U" else np.tril(t)
    np.fill_diagonal(t, 1e-80 if diag == "N" else 1.0)
    if diag == "U":
        t = t * 1e80                        # a unit triangle whose solution grows past overflow
        np.fill_diagonal(t, 1.0)
    b = rng.standard_normal(n)
    x, scale, cnorm = oracle.latrs(t, b, uplo, trans, diag)
    assert np.all(np.isfinite(x)) and 0.0 < scale <= 1.0
    assert scale < 1.0                        # the scaled path was taken
    tt = t if trans == "N" else t.T
    # scale the check down to stay clear of overflow in the product
    m = np.abs(x).max()
    r = tt @ (x / m) - (scale / m) * b
    assert np.abs(r).max() <= 1e3 * n * ck.EPS64 * np.abs(tt).max() * 1.0


def _svx_systems(n, imat, seed):
    """The DCHKGE test matrix and row / column scaled copies of it, so that
    DGEEQU + DLAQGE choose EQUED = 'N', 'R', 'C' and 'B'."""
    a, izero = oracle.ge_test_matrix(n, n, imat, seed)
    out = [(a, izero)]
    if n >= 2 and izero == 0:
        g = np.random.default_rng(seed)
        dr = 10.0 ** g.uniform(-6, 6, n)
        dc = 10.0 ** g.uniform(-6, 6, n)
        out += [(dr[:, None] * a, 0), (a * dc[None, :], 0), (dr[:, None] * a * dc[None, :], 0)]
    return out


@pytest.mark.parametrize("imat", range(1, 12))
@pytest.mark.parametrize("fact,trans", [("N", "N"), ("E", "N"), ("E", "T"), ("N", "T")])
def test_dgesvx_ddrvge_ratios(imat, fact, trans):
    """DDRVGE's DGESVX checks (TESTING/LIN/ddrvge.f:518-628): INFO = IZERO
    with RCOND = 0 for the zero-column types; otherwise DGET01 on the
    (equilibrated) factors, DGET02 and DGET07 on the original system,
    DGET04 against the original condition number, DGET06 against the
    condition number of the matrix actually factored, the reciprocal pivot
    growth recomputed from A and AF (RESULT(7)), and INFO = N+1 exactly when
    RCOND < eps."""
    for n in INPUTS["dtest"]["n"]:
        if n == 0 or (5 <= imat <= 7 and n < imat - 4):
            continue
        for a, izero in _svx_systems(n, imat, 1991 + 3 * n + imat):
            xact = oracle.random_matrix(n, 2, 7 + n, idist=2)[0]
            op = a if trans == "N" else a.T
            b = op @ xact
            o = oracle.gesvx(a, b, fact, trans)
            if izero:
                assert o["info"] == izero and o["rcond"] == 0.0
                continue
            assert o["info"] in (0, n + 1)
            assert (o["info"] == n + 1) == (o["rcond"] < ck.EPS64)
            ae, af = o["a"], o["af"]
            assert ck.dget01(ae, af, o["ipiv"]) < THRESH
            rp = oracle.lib().or_dlantr_mun
            rp.restype = ctypes.c_double
            rp.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_int]
            afc = np.asfortranarray(af)
            u = rp(n, n, afc.ctypes.data_as(ctypes.c_void_p), n)
            rpv = 1.0 if u == 0 else np.abs(ae).max() / u
            assert abs(rpv - o["rpvgrw"]) / max(rpv, o["rpvgrw"]) / ck.EPS64 < THRESH
            tr = "N" if trans == "N" else "T"
            assert ck.dget02(a, o["x"], b, tr) < THRESH
            p = 1 if trans == "N" else np.inf
            rc_orig = 1.0 / np.linalg.cond(a, p)
            assert ck.dget04(o["x"], xact, rc_orig) < THRESH
            r1, r2 = ck.dget07(a, b, o["x"], xact, o["ferr"], o["berr"], tr)
            assert r1 < THRESH and r2 < THRESH, (n, imat, o["equed"], r1, r2)
            rc_eq = 1.0 / np.linalg.cond(ae, p)
            assert ck.dget06(o["rcond"], rc_eq) < THRESH
            # FACT = 'F' with the returned factors, scalings and the original B:
            # the same X, BERR and RCOND bit for bit; FERR is divided by a
            # ROWCND / COLCND that FACT = 'F' recomputes from the reciprocal
            # scalings (dgesvx.f:395-420), equal up to rounding
            if fact == "E":
                f = oracle.gesvx(o["a"], b, "F", trans, af=o["af"], ipiv=o["ipiv"], equed=o["equed"], r=o["r"],
                                 c=o["c"])
                assert f["info"] == o["info"] and f["rcond"] == o["rcond"]
                assert f["x"].tobytes() == o["x"].tobytes() and f["berr"].tobytes() == o["berr"].tobytes()
                np.testing.assert_allclose(f["ferr"], o["ferr"], rtol=8 * ck.EPS64)


EQUED_CASES = {   # 2 x 2 systems for which DGEEQU + DLAQGE pick each EQUED
    "N": [[2.0, 1.0], [1.0, 3.0]],
    "R": [[1e8, 2e8], [1.0, 3.0]],
    "C": [[1.0, 1e-8], [1.0, 2e-8]],
    "B": [[1e8, 1.0], [1.0, 2e-8]],
}


@pytest.mark.parametrize("equed", "NRCB")
@pytest.mark.parametrize("trans", "NT")
def test_dgesvx_equed_cases(equed, trans):
    a = np.array(EQUED_CASES[equed])
    xact = np.array([[1.0, -2.0], [3.0, 0.5]])
    b = (a if trans == "N" else a.T) @ xact
    o = oracle.gesvx(a, b, "E", trans)
    assert o["equed"] == equed and o["info"] == 0
    assert np.allclose(o["x"], xact, rtol=1e-6)
    r1, r2 = ck.dget07(a, b, o["x"], xact, o["ferr"], o["berr"], trans)
    assert r1 < THRESH and r2 < THRESH


def test_dgeequ_reference_rules():
    """DGEEQU (SRC/dgeequ.f): R and C are reciprocals of the clamped row /
    column maxima, ROWCND / COLCND their ratios, INFO names the first zero
    row (i) or column (M + j)."""
    a = np.array([[4.0, 0.0, 1.0], [0.0, 0.5, 0.0], [2.0, 0.0, 8.0]])
    r, c, rowcnd, colcnd, amax, info = oracle.geequ(a)
    assert info == 0 and amax == 8.0
    assert np.array_equal(r, 1.0 / np.array([4.0, 0.5, 8.0]))
    assert np.array_equal(c, 1.0 / np.array([1.0, 1.0, 1.0]))
    assert rowcnd == 0.5 / 8.0 and colcnd == 1.0
    z = a.copy()
    z[1, :] = 0.0
    assert oracle.geequ(z)[5] == 2
    z = a.copy()
    z[:, 2] = 0.0
    z[1, 1] = 1.0
    assert oracle.geequ(z)[5] == 3 + 3


@pytest.mark.parametrize("imat", range(1, 12))
def test_dgetri_dchkge_ratio(imat):
    """DCHKGE test 2 (TESTING/LIN/dchkge.f:383-420): DGET03 < THRESH for the
    inverse from the factors, for every square N and every NB of dtest.in
    (NB = 1 and NB >= N take the unblocked loop); INFO = i for the first
    zero pivot of the zero-column types."""
    for n in INPUTS["dtest"]["n"]:
        if 5 <= imat <= 7 and n < imat - 4:
            continue
        a, izero = oracle.ge_test_matrix(n, n, imat, 1988 + 7 * n + n)
        lu, ipiv, info = oracle.getrf(a)
        for nb in sorted(set(INPUTS["dtest"]["nb"])) + [64]:
            ainv, info, _ = oracle.getri(lu, ipiv, nb=nb)
            if izero:
                assert info > 0 and lu[info - 1, info - 1] == 0.0
                continue
            assert info == 0
            if n:
                assert ck.dget03(a, ainv)[0] < THRESH, (n, imat, nb)


def test_dgetri_workspace_rules():
    """LWORK = -1 returns N*NB in WORK(1) and does nothing else; a workspace
    below N*NB shrinks the block size (dgetri.f:200-216) with the same
    result up to rounding; LWORK < N is argument 6."""
    a = oracle.random_matrix(40, 40, 3, idist=3)[0]
    lu, ipiv, _ = oracle.getrf(a)
    _, info, w0 = oracle.getri(lu, ipiv, nb=16, lwork=-1)
    assert info == 0 and w0 == 40 * 16
    x1, _, _ = oracle.getri(lu, ipiv, nb=16)
    x2, info, w0 = oracle.getri(lu, ipiv, nb=16, lwork=40 * 5)
    assert info == 0 and w0 == 40 * 16
    np.testing.assert_allclose(x2, x1, rtol=1e-9, atol=1e-12)
    oracle.xerbla_reset()
    _, info, _ = oracle.getri(lu, ipiv, nb=16, lwork=39)
    assert info == -6 and oracle.xerbla_last() == ("DGETRI", 6)


@pytest.mark.parametrize("uplo", "LU")
@pytest.mark.parametrize("cond", [2.0, 1e4, 1e8])
def test_dpotrf_dchkpo_ratios(uplo, cond):
    """DCHKPO tests 1 and 3 (TESTING/LIN/dchkpo.f): DPOT01 and DPOT02 below
    THRESH on every N, NB and NRHS of dtest.in, reading only the UPLO
    triangle (the other triangle holds 1e300); blocked and unblocked
    factors agree on INFO for a matrix that is not positive definite."""
    for n in INPUTS["dtest"]["n"]:
        a = oracle.spd_matrix(n, cond, 31 + n, uplo)
        for nb in sorted(set(INPUTS["dtest"]["nb"])) + [64]:
            f, info = oracle.potrf(a, uplo, nb=nb)
            assert info == 0
            if n:
                assert ck.dpot01(a, f, uplo) < THRESH, (n, nb)
        for nrhs in INPUTS["dtest"]["nrhs"]:
            xact = oracle.random_matrix(n, nrhs, 7 + n, idist=2)[0]
            b = ck._sym_full(a, uplo) @ xact
            x, info = oracle.potrs(f, b, uplo)
            assert info == 0
            if n:
                assert ck.dpot02(a, x, b, uplo) < THRESH
        if n >= 3:
            bad = a.copy()
            bad[n // 2, n // 2] = -1.0
            infos = {oracle.potrf(bad, uplo, nb=nb)[1] for nb in (1, 2, 3, 64)}
            assert len(infos) == 1 and infos.pop() > 0


@pytest.mark.parametrize("uplo", "LU")
@pytest.mark.parametrize("nrhs", INPUTS["dstest"]["nrhs"])
def test_dsposv_ddrvac_ratios(uplo, nrhs):
    """DDRVAC (TESTING/LIN/ddrvac.f): for ITER >= 0 the DPOT06 ratio is below
    sqrt(N) and A is returned unchanged; an ill-conditioned matrix drives
    the FP64 fallback (ITER < 0) with DPOT06 below THRESH."""
    for n in INPUTS["dstest"]["n"]:
        for cond in (2.0, 1e3, 1e10):
            a = oracle.spd_matrix(n, cond, 91 + n, uplo)
            xact = oracle.random_matrix(n, nrhs, 5 + n, idist=2)[0]
            b = ck._sym_full(a, uplo) @ xact if n else np.zeros((0, nrhs))
            ao, x, it, info = oracle.dsposv(a, b, uplo)
            assert info == 0
            if n == 0:
                continue
            r = ck.dpot06(a, x, b, uplo)
            if it >= 0:
                assert r < np.sqrt(n) or r < 1.0, (n, cond, it, r)
                assert np.array_equal(ao, a)
            else:
                assert r < THRESH, (n, cond, it, r)
            if cond >= 1e10 and n >= 10:
                assert it < 0


def test_oracle_ipiv_matches_openblas():
    scipy_linalg = pytest.importorskip("scipy.linalg")
    for n, seed in ((64, 1), (200, 2), (513, 3)):
        a = oracle.random_matrix(n, n, seed, idist=3)[0]
        lu, ip, info = oracle.getrf(a)
        lu2, piv2 = scipy_linalg.lu_factor(a)
        assert np.array_equal(piv2 + 1, ip)
        assert ck.lu_rel_diff(lu, lu2, a) < 64.0


def test_pivot_margins_recorded():
    a = oracle.random_matrix(100, 100, 4, idist=3)[0]
    lu, ip, info, margin = oracle.getrf(a, margins=True)
    assert margin.shape == (100,) and np.all(margin >= 0) and np.all(margin <= 1)
    b = a.copy()
    b[0, 0] = b[1, 0] = 10.0                      # exact tie in column 1: IDAMAX takes the first
    lu, ip, info, margin = oracle.getrf(b, margins=True)
    assert ip[0] == 1 and margin[0] == 0.0


def test_idamax_nan_rule():
    # BLAS/SRC/idamax.f:101-107: a NaN is only chosen when it is element 1
    L = oracle.lib()
    x = np.array([1.0, np.nan, 3.0, -3.0])
    assert L.or_diamax(4, x.ctypes.data_as(oracle.ctypes.c_void_p), 1) == 3
    y = np.array([np.nan, 5.0, 7.0])
    assert L.or_diamax(3, y.ctypes.data_as(oracle.ctypes.c_void_p), 1) == 1


ERR_GETRF = [((-1, 0, 1), -1), ((0, -1, 1), -2), ((2, 1, 1), -4)]          # TESTING/LIN/derrge.f:133-142
ERR_GETRS = [(("/", 0, 0, 1, 1), -1), (("N", -1, 0, 1, 1), -2), (("N", 0, -1, 1, 1), -3),
             (("N", 2, 1, 1, 2), -5), (("N", 2, 1, 2, 1), -8)]              # derrge.f:169-184
ERR_DSGESV = [((-1, 0, 1, 1, 1), -1), ((0, -1, 1, 1, 1), -2), ((2, 1, 1, 2, 2), -4),
              ((2, 1, 2, 1, 2), -7), ((2, 1, 2, 2, 1), -9)]                 # TESTING/LIN/derrab.f:113-127
ERR_GERFS = [(("/", 0, 0, 1, 1, 1, 1), -1), (("N", -1, 0, 1, 1, 1, 1), -2), (("N", 0, -1, 1, 1, 1, 1), -3),
             (("N", 2, 1, 1, 2, 2, 2), -5), (("N", 2, 1, 2, 1, 2, 2), -7), (("N", 2, 1, 2, 2, 1, 2), -10),
             (("N", 2, 1, 2, 2, 2, 1), -12)]                                 # TESTING/LIN/derrge.f:186-216
ERR_GECON = [(("/", 0, 1), -1), (("1", -1, 1), -2), (("1", 2, 1), -4)]     # TESTING/LIN/derrge.f:218-229
ERR_GETRI = [((-1, 1, 64), -1), ((2, 1, 64), -3)]                          # TESTING/LIN/derrge.f:157-165
ERR_POTRF = [(("/", 0, 1), -1), (("U", -1, 1), -2), (("U", 2, 1), -4)]     # TESTING/LIN/derrpo.f:133-142
ERR_POTRS = [(("/", 0, 0, 1, 1), -1), (("U", -1, 0, 1, 1), -2), (("U", 0, -1, 1, 1), -3),
             (("U", 2, 1, 1, 2), -5), (("U", 2, 1, 2, 1), -7)]                # derrpo.f:172-187
ERR_DSPOSV = [(("/", 0, 0, 1, 1, 1), -1), (("U", -1, 0, 1, 1, 1), -2), (("U", 0, -1, 1, 1, 1), -3),
              (("U", 2, 1, 1, 2, 2), -5), (("U", 2, 1, 2, 1, 2), -7),
              (("U", 2, 1, 2, 2, 1), -9)]                                      # TESTING/LIN/derrac.f:110-128
ERR_GEEQU = [((-1, 0, 1), -1), ((0, -1, 1), -2), ((2, 2, 1), -4)]          # TESTING/LIN/derrge.f:231-242


def _oracle_err(fn, *args):
    oracle.xerbla_reset()
    fn(*args)
    return oracle.xerbla_last()


def test_oracle_error_exits():
    import ctypes
    L = oracle.lib()
    a = np.zeros(16)
    ip = np.zeros(4, dtype=np.int32)
    info = np.zeros(1, dtype=np.int32)
    p = lambda v: v.ctypes.data_as(ctypes.c_void_p)
    for (m, n, lda), code in ERR_GETRF:
        name, inf = _oracle_err(L.or_dgetrf_nb, m, n, p(a), lda, p(ip), p(info), 64)
        assert (name, inf) == ("DGETRF", -code)
    for (tr, n, nrhs, lda, ldb), code in ERR_GETRS:
        name, inf = _oracle_err(L.or_dgetrs, tr.encode(), n, nrhs, p(a), lda, p(ip), p(a), ldb, p(info))
        assert (name, inf) == ("DGETRS", -code)
    L.or_dsgesv.argtypes = [ctypes.c_int] * 2 + [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                                                  ctypes.c_int, ctypes.c_void_p, ctypes.c_int] + [ctypes.c_void_p] * 4
    for (n, nrhs, lda, ldb, ldx), code in ERR_DSGESV:
        name, inf = _oracle_err(L.or_dsgesv, n, nrhs, p(a), lda, p(ip), p(a), ldb, p(a), ldx, p(a), p(a),
                                p(info), p(info))
        assert (name, inf) == ("DSGESV", -code)
    w = np.zeros(8)
    iw = np.zeros(4, dtype=np.int32)
    for (tr, n, nrhs, lda, ldaf, ldb, ldx), code in ERR_GERFS:
        name, inf = _oracle_err(L.or_dgerfs, tr.encode(), n, nrhs, p(a), lda, p(a), ldaf, p(ip), p(a), ldb, p(a),
                                ldx, p(w), p(w), p(w), p(iw), p(info))
        assert (name, inf) == ("DGERFS", -code)
    rc = np.zeros(1)
    for (nm, n, lda), code in ERR_GECON:
        name, inf = _oracle_err(L.or_dgecon, nm.encode(), n, p(a), lda, 1.0, p(rc), p(w), p(iw), p(info))
        assert (name, inf) == ("DGECON", -code)
    wk = np.zeros(256)
    for (n, lda, lw), code in ERR_GETRI:
        name, inf = _oracle_err(L.or_dgetri, n, p(a), lda, p(ip), p(wk), lw, 64, p(info))
        assert (name, inf) == ("DGETRI", -code)
    for (ul, n, lda), code in ERR_POTRF:
        name, inf = _oracle_err(L.or_dpotrf_nb, ul.encode(), n, p(a), lda, p(info), 64)
        assert (name, inf) == ("DPOTRF", -code)
    for (ul, n, nrhs, lda, ldb), code in ERR_POTRS:
        name, inf = _oracle_err(L.or_dpotrs, ul.encode(), n, nrhs, p(a), lda, p(a), ldb, p(info))
        assert (name, inf) == ("DPOTRS", -code)
    for (ul, n, nrhs, lda, ldb, ldx), code in ERR_DSPOSV:
        name, inf = _oracle_err(L.or_dsposv, ul.encode(), n, nrhs, p(a), lda, p(a), ldb, p(a), ldx, p(wk), p(wk),
                                p(info), p(info))
        assert (name, inf) == ("DSPOSV", -code)
    for (m, n, lda), code in ERR_GEEQU:
        name, inf = _oracle_err(L.or_dgeequ, m, n, p(a), lda, p(w), p(w), p(w), p(w), p(w), p(info))
        assert (name, inf) == ("DGEEQU", -code)


# ------------------------------------------------------------------ complex LU
@pytest.mark.parametrize("imat", range(1, 12))
@pytest.mark.parametrize("nb", sorted(set(INPUTS["dtest"]["nb"])))
def test_zgetrf_zchkge_ratios(imat, nb):
    """ZCHKGE tests 1 and 3 (TESTING/LIN/zchkge.f, the complex twin of
    DCHKGE) on every M x N of dtest.in: INFO = IZERO for the zero-column
    types, ZGET01 < THRESH, and ZGET02 < THRESH for TRANS = N, T, C."""
    for m in INPUTS["dtest"]["m"]:
        for n in INPUTS["dtest"]["n"]:
            if 5 <= imat <= 7 and n < imat - 4:
                continue
            a, izero = oracle.zge_test_matrix(m, n, imat, 2011 + 7 * m + n)
            lu, ipiv, info = oracle.zgetrf(a, nb=nb)
            assert info == izero, (m, n, imat, info, izero)
            if m and n:
                assert ck.zget01(a, lu, ipiv) < THRESH, (m, n, imat)
            if m == n and n > 0 and izero == 0:
                for nrhs in INPUTS["dtest"]["nrhs"]:
                    xact = oracle.random_zmatrix(n, nrhs, 5 + n + nrhs)
                    for trans in "NTC":
                        op = a if trans == "N" else (a.T if trans == "T" else a.conj().T)
                        b = op @ xact
                        x, info = oracle.zgetrs(lu, ipiv, b, trans)
                        assert info == 0
                        assert ck.zget02(a, x, b, trans) < THRESH, (n, imat, trans)


def test_zgetrf_blocked_equals_recursive_and_ipiv_matches_openblas():
    """ZGETRF with NB = 64 and ZGETRF2 alone apply each element's updates in
    the same order: identical bits.  OpenBLAS's zgetrf (through scipy, an
    independent implementation) picks the same pivots on random matrices."""
    import scipy.linalg as sl
    for n, seed in ((150, 3), (200, 4), (257, 5)):
        a = oracle.random_zmatrix(n, n, seed)
        lu, ip, info = oracle.zgetrf(a, nb=64)
        lu2, ip2, _ = oracle.zgetrf(a, nb=1)
        assert info == 0 and np.array_equal(ip, ip2)
        assert lu.tobytes() == lu2.tobytes()
        _, piv = sl.lu_factor(a)
        assert np.array_equal(ip, piv + 1)


def test_izamax_rules():
    """IZAMAX (BLAS/SRC/izamax.f90): first maximum of |re| + |im|; the first
    NaN wins outright; an infinite part wins unless a NaN follows; the
    0.25-scaled comparison once |re| + |im| overflows."""
    z = lambda *v: np.array(v, dtype=np.complex128)
    assert oracle.izamax(z()) == 0
    assert oracle.izamax(z(5 + 5j)) == 1
    assert oracle.izamax(z(1 + 1j, -2 + 0j, 0 + 2j)) == 1       # ties: the first
    assert oracle.izamax(z(1 + 1j, -2.5 + 0j, 0 + 2j)) == 2
    assert oracle.izamax(z(1, complex(np.nan, 0), 1e300)) == 2
    assert oracle.izamax(z(1, complex(np.inf, 0), 3, complex(0, np.nan))) == 4
    assert oracle.izamax(z(1, complex(0, -np.inf), 3)) == 2
    big = 1.5e308
    assert oracle.izamax(z(1, complex(big, big), complex(big, 0.9 * big), complex(big, 1.1 * big))) == 4


ERR_ZGETRF = [((-1, 0, 1), -1), ((0, -1, 1), -2), ((2, 1, 1), -4)]          # TESTING/LIN/zerrge.f:135-144
ERR_ZGETRS = [(("/", 0, 0, 1, 1), -1), (("N", -1, 0, 1, 1), -2), (("N", 0, -1, 1, 1), -3),
              (("N", 2, 1, 1, 2), -5), (("N", 2, 1, 2, 1), -8)]              # zerrge.f:174-190
ERR_ZGESV = [((-1, 0, 1, 1), -1), ((0, -1, 1, 1), -2), ((2, 1, 1, 2), -4), ((2, 1, 2, 1), -7)]  # zerrvx.f:142-154


def test_oracle_complex_error_exits():
    L = oracle.lib()
    a = np.zeros(16, dtype=np.complex128)
    ip = np.zeros(4, dtype=np.int32)
    info = np.zeros(1, dtype=np.int32)
    p = lambda v: v.ctypes.data_as(ctypes.c_void_p)
    for (m, n, lda), code in ERR_ZGETRF:
        assert _oracle_err(L.or_zgetrf_nb, m, n, p(a), lda, p(ip), p(info), 64) == ("ZGETRF", -code)
        assert _oracle_err(L.or_cgetrf_nb, m, n, p(a), lda, p(ip), p(info), 64) == ("CGETRF", -code)
    for (tr, n, nrhs, lda, ldb), code in ERR_ZGETRS:
        assert _oracle_err(L.or_zgetrs, tr.encode(), n, nrhs, p(a), lda, p(ip), p(a), ldb, p(info)) == ("ZGETRS", -code)
    for (n, nrhs, lda, ldb), code in ERR_ZGESV:
        name, inf = _oracle_err(L.or_zgesv, n, nrhs, p(a), lda, p(ip), p(a), ldb, p(info))
        assert (name.strip(), inf) == ("ZGESV", -code)


@pytest.mark.parametrize("nrhs", INPUTS["dstest"]["nrhs"])
def test_zcgesv_zdrvab_ratios(nrhs):
    """ZDRVAB (TESTING/LIN/zdrvab.f:315-366) on the dstest.in sizes and the
    ZCHKGE matrix types: INFO = IZERO; ZGET08 < sqrt(N) when ITER >= 0,
    < THRESH when the refinement fell back (ITER < 0); A unchanged when
    ITER >= 0, and ITER < 0 for the ill-conditioned types."""
    for n in INPUTS["dstest"]["n"]:
        for imat in range(1, 12):
            if 5 <= imat <= 7 and n < imat - 4:
                continue
            a, izero = oracle.zge_test_matrix(n, n, imat, 1988 + 3 * n + imat)
            xact = oracle.random_zmatrix(n, nrhs, 7 + n)
            b = a @ xact
            ao, ipiv, x, it, info = oracle.zcgesv(a, b)
            assert info == izero, (n, imat, info, izero)
            if info or n == 0:
                continue
            r = ck.zget08(a, x, b)
            if it >= 0:
                assert r < np.sqrt(n), (n, imat, it, r)
                assert ao.tobytes() == np.asfortranarray(a).tobytes()
            else:
                assert r < THRESH, (n, imat, it, r)


def test_zcgesv_fallback_and_exit_codes():
    """ITER = -31 with the COMPLEX*16 solution for a system too ill
    conditioned for COMPLEX refinement; ITER = -2 when B does not fit
    COMPLEX (ZLAG2C overflow); ITER = -3 when CGETRF finds a zero pivot that
    ZGETRF does not (an entry that rounds to 0 in single precision)."""
    n = 60
    u, _ = np.linalg.qr(oracle.random_zmatrix(n, n, 1))
    v, _ = np.linalg.qr(oracle.random_zmatrix(n, n, 2))
    a = (u * 1e12 ** (-np.arange(n) / (n - 1))) @ v.conj().T
    xt = oracle.random_zmatrix(n, 1, 3)
    b = a @ xt
    ao, ip, x, it, info = oracle.zcgesv(a, b)
    assert it == -31 and info == 0 and ck.zget08(a, x, b) < THRESH
    lu, ip2, _ = oracle.zgetrf(a)
    assert ao.tobytes() == lu.tobytes() and np.array_equal(ip, ip2)
    big = b.copy()
    big[3, 0] = complex(1.0, 1e39)
    assert oracle.zcgesv(a, big)[3] == -2
    d = np.diag([1.0, 1e-50, 1.0]).astype(np.complex128)
    _, _, x, it, info = oracle.zcgesv(d, np.ones((3, 1), dtype=np.complex128))
    assert it == -3 and info == 0 and abs(x[1, 0] - 1e50) < 1e36


@pytest.mark.parametrize("imat", range(1, 12))
def test_cgetrf_cchkge_ratios(imat):
    """CCHKGE tests 1 and 3 (the COMPLEX twin of ZCHKGE) with the COMPLEX eps:
    INFO = IZERO, CGET01 < THRESH, CGET02 < THRESH for TRANS = N, T, C; the
    ill-conditioned types 8 and 9 are skipped for the solve as single
    precision cannot reach them."""
    for n in INPUTS["dtest"]["n"]:
        if 5 <= imat <= 7 and n < imat - 4:
            continue
        a, izero = oracle.zge_test_matrix(n, n, imat, 2011 + 7 * n)
        if imat >= 10:
            a = a * (1e-30 / 1e-290 if imat == 10 else 1e30 / 1e290)   # scalings inside COMPLEX's range
        a = a.astype(np.complex64)
        lu, ipiv, info = oracle.zgetrf(a, dtype=np.complex64)
        assert info == izero, (n, imat, info, izero)
        if n:
            assert ck.zget01(a, lu, ipiv) < THRESH, (n, imat)
        if n and izero == 0 and imat not in (8, 9):
            xact = oracle.random_zmatrix(n, 2, 5 + n).astype(np.complex64)
            for trans in "NTC":
                op = a if trans == "N" else (a.T if trans == "T" else a.conj().T)
                b = (op.astype(np.complex128) @ xact).astype(np.complex64)
                x, info = oracle.zgetrs(lu, ipiv, b, trans)
                assert info == 0 and ck.zget02(a, x, b, trans) < THRESH, (n, imat, trans)
