"""Cholesky on the GPU (SRC/dpotrf.f, SRC/dpotrs.f, SRC/dposv.f,
SRC/dsposv.f) against the oracle's restatement.

Exact mode: DPOTRF / SPOTRF factors, INFO and DPOTRS solutions bitwise equal
to the oracle's for both triangles (the other triangle holds a value that
would show if it were read).  Default mode: DCHKPO tests 1 and 3 (DPOT01,
DPOT02 below THRESH) and DDRVAC's DSPOSV checks (DPOT06 < sqrt(N) when the
refinement converges, A untouched then; the FP64 fallback otherwise)."""
import numpy as np
import pytest

import oracle
import oracle.checks as ck

pytestmark = pytest.mark.gpu
THRESH = 30.0


@pytest.mark.parametrize("uplo", "LU")
@pytest.mark.parametrize("dtype", [np.float64, np.float32])
@pytest.mark.parametrize("n", [1, 2, 7, 64, 65, 130, 300])
def test_potrf_exact_bitwise(gpu, exact_mode, uplo, dtype, n):
    a = oracle.spd_matrix(n, 1e3, 13 + n, uplo, dtype=dtype)
    ref, rinfo = oracle.potrf(a, uplo, nb=64)
    got, ginfo = gpu.potrf(a, uplo, dtype=dtype)
    assert ginfo == rinfo == 0
    assert got.tobytes(order="F") == ref.tobytes(order="F")
    xact = oracle.random_matrix(n, 3, 3 + n, idist=2)[0].astype(dtype)
    b = (ck._sym_full(a, uplo) @ xact).astype(dtype)
    xr, _ = oracle.potrs(ref, b, uplo)
    xg, info = gpu.potrs(got, b, uplo)
    assert info == 0
    assert xg.tobytes() == xr.tobytes()


@pytest.mark.parametrize("uplo", "LU")
def test_potrf_not_positive_definite(gpu, exact_mode, uplo):
    n = 150
    a = oracle.spd_matrix(n, 1e2, 5, uplo)
    a[100, 100] = -1.0
    ref, rinfo = oracle.potrf(a, uplo, nb=64)
    got, ginfo = gpu.potrf(a, uplo)
    assert rinfo > 0 and ginfo == rinfo
    assert got.tobytes(order="F") == ref.tobytes(order="F")


@pytest.mark.parametrize("uplo", "LU")
@pytest.mark.parametrize("cond", [2.0, 1e4, 1e8])
def test_potrf_dchkpo_ratios(gpu, uplo, cond):
    for n in (3, 10, 50, 200, 520):
        a = oracle.spd_matrix(n, cond, 41 + n, uplo)
        f, info = gpu.potrf(a, uplo)
        assert info == 0 and ck.dpot01(a, f, uplo) < THRESH, (n, cond)
        xact = oracle.random_matrix(n, 2, 9 + n, idist=2)[0]
        b = ck._sym_full(a, uplo) @ xact
        x, info = gpu.potrs(f, b, uplo)
        assert info == 0 and ck.dpot02(a, x, b, uplo) < THRESH
        f2, x2, info = gpu.posv(a, b, uplo)
        assert info == 0 and ck.dpot02(a, x2, b, uplo) < THRESH


@pytest.mark.parametrize("uplo", "LU")
@pytest.mark.parametrize("nrhs", [1, 2, 15])
def test_dsposv_ddrvac(gpu, uplo, nrhs):
    for n in (1, 2, 13, 45, 101, 132, 600):
        for cond in (2.0, 1e3, 1e10):
            a = oracle.spd_matrix(n, cond, 91 + n, uplo)
            xact = oracle.random_matrix(n, nrhs, 5 + n, idist=2)[0]
            b = ck._sym_full(a, uplo) @ xact
            ao, x, it, info = gpu.dsposv(a, b, uplo)
            assert info == 0
            r = ck.dpot06(a, x, b, uplo)
            if it >= 0:
                assert r < np.sqrt(n) or r < 1.0, (n, cond, it, r)
                assert ao.tobytes(order="F") == np.asfortranarray(a).tobytes(order="F")
            else:
                assert r < THRESH, (n, cond, it, r)
            if cond >= 1e10 and n >= 13:
                assert it < 0


def test_dsposv_exact_matches_oracle(gpu, exact_mode):
    """Exact mode: ITER and X equal the oracle's DSPOSV bit for bit."""
    for uplo in "LU":
        for n, cond in ((45, 1e3), (132, 1e5), (60, 1e10)):
            a = oracle.spd_matrix(n, cond, 7 + n, uplo)
            b = ck._sym_full(a, uplo) @ oracle.random_matrix(n, 2, 8 + n, idist=2)[0]
            _, xr, itr, infr = oracle.dsposv(a, b, uplo)
            _, xg, itg, infg = gpu.dsposv(a, b, uplo)
            assert (itg, infg) == (itr, infr)
            assert xg.tobytes() == xr.tobytes()
