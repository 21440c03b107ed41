"""Streaming triangular solve (default mode): the four DGETRS cases
(SRC/dgetrs.f:187-217) against the oracle's DGETRS, at sizes around the
64-row block edges, with right-hand-side counts around the 4-wide groups,
in both precisions; and DSGESV with the diagonal blocks applied as their
inverses (option "trsv_inv"), which must converge to the same backward
error bound as substitution.

Tolerances: |x_gpu - x_ref| <= 1e3 * n * eps * max|x_ref| (the summation
order differs from the reference's), and the DGET02 ratio below the
reference's THRESH of 30.
"""
import numpy as np
import pytest

import oracle
import oracle.checks as ck

pytestmark = pytest.mark.gpu

EPS = {np.float64: ck.EPS64, np.float32: 2.0 ** -24}


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
@pytest.mark.parametrize("trans", ["N", "T"])
@pytest.mark.parametrize("n,nrhs", [(63, 1), (64, 4), (65, 5), (129, 3), (640, 9), (1000, 1), (2113, 2)])
def test_getrs_stream_vs_oracle(gpu, dtype, trans, n, nrhs):
    a = oracle.random_matrix(n, n, 31 + n, idist=3, dtype=dtype)[0]
    b = oracle.random_matrix(n, nrhs, 37 + n, idist=3, dtype=dtype)[0]
    lu, ip, info = oracle.getrf(a)
    assert info == 0
    x_r, _ = oracle.getrs(lu, ip, b, trans)
    x_g, info_g = gpu.getrs(lu, ip, b, trans)
    assert info_g == 0
    eps = EPS[dtype]
    assert np.abs(x_g.astype(np.float64) - x_r).max() <= 1e3 * n * eps * np.abs(x_r).max()
    if dtype == np.float64:
        assert ck.dget02(a, x_g, b, trans) < 30.0


@pytest.mark.parametrize("n,kappa", [(1500, 1e4), (3000, 1e6)])
def test_dsgesv_inverse_diagonal_blocks(gpu, n, kappa):
    a, _, _, _ = oracle.config_dsgesv_matrix(n, kappa, 8)
    xt = np.random.default_rng(8).standard_normal((n, 1))
    b = a @ xt
    res = {}
    for inv in (0, 1):
        old = gpu.set_option("trsv_inv", inv)
        try:
            res[inv] = gpu.dsgesv(a, b)
        finally:
            gpu.set_option("trsv_inv", old)
    for inv, (_, _, x, it, info) in res.items():
        assert info == 0 and it > 0, (inv, it, info)
        assert ck.dget08(a, x, b) < np.sqrt(n), (inv, ck.dget08(a, x, b))
    # the correction solves differ only in rounding: ITER within one
    assert abs(res[1][3] - res[0][3]) <= 1
