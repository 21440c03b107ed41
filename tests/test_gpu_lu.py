"""Parity of the GPU DGETRF / SGETRF / DGETRS / DGESV / DLASWP with the
oracle (the C restatement of the reference routines).

Two arithmetic modes are checked:
  * exact (products rounded separately): every element's updates happen in
    the reference loop order, so LU, IPIV and X must be bitwise identical
    to the oracle for any block size;
  * default (fused multiply-add): IPIV identical wherever the oracle's pivot
    margin is above rounding, |LU_gpu - LU_ref| <= 64 * n * eps * max|A|,
    and the scaled residual ||b - Ax|| / (||A|| ||x|| n eps) at most 2x the
    oracle's own value (and below the reference THRESH of 30).
"""
import numpy as np
import pytest

import oracle
import oracle.checks as ck

pytestmark = pytest.mark.gpu

SHAPES = [(1, 1), (2, 2), (3, 3), (5, 5), (10, 10), (50, 50), (64, 64), (65, 65), (100, 100), (257, 257),
          (513, 513), (50, 10), (10, 50), (300, 130), (130, 300), (3, 1), (1, 3)]


def _rand(m, n, seed, dtype=np.float64):
    return oracle.random_matrix(m, n, seed, idist=3, dtype=dtype)[0]


def _ipiv_check(ip_gpu, ip_ref, margin, n, eps):
    diff = np.nonzero(ip_gpu != ip_ref)[0]
    if diff.size == 0:
        return True
    k = diff[0]
    # the first divergence must sit on a near-tie of the oracle's pivot search
    assert margin[k] < 1e4 * n * eps, f"IPIV differs at {k} with pivot margin {margin[k]}"
    return False


@pytest.mark.parametrize("m,n", SHAPES)
@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_getrf_exact_bitwise(gpu, exact_mode, m, n, dtype):
    a = _rand(m, n, 11 + m + 3 * n, dtype)
    lu_r, ip_r, info_r = oracle.getrf(a)
    lu_g, ip_g, info_g = gpu.getrf(a)
    assert info_g == info_r
    np.testing.assert_array_equal(ip_g, ip_r)
    assert lu_g.tobytes(order="F") == lu_r.tobytes(order="F"), "LU not bitwise identical"


@pytest.mark.parametrize("nb", [32, 64, 128, 200])
def test_getrf_exact_any_block_size(gpu, exact_mode, nb):
    a = _rand(400, 400, 5)
    lu_r, ip_r, _ = oracle.getrf(a)
    old = gpu.set_option("nb64", nb)
    try:
        lu_g, ip_g, _ = gpu.getrf(a)
    finally:
        gpu.set_option("nb64", old)
    np.testing.assert_array_equal(ip_g, ip_r)
    assert np.array_equal(lu_g, lu_r)


@pytest.mark.parametrize("m,n", SHAPES)
def test_getrf_fma_parity(gpu, m, n):
    a = _rand(m, n, 101 + m + n)
    lu_r, ip_r, info_r, margin = oracle.getrf(a, margins=True)
    lu_g, ip_g, info_g = gpu.getrf(a)
    assert info_g == info_r
    if _ipiv_check(ip_g, ip_r, margin, max(m, n), ck.EPS64):
        assert ck.lu_rel_diff(lu_g, lu_r, a) <= 64.0
    assert ck.dget01(a, lu_g, ip_g) < 30.0


@pytest.mark.parametrize("n,nrhs", [(1, 1), (5, 2), (64, 3), (200, 1), (333, 15), (1024, 1)])
@pytest.mark.parametrize("trans", ["N", "T"])
def test_getrs(gpu, n, nrhs, trans):
    a = _rand(n, n, 7 + n)
    b = _rand(n, nrhs, 9 + n)
    lu, ip, _ = oracle.getrf(a)
    x_r, info_r = oracle.getrs(lu, ip, b, trans)
    x_g, info_g = gpu.getrs(lu, ip, b, trans)
    assert info_g == info_r == 0
    scale = np.abs(x_r).max() * n * ck.EPS64 * 1e3
    assert np.abs(x_g - x_r).max() <= scale
    assert ck.dget02(a, x_g, b, trans) < 30.0


@pytest.mark.parametrize("trans", ["N", "T"])
def test_getrs_exact_bitwise(gpu, exact_mode, trans):
    a = _rand(700, 700, 3)
    b = _rand(700, 5, 4)
    lu, ip, _ = oracle.getrf(a)
    x_r, _ = oracle.getrs(lu, ip, b, trans)
    x_g, _ = gpu.getrs(lu, ip, b, trans)
    assert x_g.tobytes() == x_r.tobytes()


def test_dgesv_plain_case_n1024(gpu):
    """A iid N(0,1) from seed 0, b N(0,1) drawn next, n=1024 (the plain DGESV case)."""
    a, b = oracle.config_dgesv_small(1024, 0)
    lu_r, ip_r, x_r, info_r = oracle.gesv(a, b)
    lu_g, ip_g, x_g, info_g = gpu.gesv(a, b)
    assert info_g == info_r == 0
    np.testing.assert_array_equal(ip_g, ip_r)
    assert ck.lu_rel_diff(lu_g, lu_r, a) <= 64.0
    res_r = ck.scaled_residual(a, x_r, b)
    res_g = ck.scaled_residual(a, x_g, b)
    assert res_g <= max(2.0 * res_r, 1e-3), (res_g, res_r)


def test_dgesv_plain_case_exact(gpu, exact_mode):
    a, b = oracle.config_dgesv_small(1024, 0)
    lu_r, ip_r, x_r, _ = oracle.gesv(a, b)
    lu_g, ip_g, x_g, _ = gpu.gesv(a, b)
    np.testing.assert_array_equal(ip_g, ip_r)
    assert np.array_equal(lu_g, lu_r) and np.array_equal(x_g, x_r)
    assert ck.scaled_residual(a, x_g, b) == ck.scaled_residual(a, x_r, b)


def test_singular_info(gpu):
    # zero column 3 -> INFO = first exact zero on U's diagonal (SRC/dgetrf.f:88-91)
    a = _rand(20, 20, 8)
    a[:, 2] = 0.0
    lu_r, ip_r, info_r = oracle.getrf(a)
    lu_g, ip_g, info_g = gpu.getrf(a)
    assert info_r == 3 and info_g == 3
    b = _rand(20, 1, 9)
    _, _, x_g, info = gpu.gesv(a, b)
    assert info == 3
    np.testing.assert_array_equal(x_g, b)     # DGESV skips the solve


@pytest.mark.parametrize("incx", [1, -1])
def test_laswp(gpu, incx):
    a = _rand(40, 7, 2)
    ipiv = np.array([5, 2, 40, 4, 1, 33, 7, 8], dtype=np.int32)
    r = oracle.laswp(a, 2, 7, ipiv, incx)
    g = gpu.laswp(a, 2, 7, ipiv, incx)
    assert np.array_equal(r, g)
