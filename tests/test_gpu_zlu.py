"""Complex LU on the GPU (SRC/zgetrf.f, SRC/zgetrf2.f, SRC/zgetrs.f,
SRC/zgesv.f) against the oracle's restatement.

The GPU runs the reference's block loop and panel recursion with every
element's operations in the reference order, so factors, IPIV, INFO and
solutions are compared bit for bit with the oracle (NaN results counted
equal whatever their sign or payload).  The ZCHKGE ratios (ZGET01, ZGET02
below THRESH for TRANS = N, T, C) and the device entry points are checked
too."""
import ctypes

import numpy as np
import pytest

import oracle
import oracle.checks as ck

pytestmark = pytest.mark.gpu
THRESH = 30.0


def _same_bits(x, y):
    """Bitwise equality with every NaN counted equal to every NaN (IEEE 754
    leaves the sign and payload of a NaN result open)."""
    x = np.asfortranarray(x).ravel(order="F").view(np.float64)
    y = np.asfortranarray(y).ravel(order="F").view(np.float64)
    nx, ny = np.isnan(x), np.isnan(y)
    return x.shape == y.shape and np.array_equal(nx, ny) and x[~nx].tobytes() == y[~ny].tobytes()


@pytest.mark.parametrize("m,n", [(1, 1), (5, 1), (1, 5), (7, 7), (65, 65), (130, 97), (97, 130), (200, 200),
                                 (300, 300)])
def test_zgetrf_bitwise(gpu, m, n):
    a = oracle.random_zmatrix(m, n, 17 * m + n)
    lu_r, ip_r, info_r = oracle.zgetrf(a)
    lu_g, ip_g, info_g = gpu.zgetrf(a)
    assert info_g == info_r == 0
    assert np.array_equal(ip_g, ip_r)
    assert _same_bits(lu_g, lu_r)


@pytest.mark.parametrize("kind", ["zero_cols", "tiny", "signed_zeros", "inf"])
def test_zgetrf_edge_cases_bitwise(gpu, kind):
    """Zero columns (INFO = the first), pivots below the safe minimum (the
    division branch of ZGETRF2), signed zeros (ZTRSM's ALPHA*B and ZGEMM's
    ALPHA*B(L,J) products decide their signs), an infinite entry."""
    for m, n in ((40, 40), (130, 100)):
        a = oracle.random_zmatrix(m, n, 3 * m + n)
        if kind == "zero_cols":
            a[:, n // 3] = 0
            a[:, (2 * n) // 3] = 0
        elif kind == "tiny":
            a = a * 1e-309           # subnormal pivots: the division branch of ZGETRF2
        elif kind == "signed_zeros":
            rng = np.random.default_rng(m + n)
            re = np.where(rng.random((m, n)) < 0.3, np.where(rng.random((m, n)) < 0.5, 0.0, -0.0), a.real)
            im = np.where(rng.random((m, n)) < 0.3, -0.0, a.imag)
            a = re + 1j * im
        elif kind == "inf":
            a[m // 2, n // 2] = complex(np.inf, 1.0)
        lu_r, ip_r, info_r = oracle.zgetrf(a)
        lu_g, ip_g, info_g = gpu.zgetrf(a)
        assert info_g == info_r, (kind, m, n)
        assert np.array_equal(ip_g, ip_r)
        assert _same_bits(lu_g, lu_r)
        if kind == "zero_cols":
            assert info_g == n // 3 + 1


@pytest.mark.parametrize("trans", "NTC")
@pytest.mark.parametrize("n,nrhs", [(1, 1), (5, 3), (64, 2), (130, 4), (257, 1)])
def test_zgetrs_bitwise(gpu, trans, n, nrhs):
    a = oracle.random_zmatrix(n, n, 100 + n)
    lu, ip, info = oracle.zgetrf(a)
    assert info == 0
    b = oracle.random_zmatrix(n, nrhs, 200 + n)
    x_r, _ = oracle.zgetrs(lu, ip, b, trans)
    x_g, info = gpu.zgetrs(lu, ip, b, trans)
    assert info == 0
    assert _same_bits(x_g, x_r)


@pytest.mark.parametrize("trans", "NTC")
@pytest.mark.parametrize("n,nrhs,dtype", [(3000, 2, np.complex128), (6200, 1, np.complex128),
                                          (12300, 1, np.complex64)])
def test_zgetrs_long_columns_bitwise(gpu, trans, n, nrhs, dtype):
    """Long columns take the one-CTA-per-column solve ('N' both triangles,
    'T'/'C' upper; the column in shared memory up to 96 KB -- 6144
    COMPLEX*16 or 12288 COMPLEX elements -- else in place): X bitwise the
    oracle's.  The factors are a synthetic diagonally dominant LU with valid
    pivots (ZGETRS reads nothing else), so no large factorization runs."""
    rng = np.random.default_rng(n)
    lu = (rng.uniform(-1, 1, (n, n)) + 1j * rng.uniform(-1, 1, (n, n))) / n
    lu[np.diag_indices(n)] += 2.0 + 0.5j
    lu = lu.astype(dtype)
    ip = (np.arange(n) + 1 + rng.integers(0, 4, n)).clip(max=n).astype(np.int32)
    b = oracle.random_zmatrix(n, nrhs, 7 + n).astype(dtype)
    x_r, _ = oracle.zgetrs(lu, ip, b, trans)
    x_g, info = gpu.zgetrs(lu, ip, b, trans)
    assert info == 0
    assert _same_bits(x_g, x_r)


@pytest.mark.parametrize("imat", range(1, 12))
def test_zgesv_zchkge_ratios(gpu, imat):
    """ZCHKGE tests 1 and 3 on the GPU: INFO = IZERO for the zero-column
    types, ZGET01 < THRESH, ZGET02 < THRESH for TRANS = N, T, C; ZGESV's
    solution equal to the oracle's."""
    for n in (3, 10, 50, 200):
        if 5 <= imat <= 7 and n < imat - 4:
            continue
        a, izero = oracle.zge_test_matrix(n, n, imat, 2011 + 9 * n)
        lu, ipiv, info = gpu.zgetrf(a)
        assert info == izero, (n, imat, info, izero)
        assert ck.zget01(a, lu, ipiv) < THRESH, (n, imat)
        if izero:
            continue
        xact = oracle.random_zmatrix(n, 2, 5 + n)
        for trans in "NTC":
            op = a if trans == "N" else (a.T if trans == "T" else a.conj().T)
            b = op @ xact
            x, info = gpu.zgetrs(lu, ipiv, b, trans)
            assert info == 0 and ck.zget02(a, x, b, trans) < THRESH, (n, imat, trans)
        b = a @ xact
        _, ip_g, x_g, info_g = gpu.zgesv(a, b)
        _, ip_r, x_r, info_r = oracle.zgesv(a, b)
        assert info_g == info_r == 0 and np.array_equal(ip_g, ip_r)
        assert _same_bits(x_g, x_r)


def test_zgesv_singular_leaves_b(gpu):
    """ZGESV with a zero column: INFO > 0, the factorization completed, B
    not solved (SRC/zgesv.f:165-172)."""
    n = 20
    a = oracle.random_zmatrix(n, n, 4)
    a[:, 7] = 0
    b = oracle.random_zmatrix(n, 2, 5)
    lu_g, ip_g, x_g, info_g = gpu.zgesv(a, b)
    lu_r, ip_r, x_r, info_r = oracle.zgesv(a, b)
    assert info_g == info_r == 8
    assert _same_bits(lu_g, lu_r) and np.array_equal(ip_g, ip_r)
    assert np.asfortranarray(x_g).tobytes() == np.asfortranarray(b).tobytes()


def test_zgesv_device_api_matches_host_abi(gpu):
    import torch
    n, nrhs = 150, 3
    a = oracle.random_zmatrix(n, n, 77)
    b = oracle.random_zmatrix(n, nrhs, 78)
    lu_h, ip_h, x_h, info_h = gpu.zgesv(a, b)
    A = gpu.to_colmajor(a)
    B = gpu.to_colmajor(b)
    ip = torch.zeros(n, dtype=torch.int32, device="cuda")
    inf = ctypes.c_int(-7)
    lda, pa = gpu._colmajor_view(A)
    ldb, pb = gpu._colmajor_view(B)
    rc = gpu.lib().gb300_zgesv_dev(n, nrhs, ctypes.c_void_p(pa), lda, ctypes.c_void_p(ip.data_ptr()),
                                   ctypes.c_void_p(pb), ldb, ctypes.byref(inf), gpu._stream_ptr(None))
    torch.cuda.synchronize()
    assert rc == 0 and inf.value == 0 == info_h
    assert np.array_equal(ip.cpu().numpy(), ip_h)
    assert _same_bits(A.cpu().numpy(), lu_h)
    assert _same_bits(B.cpu().numpy(), x_h)


@pytest.mark.parametrize("m,n", [(1, 1), (7, 7), (130, 97), (200, 200)])
def test_cgetrf_cgetrs_bitwise(gpu, m, n):
    """The COMPLEX twins (CGETRF, CGETRS, CGESV) against the oracle's
    single-precision restatement."""
    a = oracle.random_zmatrix(m, n, 41 * m + n).astype(np.complex64)
    lu_r, ip_r, info_r = oracle.zgetrf(a, dtype=np.complex64)
    lu_g, ip_g, info_g = gpu.zgetrf(a, dtype=np.complex64)
    assert info_g == info_r == 0 and np.array_equal(ip_g, ip_r)
    assert _same_bits(lu_g, lu_r)
    if m == n:
        b = oracle.random_zmatrix(n, 2, 43 + n).astype(np.complex64)
        for trans in "NTC":
            x_r, _ = oracle.zgetrs(lu_r, ip_r, b, trans)
            x_g, info = gpu.zgetrs(lu_g, ip_g, b, trans)
            assert info == 0 and _same_bits(x_g, x_r)
        _, _, x_g, info = gpu.zgesv(a, b, dtype=np.complex64)
        _, _, x_r, _ = oracle.zgesv(a, b, dtype=np.complex64)
        assert info == 0 and _same_bits(x_g, x_r)


def _conditioned(n, kappa, seed):
    u, _ = np.linalg.qr(oracle.random_zmatrix(n, n, seed))
    v, _ = np.linalg.qr(oracle.random_zmatrix(n, n, seed + 1))
    return np.asfortranarray((u * kappa ** (-np.arange(n) / max(n - 1, 1))) @ v.conj().T)


@pytest.mark.parametrize("kappa", [1e1, 1e5, 1e12])
@pytest.mark.parametrize("n,nrhs", [(1, 1), (13, 2), (130, 1), (300, 3)])
def test_zcgesv_matches_oracle(gpu, kappa, n, nrhs):
    """ZCGESV: ITER, INFO, IPIV, X and (after a fallback) A equal to the
    oracle's; ZDRVAB's check (ZGET08 < sqrt(N) when ITER >= 0, < THRESH
    after the fallback).  ZLANGE's moduli come from the GPU's hypot, which
    can differ from the host's in the last bit; that moves CTE by an ulp and
    could change ITER only for a residual on the threshold itself."""
    a = _conditioned(n, kappa, 3 + n)
    b = a @ oracle.random_zmatrix(n, nrhs, 5 + n)
    ao_r, ip_r, x_r, it_r, info_r = oracle.zcgesv(a, b)
    ao_g, ip_g, x_g, it_g, info_g = gpu.zcgesv(a, b)
    assert (it_g, info_g) == (it_r, info_r)
    assert np.array_equal(ip_g, ip_r)
    assert _same_bits(x_g, x_r) and _same_bits(ao_g, ao_r)
    r = ck.zget08(a, x_g, b)
    assert r < (np.sqrt(n) if it_g >= 0 else THRESH) or (n == 1 and r < 1.0)
    if it_g >= 0:
        assert np.asfortranarray(ao_g).tobytes() == np.asfortranarray(a).tobytes()
    if kappa >= 1e12 and n >= 13:
        assert it_g == -31


def test_zcgesv_exit_codes(gpu):
    """ITER = -2 (B does not fit COMPLEX) and -3 (CGETRF meets a zero pivot
    that ZGETRF does not), with the COMPLEX*16 fallback's answer."""
    n = 30
    a = oracle.random_zmatrix(n, n, 8)
    b = a @ oracle.random_zmatrix(n, 1, 9)
    b[4, 0] = complex(1e39, 0.0)
    d = np.diag([1.0, 1e-50, 1.0]).astype(np.complex128)
    for aa, bb, want in ((a, b, -2), (d, np.ones((3, 1), np.complex128), -3)):
        ao_r, ip_r, x_r, it_r, info_r = oracle.zcgesv(aa, bb)
        ao_g, ip_g, x_g, it_g, info_g = gpu.zcgesv(aa, bb)
        assert it_g == it_r == want and info_g == info_r == 0
        assert _same_bits(x_g, x_r) and _same_bits(ao_g, ao_r) and np.array_equal(ip_g, ip_r)


@pytest.mark.parametrize("dtype", [np.complex128, np.complex64])
def test_zgetrf2_recursive_alone_bitwise(gpu, dtype):
    """xGETRF2 as its own entry point: the whole matrix by the recursion, as
    the oracle's ZGETRF with block size 1."""
    for m, n in ((90, 90), (120, 70), (70, 120)):
        a = oracle.random_zmatrix(m, n, 13 * m + n).astype(dtype)
        lu_r, ip_r, info_r = oracle.zgetrf(a, nb=1, dtype=dtype)
        lu_g, ip_g, info_g = gpu.zgetrf2(a, dtype=dtype)
        assert info_g == info_r == 0 and np.array_equal(ip_g, ip_r)
        assert _same_bits(lu_g, lu_r)
