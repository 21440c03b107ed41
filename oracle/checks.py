"""ORACLE test infrastructure: the reference test-suite ratios restated in
numpy (TESTING/LIN).  Each returns the same scaled quantity the reference
test prints; a result passes when it is below THRESH (30 in
TESTING/dtest.in), or below sqrt(N) for DSGESV with ITER >= 0
(TESTING/LIN/ddrvab.f:362-365)."""
import numpy as np

EPS64 = np.finfo(np.float64).eps / 2      # DLAMCH('Epsilon'), INSTALL/dlamch.f:101-110
EPS32 = np.finfo(np.float32).eps / 2


def _ref_residual(a, x, b, trans="N"):
    """B - op(A) X with the oracle's restatement of the reference DGEMM
    (BLAS/SRC/dgemm.f), the call DGET02 / DGET08 make, so the ratio is the one
    the reference test computes."""
    import ctypes
    import oracle
    a = np.asfortranarray(np.asarray(a, dtype=np.float64))
    r = np.asfortranarray(np.array(b, dtype=np.float64, copy=True))
    x = np.asfortranarray(np.asarray(x, dtype=np.float64))
    m, n = a.shape
    n1, n2 = (m, n) if trans == "N" else (n, m)
    nrhs = r.shape[1]
    if n1 == 0 or nrhs == 0:
        return r
    p = lambda v: v.ctypes.data_as(ctypes.c_void_p)
    oracle.lib().or_dgemm(trans.encode(), b"N", n1, nrhs, n2, -1.0, p(a), max(1, m), p(x), max(1, n2), 1.0, p(r),
                          max(1, n1))
    return r


def _eps(dtype):
    return EPS64 if np.dtype(dtype) == np.float64 else EPS32


def unpack_lu(lu, ipiv):
    """P, L, U from the LAPACK packed factor and 1-based IPIV (sequential swaps)."""
    m, n = lu.shape
    k = min(m, n)
    L = np.tril(lu[:, :k], -1) + np.eye(m, k)
    U = np.triu(lu[:k, :])
    perm = np.arange(m)
    for i in range(k):
        p = int(ipiv[i]) - 1
        perm[i], perm[p] = perm[p], perm[i]
    return perm, L, U


def dget01(a, lu, ipiv):
    """||P L U - A||_1 / (N ||A||_1 eps)  (TESTING/LIN/dget01.f:147-207)."""
    a = np.asarray(a, dtype=np.float64)
    m, n = a.shape
    if m == 0 or n == 0:
        return 0.0
    eps = _eps(lu.dtype)
    perm, L, U = unpack_lu(np.asarray(lu, dtype=np.float64), ipiv)
    prod = L @ U
    pa = a[perm, :]
    anorm = np.abs(a).sum(axis=0).max()
    resid = np.abs(prod - pa).sum(axis=0).max()
    if anorm <= 0:
        return 0.0 if resid == 0 else 1.0 / eps
    return ((resid / n) / anorm) / eps


def dget02(a, x, b, trans="N", eps=None):
    """max_j ||b_j - op(A) x_j||_1 / (||op(A)||_1 ||x_j||_1 eps)
    (TESTING/LIN/dget02.f:176-219)."""
    a = np.asarray(a, dtype=np.float64)
    x = np.asarray(x, dtype=np.float64).reshape(a.shape[1] if trans == "N" else a.shape[0], -1)
    b = np.asarray(b, dtype=np.float64).reshape(x.shape[0], -1)
    eps = EPS64 if eps is None else eps
    if a.size == 0 or x.shape[1] == 0:
        return 0.0
    anorm = np.abs(a).sum(axis=0).max() if trans == "N" else np.abs(a).sum(axis=1).max()
    if anorm <= 0:
        return 1.0 / eps
    r = _ref_residual(a, x, b, trans)
    resid = 0.0
    for j in range(x.shape[1]):
        xn = np.abs(x[:, j]).sum()
        if xn <= 0:
            return 1.0 / eps
        resid = max(resid, ((np.abs(r[:, j]).sum() / anorm) / xn) / eps)
    return resid


def dget04(x, xact, rcond, eps=None):
    """max_j ||x_j - xact_j||_inf / (||xact_j||_inf * eps) * rcond
    (TESTING/LIN/dget04.f:138-171)."""
    eps = EPS64 if eps is None else eps
    x = np.asarray(x, dtype=np.float64).reshape(np.asarray(xact).shape[0], -1)
    xact = np.asarray(xact, dtype=np.float64).reshape(x.shape)
    resid = 0.0
    for j in range(x.shape[1]):
        xn = np.abs(xact[:, j]).max() if x.shape[0] else 0.0
        d = np.abs(x[:, j] - xact[:, j]).max() if x.shape[0] else 0.0
        if xn <= 0:
            if d > 0:
                resid = 1.0 / eps
        else:
            resid = max(resid, (d / xn) * rcond)
    if resid * eps < 1.0:
        resid = resid / eps
    return resid


def dget08(a, x, b, eps=None):
    """max_j ||b_j - A x_j||_inf / (||A||_inf ||x_j||_inf eps)
    (TESTING/LIN/dget08.f:175-214)."""
    a = np.asarray(a, dtype=np.float64)
    eps = EPS64 if eps is None else eps
    x = np.asarray(x, dtype=np.float64).reshape(a.shape[1], -1)
    b = np.asarray(b, dtype=np.float64).reshape(a.shape[0], -1)
    if a.size == 0 or x.shape[1] == 0:
        return 0.0
    anorm = np.abs(a).sum(axis=1).max()
    if anorm <= 0:
        return 1.0 / eps
    r = _ref_residual(a, x, b)
    resid = 0.0
    for j in range(x.shape[1]):
        xn = np.abs(x[:, j]).max()
        if xn <= 0:
            return 1.0 / eps
        resid = max(resid, ((np.abs(r[:, j]).max() / anorm) / xn) / eps)
    return resid


def dget07(a, b, x, xact, ferr, berr, trans="N", chkferr=True, eps=None):
    """RESLTS(1), RESLTS(2) of TESTING/LIN/dget07.f:203-276: the forward error
    bound test max_j (||x_j - xact_j||_inf / ||x_j||_inf) / FERR(j) (1/eps when
    the bound is violated) and the backward error test
    max_j BERR(j) / ((n+1) eps + (n+1) unfl / max(min_i (|b| + |op(A)||x|)_i, (n+1) unfl))."""
    a = np.asarray(a, dtype=np.float64)
    n = a.shape[0]
    eps = EPS64 if eps is None else eps
    x = np.asarray(x, dtype=np.float64).reshape(n, -1)
    xact = np.asarray(xact, dtype=np.float64).reshape(n, -1)
    b = np.asarray(b, dtype=np.float64).reshape(n, -1)
    nrhs = x.shape[1]
    if n <= 0 or nrhs <= 0:
        return 0.0, 0.0
    unfl = np.finfo(np.float64).tiny                 # DLAMCH('Safe minimum')
    ovfl = 1.0 / unfl
    errbnd = 0.0
    if chkferr:
        for j in range(nrhs):
            xnorm = max(np.abs(x[:, j]).max(), unfl)
            diff = np.abs(x[:, j] - xact[:, j]).max()
            if not (xnorm > 1.0 or diff <= ovfl * xnorm):
                errbnd = 1.0 / eps
                continue
            if diff / xnorm <= ferr[j]:
                errbnd = max(errbnd, (diff / xnorm) / ferr[j])
            else:
                errbnd = 1.0 / eps
    opa = np.abs(a if trans == "N" else a.T)
    r2 = 0.0
    for k in range(nrhs):
        axbi = (np.abs(b[:, k]) + opa @ np.abs(x[:, k])).min()
        tmp = berr[k] / ((n + 1) * eps + (n + 1) * unfl / max(axbi, (n + 1) * unfl))
        r2 = tmp if k == 0 else max(r2, tmp)
    return errbnd, r2


def dget06(rcond, rcondc, eps=None):
    """TESTING/LIN/dget06.f:101-120: max(RCOND, RCONDC)/min(RCOND, RCONDC) -
    (1 - eps), or the nonzero one over eps when the other is zero."""
    eps = EPS64 if eps is None else eps
    if rcond > 0:
        if rcondc > 0:
            return max(rcond, rcondc) / min(rcond, rcondc) - (1 - eps)
        return rcond / eps
    if rcondc > 0:
        return rcondc / eps
    return 0.0

def dget03(a, ainv, eps=None):
    """TESTING/LIN/dget03.f:128-157: ||I - AINV*A||_1 * RCOND / (eps * n),
    RCOND = 1/(||A||_1 ||AINV||_1); returns (resid, rcond)."""
    a = np.asarray(a, dtype=np.float64)
    ainv = np.asarray(ainv, dtype=np.float64)
    n = a.shape[0]
    eps = EPS64 if eps is None else eps
    if n <= 0:
        return 0.0, 1.0
    anorm = np.abs(a).sum(axis=0).max()
    ainvnm = np.abs(ainv).sum(axis=0).max()
    if anorm <= 0 or ainvnm <= 0:
        return 1.0 / eps, 0.0
    rcond = (1.0 / anorm) / ainvnm
    w = -(ainv @ a)
    w[np.diag_indices(n)] += 1.0
    resid = np.abs(w).sum(axis=0).max()
    return ((resid * rcond) / eps) / n, rcond

def _sym_full(a, uplo):
    a = np.asarray(a, dtype=np.float64)
    t = np.tril(a) if uplo == "L" else np.triu(a)
    return t + t.T - np.diag(np.diag(t))


def dpot01(a, f, uplo="L", eps=None):
    """TESTING/LIN/dpot01.f: ||L L^T - A||_1 / (n ||A||_1 eps) (or U^T U),
    reading only the `uplo` triangles of A and of the factor."""
    n = a.shape[0]
    if n <= 0:
        return 0.0
    eps = EPS64 if eps is None else eps
    af = _sym_full(a, uplo)
    anorm = np.abs(af).sum(axis=0).max()
    if anorm <= 0:
        return 1.0 / eps
    f = np.asarray(f, dtype=np.float64)
    t = np.tril(f) if uplo == "L" else np.triu(f)
    prod = t @ t.T if uplo == "L" else t.T @ t
    return ((np.abs(prod - af).sum(axis=0).max() / n) / anorm) / eps


def dpot02(a, x, b, uplo="L", eps=None):
    """TESTING/LIN/dpot02.f: max_j ||b_j - A x_j||_1 / (||A||_1 ||x_j||_1 eps)."""
    af = _sym_full(a, uplo)
    n = af.shape[0]
    eps = EPS64 if eps is None else eps
    x = np.asarray(x, dtype=np.float64).reshape(n, -1)
    b = np.asarray(b, dtype=np.float64).reshape(n, -1)
    if n <= 0:
        return 0.0
    anorm = np.abs(af).sum(axis=0).max()
    if anorm <= 0:
        return 1.0 / eps
    r = b - af @ x
    out = 0.0
    for j in range(x.shape[1]):
        xn = np.abs(x[:, j]).sum()
        if xn <= 0:
            return 1.0 / eps
        out = max(out, ((np.abs(r[:, j]).sum() / anorm) / xn) / eps)
    return out


def dpot06(a, x, b, uplo="L", eps=None):
    """TESTING/LIN/dpot06.f: max_j ||b_j - A x_j||_inf / (||A||_inf ||x_j||_inf
    eps), the residual by the oracle's restatement of DSYMM (the call DPOT06
    makes) and ||A|| by DLANSY('I'), so the ratio is the reference test's."""
    import ctypes
    import oracle
    a = np.asfortranarray(np.asarray(a, dtype=np.float64))
    n = a.shape[0]
    eps = EPS64 if eps is None else eps
    x = np.asfortranarray(np.asarray(x, dtype=np.float64).reshape(n, -1))
    r = np.asfortranarray(np.array(b, dtype=np.float64).reshape(n, -1))
    if n <= 0:
        return 0.0
    anorm = oracle.dlansy("I", uplo, a)
    if anorm <= 0:
        return 1.0 / eps
    L = oracle.lib()
    L.or_dsymm_l.argtypes = [ctypes.c_char, ctypes.c_int, ctypes.c_int, ctypes.c_double] + \
        [ctypes.c_void_p, ctypes.c_int] * 3
    pp = lambda v: v.ctypes.data_as(ctypes.c_void_p)
    L.or_dsymm_l(uplo.encode(), n, x.shape[1], -1.0, pp(a), n, pp(x), n, pp(r), n)
    out = 0.0
    for j in range(x.shape[1]):
        xn = np.abs(x[:, j]).max()
        out = max(out, ((np.abs(r[:, j]).max() / anorm) / xn) / eps)
    return out

def scaled_residual(a, x, b):
    """||b - A x||_inf / (||A||_inf ||x||_inf n eps): the parity measure the
    GPU result must meet (at or below the oracle's own value)."""
    a = np.asarray(a, dtype=np.float64)
    n = a.shape[0]
    x = np.asarray(x, dtype=np.float64).reshape(n, -1)
    b = np.asarray(b, dtype=np.float64).reshape(n, -1)
    r = b - a @ x
    an = np.abs(a).sum(axis=1).max()
    out = 0.0
    for j in range(x.shape[1]):
        out = max(out, np.abs(r[:, j]).max() / (an * np.abs(x[:, j]).max() * n * EPS64))
    return out


def lu_rel_diff(lu_a, lu_b, a):
    """max |LU_a - LU_b| / (||A||_max * n * eps) -- the L/U agreement measure."""
    n = a.shape[0]
    scale = max(np.abs(a).max(), 1e-300) * max(n, 1) * _eps(lu_a.dtype)
    return float(np.abs(np.asarray(lu_a, np.float64) - np.asarray(lu_b, np.float64)).max() / scale)


def zget01(a, lu, ipiv):
    """||P L U - A||_1 / (N ||A||_1 eps) for complex factors, ZLANGE('1') on
    moduli (TESTING/LIN/zget01.f; CGET01 with the COMPLEX eps for complex64
    factors)."""
    eps = EPS32 if np.asarray(lu).dtype == np.complex64 else EPS64
    a = np.asarray(a, dtype=np.complex128)
    m, n = a.shape
    if m == 0 or n == 0:
        return 0.0
    perm, L, U = unpack_lu(np.asarray(lu, dtype=np.complex128), ipiv)
    anorm = np.abs(a).sum(axis=0).max()
    resid = np.abs(L @ U - a[perm, :]).sum(axis=0).max()
    if anorm <= 0:
        return 0.0 if resid == 0 else 1.0 / eps
    return ((resid / n) / anorm) / eps


def zget02(a, x, b, trans="N", eps=None):
    """max_j DZASUM(b_j - op(A) x_j) / (||op(A)||_1 DZASUM(x_j) eps)
    (TESTING/LIN/zget02.f): ZLANGE('1') for TRANS = 'N', ZLANGE('I')
    otherwise; DZASUM sums |re| + |im|.  eps defaults to the COMPLEX*16 one,
    or the COMPLEX one for a complex64 solution."""
    if eps is None:
        eps = EPS32 if np.asarray(x).dtype == np.complex64 else EPS64
    a = np.asarray(a, dtype=np.complex128)
    x = np.asarray(x, dtype=np.complex128).reshape(a.shape[0], -1)
    b = np.asarray(b, dtype=np.complex128).reshape(a.shape[0], -1)
    if a.size == 0 or x.shape[1] == 0:
        return 0.0
    anorm = np.abs(a).sum(axis=0).max() if trans == "N" else np.abs(a).sum(axis=1).max()
    if anorm <= 0:
        return 1.0 / eps
    op = a if trans == "N" else (a.T if trans == "T" else a.conj().T)
    r = b - op @ x
    dzasum = lambda v: np.abs(v.real).sum() + np.abs(v.imag).sum()
    resid = 0.0
    for j in range(x.shape[1]):
        xn = dzasum(x[:, j])
        if xn <= 0:
            return 1.0 / eps
        resid = max(resid, ((dzasum(r[:, j]) / anorm) / xn) / eps)
    return resid


def _ref_zresidual(a, x, b):
    """B - A X with the oracle's restatement of the reference ZGEMM
    (BLAS/SRC/zgemm.f), the call ZGET08 makes."""
    import ctypes
    import oracle

    class Z(ctypes.Structure):
        _fields_ = [("re", ctypes.c_double), ("im", ctypes.c_double)]

    a = np.asfortranarray(a, dtype=np.complex128)
    x = np.asfortranarray(x, dtype=np.complex128)
    r = np.asfortranarray(np.array(b, dtype=np.complex128, copy=True))
    m, k = a.shape
    if m == 0 or r.shape[1] == 0:
        return r
    p = lambda v: v.ctypes.data_as(ctypes.c_void_p)
    f = oracle.lib().or_zgemm_nn
    f.argtypes = [ctypes.c_int] * 3 + [Z, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_int,
                                        ctypes.c_void_p, ctypes.c_int]
    f(m, r.shape[1], k, Z(-1.0, 0.0), p(a), max(1, m), p(x), max(1, k), p(r), max(1, m))
    return r


def zget08(a, x, b):
    """max_j CABS1(r(IZAMAX r)) / (||A||_inf CABS1(x(IZAMAX x)) eps), r =
    b_j - A x_j (TESTING/LIN/zget08.f), ||A||_inf = ZLANGE('I') on moduli."""
    import oracle
    a = np.asarray(a, dtype=np.complex128)
    x = np.asarray(x, dtype=np.complex128).reshape(a.shape[1], -1)
    b = np.asarray(b, dtype=np.complex128).reshape(a.shape[0], -1)
    if a.size == 0 or x.shape[1] == 0:
        return 0.0
    anorm = np.abs(a).sum(axis=1).max()
    if anorm <= 0:
        return 1.0 / EPS64
    r = _ref_zresidual(a, x, b)
    cabs1 = lambda z: abs(z.real) + abs(z.imag)
    resid = 0.0
    for j in range(x.shape[1]):
        xn = cabs1(x[oracle.izamax(x[:, j]) - 1, j])
        if xn <= 0:
            return 1.0 / EPS64
        rn = cabs1(r[oracle.izamax(np.ascontiguousarray(r[:, j])) - 1, j])
        resid = max(resid, ((rn / anorm) / xn) / EPS64)
    return resid
