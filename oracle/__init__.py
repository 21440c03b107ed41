"""ORACLE -- test infrastructure only.

ctypes bindings to ``liboracle.so``, the plain-C restatement of the reference
LAPACK dense LU solve path (see ``oracle.c`` for the per-routine citations),
plus seeded input generators.  Only ``tests/``, ``__graft_entry__.smoke`` and
the CPU-baseline leg of ``bench.py`` import this package, and only as the
checker or the timed CPU baseline.  The GPU library never calls into it.
"""
import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None

_i = ctypes.c_int
_d = ctypes.c_double
_f = ctypes.c_float
_p = ctypes.c_void_p
_c = ctypes.c_char


def build(ref=False):
    """Compile liboracle.so (and, with ref=True and the reference tree
    present, the reference LAPACKE wrappers over it into _ref/)."""
    subprocess.run(["make", "-s", "-C", _HERE, "liboracle.so"], check=True)
    if ref:
        subprocess.run(["make", "-s", "-C", _HERE, "ref"], check=True)


def lib():
    global _LIB
    if _LIB is None:
        path = os.path.join(_HERE, "liboracle.so")
        src = [os.path.join(_HERE, f) for f in ("oracle.c", "oracle_lu.inc", "oracle_chol.inc", "oracle_z.inc")]
        if not os.path.exists(path) or any(os.path.getmtime(s) > os.path.getmtime(path) for s in src):
            build()
        L = ctypes.CDLL(path)
        for pre, T in (("d", _d), ("s", _f)):
            getattr(L, f"or_{pre}getrf_nb").argtypes = [_i, _i, _p, _i, _p, _p, _i]
            getattr(L, f"or_{pre}getrf_margins").argtypes = [_i, _i, _p, _i, _p, _p, _i, _p]
            getattr(L, f"or_{pre}getrf2").argtypes = [_i, _i, _p, _i, _p, _p]
            getattr(L, f"or_{pre}getrs").argtypes = [_c, _i, _i, _p, _i, _p, _p, _i, _p]
            getattr(L, f"or_{pre}gesv").argtypes = [_i, _i, _p, _i, _p, _p, _i, _p]
            getattr(L, f"or_{pre}laswp").argtypes = [_i, _p, _i, _i, _i, _p, _i]
            getattr(L, f"or_{pre}gemm").argtypes = [_c, _c, _i, _i, _i, T, _p, _i, _p, _i, T, _p, _i]
            getattr(L, f"or_{pre}trsm_left").argtypes = [_c, _c, _c, _i, _i, T, _p, _i, _p, _i]
            getattr(L, f"or_{pre}lange").argtypes = [_c, _i, _i, _p, _i, _p]
            getattr(L, f"or_{pre}lange").restype = T
            getattr(L, f"or_{pre}iamax").argtypes = [_i, _p, _i]
        L.or_dsgesv.argtypes = [_i, _i, _p, _i, _p, _p, _i, _p, _i, _p, _p, _p, _p]
        L.or_dgerfs.argtypes = [_c, _i, _i, _p, _i, _p, _i, _p, _p, _i, _p, _i, _p, _p, _p, _p, _p]
        L.or_dlacn2.argtypes = [_i, _p, _p, _p, _p, _p, _p]
        L.or_dgecon.argtypes = [_c, _i, _p, _i, ctypes.c_double, _p, _p, _p, _p]
        L.or_dgesvx.argtypes = [_c, _c, _i, _i, _p, _i, _p, _i, _p, _p, _p, _p, _p, _i, _p, _i, _p, _p, _p, _p, _p,
                                _p]
        L.or_dgeequ.argtypes = [_i, _i, _p, _i, _p, _p, _p, _p, _p, _p]
        L.or_dgetri.argtypes = [_i, _p, _i, _p, _p, _i, _i, _p]
        for pre in "ds":
            getattr(L, f"or_{pre}potrf_nb").argtypes = [_c, _i, _p, _i, _p, _i]
            getattr(L, f"or_{pre}potrs").argtypes = [_c, _i, _i, _p, _i, _p, _i, _p]
        L.or_dsposv.argtypes = [_c, _i, _i, _p, _i, _p, _i, _p, _i, _p, _p, _p, _p]
        L.or_dlansy.argtypes = [_c, _c, _i, _p, _i, _p]
        L.or_dlansy.restype = ctypes.c_double
        L.or_dlatrs.argtypes = [_c, _c, _c, _c, _i, _p, _i, _p, _p, _p, _p]
        L.or_dtrsv.argtypes = [_c, _c, _c, _i, _p, _i, _p]
        L.or_dlag2s.argtypes = [_i, _i, _p, _i, _p, _i, _p]
        L.or_slag2d.argtypes = [_i, _i, _p, _i, _p, _i, _p]
        L.or_dlaruv.argtypes = [_p, _i, _p]
        L.or_dlarnv.argtypes = [_i, _p, ctypes.c_longlong, _p]
        L.or_dlaruv_power.argtypes = [_i, _p]
        L.or_seed_from_int.argtypes = [ctypes.c_longlong, _p]
        L.or_xerbla_last.argtypes = [_p, _i]
        for pre in "zc":
            getattr(L, f"or_{pre}getrf_nb").argtypes = [_i, _i, _p, _i, _p, _p, _i]
            getattr(L, f"or_{pre}getrf2").argtypes = [_i, _i, _p, _i, _p, _p]
            getattr(L, f"or_{pre}getrs").argtypes = [_c, _i, _i, _p, _i, _p, _p, _i, _p]
            getattr(L, f"or_{pre}gesv").argtypes = [_i, _i, _p, _i, _p, _p, _i, _p]
            getattr(L, f"or_{pre}iamax").argtypes = [_i, _p]
        L.or_zcgesv.argtypes = [_i, _i, _p, _i, _p, _p, _i, _p, _i, _p, _p, _p, _p, _p]
        L.or_zlange_inf.argtypes = [_i, _i, _p, _i, _p]
        L.or_zlange_inf.restype = _d
        L.or_dlamch.argtypes = [_c]
        L.or_dlamch.restype = _d
        L.or_slamch.argtypes = [_c]
        L.or_slamch.restype = _f
        _LIB = L
    return _LIB


def _as2d(b):
    b = np.asarray(b)
    return b.reshape(b.shape[0], b.shape[1] if b.ndim == 2 else 1)


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def _pre(a):
    return "d" if a.dtype == np.float64 else "s"


def _colmajor(a, dtype):
    return np.asfortranarray(np.array(a, dtype=dtype, copy=True))


# ---------------------------------------------------------------- routines
def getrf(a, nb=64, margins=False):
    """xGETRF (SRC/dgetrf.f) on a copy of ``a``: returns (lu, ipiv, info[, margin])."""
    a = _colmajor(a, a.dtype if a.dtype in (np.float32, np.float64) else np.float64)
    m, n = a.shape
    ipiv = np.zeros(max(1, min(m, n)), dtype=np.int32)
    info = np.zeros(1, dtype=np.int32)
    L = lib()
    lda = max(1, m)
    if margins:
        mg = np.ones(max(1, min(m, n)), dtype=np.float64)
        getattr(L, f"or_{_pre(a)}getrf_margins")(m, n, _ptr(a), lda, _ptr(ipiv), _ptr(info), nb, _ptr(mg))
        return a, ipiv[: min(m, n)], int(info[0]), mg[: min(m, n)]
    getattr(L, f"or_{_pre(a)}getrf_nb")(m, n, _ptr(a), lda, _ptr(ipiv), _ptr(info), nb)
    return a, ipiv[: min(m, n)], int(info[0])


def getrs(lu, ipiv, b, trans="N"):
    """xGETRS (SRC/dgetrs.f) on a copy of ``b``: returns (x, info)."""
    lu = _colmajor(lu, lu.dtype)
    b2 = _colmajor(_as2d(b), lu.dtype)
    n, nrhs = b2.shape
    ipiv = np.ascontiguousarray(ipiv, dtype=np.int32)
    info = np.zeros(1, dtype=np.int32)
    getattr(lib(), f"or_{_pre(lu)}getrs")(trans.encode(), n, nrhs, _ptr(lu), max(1, n), _ptr(ipiv),
                                          _ptr(b2), max(1, n), _ptr(info))
    return b2.reshape(b.shape), int(info[0])


def gerfs(a, af, ipiv, b, x, trans="N"):
    """DGERFS (SRC/dgerfs.f): refines a copy of ``x`` with the factors
    ``af``/``ipiv`` of ``a``; returns (x, ferr, berr, info)."""
    a = _colmajor(a, np.float64)
    af = _colmajor(af, np.float64)
    b2 = _colmajor(_as2d(b), np.float64)
    x2 = _colmajor(_as2d(x), np.float64).copy(order="F")
    n, nrhs = b2.shape
    ipiv = np.ascontiguousarray(ipiv, dtype=np.int32)
    ferr = np.zeros(max(nrhs, 1))
    berr = np.zeros(max(nrhs, 1))
    work = np.zeros(3 * max(n, 1))
    iwork = np.zeros(max(n, 1), dtype=np.int32)
    info = np.zeros(1, dtype=np.int32)
    ld = max(1, n)
    lib().or_dgerfs(trans.encode(), n, nrhs, _ptr(a), ld, _ptr(af), ld, _ptr(ipiv), _ptr(b2), ld, _ptr(x2), ld,
                    _ptr(ferr), _ptr(berr), _ptr(work), _ptr(iwork), _ptr(info))
    return x2.reshape(np.asarray(x).shape), ferr[:nrhs], berr[:nrhs], int(info[0])


def gecon(lu, anorm, norm="1"):
    """DGECON (SRC/dgecon.f): reciprocal condition number from the LU
    factors and the norm of A; returns (rcond, info)."""
    lu = _colmajor(lu, np.float64)
    n = lu.shape[0]
    rcond = np.zeros(1)
    work = np.zeros(4 * max(n, 1))
    iwork = np.zeros(max(n, 1), dtype=np.int32)
    info = np.zeros(1, dtype=np.int32)
    lib().or_dgecon(norm.encode(), n, _ptr(lu), max(1, n), float(anorm), _ptr(rcond), _ptr(work), _ptr(iwork),
                    _ptr(info))
    return float(rcond[0]), int(info[0])


def latrs(t, x, uplo, trans, diag, cnorm=None):
    """DLATRS (SRC/dlatrs.f) on the triangle of ``t``: returns (x, scale,
    cnorm); ``cnorm`` given means NORMIN = 'Y'."""
    t = _colmajor(t, np.float64)
    n = t.shape[0]
    x = np.array(x, dtype=np.float64, copy=True)
    scale = np.zeros(1)
    normin = b"N" if cnorm is None else b"Y"
    cn = np.zeros(max(n, 1)) if cnorm is None else np.array(cnorm, dtype=np.float64, copy=True)
    info = np.zeros(1, dtype=np.int32)
    lib().or_dlatrs(uplo.encode(), trans.encode(), diag.encode(), normin, n, _ptr(t), max(1, n), _ptr(x),
                    _ptr(scale), _ptr(cn), _ptr(info))
    return x, float(scale[0]), cn[:n]


def gesvx(a, b, fact="N", trans="N", af=None, ipiv=None, equed="N", r=None, c=None):
    """DGESVX (SRC/dgesvx.f).  Returns a dict with the outputs: a (possibly
    equilibrated), af, ipiv, equed, r, c, b (possibly scaled), x, rcond,
    ferr, berr, rpvgrw (WORK(1)), info."""
    a = _colmajor(a, np.float64).copy(order="F")
    b2 = _colmajor(_as2d(b), np.float64).copy(order="F")
    n, nrhs = b2.shape[0], b2.shape[1]
    ld = max(1, n)
    af = np.zeros((n, n), order="F") if af is None else _colmajor(af, np.float64).copy(order="F")
    ipiv = np.zeros(ld, dtype=np.int32) if ipiv is None else np.array(ipiv, dtype=np.int32)
    r = np.zeros(ld) if r is None else np.array(r, dtype=np.float64)
    c = np.zeros(ld) if c is None else np.array(c, dtype=np.float64)
    eq = ctypes.create_string_buffer(equed.encode(), 2)
    x = np.zeros((n, nrhs), order="F")
    rcond = np.zeros(1)
    ferr = np.zeros(max(nrhs, 1))
    berr = np.zeros(max(nrhs, 1))
    work = np.zeros(4 * ld)
    iwork = np.zeros(ld, dtype=np.int32)
    info = np.zeros(1, dtype=np.int32)
    lib().or_dgesvx(fact.encode(), trans.encode(), n, nrhs, _ptr(a), ld, _ptr(af), ld, _ptr(ipiv),
                    ctypes.cast(eq, ctypes.c_void_p), _ptr(r), _ptr(c), _ptr(b2), ld, _ptr(x), ld, _ptr(rcond),
                    _ptr(ferr), _ptr(berr), _ptr(work), _ptr(iwork), _ptr(info))
    return dict(a=a, af=af, ipiv=ipiv[:n], equed=eq.value.decode(), r=r[:n], c=c[:n], b=b2, x=x,
                rcond=float(rcond[0]), ferr=ferr[:nrhs], berr=berr[:nrhs], rpvgrw=float(work[0]), info=int(info[0]))


def geequ(a):
    """DGEEQU (SRC/dgeequ.f): returns (r, c, rowcnd, colcnd, amax, info)."""
    a = _colmajor(a, np.float64)
    m, n = a.shape
    r = np.zeros(max(m, 1))
    c = np.zeros(max(n, 1))
    sc = np.zeros(3)
    info = np.zeros(1, dtype=np.int32)
    lib().or_dgeequ(m, n, _ptr(a), max(1, m), _ptr(r), _ptr(c), _ptr(sc[0:]), _ptr(sc[1:]), _ptr(sc[2:]),
                    _ptr(info))
    return r[:m], c[:n], float(sc[0]), float(sc[1]), float(sc[2]), int(info[0])


def getri(lu, ipiv, nb=64, lwork=None):
    """DGETRI (SRC/dgetri.f) on a copy of the factors with block size nb;
    returns (ainv, info, work0)."""
    a = _colmajor(lu, np.float64).copy(order="F")
    n = a.shape[0]
    ipiv = np.ascontiguousarray(ipiv, dtype=np.int32)
    lw = max(1, n * max(nb, 1)) if lwork is None else lwork
    work = np.zeros(max(1, lw, n * max(nb, 1)))
    info = np.zeros(1, dtype=np.int32)
    lib().or_dgetri(n, _ptr(a), max(1, n), _ptr(ipiv), _ptr(work), lw, nb, _ptr(info))
    return a, int(info[0]), float(work[0])


def spd_matrix(n, cond, seed, uplo="L", junk=1e300, dtype=np.float64):
    """A symmetric positive definite test matrix Q diag(d) Q^T with d
    geometric from 1 to 1/cond (Q from the QR of a seeded N(0,1) matrix);
    only the `uplo` triangle is meaningful, the other holds `junk` so that a
    routine reading it is caught."""
    if n == 0:
        return np.zeros((0, 0), dtype=dtype)
    g = random_matrix(n, n, seed, idist=3)[0]
    q, _ = np.linalg.qr(g)
    d = cond ** (-np.arange(n) / max(n - 1, 1))
    a = (q * d) @ q.T
    a = (a + a.T) / 2
    full = a.astype(dtype)
    out = np.tril(full) if uplo == "L" else np.triu(full)
    mask = np.triu(np.ones((n, n), bool), 1) if uplo == "L" else np.tril(np.ones((n, n), bool), -1)
    out[mask] = min(junk, float(np.finfo(dtype).max) / 16)
    return out


def potrf(a, uplo="L", nb=64):
    """xPOTRF (SRC/dpotrf.f) with block size nb: returns (factor, info)."""
    dt = np.dtype(a.dtype if a.dtype in (np.float32, np.float64) else np.float64)
    a = _colmajor(a, dt).copy(order="F")
    n = a.shape[0]
    info = np.zeros(1, dtype=np.int32)
    getattr(lib(), f"or_{_pre(a)}potrf_nb")(uplo.encode(), n, _ptr(a), max(1, n), _ptr(info), nb)
    return a, int(info[0])


def potrs(f, b, uplo="L"):
    """xPOTRS (SRC/dpotrs.f): returns (x, info)."""
    dt = f.dtype
    f = _colmajor(f, dt)
    b2 = _colmajor(_as2d(b), dt).copy(order="F")
    n, nrhs = b2.shape
    info = np.zeros(1, dtype=np.int32)
    getattr(lib(), f"or_{_pre(f)}potrs")(uplo.encode(), n, nrhs, _ptr(f), max(1, n), _ptr(b2), max(1, n),
                                          _ptr(info))
    return b2.reshape(np.asarray(b).shape), int(info[0])


def dsposv(a, b, uplo="L"):
    """DSPOSV (SRC/dsposv.f): returns (a_out, x, iter, info)."""
    a = _colmajor(a, np.float64).copy(order="F")
    b2 = _colmajor(_as2d(b), np.float64)
    n, nrhs = b2.shape
    x = np.zeros((n, nrhs), order="F")
    work = np.zeros(max(1, n * nrhs))
    swork = np.zeros(max(1, n * (n + nrhs)), dtype=np.float32)
    it = np.zeros(1, dtype=np.int32)
    info = np.zeros(1, dtype=np.int32)
    lib().or_dsposv(uplo.encode(), n, nrhs, _ptr(a), max(1, n), _ptr(b2), max(1, n), _ptr(x), max(1, n),
                    _ptr(work), _ptr(swork), _ptr(it), _ptr(info))
    return a, x.reshape(np.asarray(b).shape), int(it[0]), int(info[0])


def dlansy(norm, uplo, a):
    a = _colmajor(a, np.float64)
    n = a.shape[0]
    return lib().or_dlansy(norm.encode(), uplo.encode(), n, _ptr(a), max(1, n), _ptr(np.zeros(max(1, n))))


def gesv(a, b):
    """xGESV (SRC/dgesv.f): returns (lu, ipiv, x, info)."""
    a = _colmajor(a, a.dtype)
    b2 = _colmajor(_as2d(b), a.dtype)
    n = a.shape[0]
    ipiv = np.zeros(max(1, n), dtype=np.int32)
    info = np.zeros(1, dtype=np.int32)
    getattr(lib(), f"or_{_pre(a)}gesv")(n, b2.shape[1], _ptr(a), max(1, n), _ptr(ipiv), _ptr(b2),
                                        max(1, n), _ptr(info))
    return a, ipiv[:n], b2.reshape(b.shape), int(info[0])


def dsgesv(a, b):
    """DSGESV (SRC/dsgesv.f): returns (a_out, ipiv, x, iter, info)."""
    a = _colmajor(a, np.float64)
    b2 = _colmajor(_as2d(b), np.float64)
    n, nrhs = b2.shape
    x = np.zeros((n, nrhs), dtype=np.float64, order="F")
    work = np.zeros(max(1, n * nrhs), dtype=np.float64)
    swork = np.zeros(max(1, n * (n + nrhs)), dtype=np.float32)
    ipiv = np.zeros(max(1, n), dtype=np.int32)
    it = np.zeros(1, dtype=np.int32)
    info = np.zeros(1, dtype=np.int32)
    lib().or_dsgesv(n, nrhs, _ptr(a), max(1, n), _ptr(ipiv), _ptr(b2), max(1, n), _ptr(x), max(1, n),
                    _ptr(work), _ptr(swork), _ptr(it), _ptr(info))
    return a, ipiv[:n], x.reshape(b.shape), int(it[0]), int(info[0])


def laswp(a, k1, k2, ipiv, incx=1):
    a = _colmajor(a, a.dtype)
    m, n = a.shape
    ipiv = np.ascontiguousarray(ipiv, dtype=np.int32)
    getattr(lib(), f"or_{_pre(a)}laswp")(n, _ptr(a), max(1, m), k1, k2, _ptr(ipiv), incx)
    return a


def lange(norm, a):
    a = _colmajor(a, a.dtype)
    m, n = a.shape
    work = np.zeros(max(1, m), dtype=a.dtype)
    return float(getattr(lib(), f"or_{_pre(a)}lange")(norm.encode(), m, n, _ptr(a), max(1, m), _ptr(work)))


def dlag2s(a):
    a = _colmajor(a, np.float64)
    m, n = a.shape
    sa = np.zeros((m, n), dtype=np.float32, order="F")
    info = np.zeros(1, dtype=np.int32)
    lib().or_dlag2s(m, n, _ptr(a), max(1, m), _ptr(sa), max(1, m), _ptr(info))
    return sa, int(info[0])


def xerbla_last():
    buf = ctypes.create_string_buffer(16)
    info = lib().or_xerbla_last(buf, 16)
    return buf.value.decode(), info


def xerbla_reset():
    lib().or_xerbla_reset()


# ------------------------------------------------------------- generators
def seed_to_iseed(seed):
    iseed = np.zeros(4, dtype=np.int32)
    lib().or_seed_from_int(int(seed), _ptr(iseed))
    return iseed


def dlarnv(idist, iseed, n):
    """DLARNV (SRC/dlarnv.f); ``iseed`` (int32[4]) is advanced in place."""
    x = np.empty(int(n), dtype=np.float64)
    lib().or_dlarnv(int(idist), _ptr(iseed), int(n), _ptr(x))
    return x


def dlaruv_power(i):
    limbs = np.zeros(4, dtype=np.int32)
    lib().or_dlaruv_power(int(i), _ptr(limbs))
    return [int(v) for v in limbs]


def random_matrix(m, n, seed, idist=3, dtype=np.float64):
    """m x n column-major matrix of DLARNV(idist) draws from the scalar seed,
    filled column by column (the order the reference test generators use)."""
    iseed = seed_to_iseed(seed)
    x = dlarnv(idist, iseed, m * n)
    return np.asfortranarray(x.reshape(n, m).T.astype(dtype)), iseed


def config_dgesv_small(n=1024, seed=0):
    """Plain DGESV case: A iid N(0,1) from the seed, b iid N(0,1) drawn next
    from the same stream."""
    iseed = seed_to_iseed(seed)
    a = dlarnv(3, iseed, n * n).reshape(n, n).T
    b = dlarnv(3, iseed, n).reshape(n, 1)
    return np.asfortranarray(a), np.asfortranarray(b)


def config_dgesv_fp64(n=16384, nrhs=16, seed=1):
    """FP64 DGESV case: A iid U[-1,1] (DLARNV idist 2) from the seed, B iid
    N(0,1) (idist 3) drawn next from the same stream, n x nrhs."""
    iseed = seed_to_iseed(seed)
    a = dlarnv(2, iseed, n * n).reshape(n, n).T
    b = dlarnv(3, iseed, n * nrhs).reshape(nrhs, n).T
    return np.asfortranarray(a), np.asfortranarray(b)


def householder_vectors(n, count, iseed):
    """``count`` DLARNV N(0,1) vectors of length n (the DLAGGE construction,
    TESTING/MATGEN/dlagge.f:185-232, draws its reflector vectors this way)."""
    return dlarnv(3, iseed, n * count).reshape(count, n)


def config_dsgesv_matrix(n, kappa, seed, nrefl=64):
    """A = Q1 diag(s) Q2^T with Qi products of ``nrefl`` Householder
    reflectors H = I - 2 v v^T / (v^T v) (v from DLARNV N(0,1)) and
    s_i = kappa^(-(i-1)/(n-1)) (DLATMS MODE 3, TESTING/MATGEN/dlatms.f:160).
    Returns (A, s, V1, V2).  Uses numpy for the dense products: input
    construction only."""
    iseed = seed_to_iseed(seed)
    v1 = householder_vectors(n, nrefl, iseed)
    v2 = householder_vectors(n, nrefl, iseed)
    i = np.arange(n, dtype=np.float64)
    s = kappa ** (-(i / (n - 1))) if n > 1 else np.ones(1)
    a = np.diag(s)
    for v in v1:            # A <- H A   (Q1 = H_1 H_2 ... H_k applied right to left)
        a -= np.outer(v, (2.0 / v.dot(v)) * (v @ a))
    for v in v2:            # A <- A H   (Q2^T = H_k ... H_1)
        a -= np.outer(a @ v, (2.0 / v.dot(v)) * v)
    return np.asfortranarray(a), s, v1, v2


def ge_test_matrix(m, n, imat, seed):
    """A matrix of the reference GE test type `imat` (TESTING/LIN/dlatb4.f:437-465,
    zero columns as TESTING/LIN/dchkge.f:325-347), built from DLARNV draws:
    1 diagonal, 2 upper / 3 lower triangular, 4 random kappa=2, 5/6/7 first /
    last / trailing-half columns zeroed, 8 kappa = sqrt(0.1/eps), 9 kappa =
    0.1/eps, 10 scaled near underflow, 11 near overflow.  Singular values are
    geometric (DLATMS MODE 3) between 1 and 1/kappa; the orthogonal factors come
    from QR of DLARNV normal matrices.  Returns (A, izero) with izero the
    expected INFO for types 5-7 (0 otherwise)."""
    eps = 2.0 ** -52
    kappa = {8: np.sqrt(0.1 / eps), 9: 0.1 / eps}.get(imat, 2.0)
    k = min(m, n)
    if k == 0:
        return np.zeros((m, n), order="F"), 0
    iseed = seed_to_iseed(seed)
    sv = kappa ** (-(np.arange(k) / max(k - 1, 1)))
    if imat == 1:
        a = np.zeros((m, n))
        a[np.arange(k), np.arange(k)] = sv * np.sign(dlarnv(2, iseed, k) + 1e-300)
    else:
        u, _ = np.linalg.qr(dlarnv(3, iseed, m * m).reshape(m, m))
        v, _ = np.linalg.qr(dlarnv(3, iseed, n * n).reshape(n, n))
        a = (u[:, :k] * sv) @ v[:, :k].T
        if imat == 2:
            a = np.triu(a)
            a[np.arange(k), np.arange(k)] = np.where(np.abs(np.diag(a)[:k]) < 0.5, 1.0, np.diag(a)[:k])
        elif imat == 3:
            a = np.tril(a)
            a[np.arange(k), np.arange(k)] = np.where(np.abs(np.diag(a)[:k]) < 0.5, 1.0, np.diag(a)[:k])
    if imat == 10:
        a = a * 1e-290
    elif imat == 11:
        a = a * 1e290
    izero = 0
    if 5 <= imat <= 7:
        izero = 1 if imat == 5 else (k if imat == 6 else k // 2 + 1)
        if imat < 7:
            a[:, izero - 1] = 0.0
        else:
            a[:, izero - 1:] = 0.0
    return np.asfortranarray(a), izero


# ---------------------------------------------------------------- complex LU
def _zpre(dtype):
    return "c" if np.dtype(dtype) == np.complex64 else "z"


def zgetrf(a, nb=64, dtype=np.complex128):
    """ZGETRF (SRC/zgetrf.f; CGETRF for dtype complex64) on a copy of ``a``
    with block size ``nb`` (nb <= 1 or >= min(m, n): xGETRF2 alone): returns
    (lu, ipiv, info)."""
    a = _colmajor(a, dtype)
    m, n = a.shape
    ipiv = np.zeros(max(1, min(m, n)), dtype=np.int32)
    info = np.zeros(1, dtype=np.int32)
    getattr(lib(), f"or_{_zpre(dtype)}getrf_nb")(m, n, _ptr(a), max(1, m), _ptr(ipiv), _ptr(info), nb)
    return a, ipiv[: min(m, n)], int(info[0])


def zgetrs(lu, ipiv, b, trans="N"):
    """ZGETRS / CGETRS (SRC/zgetrs.f), TRANS = 'N', 'T' or 'C', in the
    precision of ``lu``: returns (x, info)."""
    dtype = np.complex64 if np.asarray(lu).dtype == np.complex64 else np.complex128
    lu = _colmajor(lu, dtype)
    b2 = _colmajor(_as2d(b), dtype)
    n, nrhs = b2.shape
    ipiv = np.ascontiguousarray(ipiv, dtype=np.int32)
    info = np.zeros(1, dtype=np.int32)
    getattr(lib(), f"or_{_zpre(dtype)}getrs")(trans.encode(), n, nrhs, _ptr(lu), max(1, n), _ptr(ipiv), _ptr(b2),
                                              max(1, n), _ptr(info))
    return b2.reshape(np.asarray(b).shape), int(info[0])


def zgesv(a, b, dtype=np.complex128):
    """ZGESV / CGESV (SRC/zgesv.f): returns (lu, ipiv, x, info)."""
    a = _colmajor(a, dtype)
    b2 = _colmajor(_as2d(b), dtype)
    n, nrhs = b2.shape
    ipiv = np.zeros(max(1, n), dtype=np.int32)
    info = np.zeros(1, dtype=np.int32)
    getattr(lib(), f"or_{_zpre(dtype)}gesv")(n, nrhs, _ptr(a), max(1, n), _ptr(ipiv), _ptr(b2), max(1, n),
                                             _ptr(info))
    return a, ipiv[:n], b2.reshape(np.asarray(b).shape), int(info[0])


def zcgesv(a, b):
    """ZCGESV (SRC/zcgesv.f): returns (a_out, ipiv, x, iter, info); a_out
    holds the COMPLEX*16 factors when the refinement fell back (ITER < 0)."""
    a = _colmajor(a, np.complex128)
    b2 = _colmajor(_as2d(b), np.complex128)
    n, nrhs = b2.shape
    x = np.zeros((n, nrhs), dtype=np.complex128, order="F")
    ipiv = np.zeros(max(1, n), dtype=np.int32)
    work = np.zeros(max(1, n * nrhs), dtype=np.complex128)
    swork = np.zeros(max(1, n * (n + nrhs)), dtype=np.complex64)
    rwork = np.zeros(max(1, n))
    it = np.zeros(1, dtype=np.int32)
    info = np.zeros(1, dtype=np.int32)
    lib().or_zcgesv(n, nrhs, _ptr(a), max(1, n), _ptr(ipiv), _ptr(b2), max(1, n), _ptr(x), max(1, n), _ptr(work),
                    _ptr(swork), _ptr(rwork), _ptr(it), _ptr(info))
    return a, ipiv[:n], x.reshape(np.asarray(b).shape), int(it[0]), int(info[0])


def izamax(x):
    """IZAMAX (BLAS/SRC/izamax.f90), 1-based; ICAMAX for complex64 input."""
    x = np.asarray(x)
    dtype = np.complex64 if x.dtype == np.complex64 else np.complex128
    x = np.ascontiguousarray(x, dtype=dtype)
    return getattr(lib(), f"or_{_zpre(dtype)}iamax")(x.size, _ptr(x))


def random_zmatrix(m, n, seed):
    """Complex test matrix: real and imaginary parts iid N(0,1), each from
    the DLARNV(3) stream of its own seed (seed and seed + 7919)."""
    re = random_matrix(m, n, seed, idist=3)[0]
    im = random_matrix(m, n, seed + 7919, idist=3)[0]
    return np.asfortranarray(re + 1j * im)


def zge_test_matrix(m, n, imat, seed):
    """Complex analogue of ``ge_test_matrix``: real and imaginary parts are
    two matrices of the same GE type (from seeds seed and seed + 1), so the
    zero columns of types 5-7, the triangles of types 2-3 and the scalings of
    types 10-11 carry over.  Returns (A, izero)."""
    re, izero = ge_test_matrix(m, n, imat, seed)
    im, _ = ge_test_matrix(m, n, imat, seed + 1)
    return np.asfortranarray(re + 1j * im), izero
