"""GB300-native LAPACK dense LU solve path.

Python mirror of the library's C ABI (``include/lapack_gb300.h``): the
reference routine names and argument meanings (DGETRF, DGETRS, DGESV,
DSGESV, DLASWP, ... with column-major arrays, 1-based IPIV and LAPACK INFO
codes), called through ``liblapack_gb300.so``.  All arithmetic runs in the
hand-written sm_103a kernels of that library; there is no CPU path.  If the
shared library is missing, importing the bindings raises.
"""
import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "liblapack_gb300.so")
_LIB = None

_i = ctypes.c_int
_p = ctypes.c_void_p
_ip = ctypes.POINTER(ctypes.c_int)
_sz = ctypes.c_size_t

FORTRAN_SYMBOLS = ["dgetrf_", "sgetrf_", "dgetrf2_", "sgetrf2_", "dgetrs_", "sgetrs_", "dgesv_", "sgesv_",
                   "dsgesv_", "dgesvx_", "dgetri_", "dpotrf_", "spotrf_", "dpotrs_", "spotrs_", "dposv_", "dsposv_",
                   "dgerfs_", "dgecon_", "dlatrs_", "dlaswp_", "slaswp_", "dlag2s_", "slag2d_", "dlange_", "dlamch_",
                   "slamch_", "xerbla_"]


class LibraryMissing(RuntimeError):
    pass


def build(force=False):
    """Compiles liblapack_gb300.so in-tree (see buildlib.py)."""
    from . import buildlib
    return buildlib.build(force=force)


def lib():
    """The loaded shared library (raises LibraryMissing if it was not built)."""
    global _LIB
    if _LIB is None:
        if not os.path.exists(LIB_PATH):
            raise LibraryMissing(f"{LIB_PATH} not built; run lapack_gb300.build()")
        L = ctypes.CDLL(LIB_PATH)
        L.dlange_.restype = ctypes.c_double
        L.dlamch_.restype = ctypes.c_double
        L.slamch_.restype = ctypes.c_float
        L.gb300_version.restype = ctypes.c_char_p
        L.gb300_set_option.argtypes = [ctypes.c_char_p, _i]
        L.gb300_get_option.argtypes = [ctypes.c_char_p]
        L.gb300_xerbla_last.argtypes = [ctypes.c_char_p, _i]
        for nm in ("gb300_dgetrf_dev", "gb300_sgetrf_dev"):
            getattr(L, nm).argtypes = [_i, _i, _p, _i, _p, _ip, _p]
        for nm in ("gb300_dgetrs_dev", "gb300_sgetrs_dev"):
            getattr(L, nm).argtypes = [ctypes.c_char, _i, _i, _p, _i, _p, _p, _i, _p]
        L.gb300_dgesv_dev.argtypes = [_i, _i, _p, _i, _p, _p, _i, _ip, _p]
        L.gb300_dsgesv_dev.argtypes = [_i, _i, _p, _i, _p, _p, _i, _p, _i, _ip, _ip, _p]
        L.gb300_dgecon_dev.argtypes = [ctypes.c_char, _i, _p, _i, ctypes.c_double, _p, _ip, _p]
        L.gb300_dgetri_dev.argtypes = [_i, _p, _i, _p, _ip, _p]
        L.gb300_dgerfs_dev.argtypes = [ctypes.c_char, _i, _i, _p, _i, _p, _i, _p, _p, _i, _p, _i, _p, _p, _p]
        L.gb300_zgetrf_dev.argtypes = [_i, _i, _p, _i, _p, _ip, _p]
        L.gb300_zgetrs_dev.argtypes = [ctypes.c_char, _i, _i, _p, _i, _p, _p, _i, _p]
        L.gb300_zgesv_dev.argtypes = [_i, _i, _p, _i, _p, _p, _i, _ip, _p]
        L.gb300_zcgesv_dev.argtypes = [_i, _i, _p, _i, _p, _p, _i, _p, _i, _ip, _ip, _p]
        _LIB = L
    return _LIB


def _ref(v):
    return ctypes.byref(ctypes.c_int(int(v)))


def _as2d(b):
    b = np.asarray(b)
    return b.reshape(b.shape[0], b.shape[1] if b.ndim == 2 else 1)


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def _fortran(a, dtype):
    return np.asfortranarray(np.array(a, dtype=dtype, copy=True))


def _pre(dtype):
    return "d" if np.dtype(dtype) == np.float64 else "s"


# ------------------------------------------------------------------ options
def set_option(name, value):
    """Library options: 'exact' (0/1), 'nb64', 'nb32', 'mixed' (0 BF16x3
    tensor cores, 1 FP32 CUDA cores), 'sgetrf', 'lookahead', 'gemm_ws' (1
    warp-specialised multi-tile BF16x3 update, 0 one tile per CTA),
    'gemm_tiles' (tiles per CTA of that update, 0: one CTA per SM) and the
    others gb300_set_option names.  Returns the old value."""
    return lib().gb300_set_option(name.encode(), int(value))


def get_option(name):
    return lib().gb300_get_option(name.encode())


def status(clear=True):
    return lib().gb300_status(int(clear))


def xerbla_capture(on=True):
    lib().gb300_xerbla_capture(int(on))


def xerbla_last():
    buf = ctypes.create_string_buffer(16)
    info = lib().gb300_xerbla_last(buf, 16)
    return buf.value.decode(), info


# ------------------------------------------------- LAPACK routines (host data)
def getrf(a, dtype=None):
    """xGETRF (SRC/dgetrf.f): returns (lu, ipiv, info) for a copy of ``a``."""
    dtype = np.dtype(dtype or (a.dtype if a.dtype in (np.float32, np.float64) else np.float64))
    a = _fortran(a, dtype)
    m, n = a.shape
    ipiv = np.zeros(max(1, min(m, n)), dtype=np.int32)
    info = ctypes.c_int(0)
    getattr(lib(), f"{_pre(dtype)}getrf_")(_ref(m), _ref(n), _ptr(a), _ref(max(1, m)), _ptr(ipiv), ctypes.byref(info))
    return a, ipiv[: min(m, n)], info.value


def getrf2(a, dtype=None):
    """xGETRF2 (SRC/dgetrf2.f)."""
    dtype = np.dtype(dtype or (a.dtype if a.dtype in (np.float32, np.float64) else np.float64))
    a = _fortran(a, dtype)
    m, n = a.shape
    ipiv = np.zeros(max(1, min(m, n)), dtype=np.int32)
    info = ctypes.c_int(0)
    getattr(lib(), f"{_pre(dtype)}getrf2_")(_ref(m), _ref(n), _ptr(a), _ref(max(1, m)), _ptr(ipiv), ctypes.byref(info))
    return a, ipiv[: min(m, n)], info.value


def getrs(lu, ipiv, b, trans="N"):
    """xGETRS (SRC/dgetrs.f): returns (x, info)."""
    dtype = lu.dtype
    lu = _fortran(lu, dtype)
    b2 = _fortran(_as2d(b), dtype)
    n, nrhs = b2.shape
    ipiv = np.ascontiguousarray(ipiv, dtype=np.int32)
    info = ctypes.c_int(0)
    getattr(lib(), f"{_pre(dtype)}getrs_")(ctypes.c_char_p(trans.encode()), _ref(n), _ref(nrhs), _ptr(lu),
                                           _ref(max(1, n)), _ptr(ipiv), _ptr(b2), _ref(max(1, n)),
                                           ctypes.byref(info), _sz(1))
    return b2.reshape(np.asarray(b).shape), info.value


def gesv(a, b, dtype=None):
    """xGESV (SRC/dgesv.f): returns (lu, ipiv, x, info)."""
    dtype = np.dtype(dtype or (a.dtype if a.dtype in (np.float32, np.float64) else np.float64))
    a = _fortran(a, dtype)
    n = a.shape[0]
    b2 = _fortran(_as2d(b), dtype)
    ipiv = np.zeros(max(1, n), dtype=np.int32)
    info = ctypes.c_int(0)
    getattr(lib(), f"{_pre(dtype)}gesv_")(_ref(n), _ref(b2.shape[1]), _ptr(a), _ref(max(1, n)), _ptr(ipiv),
                                          _ptr(b2), _ref(max(1, n)), ctypes.byref(info))
    return a, ipiv[:n], b2.reshape(np.asarray(b).shape), info.value


def dsgesv(a, b):
    """DSGESV (SRC/dsgesv.f): returns (a_out, ipiv, x, iter, info)."""
    a = _fortran(a, np.float64)
    n = a.shape[0]
    b2 = _fortran(_as2d(b), np.float64)
    nrhs = b2.shape[1]
    x = np.zeros((n, nrhs), dtype=np.float64, order="F")
    work = np.zeros(max(1, n * nrhs), dtype=np.float64)
    swork = np.zeros(1, dtype=np.float32)          # the GPU works in device memory
    ipiv = np.zeros(max(1, n), dtype=np.int32)
    it = ctypes.c_int(0)
    info = ctypes.c_int(0)
    lib().dsgesv_(_ref(n), _ref(nrhs), _ptr(a), _ref(max(1, n)), _ptr(ipiv), _ptr(b2), _ref(max(1, n)), _ptr(x),
                  _ref(max(1, n)), _ptr(work), _ptr(swork), ctypes.byref(it), ctypes.byref(info))
    return a, ipiv[:n], x.reshape(np.asarray(b).shape), it.value, info.value


def gerfs(a, af, ipiv, b, x, trans="N"):
    """DGERFS (SRC/dgerfs.f): refines a copy of ``x`` with the factors
    ``af``/``ipiv`` of ``a``; returns (x, ferr, berr, info)."""
    a = _fortran(a, np.float64)
    af = _fortran(af, np.float64)
    b2 = _fortran(_as2d(b), np.float64)
    x2 = _fortran(_as2d(x), np.float64)
    n, nrhs = b2.shape
    ipiv = np.ascontiguousarray(ipiv, dtype=np.int32)
    ferr = np.zeros(max(nrhs, 1))
    berr = np.zeros(max(nrhs, 1))
    work = np.zeros(3 * max(n, 1))
    iwork = np.zeros(max(n, 1), dtype=np.int32)
    info = ctypes.c_int(0)
    ld = max(1, n)
    lib().dgerfs_(ctypes.c_char_p(trans.encode()), _ref(n), _ref(nrhs), _ptr(a), _ref(ld), _ptr(af), _ref(ld),
                  _ptr(ipiv), _ptr(b2), _ref(ld), _ptr(x2), _ref(ld), _ptr(ferr), _ptr(berr), _ptr(work),
                  _ptr(iwork), ctypes.byref(info), _sz(1))
    return x2.reshape(np.asarray(x).shape), ferr[:nrhs], berr[:nrhs], info.value


def gecon(lu, anorm, norm="1"):
    """DGECON (SRC/dgecon.f): reciprocal condition number from the LU
    factors ``lu`` and the norm ``anorm`` of A; returns (rcond, info)."""
    lu = _fortran(lu, np.float64)
    n = lu.shape[0]
    rcond = ctypes.c_double(0.0)
    info = ctypes.c_int(0)
    work = np.zeros(4 * max(n, 1))
    iwork = np.zeros(max(n, 1), dtype=np.int32)
    lib().dgecon_(ctypes.c_char_p(norm.encode()), _ref(n), _ptr(lu), _ref(max(1, n)),
                  ctypes.byref(ctypes.c_double(float(anorm))), ctypes.byref(rcond), _ptr(work), _ptr(iwork),
                  ctypes.byref(info), _sz(1))
    return rcond.value, info.value


def latrs(t, x, uplo, trans, diag, cnorm=None):
    """DLATRS (SRC/dlatrs.f) on the triangle of ``t``: returns (x, scale,
    cnorm); ``cnorm`` given means NORMIN = 'Y'."""
    t = _fortran(t, np.float64)
    n = t.shape[0]
    x = np.array(x, dtype=np.float64, copy=True)
    normin = b"N" if cnorm is None else b"Y"
    cn = np.zeros(max(n, 1)) if cnorm is None else np.array(cnorm, dtype=np.float64, copy=True)
    scale = ctypes.c_double(0.0)
    info = ctypes.c_int(0)
    lib().dlatrs_(ctypes.c_char_p(uplo.encode()), ctypes.c_char_p(trans.encode()), ctypes.c_char_p(diag.encode()),
                  ctypes.c_char_p(normin), _ref(n), _ptr(t), _ref(max(1, n)), _ptr(x), ctypes.byref(scale),
                  _ptr(cn), ctypes.byref(info), _sz(1), _sz(1), _sz(1), _sz(1))
    if info.value != 0:
        raise RuntimeError(f"dlatrs failed with INFO = {info.value}")
    return x, scale.value, cn[:n]


def gesvx(a, b, fact="N", trans="N", af=None, ipiv=None, equed="N", r=None, c=None):
    """DGESVX (SRC/dgesvx.f).  Returns a dict: a (equilibrated when
    EQUED != 'N'), af, ipiv, equed, r, c, b (scaled as the reference leaves
    it), x, rcond, ferr, berr, rpvgrw (WORK(1)), info."""
    a = _fortran(a, np.float64)
    b2 = _fortran(_as2d(b), np.float64)
    n, nrhs = b2.shape
    ld = max(1, n)
    af = np.zeros((n, n), order="F") if af is None else _fortran(af, np.float64)
    ipiv = np.zeros(ld, dtype=np.int32) if ipiv is None else np.array(ipiv, dtype=np.int32)
    r = np.zeros(ld) if r is None else np.array(r, dtype=np.float64)
    c = np.zeros(ld) if c is None else np.array(c, dtype=np.float64)
    eq = ctypes.create_string_buffer(equed.encode(), 2)
    x = np.zeros((n, nrhs), order="F")
    rcond = ctypes.c_double(0.0)
    ferr = np.zeros(max(nrhs, 1))
    berr = np.zeros(max(nrhs, 1))
    work = np.zeros(4 * ld)
    iwork = np.zeros(ld, dtype=np.int32)
    info = ctypes.c_int(0)
    lib().dgesvx_(ctypes.c_char_p(fact.encode()), ctypes.c_char_p(trans.encode()), _ref(n), _ref(nrhs), _ptr(a),
                  _ref(ld), _ptr(af), _ref(ld), _ptr(ipiv), eq, _ptr(r), _ptr(c), _ptr(b2), _ref(ld), _ptr(x),
                  _ref(ld), ctypes.byref(rcond), _ptr(ferr), _ptr(berr), _ptr(work), _ptr(iwork), ctypes.byref(info),
                  _sz(1), _sz(1), _sz(1))
    return dict(a=a, af=af, ipiv=ipiv[:n], equed=eq.value.decode(), r=r[:n], c=c[:n], b=b2, x=x,
                rcond=rcond.value, ferr=ferr[:nrhs], berr=berr[:nrhs], rpvgrw=float(work[0]), info=info.value)


def getri(lu, ipiv, lwork=None):
    """DGETRI (SRC/dgetri.f) on a copy of the factors; returns (ainv, info,
    work0).  lwork = -1 is the workspace query."""
    a = _fortran(lu, np.float64)
    n = a.shape[0]
    ipiv = np.ascontiguousarray(ipiv, dtype=np.int32)
    nb = max(1, get_option("nb64"))
    lw = max(1, n * nb) if lwork is None else lwork
    work = np.zeros(max(1, lw, n * nb))
    info = ctypes.c_int(0)
    lib().dgetri_(_ref(n), _ptr(a), _ref(max(1, n)), _ptr(ipiv), _ptr(work), _ref(lw), ctypes.byref(info))
    return a, info.value, float(work[0])


def potrf(a, uplo="L", dtype=None):
    """xPOTRF (SRC/dpotrf.f): returns (factor, info) for a copy of ``a``."""
    dtype = np.dtype(dtype or (a.dtype if a.dtype in (np.float32, np.float64) else np.float64))
    a = _fortran(a, dtype)
    n = a.shape[0]
    info = ctypes.c_int(0)
    getattr(lib(), f"{_pre(dtype)}potrf_")(ctypes.c_char_p(uplo.encode()), _ref(n), _ptr(a), _ref(max(1, n)),
                                           ctypes.byref(info), _sz(1))
    return a, info.value


def potrs(f, b, uplo="L"):
    """xPOTRS (SRC/dpotrs.f): returns (x, info)."""
    dtype = f.dtype
    f = _fortran(f, dtype)
    b2 = _fortran(_as2d(b), dtype)
    n, nrhs = b2.shape
    info = ctypes.c_int(0)
    getattr(lib(), f"{_pre(dtype)}potrs_")(ctypes.c_char_p(uplo.encode()), _ref(n), _ref(nrhs), _ptr(f),
                                           _ref(max(1, n)), _ptr(b2), _ref(max(1, n)), ctypes.byref(info), _sz(1))
    return b2.reshape(np.asarray(b).shape), info.value


def posv(a, b, uplo="L"):
    """DPOSV (SRC/dposv.f): returns (factor, x, info)."""
    a = _fortran(a, np.float64)
    b2 = _fortran(_as2d(b), np.float64)
    n, nrhs = b2.shape
    info = ctypes.c_int(0)
    lib().dposv_(ctypes.c_char_p(uplo.encode()), _ref(n), _ref(nrhs), _ptr(a), _ref(max(1, n)), _ptr(b2),
                 _ref(max(1, n)), ctypes.byref(info), _sz(1))
    return a, b2.reshape(np.asarray(b).shape), info.value


def dsposv(a, b, uplo="L"):
    """DSPOSV (SRC/dsposv.f): returns (a_out, x, iter, info)."""
    a = _fortran(a, np.float64)
    b2 = _fortran(_as2d(b), np.float64)
    n, nrhs = b2.shape
    x = np.zeros((n, nrhs), order="F")
    it = ctypes.c_int(0)
    info = ctypes.c_int(0)
    lib().dsposv_(ctypes.c_char_p(uplo.encode()), _ref(n), _ref(nrhs), _ptr(a), _ref(max(1, n)), _ptr(b2),
                  _ref(max(1, n)), _ptr(x), _ref(max(1, n)), _ptr(np.zeros(1)), _ptr(np.zeros(1, np.float32)),
                  ctypes.byref(it), ctypes.byref(info), _sz(1))
    return a, x.reshape(np.asarray(b).shape), it.value, info.value


def _zpre(dtype):
    return "c" if np.dtype(dtype) == np.complex64 else "z"


def zgetrf(a, dtype=np.complex128):
    """ZGETRF (SRC/zgetrf.f), or CGETRF for dtype complex64, on a copy of
    ``a``: returns (lu, ipiv, info)."""
    a = _fortran(a, dtype)
    m, n = a.shape
    ipiv = np.zeros(max(1, min(m, n)), dtype=np.int32)
    info = ctypes.c_int(0)
    getattr(lib(), f"{_zpre(dtype)}getrf_")(_ref(m), _ref(n), _ptr(a), _ref(max(1, m)), _ptr(ipiv), ctypes.byref(info))
    return a, ipiv[: min(m, n)], info.value


def zgetrf2(a, dtype=np.complex128):
    """ZGETRF2 / CGETRF2 (SRC/zgetrf2.f): the recursive factorization alone."""
    a = _fortran(a, dtype)
    m, n = a.shape
    ipiv = np.zeros(max(1, min(m, n)), dtype=np.int32)
    info = ctypes.c_int(0)
    getattr(lib(), f"{_zpre(dtype)}getrf2_")(_ref(m), _ref(n), _ptr(a), _ref(max(1, m)), _ptr(ipiv),
                                             ctypes.byref(info))
    return a, ipiv[: min(m, n)], info.value


def zgetrs(lu, ipiv, b, trans="N"):
    """ZGETRS / CGETRS (SRC/zgetrs.f) in the precision of ``lu``, TRANS =
    'N', 'T' or 'C': returns (x, info)."""
    dtype = np.complex64 if np.asarray(lu).dtype == np.complex64 else np.complex128
    lu = _fortran(lu, dtype)
    b2 = _fortran(_as2d(b), dtype)
    n, nrhs = b2.shape
    ipiv = np.ascontiguousarray(ipiv, dtype=np.int32)
    info = ctypes.c_int(0)
    getattr(lib(), f"{_zpre(dtype)}getrs_")(ctypes.c_char_p(trans.encode()), _ref(n), _ref(nrhs), _ptr(lu),
                                            _ref(max(1, n)), _ptr(ipiv), _ptr(b2), _ref(max(1, n)),
                                            ctypes.byref(info), _sz(1))
    return b2.reshape(np.asarray(b).shape), info.value


def zgesv(a, b, dtype=np.complex128):
    """ZGESV / CGESV (SRC/zgesv.f): returns (lu, ipiv, x, info)."""
    a = _fortran(a, dtype)
    b2 = _fortran(_as2d(b), dtype)
    n, nrhs = b2.shape
    ipiv = np.zeros(max(1, n), dtype=np.int32)
    info = ctypes.c_int(0)
    getattr(lib(), f"{_zpre(dtype)}gesv_")(_ref(n), _ref(nrhs), _ptr(a), _ref(max(1, n)), _ptr(ipiv), _ptr(b2),
                                           _ref(max(1, n)), ctypes.byref(info))
    return a, ipiv[:n], b2.reshape(np.asarray(b).shape), info.value


def zcgesv(a, b):
    """ZCGESV (SRC/zcgesv.f): returns (a_out, ipiv, x, iter, info); a_out
    holds the COMPLEX*16 factors when the refinement fell back (ITER < 0)."""
    a = _fortran(a, np.complex128)
    b2 = _fortran(_as2d(b), np.complex128)
    n, nrhs = b2.shape
    x = np.zeros((n, nrhs), dtype=np.complex128, order="F")
    ipiv = np.zeros(max(1, n), dtype=np.int32)
    it = ctypes.c_int(0)
    info = ctypes.c_int(0)
    work = np.zeros(max(1, n * nrhs), dtype=np.complex128)
    swork = np.zeros(max(1, n * (n + nrhs)), dtype=np.complex64)
    rwork = np.zeros(max(1, n))
    lib().zcgesv_(_ref(n), _ref(nrhs), _ptr(a), _ref(max(1, n)), _ptr(ipiv), _ptr(b2), _ref(max(1, n)), _ptr(x),
                  _ref(max(1, n)), _ptr(work), _ptr(swork), _ptr(rwork), ctypes.byref(it), ctypes.byref(info))
    return a, ipiv[:n], x.reshape(np.asarray(b).shape), it.value, info.value


def laswp(a, k1, k2, ipiv, incx=1):
    """xLASWP (SRC/dlaswp.f) on a copy of ``a``."""
    a = _fortran(a, a.dtype)
    m, n = a.shape
    ipiv = np.ascontiguousarray(ipiv, dtype=np.int32)
    getattr(lib(), f"{_pre(a.dtype)}laswp_")(_ref(n), _ptr(a), _ref(max(1, m)), _ref(k1), _ref(k2), _ptr(ipiv),
                                             _ref(incx))
    return a


def dlag2s(a):
    a = _fortran(a, np.float64)
    m, n = a.shape
    sa = np.zeros((m, n), dtype=np.float32, order="F")
    info = ctypes.c_int(0)
    lib().dlag2s_(_ref(m), _ref(n), _ptr(a), _ref(max(1, m)), _ptr(sa), _ref(max(1, m)), ctypes.byref(info))
    return sa, info.value


def slag2d(sa):
    sa = _fortran(sa, np.float32)
    m, n = sa.shape
    a = np.zeros((m, n), dtype=np.float64, order="F")
    info = ctypes.c_int(0)
    lib().slag2d_(_ref(m), _ref(n), _ptr(sa), _ref(max(1, m)), _ptr(a), _ref(max(1, m)), ctypes.byref(info))
    return a, info.value


def dlange(norm, a):
    a = _fortran(a, np.float64)
    m, n = a.shape
    work = np.zeros(max(1, m), dtype=np.float64)
    return lib().dlange_(ctypes.c_char_p(norm.encode()), _ref(m), _ref(n), _ptr(a), _ref(max(1, m)), _ptr(work),
                         _sz(1))


# ------------------------------------------- device entry points (torch data)
def _colmajor_view(t):
    """(ld, data_ptr) of a CUDA tensor holding a column-major matrix: shape
    (m, n) with stride (1, ld)."""
    if t.dim() != 2 or (t.stride(0) != 1 and t.shape[0] > 1):
        raise ValueError("expected a column-major (m, n) tensor with stride (1, ld)")
    return max(1, t.stride(1) if t.shape[1] > 1 else t.shape[0]), t.data_ptr()


def _stream_ptr(stream):
    import torch
    s = stream if stream is not None else torch.cuda.current_stream()
    return ctypes.c_void_p(s.cuda_stream)


def getrf_dev(A, ipiv, stream=None):
    """xGETRF on device memory; A (m, n) column-major float64/float32 CUDA
    tensor, ipiv int32 CUDA tensor of length min(m, n).  Returns INFO."""
    import torch
    ld, pa = _colmajor_view(A)
    info = ctypes.c_int(0)
    fn = lib().gb300_dgetrf_dev if A.dtype == torch.float64 else lib().gb300_sgetrf_dev
    rc = fn(A.shape[0], A.shape[1], ctypes.c_void_p(pa), ld, ctypes.c_void_p(ipiv.data_ptr()), ctypes.byref(info),
            _stream_ptr(stream))
    if rc != 0:
        raise RuntimeError(f"gb300 getrf failed with status {rc}")
    return info.value


def getrs_dev(A, ipiv, B, trans="N", stream=None):
    import torch
    ld, pa = _colmajor_view(A)
    ldb, pb = _colmajor_view(B)
    fn = lib().gb300_dgetrs_dev if A.dtype == torch.float64 else lib().gb300_sgetrs_dev
    rc = fn(trans.encode(), A.shape[0], B.shape[1], ctypes.c_void_p(pa), ld, ctypes.c_void_p(ipiv.data_ptr()),
            ctypes.c_void_p(pb), ldb, _stream_ptr(stream))
    if rc != 0:
        raise RuntimeError(f"gb300 getrs failed with status {rc}")


def dsgesv_dev(A, ipiv, B, X, stream=None):
    """DSGESV on device memory; returns (iter, info)."""
    ld, pa = _colmajor_view(A)
    ldb, pb = _colmajor_view(B)
    ldx, px = _colmajor_view(X)
    it = ctypes.c_int(0)
    info = ctypes.c_int(0)
    rc = lib().gb300_dsgesv_dev(A.shape[0], B.shape[1], ctypes.c_void_p(pa), ld, ctypes.c_void_p(ipiv.data_ptr()),
                                ctypes.c_void_p(pb), ldb, ctypes.c_void_p(px), ldx, ctypes.byref(it),
                                ctypes.byref(info), _stream_ptr(stream))
    if rc != 0:
        raise RuntimeError(f"gb300 dsgesv failed with status {rc}")
    return it.value, info.value


def gecon_dev(LU, anorm, norm="1", stream=None):
    """DGECON on device memory; returns (rcond, info)."""
    ld, pa = _colmajor_view(LU)
    rcond = ctypes.c_double(0.0)
    info = ctypes.c_int(0)
    rc = lib().gb300_dgecon_dev(norm.encode(), LU.shape[0], ctypes.c_void_p(pa), ld, float(anorm),
                                ctypes.byref(rcond), ctypes.byref(info), _stream_ptr(stream))
    if rc != 0:
        raise RuntimeError(f"gb300 dgecon failed with status {rc}")
    return rcond.value, info.value


def gerfs_dev(A, AF, ipiv, B, X, ferr, berr, trans="N", stream=None):
    """DGERFS on device memory: X refined in place; ferr, berr float64 CUDA
    tensors of length nrhs."""
    ld, pa = _colmajor_view(A)
    ldf, pf = _colmajor_view(AF)
    ldb, pb = _colmajor_view(B)
    ldx, px = _colmajor_view(X)
    rc = lib().gb300_dgerfs_dev(trans.encode(), A.shape[0], B.shape[1], ctypes.c_void_p(pa), ld, ctypes.c_void_p(pf),
                                ldf, ctypes.c_void_p(ipiv.data_ptr()), ctypes.c_void_p(pb), ldb, ctypes.c_void_p(px),
                                ldx, ctypes.c_void_p(ferr.data_ptr()), ctypes.c_void_p(berr.data_ptr()),
                                _stream_ptr(stream))
    if rc != 0:
        raise RuntimeError(f"gb300 dgerfs failed with status {rc}")


def colmajor_empty(m, n, dtype, device="cuda"):
    """A column-major (m, n) CUDA tensor (stride (1, m))."""
    import torch
    return torch.empty((n, m), dtype=dtype, device=device).t()


def to_colmajor(a_np, device="cuda"):
    import torch
    a = np.asarray(a_np)
    return torch.from_numpy(np.ascontiguousarray(a.T)).to(device).t()


# ------------------------------------------------------- batched (device)
class VBatch:
    """Device storage for a batch of independent systems of uneven size:
    packed column-major matrices plus the per-system pointer and size
    arrays the batched entry points take."""

    def __init__(self, As, Bs, dtype=None, device="cuda"):
        import torch
        dtype = dtype or torch.float64
        self.dtype = dtype
        self.ns = [int(a.shape[0]) for a in As]
        self.nrhs = [int(np.asarray(b).reshape(a.shape[0], -1).shape[1]) for a, b in zip(As, Bs)]
        ne = np.dtype(np.float64 if dtype == torch.float64 else np.float32)
        aoff = np.cumsum([0] + [n * n for n in self.ns])
        boff = np.cumsum([0] + [n * r for n, r in zip(self.ns, self.nrhs)])
        poff = np.cumsum([0] + self.ns)
        ha = np.concatenate([np.asarray(a, dtype=ne).T.reshape(-1) for a in As]) if As else np.zeros(0, ne)
        hb = np.concatenate([np.asarray(b, dtype=ne).reshape(n, -1).T.reshape(-1) for b, n in zip(Bs, self.ns)])
        self.A = torch.from_numpy(ha).to(device)
        self.B = torch.from_numpy(hb).to(device)
        self.ipiv = torch.zeros(int(poff[-1]), dtype=torch.int32, device=device)
        es = self.A.element_size()
        self.aoff, self.boff, self.poff = aoff, boff, poff
        self.d_n = torch.tensor(self.ns, dtype=torch.int32, device=device)
        self.d_nrhs = torch.tensor(self.nrhs, dtype=torch.int32, device=device)
        self.d_ld = self.d_n.clone()
        self.d_Ap = torch.tensor([self.A.data_ptr() + int(o) * es for o in aoff[:-1]], dtype=torch.int64, device=device)
        self.d_Bp = torch.tensor([self.B.data_ptr() + int(o) * es for o in boff[:-1]], dtype=torch.int64, device=device)
        self.d_Pp = torch.tensor([self.ipiv.data_ptr() + int(o) * 4 for o in poff[:-1]], dtype=torch.int64,
                                 device=device)
        self.info = torch.zeros(len(self.ns), dtype=torch.int32, device=device)

    def launch(self, stream=None, factor_only=False):
        import torch
        L = lib()
        p = lambda t: ctypes.c_void_p(t.data_ptr())
        batch = len(self.ns)
        if factor_only:
            rc = L.gb300_dgetrf_vbatched_dev(batch, p(self.d_n), p(self.d_Ap), p(self.d_ld), p(self.d_Pp),
                                             p(self.info), _stream_ptr(stream))
        else:
            fn = L.gb300_dgesv_vbatched_dev if self.dtype == torch.float64 else L.gb300_sgesv_vbatched_dev
            rc = fn(batch, p(self.d_n), p(self.d_nrhs), p(self.d_Ap), p(self.d_ld), p(self.d_Pp), p(self.d_Bp),
                    p(self.d_ld), p(self.info), _stream_ptr(stream))
        if rc != 0:
            raise RuntimeError(f"gb300 batched solve failed with status {rc}")

    def results(self):
        """Lists (lu, ipiv, x) on the host and the INFO array."""
        ha = self.A.cpu().numpy()
        hb = self.B.cpu().numpy()
        hp = self.ipiv.cpu().numpy()
        lus, ips, xs = [], [], []
        for i, n in enumerate(self.ns):
            lus.append(ha[self.aoff[i]:self.aoff[i + 1]].reshape(n, n).T)
            xs.append(hb[self.boff[i]:self.boff[i + 1]].reshape(self.nrhs[i], n).T)
            ips.append(hp[self.poff[i]:self.poff[i + 1]])
        return lus, ips, xs, self.info.cpu().numpy()


def gesv_vbatched(As, Bs, dtype=None):
    """Batched xGESV of independent systems (n <= 512, nrhs <= 4) in one
    persistent launch.  Returns (lu list, ipiv list, x list, info array)."""
    vb = VBatch(As, Bs, dtype)
    vb.launch()
    import torch
    torch.cuda.synchronize()
    return vb.results()


def vbatched_nb(dtype_code):
    tab = (ctypes.c_int * 8)()
    lib().gb300_vbatched_get_nb(int(dtype_code), tab)
    return list(tab)


def set_vbatched_nb(dtype_code, table):
    arr = (ctypes.c_int * 8)(*[int(v) for v in table])
    return lib().gb300_vbatched_set_nb(int(dtype_code), arr)


def autotune_batched(dtype_code, count=600):
    """Times every candidate panel width per size bucket and installs the
    fastest (see lapack_gb300.autotune)."""
    from . import autotune
    return autotune.tune_batched(dtype_code, count)


# ------------------------------------------------------------------ adjoint
def adjoint_dev(LU, ipiv, X, gX, want_gA=True, stream=None):
    """gB = A^{-T} gX and gA = -gB X^T from stored factors (column-major CUDA
    float64 tensors).  Returns (gB, gA)."""
    import torch
    n, nrhs = X.shape
    ldlu, plu = _colmajor_view(LU)
    ldx, px = _colmajor_view(X)
    ldg, pg = _colmajor_view(gX)
    gB = colmajor_empty(n, nrhs, torch.float64, X.device)
    gA = colmajor_empty(n, n, torch.float64, X.device) if want_gA else None
    ldgb, pgb = _colmajor_view(gB)
    vp = ctypes.c_void_p
    rc = lib().gb300_dgesv_adjoint_dev(n, nrhs, vp(plu), ldlu, vp(ipiv.data_ptr()), vp(px), ldx, vp(pg), ldg, vp(pgb),
                                       ldgb, vp(gA.data_ptr()) if want_gA else None, n, _stream_ptr(stream))
    if rc != 0:
        raise RuntimeError(f"gb300 adjoint failed with status {rc}")
    return gB, gA


def _solve_autograd_class():
    import torch

    class Solve(torch.autograd.Function):
        """X = A^{-1} B on the GPU (DGETRF + DGETRS); the backward pass runs
        the library's adjoint on the saved factors.  Meant for gradient
        checks, not as a training op."""

        @staticmethod
        def forward(ctx, A, B):
            n = A.shape[0]
            LU = colmajor_empty(n, n, torch.float64, A.device)
            LU.copy_(A)
            ipiv = torch.empty(n, dtype=torch.int32, device=A.device)
            info = getrf_dev(LU, ipiv)
            if info != 0:
                raise RuntimeError(f"singular matrix (INFO={info})")
            X = colmajor_empty(n, B.shape[1], torch.float64, A.device)
            X.copy_(B)
            getrs_dev(LU, ipiv, X)
            ctx.save_for_backward(LU, ipiv, X)
            return X.clone()

        @staticmethod
        def backward(ctx, gX):
            LU, ipiv, X = ctx.saved_tensors
            g = colmajor_empty(gX.shape[0], gX.shape[1], torch.float64, gX.device)
            g.copy_(gX)
            gB, gA = adjoint_dev(LU, ipiv, X, g, want_gA=ctx.needs_input_grad[0])
            return gA, gB

    return Solve


_SOLVE = None


def solve(A, B):
    """Differentiable X = A^{-1} B (float64 CUDA tensors, B of shape (n, nrhs))."""
    global _SOLVE
    if _SOLVE is None:
        _SOLVE = _solve_autograd_class()
    return _SOLVE.apply(A, B)
