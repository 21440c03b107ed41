"""This library's LAPACKE layer against the reference's own LAPACKE C
sources, both compiled over the oracle's Fortran-ABI shim
(`make -C oracle ref ours`), so the arithmetic underneath is identical and
any difference is a difference in the wrapper semantics: layouts, NaN
checks, INFO shifts, leading-dimension codes, transposition, IPIV handling.
Needs the reference LAPACKE build in oracle/_ref, or the reference tree
(LAPACK_REFERENCE_DIR) to compile it; skipped where neither is present."""
import ctypes
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE = os.path.join(ROOT, "oracle")


def _ref_tree():
    """The reference tree the oracle recipe reads (its REF variable)."""
    out = subprocess.run(["make", "-s", "-C", ORACLE, "ref-path"], capture_output=True, text=True)
    return out.stdout.strip()


@pytest.fixture(scope="module")
def libs():
    built = os.path.join(ORACLE, "_ref", "libref_lapacke.so")
    if os.path.isdir(os.path.join(_ref_tree(), "LAPACKE")):
        subprocess.run(["make", "-s", "-C", ORACLE, "ref"], check=True)
    elif not os.path.exists(built):
        pytest.skip("reference LAPACKE sources not present (set LAPACK_REFERENCE_DIR)")
    subprocess.run(["make", "-s", "-C", ORACLE, "ours"], check=True)
    ref = ctypes.CDLL(os.path.join(ORACLE, "_ref", "libref_lapacke.so"))
    ours = ctypes.CDLL(os.path.join(ORACLE, "_ref", "libours_lapacke.so"))
    return ref, ours


def p(v):
    return v.ctypes.data_as(ctypes.c_void_p)


def _mat(m, n, seed, layout, ld_extra=0):
    rng = np.random.default_rng(seed)
    a = rng.standard_normal((m, n))
    if layout == 102:          # column-major storage with ld = m + extra
        ld = max(1, m + ld_extra)
        buf = np.full((max(n, 1), ld), 7.25)
        buf[:n, :m] = a.T
    else:                      # row-major, ld = n + extra
        ld = max(1, n + ld_extra)
        buf = np.full((max(m, 1), ld), 7.25)
        buf[:m, :n] = a
    return buf, ld


def _both(libs, fname, build, capfd):
    outs = []
    for L in libs:
        args, arrays = build()
        L.LAPACKE_set_nancheck(1)
        rc = getattr(L, fname)(*args)
        ctypes.CDLL(None).fflush(None)
        printed = capfd.readouterr().out
        outs.append((rc, [x.copy() for x in arrays], printed))
    (r1, a1, p1), (r2, a2, p2) = outs
    assert r1 == r2, (fname, r1, r2)
    for x, y in zip(a1, a2):
        assert x.tobytes() == y.tobytes(), fname
    assert p1 == p2, (p1, p2)
    return r1


CASES = [(layout, n, nrhs, extra) for layout in (101, 102) for n in (0, 1, 5, 17) for nrhs in (0, 1, 3)
         for extra in (0, 2)]


@pytest.mark.parametrize("layout,n,nrhs,extra", CASES)
def test_gesv_getrf_getrs_dsgesv(libs, capfd, layout, n, nrhs, extra):
    def gesv():
        a, lda = _mat(n, n, 1 + n, layout, extra)
        b, ldb = _mat(n, nrhs, 2 + n, layout, extra)
        ip = np.zeros(max(n, 1), dtype=np.int32)
        return (layout, n, nrhs, p(a), lda, p(ip), p(b), ldb), (a, b, ip)
    _both(libs, "LAPACKE_dgesv", gesv, capfd)

    def getrf():
        a, lda = _mat(n, n + 2, 3 + n, layout, extra)
        ip = np.zeros(max(n, 1), dtype=np.int32)
        return (layout, n, n + 2, p(a), lda, p(ip)), (a, ip)
    _both(libs, "LAPACKE_dgetrf", getrf, capfd)

    for tr in (b"N", b"T"):
        def getrs():
            a, lda = _mat(n, n, 4 + n, layout, extra)
            a[np.arange(min(a.shape)), np.arange(min(a.shape))] += 4.0
            b, ldb = _mat(n, nrhs, 5 + n, layout, extra)
            ip = np.arange(1, max(n, 1) + 1, dtype=np.int32)[::-1].copy()
            ip = np.maximum(ip, np.arange(1, max(n, 1) + 1, dtype=np.int32))
            return (layout, ctypes.c_char(tr), n, nrhs, p(a), lda, p(ip), p(b), ldb), (b,)
        _both(libs, "LAPACKE_dgetrs", getrs, capfd)

    def dsgesv():
        a, lda = _mat(n, n, 6 + n, layout, extra)
        b, ldb = _mat(n, nrhs, 7 + n, layout, extra)
        x, ldx = _mat(n, nrhs, 8 + n, layout, extra)
        ip = np.zeros(max(n, 1), dtype=np.int32)
        it = np.zeros(1, dtype=np.int32)
        return (layout, n, nrhs, p(a), lda, p(ip), p(b), ldb, p(x), ldx, p(it)), (a, x, ip, it)
    _both(libs, "LAPACKE_dsgesv", dsgesv, capfd)


@pytest.mark.parametrize("layout", [101, 102])
def test_error_and_nan_paths(libs, capfd, layout):
    def bad_layout():
        a = np.eye(3)
        b = np.ones(3)
        ip = np.zeros(3, dtype=np.int32)
        return (55, 3, 1, p(a), 3, p(ip), p(b), 3), (a,)
    assert _both(libs, "LAPACKE_dgesv", bad_layout, capfd) == -1

    def nan_a():
        a, lda = _mat(4, 4, 1, layout)
        a.flat[1] = np.nan
        b, ldb = _mat(4, 1, 2, layout)
        ip = np.zeros(4, dtype=np.int32)
        return (layout, 4, 1, p(a), lda, p(ip), p(b), ldb), (a, b)
    assert _both(libs, "LAPACKE_dgesv", nan_a, capfd) == -4

    def small_ld():
        a, lda = _mat(4, 4, 1, layout)
        b, ldb = _mat(4, 2, 2, layout)
        ip = np.zeros(4, dtype=np.int32)
        return (layout, 4, 2, p(a), 3, p(ip), p(b), ldb), (a, b)
    _both(libs, "LAPACKE_dgesv", small_ld, capfd)

    for fn in ("LAPACKE_dlag2s",):
        def lag2s():
            a, lda = _mat(5, 3, 9, layout)
            sa = np.full(a.shape, 1.5, dtype=np.float32)
            return (layout, 5, 3, p(a), lda, p(sa), lda), (sa,)
        _both(libs, fn, lag2s, capfd)


@pytest.mark.parametrize("layout", [101, 102])
@pytest.mark.parametrize("incx", [1, -1])
def test_laswp(libs, capfd, layout, incx):
    def laswp():
        a, lda = _mat(9, 4, 3, layout)
        ip = np.array([1, 3, 2, 9, 5, 5], dtype=np.int32)   # IPIV(K1..K2) = IPIV(2..6) is read
        return (layout, 4, p(a), lda, 2, 6, p(ip), incx), (a,)
    _both(libs, "LAPACKE_dlaswp", laswp, capfd)


WIDE_CASES = [(layout, n, nrhs, extra) for layout in (101, 102) for n in (0, 1, 6, 13) for nrhs in (0, 2)
              for extra in (0, 3)]


def _factored(libs, n, layout, extra, seed):
    """A, its LU (through the oracle's DGETRF) and IPIV in the given layout."""
    import oracle
    a, lda = _mat(n, n, seed, layout, extra)
    lu = a.copy()
    ip = np.zeros(max(n, 1), dtype=np.int32)
    if n:
        if layout == 102:
            f = np.asfortranarray(lu[:n, :n].T)
        else:
            f = np.asfortranarray(lu[:n, :n])
        lu_f, ipv, _ = oracle.getrf(f)
        if layout == 102:
            lu[:n, :n] = lu_f.T
        else:
            lu[:n, :n] = lu_f
        ip[:n] = ipv
    return a, lda, lu, ip


@pytest.mark.parametrize("layout,n,nrhs,extra", WIDE_CASES)
def test_gecon_gerfs_gesvx(libs, capfd, layout, n, nrhs, extra):
    """LAPACKE_dgecon / dgerfs / dgesvx (and _work via them): same return
    codes, outputs and messages as the reference wrappers."""
    def gecon():
        a, lda, lu, ip = _factored(libs, n, layout, extra, 40 + n)
        rc = np.zeros(1)
        return (layout, ctypes.c_char(b"1"), n, p(lu), lda, ctypes.c_double(3.5), p(rc)), (rc,)
    _both(libs, "LAPACKE_dgecon", gecon, capfd)

    def gerfs():
        a, lda, lu, ip = _factored(libs, n, layout, extra, 50 + n)
        b, ldb = _mat(n, nrhs, 51 + n, layout, extra)
        x = b.copy()
        fe = np.zeros(max(nrhs, 1))
        be = np.zeros(max(nrhs, 1))
        return ((layout, ctypes.c_char(b"N"), n, nrhs, p(a), lda, p(lu), lda, p(ip), p(b), ldb, p(x), ldb, p(fe),
                 p(be)), (x, fe, be))
    _both(libs, "LAPACKE_dgerfs", gerfs, capfd)

    for fact in (b"N", b"E"):
        for trans in (b"N", b"T"):
            def gesvx():
                a, lda = _mat(n, n, 60 + n, layout, extra)
                if n:
                    a[0, :] *= 1e7                     # badly scaled, so EQUED != 'N' with FACT = 'E'
                af = np.zeros_like(a)
                ip = np.zeros(max(n, 1), dtype=np.int32)
                eq = ctypes.create_string_buffer(b"N", 2)
                r = np.zeros(max(n, 1))
                c = np.zeros(max(n, 1))
                b, ldb = _mat(n, nrhs, 61 + n, layout, extra)
                x = np.zeros_like(b)
                rc = np.zeros(1)
                fe = np.zeros(max(nrhs, 1))
                be = np.zeros(max(nrhs, 1))
                rp = np.zeros(1)
                eqa = np.frombuffer(eq, dtype=np.uint8)
                return ((layout, ctypes.c_char(fact), ctypes.c_char(trans), n, nrhs, p(a), lda, p(af), lda, p(ip),
                         eq, p(r), p(c), p(b), ldb, p(x), ldb, p(rc), p(fe), p(be), p(rp)),
                        (a, af, ip, eqa, r, c, b, x, rc, fe, be, rp))
            _both(libs, "LAPACKE_dgesvx", gesvx, capfd)


def test_gesvx_nan_and_ld_codes(libs, capfd):
    """The NaN-check and row-major leading-dimension codes of the three
    wrappers (including the FACT = 'F' checks of AF, R and C)."""
    n, nrhs = 3, 1
    for layout in (101, 102):
        def call(fact, equed, nan_in, lda_off=0, ldb_off=0):
            def build():
                a, lda = _mat(n, n, 3, layout)
                af = a.copy()
                ip = np.array([1, 2, 3], dtype=np.int32)
                r = np.ones(n)
                c = np.ones(n)
                b, ldb = _mat(n, nrhs, 4, layout)
                x = np.zeros_like(b)
                {"a": a, "af": af, "b": b, "r": r, "c": c}.get(nan_in, np.zeros(1))[0] = np.nan
                eq = ctypes.create_string_buffer(equed, 2)
                return ((layout, ctypes.c_char(fact), ctypes.c_char(b"N"), n, nrhs, p(a), lda - lda_off, p(af),
                         lda, p(ip), eq, p(r), p(c), p(b), ldb - ldb_off, p(x), ldb, p(np.zeros(1)),
                         p(np.zeros(1)), p(np.zeros(1)), p(np.zeros(1))), (x,))
            return _both(libs, "LAPACKE_dgesvx", build, capfd)
        assert call(b"N", b"N", "a") == -6
        assert call(b"F", b"N", "af") == -8
        assert call(b"N", b"N", "b") == -14
        assert call(b"F", b"C", "c") == -13
        assert call(b"F", b"R", "r") == -12
        if layout == 101:
            assert call(b"N", b"N", None, lda_off=1) == -7
            assert call(b"N", b"N", None, ldb_off=1) == -15


@pytest.mark.parametrize("layout,n,extra", [(l, n, e) for l in (101, 102) for n in (0, 1, 6, 13, 70) for e in (0, 3)])
def test_getri(libs, capfd, layout, n, extra):
    """LAPACKE_dgetri (workspace query, then the inverse) and its error codes."""
    def getri():
        a, lda, lu, ip = _factored(libs, n, layout, extra, 80 + n)
        return (layout, n, p(lu), lda, p(ip)), (lu,)
    _both(libs, "LAPACKE_dgetri", getri, capfd)

    def bad_ld():
        a, lda, lu, ip = _factored(libs, max(n, 2), layout, 0, 81)
        return (layout, max(n, 2), p(lu), lda - 1, p(ip)), (lu,)
    _both(libs, "LAPACKE_dgetri", bad_ld, capfd)


def _spd(n, seed, layout, extra, dtype=np.float64, shift=1.0):
    """A symmetric positive definite n x n matrix M M^T / n + shift * I in
    the layout's storage (padding 7.25); `shift` < 0 makes it indefinite."""
    rng = np.random.default_rng(seed)
    m = rng.standard_normal((n, n))
    a = m @ m.T / max(n, 1) + shift * np.eye(n)
    ld = max(1, n + extra)
    buf = np.full((max(n, 1), ld), 7.25)
    buf[:n, :n] = a            # symmetric: the same bytes in either layout
    return buf.astype(dtype), ld


CHOL_CASES = [(layout, uplo, n, nrhs, extra) for layout in (101, 102) for uplo in (b"U", b"L")
              for n in (0, 1, 5, 17, 70) for nrhs in (0, 2) for extra in (0, 3)]


@pytest.mark.parametrize("layout,uplo,n,nrhs,extra", CHOL_CASES)
def test_potrf_potrs_posv_dsposv(libs, capfd, layout, uplo, n, nrhs, extra):
    """LAPACKE_{d,s}potrf, {d,s}potrs, dposv and dsposv (and their _work
    forms through them): the stored triangle transposed for row-major, the
    other triangle untouched, the same INFO and ITER as the reference
    wrappers (LAPACKE/src/lapacke_dpotrf.c, dpotrs.c, dposv.c, dsposv.c)."""
    u = ctypes.c_char(uplo)
    for fn, dt in (("LAPACKE_dpotrf", np.float64), ("LAPACKE_spotrf", np.float32)):
        def potrf():
            a, lda = _spd(n, 90 + n, layout, extra, dt)
            return (layout, u, n, p(a), lda), (a,)
        _both(libs, fn, potrf, capfd)

    for fn, dt in (("LAPACKE_dpotrs", np.float64), ("LAPACKE_spotrs", np.float32)):
        def potrs():
            a, lda = _spd(n, 91 + n, layout, extra, dt, shift=4.0)   # used as a factor as it stands
            b, ldb = _mat(n, nrhs, 92 + n, layout, extra)
            b = b.astype(dt)
            return (layout, u, n, nrhs, p(a), lda, p(b), ldb), (a, b)
        _both(libs, fn, potrs, capfd)

    def posv():
        a, lda = _spd(n, 93 + n, layout, extra)
        b, ldb = _mat(n, nrhs, 94 + n, layout, extra)
        return (layout, u, n, nrhs, p(a), lda, p(b), ldb), (a, b)
    _both(libs, "LAPACKE_dposv", posv, capfd)

    for shift in (1.0, -0.5):                  # -0.5: not positive definite, ITER = -3, FP64 fallback INFO > 0
        def dsposv():
            a, lda = _spd(n, 95 + n, layout, extra, shift=shift)
            b, ldb = _mat(n, nrhs, 96 + n, layout, extra)
            x, ldx = _mat(n, nrhs, 97 + n, layout, extra)
            it = np.zeros(1, dtype=np.int32)
            # INFO > 0 leaves X unset; row-major then copies back the
            # wrapper's uninitialised X buffer, so X is compared only on success
            outs = (a, x, it) if shift > 0 or layout == 102 else (a, it)
            return (layout, u, n, nrhs, p(a), lda, p(b), ldb, p(x), ldx, p(it)), outs
        _both(libs, "LAPACKE_dsposv", dsposv, capfd)


@pytest.mark.parametrize("layout", [101, 102])
def test_chol_error_and_nan_codes(libs, capfd, layout):
    """Bad layout (-1), bad UPLO (Fortran -1, LAPACKE -2), row-major leading
    dimensions (-5 / -6 / -8 / -10), NaN inside the stored triangle (-4 / -5 /
    -7) and outside it (not checked), an indefinite matrix (INFO > 0)."""
    def call(fn, uplo=b"U", n=6, nrhs=2, lda_off=0, ldb_off=0, ldx_off=0, nan_at=None, shift=1.0, lay=layout):
        def build():
            a, lda = _spd(n, 7, layout, 0, shift=shift)
            if nan_at is not None:
                a[nan_at] = np.nan
            b, ldb = _mat(n, nrhs, 8, layout)
            x, ldx = _mat(n, nrhs, 9, layout)
            it = np.zeros(1, dtype=np.int32)
            u = ctypes.c_char(uplo)
            if fn == "LAPACKE_dpotrf":
                return (lay, u, n, p(a), lda - lda_off), (a,)
            if fn in ("LAPACKE_dpotrs", "LAPACKE_dposv"):
                return (lay, u, n, nrhs, p(a), lda - lda_off, p(b), ldb - ldb_off), (a, b)
            # INFO != 0 leaves X unset, and row-major copies back the
            # wrapper's uninitialised X buffer: X is compared column-major only
            outs = (a, x, it) if layout == 102 else (a, it)
            return ((lay, u, n, nrhs, p(a), lda - lda_off, p(b), ldb - ldb_off, p(x), ldx - ldx_off, p(it)),
                    outs)
        return _both(libs, fn, build, capfd)

    for fn in ("LAPACKE_dpotrf", "LAPACKE_dpotrs", "LAPACKE_dposv", "LAPACKE_dsposv"):
        assert call(fn, lay=7) == -1
        assert call(fn, uplo=b"X") == -2
        # NaN in row 0, column 3: upper triangle in column-major storage
        # (buf[col, row]) is buf[3, 0]; row-major upper is buf[0, 3]
        upper_nan = (3, 0) if layout == 102 else (0, 3)
        lower_nan = upper_nan[::-1]
        code = -4 if fn == "LAPACKE_dpotrf" else -5
        assert call(fn, uplo=b"U", nan_at=upper_nan) == code
        assert call(fn, uplo=b"L", nan_at=lower_nan) == code
        call(fn, uplo=b"U", nan_at=lower_nan)       # outside the stored triangle: no NaN code
        call(fn, uplo=b"L", nan_at=upper_nan)
        if fn != "LAPACKE_dpotrs":
            assert call(fn, shift=-0.5) > 0
        if layout == 101:
            assert call(fn, lda_off=1) == (-5 if fn == "LAPACKE_dpotrf" else -6)
            if fn != "LAPACKE_dpotrf":
                assert call(fn, ldb_off=1) == -8
            if fn == "LAPACKE_dsposv":
                assert call(fn, ldx_off=1) == -10


def _zmat(m, n, seed, layout, ld_extra=0, dtype=np.complex128):
    rng = np.random.default_rng(seed)
    a = rng.standard_normal((m, n)) + 1j * rng.standard_normal((m, n))
    if layout == 102:
        ld = max(1, m + ld_extra)
        buf = np.full((max(n, 1), ld), 7.25 - 3.5j)
        buf[:n, :m] = a.T
    else:
        ld = max(1, n + ld_extra)
        buf = np.full((max(m, 1), ld), 7.25 - 3.5j)
        buf[:m, :n] = a
    return buf.astype(dtype), ld


@pytest.mark.parametrize("pre,dtype", [("z", np.complex128), ("c", np.complex64)])
@pytest.mark.parametrize("layout,n,nrhs,extra", CASES)
def test_complex_getrf_getrs_gesv(libs, capfd, pre, dtype, layout, n, nrhs, extra):
    """LAPACKE_{z,c}gesv, {z,c}getrf, {z,c}getrs (TRANS N, T, C) against the
    reference wrappers (LAPACKE/src/lapacke_zgesv.c ...)."""
    def gesv():
        a, lda = _zmat(n, n, 1 + n, layout, extra, dtype)
        b, ldb = _zmat(n, nrhs, 2 + n, layout, extra, dtype)
        ip = np.zeros(max(n, 1), dtype=np.int32)
        return (layout, n, nrhs, p(a), lda, p(ip), p(b), ldb), (a, b, ip)
    _both(libs, f"LAPACKE_{pre}gesv", gesv, capfd)

    def getrf():
        a, lda = _zmat(n, n + 2, 3 + n, layout, extra, dtype)
        ip = np.zeros(max(n, 1), dtype=np.int32)
        return (layout, n, n + 2, p(a), lda, p(ip)), (a, ip)
    _both(libs, f"LAPACKE_{pre}getrf", getrf, capfd)

    for tr in (b"N", b"T", b"C"):
        def getrs():
            a, lda = _zmat(n, n, 4 + n, layout, extra, dtype)
            a[np.arange(min(a.shape)), np.arange(min(a.shape))] += 4.0
            b, ldb = _zmat(n, nrhs, 5 + n, layout, extra, dtype)
            ip = np.maximum(np.arange(1, max(n, 1) + 1, dtype=np.int32)[::-1].copy(),
                            np.arange(1, max(n, 1) + 1, dtype=np.int32))
            return (layout, ctypes.c_char(tr), n, nrhs, p(a), lda, p(ip), p(b), ldb), (b,)
        _both(libs, f"LAPACKE_{pre}getrs", getrs, capfd)


@pytest.mark.parametrize("layout,n,nrhs,extra", CASES)
def test_zcgesv(libs, capfd, layout, n, nrhs, extra):
    """LAPACKE_zcgesv (and _work through it): ITER, A, X, IPIV as the
    reference wrapper (LAPACKE/src/lapacke_zcgesv.c)."""
    def zcgesv():
        a, lda = _zmat(n, n, 6 + n, layout, extra)
        a[np.arange(min(a.shape)), np.arange(min(a.shape))] += 3.0
        b, ldb = _zmat(n, nrhs, 7 + n, layout, extra)
        x, ldx = _zmat(n, nrhs, 8 + n, layout, extra)
        ip = np.zeros(max(n, 1), dtype=np.int32)
        it = np.zeros(1, dtype=np.int32)
        return (layout, n, nrhs, p(a), lda, p(ip), p(b), ldb, p(x), ldx, p(it)), (a, x, ip, it)
    _both(libs, "LAPACKE_zcgesv", zcgesv, capfd)


@pytest.mark.parametrize("layout", [101, 102])
def test_complex_error_and_nan_codes(libs, capfd, layout):
    """Bad layout (-1); a NaN in either part of A or B (-4 / -7, -5 / -8 for
    xGETRS); row-major leading dimensions too small; INFO > 0 for a zero
    column."""
    def gesv(lay=layout, nan=None, lda_off=0, ldb_off=0, zero_col=False):
        def build():
            a, lda = _zmat(4, 4, 1, layout)
            b, ldb = _zmat(4, 2, 2, layout)
            if nan == "a_re":
                a.flat[1] = complex(np.nan, 1.0)
            elif nan == "a_im":
                a.flat[2] = complex(1.0, np.nan)
            elif nan == "b":
                b.flat[0] = complex(0.0, np.nan)
            if zero_col:
                if layout == 102:
                    a[2, :4] = 0
                else:
                    a[:4, 2] = 0
            ip = np.zeros(4, dtype=np.int32)
            return (lay, 4, 2, p(a), lda - lda_off, p(ip), p(b), ldb - ldb_off), (a, b, ip)
        return build
    for fn in ("LAPACKE_zgesv",):
        assert _both(libs, fn, gesv(lay=9), capfd) == -1
        assert _both(libs, fn, gesv(nan="a_re"), capfd) == -4
        assert _both(libs, fn, gesv(nan="a_im"), capfd) == -4
        assert _both(libs, fn, gesv(nan="b"), capfd) == -7
        assert _both(libs, fn, gesv(zero_col=True), capfd) == 3
        if layout == 101:
            assert _both(libs, fn, gesv(lda_off=1), capfd) == -5
            assert _both(libs, fn, gesv(ldb_off=1), capfd) == -8
