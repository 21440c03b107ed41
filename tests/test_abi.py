"""The C-ABI boundary on the CPU (no GPU work is started): the shared
library loads and exports every function declared in include/lapack_gb300.h,
argument errors are reported through xerbla_ with the reference's INFO codes
(the INFOT tables of TESTING/LIN/derrge.f and derrab.f) before any device
work, and the LAPACKE layer's own argument checks return the reference codes."""
import ctypes
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "lapack_gb300.h")


def _declared():
    txt = open(HEADER).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    names = re.findall(r"\b([A-Za-z_][A-Za-z0-9_]*)\s*\(", txt)
    skip = {"if", "defined", "sizeof", "void"}
    return sorted({n for n in names if n not in skip and not n.isupper() and n not in ("malloc_fn", "free_fn")})


@pytest.fixture(scope="module")
def lib():
    import lapack_gb300
    try:
        return lapack_gb300.lib()
    except lapack_gb300.LibraryMissing:
        lapack_gb300.build()
        return lapack_gb300.lib()


def test_every_declared_symbol_is_exported(lib):
    names = _declared()
    assert len(names) > 50
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


ERR_GETRF = [((-1, 0, 1), 1), ((0, -1, 1), 2), ((2, 1, 1), 4)]
ERR_GETRS = [(("/", 0, 0, 1, 1), 1), (("N", -1, 0, 1, 1), 2), (("N", 0, -1, 1, 1), 3),
             (("N", 2, 1, 1, 2), 5), (("N", 2, 1, 2, 1), 8)]
ERR_GESV = [((-1, 0, 1, 1), 1), ((0, -1, 1, 1), 2), ((2, 1, 1, 2), 4), ((2, 1, 2, 1), 7)]
ERR_DSGESV = [((-1, 0, 1, 1, 1), 1), ((0, -1, 1, 1, 1), 2), ((2, 1, 1, 2, 2), 4), ((2, 1, 2, 1, 2), 7),
              ((2, 1, 2, 2, 1), 9)]
ERR_GERFS = [(("/", 0, 0, 1, 1, 1, 1), 1), (("N", -1, 0, 1, 1, 1, 1), 2), (("N", 0, -1, 1, 1, 1, 1), 3),
             (("N", 2, 1, 1, 2, 2, 2), 5), (("N", 2, 1, 2, 1, 2, 2), 7), (("N", 2, 1, 2, 2, 1, 2), 10),
             (("N", 2, 1, 2, 2, 2, 1), 12)]        # TESTING/LIN/derrge.f:186-216
ERR_LATRS = [(("/", "N", "N", "N", 0, 1), 1), (("U", "/", "N", "N", 0, 1), 2), (("U", "N", "/", "N", 0, 1), 3),
             (("U", "N", "N", "/", 0, 1), 4), (("U", "N", "N", "N", -1, 1), 5),
             (("U", "N", "N", "N", 2, 1), 7)]       # TESTING/LIN/derrtr.f:228-247
ERR_GESVX = [(("/", "N", 0, 0, 1, 1, "N", 1, 1), 1), (("N", "/", 0, 0, 1, 1, "N", 1, 1), 2),
             (("N", "N", -1, 0, 1, 1, "N", 1, 1), 3), (("N", "N", 0, -1, 1, 1, "N", 1, 1), 4),
             (("N", "N", 2, 1, 1, 2, "N", 2, 2), 6), (("N", "N", 2, 1, 2, 1, "N", 2, 2), 8),
             (("F", "N", 0, 0, 1, 1, "/", 1, 1), 10), (("F", "N", 1, 0, 1, 1, "R", 1, 1), 11),
             (("F", "N", 1, 0, 1, 1, "C", 1, 1), 12), (("N", "N", 2, 1, 2, 2, "N", 1, 2), 14),
             (("N", "N", 2, 1, 2, 2, "N", 2, 1), 16)]   # TESTING/LIN/derrvx.f:151-200
ERR_GETRI = [((-1, 1, 1), 1), ((2, 1, 4), 3), ((2, 2, 1), 6)]   # TESTING/LIN/derrge.f:157-165, and LWORK < N
ERR_POTRF = [(("/", 0, 1), 1), (("U", -1, 1), 2), (("U", 2, 1), 4)]      # TESTING/LIN/derrpo.f:133-142
ERR_POTRS = [(("/", 0, 0, 1, 1), 1), (("U", -1, 0, 1, 1), 2), (("U", 0, -1, 1, 1), 3),
             (("U", 2, 1, 1, 2), 5), (("U", 2, 1, 2, 1), 7)]                 # derrpo.f:172-187
ERR_SPOSV = [(("/", 0, 0, 1, 1, 1), 1), (("U", -1, 0, 1, 1, 1), 2), (("U", 0, -1, 1, 1, 1), 3),
             (("U", 2, 1, 1, 2, 2), 5), (("U", 2, 1, 2, 1, 2), 7), (("U", 2, 1, 2, 2, 1), 9)]   # derrac.f:110-128
ERR_GECON = [(("/", 0, 1, 1.0), 1), (("1", -1, 1, 1.0), 2), (("1", 2, 1, 1.0), 4),
             (("1", 2, 2, -1.0), 5)]                # derrge.f:218-229, and ANORM < 0


def _i(v):
    return ctypes.byref(ctypes.c_int(v))


def test_fortran_abi_error_exits(lib):
    import lapack_gb300 as g
    g.xerbla_capture(True)
    try:
        a = np.zeros(16)
        ip = np.zeros(4, dtype=np.int32)
        p = lambda v: v.ctypes.data_as(ctypes.c_void_p)
        info = ctypes.c_int(0)
        for (m, n, lda), code in ERR_GETRF:
            lib.dgetrf_(_i(m), _i(n), p(a), _i(lda), p(ip), ctypes.byref(info))
            assert info.value == -code and g.xerbla_last() == ("DGETRF", code)
            lib.sgetrf_(_i(m), _i(n), p(a), _i(lda), p(ip), ctypes.byref(info))
            assert info.value == -code and g.xerbla_last() == ("SGETRF", code)
        for (tr, n, nrhs, lda, ldb), code in ERR_GETRS:
            lib.dgetrs_(ctypes.c_char_p(tr.encode()), _i(n), _i(nrhs), p(a), _i(lda), p(ip), p(a), _i(ldb),
                        ctypes.byref(info), ctypes.c_size_t(1))
            assert info.value == -code and g.xerbla_last() == ("DGETRS", code)
        for (n, nrhs, lda, ldb), code in ERR_GESV:
            lib.dgesv_(_i(n), _i(nrhs), p(a), _i(lda), p(ip), p(a), _i(ldb), ctypes.byref(info))
            assert info.value == -code and g.xerbla_last() == ("DGESV", code)
        it = ctypes.c_int(0)
        for (n, nrhs, lda, ldb, ldx), code in ERR_DSGESV:
            lib.dsgesv_(_i(n), _i(nrhs), p(a), _i(lda), p(ip), p(a), _i(ldb), p(a), _i(ldx), p(a), p(a),
                        ctypes.byref(it), ctypes.byref(info))
            assert info.value == -code and g.xerbla_last() == ("DSGESV", code)
        w = np.zeros(8)
        for (tr, n, nrhs, lda, ldaf, ldb, ldx), code in ERR_GERFS:
            lib.dgerfs_(ctypes.c_char_p(tr.encode()), _i(n), _i(nrhs), p(a), _i(lda), p(a), _i(ldaf), p(ip), p(a),
                        _i(ldb), p(a), _i(ldx), p(w), p(w), p(w), p(ip), ctypes.byref(info), ctypes.c_size_t(1))
            assert info.value == -code and g.xerbla_last() == ("DGERFS", code)
        rc = ctypes.c_double(0.0)
        for (ul, tr, dg, nm, n, lda), code in ERR_LATRS:
            c = lambda ch: ctypes.c_char_p(ch.encode())
            lib.dlatrs_(c(ul), c(tr), c(dg), c(nm), _i(n), p(a), _i(lda), p(w), ctypes.byref(rc), p(w),
                        ctypes.byref(info), *([ctypes.c_size_t(1)] * 4))
            assert info.value == -code and g.xerbla_last() == ("DLATRS", code)
        zero = np.zeros(4)                           # R, C with a non-positive entry
        for (fa, tr, n, nrhs, lda, ldaf, eq, ldb, ldx), code in ERR_GESVX:
            c = lambda ch: ctypes.c_char_p(ch.encode())
            lib.dgesvx_(c(fa), c(tr), _i(n), _i(nrhs), p(a), _i(lda), p(a), _i(ldaf), p(ip), c(eq), p(zero),
                        p(zero), p(a), _i(ldb), p(a), _i(ldx), ctypes.byref(rc), p(w), p(w), p(w), p(ip),
                        ctypes.byref(info), *([ctypes.c_size_t(1)] * 3))
            assert info.value == -code and g.xerbla_last() == ("DGESVX", code)
        for (n, lda, lw), code in ERR_GETRI:
            lib.dgetri_(_i(n), p(a), _i(lda), p(ip), p(w), _i(lw), ctypes.byref(info))
            assert info.value == -code and g.xerbla_last() == ("DGETRI", code)
        wq = np.zeros(2)
        lib.dgetri_(_i(10), p(a), _i(10), p(ip), p(wq), _i(-1), ctypes.byref(info))   # workspace query: no GPU work
        assert info.value == 0 and wq[0] == 10 * g.get_option("nb64")
        cc = lambda ch: ctypes.c_char_p(ch.encode())
        for (ul, n, lda), code in ERR_POTRF:
            for pre in "ds":
                getattr(lib, pre + "potrf_")(cc(ul), _i(n), p(a), _i(lda), ctypes.byref(info), ctypes.c_size_t(1))
                assert info.value == -code and g.xerbla_last() == (pre.upper() + "POTRF", code)
        for (ul, n, nrhs, lda, ldb), code in ERR_POTRS:
            lib.dpotrs_(cc(ul), _i(n), _i(nrhs), p(a), _i(lda), p(a), _i(ldb), ctypes.byref(info), ctypes.c_size_t(1))
            assert info.value == -code and g.xerbla_last() == ("DPOTRS", code)
            lib.dposv_(cc(ul), _i(n), _i(nrhs), p(a), _i(lda), p(a), _i(ldb), ctypes.byref(info), ctypes.c_size_t(1))
            assert info.value == -code and g.xerbla_last() == ("DPOSV", code)
        itr = ctypes.c_int(0)
        for (ul, n, nrhs, lda, ldb, ldx), code in ERR_SPOSV:
            lib.dsposv_(cc(ul), _i(n), _i(nrhs), p(a), _i(lda), p(a), _i(ldb), p(a), _i(ldx), p(w), p(w),
                        ctypes.byref(itr), ctypes.byref(info), ctypes.c_size_t(1))
            assert info.value == -code and g.xerbla_last() == ("DSPOSV", code)
        for (nm, n, lda, anorm), code in ERR_GECON:
            lib.dgecon_(ctypes.c_char_p(nm.encode()), _i(n), p(a), _i(lda), ctypes.byref(ctypes.c_double(anorm)),
                        ctypes.byref(rc), p(w), p(ip), ctypes.byref(info), ctypes.c_size_t(1))
            assert info.value == -code and g.xerbla_last() == ("DGECON", code)
        # quick returns touch nothing on the device (SRC/dgecon.f:197-212)
        for n, anorm, want_rc, want_info in ((0, 1.0, 1.0, 0), (2, 0.0, 0.0, 0), (2, float("inf"), 0.0, -5)):
            lib.dgecon_(ctypes.c_char_p(b"I"), _i(n), p(a), _i(2), ctypes.byref(ctypes.c_double(anorm)),
                        ctypes.byref(rc), p(w), p(ip), ctypes.byref(info), ctypes.c_size_t(1))
            assert rc.value == want_rc and info.value == want_info
        lib.dgecon_(ctypes.c_char_p(b"O"), _i(2), p(a), _i(2), ctypes.byref(ctypes.c_double(float("nan"))),
                    ctypes.byref(rc), p(w), p(ip), ctypes.byref(info), ctypes.c_size_t(1))
        assert np.isnan(rc.value) and info.value == -5
        lib.dgetrf_(_i(0), _i(5), p(a), _i(1), p(ip), ctypes.byref(info))
        assert info.value == 0
        # complex LU: TESTING/LIN/zerrge.f:135-190, zerrvx.f:142-154
        for (m, n, lda), code in ERR_GETRF:
            lib.zgetrf_(_i(m), _i(n), p(a), _i(lda), p(ip), ctypes.byref(info))
            assert info.value == -code and g.xerbla_last() == ("ZGETRF", code)
        for (tr, n, nrhs, lda, ldb), code in ERR_GETRS:
            lib.zgetrs_(ctypes.c_char_p(tr.encode()), _i(n), _i(nrhs), p(a), _i(lda), p(ip), p(a), _i(ldb),
                        ctypes.byref(info), ctypes.c_size_t(1))
            assert info.value == -code and g.xerbla_last() == ("ZGETRS", code)
        for (n, nrhs, lda, ldb), code in ERR_GESV:
            lib.zgesv_(_i(n), _i(nrhs), p(a), _i(lda), p(ip), p(a), _i(ldb), ctypes.byref(info))
            assert info.value == -code and g.xerbla_last() == ("ZGESV", code)
        for (m, n, lda), code in ERR_GETRF:
            lib.cgetrf_(_i(m), _i(n), p(a), _i(lda), p(ip), ctypes.byref(info))
            assert info.value == -code and g.xerbla_last() == ("CGETRF", code)
            for pre in "zc":
                getattr(lib, pre + "getrf2_")(_i(m), _i(n), p(a), _i(lda), p(ip), ctypes.byref(info))
                assert info.value == -code and g.xerbla_last() == (pre.upper() + "GETRF2", code)
        for (tr, n, nrhs, lda, ldb), code in ERR_GETRS:
            lib.cgetrs_(ctypes.c_char_p(tr.encode()), _i(n), _i(nrhs), p(a), _i(lda), p(ip), p(a), _i(ldb),
                        ctypes.byref(info), ctypes.c_size_t(1))
            assert info.value == -code and g.xerbla_last() == ("CGETRS", code)
        for (n, nrhs, lda, ldb), code in ERR_GESV:
            lib.cgesv_(_i(n), _i(nrhs), p(a), _i(lda), p(ip), p(a), _i(ldb), ctypes.byref(info))
            assert info.value == -code and g.xerbla_last() == ("CGESV", code)
        for (n, nrhs, lda, ldb, ldx), code in ERR_DSGESV:      # TESTING/LIN/zerrab.f: the same table
            lib.zcgesv_(_i(n), _i(nrhs), p(a), _i(lda), p(ip), p(a), _i(ldb), p(a), _i(ldx), p(a), p(a), p(w),
                        ctypes.byref(it), ctypes.byref(info))
            assert info.value == -code and g.xerbla_last() == ("ZCGESV", code)
        lib.zgetrf_(_i(0), _i(5), p(a), _i(1), p(ip), ctypes.byref(info))
        assert info.value == 0
        lib.zcgesv_(_i(0), _i(1), p(a), _i(1), p(ip), p(a), _i(1), p(a), _i(1), p(a), p(a), p(w),
                    ctypes.byref(it), ctypes.byref(info))
        assert info.value == 0 and it.value == 0
        fb = np.full(4, 7.0)
        lib.dgerfs_(ctypes.c_char_p(b"T"), _i(0), _i(2), p(a), _i(1), p(a), _i(1), p(ip), p(a), _i(1), p(a), _i(1),
                    p(fb), p(fb[2:]), p(w), p(ip), ctypes.byref(info), ctypes.c_size_t(1))
        assert info.value == 0 and np.array_equal(fb, [0.0, 0.0, 0.0, 0.0])   # DGERFS: FERR = BERR = 0 for N = 0
    finally:
        g.xerbla_capture(False)


def test_lapacke_argument_codes(lib, capfd):
    """LAPACKE_dgesv.c / _work.c codes: bad layout -1; NaN in A -4, in B -7;
    row-major lda < n -5, ldb < nrhs -8 (no GPU work reached)."""
    import lapack_gb300 as g
    g.xerbla_capture(True)
    try:
        p = lambda v: v.ctypes.data_as(ctypes.c_void_p)
        a = np.eye(3)
        b = np.ones((3, 1))
        ip = np.zeros(3, dtype=np.int32)
        lib.LAPACKE_set_nancheck(1)
        assert lib.LAPACKE_dgesv(7, 3, 1, p(a), 3, p(ip), p(b), 3) == -1
        an = a.copy()
        an[1, 1] = np.nan
        assert lib.LAPACKE_dgesv(102, 3, 1, p(an), 3, p(ip), p(b), 3) == -4
        bn = b.copy()
        bn[2, 0] = np.nan
        assert lib.LAPACKE_dgesv(102, 3, 1, p(a), 3, p(ip), p(bn), 3) == -7
        assert lib.LAPACKE_dgesv(101, 3, 1, p(a), 2, p(ip), p(b), 1) == -5
        assert lib.LAPACKE_dgesv(101, 3, 2, p(a), 3, p(ip), p(b), 1) == -8
        assert lib.LAPACKE_dgetrs(101, ord("N"), 3, 1, p(a), 2, p(ip), p(b), 1) == -6
        assert lib.LAPACKE_dsgesv(101, 3, 2, p(a), 3, p(ip), p(b), 2, p(b), 1, p(ip)) == -10
        # column-major argument errors come back from the Fortran routine shifted by one
        assert lib.LAPACKE_dgesv(102, 3, 1, p(a), 2, p(ip), p(b), 3) == -5
        ctypes.CDLL(None).fflush(None)
        out = capfd.readouterr().out
        assert "Wrong parameter 1 in LAPACKE_dgesv" in out
        assert "Wrong parameter 5 in LAPACKE_dgesv_work" in out
    finally:
        g.xerbla_capture(False)


def test_header_accepts_c_complex_arrays(tmp_path):
    """A C caller's double _Complex / float _Complex arrays (LAPACKE's
    lapack_complex_double / _float in C) pass to the complex entry points
    without casts, and the header compiles as C99 and as C++."""
    import shutil
    import subprocess
    if shutil.which("gcc") is None:
        pytest.skip("needs gcc")
    src = tmp_path / "caller.c"
    src.write_text(
        '#include <complex.h>\n#include "lapack_gb300.h"\n'
        "void use(double _Complex *a, double _Complex *b, float _Complex *c, lapack_int *ip) {\n"
        "  lapack_int n = 2, nrhs = 1, info = 0, it = 0;\n"
        "  zgesv_(&n, &nrhs, a, &n, ip, b, &n, &info);\n"
        "  cgetrf_(&n, &n, c, &n, ip, &info);\n"
        "  (void)LAPACKE_zgesv(LAPACK_COL_MAJOR, n, nrhs, a, n, ip, b, n);\n"
        "  (void)LAPACKE_zcgesv(LAPACK_COL_MAJOR, n, nrhs, a, n, ip, b, n, b, n, &it);\n"
        "}\n")
    inc = os.path.join(ROOT, "include")
    r = subprocess.run(["gcc", "-std=c99", "-Wall", "-Werror", "-c", str(src), "-I", inc, "-o",
                        str(tmp_path / "caller.o")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    cpp = tmp_path / "caller.cpp"
    cpp.write_text('#include "lapack_gb300.h"\nint main() { return 0; }\n')
    r = subprocess.run(["g++", "-std=c++11", "-Wall", "-Werror", "-c", str(cpp), "-I", inc, "-o",
                        str(tmp_path / "caller2.o")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
