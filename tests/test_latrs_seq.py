"""Host/device code checked on the CPU.  The sequential DLATRS plan, careful
solve and DGECON rescaling step (lapack_gb300/csrc/latrs_seq.h, run on the
GPU as one-thread kernels), DGEEQU's finishing steps and the element steps
of DGETRI (lapack_gb300/csrc/getri_seq.h, one GPU thread each) and the
Cholesky steps (lapack_gb300/csrc/potrf_seq.h) are compiled with g++
from the same headers and composed exactly as the library composes them
(CNORM by sequential column sums, the plain solve by DTRSV in the reference
loop order, DLACN2 for the estimate; DGEMM for DGETRI's update), then
checked bit for bit against the oracle (SRC/dlatrs.f, SRC/dgecon.f,
SRC/dgetri.f): x, SCALE and CNORM for every UPLO / TRANS / DIAG on
well-scaled, badly scaled and overflowing triangles; RCOND on the DCHKGE
matrix types and on factors with tiny pivots; R, C and the condition
numbers of DGEEQU; the inverse for blocked and unblocked block sizes; the
Cholesky factor (D and S, both triangles, blocked and unblocked), DLANSY and
DSYMM as the Cholesky kernels compute them."""
import ctypes
import os
import shutil
import subprocess

import numpy as np
import pytest

import oracle

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "..", "lapack_gb300", "csrc")
ORACLE_DIR = os.path.join(HERE, "..", "oracle")

HARNESS = r"""
#include <cstddef>
#include <vector>
#include "latrs_seq.h"
#include "getri_seq.h"
#include "potrf_seq.h"
// xPOTRF as the library's GPU driver runs it (per-element DSYRK and DGEMM,
// per-row / per-column DTRSM, one-thread DPOTRF2 of each diagonal block).
template <typename T>
int seq_potrf_t(int upper, int n, T *a, int lda, int nb) {
  if (n == 0) return 0;
  if (nb <= 1 || nb >= n) return gb::potrf2_seq(upper, n, a, lda);
  for (int j = 0; j < n; j += nb) {
    const int jb = nb < n - j ? nb : n - j;
    T *d = a + j + (size_t)j * lda;
    if (j > 0) {
      const T *aop = upper ? a + (size_t)j * lda : a + j;
      for (int jj = 0; jj < jb; ++jj)
        for (int i = upper ? 0 : jj; i < (upper ? jj + 1 : jb); ++i) gb::syrk_elem(upper, i, jj, j, T(-1), aop, lda, d, lda);
    }
    const int info = gb::potrf2_seq(upper, jb, d, lda);
    if (info) return info + j;
    const int rest = n - j - jb;
    if (rest > 0) {
      if (!upper) {
        T *c = a + (j + jb) + (size_t)j * lda;
        if (j > 0)
          for (int jj = 0; jj < jb; ++jj)
            for (int i = 0; i < rest; ++i) gb::gemm_chol_elem(0, i, jj, j, T(-1), a + j + jb, lda, a + j, lda, c, lda);
        for (int i = 0; i < rest; ++i) gb::trsm_rltn_row(i, jb, d, lda, c, lda);
      } else {
        T *c = a + j + (size_t)(j + jb) * lda;
        if (j > 0)
          for (int jj = 0; jj < rest; ++jj)
            for (int i = 0; i < jb; ++i)
              gb::gemm_chol_elem(1, i, jj, j, T(-1), a + (size_t)j * lda, lda, a + (size_t)(j + jb) * lda, lda, c, lda);
        for (int jj = 0; jj < rest; ++jj) gb::trsm_lutn_col(jj, jb, d, lda, c, lda);
      }
    }
  }
  return 0;
}
extern "C" {
int seq_dpotrf(int upper, int n, double *a, int lda, int nb) { return seq_potrf_t<double>(upper, n, a, lda, nb); }
int seq_spotrf(int upper, int n, float *a, int lda, int nb) { return seq_potrf_t<float>(upper, n, a, lda, nb); }
double seq_dlansy_i(int upper, int n, const double *a, int lda) {
  double v = 0.0;
  for (int i = 0; i < n; ++i) {
    const double s = gb::lansy_row_sum(upper, i, n, a, lda);
    if (v < s || s != s) v = s;
  }
  return v;
}
void seq_dsymm_l(int upper, int m, int n, double alpha, const double *a, int lda, const double *b, int ldb, double *c,
                 int ldc, double *out) {
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < m; ++i) out[(size_t)i + (size_t)j * m] = gb::symm_l_elem(upper, i, j, m, alpha, a, lda, b, ldb, c, ldc);
}
void or_dtrsv(char uplo, char trans, char diag, int n, const double *a, int lda, double *x);
void or_dgemm(char ta, char tb, int m, int n, int k, double alpha, const double *a, int lda, const double *b, int ldb,
              double beta, double *c, int ldc);

// DGEEQU as the library's GPU kernels compute it: row maxima (one thread
// per row), the row finishing step, column maxima of |A|*R (any order: a
// maximum), the column finishing step.
int seq_dgeequ(int m, int n, const double *a, int lda, double *r, double *c, double *rowcnd, double *colcnd,
               double *amax) {
  for (int i = 0; i < m; ++i) {
    double v = 0.0;
    for (int j = 0; j < n; ++j) v = fmax(v, fabs(a[(size_t)i + (size_t)j * lda]));
    r[i] = v;
  }
  int info = gb::equ_finish_seq(m, r, 0, rowcnd, amax);
  if (info) return info;
  for (int j = 0; j < n; ++j) {
    double v = 0.0;
    for (int i = m - 1; i >= 0; --i) v = fmax(v, fabs(a[(size_t)i + (size_t)j * lda]) * r[i]);
    c[j] = v;
  }
  double cmax;
  return gb::equ_finish_seq(n, c, m, colcnd, &cmax);
}

// DGETRI as the library's GPU driver runs it: each kernel's per-thread
// function applied to every thread index, the update through DGEMM.
int seq_dgetri(int n, double *a, int lda, const int *ipiv, int nb) {
  for (int i = 0; i < n; ++i)
    if (a[(size_t)i + (size_t)i * lda] == 0.0) return i + 1;
  if (nb <= 1 || nb >= n) {
    gb::trti2_upper_seq(n, a, lda);
  } else {
    std::vector<double> cp((size_t)n * nb);
    for (int j = 0; j < n; j += nb) {
      const int jb = nb < n - j ? nb : n - j;
      double *bj = a + (size_t)j * lda;
      if (j > 0) {
        for (int c = 0; c < jb; ++c)
          for (int i = 0; i < j; ++i) cp[(size_t)i + (size_t)c * j] = bj[(size_t)i + (size_t)c * lda];
        for (int c = 0; c < jb; ++c)
          for (int i = 0; i < j; ++i) bj[(size_t)i + (size_t)c * lda] = gb::trmm_lun_elem(i, c, j, a, lda, cp.data(), j);
        for (int i = 0; i < j; ++i) gb::trsm_rn_row(i, 1, 1, jb, -1.0, a + j + (size_t)j * lda, lda, bj, lda);
      }
      gb::trti2_upper_seq(jb, a + j + (size_t)j * lda, lda);
    }
  }
  const int ldw = n;
  std::vector<double> w((size_t)ldw * (nb > 1 ? nb : 1));
  if (nb < 2 || nb >= n) {
    for (int j = n - 1; j >= 0; --j) {
      for (int i = j + 1; i < n; ++i) { w[i] = a[(size_t)i + (size_t)j * lda]; a[(size_t)i + (size_t)j * lda] = 0.0; }
      if (j < n - 1)
        for (int i = 0; i < n; ++i) gb::getri_gemv_row(i, j, n, a, lda, w.data());
    }
  } else {
    const int nn = ((n - 1) / nb) * nb;
    for (int j = nn; j >= 0; j -= nb) {
      const int jb = nb < n - j ? nb : n - j;
      for (int c = 0; c < jb; ++c)
        for (int i = j + c + 1; i < n; ++i) {
          w[(size_t)i + (size_t)c * ldw] = a[(size_t)i + (size_t)(j + c) * lda];
          a[(size_t)i + (size_t)(j + c) * lda] = 0.0;
        }
      if (j + jb < n)
        or_dgemm('N', 'N', n, jb, n - j - jb, -1.0, a + (size_t)(j + jb) * lda, lda, w.data() + j + jb, ldw, 1.0,
                 a + (size_t)j * lda, lda);
      for (int i = 0; i < n; ++i) gb::trsm_rn_row(i, 0, 0, jb, 1.0, w.data() + j, ldw, a + (size_t)j * lda, lda);
    }
  }
  for (int i = 0; i < n; ++i) gb::getri_swap_row(i, n, a, lda, ipiv);
  return 0;
}
void or_dlacn2(int n, double *v, double *x, int *isgn, double *est, int *kase, int isave[3]);

// DLATRS as the library runs it: CNORM (NORMIN = 'N'), plan, then the
// careful sweep or DTRSV.
void seq_dlatrs(int upper, int notran, int nounit, int normin_y, int n, const double *a, int lda, double *x,
                double *scale, double *cnorm) {
  *scale = 1.0;
  if (n == 0) return;
  if (!normin_y)
    for (int j = 0; j < n; ++j) {
      const int i0 = upper ? 0 : j + 1, i1 = upper ? j : n;
      double s = 0.0;
      for (int i = i0; i < i1; ++i) s = s + fabs(a[(size_t)i + (size_t)j * lda]);
      cnorm[j] = s;
    }
  gb::LatrsPlan p;
  gb::latrs_plan_seq(upper, notran, nounit, n, a, lda, x, cnorm, &p);
  if (p.mode == gb::kLatrsCareful) {
    gb::latrs_careful_seq(upper, notran, nounit, n, a, lda, x, cnorm, &p);
    *scale = p.scale;
  } else {
    or_dtrsv(upper ? 'U' : 'L', notran ? 'N' : 'T', nounit ? 'N' : 'U', n, a, lda, x);
  }
}

// DGECON as the library's host loop runs it (n > 0, 0 < ANORM finite).
double seq_dgecon(int onenrm, int n, const double *a, int lda, double anorm, double *work, int *iwork) {
  double ainvnm = 0.0;
  int kase = 0, isave[3] = {0, 0, 0}, normin_y = 0;
  const int kase1 = onenrm ? 1 : 2;
  double *x = work, *v = work + n, *cl = work + 2 * (size_t)n, *cu = work + 3 * (size_t)n;
  for (;;) {
    or_dlacn2(n, v, x, iwork, &ainvnm, &kase, isave);
    if (kase == 0) break;
    double sl = 1.0, su = 1.0;
    if (kase == kase1) {
      seq_dlatrs(0, 1, 0, normin_y, n, a, lda, x, &sl, cl);
      seq_dlatrs(1, 1, 1, normin_y, n, a, lda, x, &su, cu);
    } else {
      seq_dlatrs(1, 0, 1, normin_y, n, a, lda, x, &su, cu);
      seq_dlatrs(0, 0, 0, normin_y, n, a, lda, x, &sl, cl);
    }
    normin_y = 1;
    if (gb::gecon_rescale_seq(n, x, sl, su)) return 0.0;
  }
  return ainvnm != 0.0 ? (1.0 / ainvnm) / anorm : 0.0;
}
}
"""


@pytest.fixture(scope="module")
def seq(tmp_path_factory):
    if shutil.which("g++") is None:
        pytest.skip("needs g++")
    d = tmp_path_factory.mktemp("latrs")
    src = d / "seq.cpp"
    src.write_text(HARNESS)
    so = d / "libseq.so"
    oracle.lib()   # builds liboracle.so when missing
    cmd = ["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fPIC", "-shared", "-I", CSRC, str(src), "-o", str(so),
           "-L", ORACLE_DIR, "-loracle", "-Wl,-rpath," + os.path.abspath(ORACLE_DIR)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    L = ctypes.CDLL(str(so))
    p = ctypes.c_void_p
    L.seq_dlatrs.argtypes = [ctypes.c_int] * 5 + [p, ctypes.c_int, p, p, p]
    L.seq_dgecon.argtypes = [ctypes.c_int, ctypes.c_int, p, ctypes.c_int, ctypes.c_double, p, p]
    L.seq_dgecon.restype = ctypes.c_double
    L.seq_dgetri.argtypes = [ctypes.c_int, p, ctypes.c_int, p, ctypes.c_int]
    L.seq_dgeequ.argtypes = [ctypes.c_int, ctypes.c_int, p, ctypes.c_int, p, p, p, p, p]
    L.seq_dpotrf.argtypes = [ctypes.c_int, ctypes.c_int, p, ctypes.c_int, ctypes.c_int]
    L.seq_spotrf.argtypes = [ctypes.c_int, ctypes.c_int, p, ctypes.c_int, ctypes.c_int]
    L.seq_dlansy_i.argtypes = [ctypes.c_int, ctypes.c_int, p, ctypes.c_int]
    L.seq_dlansy_i.restype = ctypes.c_double
    L.seq_dsymm_l.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double, p, ctypes.c_int, p,
                              ctypes.c_int, p, ctypes.c_int, p]
    return L


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def _seq_latrs(L, t, b, uplo, trans, diag, cnorm=None):
    t = np.asfortranarray(t, dtype=np.float64)
    n = t.shape[0]
    x = np.array(b, dtype=np.float64, copy=True)
    cn = np.zeros(max(n, 1)) if cnorm is None else np.array(cnorm, dtype=np.float64, copy=True)
    sc = np.zeros(1)
    L.seq_dlatrs(int(uplo == "U"), int(trans == "N"), int(diag == "N"), int(cnorm is not None), n, _ptr(t),
                 max(1, n), _ptr(x), _ptr(sc), _ptr(cn))
    return x, float(sc[0]), cn[:n]


COMBOS = [(u, t, d) for u in "UL" for t in "NT" for d in "NU"]


def _cases(uplo, diag, seed):
    rng = np.random.default_rng(seed)
    out = []
    for n, kind in ((1, "plain"), (7, "plain"), (120, "plain"), (6, "tiny"), (33, "tiny"), (200, "tiny"),
                    (40, "mixed"), (25, "huge")):
        t = rng.standard_normal((n, n))
        if kind == "plain":
            t[np.diag_indices(n)] = 2.0 + rng.random(n)
        elif kind == "tiny":
            if diag == "N":
                t[np.diag_indices(n)] = 1e-80 * (1 + rng.random(n))
            else:
                t *= 1e80
        elif kind == "mixed":
            d = np.ones(n)
            d[::7] = 1e-60
            t[np.diag_indices(n)] = d
        else:   # column sums beyond BIGNUM and beyond overflow: the TSCAL branches
            t *= 1e300
            t[0, n - 1] = t[n - 1, 0] = 1.7e308
        t = np.triu(t) if uplo == "U" else np.tril(t)
        out.append((n, kind, t, rng.standard_normal(n)))
    return out


@pytest.mark.parametrize("uplo,trans,diag", COMBOS)
def test_dlatrs_seq_bitwise_vs_oracle(seq, uplo, trans, diag):
    took_careful = False
    for n, kind, t, b in _cases(uplo, diag, 7 + ord(uplo) * 3 + ord(trans) * 5 + ord(diag)):
        xr, sr, cr = oracle.latrs(t, b, uplo, trans, diag)
        xs, ss, cs = _seq_latrs(seq, t, b, uplo, trans, diag)
        assert np.float64(ss).tobytes() == np.float64(sr).tobytes(), (n, kind, ss, sr)
        assert xs.tobytes() == xr.tobytes(), (n, kind)
        assert cs.tobytes() == cr.tobytes(), (n, kind)
        took_careful |= sr < 1.0
        # NORMIN = 'Y' with the CNORM just returned
        xr2, sr2, _ = oracle.latrs(t, b, uplo, trans, diag, cnorm=cr)
        xs2, ss2, _ = _seq_latrs(seq, t, b, uplo, trans, diag, cnorm=cs)
        assert xs2.tobytes() == xr2.tobytes() and ss2 == sr2 or (np.isnan(ss2) and np.isnan(sr2))
    assert took_careful


@pytest.mark.parametrize("imat", range(1, 12))
def test_dgecon_seq_bitwise_vs_oracle(seq, imat):
    for n in (1, 2, 5, 10, 50, 120):
        if 5 <= imat <= 7 and n < imat - 4:
            continue
        a, izero = oracle.ge_test_matrix(n, n, imat, 31 + 5 * n + imat)
        if izero:
            continue
        lu, ipiv, info = oracle.getrf(a)
        luf = np.asfortranarray(lu)
        for norm, p in (("1", 1), ("I", np.inf)):
            anorm = np.linalg.norm(a, p)
            r_ref, _ = oracle.gecon(lu, anorm, norm)
            work = np.zeros(4 * n)
            iwork = np.zeros(n, dtype=np.int32)
            r_seq = seq.seq_dgecon(int(norm == "1"), n, _ptr(luf), n, anorm, _ptr(work), _ptr(iwork))
            assert np.float64(r_seq).tobytes() == np.float64(r_ref).tobytes(), (n, imat, norm, r_seq, r_ref)


@pytest.mark.parametrize("tiny", [1e-40, 1e-60, 1e-80, 1e-150])
def test_dgecon_seq_tiny_pivots(seq, tiny):
    """Factors whose U has tiny pivots every 7th column: the careful solve
    and the rescaling step run; RCOND (or the early 0) equals the oracle's."""
    n = 40
    rng = np.random.default_rng(int(-np.log10(tiny)))
    lu = rng.standard_normal((n, n))
    d = np.ones(n)
    d[::7] = tiny
    lu[np.diag_indices(n)] = d
    luf = np.asfortranarray(lu)
    for norm in "1I":
        r_ref, _ = oracle.gecon(lu, 3.0, norm)
        work = np.zeros(4 * n)
        iwork = np.zeros(n, dtype=np.int32)
        r_seq = seq.seq_dgecon(int(norm == "1"), n, _ptr(luf), n, 3.0, _ptr(work), _ptr(iwork))
        assert np.float64(r_seq).tobytes() == np.float64(r_ref).tobytes(), (tiny, norm, r_seq, r_ref)


@pytest.mark.parametrize("nb", [1, 3, 20, 64, 200])
def test_dgetri_seq_bitwise_vs_oracle(seq, nb):
    """The DGETRI element steps composed as the GPU driver composes them
    give the oracle's DGETRI bit for bit, blocked and unblocked, over the
    DCHKGE types; the zero-pivot INFO matches."""
    for n in (1, 2, 7, 65, 130):
        for imat in (1, 4, 6, 9):
            if imat == 6 and n < 2:
                continue
            a, izero = oracle.ge_test_matrix(n, n, imat, 11 + n + imat)
            lu, ipiv, info = oracle.getrf(a)
            ref, rinfo, _ = oracle.getri(lu, ipiv, nb=nb)
            got = np.asfortranarray(lu.copy())
            ip = np.ascontiguousarray(ipiv, dtype=np.int32)
            ginfo = seq.seq_dgetri(n, _ptr(got), n, _ptr(ip), nb)
            assert ginfo == rinfo, (n, imat, nb)
            if rinfo == 0:
                assert got.tobytes() == np.asfortranarray(ref).tobytes(), (n, imat, nb)


def test_dgeequ_seq_bitwise_vs_oracle(seq):
    """DGEEQU as the GPU kernels compute it (maxima in another order, the
    finishing steps of latrs_seq.h) equals the oracle's DGEEQU bit for bit:
    R, C, ROWCND, COLCND, AMAX and INFO, on random, badly scaled,
    zero-row, zero-column and extreme-range matrices."""
    rng = np.random.default_rng(4)
    cases = []
    for m, n in ((1, 1), (5, 5), (40, 33), (70, 70)):
        a = rng.standard_normal((m, n))
        cases.append(a)
        cases.append(a * 10.0 ** rng.uniform(-200, 200, (m, 1)) * 10.0 ** rng.uniform(-100, 100, (1, n)))
        if m > 2:
            z = a.copy()
            z[2, :] = 0.0
            cases.append(z)
            z = a.copy()
            z[:, n - 1] = 0.0
            cases.append(z)
    cases.append(np.array([[1e-320, 1.0], [3.0, 1e308]]))
    for a in cases:
        m, n = a.shape
        rr, cr, rowr, colr, amr, infr = oracle.geequ(a)
        af = np.asfortranarray(a)
        r = np.zeros(m)
        c = np.zeros(n)
        sc = np.zeros(3)
        info = seq.seq_dgeequ(m, n, _ptr(af), m, _ptr(r), _ptr(c), _ptr(sc[0:]), _ptr(sc[1:]), _ptr(sc[2:]))
        assert info == infr
        assert r.tobytes() == rr.tobytes() and sc[2] == amr
        if infr == 0:
            assert c.tobytes() == cr.tobytes() and sc[0] == rowr and sc[1] == colr
        elif infr > m:
            assert sc[0] == rowr


@pytest.mark.parametrize("uplo", "LU")
@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_potrf_seq_bitwise_vs_oracle(seq, uplo, dtype):
    """xPOTRF as the GPU driver composes its per-thread steps equals the
    oracle's xPOTRF bit for bit (blocked and unblocked, D and S), INFO
    included for a matrix that is not positive definite."""
    fn = seq.seq_dpotrf if dtype == np.float64 else seq.seq_spotrf
    for n in (1, 2, 7, 33, 70, 130):
        for nb in (1, 3, 20, 64, 200):
            a = oracle.spd_matrix(n, 1e3, 17 + n, uplo, dtype=dtype)
            if n > 4 and nb == 3:
                a[n // 2, n // 2] = -1.0
            ref, rinfo = oracle.potrf(a, uplo, nb=nb)
            got = np.asfortranarray(a.copy())
            ginfo = fn(int(uplo == "U"), n, _ptr(got), n, nb)
            assert ginfo == rinfo, (n, nb)
            assert got.tobytes() == ref.tobytes(), (n, nb)


@pytest.mark.parametrize("uplo", "LU")
def test_lansy_symm_seq_bitwise_vs_oracle(seq, uplo):
    for n in (1, 5, 40, 97):
        a = np.asfortranarray(oracle.spd_matrix(n, 1e2, 3 + n, uplo))
        assert seq.seq_dlansy_i(int(uplo == "U"), n, _ptr(a), n) == oracle.dlansy("I", uplo, a)
        x = np.asfortranarray(oracle.random_matrix(n, 3, 5, idist=3)[0])
        c = np.asfortranarray(oracle.random_matrix(n, 3, 6, idist=3)[0])
        out = np.zeros((n, 3), order="F")
        seq.seq_dsymm_l(int(uplo == "U"), n, 3, -1.0, _ptr(a), n, _ptr(x), n, _ptr(c), n, _ptr(out))
        L = oracle.lib()
        L.or_dsymm_l.argtypes = [ctypes.c_char, ctypes.c_int, ctypes.c_int, ctypes.c_double] + \
            [ctypes.c_void_p, ctypes.c_int] * 3
        ref = c.copy(order="F")
        L.or_dsymm_l(uplo.encode(), n, 3, -1.0, _ptr(a), n, _ptr(x), n, _ptr(ref), n)
        assert out.tobytes() == ref.tobytes()
