"""The complex LU's host/device code checked on the CPU.  The per-thread
steps and the ZGETRF2 / ZGETRF / ZGETRS schedules of
lapack_gb300/csrc/zlu_seq.h (on the GPU: one kernel launch per step, one
thread per column or element) are compiled with g++ over a backend that runs
every step as a loop, then compared bit for bit with the oracle's
restatement of SRC/zgetrf.f, SRC/zgetrf2.f and SRC/zgetrs.f: factors, IPIV,
INFO and solutions, for block sizes 1 (ZGETRF2 alone), 3, 20 and 64, square
and rectangular shapes, zero columns, pivots below the safe minimum (the
division branch of ZGETRF2), signed zeros and infinite entries."""
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
#include <climits>
#include <cstring>
#include <vector>
#include "zlu_seq.h"
using gb::cpx;
using gb::zdc;
using gb::cfc;
// Every step of the schedules as a loop over its threads' work, in any
// order: the GPU threads of one step touch disjoint data.
struct CpuOps {
  int info = INT_MAX, ovf = 0, nc = 0;
  int info_reset() { info = INT_MAX; return 0; }
  int info_read(int *out) { *out = info == INT_MAX ? 0 : info; return 0; }
  template <typename R> int col(int m, cpx<R> *a, int *ipiv, int gcol) {
    if (gb::zgetrf2_col(m, a, ipiv) && gcol < info) info = gcol;
    return 0;
  }
  template <typename R> int laswp(int ncols, cpx<R> *A, int lda, int k1, int k2, const int *ipiv, int incx) {
    for (int j = ncols - 1; j >= 0; --j) gb::zlaswp_col(A + (size_t)j * lda, k1, k2, ipiv, incx);
    return 0;
  }
  template <typename R>
  int trsm(int upper, int trans, int unit, int m, int ncols, const cpx<R> *A, int lda, cpx<R> *B, int ldb) {
    for (int j = ncols - 1; j >= 0; --j) gb::ztrsm_left_col(upper, trans, unit, m, A, lda, B + (size_t)j * ldb);
    return 0;
  }
  template <typename R>
  int gemm(int m, int n, int k, const cpx<R> *A, int lda, const cpx<R> *B, int ldb, cpx<R> *C, int ldc) {
    for (int j = n - 1; j >= 0; --j)
      for (int i = m - 1; i >= 0; --i) gb::zgemm_nn_elem(i, j, k, A, lda, B, ldb, C, ldc);
    return 0;
  }
  int ipiv_add(int *ipiv, int cnt, int off) {
    for (int i = 0; i < cnt; ++i) ipiv[i] += off;
    return 0;
  }
  int lange_inf(int n, const zdc *A, int lda, double *anrm) {
    std::vector<double> rows(n);
    for (int i = n - 1; i >= 0; --i) rows[i] = gb::zlange_row(i, n, A, lda);
    *anrm = gb::zlange_max(n, rows.data());
    return 0;
  }
  int flags_reset() { ovf = nc = 0; return 0; }
  int flags_read(int *o, int *c) { *o = ovf; *c = nc; return 0; }
  int lag2c(int m, int ncols, const zdc *A, int lda, cfc *S, int lds) {
    for (int j = 0; j < ncols; ++j)
      for (int i = 0; i < m; ++i)
        if (!gb::zlag2c_elem(A[(size_t)i + (size_t)j * lda], S + (size_t)i + (size_t)j * lds)) ovf = 1;
    return 0;
  }
  int lag2z(int m, int ncols, const cfc *S, int lds, zdc *X, int ldx, bool add) {
    for (int j = 0; j < ncols; ++j)
      for (int i = 0; i < m; ++i) gb::zlag2z_elem(S[(size_t)i + (size_t)j * lds], X + (size_t)i + (size_t)j * ldx, add);
    return 0;
  }
  int copy(int m, int ncols, const zdc *B, int ldb, zdc *R, int ldr) {
    for (int j = 0; j < ncols; ++j) memcpy(R + (size_t)j * ldr, B + (size_t)j * ldb, sizeof(zdc) * m);
    return 0;
  }
  int check(int n, int nrhs, const zdc *X, int ldx, const zdc *R, int ldr, double cte) {
    for (int j = nrhs - 1; j >= 0; --j)
      if (gb::zcgesv_col_notconv(n, X + (size_t)j * ldx, R + (size_t)j * ldr, cte)) nc = 1;
    return 0;
  }
};
template <typename R> int getrf_t(int m, int n, R *a, int lda, int *ipiv, int nb) {
  CpuOps ops;
  int info = 0;
  gb::zgetrf_full(ops, m, n, reinterpret_cast<cpx<R> *>(a), lda, ipiv, nb, &info);
  return info;
}
template <typename R> void getrs_t(int trans, int n, int nrhs, const R *a, int lda, const int *ipiv, R *b, int ldb) {
  CpuOps ops;
  gb::zgetrs_sched(ops, trans, n, nrhs, reinterpret_cast<const cpx<R> *>(a), lda, ipiv, reinterpret_cast<cpx<R> *>(b),
                   ldb);
}
template <typename R> int izamax_split_t(int n, const R *xr, int nt) {
  // the pivot kernel's IZAMAX: nt thread parts, combined pairwise as its
  // shared-memory tree does (nt a power of two) or in a row
  const cpx<R> *x = reinterpret_cast<const cpx<R> *>(xr);
  std::vector<gb::ZamaxPart<R>> part(nt);
  for (int t = 0; t < nt; ++t) part[t] = gb::zamax_part(n, x, t, nt);
  const bool pow2 = (nt & (nt - 1)) == 0;
  if (pow2)
    for (int h = nt / 2; h > 0; h >>= 1)
      for (int t = 0; t < h; ++t) part[t] = gb::zamax_combine(part[t], part[t + h]);
  else
    for (int t = 1; t < nt; ++t) part[0] = gb::zamax_combine(part[0], part[t]);
  const gb::ZamaxPart<R> all = part[0];
  int sidx = gb::kZamaxNone;
  if (all.nan == gb::kZamaxNone && all.inf == gb::kZamaxNone && all.over != gb::kZamaxNone) {
    R best = R(-1);
    for (int t = nt - 1; t >= 0; --t) {
      R v;
      int i;
      gb::zamax_scaled_part(n, x, all.over, t, nt, &v, &i);
      gb::zamax_pick(best, sidx, v, i);
    }
  }
  return gb::zamax_result(all, sidx);
}
extern "C" {
int seq_zgetrf(int m, int n, double *a, int lda, int *ipiv, int nb) { return getrf_t(m, n, a, lda, ipiv, nb); }
int seq_cgetrf(int m, int n, float *a, int lda, int *ipiv, int nb) { return getrf_t(m, n, a, lda, ipiv, nb); }
void seq_zgetrs(int trans, int n, int nrhs, const double *a, int lda, const int *ipiv, double *b, int ldb) {
  getrs_t(trans, n, nrhs, a, lda, ipiv, b, ldb);
}
void seq_cgetrs(int trans, int n, int nrhs, const float *a, int lda, const int *ipiv, float *b, int ldb) {
  getrs_t(trans, n, nrhs, a, lda, ipiv, b, ldb);
}
int seq_izamax(int n, const double *x) { return gb::izamax_seq(n, reinterpret_cast<const zdc *>(x)); }
int seq_icamax(int n, const float *x) { return gb::izamax_seq(n, reinterpret_cast<const cfc *>(x)); }
int seq_izamax_split(int n, const double *x, int nt) { return izamax_split_t(n, x, nt); }
int seq_icamax_split(int n, const float *x, int nt) { return izamax_split_t(n, x, nt); }
int seq_zcgesv(int n, int nrhs, double *a, int lda, int *ipiv, const double *b, int ldb, double *x, int ldx,
               int *iter) {
  CpuOps ops;
  std::vector<cfc> sa((size_t)n * n + 1), sx((size_t)n * nrhs + 1);
  std::vector<zdc> r((size_t)n * nrhs + 1);
  int info = 0;
  gb::zcgesv_sched(ops, n, nrhs, reinterpret_cast<zdc *>(a), lda, ipiv, reinterpret_cast<const zdc *>(b), ldb,
                   reinterpret_cast<zdc *>(x), ldx, sa.data(), sx.data(), r.data(), iter, &info);
  return info;
}
}
"""


@pytest.fixture(scope="module")
def seq(tmp_path_factory):
    if shutil.which("g++") is None:
        pytest.skip("needs g++")
    d = tmp_path_factory.mktemp("zlu")
    src = d / "zseq.cpp"
    src.write_text(HARNESS)
    so = d / "libzseq.so"
    cmd = ["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fPIC", "-shared", "-I", CSRC, str(src), "-o", str(so)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    L = ctypes.CDLL(str(so))
    p = ctypes.c_void_p
    L.seq_zgetrf.argtypes = [ctypes.c_int, ctypes.c_int, p, ctypes.c_int, p, ctypes.c_int]
    L.seq_zgetrs.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, p, ctypes.c_int, p, p, ctypes.c_int]
    L.seq_izamax.argtypes = [ctypes.c_int, p]
    L.seq_icamax.argtypes = [ctypes.c_int, p]
    L.seq_izamax_split.argtypes = [ctypes.c_int, p, ctypes.c_int]
    L.seq_icamax_split.argtypes = [ctypes.c_int, p, ctypes.c_int]
    L.seq_cgetrf.argtypes = [ctypes.c_int, ctypes.c_int, p, ctypes.c_int, p, ctypes.c_int]
    L.seq_cgetrs.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, p, ctypes.c_int, p, p, ctypes.c_int]
    L.seq_zcgesv.argtypes = [ctypes.c_int, ctypes.c_int, p, ctypes.c_int, p, p, ctypes.c_int, p, ctypes.c_int, p]
    return L


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def _same_bits(x, y):
    """Bitwise equality with every NaN counted equal to every NaN: which NaN
    an operation on two NaN operands returns (its sign and payload) is left
    open by IEEE 754 and depends on the compiler's operand order."""
    x = np.ascontiguousarray(x).view(np.float64)
    y = np.ascontiguousarray(y).view(np.float64)
    nx, ny = np.isnan(x), np.isnan(y)
    return x.shape == y.shape and np.array_equal(nx, ny) and x[~nx].tobytes() == y[~ny].tobytes()


def _seq_getrf(L, a, nb, dtype=np.complex128):
    a = np.asfortranarray(np.array(a, dtype=dtype, copy=True))
    m, n = a.shape
    ipiv = np.zeros(max(1, min(m, n)), dtype=np.int32)
    fn = L.seq_cgetrf if dtype == np.complex64 else L.seq_zgetrf
    info = fn(m, n, _ptr(a), max(1, m), _ptr(ipiv), nb)
    return a, ipiv[: min(m, n)], info


def _seq_getrs(L, lu, ipiv, b, trans):
    dtype = lu.dtype
    b = np.asfortranarray(np.array(b, dtype=dtype, copy=True))
    n, nrhs = b.shape
    fn = L.seq_cgetrs if dtype == np.complex64 else L.seq_zgetrs
    fn("NTC".index(trans), n, nrhs, _ptr(np.asfortranarray(lu)), max(1, n),
       _ptr(np.ascontiguousarray(ipiv, dtype=np.int32)), _ptr(b), max(1, n))
    return b


def _special(kind, m, n, seed):
    a = oracle.random_zmatrix(m, n, seed)
    if kind == "zero_cols":
        a[:, n // 3] = 0
        a[:, (2 * n) // 3] = 0
    elif kind == "tiny":
        a = a * 1e-309            # subnormal pivots, below the safe minimum: ZGETRF2 divides
    elif kind == "signed_zeros":
        z = np.array([0.0, -0.0])
        mask = np.random.default_rng(seed).random((m, n)) < 0.3
        re = np.where(mask, z[np.random.default_rng(seed + 1).integers(0, 2, (m, n))], a.real)
        im = np.where(np.random.default_rng(seed + 2).random((m, n)) < 0.3, -0.0, a.imag)
        a = re + 1j * im
    elif kind == "inf":
        a[m // 2, n // 2] = complex(np.inf, 1.0)
    elif kind == "huge":
        a = a * 1e307             # |re| + |im| overflows: IZAMAX's scaled comparison
    return np.asfortranarray(a)


SHAPES = [(1, 1), (1, 5), (5, 1), (2, 2), (7, 7), (33, 20), (20, 33), (65, 65), (130, 130), (150, 97)]


@pytest.mark.parametrize("nb", [1, 3, 20, 64])
@pytest.mark.parametrize("m,n", SHAPES)
def test_zgetrf_schedule_bitwise(seq, nb, m, n):
    for seed in (1, 2):
        a = oracle.random_zmatrix(m, n, 31 * m + n + seed)
        lu_r, ip_r, info_r = oracle.zgetrf(a, nb=nb)
        lu_g, ip_g, info_g = _seq_getrf(seq, a, nb)
        assert info_g == info_r
        assert np.array_equal(ip_g, ip_r)
        assert lu_g.tobytes() == lu_r.tobytes()


@pytest.mark.parametrize("kind", ["zero_cols", "tiny", "signed_zeros", "inf", "huge"])
@pytest.mark.parametrize("nb", [1, 20, 64])
def test_zgetrf_schedule_edge_cases(seq, kind, nb):
    for m, n in ((40, 40), (90, 70), (130, 130)):
        a = _special(kind, m, n, 7 * m + n)
        lu_r, ip_r, info_r = oracle.zgetrf(a, nb=nb)
        lu_g, ip_g, info_g = _seq_getrf(seq, a, nb)
        assert info_g == info_r, (kind, m, n)
        assert np.array_equal(ip_g, ip_r)
        assert _same_bits(lu_g, lu_r)
        if kind == "zero_cols":
            assert info_r == n // 3 + 1


@pytest.mark.parametrize("trans", "NTC")
@pytest.mark.parametrize("n,nrhs", [(1, 1), (5, 3), (64, 2), (130, 4), (200, 1)])
def test_zgetrs_schedule_bitwise(seq, trans, n, nrhs):
    a = oracle.random_zmatrix(n, n, 100 + n)
    lu, ip, info = oracle.zgetrf(a)
    assert info == 0
    b = oracle.random_zmatrix(n, nrhs, 200 + n)
    x_r, _ = oracle.zgetrs(lu, ip, b, trans)
    x_g = _seq_getrs(seq, lu, ip, b, trans)
    assert x_g.tobytes() == np.asfortranarray(x_r.reshape(n, nrhs)).tobytes()


def test_izamax_seq_matches_oracle(seq):
    rng = np.random.default_rng(5)
    cases = [np.zeros(0), rng.standard_normal(7) + 1j * rng.standard_normal(7),
             np.array([1 + 1j, -2, 2j]), np.array([1, complex(np.nan, 0), 1e300]),
             np.array([1, complex(np.inf, 0), 3, complex(0, np.nan)]), np.array([1, complex(0, -np.inf), 3]),
             np.array([1, complex(1.5e308, 1.5e308), complex(1.5e308, 1.35e308), complex(1.5e308, 1.65e308)])]
    for x in cases:
        x = np.ascontiguousarray(x, dtype=np.complex128)
        assert seq.seq_izamax(x.size, _ptr(x)) == oracle.izamax(x)


def _izamax_cases(rng, big):
    cases = []
    for n in (2, 3, 5, 17, 64, 255, 256, 257, 1000):
        x = rng.standard_normal(n) + 1j * rng.standard_normal(n)
        cases.append(x)
        t = x.copy()
        t[rng.integers(0, n, 3)] = 4 + 4j                    # ties of the maximum
        cases.append(t)
        t = np.round(x)                                     # many exact ties, zeros
        cases.append(t)
        for bad in (complex(np.nan, 0), complex(0, np.inf), complex(-np.inf, np.nan)):
            t = x.copy()
            t[rng.integers(0, n)] = bad
            cases.append(t)
        t = x.copy()
        t[rng.integers(0, n, 2)] = complex(np.inf, 0)
        t[rng.integers(0, n)] = complex(np.nan, 1)           # a NaN before or after the infinities
        cases.append(t)
        t = x * (big / 8)                                   # large finite sums, then some that overflow
        t[rng.integers(0, n, 3)] = complex(0.75 * big, 0.75 * big)
        t[rng.integers(0, n)] = complex(0.8 * big, 0.7 * big)
        cases.append(t)
        t = np.full(n, complex(0.75 * big, 0.75 * big))    # all overflowing and tied
        cases.append(t)
        cases.append(np.zeros(n, dtype=complex))
    return cases


@pytest.mark.parametrize("nt", [1, 2, 3, 7, 32, 256])
def test_izamax_split_equals_sequential(seq, nt):
    """The pivot kernel's IZAMAX, split over nt threads (first NaN, first
    infinity, first overflowing sum and the largest finite sum per thread,
    then the scaled pass), returns izamax_seq's index on ties, NaNs,
    infinities and overflowing sums, in both precisions."""
    rng = np.random.default_rng(nt)
    for x in _izamax_cases(rng, 1.7976931348623157e308):
        x = np.ascontiguousarray(x, dtype=np.complex128)
        assert seq.seq_izamax_split(x.size, _ptr(x), nt) == seq.seq_izamax(x.size, _ptr(x)), x
    for x in _izamax_cases(rng, 3.4028234663852886e38):
        with np.errstate(over="ignore", invalid="ignore"):
            x = np.ascontiguousarray(x, dtype=np.complex64)
        assert seq.seq_icamax_split(x.size, _ptr(x), nt) == seq.seq_icamax(x.size, _ptr(x)), x


@pytest.mark.parametrize("nb", [1, 20, 64])
@pytest.mark.parametrize("m,n", [(1, 1), (7, 7), (33, 20), (20, 33), (130, 130)])
def test_cgetrf_cgetrs_schedule_bitwise(seq, nb, m, n):
    """The COMPLEX twins (CGETRF, CGETRF2, CGETRS) through the same
    templates, against the oracle's single-precision restatement."""
    a = oracle.random_zmatrix(m, n, 5 * m + n).astype(np.complex64)
    lu_r, ip_r, info_r = oracle.zgetrf(a, nb=nb, dtype=np.complex64)
    lu_g, ip_g, info_g = _seq_getrf(seq, a, nb, np.complex64)
    assert info_g == info_r and np.array_equal(ip_g, ip_r)
    assert lu_g.tobytes() == lu_r.tobytes()
    if m == n:
        b = oracle.random_zmatrix(n, 2, 9).astype(np.complex64)
        for trans in "NTC":
            x_r, _ = oracle.zgetrs(lu_r, ip_r, b, trans)
            assert _seq_getrs(seq, lu_r, ip_r, b, trans).tobytes() == np.asfortranarray(x_r).tobytes()


def _seq_zcgesv(L, a, b):
    a = np.asfortranarray(np.array(a, dtype=np.complex128, copy=True))
    b = np.asfortranarray(np.array(b, dtype=np.complex128, copy=True)).reshape(a.shape[0], -1)
    n, nrhs = b.shape
    x = np.zeros((n, nrhs), dtype=np.complex128, order="F")
    ipiv = np.zeros(max(1, n), dtype=np.int32)
    it = np.zeros(1, dtype=np.int32)
    info = L.seq_zcgesv(n, nrhs, _ptr(a), max(1, n), _ptr(ipiv), _ptr(b), max(1, n), _ptr(x), max(1, n), _ptr(it))
    return a, ipiv[:n], x, int(it[0]), info


@pytest.mark.parametrize("kappa", [1e1, 1e4, 1e7, 1e12])
@pytest.mark.parametrize("n,nrhs", [(1, 1), (13, 2), (70, 1), (130, 3)])
def test_zcgesv_schedule_bitwise(seq, kappa, n, nrhs):
    """ZCGESV's schedule (ITER, X, IPIV, and A after a fallback) equal to the
    oracle's, from converged refinement to the ITER = -31 fallback."""
    u, _ = np.linalg.qr(oracle.random_zmatrix(n, n, 1 + n))
    v, _ = np.linalg.qr(oracle.random_zmatrix(n, n, 2 + n))
    a = np.asfortranarray((u * kappa ** (-np.arange(n) / max(n - 1, 1))) @ v.conj().T)
    b = a @ oracle.random_zmatrix(n, nrhs, 3 + n)
    ao_r, ip_r, x_r, it_r, info_r = oracle.zcgesv(a, b)
    ao_g, ip_g, x_g, it_g, info_g = _seq_zcgesv(seq, a, b)
    assert (it_g, info_g) == (it_r, info_r)
    assert np.array_equal(ip_g, ip_r)
    assert x_g.tobytes() == np.asfortranarray(x_r.reshape(n, nrhs)).tobytes()
    assert ao_g.tobytes() == ao_r.tobytes()


def test_zcgesv_schedule_exits(seq):
    """ITER = -2 (B does not fit COMPLEX) and -3 (CGETRF meets a zero pivot
    that ZGETRF does not) as the oracle."""
    n = 30
    a = oracle.random_zmatrix(n, n, 8)
    b = a @ oracle.random_zmatrix(n, 1, 9)
    b[4, 0] = complex(1e39, 0.0)
    for aa, bb in ((a, b), (np.diag([1.0, 1e-50, 1.0]).astype(np.complex128), np.ones((3, 1), np.complex128))):
        ao_r, ip_r, x_r, it_r, info_r = oracle.zcgesv(aa, bb)
        ao_g, ip_g, x_g, it_g, info_g = _seq_zcgesv(seq, aa, bb)
        assert (it_g, info_g) == (it_r, info_r) and it_r in (-2, -3)
        assert x_g.tobytes() == np.asfortranarray(x_r.reshape(x_g.shape)).tobytes()
        assert ao_g.tobytes() == ao_r.tobytes() and np.array_equal(ip_g, ip_r)
