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
#include "zlu_seq.h"
using gb::zdc;
// Every step of the schedules as a loop over its threads' work, in any
// order: the GPU threads of one step touch disjoint data.
struct CpuOps {
  int info = INT_MAX;
  int col(int m, zdc *a, int *ipiv, int gcol) {
    if (gb::zgetrf2_col(m, a, ipiv) && gcol < info) info = gcol;
    return 0;
  }
  int laswp(int ncols, zdc *A, int lda, int k1, int k2, const int *ipiv, int incx) {
    for (int j = ncols - 1; j >= 0; --j) gb::zlaswp_col(A + (size_t)j * lda, k1, k2, ipiv, incx);
    return 0;
  }
  int trsm(int upper, int trans, int unit, int m, int ncols, const zdc *A, int lda, zdc *B, int ldb) {
    for (int j = ncols - 1; j >= 0; --j) gb::ztrsm_left_col(upper, trans, unit, m, A, lda, B + (size_t)j * ldb);
    return 0;
  }
  int gemm(int m, int n, int k, const zdc *A, int lda, const zdc *B, int ldb, zdc *C, int ldc) {
    for (int j = n - 1; j >= 0; --j)
      for (int i = m - 1; i >= 0; --i) gb::zgemm_nn_elem(i, j, k, A, lda, B, ldb, C, ldc);
    return 0;
  }
  int ipiv_add(int *ipiv, int cnt, int off) {
    for (int i = 0; i < cnt; ++i) ipiv[i] += off;
    return 0;
  }
};
extern "C" {
int seq_zgetrf(int m, int n, double *a, int lda, int *ipiv, int nb) {
  CpuOps ops;
  gb::zgetrf_sched(ops, m, n, reinterpret_cast<zdc *>(a), lda, ipiv, nb);
  return ops.info == INT_MAX ? 0 : ops.info;
}
void seq_zgetrs(int trans, int n, int nrhs, const double *a, int lda, const int *ipiv, double *b, int ldb) {
  CpuOps ops;
  gb::zgetrs_sched(ops, trans, n, nrhs, reinterpret_cast<const zdc *>(a), lda, ipiv, reinterpret_cast<zdc *>(b), ldb);
}
int seq_izamax(int n, const double *x) { return gb::izamax_seq(n, reinterpret_cast<const zdc *>(x)); }
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


def _seq_getrf(L, a, nb):
    a = np.asfortranarray(np.array(a, dtype=np.complex128, copy=True))
    m, n = a.shape
    ipiv = np.zeros(max(1, min(m, n)), dtype=np.int32)
    info = L.seq_zgetrf(m, n, _ptr(a), max(1, m), _ptr(ipiv), nb)
    return a, ipiv[: min(m, n)], info


def _seq_getrs(L, lu, ipiv, b, trans):
    b = np.asfortranarray(np.array(b, dtype=np.complex128, copy=True))
    n, nrhs = b.shape
    L.seq_zgetrs("NTC".index(trans), n, nrhs, _ptr(np.asfortranarray(lu)), max(1, n),
                 _ptr(np.ascontiguousarray(ipiv, dtype=np.int32)), _ptr(b), max(1, n))
    return b


def _special(kind, m, n, seed):
    a = oracle.random_zmatrix(m, n, seed)
    if kind == "zero_cols":
        a[:, n // 3] = 0
        a[:, (2 * n) // 3] = 0
    elif kind == "tiny":
        a = a * 1e-306            # pivots below the safe minimum: ZGETRF2 divides
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
