"""DGETRI's GPU source run on the CPU: dgetri_dev (lapack_gb300/csrc/
refine.cu) with the DGETRI kernels of condest_kernels.cuh.

Those kernels are one-dimensional launches whose threads touch disjoint data
(one thread per element of the DTRMM, per row of the DTRSM and of the
column interchanges, one thread for each diagonal block's DTRTI2), so running
blocks and threads one after another computes what the GPU computes.  The
test takes the two pieces out of the sources, rewrites their launches into a
sequential launcher over a stand-in for the CUDA runtime (tests/cuda_emu.py)
and puts the oracle's reference-order DGEMM in place of the library's update
kernel (whose exact mode the GPU LU tests show to be that DGEMM bit for bit).
The inverse, INFO for a singular factor and the workspace-limited block
sizes are compared with the oracle's DGETRI bit for bit."""
import ctypes
import os
import shutil

import numpy as np
import pytest

import cuda_emu
import oracle

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "..", "lapack_gb300", "csrc")
ORACLE_DIR = os.path.join(HERE, "..", "oracle")

PRELUDE = r"""
#include <algorithm>
#include "getri_seq.h"
extern "C" void or_dgemm(char ta, char tb, int m, int n, int k, double alpha, const double *a, int lda,
                         const double *b, int ldb, double beta, double *c, int ldc);
namespace gb {
unsigned blocks256(size_t n) { return (unsigned)((n + 255) / 256); }
// the library's update C -= A*B, as the reference DGEMM('N','N', alpha = -1, beta = 1)
template <typename T>
int gemm_update_dev(int m, int n, int k, const T* A, int lda, const T* B, int ldb, T* C, int ldc, cudaStream_t, int) {
  if (m > 0 && n > 0 && k > 0) or_dgemm('N', 'N', m, n, k, -1.0, A, lda, B, ldb, 1.0, C, ldc);
  return 0;
}
"""

ENTRY = r"""
}  // namespace gb
extern "C" int emu_dgetri(int n, double* a, int lda, const int* ipiv, int nb_trtri, int nb) {
  int info = 0;
  gb::dgetri_dev(n, a, lda, ipiv, nb_trtri, nb, &info, nullptr);
  return info;
}
"""


def _slice(text, start, end):
    i = text.index(start)
    j = text.index(end, i)
    return text[i:j]


@pytest.fixture(scope="module")
def emu(tmp_path_factory):
    if shutil.which("g++") is None:
        pytest.skip("needs g++")
    kern = open(os.path.join(CSRC, "condest_kernels.cuh")).read()
    kern = _slice(kern, "// ------------------------------------------------------------- DGETRI", "}  // namespace gb")
    drv = open(os.path.join(CSRC, "refine.cu")).read()
    drv = _slice(drv, "int dgetri_dev(int n, double* A, int lda, const int* ipiv, int nb_trtri, int nb, int* info,",
                 "\n}  // namespace gb") + "\n"
    src = cuda_emu.translate(PRELUDE + kern + drv + ENTRY, drop_includes=(), min_launches=7)
    oracle.lib()
    so = cuda_emu.build(str(tmp_path_factory.mktemp("getriemu")), "getriemu", src, [CSRC])
    ctypes.CDLL(os.path.join(ORACLE_DIR, "liboracle.so"), mode=ctypes.RTLD_GLOBAL)
    L = ctypes.CDLL(so)
    L.emu_dgetri.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_int,
                             ctypes.c_int]
    return L


@pytest.mark.parametrize("nb", [1, 3, 20, 64, 512])
@pytest.mark.parametrize("n,imat", [(1, 1), (2, 2), (7, 3), (65, 4), (130, 1), (200, 9), (200, 6)])
def test_getri_cu_bitwise(emu, nb, n, imat):
    a, izero = oracle.ge_test_matrix(n, n, imat, 23 + n + imat)
    lu, ipiv, info = oracle.getrf(a)
    ref, rinfo, _ = oracle.getri(lu, ipiv, nb=nb)
    got = np.asfortranarray(lu.copy())
    ginfo = emu.emu_dgetri(n, got.ctypes.data_as(ctypes.c_void_p), n,
                           np.ascontiguousarray(ipiv, dtype=np.int32).ctypes.data_as(ctypes.c_void_p), nb, nb)
    assert ginfo == rinfo
    if rinfo == 0:
        assert got.tobytes(order="F") == np.asfortranarray(ref).tobytes(order="F")
    else:
        assert got.tobytes(order="F") == np.asfortranarray(lu).tobytes(order="F")   # untouched, as DTRTRI returns


@pytest.mark.parametrize("n,lwork_cols", [(200, 5), (200, 1), (130, 2), (300, 63)])
def test_getri_cu_short_workspace_bitwise(emu, n, lwork_cols):
    """A workspace shorter than N*NB: DTRTRI keeps its block size of 64
    (SRC/dtrtri.f:180) while the inv(A)*L loop runs with LWORK/N columns
    (SRC/dgetri.f:184-190), or unblocked below NBMIN = 2."""
    a, _ = oracle.ge_test_matrix(n, n, 1, 41 + n)
    lu, ipiv, _ = oracle.getrf(a)
    ref, rinfo, _ = oracle.getri(lu, ipiv, nb=64, lwork=n * lwork_cols)
    assert rinfo == 0
    nb_loop = lwork_cols if lwork_cols >= 2 else 1
    got = np.asfortranarray(lu.copy())
    emu.emu_dgetri(n, got.ctypes.data_as(ctypes.c_void_p), n,
                   np.ascontiguousarray(ipiv, dtype=np.int32).ctypes.data_as(ctypes.c_void_p), 64, nb_loop)
    assert got.tobytes(order="F") == np.asfortranarray(ref).tobytes(order="F")
