"""The Cholesky factorization's GPU source (potrf_dev and its kernels in
lapack_gb300/csrc/chol.cu) run on the CPU.

Its kernels are one-dimensional launches whose threads touch disjoint data
(one thread per element of a DSYRK or DGEMM update, per row or column of a
DTRSM, one thread for each diagonal block's DPOTRF2), so running blocks and
threads one after another computes what the GPU computes.  The test takes
chol.cu up to the factorization (the solves use the library's blocked
triangular-solve kernels, which cooperate through shared memory and are not
run here), rewrites its launches into a sequential launcher over a stand-in
for the CUDA runtime, and compares DPOTRF / SPOTRF for both triangles,
blocked and unblocked, and INFO for a matrix that is not positive definite,
with the oracle bit for bit."""
import ctypes
import os
import shutil

import numpy as np
import pytest

import cuda_emu
import oracle

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "..", "lapack_gb300", "csrc")

ENTRY = r"""
extern "C" {
int emu_dpotrf(int upper, int n, double* a, int lda, int nb) {
  int info = 0;
  gb::potrf_dev<double>(upper != 0, n, a, lda, nb, &info, nullptr);
  return info;
}
int emu_spotrf(int upper, int n, float* a, int lda, int nb) {
  int info = 0;
  gb::potrf_dev<float>(upper != 0, n, a, lda, nb, &info, nullptr);
  return info;
}
}
"""


@pytest.fixture(scope="module")
def emu(tmp_path_factory):
    if shutil.which("g++") is None:
        pytest.skip("needs g++")
    src = open(os.path.join(CSRC, "chol.cu")).read()
    cut = src.index("template <typename T>\nint potrs_dev(")
    src = src[:cut] + "}  // namespace gb\n"
    src = cuda_emu.translate(src, drop_includes=("driver.h", "prof.h", "solve_kernels.cuh"), min_launches=5)
    so = cuda_emu.build(str(tmp_path_factory.mktemp("cholemu")), "cholemu", src + ENTRY, [CSRC])
    L = ctypes.CDLL(so)
    i, p = ctypes.c_int, ctypes.c_void_p
    L.emu_dpotrf.argtypes = [i, i, p, i, i]
    L.emu_spotrf.argtypes = [i, i, p, i, i]
    return L


@pytest.mark.parametrize("uplo", "LU")
@pytest.mark.parametrize("dtype", [np.float64, np.float32])
@pytest.mark.parametrize("n,nb", [(1, 64), (7, 64), (64, 64), (65, 64), (130, 64), (200, 64), (150, 20), (90, 1)])
def test_chol_cu_potrf_bitwise(emu, uplo, dtype, n, nb):
    a = oracle.spd_matrix(n, 1e3, 13 + n, uplo, dtype=dtype)
    ref, rinfo = oracle.potrf(a, uplo, nb=nb)
    got = np.asfortranarray(np.array(a, dtype=dtype, copy=True))
    fn = emu.emu_dpotrf if dtype == np.float64 else emu.emu_spotrf
    info = fn(int(uplo == "U"), n, got.ctypes.data_as(ctypes.c_void_p), max(1, n), nb)
    assert info == rinfo == 0
    assert got.tobytes(order="F") == np.asfortranarray(ref).tobytes(order="F")


@pytest.mark.parametrize("uplo", "LU")
def test_chol_cu_potrf_not_positive_definite(emu, uplo):
    n = 150
    a = oracle.spd_matrix(n, 1e2, 5, uplo)
    a[100, 100] = -1.0
    ref, rinfo = oracle.potrf(a, uplo, nb=64)
    got = np.asfortranarray(a.copy())
    info = emu.emu_dpotrf(int(uplo == "U"), n, got.ctypes.data_as(ctypes.c_void_p), n, 64)
    assert rinfo > 0 and info == rinfo
    assert got.tobytes(order="F") == np.asfortranarray(ref).tobytes(order="F")
