"""The complex LU's GPU source (lapack_gb300/csrc/zlu.cu) run on the CPU.

Every kernel in zlu.cu is a one-dimensional launch whose threads touch
disjoint data (no barriers, the one shared word updated by atomicMin or by
identical stores; the small-triangle ZTRSM stages through shared memory on
the GPU only and runs its direct form here), so running its blocks and
threads one after another computes what the GPU computes.  The test rewrites each
`kernel<<<grid, block, smem, stream>>>(args)` of the file into a call of a
sequential launcher, compiles the file with g++ over a small stand-in for
the CUDA runtime calls it makes (copies, memsets, synchronisation, stream-
ordered scratch as host memory), and compares ZGETRF / CGETRF, ZGETRS and
ZCGESV, driven through the file's own zgetrf_dev / zgetrs_dev / zcgesv_dev,
with the oracle bit for bit.  This checks the kernels' index arithmetic,
launch geometry and the backend that drives the shared schedules."""
import ctypes
import os
import shutil

import numpy as np
import pytest

import cuda_emu
import oracle

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "..", "lapack_gb300", "csrc")

# The tiled ZGEMM, the CTA triangular solve and the CTA pivot step
# (zlu_tiles.cu) cooperate through
# shared memory and run on the GB300 only; here they are their reference-
# order equivalents, the per-element functions the tiles compute (the split
# IZAMAX is checked against izamax_seq in test_zlu_seq.py).
STANDIN = r"""
namespace gb {
template <typename R>
int zgemm_tile_dev(int m, int n, int k, const cpx<R>* A, int lda, const cpx<R>* B, int ldb, cpx<R>* C, int ldc,
                   cudaStream_t) {
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < m; ++i) zgemm_nn_elem(i, j, k, A, lda, B, ldb, C, ldc);
  return 0;
}
template <typename R>
bool ztrsm_cta_dev(int upper, int trans, int unit, int m, int ncols, const cpx<R>* A, int lda, cpx<R>* B, int ldb,
                   cudaStream_t, int* rc) {
  *rc = 0;
  if (trans != 0 && !upper) return false;
  for (int j = 0; j < ncols; ++j) ztrsm_left_col(upper, trans, unit, m, A, lda, B + (size_t)j * ldb);
  return true;
}
template <typename R>
int zcol_cta_dev(int m, cpx<R>* a, int* ipiv, int gcol, int* info, cudaStream_t) {
  if (zgetrf2_col(m, a, ipiv)) atomicMin(info, gcol);
  return 0;
}
}  // namespace gb
"""

ENTRY = r"""
extern "C" {
int emu_zgetrf(int m, int n, double* a, int lda, int* ipiv, int nb) {
  int info = 0;
  gb::zgetrf_dev<double>(m, n, reinterpret_cast<gb::zdc*>(a), lda, ipiv, nb, &info, nullptr);
  return info;
}
int emu_cgetrf(int m, int n, float* a, int lda, int* ipiv, int nb) {
  int info = 0;
  gb::zgetrf_dev<float>(m, n, reinterpret_cast<gb::cfc*>(a), lda, ipiv, nb, &info, nullptr);
  return info;
}
int emu_zgetrs(int trans, int n, int nrhs, const double* a, int lda, const int* ipiv, double* b, int ldb) {
  return gb::zgetrs_dev<double>(trans, n, nrhs, reinterpret_cast<const gb::zdc*>(a), lda, ipiv,
                                reinterpret_cast<gb::zdc*>(b), ldb, nullptr);
}
int emu_zcgesv(int n, int nrhs, double* a, int lda, int* ipiv, const double* b, int ldb, double* x, int ldx,
               int* iter) {
  int info = 0;
  gb::zcgesv_dev(n, nrhs, reinterpret_cast<gb::zdc*>(a), lda, ipiv, reinterpret_cast<const gb::zdc*>(b), ldb,
                 reinterpret_cast<gb::zdc*>(x), ldx, iter, &info, nullptr);
  return info;
}
}
"""


@pytest.fixture(scope="module")
def emu(tmp_path_factory):
    if shutil.which("g++") is None:
        pytest.skip("needs g++")
    d = str(tmp_path_factory.mktemp("zluemu"))
    src = cuda_emu.translate(open(os.path.join(CSRC, "zlu.cu")).read(), min_launches=8)
    so = cuda_emu.build(d, "zluemu", src + STANDIN + ENTRY, [CSRC])
    L = ctypes.CDLL(so)
    p, i = ctypes.c_void_p, ctypes.c_int
    L.emu_zgetrf.argtypes = [i, i, p, i, p, i]
    L.emu_cgetrf.argtypes = [i, i, p, i, p, i]
    L.emu_zgetrs.argtypes = [i, i, i, p, i, p, p, i]
    L.emu_zcgesv.argtypes = [i, i, p, i, p, p, i, p, i, p]
    return L


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def _same_bits(x, y):
    x = np.asfortranarray(x).ravel(order="F").view(np.float32 if x.dtype == np.complex64 else np.float64)
    y = np.asfortranarray(y).ravel(order="F").view(np.float32 if y.dtype == np.complex64 else np.float64)
    nx, ny = np.isnan(x), np.isnan(y)
    return x.shape == y.shape and np.array_equal(nx, ny) and x[~nx].tobytes() == y[~ny].tobytes()


@pytest.mark.parametrize("dtype", [np.complex128, np.complex64])
@pytest.mark.parametrize("m,n,nb", [(1, 1, 64), (5, 1, 64), (1, 5, 64), (40, 40, 64), (130, 97, 64), (97, 130, 64),
                                    (70, 70, 1), (70, 70, 20)])
def test_zlu_cu_getrf_bitwise(emu, dtype, m, n, nb):
    a = oracle.random_zmatrix(m, n, 7 * m + n).astype(dtype)
    if m >= 40:
        a[:, n // 3] = 0                  # a zero column: INFO, the factorization completed
    lu_r, ip_r, info_r = oracle.zgetrf(a, nb=nb, dtype=dtype)
    lu = np.asfortranarray(a.copy())
    ip = np.zeros(max(1, min(m, n)), dtype=np.int32)
    fn = emu.emu_cgetrf if dtype == np.complex64 else emu.emu_zgetrf
    info = fn(m, n, _ptr(lu), max(1, m), _ptr(ip), nb)
    assert info == info_r and np.array_equal(ip[: min(m, n)], ip_r)
    assert _same_bits(lu, lu_r)


@pytest.mark.parametrize("trans", "NTC")
def test_zlu_cu_getrs_bitwise(emu, trans):
    n, nrhs = 90, 3
    a = oracle.random_zmatrix(n, n, 3)
    lu, ip, _ = oracle.zgetrf(a)
    b = oracle.random_zmatrix(n, nrhs, 4)
    x_r, _ = oracle.zgetrs(lu, ip, b, trans)
    x = np.asfortranarray(b.copy())
    assert emu.emu_zgetrs("NTC".index(trans), n, nrhs, _ptr(np.asfortranarray(lu)), n, _ptr(ip), _ptr(x), n) == 0
    assert _same_bits(x, x_r)


@pytest.mark.parametrize("kappa", [1e2, 1e6, 1e12])
def test_zlu_cu_zcgesv_bitwise(emu, kappa):
    n, nrhs = 60, 2
    u, _ = np.linalg.qr(oracle.random_zmatrix(n, n, 1))
    v, _ = np.linalg.qr(oracle.random_zmatrix(n, n, 2))
    a = np.asfortranarray((u * kappa ** (-np.arange(n) / (n - 1))) @ v.conj().T)
    b = np.asfortranarray(a @ oracle.random_zmatrix(n, nrhs, 3))
    ao_r, ip_r, x_r, it_r, info_r = oracle.zcgesv(a, b)
    ao = np.asfortranarray(a.copy())
    x = np.zeros((n, nrhs), dtype=np.complex128, order="F")
    ip = np.zeros(n, dtype=np.int32)
    it = np.zeros(1, dtype=np.int32)
    info = emu.emu_zcgesv(n, nrhs, _ptr(ao), n, _ptr(ip), _ptr(b), n, _ptr(x), n, _ptr(it))
    assert (int(it[0]), info) == (it_r, info_r)
    assert np.array_equal(ip, ip_r) and _same_bits(x, x_r) and _same_bits(ao, ao_r)
