"""The Cholesky factorization's GPU source (potrf_dev and its kernels in
lapack_gb300/csrc/chol.cu) run on the CPU.

Its kernels are one-dimensional launches whose threads touch disjoint data
(one thread per element of a DSYRK update or of an operand transpose, per
row or column of a DTRSM, one thread for each diagonal block's DPOTRF2), so
running blocks and threads one after another computes what the GPU
computes; the DGEMM update, on the tiled update kernel, is a stand-in in the
same order.  The test takes
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


# The DGEMM and DSYRK updates of chol.cu run on the library's tiled update
# kernel (it cooperates through shared memory and is not run here; the GB300
# tests check its bits against the oracle); these stand-ins compute them in
# the same per-element orders with separately rounded products (DSYRK's zero
# skip and triangle included), so what is checked
# here is chol.cu's own part: the operand transposes, offsets and the
# sequence of steps.
GEMM_STANDIN = r"""
namespace gb {
template <typename T>
int gemm_ordered_dev(bool sum_first, int M, int N, int K, const T* A, int lda, const T* B, int ldb, T* C, int ldc,
                   cudaStream_t) {
  for (int j = 0; j < N; ++j)
    for (int i = 0; i < M; ++i) {
      T* c = C + i + (size_t)j * ldc;
      if (!sum_first) {
        T acc = *c;
        for (int l = 0; l < K; ++l) acc = acc - A[i + (size_t)l * lda] * B[l + (size_t)j * ldb];
        *c = acc;
      } else {
        T t = 0;
        for (int l = 0; l < K; ++l) t = t + A[i + (size_t)l * lda] * B[l + (size_t)j * ldb];
        *c = *c - t;
      }
    }
  return 0;
}
template <typename T>
int syrk_ordered_dev(bool upper, int n, int K, const T* A, int lda, const T* B, int ldb, T* C, int ldc, cudaStream_t) {
  for (int j = 0; j < n; ++j)
    for (int i = upper ? 0 : j; i < (upper ? j + 1 : n); ++i) {
      T* c = C + i + (size_t)j * ldc;
      if (!upper) {
        T acc = *c;
        for (int l = 0; l < K; ++l)
          if (B[l + (size_t)j * ldb] != T(0)) acc = acc - A[i + (size_t)l * lda] * B[l + (size_t)j * ldb];
        *c = acc;
      } else {
        T t = 0;
        for (int l = 0; l < K; ++l) t = t + A[i + (size_t)l * lda] * B[l + (size_t)j * ldb];
        *c = *c - t;
      }
    }
  return 0;
}
}  // namespace gb
"""


@pytest.fixture(scope="module")
def emu(tmp_path_factory):
    if shutil.which("g++") is None:
        pytest.skip("needs g++")
    src = open(os.path.join(CSRC, "chol.cu")).read()
    cut = src.index("template <typename T>\nint potrs_dev(")
    src = GEMM_STANDIN + src[:cut] + "}  // namespace gb\n"
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


# DSPOSV (dsposv_dev) through the same stand-in.  The kernels it borrows from
# the solve path cooperate within a CTA (the triangular solves, the
# NaN-propagating maximum, the convergence test) and are replaced here by
# their reference-order equivalents; they run on the GB300 in the DSGESV
# tests.  What is checked is chol.cu's own part: the DSPOSV sequence, its
# flags, the DLANSY rows, DLAT2S, the DSYMM-order residual and the fallback.
SOLVE_STANDINS = r"""
#include <cmath>
extern "C" void or_dtrsm_left(char, char, char, int, int, double, const double*, int, double*, int);
extern "C" void or_strsm_left(char, char, char, int, int, float, const float*, int, float*, int);
namespace gb {
enum { kProfResidual = 0 };
inline void prof_begin(int, cudaStream_t) {}
inline void prof_end(int, cudaStream_t, double, double) {}
template <typename T>
int trsm_left_dev(bool upper, bool trans, bool unit, int n, int nrhs, const T* A, int lda, T* B, int ldb, cudaStream_t);
template <>
int trsm_left_dev<double>(bool upper, bool trans, bool unit, int n, int nrhs, const double* A, int lda, double* B,
                          int ldb, cudaStream_t) {
  if (n > 0 && nrhs > 0) or_dtrsm_left(upper ? 'U' : 'L', trans ? 'T' : 'N', unit ? 'U' : 'N', n, nrhs, 1.0, A, lda, B, ldb);
  return 0;
}
template <>
int trsm_left_dev<float>(bool upper, bool trans, bool unit, int n, int nrhs, const float* A, int lda, float* B, int ldb,
                         cudaStream_t) {
  if (n > 0 && nrhs > 0) or_strsm_left(upper ? 'U' : 'L', trans ? 'T' : 'N', unit ? 'U' : 'N', n, nrhs, 1.0f, A, lda, B, ldb);
  return 0;
}
template <typename T>
__global__ void max_nan_kernel(const T* x, int m, T* out) {
  if (blockIdx.x || threadIdx.x) return;
  T v = 0;
  bool nan = false;
  for (int i = 0; i < m; ++i) {
    if (x[i] != x[i]) nan = true;
    else if (x[i] > v) v = x[i];
  }
  *out = nan ? T(NAN) : v;
}
__global__ void dlag2s_kernel(const double* A, int lda, float* S, int lds, int m, int n, int* overflow) {
  const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (size_t)m * n) return;
  const int c = (int)(e / m), r = (int)(e - (size_t)c * m);
  const double v = A[(size_t)r + (size_t)c * lda];
  if (v < -3.4028234663852886e38 || v > 3.4028234663852886e38) *overflow = 1;
  S[(size_t)r + (size_t)c * lds] = (float)v;
}
__global__ void slag2d_kernel(const float* S, int lds, double* A, int lda, int m, int n) {
  const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (size_t)m * n) return;
  const int c = (int)(e / m), r = (int)(e - (size_t)c * m);
  A[(size_t)r + (size_t)c * lda] = (double)S[(size_t)r + (size_t)c * lds];
}
__global__ void lag2d_axpy_kernel(const float* S, int lds, double* X, int ldx, int n, int nrhs) {
  const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (size_t)n * nrhs) return;
  const int c = (int)(e / n), r = (int)(e - (size_t)c * n);
  X[(size_t)r + (size_t)c * ldx] = X[(size_t)r + (size_t)c * ldx] + (double)S[(size_t)r + (size_t)c * lds];
}
template <typename T>
__global__ void copy_cols_kernel(const T* S, int lds, T* D, int ldd, int m, int ncols) {
  const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (size_t)m * ncols) return;
  const int c = (int)(e / m), r = (int)(e - (size_t)c * m);
  D[(size_t)r + (size_t)c * ldd] = S[(size_t)r + (size_t)c * lds];
}
// SRC/dsgesv.f:337-342 / dsposv.f: IDAMAX of X and R, RNRM > XNRM*CTE
__global__ void ir_check_kernel(const double* X, int ldx, const double* R, int ldr, int n, const double* anrm,
                                int* notconv, double*) {
  if (threadIdx.x) return;
  const int j = blockIdx.x;
  int ix = 0, ir = 0;
  for (int i = 1; i < n; ++i) {
    if (fabs(X[(size_t)i + (size_t)j * ldx]) > fabs(X[(size_t)ix + (size_t)j * ldx])) ix = i;
    if (fabs(R[(size_t)i + (size_t)j * ldr]) > fabs(R[(size_t)ir + (size_t)j * ldr])) ir = i;
  }
  const double cte = (*anrm) * 1.1102230246251565e-16 * sqrt((double)n) * 1.0;
  if (fabs(R[(size_t)ir + (size_t)j * ldr]) > fabs(X[(size_t)ix + (size_t)j * ldx]) * cte) *notconv += 1;
}
}  // namespace gb
"""

SPOSV_ENTRY = r"""
extern "C" int emu_dsposv(int upper, int n, int nrhs, double* a, int lda, const double* b, int ldb, double* x, int ldx,
                          int* iter) {
  int info = 0;
  gb::dsposv_dev(upper != 0, n, nrhs, a, lda, b, ldb, x, ldx, iter, &info, nullptr);
  return info;
}
"""


@pytest.fixture(scope="module")
def emu_sposv(tmp_path_factory):
    if shutil.which("g++") is None:
        pytest.skip("needs g++")
    src = open(os.path.join(CSRC, "chol.cu")).read()
    src = GEMM_STANDIN + SOLVE_STANDINS + src
    src = cuda_emu.translate(src, drop_includes=("driver.h", "prof.h", "solve_kernels.cuh"), min_launches=10)
    oracle.lib()
    so = cuda_emu.build(str(tmp_path_factory.mktemp("sposvemu")), "sposvemu", src + SPOSV_ENTRY, [CSRC])
    ctypes.CDLL(os.path.join(HERE, "..", "oracle", "liboracle.so"), mode=ctypes.RTLD_GLOBAL)
    L = ctypes.CDLL(so)
    i, p = ctypes.c_int, ctypes.c_void_p
    L.emu_dsposv.argtypes = [i, i, i, p, i, p, i, p, i, p]
    return L


@pytest.mark.parametrize("uplo", "LU")
@pytest.mark.parametrize("n,cond", [(1, 2.0), (13, 1e3), (45, 1e3), (132, 1e5), (60, 1e10), (101, 1e12)])
def test_chol_cu_dsposv_matches_oracle(emu_sposv, uplo, n, cond):
    """ITER, INFO, X and (after the FP64 fallback) A equal to the oracle's
    DSPOSV, from converged refinement to ITER = -3 / -31."""
    a = oracle.spd_matrix(n, cond, 7 + n, uplo)
    from oracle import checks as ck
    b = np.asfortranarray(ck._sym_full(a, uplo) @ oracle.random_matrix(n, 2, 8 + n, idist=2)[0])
    ao_r, x_r, it_r, info_r = oracle.dsposv(a, b, uplo)
    ao = np.asfortranarray(a.copy())
    x = np.zeros((n, 2), order="F")
    it = np.zeros(1, dtype=np.int32)
    p = lambda v: v.ctypes.data_as(ctypes.c_void_p)
    info = emu_sposv.emu_dsposv(int(uplo == "U"), n, 2, p(ao), n, p(b), n, p(x), n, p(it))
    assert (int(it[0]), info) == (it_r, info_r)
    assert x.tobytes(order="F") == np.asfortranarray(x_r).tobytes(order="F")
    assert ao.tobytes(order="F") == np.asfortranarray(ao_r).tobytes(order="F")
