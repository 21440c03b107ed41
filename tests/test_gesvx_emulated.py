"""DGESVX's GPU driver (dgesvx_dev in lapack_gb300/csrc/refine.cu) with the
equilibration kernels of condest_kernels.cuh, run on the CPU.

dgesvx_dev composes the GPU DGETRF, DGETRS, DGECON and DGERFS (whose kernels
cooperate within CTAs and run on the GB300 in their own tests, bitwise equal
to the oracle in exact mode) with its own one-dimensional kernels: DGEEQU's
row maxima and finishing steps, DLAQGE and the right-hand-side scalings, the
pivot-growth maxima, the FERR division.  The test takes dgesvx_dev and those
kernels out of the sources, runs their launches sequentially over a stand-in
for the CUDA runtime (tests/cuda_emu.py), puts the oracle's restatements in
place of the composed routines (and of the one-warp-per-column DGEEQU column
maxima, an order-free maximum), and compares every DGESVX output (A, AF,
IPIV, EQUED, R, C, B, X, RCOND, FERR, BERR, the pivot growth, INFO) with the
oracle's DGESVX bit for bit."""
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
#include <cmath>
#include <cstring>
#include <vector>
#include "latrs_seq.h"
static inline double __dmul_rn(double a, double b) { return a * b; }
static inline double __ddiv_rn(double a, double b) { return a / b; }
static inline long long __double_as_longlong(double v) { long long b; memcpy(&b, &v, 8); return b; }
static inline double __shfl_xor_sync(unsigned, double v, int) { return v; }   // compiles the unused warp kernel
extern "C" {
void or_dgetrf_nb(int, int, double*, int, int*, int*, int);
void or_dgetrs(char, int, int, const double*, int, const int*, double*, int, int*);
void or_dgerfs(char, int, int, const double*, int, const double*, int, const int*, const double*, int, double*, int,
               double*, double*, double*, int*, int*);
void or_dgecon(char, int, const double*, int, double, double*, double*, int*, int*);
double or_dlange(char, int, int, const double*, int, double*);
}
namespace gb {
unsigned blocks256(size_t n) { return (unsigned)((n + 255) / 256); }
struct Options { int nb_f64 = 64; int exact = 1; };
inline const Options& options() { static Options o; return o; }
// the composed routines, as the oracle computes them
template <typename T>
int getrf_dev(int m, int n, T* A, int lda, int* ipiv, int* dinfo, cudaStream_t, int, int nb) {
  or_dgetrf_nb(m, n, A, lda, ipiv, dinfo, nb);
  return 0;
}
template <typename T>
int getrs_dev(char trans, int n, int nrhs, const T* A, int lda, const int* ipiv, const int*, T* B, int ldb,
              cudaStream_t) {
  int info = 0;
  or_dgetrs(trans, n, nrhs, A, lda, ipiv, B, ldb, &info);
  return 0;
}
int dgerfs_dev(char trans, int n, int nrhs, const double* A, int lda, const double* AF, int ldaf, const int* ipiv,
               const double* B, int ldb, double* X, int ldx, double* ferr, double* berr, cudaStream_t) {
  std::vector<double> w(3 * (size_t)std::max(n, 1));
  std::vector<int> iw(std::max(n, 1));
  int info = 0;
  or_dgerfs(trans, n, nrhs, A, lda, AF, ldaf, ipiv, B, ldb, X, ldx, ferr, berr, w.data(), iw.data(), &info);
  return 0;
}
int dgecon_dev(char norm, int n, const double* LU, int lda, double anorm, double* rcond, int* info, cudaStream_t) {
  std::vector<double> w(4 * (size_t)std::max(n, 1));
  std::vector<int> iw(std::max(n, 1));
  or_dgecon(norm, n, LU, lda, anorm, rcond, w.data(), iw.data(), info);
  return 0;
}
int dlange_dev(int which, int m, int n, const double* A, int lda, double* out, cudaStream_t) {
  std::vector<double> w(std::max(m, 1));
  *out = or_dlange(which == 1 ? '1' : 'I', m, n, A, lda, w.data());
  return 0;
}
"""

COLMAX = r"""
// DGEEQU column maxima, one warp per column on the GPU (a maximum, so the
// order does not matter): here lane 0 of each warp takes its column.
__global__ void geequ_colmax_kernel(const double* A, int lda, int m, int n, const double* r, double* c) {
  const int j = blockIdx.x * 8 + (threadIdx.x >> 5), lane = threadIdx.x & 31;
  if (j >= n || lane) return;
  double v = 0.0;
  for (int i = 0; i < m; ++i) v = fmax(v, fabs(A[(size_t)i + (size_t)j * lda]) * r[i]);
  c[j] = v;
}
"""

ENTRY = r"""
}  // namespace gb
extern "C" int emu_dgesvx(char fact, char trans, int n, int nrhs, double* a, int lda, double* af, int ldaf,
                          int* ipiv, char* equed, double* r, double* c, double* b, int ldb, double* x, int ldx,
                          double rowcnd, double colcnd, double* rcond, double* ferr, double* berr, double* rpvgrw) {
  int info = 0;
  gb::dgesvx_dev(fact, trans, n, nrhs, a, lda, af, ldaf, ipiv, equed, r, c, b, ldb, x, ldx, rowcnd, colcnd, rcond,
                 ferr, berr, rpvgrw, &info, nullptr);
  return info;
}
"""


def _slice(text, start, end):
    i = text.index(start)
    return text[i:text.index(end, i)]


@pytest.fixture(scope="module")
def emu(tmp_path_factory):
    if shutil.which("g++") is None:
        pytest.skip("needs g++")
    kern = open(os.path.join(CSRC, "condest_kernels.cuh")).read()
    kern = _slice(kern, "// ------------------------------------------------------------- DGESVX",
                  "}  // namespace gb")
    kern = kern.replace("geequ_colmax_kernel(", "geequ_colmax_kernel_warp(")    # the warp form, replaced below
    drv = open(os.path.join(CSRC, "refine.cu")).read()
    helpers = _slice(drv, "// max |A| over the upper triangle (upper) or the whole m x n block",
                     "int dgesvx_dev(")
    body = _slice(drv, "int dgesvx_dev(", "// FACT = 'F' on device scalings")
    src = cuda_emu.translate(PRELUDE + kern + COLMAX + "namespace {\n" + helpers + body + ENTRY, drop_includes=(),
                             min_launches=8)
    oracle.lib()
    so = cuda_emu.build(str(tmp_path_factory.mktemp("gesvxemu")), "gesvxemu", src, [CSRC])
    ctypes.CDLL(os.path.join(ORACLE_DIR, "liboracle.so"), mode=ctypes.RTLD_GLOBAL)
    L = ctypes.CDLL(so)
    p, i, d = ctypes.c_void_p, ctypes.c_int, ctypes.c_double
    L.emu_dgesvx.argtypes = [ctypes.c_char, ctypes.c_char, i, i, p, i, p, i, p, p, p, p, p, i, p, i, d, d, p, p, p, p]
    return L


def _run(emu, a, b, fact, trans):
    a = np.asfortranarray(np.array(a, dtype=np.float64, copy=True))
    b = np.asfortranarray(np.array(b, dtype=np.float64, copy=True))
    n, nrhs = b.shape
    ld = max(1, n)
    af = np.zeros((n, n), order="F")
    ipiv = np.zeros(ld, dtype=np.int32)
    r, c = np.zeros(ld), np.zeros(ld)
    eq = ctypes.create_string_buffer(b"N", 2)
    x = np.zeros((n, nrhs), order="F")
    rc, rp = np.zeros(1), np.zeros(1)
    ferr, berr = np.zeros(max(nrhs, 1)), np.zeros(max(nrhs, 1))
    p = lambda v: v.ctypes.data_as(ctypes.c_void_p)
    info = emu.emu_dgesvx(fact.encode(), trans.encode(), n, nrhs, p(a), ld, p(af), ld, p(ipiv), eq, p(r), p(c), p(b),
                          ld, p(x), ld, 1.0, 1.0, p(rc), p(ferr), p(berr), p(rp))
    return dict(a=a, af=af, ipiv=ipiv[:n], equed=eq.value.decode(), r=r[:n], c=c[:n], b=b, x=x, rcond=rc[0],
                ferr=ferr[:nrhs], berr=berr[:nrhs], rpvgrw=rp[0], info=info)


@pytest.mark.parametrize("fact", ["N", "E"])
@pytest.mark.parametrize("trans", ["N", "T"])
@pytest.mark.parametrize("n,imat,scale", [(1, 1, None), (10, 4, None), (50, 1, None), (50, 6, None), (50, 9, None),
                                          (60, 4, "rows"), (60, 4, "cols"), (60, 4, "both")])
def test_gesvx_cu_bitwise(emu, fact, trans, n, imat, scale):
    a, _ = oracle.ge_test_matrix(n, n, imat, 31 + n + imat)
    rng = np.random.default_rng(n)
    if scale in ("rows", "both"):
        a = a * (10.0 ** rng.uniform(-8, 8, n))[:, None]       # EQUED = 'R' (or 'B')
    if scale in ("cols", "both"):
        a = a * (10.0 ** rng.uniform(-8, 8, n))[None, :]       # EQUED = 'C' (or 'B')
    b = oracle.random_matrix(n, 2, 7 + n, idist=2)[0]
    ref = oracle.gesvx(a, b, fact=fact, trans=trans)
    got = _run(emu, a, b, fact, trans)
    assert got["info"] == ref["info"] and got["equed"] == ref["equed"], (got["info"], ref["info"], got["equed"])
    for key in ("a", "af", "ipiv", "r", "c", "b", "x", "ferr", "berr"):
        if ref["info"] > n and key in ("ferr", "berr"):
            continue
        g, r = np.asarray(got[key]), np.asarray(ref[key])
        if key in ("r", "c") and ref["equed"] == "N" and fact == "N":
            continue
        assert g.tobytes() == np.asfortranarray(r).astype(g.dtype).tobytes(), key
    assert np.float64(got["rcond"]).tobytes() == np.float64(ref["rcond"]).tobytes()
    assert np.float64(got["rpvgrw"]).tobytes() == np.float64(ref["rpvgrw"]).tobytes()
