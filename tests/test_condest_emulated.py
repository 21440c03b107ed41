"""DGECON and DLATRS's GPU drivers (latrs_dev, dgecon_dev, dlatrs_dev in
lapack_gb300/csrc/refine.cu) with the DLATRS kernels of condest_kernels.cuh,
run on the CPU.

The CNORM kernel in exact mode (one thread per column), the growth-bound
plan, the careful scaled solve and DGECON's rescaling step (one thread each)
are one-dimensional launches, so running their blocks and threads one after
another computes what the GPU computes.  The test takes the drivers and those
kernels out of the sources, runs their launches sequentially over a stand-in
for the CUDA runtime (tests/cuda_emu.py), and puts the oracle in place of the
two pieces that cooperate within a CTA and run on the GB300 in their own
tests: the DLACN2 step on device vectors (bitwise the oracle's in the DGERFS
tests) and the DTRSV-order plain solve (bitwise the oracle's in the DLATRS
tests).  x, SCALE and CNORM of DLATRS for every UPLO / TRANS / DIAG on plain,
tiny-pivot, mixed and overflowing triangles, and DGECON's RCOND on the
DCHKGE types and on factors with tiny pivots, are compared with the oracle
bit for bit; these are the careful-path cases."""
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
#include "latrs_seq.h"
static inline double __dadd_rn(double a, double b) { return a + b; }
static inline double __shfl_xor_sync(unsigned, double v, int) { return v; }   // compiles the unused warp branch
extern "C" {
void or_dlacn2(int n, double* v, double* x, int* isgn, double* est, int* kase, int isave[3]);
void or_dtrsv(char uplo, char trans, char diag, int n, const double* a, int lda, double* x);
}
namespace gb {
enum { kStatusCapacity = 3 };
struct Options { int exact = 1; };
inline const Options& options() { static Options o; return o; }
struct ColList { int n; int c[64]; };
struct LacnState { double est; int kase; int jump; int j; int iter; };
// one DLACN2 step per listed column, as the oracle computes it
template <bool EXACT>
__global__ void lacn2_step_kernel(int n, double* Xe, int ldx, double* V, int* Isgn, LacnState* st, ColList cols) {
  if (threadIdx.x) return;
  const int c = cols.c[blockIdx.x];
  LacnState& S = st[c];
  int isave[3] = {S.jump, S.j, S.iter};
  or_dlacn2(n, V + (size_t)c * n, Xe + (size_t)c * ldx, Isgn + (size_t)c * n, &S.est, &S.kase, isave);
  S.jump = isave[0];
  S.j = isave[1];
  S.iter = isave[2];
}
// the plain solve in the DTRSV loop order
int dtrsv_dev(bool upper, bool trans, bool unit, int n, const double* dA, int lda, double* dX, cudaStream_t) {
  if (n > 0) or_dtrsv(upper ? 'U' : 'L', trans ? 'T' : 'N', unit ? 'U' : 'N', n, dA, lda, dX);
  return 0;
}
"""

ENTRY = r"""
}  // namespace gb
extern "C" {
int emu_dlatrs(int upper, int trans, int unit, int normin_y, int n, const double* a, int lda, double* x,
               double* scale, double* cnorm) {
  return gb::dlatrs_dev(upper != 0, trans != 0, unit != 0, normin_y != 0, n, a, lda, x, scale, cnorm, nullptr);
}
int emu_dgecon(char norm, int n, const double* lu, int lda, double anorm, double* rcond) {
  int info = 0;
  int rc = gb::dgecon_dev(norm, n, lu, lda, anorm, rcond, &info, nullptr);
  return rc ? -1000 - rc : info;
}
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
    kern = _slice(kern, "// ------------------------------------------------------------- CNORM", "}  // namespace gb")
    drv = open(os.path.join(CSRC, "refine.cu")).read()
    latrs = _slice(drv, "// One DLATRS call on the device vector x", "}  // namespace\n")
    gecon = _slice(drv, "int dgecon_dev(", "namespace {\n")
    src = cuda_emu.translate(PRELUDE + kern + "namespace {\n" + latrs + "}  // namespace\n" + gecon + ENTRY,
                             drop_includes=(), min_launches=6)
    oracle.lib()
    so = cuda_emu.build(str(tmp_path_factory.mktemp("gecon_emu")), "geconemu", src, [CSRC])
    ctypes.CDLL(os.path.join(ORACLE_DIR, "liboracle.so"), mode=ctypes.RTLD_GLOBAL)
    L = ctypes.CDLL(so)
    i, p, d = ctypes.c_int, ctypes.c_void_p, ctypes.c_double
    L.emu_dlatrs.argtypes = [i, i, i, i, i, p, i, p, p, p]
    L.emu_dgecon.argtypes = [ctypes.c_char, i, p, i, d, p]
    return L


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p)


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
        out.append((n, kind, np.asfortranarray(t), rng.standard_normal(n)))
    return out


@pytest.mark.parametrize("uplo,trans,diag", [(u, t, d) for u in "UL" for t in "NT" for d in "NU"])
def test_latrs_cu_bitwise(emu, uplo, trans, diag):
    careful = False
    for n, kind, t, b in _cases(uplo, diag, 7 + ord(uplo) * 3 + ord(trans) * 5 + ord(diag)):
        xr, sr, cr = oracle.latrs(t, b, uplo, trans, diag)
        x = np.array(b, dtype=np.float64, copy=True)
        sc = np.zeros(1)
        cn = np.zeros(max(n, 1))
        rc = emu.emu_dlatrs(int(uplo == "U"), int(trans != "N"), int(diag == "U"), 0, n, _ptr(t), n, _ptr(x),
                            _ptr(sc), _ptr(cn))
        assert rc == 0
        assert np.float64(sc[0]).tobytes() == np.float64(sr).tobytes(), (n, kind, sc[0], sr)
        assert x.tobytes() == xr.tobytes(), (n, kind)
        assert cn[:n].tobytes() == cr.tobytes(), (n, kind)
        careful |= sr < 1.0
    assert careful


@pytest.mark.parametrize("imat", range(1, 12))
def test_gecon_cu_bitwise_dchkge(emu, imat):
    for n in (3, 10, 50, 130):
        if 5 <= imat <= 7 and n < imat - 4:
            continue
        a, izero = oracle.ge_test_matrix(n, n, imat, 1988 + 9 * n)
        lu, ipiv, info = oracle.getrf(a)
        if info:
            continue
        for norm, p in (("1", 1), ("I", np.inf)):
            anorm = np.linalg.norm(a, p)
            r_ref, i_ref = oracle.gecon(lu, anorm, norm)
            rc = np.zeros(1)
            inf = emu.emu_dgecon(norm.encode(), n, _ptr(np.asfortranarray(lu)), n, anorm, _ptr(rc))
            assert inf == i_ref
            assert np.float64(rc[0]).tobytes() == np.float64(r_ref).tobytes(), (n, imat, norm, rc[0], r_ref)


@pytest.mark.parametrize("tiny", [1e-10, 1e-200, 1e-300, 1e-310])
def test_gecon_cu_tiny_pivots(emu, tiny):
    """U with tiny pivots every 7th column: the careful solve and the
    rescaling step (or its early RCOND = 0) as the oracle."""
    n = 40
    rng = np.random.default_rng(int(-np.log10(tiny)))
    lu = rng.standard_normal((n, n))
    d = np.ones(n)
    d[::7] = tiny
    lu[np.diag_indices(n)] = d
    luf = np.asfortranarray(lu)
    for norm in "1I":
        r_ref, i_ref = oracle.gecon(lu, 3.0, norm)
        rc = np.zeros(1)
        inf = emu.emu_dgecon(norm.encode(), n, _ptr(luf), n, 3.0, _ptr(rc))
        assert inf == i_ref
        assert np.float64(rc[0]).tobytes() == np.float64(r_ref).tobytes(), (tiny, norm, rc[0], r_ref)
