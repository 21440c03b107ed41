// The per-thread steps of the complex LU on the GPU (ZGETRF, SRC/zgetrf.f:
// 144-225; ZGETRF2, SRC/zgetrf2.f:154-272; ZGETRS, SRC/zgetrs.f:157-223),
// written once for host and device.  Each function computes what one GPU
// thread computes -- one column of a ZLASWP or a ZTRSM, one element of a
// ZGEMM update, or the pivot step of one panel column -- in the reference
// loop order, so that the CPU tests can compose them exactly as the GPU
// driver does and compare with the oracle bit for bit.
//
// Templated on the component type R: COMPLEX*16 (R = double, the Z
// routines) and COMPLEX (R = float, the C twins, identical code modulo
// type).  A complex value is an (re, im) pair (the Fortran layout, aligned
// as R so that any caller's array is valid).  The arithmetic is that
// of gfortran's default complex rules: a product is (ar*br - ai*bi,
// ar*bi + ai*br), a quotient is Smith's method (R. L. Smith, "Algorithm 116:
// Complex division", CACM 5(8), 1962) branching on |br| < |bi|, every
// operation separately rounded (no contraction).  ABS of a complex value is
// hypot, which the reference only compares with the safe minimum.
#pragma once
#include <cmath>
#include <cstddef>

#include "latrs_seq.h"   // GB_HD, rn_*

namespace gb {

template <typename R>
struct cpx {
  R re, im;
};
using zdc = cpx<double>;
using cfc = cpx<float>;

// Per-type constants: SLAMCH/DLAMCH('O') (HUGE) and ('S') (TINY).
template <typename R> struct CpxLim;
template <> struct CpxLim<double> {
  static constexpr double huge = 1.7976931348623157e308, tiny = 2.2250738585072014e-308;
};
template <> struct CpxLim<float> {
  static constexpr float huge = 3.4028234663852886e38f, tiny = 1.17549435082228751e-38f;
};
GB_HD inline double zhypot(double a, double b) { return hypot(a, b); }
GB_HD inline float zhypot(float a, float b) { return hypotf(a, b); }

template <typename R>
GB_HD inline cpx<R> zmk(R re, R im) {
  cpx<R> z;
  z.re = re;
  z.im = im;
  return z;
}
template <typename R>
GB_HD inline cpx<R> zadd(cpx<R> a, cpx<R> b) { return zmk(rn_add(a.re, b.re), rn_add(a.im, b.im)); }
template <typename R>
GB_HD inline cpx<R> zsub(cpx<R> a, cpx<R> b) { return zmk(rn_sub(a.re, b.re), rn_sub(a.im, b.im)); }
template <typename R>
GB_HD inline cpx<R> zmul(cpx<R> a, cpx<R> b) {
  return zmk(rn_sub(rn_mul(a.re, b.re), rn_mul(a.im, b.im)), rn_add(rn_mul(a.re, b.im), rn_mul(a.im, b.re)));
}
template <typename R>
GB_HD inline cpx<R> zconj(cpx<R> a) { return zmk(a.re, -a.im); }
template <typename R>
GB_HD inline bool zis0(cpx<R> a) { return a.re == R(0) && a.im == R(0); }
template <typename R>
GB_HD inline cpx<R> zdiv(cpx<R> a, cpx<R> b) {
  if (fabs(b.re) < fabs(b.im)) {
    const R ratio = rn_div(b.re, b.im);
    const R div = rn_add(rn_mul(b.re, ratio), b.im);
    return zmk(rn_div(rn_add(rn_mul(a.re, ratio), a.im), div), rn_div(rn_sub(rn_mul(a.im, ratio), a.re), div));
  }
  const R ratio = rn_div(b.im, b.re);
  const R div = rn_add(rn_mul(b.im, ratio), b.re);
  return zmk(rn_div(rn_add(rn_mul(a.im, ratio), a.re), div), rn_div(rn_sub(a.im, rn_mul(a.re, ratio)), div));
}

// IZAMAX (BLAS/SRC/izamax.f90:95-147, INCX = 1), 1-based: the first NaN;
// else the first infinite part unless a NaN follows it; else the first
// maximum of |re| + |im|, compared as 0.25|re| + 0.25|im| once that sum
// overflows.
template <typename R>
GB_HD inline int izamax_seq(int n, const cpx<R>* x) {
  if (n < 1) return 0;
  if (n == 1) return 1;
  const R hugeval = CpxLim<R>::huge, q = R(0.25);
  int best = 0;
  bool scaled = false;
  R smax = R(-1);
  for (int i = 0; i < n; ++i) {
    const R ar = fabs(x[i].re), ai = fabs(x[i].im);
    if (x[i].re != x[i].re || x[i].im != x[i].im) return i + 1;
    if (ar > hugeval || ai > hugeval) {
      for (int j = i + 1; j < n; ++j)
        if (x[j].re != x[j].re || x[j].im != x[j].im) return j + 1;
      return i + 1;
    }
    if (!scaled) {
      const R val = rn_add(ar, ai);
      if (val > hugeval) {
        scaled = true;
        smax = rn_add(rn_mul(q, ar), rn_mul(q, ai));
        best = i + 1;
      } else if (val > smax) {
        smax = val;
        best = i + 1;
      }
    } else {
      const R val = rn_add(rn_mul(q, ar), rn_mul(q, ai));
      if (val > smax) {
        smax = val;
        best = i + 1;
      }
    }
  }
  return best;
}

// IZAMAX split over nt threads (thread t scans i = t, t + nt, ... in
// increasing order) and combined in any order: what izamax_seq returns,
// restated as independent reductions.  izamax_seq returns the first NaN if
// there is one (an infinite part only starts a search for a later NaN);
// else the first infinite part; else, when some |re| + |im| overflows (the
// first such index s), the first maximum of the scaled sums over i >= s
// (every earlier sum is finite and smaller); else the first maximum of the
// sums.  kNone marks an empty minimum.
constexpr int kZamaxNone = 0x7fffffff;
template <typename R>
struct ZamaxPart {
  int nan, inf, over;   // first index with a NaN part / an infinite part / an overflowing sum
  R val;                // the largest finite sum seen, at the first index idx
  int idx;
};
template <typename R>
GB_HD inline ZamaxPart<R> zamax_part(int n, const cpx<R>* x, int t, int nt) {
  const R hugeval = CpxLim<R>::huge;
  ZamaxPart<R> p{kZamaxNone, kZamaxNone, kZamaxNone, R(-1), kZamaxNone};
  for (int i = t; i < n; i += nt) {
    const R ar = fabs(x[i].re), ai = fabs(x[i].im);
    if (x[i].re != x[i].re || x[i].im != x[i].im) {
      if (p.nan == kZamaxNone) p.nan = i;
      continue;
    }
    if (ar > hugeval || ai > hugeval) {
      if (p.inf == kZamaxNone) p.inf = i;
      continue;
    }
    const R val = rn_add(ar, ai);
    if (val > hugeval) {
      if (p.over == kZamaxNone) p.over = i;
    } else if (val > p.val) {
      p.val = val;
      p.idx = i;
    }
  }
  return p;
}
// the larger value wins, the smaller index on a tie
template <typename R>
GB_HD inline void zamax_pick(R& val, int& idx, R v2, int i2) {
  if (v2 > val || (v2 == val && i2 < idx)) {
    val = v2;
    idx = i2;
  }
}
template <typename R>
GB_HD inline ZamaxPart<R> zamax_combine(ZamaxPart<R> a, const ZamaxPart<R>& b) {
  a.nan = a.nan < b.nan ? a.nan : b.nan;
  a.inf = a.inf < b.inf ? a.inf : b.inf;
  a.over = a.over < b.over ? a.over : b.over;
  zamax_pick(a.val, a.idx, b.val, b.idx);
  return a;
}
// The scaled pass (only when some sum overflowed, from index s): the first
// maximum of 0.25|re| + 0.25|im| over this thread's i >= s.
template <typename R>
GB_HD inline void zamax_scaled_part(int n, const cpx<R>* x, int s, int t, int nt, R* val, int* idx) {
  const R q = R(0.25);
  *val = R(-1);
  *idx = kZamaxNone;
  int i0 = t;
  if (i0 < s) i0 += (s - i0 + nt - 1) / nt * nt;
  for (int i = i0; i < n; i += nt) {
    const R ar = fabs(x[i].re), ai = fabs(x[i].im);
    const R v = rn_add(rn_mul(q, ar), rn_mul(q, ai));
    if (v > *val) {
      *val = v;
      *idx = i;
    }
  }
}
// 1-based result from the combined first pass (n >= 2); the scaled pass is
// consulted only when p.nan and p.inf are empty and p.over is not.
template <typename R>
GB_HD inline int zamax_result(const ZamaxPart<R>& p, int scaled_idx) {
  if (p.nan != kZamaxNone) return p.nan + 1;
  if (p.inf != kZamaxNone) return p.inf + 1;
  if (p.over != kZamaxNone) return scaled_idx + 1;
  return p.idx + 1;
}

// The one-column step of ZGETRF2 (SRC/zgetrf2.f:176-211): the M = 1 branch
// (IPIV = 1, a zero flagged) or the N = 1 branch (pivot search, swap, and
// the column scaled by the reciprocal of the pivot when |pivot| >= SFMIN,
// through ZSCAL with its ZA = ONE quick return, else divided by it).  Column
// `a` has m rows; returns the local INFO (0 or 1) and sets *ipiv (1-based).
template <typename R>
GB_HD inline int zgetrf2_col(int m, cpx<R>* a, int* ipiv) {
  if (m == 1) {
    *ipiv = 1;
    return zis0(a[0]) ? 1 : 0;
  }
  const int p = izamax_seq(m, a);
  *ipiv = p;
  if (zis0(a[p - 1])) return 1;
  if (p != 1) {
    const cpx<R> t = a[0];
    a[0] = a[p - 1];
    a[p - 1] = t;
  }
  if (zhypot(a[0].re, a[0].im) >= CpxLim<R>::tiny) {   // ABS(A(1,1)) >= SFMIN
    const cpx<R> r = zdiv(zmk(R(1), R(0)), a[0]);
    if (!(r.re == R(1) && r.im == R(0)))
      for (int i = 1; i < m; ++i) a[i] = zmul(r, a[i]);
  } else {
    for (int i = 1; i < m; ++i) a[i] = zdiv(a[i], a[0]);
  }
  return 0;
}

// One column of ZLASWP (SRC/zlaswp.f:138-189): rows K1..K2 (1-based)
// interchanged with IPIV(K1..K2) in order, or in reverse order for INCX < 0.
template <typename R>
GB_HD inline void zlaswp_col(cpx<R>* col, int k1, int k2, const int* ipiv, int incx) {
  if (incx > 0) {
    for (int i = k1; i <= k2; ++i) {
      const int ip = ipiv[i - 1];
      if (ip != i) {
        const cpx<R> t = col[i - 1];
        col[i - 1] = col[ip - 1];
        col[ip - 1] = t;
      }
    }
  } else if (incx < 0) {
    for (int i = k2; i >= k1; --i) {
      const int ip = ipiv[i - 1];
      if (ip != i) {
        const cpx<R> t = col[i - 1];
        col[i - 1] = col[ip - 1];
        col[ip - 1] = t;
      }
    }
  }
}

// One column b of ZTRSM('L', UPLO, TRANSA, DIAG) with ALPHA = ONE
// (BLAS/SRC/ztrsm.f:272-345): trans 0 = 'N', 1 = 'T', 2 = 'C'.  The column
// is first multiplied by ALPHA, as the reference does.  The triangle and the
// column never overlap (restrict: a step's loads can be issued ahead).
template <typename R>
GB_HD inline void ztrsm_left_col(int upper, int trans, int unit, int m, const cpx<R>* __restrict__ A, int lda,
                                 cpx<R>* __restrict__ b) {
  auto a = [&](int i, int j) -> cpx<R> { return A[(size_t)i + (size_t)j * lda]; };
  const cpx<R> one = zmk(R(1), R(0));
  if (trans == 0) {
    for (int i = 0; i < m; ++i) b[i] = zmul(one, b[i]);
    if (upper) {
      for (int k = m - 1; k >= 0; --k) {
        if (!unit) b[k] = zdiv(b[k], a(k, k));
        for (int i = 0; i < k; ++i) b[i] = zsub(b[i], zmul(b[k], a(i, k)));
      }
    } else {
      for (int k = 0; k < m; ++k) {
        if (!unit) b[k] = zdiv(b[k], a(k, k));
        for (int i = k + 1; i < m; ++i) b[i] = zsub(b[i], zmul(b[k], a(i, k)));
      }
    }
    return;
  }
  const bool cj = trans == 2;
  if (upper) {
    for (int i = 0; i < m; ++i) {
      cpx<R> t = zmul(one, b[i]);
      for (int k = 0; k < i; ++k) t = zsub(t, zmul(cj ? zconj(a(k, i)) : a(k, i), b[k]));
      if (!unit) t = zdiv(t, cj ? zconj(a(i, i)) : a(i, i));
      b[i] = t;
    }
  } else {
    for (int i = m - 1; i >= 0; --i) {
      cpx<R> t = zmul(one, b[i]);
      for (int k = i + 1; k < m; ++k) t = zsub(t, zmul(cj ? zconj(a(k, i)) : a(k, i), b[k]));
      if (!unit) t = zdiv(t, cj ? zconj(a(i, i)) : a(i, i));
      b[i] = t;
    }
  }
}

// One element (i, j) of ZGEMM('N', 'N') with ALPHA = -ONE, BETA = ONE
// (BLAS/SRC/zgemm.f:326-340): TEMP = ALPHA*B(L,J), C(I,J) = C(I,J) +
// TEMP*A(I,L), L increasing.
template <typename R>
GB_HD inline void zgemm_nn_elem(int i, int j, int k, const cpx<R>* A, int lda, const cpx<R>* B, int ldb, cpx<R>* C,
                                int ldc) {
  const cpx<R> alpha = zmk(R(-1), R(0));
  cpx<R> c = C[(size_t)i + (size_t)j * ldc];
  for (int l = 0; l < k; ++l) {
    const cpx<R> temp = zmul(alpha, B[(size_t)l + (size_t)j * ldb]);
    c = zadd(c, zmul(temp, A[(size_t)i + (size_t)l * lda]));
  }
  C[(size_t)i + (size_t)j * ldc] = c;
}

// ---- the per-thread steps of ZCGESV (SRC/zcgesv.f:259-448)

// ZLAG2C of one element (SRC/zlag2c.f:135-147): false when a part lies
// outside [-RMAX, RMAX] (RMAX = SLAMCH('O')), else SA = CMPLX(A), each part
// rounded to nearest.  (The reference stops converting at the first such
// element; the driver then falls back and SA is not used.)
GB_HD inline bool zlag2c_elem(zdc a, cfc* sa) {
  const double rmax = CpxLim<float>::huge;
  if (a.re < -rmax || a.re > rmax || a.im < -rmax || a.im > rmax) return false;
  sa->re = (float)a.re;
  sa->im = (float)a.im;
  return true;
}

// Row sum i of ZLANGE('I') (SRC/zlange.f:175-185): |A(i,j)| = hypot added in
// column order.
GB_HD inline double zlange_row(int i, int n, const zdc* A, int lda) {
  double s = 0.0;
  for (int j = 0; j < n; ++j) {
    const zdc v = A[(size_t)i + (size_t)j * lda];
    s = rn_add(s, zhypot(v.re, v.im));
  }
  return s;
}

// ZLANGE's maximum of the row sums, a NaN taking over (SRC/zlange.f:186-190).
GB_HD inline double zlange_max(int n, const double* rows) {
  double v = 0.0;
  for (int i = 0; i < n; ++i)
    if (v < rows[i] || rows[i] != rows[i]) v = rows[i];
  return v;
}

// The convergence test of one column (SRC/zcgesv.f:350-357): true when
// CABS1(R(IZAMAX(R))) > CABS1(X(IZAMAX(X)))*CTE, i.e. not converged.
GB_HD inline bool zcgesv_col_notconv(int n, const zdc* x, const zdc* r, double cte) {
  const zdc xv = x[izamax_seq(n, x) - 1], rv = r[izamax_seq(n, r) - 1];
  const double xnrm = rn_add(fabs(xv.re), fabs(xv.im)), rnrm = rn_add(fabs(rv.re), fabs(rv.im));
  return rnrm > rn_mul(xnrm, cte);
}

// CLAG2Z of one element, or CLAG2Z then ZAXPY with ZA = ONE
// (BLAS/SRC/zaxpy.f:114-118: ZY = ZY + ZA*ZX) when `add`.
GB_HD inline void zlag2z_elem(cfc s, zdc* x, bool add) {
  const zdc w = zmk((double)s.re, (double)s.im);
  *x = add ? zadd(*x, zmul(zmk(1.0, 0.0), w)) : w;
}

// The schedules of ZGETRF2, ZGETRF and ZGETRS, written once over a backend
// that runs each step: on the GPU every step is one kernel launch (zlu.cu),
// in the CPU tests the same steps run as loops over the functions above.
// A backend provides
//   col(m, a, ipiv, gcol)   zgetrf2_col on one column; a zero pivot records
//                           INFO = gcol (1-based global column), the first
//                           in column order winning
//   laswp(ncols, A, lda, k1, k2, ipiv, incx)
//   trsm(upper, trans, unit, m, ncols, A, lda, B, ldb)
//   gemm(m, n, k, A, lda, B, ldb, C, ldc)        C -= A*B
//   ipiv_add(ipiv, count, off)
// each returning 0 or an error code.

// ZGETRF2 (SRC/zgetrf2.f:172-268) of the m x n panel A whose first column is
// global column col0 (0-based).
template <class Ops, typename R>
int zgetrf2_sched(Ops& ops, int m, int n, cpx<R>* A, int lda, int* ipiv, int col0) {
  if (m == 0 || n == 0) return 0;
  if (m == 1 || n == 1) return ops.col(m, A, ipiv, col0 + 1);
  const int mn = m < n ? m : n;
  const int n1 = mn / 2, n2 = n - n1;
  int rc;
  cpx<R>* A12 = A + (size_t)n1 * lda;
  if ((rc = zgetrf2_sched(ops, m, n1, A, lda, ipiv, col0))) return rc;
  if ((rc = ops.laswp(n2, A12, lda, 1, n1, ipiv, 1))) return rc;
  if ((rc = ops.trsm(0, 0, 1, n1, n2, A, lda, A12, lda))) return rc;
  if ((rc = ops.gemm(m - n1, n2, n1, A + n1, lda, A12, lda, A12 + n1, lda))) return rc;
  if ((rc = zgetrf2_sched(ops, m - n1, n2, A12 + n1, lda, ipiv + n1, col0 + n1))) return rc;
  if ((rc = ops.ipiv_add(ipiv + n1, mn - n1, n1))) return rc;
  return ops.laswp(n1, A, lda, n1 + 1, mn, ipiv, 1);
}

// ZGETRF (SRC/zgetrf.f:175-222) with block size nb.
template <class Ops, typename R>
int zgetrf_sched(Ops& ops, int m, int n, cpx<R>* A, int lda, int* ipiv, int nb) {
  if (m == 0 || n == 0) return 0;
  const int mn = m < n ? m : n;
  if (nb <= 1 || nb >= mn) return zgetrf2_sched(ops, m, n, A, lda, ipiv, 0);
  int rc;
  for (int j = 0; j < mn; j += nb) {
    const int jb = mn - j < nb ? mn - j : nb;
    cpx<R>* Ajj = A + j + (size_t)j * lda;
    if ((rc = zgetrf2_sched(ops, m - j, jb, Ajj, lda, ipiv + j, j))) return rc;
    if ((rc = ops.ipiv_add(ipiv + j, (m < j + jb ? m : j + jb) - j, j))) return rc;
    if ((rc = ops.laswp(j, A, lda, j + 1, j + jb, ipiv, 1))) return rc;
    if (j + jb < n) {
      cpx<R>* right = A + (size_t)(j + jb) * lda;
      if ((rc = ops.laswp(n - j - jb, right, lda, j + 1, j + jb, ipiv, 1))) return rc;
      if ((rc = ops.trsm(0, 0, 1, jb, n - j - jb, Ajj, lda, right + j, lda))) return rc;
      if (j + jb < m && (rc = ops.gemm(m - j - jb, n - j - jb, jb, Ajj + jb, lda, right + j, lda, right + j + jb, lda)))
        return rc;
    }
  }
  return 0;
}

// ZGETRS (SRC/zgetrs.f:207-220); trans 0 = 'N', 1 = 'T', 2 = 'C'.
template <class Ops, typename R>
int zgetrs_sched(Ops& ops, int trans, int n, int nrhs, const cpx<R>* A, int lda, const int* ipiv, cpx<R>* B,
                 int ldb) {
  if (n == 0 || nrhs == 0) return 0;
  int rc;
  if (trans == 0) {
    if ((rc = ops.laswp(nrhs, B, ldb, 1, n, ipiv, 1))) return rc;
    if ((rc = ops.trsm(0, 0, 1, n, nrhs, A, lda, B, ldb))) return rc;
    return ops.trsm(1, 0, 0, n, nrhs, A, lda, B, ldb);
  }
  if ((rc = ops.trsm(1, trans, 0, n, nrhs, A, lda, B, ldb))) return rc;
  if ((rc = ops.trsm(0, trans, 1, n, nrhs, A, lda, B, ldb))) return rc;
  return ops.laswp(nrhs, B, ldb, 1, n, ipiv, -1);
}

// xGETRF with its INFO: the backend's INFO word is reset, the schedule run,
// the word read back (0 when no pivot was zero).
template <class Ops, typename R>
int zgetrf_full(Ops& ops, int m, int n, cpx<R>* A, int lda, int* ipiv, int nb, int* info) {
  int rc = ops.info_reset();
  if (rc) return rc;
  if ((rc = zgetrf_sched(ops, m, n, A, lda, ipiv, nb))) return rc;
  return ops.info_read(info);
}

// ZCGESV (SRC/zcgesv.f:294-448): ANRM = ZLANGE('I'), CTE = ANRM*EPS*
// SQRT(N)*BWDMAX; B and A to COMPLEX (ITER = -2 on overflow); CGETRF
// (ITER = -3 on a zero pivot); CGETRS, CLAG2Z; then up to ITERMAX = 30
// corrections, each ZLAG2C of the residual, CGETRS, CLAG2Z + ZAXPY, the
// COMPLEX*16 residual by ZGEMM and the convergence test; ITER = -31, or any
// exit above, falls back to ZGETRF / ZGETRS on A.  SA (n x n), SX and R
// (n x nrhs, leading dimension n) are workspace.  The backend adds
//   lange_inf(n, A, lda, &anrm)       ANRM into a host double
//   flags_reset(), flags_read(&overflow, &notconv)
//   lag2c(m, ncols, A, lda, SA, ldsa) sets the overflow flag
//   lag2z(m, ncols, SX, ldsx, X, ldx, add)
//   copy(m, ncols, B, ldb, R, ldr)
//   check(n, nrhs, X, ldx, R, ldr, cte) sets the notconv flag.
// A conversion overflow inside the loop is acted on after that iteration's
// residual: X is replaced by the fallback anyway, so the result is the
// reference's.
template <class Ops>
int zcgesv_sched(Ops& ops, int n, int nrhs, zdc* A, int lda, int* ipiv, const zdc* B, int ldb, zdc* X, int ldx,
                 cfc* SA, cfc* SX, zdc* R, int* iter, int* info) {
  const int itermax = 30;
  const double bwdmax = 1.0, eps = 1.1102230246251565e-16;   // DLAMCH('Epsilon')
  *iter = 0;
  *info = 0;
  if (n == 0) return 0;
  int rc, ovf = 0, nc = 0, sinfo = 0;
  double anrm = 0.0;
  if ((rc = ops.lange_inf(n, (const zdc*)A, lda, &anrm))) return rc;
  const double cte = anrm * eps * sqrt((double)n) * bwdmax;
  auto fallback = [&]() -> int {
    if ((rc = zgetrf_full(ops, n, n, A, lda, ipiv, 64, info))) return rc;
    if (*info != 0) return 0;
    if ((rc = ops.copy(n, nrhs, B, ldb, X, ldx))) return rc;
    return zgetrs_sched(ops, 0, n, nrhs, (const zdc*)A, lda, ipiv, X, ldx);
  };
  auto residual = [&]() -> int {
    if ((rc = ops.copy(n, nrhs, B, ldb, R, n))) return rc;
    if ((rc = ops.gemm(n, nrhs, n, (const zdc*)A, lda, (const zdc*)X, ldx, R, n))) return rc;
    if ((rc = ops.check(n, nrhs, (const zdc*)X, ldx, (const zdc*)R, n, cte))) return rc;
    return ops.flags_read(&ovf, &nc);
  };
  if ((rc = ops.flags_reset())) return rc;
  if ((rc = ops.lag2c(n, nrhs, B, ldb, SX, n))) return rc;
  if ((rc = ops.lag2c(n, n, (const zdc*)A, lda, SA, n))) return rc;
  if ((rc = ops.flags_read(&ovf, &nc))) return rc;
  if (ovf) {
    *iter = -2;
    return fallback();
  }
  if ((rc = zgetrf_full(ops, n, n, SA, n, ipiv, 64, &sinfo))) return rc;
  if (sinfo != 0) {
    *iter = -3;
    return fallback();
  }
  if ((rc = zgetrs_sched(ops, 0, n, nrhs, (const cfc*)SA, n, ipiv, SX, n))) return rc;
  if ((rc = ops.lag2z(n, nrhs, (const cfc*)SX, n, X, ldx, false))) return rc;
  if ((rc = residual())) return rc;
  if (!nc) return 0;
  for (int it = 1; it <= itermax; ++it) {
    if ((rc = ops.flags_reset())) return rc;
    if ((rc = ops.lag2c(n, nrhs, (const zdc*)R, n, SX, n))) return rc;
    if ((rc = zgetrs_sched(ops, 0, n, nrhs, (const cfc*)SA, n, ipiv, SX, n))) return rc;
    if ((rc = ops.lag2z(n, nrhs, (const cfc*)SX, n, X, ldx, true))) return rc;
    if ((rc = residual())) return rc;
    if (ovf) {
      *iter = -2;
      return fallback();
    }
    if (!nc) {
      *iter = it;
      return 0;
    }
  }
  *iter = -itermax - 1;
  return fallback();
}

}  // namespace gb
