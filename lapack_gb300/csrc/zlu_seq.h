// The per-thread steps of the complex LU on the GPU (ZGETRF, SRC/zgetrf.f:
// 144-225; ZGETRF2, SRC/zgetrf2.f:154-272; ZGETRS, SRC/zgetrs.f:157-223),
// written once for host and device.  Each function computes what one GPU
// thread computes -- one column of a ZLASWP or a ZTRSM, one element of a
// ZGEMM update, or the pivot step of one panel column -- in the reference
// loop order, so that the CPU tests can compose them exactly as the GPU
// driver does and compare with the oracle bit for bit.
//
// COMPLEX*16 is a (re, im) pair of doubles (the Fortran layout, 8-byte
// aligned here so that any caller's array is valid).  The arithmetic is that
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

struct zdc {
  double re, im;
};

GB_HD inline zdc zmk(double re, double im) {
  zdc z;
  z.re = re;
  z.im = im;
  return z;
}
GB_HD inline zdc zadd(zdc a, zdc b) { return zmk(rn_add(a.re, b.re), rn_add(a.im, b.im)); }
GB_HD inline zdc zsub(zdc a, zdc b) { return zmk(rn_sub(a.re, b.re), rn_sub(a.im, b.im)); }
GB_HD inline zdc zmul(zdc a, zdc b) {
  return zmk(rn_sub(rn_mul(a.re, b.re), rn_mul(a.im, b.im)), rn_add(rn_mul(a.re, b.im), rn_mul(a.im, b.re)));
}
GB_HD inline zdc zconj(zdc a) { return zmk(a.re, -a.im); }
GB_HD inline bool zis0(zdc a) { return a.re == 0.0 && a.im == 0.0; }
GB_HD inline zdc zdiv(zdc a, zdc b) {
  if (fabs(b.re) < fabs(b.im)) {
    const double ratio = rn_div(b.re, b.im);
    const double div = rn_add(rn_mul(b.re, ratio), b.im);
    return zmk(rn_div(rn_add(rn_mul(a.re, ratio), a.im), div), rn_div(rn_sub(rn_mul(a.im, ratio), a.re), div));
  }
  const double ratio = rn_div(b.im, b.re);
  const double div = rn_add(rn_mul(b.im, ratio), b.re);
  return zmk(rn_div(rn_add(rn_mul(a.im, ratio), a.re), div), rn_div(rn_sub(a.im, rn_mul(a.re, ratio)), div));
}

// IZAMAX (BLAS/SRC/izamax.f90:95-147, INCX = 1), 1-based: the first NaN;
// else the first infinite part unless a NaN follows it; else the first
// maximum of |re| + |im|, compared as 0.25|re| + 0.25|im| once that sum
// overflows.
GB_HD inline int izamax_seq(int n, const zdc* x) {
  if (n < 1) return 0;
  if (n == 1) return 1;
  const double hugeval = 1.7976931348623157e308;
  int best = 0;
  bool scaled = false;
  double smax = -1.0;
  for (int i = 0; i < n; ++i) {
    const double ar = fabs(x[i].re), ai = fabs(x[i].im);
    if (x[i].re != x[i].re || x[i].im != x[i].im) return i + 1;
    if (ar > hugeval || ai > hugeval) {
      for (int j = i + 1; j < n; ++j)
        if (x[j].re != x[j].re || x[j].im != x[j].im) return j + 1;
      return i + 1;
    }
    if (!scaled) {
      const double val = rn_add(ar, ai);
      if (val > hugeval) {
        scaled = true;
        smax = rn_add(rn_mul(0.25, ar), rn_mul(0.25, ai));
        best = i + 1;
      } else if (val > smax) {
        smax = val;
        best = i + 1;
      }
    } else {
      const double val = rn_add(rn_mul(0.25, ar), rn_mul(0.25, ai));
      if (val > smax) {
        smax = val;
        best = i + 1;
      }
    }
  }
  return best;
}

// The one-column step of ZGETRF2 (SRC/zgetrf2.f:176-211): the M = 1 branch
// (IPIV = 1, a zero flagged) or the N = 1 branch (pivot search, swap, and
// the column scaled by the reciprocal of the pivot when |pivot| >= SFMIN,
// through ZSCAL with its ZA = ONE quick return, else divided by it).  Column
// `a` has m rows; returns the local INFO (0 or 1) and sets *ipiv (1-based).
GB_HD inline int zgetrf2_col(int m, zdc* a, int* ipiv) {
  if (m == 1) {
    *ipiv = 1;
    return zis0(a[0]) ? 1 : 0;
  }
  const int p = izamax_seq(m, a);
  *ipiv = p;
  if (zis0(a[p - 1])) return 1;
  if (p != 1) {
    const zdc t = a[0];
    a[0] = a[p - 1];
    a[p - 1] = t;
  }
  const double sfmin = 2.2250738585072014e-308;   // DLAMCH('S')
  if (hypot(a[0].re, a[0].im) >= sfmin) {
    const zdc r = zdiv(zmk(1.0, 0.0), a[0]);
    if (!(r.re == 1.0 && r.im == 0.0))
      for (int i = 1; i < m; ++i) a[i] = zmul(r, a[i]);
  } else {
    for (int i = 1; i < m; ++i) a[i] = zdiv(a[i], a[0]);
  }
  return 0;
}

// One column of ZLASWP (SRC/zlaswp.f:138-189): rows K1..K2 (1-based)
// interchanged with IPIV(K1..K2) in order, or in reverse order for INCX < 0.
GB_HD inline void zlaswp_col(zdc* col, int k1, int k2, const int* ipiv, int incx) {
  if (incx > 0) {
    for (int i = k1; i <= k2; ++i) {
      const int ip = ipiv[i - 1];
      if (ip != i) {
        const zdc t = col[i - 1];
        col[i - 1] = col[ip - 1];
        col[ip - 1] = t;
      }
    }
  } else if (incx < 0) {
    for (int i = k2; i >= k1; --i) {
      const int ip = ipiv[i - 1];
      if (ip != i) {
        const zdc t = col[i - 1];
        col[i - 1] = col[ip - 1];
        col[ip - 1] = t;
      }
    }
  }
}

// One column b of ZTRSM('L', UPLO, TRANSA, DIAG) with ALPHA = ONE
// (BLAS/SRC/ztrsm.f:272-345): trans 0 = 'N', 1 = 'T', 2 = 'C'.  The column
// is first multiplied by ALPHA, as the reference does.
GB_HD inline void ztrsm_left_col(int upper, int trans, int unit, int m, const zdc* A, int lda, zdc* b) {
  auto a = [&](int i, int j) -> zdc { return A[(size_t)i + (size_t)j * lda]; };
  const zdc one = zmk(1.0, 0.0);
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
      zdc t = zmul(one, b[i]);
      for (int k = 0; k < i; ++k) t = zsub(t, zmul(cj ? zconj(a(k, i)) : a(k, i), b[k]));
      if (!unit) t = zdiv(t, cj ? zconj(a(i, i)) : a(i, i));
      b[i] = t;
    }
  } else {
    for (int i = m - 1; i >= 0; --i) {
      zdc t = zmul(one, b[i]);
      for (int k = i + 1; k < m; ++k) t = zsub(t, zmul(cj ? zconj(a(k, i)) : a(k, i), b[k]));
      if (!unit) t = zdiv(t, cj ? zconj(a(i, i)) : a(i, i));
      b[i] = t;
    }
  }
}

// One element (i, j) of ZGEMM('N', 'N') with ALPHA = -ONE, BETA = ONE
// (BLAS/SRC/zgemm.f:326-340): TEMP = ALPHA*B(L,J), C(I,J) = C(I,J) +
// TEMP*A(I,L), L increasing.
GB_HD inline void zgemm_nn_elem(int i, int j, int k, const zdc* A, int lda, const zdc* B, int ldb, zdc* C, int ldc) {
  const zdc alpha = zmk(-1.0, 0.0);
  zdc c = C[(size_t)i + (size_t)j * ldc];
  for (int l = 0; l < k; ++l) {
    const zdc temp = zmul(alpha, B[(size_t)l + (size_t)j * ldb]);
    c = zadd(c, zmul(temp, A[(size_t)i + (size_t)l * lda]));
  }
  C[(size_t)i + (size_t)j * ldc] = c;
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
template <class Ops>
int zgetrf2_sched(Ops& ops, int m, int n, zdc* A, int lda, int* ipiv, int col0) {
  if (m == 0 || n == 0) return 0;
  if (m == 1 || n == 1) return ops.col(m, A, ipiv, col0 + 1);
  const int mn = m < n ? m : n;
  const int n1 = mn / 2, n2 = n - n1;
  int rc;
  zdc* A12 = A + (size_t)n1 * lda;
  if ((rc = zgetrf2_sched(ops, m, n1, A, lda, ipiv, col0))) return rc;
  if ((rc = ops.laswp(n2, A12, lda, 1, n1, ipiv, 1))) return rc;
  if ((rc = ops.trsm(0, 0, 1, n1, n2, A, lda, A12, lda))) return rc;
  if ((rc = ops.gemm(m - n1, n2, n1, A + n1, lda, A12, lda, A12 + n1, lda))) return rc;
  if ((rc = zgetrf2_sched(ops, m - n1, n2, A12 + n1, lda, ipiv + n1, col0 + n1))) return rc;
  if ((rc = ops.ipiv_add(ipiv + n1, mn - n1, n1))) return rc;
  return ops.laswp(n1, A, lda, n1 + 1, mn, ipiv, 1);
}

// ZGETRF (SRC/zgetrf.f:175-222) with block size nb.
template <class Ops>
int zgetrf_sched(Ops& ops, int m, int n, zdc* A, int lda, int* ipiv, int nb) {
  if (m == 0 || n == 0) return 0;
  const int mn = m < n ? m : n;
  if (nb <= 1 || nb >= mn) return zgetrf2_sched(ops, m, n, A, lda, ipiv, 0);
  int rc;
  for (int j = 0; j < mn; j += nb) {
    const int jb = mn - j < nb ? mn - j : nb;
    zdc* Ajj = A + j + (size_t)j * lda;
    if ((rc = zgetrf2_sched(ops, m - j, jb, Ajj, lda, ipiv + j, j))) return rc;
    if ((rc = ops.ipiv_add(ipiv + j, (m < j + jb ? m : j + jb) - j, j))) return rc;
    if ((rc = ops.laswp(j, A, lda, j + 1, j + jb, ipiv, 1))) return rc;
    if (j + jb < n) {
      zdc* right = A + (size_t)(j + jb) * lda;
      if ((rc = ops.laswp(n - j - jb, right, lda, j + 1, j + jb, ipiv, 1))) return rc;
      if ((rc = ops.trsm(0, 0, 1, jb, n - j - jb, Ajj, lda, right + j, lda))) return rc;
      if (j + jb < m && (rc = ops.gemm(m - j - jb, n - j - jb, jb, Ajj + jb, lda, right + j, lda, right + j + jb, lda)))
        return rc;
    }
  }
  return 0;
}

// ZGETRS (SRC/zgetrs.f:207-220); trans 0 = 'N', 1 = 'T', 2 = 'C'.
template <class Ops>
int zgetrs_sched(Ops& ops, int trans, int n, int nrhs, const zdc* A, int lda, const int* ipiv, zdc* B, int ldb) {
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

}  // namespace gb
