/*
 * ORACLE -- test infrastructure, not product code.
 *
 * A plain-C restatement of the reference LAPACK 3.12.1 routines on the dense
 * LU solve path (DGETRF/DGETRF2/DLASWP/DGETRS/DGESV, their single-precision
 * twins, DSGESV with DLAG2S/SLAG2D/DLANGE/DLACPY) and of the reference BLAS
 * they call (xGEMM, xTRSM, IxAMAX, xSCAL, xAXPY), plus the seeded generator
 * DLARUV/DLARNV used to build test matrices.  Only the tests, the smoke check
 * and the CPU-baseline leg of the benchmark load this library, and only to
 * check or time against; the GPU library never links it.
 *
 * Build with -O2 -ffp-contract=off (gfortran on x86 does not contract a*b+c
 * into an FMA; aarch64 gcc does unless told not to).  The optional OpenMP
 * split is over independent columns only, so results are bit-identical with
 * and without it.
 *
 * Parity pins: no golden output vectors exist in the reference.  The oracle
 * is pinned by (1) the DLARUV multiplier table read from the reference's own
 * SRC/dlaruv.f (tests/golden), (2) the reference LAPACKE C wrappers compiled
 * from the reference sources over this oracle's Fortran-ABI shim and checked
 * case by case, and (3) the reference test-suite ratios (DGET01/02/04/08,
 * TESTING/LIN) restated in oracle/checks.py, all passing under THRESH=30.
 */
#include <math.h>
#include <float.h>
#include <stdio.h>
#include <stdint.h>
#include <string.h>

/* ---- XERBLA: SRC/xerbla.f:67-95 prints and STOPs.  Like the test-suite
 * XERBLA (TESTING/LIN/xerbla.f:74-130) the oracle records the call instead
 * so that error-exit tests can inspect it. */
static char or_xerbla_name[16];
static int or_xerbla_info = 0;
static int or_xerbla_count = 0;
void or_xerbla(const char *name, int info) {
  snprintf(or_xerbla_name, sizeof or_xerbla_name, "%s", name);
  or_xerbla_info = info;
  or_xerbla_count++;
}
int or_xerbla_last(char *name_out, int cap) {
  if (name_out && cap > 0) snprintf(name_out, (size_t)cap, "%s", or_xerbla_name);
  return or_xerbla_info;
}
int or_xerbla_calls(void) { return or_xerbla_count; }
void or_xerbla_reset(void) { or_xerbla_count = 0; or_xerbla_info = 0; or_xerbla_name[0] = 0; }

/* ---- DLAMCH/SLAMCH (INSTALL/dlamch.f:101-141): eps is EPSILON*0.5 for a
 * rounding arithmetic, sfmin is TINY (1/HUGE is smaller), 'O' is HUGE. */
double or_dlamch(char c) {
  switch (c) {
    case 'E': case 'e': return DBL_EPSILON * 0.5;
    case 'S': case 's': return DBL_MIN;
    case 'O': case 'o': return DBL_MAX;
    case 'P': case 'p': return DBL_EPSILON;
    case 'B': case 'b': return 2.0;
    case 'U': case 'u': return DBL_MIN;
    default: return 0.0;
  }
}
float or_slamch(char c) {
  switch (c) {
    case 'E': case 'e': return FLT_EPSILON * 0.5f;
    case 'S': case 's': return FLT_MIN;
    case 'O': case 'o': return FLT_MAX;
    case 'P': case 'p': return FLT_EPSILON;
    case 'B': case 'b': return 2.0f;
    case 'U': case 'u': return FLT_MIN;
    default: return 0.0f;
  }
}

#define T double
#define P d
#define PNAME "D"
#define ABS_T fabs
#define SFMIN_T DBL_MIN
#include "oracle_lu.inc"
#include "oracle_chol.inc"
#undef T
#undef P
#undef PNAME
#undef ABS_T
#undef SFMIN_T

#define T float
#define P s
#define PNAME "S"
#define ABS_T fabsf
#define SFMIN_T FLT_MIN
#include "oracle_lu.inc"
#include "oracle_chol.inc"
#undef T
#undef P
#undef PNAME
#undef ABS_T
#undef SFMIN_T

/* Complex LU: COMPLEX*16 (or_z...) and COMPLEX (or_c...) from one source. */
#define ZT double
#define ZC zcd
#define ZH(x) zcd_##x
#define ZFN(x) or_z##x
#define ZNAME "Z"
#define ZABS fabs
#define ZHYPOT hypot
#define ZHUGE DBL_MAX
#define ZSFMIN DBL_MIN
#include "oracle_z.inc"
#undef ZT
#undef ZC
#undef ZH
#undef ZFN
#undef ZNAME
#undef ZABS
#undef ZHYPOT
#undef ZHUGE
#undef ZSFMIN
#define ZT float
#define ZC zcf
#define ZH(x) zcf_##x
#define ZFN(x) or_c##x
#define ZNAME "C"
#define ZABS fabsf
#define ZHYPOT hypotf
#define ZHUGE FLT_MAX
#define ZSFMIN FLT_MIN
#include "oracle_z.inc"
#undef ZT
#undef ZC
#undef ZH
#undef ZFN
#undef ZNAME
#undef ZABS
#undef ZHYPOT
#undef ZHUGE
#undef ZSFMIN

/* ---- ZCGESV (SRC/zcgesv.f:259-448): COMPLEX factorization and solves,
 * COMPLEX*16 residual, convergence test and update, ITERMAX = 30,
 * BWDMAX = 1, the ZGETRF / ZGETRS fallback. */

/* ZLAG2C (SRC/zlag2c.f:134-153): INFO = 1 at the first part outside
 * [-RMAX, RMAX] (RMAX = SLAMCH('O')), in column order, stopping there; a
 * NaN passes and converts to NaN. */
void or_zlag2c(int m, int n, const zcd *a, int lda, zcf *sa, int ldsa, int *info) {
  const double rmax = FLT_MAX;
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < m; ++i) {
      const zcd v = a[(size_t)i + (size_t)j * lda];
      if (v.re < -rmax || v.re > rmax || v.im < -rmax || v.im > rmax) { *info = 1; return; }
      sa[(size_t)i + (size_t)j * ldsa].re = (float)v.re;
      sa[(size_t)i + (size_t)j * ldsa].im = (float)v.im;
    }
  *info = 0;
}

/* CLAG2Z (SRC/clag2z.f:120-132): exact widening. */
void or_clag2z(int m, int n, const zcf *sa, int ldsa, zcd *a, int lda, int *info) {
  *info = 0;
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < m; ++i) {
      a[(size_t)i + (size_t)j * lda].re = sa[(size_t)i + (size_t)j * ldsa].re;
      a[(size_t)i + (size_t)j * lda].im = sa[(size_t)i + (size_t)j * ldsa].im;
    }
}

/* ZLANGE('I') (SRC/zlange.f:175-190): row sums of moduli accumulated column
 * by column, the maximum taken with NaN propagation. */
double or_zlange_inf(int m, int n, const zcd *a, int lda, double *work) {
  for (int i = 0; i < m; ++i) work[i] = 0.0;
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < m; ++i) work[i] = work[i] + hypot(a[(size_t)i + (size_t)j * lda].re, a[(size_t)i + (size_t)j * lda].im);
  double value = 0.0;
  for (int i = 0; i < m; ++i)
    if (value < work[i] || work[i] != work[i]) value = work[i];
  return value;
}

static double zcd_cabs1(zcd z) { return fabs(z.re) + fabs(z.im); }

/* Convergence test of SRC/zcgesv.f:350-357: 1 when some column has
 * CABS1(R(IZAMAX(R))) > CABS1(X(IZAMAX(X)))*CTE. */
static int zcgesv_notconv(int n, int nrhs, const zcd *x, int ldx, const zcd *r, int ldr, double cte) {
  for (int j = 0; j < nrhs; ++j) {
    const zcd *xc = x + (size_t)j * ldx, *rc = r + (size_t)j * ldr;
    const double xnrm = zcd_cabs1(xc[or_ziamax(n, xc) - 1]);
    const double rnrm = zcd_cabs1(rc[or_ziamax(n, rc) - 1]);
    if (rnrm > xnrm * cte) return 1;
  }
  return 0;
}

void or_zcgesv(int n, int nrhs, zcd *a, int lda, int *ipiv, const zcd *b, int ldb, zcd *x, int ldx, zcd *work,
               zcf *swork, double *rwork, int *iter, int *info) {
  const int itermax = 30;
  const double bwdmax = 1.0;
  const zcd one = {1.0, 0.0}, negone = {-1.0, 0.0};
  *info = 0;
  *iter = 0;
  if (n < 0) *info = -1;
  else if (nrhs < 0) *info = -2;
  else if (lda < (n > 1 ? n : 1)) *info = -4;
  else if (ldb < (n > 1 ? n : 1)) *info = -7;
  else if (ldx < (n > 1 ? n : 1)) *info = -9;
  if (*info != 0) { or_xerbla("ZCGESV", -*info); return; }
  if (n == 0) return;
  const double anrm = or_zlange_inf(n, n, a, lda, rwork);
  const double eps = DBL_EPSILON * 0.5;
  const double cte = anrm * eps * sqrt((double)n) * bwdmax;
  zcf *sa = swork, *sx = swork + (size_t)n * n;
  int inf2;
  or_zlag2c(n, nrhs, b, ldb, sx, n, &inf2);
  if (inf2 != 0) { *iter = -2; goto fallback; }
  or_zlag2c(n, n, a, lda, sa, n, &inf2);
  if (inf2 != 0) { *iter = -2; goto fallback; }
  or_cgetrf(n, n, sa, n, ipiv, &inf2);
  if (inf2 != 0) { *iter = -3; goto fallback; }
  or_cgetrs('N', n, nrhs, sa, n, ipiv, sx, n, &inf2);
  or_clag2z(n, nrhs, sx, n, x, ldx, &inf2);
  for (int j = 0; j < nrhs; ++j)
    for (int i = 0; i < n; ++i) work[(size_t)i + (size_t)j * n] = b[(size_t)i + (size_t)j * ldb];
  or_zgemm_nn(n, nrhs, n, negone, a, lda, x, ldx, work, n);
  if (!zcgesv_notconv(n, nrhs, x, ldx, work, n, cte)) { *iter = 0; return; }
  for (int it = 1; it <= itermax; ++it) {
    or_zlag2c(n, nrhs, work, n, sx, n, &inf2);
    if (inf2 != 0) { *iter = -2; goto fallback; }
    or_cgetrs('N', n, nrhs, sa, n, ipiv, sx, n, &inf2);
    or_clag2z(n, nrhs, sx, n, work, n, &inf2);
    for (int j = 0; j < nrhs; ++j)   /* ZAXPY (BLAS/SRC/zaxpy.f:114-122) with ZA = ONE */
      for (int i = 0; i < n; ++i) {
        zcd *y = &x[(size_t)i + (size_t)j * ldx];
        *y = zcd_add(*y, zcd_mul(one, work[(size_t)i + (size_t)j * n]));
      }
    for (int j = 0; j < nrhs; ++j)
      for (int i = 0; i < n; ++i) work[(size_t)i + (size_t)j * n] = b[(size_t)i + (size_t)j * ldb];
    or_zgemm_nn(n, nrhs, n, negone, a, lda, x, ldx, work, n);
    if (!zcgesv_notconv(n, nrhs, x, ldx, work, n, cte)) { *iter = it; return; }
  }
  *iter = -itermax - 1;
fallback:
  or_zgetrf(n, n, a, lda, ipiv, info);
  if (*info != 0) return;
  for (int j = 0; j < nrhs; ++j)
    for (int i = 0; i < n; ++i) x[(size_t)i + (size_t)j * ldx] = b[(size_t)i + (size_t)j * ldb];
  or_zgetrs('N', n, nrhs, a, lda, ipiv, x, ldx, info);
}

/* ---- DLAG2S: SRC/dlag2s.f:135-146.  INFO=1 (and stop converting) at the
 * first |a| > SLAMCH('O'); a NaN passes the test and converts to NaN. */
void or_dlag2s(int m, int n, const double *a, int lda, float *sa, int ldsa, int *info) {
  double rmax = (double)FLT_MAX;
  for (int j = 0; j < n; j++)
    for (int i = 0; i < m; i++) {
      double v = a[(size_t)i + (size_t)j * lda];
      if (v < -rmax || v > rmax) { *info = 1; return; }
      sa[(size_t)i + (size_t)j * ldsa] = (float)v;
    }
  *info = 0;
}

/* ---- SLAG2D: SRC/slag2d.f:123-128. */
void or_slag2d(int m, int n, const float *sa, int ldsa, double *a, int lda, int *info) {
  *info = 0;
  for (int j = 0; j < n; j++)
    for (int i = 0; i < m; i++) a[(size_t)i + (size_t)j * lda] = (double)sa[(size_t)i + (size_t)j * ldsa];
}

/* ---- DSGESV: SRC/dsgesv.f:243-429.  FP32 LU (SGETRF, NB=64) plus FP64
 * iterative refinement; ITERMAX=30, BWDMAX=1, CTE=||A||_inf*eps*sqrt(n).
 * Falls back to FP64 DGETRF/DGETRS with ITER<0 exactly as the reference. */
void or_dsgesv(int n, int nrhs, double *a, int lda, int *ipiv, const double *b, int ldb,
               double *x, int ldx, double *work, float *swork, int *iter, int *info) {
  const int itermax = 30;
  const double bwdmax = 1.0;
  *info = 0;
  *iter = 0;
  if (n < 0) *info = -1;
  else if (nrhs < 0) *info = -2;
  else if (lda < (n > 1 ? n : 1)) *info = -4;
  else if (ldb < (n > 1 ? n : 1)) *info = -7;
  else if (ldx < (n > 1 ? n : 1)) *info = -9;
  if (*info != 0) { or_xerbla("DSGESV", -*info); return; }
  if (n == 0) return;
  double anrm = or_dlange('I', n, n, a, lda, work);
  double eps = or_dlamch('E');
  double cte = anrm * eps * sqrt((double)n) * bwdmax;
  float *sa = swork;
  float *sx = swork + (size_t)n * n;
  or_dlag2s(n, nrhs, b, ldb, sx, n, info);
  if (*info != 0) { *iter = -2; goto fallback; }
  or_dlag2s(n, n, a, lda, sa, n, info);
  if (*info != 0) { *iter = -2; goto fallback; }
  or_sgetrf(n, n, sa, n, ipiv, info);
  if (*info != 0) { *iter = -3; goto fallback; }
  or_sgetrs('N', n, nrhs, sa, n, ipiv, sx, n, info);
  or_slag2d(n, nrhs, sx, n, x, ldx, info);
  or_dlacpy(n, nrhs, b, ldb, work, n);
  or_dgemm('N', 'N', n, nrhs, n, -1.0, a, lda, x, ldx, 1.0, work, n);
  {
    int conv = 1;
    for (int i = 0; i < nrhs; i++) {
      double xnrm = fabs(x[(size_t)(or_diamax(n, x + (size_t)i * ldx, 1) - 1) + (size_t)i * ldx]);
      double rnrm = fabs(work[(size_t)(or_diamax(n, work + (size_t)i * n, 1) - 1) + (size_t)i * n]);
      if (rnrm > xnrm * cte) { conv = 0; break; }
    }
    if (conv) { *iter = 0; return; }
  }
  for (int iiter = 1; iiter <= itermax; iiter++) {
    or_dlag2s(n, nrhs, work, n, sx, n, info);
    if (*info != 0) { *iter = -2; goto fallback; }
    or_sgetrs('N', n, nrhs, sa, n, ipiv, sx, n, info);
    or_slag2d(n, nrhs, sx, n, work, n, info);
    for (int i = 0; i < nrhs; i++) or_daxpy(n, 1.0, work + (size_t)i * n, 1, x + (size_t)i * ldx, 1);
    or_dlacpy(n, nrhs, b, ldb, work, n);
    or_dgemm('N', 'N', n, nrhs, n, -1.0, a, lda, x, ldx, 1.0, work, n);
    int conv = 1;
    for (int i = 0; i < nrhs; i++) {
      double xnrm = fabs(x[(size_t)(or_diamax(n, x + (size_t)i * ldx, 1) - 1) + (size_t)i * ldx]);
      double rnrm = fabs(work[(size_t)(or_diamax(n, work + (size_t)i * n, 1) - 1) + (size_t)i * n]);
      if (rnrm > xnrm * cte) { conv = 0; break; }
    }
    if (conv) { *iter = iiter; return; }
  }
  *iter = -itermax - 1;
fallback:
  or_dgetrf(n, n, a, lda, ipiv, info);
  if (*info != 0) return;
  or_dlacpy(n, nrhs, b, ldb, x, ldx);
  or_dgetrs('N', n, nrhs, a, lda, ipiv, x, ldx, info);
}

/* ---- DLARUV: SRC/dlaruv.f:92-447.  48-bit multiplicative congruential
 * generator; x_i = seed * a^i mod 2^48 for i = 1..n, the new seed is
 * seed * a^n.  The reference stores a^i (i = 1..128) as a table of 12-bit
 * limbs; here the powers are computed from the base multiplier
 * a = 33952834046453 (the table's first row), and the tests compare them
 * with the table read from the reference source. */
static const uint64_t OR_RUV_A = 33952834046453ULL;
static const uint64_t OR_M48 = (1ULL << 48) - 1;

void or_dlaruv_power(int i, int limbs[4]) {
  uint64_t p = 1;
  for (int k = 0; k < i; k++) p = (p * OR_RUV_A) & OR_M48;   /* products fit: wraps mod 2^64 then masked */
  limbs[0] = (int)((p >> 36) & 4095);
  limbs[1] = (int)((p >> 24) & 4095);
  limbs[2] = (int)((p >> 12) & 4095);
  limbs[3] = (int)(p & 4095);
}

static uint64_t or_seed_pack(const int iseed[4]) {
  return ((uint64_t)iseed[0] << 36) | ((uint64_t)iseed[1] << 24) | ((uint64_t)iseed[2] << 12) | (uint64_t)iseed[3];
}
static void or_seed_unpack(uint64_t s, int iseed[4]) {
  iseed[0] = (int)((s >> 36) & 4095);
  iseed[1] = (int)((s >> 24) & 4095);
  iseed[2] = (int)((s >> 12) & 4095);
  iseed[3] = (int)(s & 4095);
}
/* 48-bit value -> real in (0,1) with the reference's nesting:
 * R*(IT1 + R*(IT2 + R*(IT3 + R*IT4))), R = 1/4096 (every step exact). */
static double or_ruv_real(uint64_t v) {
  const double r = 1.0 / 4096.0;
  double it1 = (double)((v >> 36) & 4095), it2 = (double)((v >> 24) & 4095);
  double it3 = (double)((v >> 12) & 4095), it4 = (double)(v & 4095);
  return r * (it1 + r * (it2 + r * (it3 + r * it4)));
}

void or_dlaruv(int iseed[4], int n, double *x) {
  if (n < 1) return;
  int lv = n < 128 ? n : 128;
  uint64_t s = or_seed_pack(iseed);
  uint64_t pw[129];
  pw[0] = 1;
  for (int k = 1; k <= lv; k++) pw[k] = (pw[k - 1] * OR_RUV_A) & OR_M48;
  uint64_t it = s;
  for (int i = 1; i <= lv; i++) {
    for (;;) {
      it = (s * pw[i]) & OR_M48;
      x[i - 1] = or_ruv_real(it);
      if (x[i - 1] != 1.0) break;
      s = it;                             /* dlaruv.f:424-433: iterate again */
    }
  }
  or_seed_unpack(it, iseed);
}

/* ---- DGEMV with alpha = -1, beta = 1, as DGERFS calls it
 * (BLAS/SRC/dgemv.f:256-276 for 'N': y += (-x(j)) * A(:,j) column by column;
 * :292-311 for 'T': y(j) += -1 * (sum_i A(i,j) x(i))). */
static void or_dgemv_m1(char trans, int n, const double *a, int lda, const double *x, double *y) {
  if (trans == 'N' || trans == 'n') {
    for (int j = 0; j < n; j++) {
      const double temp = -x[j];
      for (int i = 0; i < n; i++) y[i] = y[i] + temp * a[i + (size_t)j * lda];
    }
  } else {
    for (int j = 0; j < n; j++) {
      double temp = 0.0;
      for (int i = 0; i < n; i++) temp = temp + a[i + (size_t)j * lda] * x[i];
      y[j] = y[j] + (-1.0) * temp;
    }
  }
}

static double or_dasum(int n, const double *x) {
  double s = 0.0;
  for (int i = 0; i < n; i++) s = s + fabs(x[i]);
  return s;
}

/* ---- DLACN2: SRC/dlacn2.f:134-263 (Hager / Higham 1-norm estimator,
 * reverse communication: KASE 1 asks for x := A x, KASE 2 for x := A^T x). */
void or_dlacn2(int n, double *v, double *x, int *isgn, double *est, int *kase, int isave[3]) {
  const int itmax = 5;
  if (*kase == 0) {
    for (int i = 0; i < n; i++) x[i] = 1.0 / (double)n;
    *kase = 1;
    isave[0] = 1;
    return;
  }
  switch (isave[0]) {
    case 1: {
      if (n == 1) {
        v[0] = x[0];
        *est = fabs(v[0]);
        *kase = 0;
        return;
      }
      *est = or_dasum(n, x);
      for (int i = 0; i < n; i++) {
        x[i] = (x[i] >= 0.0) ? 1.0 : -1.0;
        isgn[i] = (int)lrint(x[i]);
      }
      *kase = 2;
      isave[0] = 2;
      return;
    }
    case 2:
      isave[1] = or_diamax(n, x, 1);
      isave[2] = 2;
      goto L50;
    case 3: {
      for (int i = 0; i < n; i++) v[i] = x[i];
      const double estold = *est;
      *est = or_dasum(n, v);
      int changed = 0;
      for (int i = 0; i < n; i++) {
        const double xs = (x[i] >= 0.0) ? 1.0 : -1.0;
        if ((int)lrint(xs) != isgn[i]) { changed = 1; break; }
      }
      if (!changed || *est <= estold) goto L120;
      for (int i = 0; i < n; i++) {
        x[i] = (x[i] >= 0.0) ? 1.0 : -1.0;
        isgn[i] = (int)lrint(x[i]);
      }
      *kase = 2;
      isave[0] = 4;
      return;
    }
    case 4: {
      const int jlast = isave[1];
      isave[1] = or_diamax(n, x, 1);
      if (x[jlast - 1] != fabs(x[isave[1] - 1]) && isave[2] < itmax) {
        isave[2] = isave[2] + 1;
        goto L50;
      }
      goto L120;
    }
    case 5: {
      const double temp = 2.0 * (or_dasum(n, x) / (double)(3 * n));
      if (temp > *est) {
        for (int i = 0; i < n; i++) v[i] = x[i];
        *est = temp;
      }
      *kase = 0;
      return;
    }
  }
  return;
L50:
  for (int i = 0; i < n; i++) x[i] = 0.0;
  x[isave[1] - 1] = 1.0;
  *kase = 1;
  isave[0] = 3;
  return;
L120: {
    double altsgn = 1.0;
    for (int i = 0; i < n; i++) {
      x[i] = altsgn * (1.0 + (double)i / (double)(n - 1));
      altsgn = -altsgn;
    }
    *kase = 1;
    isave[0] = 5;
    return;
  }
}

/* ---- DGERFS: SRC/dgerfs.f:186-424.  Iterative refinement of X with the
 * factors AF/IPIV (ITMAX = 5), componentwise backward error BERR and the
 * DLACN2 estimate of the forward error bound FERR.  work: 3n doubles, iwork:
 * n ints. */
void or_dgerfs(char trans, int n, int nrhs, const double *a, int lda, const double *af, int ldaf, const int *ipiv,
               const double *b, int ldb, double *x, int ldx, double *ferr, double *berr, double *work, int *iwork,
               int *info) {
  const int itmax = 5;
  *info = 0;
  const int notran = (trans == 'N' || trans == 'n');
  if (!notran && trans != 'T' && trans != 't' && trans != 'C' && trans != 'c') *info = -1;
  else if (n < 0) *info = -2;
  else if (nrhs < 0) *info = -3;
  else if (lda < (n > 1 ? n : 1)) *info = -5;
  else if (ldaf < (n > 1 ? n : 1)) *info = -7;
  else if (ldb < (n > 1 ? n : 1)) *info = -10;
  else if (ldx < (n > 1 ? n : 1)) *info = -12;
  if (*info != 0) { or_xerbla("DGERFS", -*info); return; }
  if (n == 0 || nrhs == 0) {
    for (int j = 0; j < nrhs; j++) { ferr[j] = 0.0; berr[j] = 0.0; }
    return;
  }
  const char transt = notran ? 'T' : 'N';
  const int nz = n + 1;
  const double eps = or_dlamch('E'), safmin = or_dlamch('S');
  const double safe1 = nz * safmin, safe2 = safe1 / eps;
  double *w = work, *r = work + n, *v = work + 2 * n;
  for (int j = 0; j < nrhs; j++) {
    const double *bj = b + (size_t)j * ldb;
    double *xj = x + (size_t)j * ldx;
    int count = 1;
    double lstres = 3.0;
    for (;;) {
      for (int i = 0; i < n; i++) r[i] = bj[i];
      or_dgemv_m1(notran ? 'N' : 'T', n, a, lda, xj, r);
      for (int i = 0; i < n; i++) w[i] = fabs(bj[i]);
      if (notran) {
        for (int k = 0; k < n; k++) {
          const double xk = fabs(xj[k]);
          for (int i = 0; i < n; i++) w[i] = w[i] + fabs(a[i + (size_t)k * lda]) * xk;
        }
      } else {
        for (int k = 0; k < n; k++) {
          double s = 0.0;
          for (int i = 0; i < n; i++) s = s + fabs(a[i + (size_t)k * lda]) * fabs(xj[i]);
          w[k] = w[k] + s;
        }
      }
      double s = 0.0;
      for (int i = 0; i < n; i++) {
        const double q = (w[i] > safe2) ? fabs(r[i]) / w[i] : (fabs(r[i]) + safe1) / (w[i] + safe1);
        s = (q > s) ? q : s;
      }
      berr[j] = s;
      if (berr[j] > eps && 2.0 * berr[j] <= lstres && count <= itmax) {
        int inf2 = 0;
        or_dgetrs(trans, n, 1, af, ldaf, ipiv, r, n, &inf2);
        for (int i = 0; i < n; i++) xj[i] = xj[i] + 1.0 * r[i];
        lstres = berr[j];
        count++;
        continue;
      }
      break;
    }
    for (int i = 0; i < n; i++)
      w[i] = (w[i] > safe2) ? fabs(r[i]) + nz * eps * w[i] : fabs(r[i]) + nz * eps * w[i] + safe1;
    int kase = 0, isave[3] = {0, 0, 0};
    for (;;) {
      or_dlacn2(n, v, r, iwork, &ferr[j], &kase, isave);
      if (kase == 0) break;
      int inf2 = 0;
      if (kase == 1) {
        or_dgetrs(transt, n, 1, af, ldaf, ipiv, r, n, &inf2);
        for (int i = 0; i < n; i++) r[i] = w[i] * r[i];
      } else {
        for (int i = 0; i < n; i++) r[i] = w[i] * r[i];
        or_dgetrs(trans, n, 1, af, ldaf, ipiv, r, n, &inf2);
      }
    }
    lstres = 0.0;
    for (int i = 0; i < n; i++) lstres = (fabs(xj[i]) > lstres) ? fabs(xj[i]) : lstres;
    if (lstres != 0.0) ferr[j] = ferr[j] / lstres;
  }
}

/* ---- DDOT: BLAS/SRC/ddot.f:82-112 (incx = incy = 1): one running sum in
 * index order (the unrolled loop adds left to right). */
static double or_ddot(int n, const double *x, const double *y) {
  double s = 0.0;
  for (int i = 0; i < n; i++) s = s + x[i] * y[i];
  return s;
}

/* ---- DTRSV, INCX = 1: BLAS/SRC/dtrsv.f:219-320.  'N': column sweeps
 * X(i) -= X(j)*A(i,j); 'T' upper: dot products over i = 1..j-1 in increasing
 * order; 'T' lower: over i = N..j+1 in decreasing order. */
void or_dtrsv(char uplo, char trans, char diag, int n, const double *a, int lda, double *x) {
  const int upper = (uplo == 'U' || uplo == 'u');
  const int notr = (trans == 'N' || trans == 'n');
  const int nounit = (diag == 'N' || diag == 'n');
  if (n == 0) return;
#define A_(i, j) a[(size_t)(i) + (size_t)(j) * lda]
  if (notr) {
    if (upper) {
      for (int j = n - 1; j >= 0; j--) {
        if (nounit) x[j] = x[j] / A_(j, j);
        const double temp = x[j];
        for (int i = j - 1; i >= 0; i--) x[i] = x[i] - temp * A_(i, j);
      }
    } else {
      for (int j = 0; j < n; j++) {
        if (nounit) x[j] = x[j] / A_(j, j);
        const double temp = x[j];
        for (int i = j + 1; i < n; i++) x[i] = x[i] - temp * A_(i, j);
      }
    }
  } else {
    if (upper) {
      for (int j = 0; j < n; j++) {
        double temp = x[j];
        for (int i = 0; i < j; i++) temp = temp - A_(i, j) * x[i];
        if (nounit) temp = temp / A_(j, j);
        x[j] = temp;
      }
    } else {
      for (int j = n - 1; j >= 0; j--) {
        double temp = x[j];
        for (int i = n - 1; i > j; i--) temp = temp - A_(i, j) * x[i];
        if (nounit) temp = temp / A_(j, j);
        x[j] = temp;
      }
    }
  }
#undef A_
}

/* ---- DRSCL: SRC/drscl.f:105-133.  X := X / SA in steps of SMLNUM or
 * BIGNUM so that no intermediate overflows or underflows. */
void or_drscl(int n, double sa, double *x) {
  if (n <= 0) return;
  const double smlnum = or_dlamch('S'), bignum = 1.0 / smlnum;
  double cden = sa, cnum = 1.0;
  for (;;) {
    const double cden1 = cden * smlnum, cnum1 = cnum / bignum;
    double mul;
    int done;
    if (fabs(cden1) > fabs(cnum) && cnum != 0.0) {
      mul = smlnum;
      done = 0;
      cden = cden1;
    } else if (fabs(cnum1) > fabs(cden)) {
      mul = bignum;
      done = 0;
      cnum = cnum1;
    } else {
      mul = cnum / cden;
      done = 1;
    }
    or_dscal(n, mul, x, 1);
    if (done) break;
  }
}

/* ---- DLATRS: SRC/dlatrs.f:264-847.  Triangular solve op(A) x = s*b with
 * a scale factor s <= 1 chosen so that no intermediate result overflows:
 * column norms CNORM of the off-diagonal part, a growth bound, then DTRSV
 * when the bound allows it, else the careful column-by-column solve.
 * MIN / MAX are fmin / fmax. */
void or_dlatrs(char uplo, char trans, char diag, char normin, int n, const double *a, int lda, double *x,
               double *scale, double *cnorm, int *info) {
  const int upper = (uplo == 'U' || uplo == 'u');
  const int notran = (trans == 'N' || trans == 'n');
  const int nounit = (diag == 'N' || diag == 'n');
  *info = 0;
  if (!upper && uplo != 'L' && uplo != 'l') *info = -1;
  else if (!notran && trans != 'T' && trans != 't' && trans != 'C' && trans != 'c') *info = -2;
  else if (!nounit && diag != 'U' && diag != 'u') *info = -3;
  else if (normin != 'Y' && normin != 'y' && normin != 'N' && normin != 'n') *info = -4;
  else if (n < 0) *info = -5;
  else if (lda < (n > 1 ? n : 1)) *info = -7;
  if (*info != 0) { or_xerbla("DLATRS", -*info); return; }
  *scale = 1.0;
  if (n == 0) return;
#define A_(i, j) a[(size_t)(i) + (size_t)(j) * lda]
  const double smlnum = or_dlamch('S') / or_dlamch('P');
  const double bignum = 1.0 / smlnum;
  const double ovfl = or_dlamch('O');
  if (normin == 'N' || normin == 'n') {                       /* dlatrs.f:322-338 */
    if (upper) {
      for (int j = 0; j < n; j++) cnorm[j] = or_dasum(j, &A_(0, j));
    } else {
      for (int j = 0; j < n - 1; j++) cnorm[j] = or_dasum(n - j - 1, &A_(j + 1, j));
      cnorm[n - 1] = 0.0;
    }
  }
  int imax = or_diamax(n, cnorm, 1);                          /* dlatrs.f:343-397 */
  double tmax = cnorm[imax - 1];
  double tscal;
  if (tmax <= bignum) {
    tscal = 1.0;
  } else if (tmax <= ovfl) {
    tscal = 1.0 / (smlnum * tmax);
    or_dscal(n, tscal, cnorm, 1);
  } else {
    tmax = 0.0;
    for (int j = 0; j < n; j++) {
      const int i0 = upper ? 0 : j + 1, i1 = upper ? j : n;   /* the off-diagonal part of column j */
      double m = 0.0;
      for (int i = i0; i < i1; i++) {
        const double t = fabs(A_(i, j));
        if (m < t || isnan(t)) m = t;
      }
      if (i1 > i0) tmax = fmax(m, tmax);
    }
    if (tmax <= ovfl) {
      tscal = 1.0 / (smlnum * tmax);
      for (int j = 0; j < n; j++) {
        if (cnorm[j] <= ovfl) {
          cnorm[j] = cnorm[j] * tscal;
        } else {
          cnorm[j] = 0.0;
          const int i0 = upper ? 0 : j + 1, i1 = upper ? j : n;
          for (int i = i0; i < i1; i++) cnorm[j] = cnorm[j] + tscal * fabs(A_(i, j));
        }
      }
    } else {
      or_dtrsv(uplo, trans, diag, n, a, lda, x);
      return;
    }
  }
  int jx = or_diamax(n, x, 1);                                /* dlatrs.f:401-497 */
  double xmax = fabs(x[jx - 1]);
  double xbnd = xmax, grow;
  int jfirst, jlast, jinc;
  if (notran) {
    if (upper) { jfirst = n - 1; jlast = 0; jinc = -1; }
    else { jfirst = 0; jlast = n - 1; jinc = 1; }
  } else {
    if (upper) { jfirst = 0; jlast = n - 1; jinc = 1; }
    else { jfirst = n - 1; jlast = 0; jinc = -1; }
  }
  if (tscal != 1.0) {
    grow = 0.0;
  } else if (notran) {
    if (nounit) {
      grow = 1.0 / fmax(xbnd, smlnum);
      xbnd = grow;
      int cut = 0;
      for (int j = jfirst; j != jlast + jinc; j += jinc) {
        if (grow <= smlnum) { cut = 1; break; }
        const double tjj = fabs(A_(j, j));
        xbnd = fmin(xbnd, fmin(1.0, tjj) * grow);
        if (tjj + cnorm[j] >= smlnum) grow = grow * (tjj / (tjj + cnorm[j]));
        else grow = 0.0;
      }
      if (!cut) grow = xbnd;
    } else {
      grow = fmin(1.0, 1.0 / fmax(xbnd, smlnum));
      for (int j = jfirst; j != jlast + jinc; j += jinc) {
        if (grow <= smlnum) break;
        grow = grow * (1.0 / (1.0 + cnorm[j]));
      }
    }
  } else {
    if (nounit) {
      grow = 1.0 / fmax(xbnd, smlnum);
      xbnd = grow;
      int cut = 0;
      for (int j = jfirst; j != jlast + jinc; j += jinc) {
        if (grow <= smlnum) { cut = 1; break; }
        const double xj = 1.0 + cnorm[j];
        grow = fmin(grow, xbnd / xj);
        const double tjj = fabs(A_(j, j));
        if (xj > tjj) xbnd = xbnd * (tjj / xj);
      }
      if (!cut) grow = fmin(grow, xbnd);
    } else {
      grow = fmin(1.0, 1.0 / fmax(xbnd, smlnum));
      for (int j = jfirst; j != jlast + jinc; j += jinc) {
        if (grow <= smlnum) break;
        const double xj = 1.0 + cnorm[j];
        grow = grow / xj;
      }
    }
  }
  if (grow * tscal > smlnum) {                                /* dlatrs.f:499-503 */
    or_dtrsv(uplo, trans, diag, n, a, lda, x);
  } else {
    if (xmax > bignum) {                                      /* dlatrs.f:509-516 */
      *scale = bignum / xmax;
      or_dscal(n, *scale, x, 1);
      xmax = bignum;
    }
    if (notran) {                                             /* dlatrs.f:518-640 */
      for (int j = jfirst; j != jlast + jinc; j += jinc) {
        double xj = fabs(x[j]), tjjs, rec;
        int skip = 0;
        if (nounit) {
          tjjs = A_(j, j) * tscal;
        } else {
          tjjs = tscal;
          if (tscal == 1.0) skip = 1;
        }
        if (!skip) {
          const double tjj = fabs(tjjs);
          if (tjj > smlnum) {
            if (tjj < 1.0 && xj > tjj * bignum) {
              rec = 1.0 / xj;
              or_dscal(n, rec, x, 1);
              *scale = *scale * rec;
              xmax = xmax * rec;
            }
            x[j] = x[j] / tjjs;
            xj = fabs(x[j]);
          } else if (tjj > 0.0) {
            if (xj > tjj * bignum) {
              rec = (tjj * bignum) / xj;
              if (cnorm[j] > 1.0) rec = rec / cnorm[j];
              or_dscal(n, rec, x, 1);
              *scale = *scale * rec;
              xmax = xmax * rec;
            }
            x[j] = x[j] / tjjs;
            xj = fabs(x[j]);
          } else {
            for (int i = 0; i < n; i++) x[i] = 0.0;
            x[j] = 1.0;
            xj = 1.0;
            *scale = 0.0;
            xmax = 0.0;
          }
        }
        if (xj > 1.0) {
          rec = 1.0 / xj;
          if (cnorm[j] > (bignum - xmax) * rec) {
            rec = rec * 0.5;
            or_dscal(n, rec, x, 1);
            *scale = *scale * rec;
          }
        } else if (xj * cnorm[j] > (bignum - xmax)) {
          or_dscal(n, 0.5, x, 1);
          *scale = *scale * 0.5;
        }
        if (upper) {
          if (j > 0) {
            or_daxpy(j, -x[j] * tscal, &A_(0, j), 1, x, 1);
            const int i = or_diamax(j, x, 1);
            xmax = fabs(x[i - 1]);
          }
        } else if (j < n - 1) {
          or_daxpy(n - j - 1, -x[j] * tscal, &A_(j + 1, j), 1, x + j + 1, 1);
          const int i = j + or_diamax(n - j - 1, x + j + 1, 1);
          xmax = fabs(x[i]);
        }
      }
    } else {                                                  /* dlatrs.f:642-764 */
      for (int j = jfirst; j != jlast + jinc; j += jinc) {
        double xj = fabs(x[j]), uscal = tscal, tjjs = 0.0, tjj;
        double rec = 1.0 / fmax(xmax, 1.0);
        if (cnorm[j] > (bignum - xj) * rec) {
          rec = rec * 0.5;
          tjjs = nounit ? A_(j, j) * tscal : tscal;
          tjj = fabs(tjjs);
          if (tjj > 1.0) {
            rec = fmin(1.0, rec * tjj);
            uscal = uscal / tjjs;
          }
          if (rec < 1.0) {
            or_dscal(n, rec, x, 1);
            *scale = *scale * rec;
            xmax = xmax * rec;
          }
        }
        double sumj = 0.0;
        if (uscal == 1.0) {
          if (upper) sumj = or_ddot(j, &A_(0, j), x);
          else if (j < n - 1) sumj = or_ddot(n - j - 1, &A_(j + 1, j), x + j + 1);
        } else {
          if (upper) {
            for (int i = 0; i < j; i++) sumj = sumj + (A_(i, j) * uscal) * x[i];
          } else if (j < n - 1) {
            for (int i = j + 1; i < n; i++) sumj = sumj + (A_(i, j) * uscal) * x[i];
          }
        }
        if (uscal == tscal) {
          x[j] = x[j] - sumj;
          xj = fabs(x[j]);
          int skip = 0;
          if (nounit) {
            tjjs = A_(j, j) * tscal;
          } else {
            tjjs = tscal;
            if (tscal == 1.0) skip = 1;
          }
          if (!skip) {
            tjj = fabs(tjjs);
            if (tjj > smlnum) {
              if (tjj < 1.0 && xj > tjj * bignum) {
                rec = 1.0 / xj;
                or_dscal(n, rec, x, 1);
                *scale = *scale * rec;
                xmax = xmax * rec;
              }
              x[j] = x[j] / tjjs;
            } else if (tjj > 0.0) {
              if (xj > tjj * bignum) {
                rec = (tjj * bignum) / xj;
                or_dscal(n, rec, x, 1);
                *scale = *scale * rec;
                xmax = xmax * rec;
              }
              x[j] = x[j] / tjjs;
            } else {
              for (int i = 0; i < n; i++) x[i] = 0.0;
              x[j] = 1.0;
              *scale = 0.0;
              xmax = 0.0;
            }
          }
        } else {
          x[j] = x[j] / tjjs - sumj;
        }
        xmax = fmax(xmax, fabs(x[j]));
      }
    }
    *scale = *scale / tscal;
  }
  if (tscal != 1.0) or_dscal(n, 1.0 / tscal, cnorm, 1);          /* dlatrs.f:770-772 */
#undef A_
}

/* ---- DGECON: SRC/dgecon.f:166-252.  Reciprocal condition number in the
 * 1- or infinity-norm from the LU factors: DLACN2 estimate of
 * ||inv(A)|| with DLATRS solves.  work: 4n doubles, iwork: n ints. */
void or_dgecon(char norm, int n, const double *a, int lda, double anorm, double *rcond, double *work, int *iwork,
               int *info) {
  const double hugeval = or_dlamch('O');
  const int onenrm = (norm == '1' || norm == 'O' || norm == 'o');
  *info = 0;
  if (!onenrm && norm != 'I' && norm != 'i') *info = -1;
  else if (n < 0) *info = -2;
  else if (lda < (n > 1 ? n : 1)) *info = -4;
  else if (anorm < 0.0) *info = -5;
  if (*info != 0) { or_xerbla("DGECON", -*info); return; }
  *rcond = 0.0;
  if (n == 0) { *rcond = 1.0; return; }
  if (anorm == 0.0) return;
  if (isnan(anorm)) { *rcond = anorm; *info = -5; return; }
  if (anorm > hugeval) { *info = -5; return; }
  const double smlnum = or_dlamch('S');
  double ainvnm = 0.0;
  char normin = 'N';
  const int kase1 = onenrm ? 1 : 2;
  int kase = 0, isave[3] = {0, 0, 0};
  double *x = work, *v = work + n, *cl = work + 2 * (size_t)n, *cu = work + 3 * (size_t)n;
  for (;;) {
    or_dlacn2(n, v, x, iwork, &ainvnm, &kase, isave);
    if (kase == 0) break;
    double sl = 1.0, su = 1.0;
    int inf2 = 0;
    if (kase == kase1) {
      or_dlatrs('L', 'N', 'U', normin, n, a, lda, x, &sl, cl, &inf2);
      or_dlatrs('U', 'N', 'N', normin, n, a, lda, x, &su, cu, &inf2);
    } else {
      or_dlatrs('U', 'T', 'N', normin, n, a, lda, x, &su, cu, &inf2);
      or_dlatrs('L', 'T', 'U', normin, n, a, lda, x, &sl, cl, &inf2);
    }
    const double scale = sl * su;
    normin = 'Y';
    if (scale != 1.0) {
      const int ix = or_diamax(n, x, 1);
      if (scale < fabs(x[ix - 1]) * smlnum || scale == 0.0) return;
      or_drscl(n, scale, x);
    }
  }
  if (ainvnm != 0.0) {
    *rcond = (1.0 / ainvnm) / anorm;
  } else {
    *info = 1;
    return;
  }
  if (isnan(*rcond) || *rcond > hugeval) *info = 1;
}

/* ---- DGEEQU: SRC/dgeequ.f:139-226.  Row scalings R(i) = 1/max_j |A(i,j)|,
 * then column scalings C(j) = 1/max_i |A(i,j)|*R(i), each clamped to
 * [SMLNUM, BIGNUM]; INFO = i (row i zero) or M + j (column j zero). */
void or_dgeequ(int m, int n, const double *a, int lda, double *r, double *c, double *rowcnd, double *colcnd,
               double *amax, int *info) {
  *info = 0;
  if (m < 0) *info = -1;
  else if (n < 0) *info = -2;
  else if (lda < (m > 1 ? m : 1)) *info = -4;
  if (*info != 0) { or_xerbla("DGEEQU", -*info); return; }
  if (m == 0 || n == 0) {
    *rowcnd = 1.0;
    *colcnd = 1.0;
    *amax = 0.0;
    return;
  }
  const double smlnum = or_dlamch('S'), bignum = 1.0 / smlnum;
  for (int i = 0; i < m; i++) r[i] = 0.0;
  for (int j = 0; j < n; j++)
    for (int i = 0; i < m; i++) r[i] = fmax(r[i], fabs(a[i + (size_t)j * lda]));
  double rcmin = bignum, rcmax = 0.0;
  for (int i = 0; i < m; i++) {
    rcmax = fmax(rcmax, r[i]);
    rcmin = fmin(rcmin, r[i]);
  }
  *amax = rcmax;
  if (rcmin == 0.0) {
    for (int i = 0; i < m; i++)
      if (r[i] == 0.0) { *info = i + 1; return; }
  } else {
    for (int i = 0; i < m; i++) r[i] = 1.0 / fmin(fmax(r[i], smlnum), bignum);
    *rowcnd = fmax(rcmin, smlnum) / fmin(rcmax, bignum);
  }
  for (int j = 0; j < n; j++) c[j] = 0.0;
  for (int j = 0; j < n; j++)
    for (int i = 0; i < m; i++) c[j] = fmax(c[j], fabs(a[i + (size_t)j * lda]) * r[i]);
  rcmin = bignum;
  rcmax = 0.0;
  for (int j = 0; j < n; j++) {
    rcmin = fmin(rcmin, c[j]);
    rcmax = fmax(rcmax, c[j]);
  }
  if (rcmin == 0.0) {
    for (int j = 0; j < n; j++)
      if (c[j] == 0.0) { *info = m + j + 1; return; }
  } else {
    for (int j = 0; j < n; j++) c[j] = 1.0 / fmin(fmax(c[j], smlnum), bignum);
    *colcnd = fmax(rcmin, smlnum) / fmin(rcmax, bignum);
  }
}

/* ---- DLAQGE: SRC/dlaqge.f:145-189 (THRESH = 0.1).  Returns EQUED. */
char or_dlaqge(int m, int n, double *a, int lda, const double *r, const double *c, double rowcnd, double colcnd,
               double amax) {
  const double thresh = 0.1;
  if (m <= 0 || n <= 0) return 'N';
  const double small = or_dlamch('S') / or_dlamch('P'), large = 1.0 / small;
  if (rowcnd >= thresh && amax >= small && amax <= large) {
    if (colcnd >= thresh) return 'N';
    for (int j = 0; j < n; j++)
      for (int i = 0; i < m; i++) a[i + (size_t)j * lda] = c[j] * a[i + (size_t)j * lda];
    return 'C';
  }
  if (colcnd >= thresh) {
    for (int j = 0; j < n; j++)
      for (int i = 0; i < m; i++) a[i + (size_t)j * lda] = r[i] * a[i + (size_t)j * lda];
    return 'R';
  }
  for (int j = 0; j < n; j++)
    for (int i = 0; i < m; i++) a[i + (size_t)j * lda] = c[j] * r[i] * a[i + (size_t)j * lda];
  return 'B';
}

/* ---- DLANTR('M', 'U', 'N'): SRC/dlantr.f:173-182, max |A(i,j)| over
 * i <= min(m, j), NaN propagating. */
double or_dlantr_mun(int m, int n, const double *a, int lda) {
  if ((m < n ? m : n) == 0) return 0.0;
  double value = 0.0;
  for (int j = 1; j <= n; j++)
    for (int i = 1; i <= (m < j ? m : j); i++) {
      const double sum = fabs(a[(i - 1) + (size_t)(j - 1) * lda]);
      if (value < sum || sum != sum) value = sum;
    }
  return value;
}

/* ---- DGESVX: SRC/dgesvx.f:350-597.  FACT 'N' / 'E' / 'F', optional
 * equilibration, DGETRF, the reciprocal pivot growth (returned in
 * work[0]), DGECON, DGETRS, DGERFS, unscaling; INFO = N+1 when RCOND < eps.
 * *equed is in/out.  work: 4n doubles, iwork: n ints. */
void or_dgesvx(char fact, char trans, int n, int nrhs, double *a, int lda, double *af, int ldaf, int *ipiv,
               char *equed, double *r, double *c, double *b, int ldb, double *x, int ldx, double *rcond, double *ferr,
               double *berr, double *work, int *iwork, int *info) {
  *info = 0;
  const int nofact = (fact == 'N' || fact == 'n'), equil = (fact == 'E' || fact == 'e');
  const int notran = (trans == 'N' || trans == 'n');
  int rowequ = 0, colequ = 0;
  double smlnum = 0.0, bignum = 0.0, rowcnd = 1.0, colcnd = 1.0, amax = 0.0;
  if (nofact || equil) {
    *equed = 'N';
  } else {
    rowequ = (*equed == 'R' || *equed == 'r' || *equed == 'B' || *equed == 'b');
    colequ = (*equed == 'C' || *equed == 'c' || *equed == 'B' || *equed == 'b');
    smlnum = or_dlamch('S');
    bignum = 1.0 / smlnum;
  }
  if (!nofact && !equil && fact != 'F' && fact != 'f') *info = -1;
  else if (!notran && trans != 'T' && trans != 't' && trans != 'C' && trans != 'c') *info = -2;
  else if (n < 0) *info = -3;
  else if (nrhs < 0) *info = -4;
  else if (lda < (n > 1 ? n : 1)) *info = -6;
  else if (ldaf < (n > 1 ? n : 1)) *info = -8;
  else if ((fact == 'F' || fact == 'f') && !(rowequ || colequ || *equed == 'N' || *equed == 'n')) *info = -10;
  else {
    if (rowequ) {
      double rcmin = bignum, rcmax = 0.0;
      for (int j = 0; j < n; j++) { rcmin = fmin(rcmin, r[j]); rcmax = fmax(rcmax, r[j]); }
      if (rcmin <= 0.0) *info = -11;
      else if (n > 0) rowcnd = fmax(rcmin, smlnum) / fmin(rcmax, bignum);
      else rowcnd = 1.0;
    }
    if (colequ && *info == 0) {
      double rcmin = bignum, rcmax = 0.0;
      for (int j = 0; j < n; j++) { rcmin = fmin(rcmin, c[j]); rcmax = fmax(rcmax, c[j]); }
      if (rcmin <= 0.0) *info = -12;
      else if (n > 0) colcnd = fmax(rcmin, smlnum) / fmin(rcmax, bignum);
      else colcnd = 1.0;
    }
    if (*info == 0) {
      if (ldb < (n > 1 ? n : 1)) *info = -14;
      else if (ldx < (n > 1 ? n : 1)) *info = -16;
    }
  }
  if (*info != 0) { or_xerbla("DGESVX", -*info); return; }
  if (equil) {
    int infequ = 0;
    or_dgeequ(n, n, a, lda, r, c, &rowcnd, &colcnd, &amax, &infequ);
    if (infequ == 0) {
      *equed = or_dlaqge(n, n, a, lda, r, c, rowcnd, colcnd, amax);
      rowequ = (*equed == 'R' || *equed == 'B');
      colequ = (*equed == 'C' || *equed == 'B');
    }
  }
  if (notran) {
    if (rowequ)
      for (int j = 0; j < nrhs; j++)
        for (int i = 0; i < n; i++) b[i + (size_t)j * ldb] = r[i] * b[i + (size_t)j * ldb];
  } else if (colequ) {
    for (int j = 0; j < nrhs; j++)
      for (int i = 0; i < n; i++) b[i + (size_t)j * ldb] = c[i] * b[i + (size_t)j * ldb];
  }
  if (nofact || equil) {
    or_dlacpy(n, n, a, lda, af, ldaf);
    or_dgetrf(n, n, af, ldaf, ipiv, info);
    if (*info > 0) {
      double rpvgrw = or_dlantr_mun(*info, *info, af, ldaf);
      if (rpvgrw == 0.0) rpvgrw = 1.0;
      else rpvgrw = or_dlange('M', n, *info, a, lda, work) / rpvgrw;
      work[0] = rpvgrw;
      *rcond = 0.0;
      return;
    }
  }
  const char norm = notran ? '1' : 'I';
  const double anorm = or_dlange(norm, n, n, a, lda, work);
  double rpvgrw = or_dlantr_mun(n, n, af, ldaf);
  if (rpvgrw == 0.0) rpvgrw = 1.0;
  else rpvgrw = or_dlange('M', n, n, a, lda, work) / rpvgrw;
  or_dgecon(norm, n, af, ldaf, anorm, rcond, work, iwork, info);
  or_dlacpy(n, nrhs, b, ldb, x, ldx);
  or_dgetrs(trans, n, nrhs, af, ldaf, ipiv, x, ldx, info);
  or_dgerfs(trans, n, nrhs, a, lda, af, ldaf, ipiv, b, ldb, x, ldx, ferr, berr, work, iwork, info);
  if (notran) {
    if (colequ) {
      for (int j = 0; j < nrhs; j++)
        for (int i = 0; i < n; i++) x[i + (size_t)j * ldx] = c[i] * x[i + (size_t)j * ldx];
      for (int j = 0; j < nrhs; j++) ferr[j] = ferr[j] / colcnd;
    }
  } else if (rowequ) {
    for (int j = 0; j < nrhs; j++)
      for (int i = 0; i < n; i++) x[i + (size_t)j * ldx] = r[i] * x[i + (size_t)j * ldx];
    for (int j = 0; j < nrhs; j++) ferr[j] = ferr[j] / rowcnd;
  }
  work[0] = rpvgrw;
  if (*rcond < or_dlamch('E')) *info = n + 1;
}

/* ---- DGETRI and the routines it calls, in the reference loop order
 * (BLAS/SRC/dtrmv.f:226-235, dtrmm.f:271-283, dtrsm.f:333-367,
 * SRC/dtrti2.f:128-160, dtrtri.f:149-196, dgetri.f:169-262).  NB is a
 * parameter (ILAENV's 64 by default; the test suite varies it). */
#define A_(i, j) a[(size_t)(i) + (size_t)(j) * lda]
static void or_dtrmv_un(int nounit, int n, const double *a, int lda, double *x) {
  for (int j = 0; j < n; j++) {
    const double temp = x[j];
    for (int i = 0; i < j; i++) x[i] = x[i] + temp * A_(i, j);
    if (nounit) x[j] = x[j] * A_(j, j);
  }
}
/* B := alpha*A*B, A upper (m x m), B m x n */
static void or_dtrmm_lun(int nounit, int m, int n, double alpha, const double *a, int lda, double *b, int ldb) {
  for (int j = 0; j < n; j++)
    for (int k = 0; k < m; k++) {
      double temp = alpha * b[k + (size_t)j * ldb];
      for (int i = 0; i < k; i++) b[i + (size_t)j * ldb] = b[i + (size_t)j * ldb] + temp * A_(i, k);
      if (nounit) temp = temp * A_(k, k);
      b[k + (size_t)j * ldb] = temp;
    }
}
/* B := alpha*B*inv(A), A upper (n x n) or lower, B m x n */
static void or_dtrsm_rn(int upper, int nounit, int m, int n, double alpha, const double *a, int lda, double *b,
                        int ldb) {
  if (upper) {
    for (int j = 0; j < n; j++) {
      for (int i = 0; i < m; i++) b[i + (size_t)j * ldb] = alpha * b[i + (size_t)j * ldb];
      for (int k = 0; k < j; k++)
        for (int i = 0; i < m; i++) b[i + (size_t)j * ldb] = b[i + (size_t)j * ldb] - A_(k, j) * b[i + (size_t)k * ldb];
      if (nounit)
        for (int i = 0; i < m; i++) b[i + (size_t)j * ldb] = b[i + (size_t)j * ldb] / A_(j, j);
    }
  } else {
    for (int j = n - 1; j >= 0; j--) {
      for (int i = 0; i < m; i++) b[i + (size_t)j * ldb] = alpha * b[i + (size_t)j * ldb];
      for (int k = j + 1; k < n; k++)
        for (int i = 0; i < m; i++) b[i + (size_t)j * ldb] = b[i + (size_t)j * ldb] - A_(k, j) * b[i + (size_t)k * ldb];
      if (nounit)
        for (int i = 0; i < m; i++) b[i + (size_t)j * ldb] = b[i + (size_t)j * ldb] / A_(j, j);
    }
  }
}
/* DTRTI2 upper */
static void or_dtrti2_u(int nounit, int n, double *a, int lda) {
  for (int j = 0; j < n; j++) {
    double ajj;
    if (nounit) {
      A_(j, j) = 1.0 / A_(j, j);
      ajj = -A_(j, j);
    } else {
      ajj = -1.0;
    }
    or_dtrmv_un(nounit, j, a, lda, &A_(0, j));
    or_dscal(j, ajj, &A_(0, j), 1);
  }
}
/* DTRTRI('U', diag): INFO = first zero diagonal (non-unit) */
void or_dtrtri_u(char diag, int n, double *a, int lda, int nb, int *info) {
  const int nounit = (diag == 'N' || diag == 'n');
  *info = 0;
  if (n == 0) return;
  if (nounit)
    for (int i = 0; i < n; i++)
      if (A_(i, i) == 0.0) { *info = i + 1; return; }
  if (nb <= 1 || nb >= n) {
    or_dtrti2_u(nounit, n, a, lda);
    return;
  }
  for (int j = 0; j < n; j += nb) {
    const int jb = (nb < n - j) ? nb : n - j;
    or_dtrmm_lun(nounit, j, jb, 1.0, a, lda, &A_(0, j), lda);
    or_dtrsm_rn(1, nounit, j, jb, -1.0, &A_(j, j), lda, &A_(0, j), lda);
    or_dtrti2_u(nounit, jb, &A_(j, j), lda);
  }
}
/* DGETRI; lwork = -1 is the workspace query (work[0] = max(1, n*nb)) */
void or_dgetri(int n, double *a, int lda, const int *ipiv, double *work, int lwork, int nb, int *info) {
  *info = 0;
  const int lwkopt = (n * nb > 1) ? n * nb : 1;
  work[0] = (double)lwkopt;
  const int lquery = (lwork == -1);
  if (n < 0) *info = -1;
  else if (lda < (n > 1 ? n : 1)) *info = -3;
  else if (lwork < (n > 1 ? n : 1) && !lquery) *info = -6;
  if (*info != 0) { or_xerbla("DGETRI", -*info); return; }
  if (lquery) return;
  if (n == 0) return;
  or_dtrtri_u('N', n, a, lda, nb, info);
  if (*info > 0) return;
  int nbmin = 2;
  const int ldwork = n;
  int iws;
  if (nb > 1 && nb < n) {
    iws = (ldwork * nb > 1) ? ldwork * nb : 1;
    if (lwork < iws) {
      nb = lwork / ldwork;
      nbmin = 2;   /* ILAENV(2, 'DGETRI') */
    }
  } else {
    iws = n;
  }
  if (nb < nbmin || nb >= n) {
    for (int j = n - 1; j >= 0; j--) {
      for (int i = j + 1; i < n; i++) {
        work[i] = A_(i, j);
        A_(i, j) = 0.0;
      }
      if (j < n - 1) {
        /* DGEMV('N', N, N-J, -1, A(1,J+1), LDA, WORK(J+1), 1, 1, A(1,J), 1) */
        for (int jj = j + 1; jj < n; jj++) {
          const double temp = -1.0 * work[jj];
          for (int i = 0; i < n; i++) A_(i, j) = A_(i, j) + temp * A_(i, jj);
        }
      }
    }
  } else {
    const int nn = ((n - 1) / nb) * nb;
    for (int j = nn; j >= 0; j -= nb) {
      const int jb = (nb < n - j) ? nb : n - j;
      for (int jj = j; jj < j + jb; jj++)
        for (int i = jj + 1; i < n; i++) {
          work[i + (size_t)(jj - j) * ldwork] = A_(i, jj);
          A_(i, jj) = 0.0;
        }
      if (j + jb < n)
        or_dgemm('N', 'N', n, jb, n - j - jb, -1.0, &A_(0, j + jb), lda, work + j + jb, ldwork, 1.0, &A_(0, j),
                 lda);
      or_dtrsm_rn(0, 0, n, jb, 1.0, work + j, ldwork, &A_(0, j), lda);
    }
  }
  for (int j = n - 2; j >= 0; j--) {
    const int jp = ipiv[j] - 1;
    if (jp != j)
      for (int i = 0; i < n; i++) {
        const double t = A_(i, j);
        A_(i, j) = A_(i, jp);
        A_(i, jp) = t;
      }
  }
  work[0] = (double)iws;
}
#undef A_

/* ---- DLANSY ('M', 'I' / '1' / 'O'): SRC/dlansy.f:144-200.  work: n. */
double or_dlansy(char norm, char uplo, int n, const double *a, int lda, double *work) {
  const int upper = (uplo == 'U' || uplo == 'u');
  double value = 0.0;
  if (n == 0) return 0.0;
  if (norm == 'M' || norm == 'm') {
    for (int j = 0; j < n; j++) {
      const int i0 = upper ? 0 : j, i1 = upper ? j : n - 1;
      for (int i = i0; i <= i1; i++) {
        const double sum = fabs(a[i + (size_t)j * lda]);
        if (value < sum || sum != sum) value = sum;
      }
    }
  } else if (upper) {
    for (int j = 0; j < n; j++) {
      double sum = 0.0;
      for (int i = 0; i < j; i++) {
        const double absa = fabs(a[i + (size_t)j * lda]);
        sum = sum + absa;
        work[i] = work[i] + absa;
      }
      work[j] = sum + fabs(a[j + (size_t)j * lda]);
    }
    for (int i = 0; i < n; i++) {
      const double sum = work[i];
      if (value < sum || sum != sum) value = sum;
    }
  } else {
    for (int i = 0; i < n; i++) work[i] = 0.0;
    for (int j = 0; j < n; j++) {
      double sum = work[j] + fabs(a[j + (size_t)j * lda]);
      for (int i = j + 1; i < n; i++) {
        const double absa = fabs(a[i + (size_t)j * lda]);
        sum = sum + absa;
        work[i] = work[i] + absa;
      }
      if (value < sum || sum != sum) value = sum;
    }
  }
  return value;
}

/* ---- DLAT2S: SRC/dlat2s.f:128-158.  Stops with INFO = 1 at the first
 * element of the triangle (column order) outside [-RMAX, RMAX]. */
void or_dlat2s(char uplo, int n, const double *a, int lda, float *sa, int ldsa, int *info) {
  const double rmax = (double)or_slamch('O');
  const int upper = (uplo == 'U' || uplo == 'u');
  *info = 0;
  for (int j = 0; j < n; j++) {
    const int i0 = upper ? 0 : j, i1 = upper ? j : n - 1;
    for (int i = i0; i <= i1; i++) {
      const double v = a[i + (size_t)j * lda];
      if (v < -rmax || v > rmax) { *info = 1; return; }
      sa[i + (size_t)j * ldsa] = (float)v;
    }
  }
}

/* ---- DSYMM('L', uplo), C := alpha*A*B + C (BETA = 1): BLAS/SRC/dsymm.f:289-323. */
void or_dsymm_l(char uplo, int m, int n, double alpha, const double *a, int lda, const double *b, int ldb, double *c,
                int ldc) {
  const int upper = (uplo == 'U' || uplo == 'u');
  if (m == 0 || n == 0 || alpha == 0.0) return;
  for (int j = 0; j < n; j++) {
    if (upper) {
      for (int i = 0; i < m; i++) {
        const double temp1 = alpha * b[i + (size_t)j * ldb];
        double temp2 = 0.0;
        for (int k = 0; k < i; k++) {
          c[k + (size_t)j * ldc] = c[k + (size_t)j * ldc] + temp1 * a[k + (size_t)i * lda];
          temp2 = temp2 + b[k + (size_t)j * ldb] * a[k + (size_t)i * lda];
        }
        c[i + (size_t)j * ldc] = c[i + (size_t)j * ldc] + temp1 * a[i + (size_t)i * lda] + alpha * temp2;
      }
    } else {
      for (int i = m - 1; i >= 0; i--) {
        const double temp1 = alpha * b[i + (size_t)j * ldb];
        double temp2 = 0.0;
        for (int k = i + 1; k < m; k++) {
          c[k + (size_t)j * ldc] = c[k + (size_t)j * ldc] + temp1 * a[k + (size_t)i * lda];
          temp2 = temp2 + b[k + (size_t)j * ldb] * a[k + (size_t)i * lda];
        }
        c[i + (size_t)j * ldc] = c[i + (size_t)j * ldc] + temp1 * a[i + (size_t)i * lda] + alpha * temp2;
      }
    }
  }
}

/* ---- DSPOSV: SRC/dsposv.f:237-420 (ITERMAX = 30, BWDMAX = 1).
 * work: n*nrhs doubles, swork: n*(n+nrhs) floats. */
void or_dsposv(char uplo, int n, int nrhs, double *a, int lda, const double *b, int ldb, double *x, int ldx,
               double *work, float *swork, int *iter, int *info) {
  const int itermax = 30;
  const double bwdmax = 1.0;
  *info = 0;
  *iter = 0;
  if (uplo != 'U' && uplo != 'u' && uplo != 'L' && uplo != 'l') *info = -1;
  else if (n < 0) *info = -2;
  else if (nrhs < 0) *info = -3;
  else if (lda < (n > 1 ? n : 1)) *info = -5;
  else if (ldb < (n > 1 ? n : 1)) *info = -7;
  else if (ldx < (n > 1 ? n : 1)) *info = -9;
  if (*info != 0) { or_xerbla("DSPOSV", -*info); return; }
  if (n == 0) return;
  const double anrm = or_dlansy('I', uplo, n, a, lda, work);
  const double eps = or_dlamch('E');
  const double cte = anrm * eps * sqrt((double)n) * bwdmax;
  float *sa = swork;
  float *sx = swork + (size_t)n * n;
  int i;
  or_dlag2s(n, nrhs, b, ldb, sx, n, info);
  if (*info != 0) { *iter = -2; goto fallback; }
  or_dlat2s(uplo, n, a, lda, sa, n, info);
  if (*info != 0) { *iter = -2; goto fallback; }
  or_spotrf(uplo, n, sa, n, info);
  if (*info != 0) { *iter = -3; goto fallback; }
  or_spotrs(uplo, n, nrhs, sa, n, sx, n, info);
  or_slag2d(n, nrhs, sx, n, x, ldx, info);
  or_dlacpy(n, nrhs, b, ldb, work, n);
  or_dsymm_l(uplo, n, nrhs, -1.0, a, lda, x, ldx, work, n);
  for (i = 0; i < nrhs; i++) {
    const double xnrm = fabs(x[(size_t)(or_diamax(n, x + (size_t)i * ldx, 1) - 1) + (size_t)i * ldx]);
    const double rnrm = fabs(work[(size_t)(or_diamax(n, work + (size_t)i * n, 1) - 1) + (size_t)i * n]);
    if (rnrm > xnrm * cte) break;
  }
  if (i == nrhs) { *iter = 0; return; }
  for (int iiter = 1; iiter <= itermax; iiter++) {
    or_dlag2s(n, nrhs, work, n, sx, n, info);
    if (*info != 0) { *iter = -2; goto fallback; }
    or_spotrs(uplo, n, nrhs, sa, n, sx, n, info);
    or_slag2d(n, nrhs, sx, n, work, n, info);
    for (int k = 0; k < nrhs; k++) or_daxpy(n, 1.0, work + (size_t)k * n, 1, x + (size_t)k * ldx, 1);
    or_dlacpy(n, nrhs, b, ldb, work, n);
    or_dsymm_l(uplo, n, nrhs, -1.0, a, lda, x, ldx, work, n);
    for (i = 0; i < nrhs; i++) {
      const double xnrm = fabs(x[(size_t)(or_diamax(n, x + (size_t)i * ldx, 1) - 1) + (size_t)i * ldx]);
      const double rnrm = fabs(work[(size_t)(or_diamax(n, work + (size_t)i * n, 1) - 1) + (size_t)i * n]);
      if (rnrm > xnrm * cte) break;
    }
    if (i == nrhs) { *iter = iiter; return; }
  }
  *iter = -itermax - 1;
fallback:
  or_dpotrf(uplo, n, a, lda, info);
  if (*info != 0) return;
  or_dlacpy(n, nrhs, b, ldb, x, ldx);
  or_dpotrs(uplo, n, nrhs, a, lda, x, ldx, info);
}

/* ---- DLARNV: SRC/dlarnv.f:94-174.  Chunks of 64 outputs; IDIST 1 U(0,1),
 * 2 U(-1,1), 3 N(0,1) by Box-Muller on consecutive pairs. */
void or_dlarnv(int idist, int iseed[4], long long n, double *x) {
  const double twopi = 6.28318530717958647692528676655900576839;
  double u[128];
  for (long long iv = 1; iv <= n; iv += 64) {
    int il = (int)((n - iv + 1) < 64 ? (n - iv + 1) : 64);
    int il2 = (idist == 3) ? 2 * il : il;
    or_dlaruv(iseed, il2, u);
    if (idist == 1) {
      for (int i = 0; i < il; i++) x[iv - 1 + i] = u[i];
    } else if (idist == 2) {
      for (int i = 0; i < il; i++) x[iv - 1 + i] = 2.0 * u[i] - 1.0;
    } else if (idist == 3) {
      for (int i = 0; i < il; i++) x[iv - 1 + i] = sqrt(-2.0 * log(u[2 * i])) * cos(twopi * u[2 * i + 1]);
    }
  }
}

/* Scalar-seed convention of this project (the reference has none): seed s
 * maps to ISEED = (0, 0, (2s+1)/4096 mod 4096, (2s+1) mod 4096); ISEED(4)
 * is odd as DLARUV requires. */
void or_seed_from_int(long long seed, int iseed[4]) {
  uint64_t v = ((uint64_t)(2 * seed + 1)) & OR_M48;
  or_seed_unpack(v, iseed);
  iseed[0] = 0;
  iseed[1] = 0;
}
