// The sequential parts of DLATRS (SRC/dlatrs.f:264-847) and of DGECON's
// rescaling step (SRC/dgecon.f:230-238 with DRSCL, SRC/drscl.f:105-133),
// written once for host and device: on the GPU each runs on a single
// thread (one short kernel), and the CPU tests compile the same code with
// g++ to check it bit for bit against the oracle.
//
// These are recurrences over the columns in which every step may rescale
// the whole vector, so they run as one thread: the careful solve is the
// path DLATRS takes only when its growth bound rejects a plain triangular
// solve (badly scaled or nearly singular triangles).  Every operation is
// separately rounded (no contraction), MIN / MAX are fmin / fmax.
#pragma once
#include <cmath>

#include "fp_convert.h"   // GB_HD

namespace gb {

constexpr double kSafeMin = 2.2250738585072014e-308;   // DLAMCH('Safe minimum')
constexpr double kPrec = 2.220446049250313e-16;        // DLAMCH('Precision')
constexpr double kOvfl = 1.7976931348623157e308;       // DLAMCH('Overflow')

enum LatrsMode : int { kLatrsTrsv = 0, kLatrsCareful = 1, kLatrsDirect = 2 };

// What the plan step decided for one DLATRS call.
struct LatrsPlan {
  int mode;        // LatrsMode
  double tscal;    // TSCAL
  double xmax;     // |X(IDAMAX(X))| before the solve
  double scale;    // SCALE (1 unless the careful solve scaled X)
};

#if defined(__CUDA_ARCH__)
GB_HD inline double rn_add(double a, double b) { return __dadd_rn(a, b); }
GB_HD inline double rn_sub(double a, double b) { return __dsub_rn(a, b); }
GB_HD inline double rn_mul(double a, double b) { return __dmul_rn(a, b); }
GB_HD inline double rn_div(double a, double b) { return __ddiv_rn(a, b); }
GB_HD inline double rn_sqrt(double a) { return __dsqrt_rn(a); }
GB_HD inline float rn_add(float a, float b) { return __fadd_rn(a, b); }
GB_HD inline float rn_sub(float a, float b) { return __fsub_rn(a, b); }
GB_HD inline float rn_mul(float a, float b) { return __fmul_rn(a, b); }
GB_HD inline float rn_div(float a, float b) { return __fdiv_rn(a, b); }
GB_HD inline float rn_sqrt(float a) { return __fsqrt_rn(a); }
#else
GB_HD inline double rn_add(double a, double b) { return a + b; }
GB_HD inline double rn_sub(double a, double b) { return a - b; }
GB_HD inline double rn_mul(double a, double b) { return a * b; }
GB_HD inline double rn_div(double a, double b) { return a / b; }
GB_HD inline double rn_sqrt(double a) { return std::sqrt(a); }
GB_HD inline float rn_add(float a, float b) { return a + b; }
GB_HD inline float rn_sub(float a, float b) { return a - b; }
GB_HD inline float rn_mul(float a, float b) { return a * b; }
GB_HD inline float rn_div(float a, float b) { return a / b; }
GB_HD inline float rn_sqrt(float a) { return std::sqrt(a); }
#endif

// IDAMAX (BLAS/SRC/idamax.f:93-123), 1-based, 0 for n < 1.
GB_HD inline int seq_idamax(int n, const double* x) {
  if (n < 1) return 0;
  int best = 1;
  double dmax = fabs(x[0]);
  for (int i = 2; i <= n; ++i) {
    const double v = fabs(x[i - 1]);
    if (v > dmax) {
      best = i;
      dmax = v;
    }
  }
  return best;
}

// DSCAL (BLAS/SRC/dscal.f), with its DA = 1 quick return.
GB_HD inline void seq_scal(int n, double a, double* x) {
  if (n <= 0 || a == 1.0) return;
  for (int i = 0; i < n; ++i) x[i] = rn_mul(a, x[i]);
}

// dlatrs.f:340-503 up to the choice of solve: TSCAL from max CNORM (CNORM
// scaled in place when it exceeds BIGNUM), XMAX, the growth bound, then
// DTRSV when GROW*TSCAL > SMLNUM, else the careful solve.  CNORM holds the
// off-diagonal column sums of the triangle on entry.
GB_HD inline void latrs_plan_seq(int upper, int notran, int nounit, int n, const double* A, int lda, const double* x,
                                 double* cnorm, LatrsPlan* plan) {
  const double smlnum = rn_div(kSafeMin, kPrec), bignum = rn_div(1.0, smlnum);
  auto Aij = [&](int i, int j) { return A[(size_t)i + (size_t)j * lda]; };
  const int imax = seq_idamax(n, cnorm);
  double tmax = cnorm[imax - 1];
  double tscal = 1.0;
  bool direct = false;
  if (tmax <= bignum) {
    tscal = 1.0;
  } else if (tmax <= kOvfl) {
    tscal = rn_div(1.0, rn_mul(smlnum, tmax));
    seq_scal(n, tscal, cnorm);
  } else {
    // a column sum overflowed: TMAX = the largest off-diagonal |A(i,j)|
    // (DLANGE('M') per column, NaN propagating)
    tmax = 0.0;
    for (int j = 0; j < n; ++j) {
      const int i0 = upper ? 0 : j + 1, i1 = upper ? j : n;
      if (i1 <= i0) continue;
      double m = 0.0;
      for (int i = i0; i < i1; ++i) {
        const double t = fabs(Aij(i, j));
        if (m < t || t != t) m = t;
      }
      tmax = fmax(m, tmax);
    }
    if (tmax <= kOvfl) {
      tscal = rn_div(1.0, rn_mul(smlnum, tmax));
      for (int j = 0; j < n; ++j) {
        if (cnorm[j] <= kOvfl) {
          cnorm[j] = rn_mul(cnorm[j], tscal);
        } else {
          const int i0 = upper ? 0 : j + 1, i1 = upper ? j : n;
          double s = 0.0;
          for (int i = i0; i < i1; ++i) s = rn_add(s, rn_mul(tscal, fabs(Aij(i, j))));
          cnorm[j] = s;
        }
      }
    } else {
      direct = true;   // dlatrs.f:395: DTRSV without scaling
    }
  }
  const int jx = seq_idamax(n, x);
  const double xmax = fabs(x[jx - 1]);
  double grow = 0.0;
  if (!direct) {
    double xbnd = xmax;
    int jfirst, jlast, jinc;
    if (notran == upper) { jfirst = n - 1; jlast = 0; jinc = -1; }   // 'N' upper, 'T' lower
    else { jfirst = 0; jlast = n - 1; jinc = 1; }
    if (tscal != 1.0) {
      grow = 0.0;
    } else if (notran) {
      if (nounit) {   // dlatrs.f:422-442
        grow = rn_div(1.0, fmax(xbnd, smlnum));
        xbnd = grow;
        bool cut = false;
        for (int j = jfirst; j != jlast + jinc; j += jinc) {
          if (grow <= smlnum) { cut = true; break; }
          const double tjj = fabs(Aij(j, j));
          xbnd = fmin(xbnd, rn_mul(fmin(1.0, tjj), grow));
          const double den = rn_add(tjj, cnorm[j]);
          grow = (den >= smlnum) ? rn_mul(grow, rn_div(tjj, den)) : 0.0;
        }
        if (!cut) grow = xbnd;
      } else {        // dlatrs.f:443-455
        grow = fmin(1.0, rn_div(1.0, fmax(xbnd, smlnum)));
        for (int j = jfirst; j != jlast + jinc; j += jinc) {
          if (grow <= smlnum) break;
          grow = rn_mul(grow, rn_div(1.0, rn_add(1.0, cnorm[j])));
        }
      }
    } else {
      if (nounit) {   // dlatrs.f:470-484
        grow = rn_div(1.0, fmax(xbnd, smlnum));
        xbnd = grow;
        bool cut = false;
        for (int j = jfirst; j != jlast + jinc; j += jinc) {
          if (grow <= smlnum) { cut = true; break; }
          const double xj = rn_add(1.0, cnorm[j]);
          grow = fmin(grow, rn_div(xbnd, xj));
          const double tjj = fabs(Aij(j, j));
          if (xj > tjj) xbnd = rn_mul(xbnd, rn_div(tjj, xj));
        }
        if (!cut) grow = fmin(grow, xbnd);
      } else {        // dlatrs.f:485-495
        grow = fmin(1.0, rn_div(1.0, fmax(xbnd, smlnum)));
        for (int j = jfirst; j != jlast + jinc; j += jinc) {
          if (grow <= smlnum) break;
          grow = rn_div(grow, rn_add(1.0, cnorm[j]));
        }
      }
    }
  }
  plan->tscal = tscal;
  plan->xmax = xmax;
  plan->scale = 1.0;
  plan->mode = direct ? kLatrsDirect : (rn_mul(grow, tscal) > smlnum ? kLatrsTrsv : kLatrsCareful);
}

// dlatrs.f:505-772: the careful column sweep.  X is rescaled (and SCALE
// with it) whenever the next step could overflow; at the end SCALE =
// SCALE / TSCAL and CNORM is returned to its unscaled value.
GB_HD inline void latrs_careful_seq(int upper, int notran, int nounit, int n, const double* A, int lda, double* x,
                                    double* cnorm, LatrsPlan* plan) {
  const double smlnum = rn_div(kSafeMin, kPrec), bignum = rn_div(1.0, smlnum);
  auto Aij = [&](int i, int j) { return A[(size_t)i + (size_t)j * lda]; };
  const double tscal = plan->tscal;
  double xmax = plan->xmax, scale = 1.0;
  int jfirst, jinc;
  if (notran == upper) { jfirst = n - 1; jinc = -1; }
  else { jfirst = 0; jinc = 1; }
  if (xmax > bignum) {   // dlatrs.f:509-516
    scale = rn_div(bignum, xmax);
    seq_scal(n, scale, x);
    xmax = bignum;
  }
  for (int step = 0, j = jfirst; step < n; ++step, j += jinc) {
    double xj = fabs(x[j]), tjjs = 0.0, tjj, rec;
    if (notran) {          // dlatrs.f:518-640
      bool skip = false;
      if (nounit) {
        tjjs = rn_mul(Aij(j, j), tscal);
      } else {
        tjjs = tscal;
        if (tscal == 1.0) skip = true;
      }
      if (!skip) {
        tjj = fabs(tjjs);
        if (tjj > smlnum) {
          if (tjj < 1.0 && xj > rn_mul(tjj, bignum)) {
            rec = rn_div(1.0, xj);
            seq_scal(n, rec, x);
            scale = rn_mul(scale, rec);
            xmax = rn_mul(xmax, rec);
          }
          x[j] = rn_div(x[j], tjjs);
          xj = fabs(x[j]);
        } else if (tjj > 0.0) {
          if (xj > rn_mul(tjj, bignum)) {
            rec = rn_div(rn_mul(tjj, bignum), xj);
            if (cnorm[j] > 1.0) rec = rn_div(rec, cnorm[j]);
            seq_scal(n, rec, x);
            scale = rn_mul(scale, rec);
            xmax = rn_mul(xmax, rec);
          }
          x[j] = rn_div(x[j], tjjs);
          xj = fabs(x[j]);
        } else {
          for (int i = 0; i < n; ++i) x[i] = 0.0;
          x[j] = 1.0;
          xj = 1.0;
          scale = 0.0;
          xmax = 0.0;
        }
      }
      if (xj > 1.0) {
        rec = rn_div(1.0, xj);
        if (cnorm[j] > rn_mul(rn_sub(bignum, xmax), rec)) {
          rec = rn_mul(rec, 0.5);
          seq_scal(n, rec, x);
          scale = rn_mul(scale, rec);
        }
      } else if (rn_mul(xj, cnorm[j]) > rn_sub(bignum, xmax)) {
        seq_scal(n, 0.5, x);
        scale = rn_mul(scale, 0.5);
      }
      // DAXPY (quick return for a zero multiplier) and IDAMAX of the rest
      const int lo = upper ? 0 : j + 1, len = upper ? j : n - j - 1;
      if (len > 0) {
        const double alpha = rn_mul(-x[j], tscal);
        if (alpha != 0.0)
          for (int i = 0; i < len; ++i) x[lo + i] = rn_add(x[lo + i], rn_mul(alpha, Aij(lo + i, j)));
        const int im = seq_idamax(len, x + lo);
        xmax = fabs(x[lo + im - 1]);
      }
    } else {               // dlatrs.f:642-764
      double uscal = tscal;
      rec = rn_div(1.0, fmax(xmax, 1.0));
      if (cnorm[j] > rn_mul(rn_sub(bignum, xj), rec)) {
        rec = rn_mul(rec, 0.5);
        tjjs = nounit ? rn_mul(Aij(j, j), tscal) : tscal;
        tjj = fabs(tjjs);
        if (tjj > 1.0) {
          rec = fmin(1.0, rn_mul(rec, tjj));
          uscal = rn_div(uscal, tjjs);
        }
        if (rec < 1.0) {
          seq_scal(n, rec, x);
          scale = rn_mul(scale, rec);
          xmax = rn_mul(xmax, rec);
        }
      }
      const int lo = upper ? 0 : j + 1, len = upper ? j : n - j - 1;
      double sumj = 0.0;   // DDOT in index order, or the explicit USCAL loop
      if (uscal == 1.0) {
        for (int i = 0; i < len; ++i) sumj = rn_add(sumj, rn_mul(Aij(lo + i, j), x[lo + i]));
      } else {
        for (int i = 0; i < len; ++i) sumj = rn_add(sumj, rn_mul(rn_mul(Aij(lo + i, j), uscal), x[lo + i]));
      }
      if (uscal == tscal) {
        x[j] = rn_sub(x[j], sumj);
        xj = fabs(x[j]);
        bool skip = false;
        if (nounit) {
          tjjs = rn_mul(Aij(j, j), tscal);
        } else {
          tjjs = tscal;
          if (tscal == 1.0) skip = true;
        }
        if (!skip) {
          tjj = fabs(tjjs);
          if (tjj > smlnum) {
            if (tjj < 1.0 && xj > rn_mul(tjj, bignum)) {
              rec = rn_div(1.0, xj);
              seq_scal(n, rec, x);
              scale = rn_mul(scale, rec);
              xmax = rn_mul(xmax, rec);
            }
            x[j] = rn_div(x[j], tjjs);
          } else if (tjj > 0.0) {
            if (xj > rn_mul(tjj, bignum)) {
              rec = rn_div(rn_mul(tjj, bignum), xj);
              seq_scal(n, rec, x);
              scale = rn_mul(scale, rec);
              xmax = rn_mul(xmax, rec);
            }
            x[j] = rn_div(x[j], tjjs);
          } else {
            for (int i = 0; i < n; ++i) x[i] = 0.0;
            x[j] = 1.0;
            scale = 0.0;
            xmax = 0.0;
          }
        }
      } else {
        x[j] = rn_sub(rn_div(x[j], tjjs), sumj);
      }
      xmax = fmax(xmax, fabs(x[j]));
    }
  }
  scale = rn_div(scale, tscal);
  if (tscal != 1.0) seq_scal(n, rn_div(1.0, tscal), cnorm);   // dlatrs.f:770-772
  plan->scale = scale;
}

// DGECON's step after the two DLATRS solves (dgecon.f:230-238): SCALE =
// SL*SU; when SCALE != 1, stop (RCOND = 0) if SCALE < |X(IDAMAX)|*SMLNUM
// or SCALE = 0, else X := X / SCALE by DRSCL.  Returns 1 to stop.
GB_HD inline int gecon_rescale_seq(int n, double* x, double sl, double su) {
  const double scale = rn_mul(sl, su);
  if (scale == 1.0) return 0;
  const int ix = seq_idamax(n, x);
  if (scale < rn_mul(fabs(x[ix - 1]), kSafeMin) || scale == 0.0) return 1;
  // DRSCL: multiply by SMLNUM or BIGNUM until the remaining factor is safe
  const double smlnum = kSafeMin, bignum = rn_div(1.0, smlnum);
  double cden = scale, cnum = 1.0;
  for (int guard = 0; guard < 64; ++guard) {
    const double cden1 = rn_mul(cden, smlnum), cnum1 = rn_div(cnum, bignum);
    double mul;
    bool done;
    if (fabs(cden1) > fabs(cnum) && cnum != 0.0) {
      mul = smlnum;
      done = false;
      cden = cden1;
    } else if (fabs(cnum1) > fabs(cden)) {
      mul = bignum;
      done = false;
      cnum = cnum1;
    } else {
      mul = rn_div(cnum, cden);
      done = true;
    }
    seq_scal(n, mul, x);
    if (done) break;
  }
  return 0;
}

// DGEEQU's finishing step for one set of scalings (SRC/dgeequ.f:166-189
// for R, :203-225 for C): the smallest and largest of the maxima s[0..m),
// INFO = info_base + (first zero) when one is zero, else s(i) =
// 1/MIN(MAX(s(i), SMLNUM), BIGNUM) and *cnd = MAX(min, SMLNUM)/MIN(max,
// BIGNUM).  *smax receives the largest maximum (AMAX for the rows).
GB_HD inline int equ_finish_seq(int m, double* s, int info_base, double* cnd, double* smax) {
  const double smlnum = kSafeMin, bignum = rn_div(1.0, smlnum);
  double rcmin = bignum, rcmax = 0.0;
  for (int i = 0; i < m; ++i) {
    rcmax = fmax(rcmax, s[i]);
    rcmin = fmin(rcmin, s[i]);
  }
  *smax = rcmax;
  if (rcmin == 0.0) {
    for (int i = 0; i < m; ++i)
      if (s[i] == 0.0) return info_base + i + 1;
  }
  for (int i = 0; i < m; ++i) s[i] = rn_div(1.0, fmin(fmax(s[i], smlnum), bignum));
  *cnd = rn_div(fmax(rcmin, smlnum), fmin(rcmax, bignum));
  return 0;
}

// DGESVX's check of given scalings (FACT = 'F', SRC/dgesvx.f:395-420):
// returns 1 when min s(i) <= 0, else 0 with *cnd = MAX(min, SMLNUM) /
// MIN(max, BIGNUM) (1 for m = 0).
GB_HD inline int scalings_cnd_seq(int m, const double* s, double* cnd) {
  const double smlnum = kSafeMin, bignum = rn_div(1.0, smlnum);
  double rcmin = bignum, rcmax = 0.0;
  for (int i = 0; i < m; ++i) {
    rcmin = fmin(rcmin, s[i]);
    rcmax = fmax(rcmax, s[i]);
  }
  if (rcmin <= 0.0) return 1;
  *cnd = m > 0 ? rn_div(fmax(rcmin, smlnum), fmin(rcmax, bignum)) : 1.0;
  return 0;
}

}  // namespace gb
