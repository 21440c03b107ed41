// Kernels of DGECON on the GPU (SRC/dgecon.f:166-252): the DLATRS
// (SRC/dlatrs.f:264-847) triangular solves with overflow protection and the
// DRSCL (SRC/drscl.f:105-133) rescaling, for one vector in device memory.
//
// DLATRS runs in three parts: CNORM (column sums of the off-diagonal
// part, once per triangle), a one-CTA plan kernel (TSCAL, the growth bound
// and the choice between a plain DTRSV and the careful solve), then either
// the library's triangular solve or the one-CTA careful column sweep.  All
// scalar arithmetic is separately rounded (no contraction), as the
// reference Fortran evaluates it; MIN / MAX are fmin / fmax.
#pragma once
#include "refine_kernels.cuh"

namespace gb {

constexpr double kSafeMin = 2.2250738585072014e-308;   // DLAMCH('Safe minimum')
constexpr double kPrec = 2.220446049250313e-16;        // DLAMCH('Precision')
constexpr double kOvfl = 1.7976931348623157e308;       // DLAMCH('Overflow')

enum LatrsMode : int { kLatrsTrsv = 0, kLatrsCareful = 1, kLatrsDirect = 2 };

// What the plan kernel decided for one DLATRS call.
struct LatrsPlan {
  int mode;        // LatrsMode
  double tscal;    // TSCAL
  double xmax;     // |X(IDAMAX(X))| before the solve
  double scale;    // SCALE (1 unless the careful solve scaled X)
};

// ------------------------------------------------------------- CNORM
// CNORM(j) = DASUM of the off-diagonal part of column j (dlatrs.f:322-338):
// rows 1..j-1 for the upper triangle, j+1..n for the lower.  EXACT: one
// thread per column, the reference's left-to-right sum; otherwise one warp
// per column with a fixed shuffle tree.
template <bool EXACT>
__global__ void __launch_bounds__(256)
latrs_cnorm_kernel(int upper, int n, const double* __restrict__ A, int lda, double* __restrict__ cnorm) {
  if (EXACT) {
    const int j = blockIdx.x * 256 + threadIdx.x;
    if (j >= n) return;
    const int i0 = upper ? 0 : j + 1, i1 = upper ? j : n;
    const double* col = A + (size_t)j * lda;
    double s = 0.0;
    for (int i = i0; i < i1; ++i) s = __dadd_rn(s, fabs(col[i]));
    cnorm[j] = s;
  } else {
    const int j = blockIdx.x * 8 + (threadIdx.x >> 5), lane = threadIdx.x & 31;
    if (j >= n) return;
    const int i0 = upper ? 0 : j + 1, i1 = upper ? j : n;
    const double* col = A + (size_t)j * lda;
    double s = 0.0;
    for (int i = i0 + lane; i < i1; i += 32) s += fabs(col[i]);
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
    if (lane == 0) cnorm[j] = s;
  }
}

// ------------------------------------------------------------- block tools
// For one CTA of kCtaThreads threads; each ends with a barrier so that the
// next step sees the result.
constexpr int kCtaThreads = 1024;

__device__ __forceinline__ void cta_scal(int n, double a, double* x) {
  if (a == 1.0) return;   // BLAS/SRC/dscal.f quick return
  __syncthreads();        // every earlier read of x precedes the update
  for (int i = threadIdx.x; i < n; i += kCtaThreads) x[i] = __dmul_rn(a, x[i]);
  __syncthreads();
}

// IDAMAX over x[0..n), 1-based (0 for n < 1).
__device__ int cta_idamax(int n, const double* x, Cand<double>* red) {
  if (n < 1) return 0;
  Cand<double> best;
  best.absval = 0;
  best.row = -1;
  best.cls = -1;
  for (int i = threadIdx.x; i < n; i += kCtaThreads) {
    Cand<double> c = make_cand(x[i], i, 0);
    if (cand_better(c, best)) best = c;
  }
  best = warp_best(best);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = best;
  __syncthreads();
  Cand<double> b = red[0];
  for (int w = 1; w < kCtaThreads / 32; ++w)
    if (cand_better(red[w], b)) b = red[w];
  __syncthreads();
  return b.row + 1;
}

// sum_i f(i) over i in [0, n): EXACT left to right on one thread, else a
// fixed tree.  Every thread gets the result.
template <bool EXACT, typename F>
__device__ double cta_sum(int n, F f, double* red) {
  double s = 0.0;
  if (EXACT) {
    if (threadIdx.x == 0)
      for (int i = 0; i < n; ++i) s = __dadd_rn(s, f(i));
  } else {
    for (int i = threadIdx.x; i < n; i += kCtaThreads) s += f(i);
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
  }
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  double t = red[0];
  if (!EXACT)
    for (int w = 1; w < kCtaThreads / 32; ++w) t += red[w];
  __syncthreads();
  return t;
}

__device__ __forceinline__ double cta_max_abs(int n, const double* x, double* red) {
  double m = 0.0;
  for (int i = threadIdx.x; i < n; i += kCtaThreads) {
    const double t = fabs(x[i]);
    if (m < t || t != t) m = t;
  }
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    const double o = __shfl_xor_sync(0xffffffffu, m, off);
    if (m < o || o != o) m = o;
  }
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
  __syncthreads();
  double t = red[0];
  for (int w = 1; w < kCtaThreads / 32; ++w)
    if (t < red[w] || red[w] != red[w]) t = red[w];
  __syncthreads();
  return t;
}

// ------------------------------------------------------------- plan
// dlatrs.f:340-503 up to the choice of solve: TSCAL from max CNORM (with
// CNORM scaled in place when it exceeds BIGNUM), XMAX, the growth bound
// GROW, then DTRSV when GROW*TSCAL > SMLNUM, else the careful solve.  One
// CTA; the growth loops run on thread 0 (they are sequential recurrences).
__global__ void __launch_bounds__(kCtaThreads)
latrs_plan_kernel(int upper, int notran, int nounit, int n, const double* __restrict__ A, int lda,
                  const double* __restrict__ x, double* __restrict__ cnorm, LatrsPlan* __restrict__ plan) {
  __shared__ Cand<double> cred[kCtaThreads / 32];
  __shared__ double red[kCtaThreads / 32];
  __shared__ double grow_s;
  const double smlnum = __ddiv_rn(kSafeMin, kPrec), bignum = __ddiv_rn(1.0, smlnum);
  const int imax = cta_idamax(n, cnorm, cred);
  double tmax = cnorm[imax - 1];
  double tscal = 1.0;
  int direct = 0;
  if (tmax <= bignum) {
    tscal = 1.0;
  } else if (tmax <= kOvfl) {
    tscal = __ddiv_rn(1.0, __dmul_rn(smlnum, tmax));
    cta_scal(n, tscal, cnorm);
  } else {
    // a column sum overflowed: TMAX = the largest off-diagonal |A(i,j)|
    double m = 0.0;
    for (int j = 0; j < n; ++j) {
      const int i0 = upper ? 0 : j + 1, i1 = upper ? j : n;
      if (i1 <= i0) continue;
      const double mj = cta_max_abs(i1 - i0, A + (size_t)j * lda + i0, red);
      m = fmax(mj, m);
    }
    tmax = m;
    if (tmax <= kOvfl) {
      tscal = __ddiv_rn(1.0, __dmul_rn(smlnum, tmax));
      for (int j = threadIdx.x; j < n; j += kCtaThreads) {
        if (cnorm[j] <= kOvfl) {
          cnorm[j] = __dmul_rn(cnorm[j], tscal);
        } else {
          const int i0 = upper ? 0 : j + 1, i1 = upper ? j : n;
          double s = 0.0;
          for (int i = i0; i < i1; ++i) s = __dadd_rn(s, __dmul_rn(tscal, fabs(A[(size_t)i + (size_t)j * lda])));
          cnorm[j] = s;
        }
      }
      __syncthreads();
    } else {
      direct = 1;
    }
  }
  const int jx = cta_idamax(n, x, cred);
  const double xmax = fabs(x[jx - 1]);
  if (threadIdx.x == 0 && !direct) {
    double xbnd = xmax, grow;
    int jfirst, jlast, jinc;
    if (notran == upper) { jfirst = n - 1; jlast = 0; jinc = -1; }   // 'N' upper, 'T' lower
    else { jfirst = 0; jlast = n - 1; jinc = 1; }
    const double* diag = A;
    if (tscal != 1.0) {
      grow = 0.0;
    } else if (notran) {
      if (nounit) {
        grow = __ddiv_rn(1.0, fmax(xbnd, smlnum));
        xbnd = grow;
        bool cut = false;
        for (int j = jfirst; j != jlast + jinc; j += jinc) {
          if (grow <= smlnum) { cut = true; break; }
          const double tjj = fabs(diag[(size_t)j * (lda + 1)]);
          xbnd = fmin(xbnd, __dmul_rn(fmin(1.0, tjj), grow));
          const double den = __dadd_rn(tjj, cnorm[j]);
          grow = (den >= smlnum) ? __dmul_rn(grow, __ddiv_rn(tjj, den)) : 0.0;
        }
        if (!cut) grow = xbnd;
      } else {
        grow = fmin(1.0, __ddiv_rn(1.0, fmax(xbnd, smlnum)));
        for (int j = jfirst; j != jlast + jinc; j += jinc) {
          if (grow <= smlnum) break;
          grow = __dmul_rn(grow, __ddiv_rn(1.0, __dadd_rn(1.0, cnorm[j])));
        }
      }
    } else {
      if (nounit) {
        grow = __ddiv_rn(1.0, fmax(xbnd, smlnum));
        xbnd = grow;
        bool cut = false;
        for (int j = jfirst; j != jlast + jinc; j += jinc) {
          if (grow <= smlnum) { cut = true; break; }
          const double xj = __dadd_rn(1.0, cnorm[j]);
          grow = fmin(grow, __ddiv_rn(xbnd, xj));
          const double tjj = fabs(diag[(size_t)j * (lda + 1)]);
          if (xj > tjj) xbnd = __dmul_rn(xbnd, __ddiv_rn(tjj, xj));
        }
        if (!cut) grow = fmin(grow, xbnd);
      } else {
        grow = fmin(1.0, __ddiv_rn(1.0, fmax(xbnd, smlnum)));
        for (int j = jfirst; j != jlast + jinc; j += jinc) {
          if (grow <= smlnum) break;
          grow = __ddiv_rn(grow, __dadd_rn(1.0, cnorm[j]));
        }
      }
    }
    grow_s = grow;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    LatrsPlan p;
    p.tscal = tscal;
    p.xmax = xmax;
    p.scale = 1.0;
    p.mode = direct ? kLatrsDirect : (__dmul_rn(grow_s, tscal) > smlnum ? kLatrsTrsv : kLatrsCareful);
    *plan = p;
  }
}

// ------------------------------------------------------------- careful solve
// dlatrs.f:505-772: the column sweep that rescales X (and SCALE) whenever
// the next step could overflow, then SCALE = SCALE / TSCAL and CNORM back
// to its unscaled value.  One CTA; scalar decisions are computed by every
// thread from the same values, vector updates are spread over the CTA and
// end with a barrier, X(j) is written by thread 0.
template <bool EXACT>
__global__ void __launch_bounds__(kCtaThreads)
latrs_careful_kernel(int upper, int notran, int nounit, int n, const double* __restrict__ A, int lda,
                     double* __restrict__ x, double* __restrict__ cnorm, LatrsPlan* __restrict__ plan) {
  __shared__ Cand<double> cred[kCtaThreads / 32];
  __shared__ double red[kCtaThreads / 32];
  const double smlnum = __ddiv_rn(kSafeMin, kPrec), bignum = __ddiv_rn(1.0, smlnum);
  const double tscal = plan->tscal;
  double xmax = plan->xmax, scale = 1.0;
  auto Aij = [&](int i, int j) { return A[(size_t)i + (size_t)j * lda]; };
  auto set_xj = [&](int j, double v) {
    __syncthreads();
    if (threadIdx.x == 0) x[j] = v;
    __syncthreads();
  };
  auto zero_but = [&](int j) {   // X = e_j
    __syncthreads();
    for (int i = threadIdx.x; i < n; i += kCtaThreads) x[i] = (i == j) ? 1.0 : 0.0;
    __syncthreads();
  };
  int jfirst, jinc;
  if (notran == upper) { jfirst = n - 1; jinc = -1; }
  else { jfirst = 0; jinc = 1; }
  if (xmax > bignum) {
    scale = __ddiv_rn(bignum, xmax);
    cta_scal(n, scale, x);
    xmax = bignum;
  }
  for (int step = 0, j = jfirst; step < n; ++step, j += jinc) {
    double xj = fabs(x[j]), tjjs = 0.0, tjj, rec;
    if (notran) {
      bool skip = false;
      if (nounit) {
        tjjs = __dmul_rn(Aij(j, j), tscal);
      } else {
        tjjs = tscal;
        if (tscal == 1.0) skip = true;
      }
      if (!skip) {
        tjj = fabs(tjjs);
        if (tjj > smlnum) {
          if (tjj < 1.0 && xj > __dmul_rn(tjj, bignum)) {
            rec = __ddiv_rn(1.0, xj);
            cta_scal(n, rec, x);
            scale = __dmul_rn(scale, rec);
            xmax = __dmul_rn(xmax, rec);
          }
          set_xj(j, __ddiv_rn(x[j], tjjs));
          xj = fabs(x[j]);
        } else if (tjj > 0.0) {
          if (xj > __dmul_rn(tjj, bignum)) {
            rec = __ddiv_rn(__dmul_rn(tjj, bignum), xj);
            if (cnorm[j] > 1.0) rec = __ddiv_rn(rec, cnorm[j]);
            cta_scal(n, rec, x);
            scale = __dmul_rn(scale, rec);
            xmax = __dmul_rn(xmax, rec);
          }
          set_xj(j, __ddiv_rn(x[j], tjjs));
          xj = fabs(x[j]);
        } else {
          zero_but(j);
          xj = 1.0;
          scale = 0.0;
          xmax = 0.0;
        }
      }
      if (xj > 1.0) {
        rec = __ddiv_rn(1.0, xj);
        if (cnorm[j] > __dmul_rn(__dsub_rn(bignum, xmax), rec)) {
          rec = __dmul_rn(rec, 0.5);
          cta_scal(n, rec, x);
          scale = __dmul_rn(scale, rec);
        }
      } else if (__dmul_rn(xj, cnorm[j]) > __dsub_rn(bignum, xmax)) {
        cta_scal(n, 0.5, x);
        scale = __dmul_rn(scale, 0.5);
      }
      // DAXPY of the rest of column j, then XMAX over the part still to solve
      const int lo = upper ? 0 : j + 1, len = upper ? j : n - j - 1;
      if (len > 0) {
        const double alpha = __dmul_rn(-x[j], tscal);
        __syncthreads();
        if (alpha != 0.0)   // BLAS/SRC/daxpy.f quick return
          for (int i = threadIdx.x; i < len; i += kCtaThreads)
            x[lo + i] = __dadd_rn(x[lo + i], __dmul_rn(alpha, Aij(lo + i, j)));
        __syncthreads();
        const int im = cta_idamax(len, x + lo, cred);
        xmax = fabs(x[lo + im - 1]);
      }
    } else {
      double uscal = tscal;
      rec = __ddiv_rn(1.0, fmax(xmax, 1.0));
      if (cnorm[j] > __dmul_rn(__dsub_rn(bignum, xj), rec)) {
        rec = __dmul_rn(rec, 0.5);
        tjjs = nounit ? __dmul_rn(Aij(j, j), tscal) : tscal;
        tjj = fabs(tjjs);
        if (tjj > 1.0) {
          rec = fmin(1.0, __dmul_rn(rec, tjj));
          uscal = __ddiv_rn(uscal, tjjs);
        }
        if (rec < 1.0) {
          cta_scal(n, rec, x);
          scale = __dmul_rn(scale, rec);
          xmax = __dmul_rn(xmax, rec);
        }
      }
      const int lo = upper ? 0 : j + 1, len = upper ? j : n - j - 1;
      double sumj = 0.0;
      if (len > 0) {
        __syncthreads();
        if (uscal == 1.0)
          sumj = cta_sum<EXACT>(len, [&](int i) { return __dmul_rn(Aij(lo + i, j), x[lo + i]); }, red);
        else
          sumj = cta_sum<EXACT>(len, [&](int i) { return __dmul_rn(__dmul_rn(Aij(lo + i, j), uscal), x[lo + i]); },
                                red);
      }
      if (uscal == tscal) {
        set_xj(j, __dsub_rn(x[j], sumj));
        xj = fabs(x[j]);
        bool skip = false;
        if (nounit) {
          tjjs = __dmul_rn(Aij(j, j), tscal);
        } else {
          tjjs = tscal;
          if (tscal == 1.0) skip = true;
        }
        if (!skip) {
          tjj = fabs(tjjs);
          if (tjj > smlnum) {
            if (tjj < 1.0 && xj > __dmul_rn(tjj, bignum)) {
              rec = __ddiv_rn(1.0, xj);
              cta_scal(n, rec, x);
              scale = __dmul_rn(scale, rec);
              xmax = __dmul_rn(xmax, rec);
            }
            set_xj(j, __ddiv_rn(x[j], tjjs));
          } else if (tjj > 0.0) {
            if (xj > __dmul_rn(tjj, bignum)) {
              rec = __ddiv_rn(__dmul_rn(tjj, bignum), xj);
              cta_scal(n, rec, x);
              scale = __dmul_rn(scale, rec);
              xmax = __dmul_rn(xmax, rec);
            }
            set_xj(j, __ddiv_rn(x[j], tjjs));
          } else {
            zero_but(j);
            scale = 0.0;
            xmax = 0.0;
          }
        }
      } else {
        set_xj(j, __dsub_rn(__ddiv_rn(x[j], tjjs), sumj));
      }
      xmax = fmax(xmax, fabs(x[j]));
    }
    __syncthreads();
  }
  scale = __ddiv_rn(scale, tscal);
  if (tscal != 1.0) cta_scal(n, __ddiv_rn(1.0, tscal), cnorm);
  if (threadIdx.x == 0) plan->scale = scale;
}

// ------------------------------------------------------------- DGECON step
// After the two DLATRS solves of one estimator step (dgecon.f:222-238):
// SCALE = SL*SU; if SCALE != 1, stop the estimate (RCOND = 0) when
// SCALE < |X(IDAMAX)|*SMLNUM or SCALE = 0, else X := X / SCALE by DRSCL.
// *stop receives 1 when the estimate stops.
__global__ void __launch_bounds__(kCtaThreads)
gecon_rescale_kernel(int n, double* __restrict__ x, const LatrsPlan* __restrict__ pl,
                     const LatrsPlan* __restrict__ pu, int* __restrict__ stop) {
  __shared__ Cand<double> cred[kCtaThreads / 32];
  const double scale = __dmul_rn(pl->scale, pu->scale);
  if (scale == 1.0) return;
  const int ix = cta_idamax(n, x, cred);
  if (scale < __dmul_rn(fabs(x[ix - 1]), kSafeMin) || scale == 0.0) {
    if (threadIdx.x == 0) *stop = 1;
    return;
  }
  // DRSCL: multiply by SMLNUM or BIGNUM until the remaining factor is safe
  const double smlnum = kSafeMin, bignum = __ddiv_rn(1.0, smlnum);
  double cden = scale, cnum = 1.0;
  for (int guard = 0; guard < 64; ++guard) {
    const double cden1 = __dmul_rn(cden, smlnum), cnum1 = __ddiv_rn(cnum, bignum);
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
      mul = __ddiv_rn(cnum, cden);
      done = true;
    }
    cta_scal(n, mul, x);
    if (done) break;
  }
}

}  // namespace gb
