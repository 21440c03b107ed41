// The per-thread steps of the Cholesky factorization and of DSPOSV's
// refinement on the GPU (SRC/dpotrf.f:131-207, SRC/dpotrf2.f:146-205,
// SRC/dsposv.f:237-420), written once for host and device and templated on
// the element type (DPOTRF / SPOTRF).  Each function computes what one GPU
// thread computes — one element of a DSYRK / DGEMM update, one row or
// column of a DTRSM, one row sum of DLANSY, one element of DSYMM, or its
// share of a DPOTRF2 of a diagonal block — in the reference loop order with separately
// rounded operations, so that the CPU tests can compose them exactly as the
// GPU driver does and compare with the oracle bit for bit.
#pragma once
#include <cstddef>

#include "latrs_seq.h"   // GB_HD, rn_*

namespace gb {

template <typename T>
GB_HD inline T& el(T* A, int lda, int i, int j) { return A[(size_t)i + (size_t)j * lda]; }
template <typename T>
GB_HD inline T elc(const T* A, int lda, int i, int j) { return A[(size_t)i + (size_t)j * lda]; }

// The operands of these functions never overlap (a block and the block
// beside or below it), so they are restrict-qualified: the loads of a step
// can then be issued ahead of its stores.
//
// One element (i, j) of C += ALPHA*A*A**T (lower, 'L','N': i >= j; each
// term skipped when A(j, l) = 0, BLAS/SRC/dsyrk.f:313-320) or of
// C := ALPHA*(A**T*A)(i, j) + C (upper, 'U','T': i <= j, dsyrk.f:327-339).
template <typename T>
GB_HD inline void syrk_elem(int upper, int i, int j, int k, T alpha, const T* __restrict__ A, int lda,
                            T* __restrict__ C, int ldc) {
  if (!upper) {
    T c = elc(C, ldc, i, j);
    for (int l = 0; l < k; ++l) {
      const T ajl = elc(A, lda, j, l);
      if (ajl != T(0)) c = rn_add(c, rn_mul(rn_mul(alpha, ajl), elc(A, lda, i, l)));
    }
    el(C, ldc, i, j) = c;
  } else {
    T temp = T(0);
    for (int l = 0; l < k; ++l) temp = rn_add(temp, rn_mul(elc(A, lda, l, i), elc(A, lda, l, j)));
    el(C, ldc, i, j) = rn_add(rn_mul(alpha, temp), elc(C, ldc, i, j));
  }
}

// One element (i, j) of DPOTRF's DGEMM update (BETA = 1): 'N','T' (lower,
// dgemm.f:367-383) C += sum_l (ALPHA*B(j,l))*A(i,l) in l order, or 'T','N'
// (upper, dgemm.f:348-360) C := ALPHA*(sum_l A(l,i)*B(l,j)) + C.
template <typename T>
GB_HD inline void gemm_chol_elem(int upper, int i, int j, int k, T alpha, const T* A, int lda, const T* B, int ldb,
                                 T* C, int ldc) {
  if (!upper) {
    T c = elc(C, ldc, i, j);
    for (int l = 0; l < k; ++l) c = rn_add(c, rn_mul(rn_mul(alpha, elc(B, ldb, j, l)), elc(A, lda, i, l)));
    el(C, ldc, i, j) = c;
  } else {
    T temp = T(0);
    for (int l = 0; l < k; ++l) temp = rn_add(temp, rn_mul(elc(A, lda, l, i), elc(B, ldb, l, j)));
    el(C, ldc, i, j) = rn_add(rn_mul(alpha, temp), elc(C, ldc, i, j));
  }
}

// Row i of B := B*inv(A**T), A lower non-unit n x n ('R','L','T','N',
// BLAS/SRC/dtrsm.f:389-403, ALPHA = 1).
template <typename T>
GB_HD inline void trsm_rltn_row(int i, int n, const T* __restrict__ A, int lda, T* __restrict__ B, int ldb) {
  for (int k = 0; k < n; ++k) {
    el(B, ldb, i, k) = rn_div(elc(B, ldb, i, k), elc(A, lda, k, k));
    const T bk = elc(B, ldb, i, k);
    for (int j = k + 1; j < n; ++j) el(B, ldb, i, j) = rn_sub(elc(B, ldb, i, j), rn_mul(elc(A, lda, j, k), bk));
  }
}

// Column j of B := inv(A**T)*B, A upper non-unit m x m ('L','U','T','N',
// dtrsm.f:306-316, ALPHA = 1).
template <typename T>
GB_HD inline void trsm_lutn_col(int j, int m, const T* __restrict__ A, int lda, T* __restrict__ B, int ldb) {
  for (int i = 0; i < m; ++i) {
    T temp = elc(B, ldb, i, j);
    for (int k = 0; k < i; ++k) temp = rn_sub(temp, rn_mul(elc(A, lda, k, i), elc(B, ldb, k, j)));
    el(B, ldb, i, j) = rn_div(temp, elc(A, lda, i, i));
  }
}

// DPOTRF2 (SRC/dpotrf2.f:168-205) of an n x n block; returns INFO (the
// order of the first leading minor that is not positive).  The reference
// recursion (factor A11 of order N/2, DTRSM, DSYRK, factor A22) runs as a
// loop over an explicit stack of blocks, so the device code needs no call
// stack for it.  The nthr threads of a CTA (thread tid) share the work: each
// DTRSM row (lower) or column (upper) and each DSYRK element is one thread's,
// computed in the reference order as above, with sync() (a CTA barrier)
// between the dependent steps; every thread walks the same stack and returns
// the same INFO.  With tid = 0, nthr = 1 and no barrier it is the reference's
// sequential order step for step.
struct NoSync {
  GB_HD void operator()() const {}
};
template <typename T, typename Sync>
GB_HD inline int potrf2_par(int upper, int n, T* A, int lda, int tid, int nthr, Sync sync) {
  if (n == 0) return 0;
  struct Blk { int off, n, phase; };
  Blk st[40];                          // depth <= log2(n) + 1
  int top = 0;
  st[top++] = Blk{0, n, 0};
  while (top > 0) {
    Blk& b = st[top - 1];
    T* a11 = A + b.off + (size_t)b.off * lda;
    if (b.n == 1) {
      const T a = a11[0];
      sync();                          // every thread has read A(off, off)
      if (a <= T(0) || a != a) return b.off + 1;
      if (tid == 0) a11[0] = rn_sqrt(a);
      sync();
      --top;
      continue;
    }
    const int n1 = b.n / 2, n2 = b.n - n1;
    if (b.phase == 0) {
      b.phase = 1;
      st[top++] = Blk{b.off, n1, 0};
    } else if (b.phase == 1) {
      T* a12 = upper ? a11 + (size_t)n1 * lda : a11 + n1;   // A(1, N1+1) or A(N1+1, 1) of the block
      T* a22 = a11 + n1 + (size_t)n1 * lda;
      if (upper) {
        for (int j = tid; j < n2; j += nthr) trsm_lutn_col(j, n1, a11, lda, a12, lda);
        sync();
        for (int e = tid; e < n2 * n2; e += nthr) {
          const int j = e / n2, i = e - j * n2;
          if (i <= j) syrk_elem(1, i, j, n1, T(-1), a12, lda, a22, lda);
        }
      } else {
        for (int i = tid; i < n2; i += nthr) trsm_rltn_row(i, n1, a11, lda, a12, lda);
        sync();
        for (int e = tid; e < n2 * n2; e += nthr) {
          const int j = e / n2, i = e - j * n2;
          if (i >= j) syrk_elem(0, i, j, n1, T(-1), a12, lda, a22, lda);
        }
      }
      sync();
      b.phase = 2;
      st[top++] = Blk{b.off + n1, n2, 0};
    } else {
      --top;
    }
  }
  return 0;
}

// DPOTRF2 on one thread: the reference's sequential order.
template <typename T>
GB_HD inline int potrf2_seq(int upper, int n, T* A, int lda) {
  return potrf2_par(upper, n, A, lda, 0, 1, NoSync{});
}

// Row sum i of DLANSY('I') (SRC/dlansy.f:159-186) in the order the reference
// accumulates WORK(i).
GB_HD inline double lansy_row_sum(int upper, int i, int n, const double* A, int lda) {
  if (upper) {
    double s = 0.0;
    for (int k = 0; k < i; ++k) s = rn_add(s, fabs(elc(A, lda, k, i)));
    s = rn_add(s, fabs(elc(A, lda, i, i)));
    for (int j = i + 1; j < n; ++j) s = rn_add(s, fabs(elc(A, lda, i, j)));
    return s;
  }
  double s = 0.0;
  for (int j = 0; j < i; ++j) s = rn_add(s, fabs(elc(A, lda, i, j)));
  s = rn_add(s, fabs(elc(A, lda, i, i)));
  for (int k = i + 1; k < n; ++k) s = rn_add(s, fabs(elc(A, lda, k, i)));
  return s;
}

// One element (i, j) of C := ALPHA*A*B + C for symmetric A stored in one
// triangle (DSYMM('L', ...), BLAS/SRC/dsymm.f:289-323, BETA = 1), in the
// order the reference updates C(i, j).
GB_HD inline double symm_l_elem(int upper, int i, int j, int m, double alpha, const double* A, int lda,
                                const double* B, int ldb, const double* C, int ldc) {
  const double temp1 = rn_mul(alpha, elc(B, ldb, i, j));
  double temp2 = 0.0;
  double c;
  if (upper) {
    for (int k = 0; k < i; ++k) temp2 = rn_add(temp2, rn_mul(elc(B, ldb, k, j), elc(A, lda, k, i)));
    c = rn_add(rn_add(elc(C, ldc, i, j), rn_mul(temp1, elc(A, lda, i, i))), rn_mul(alpha, temp2));
    for (int ii = i + 1; ii < m; ++ii) c = rn_add(c, rn_mul(rn_mul(alpha, elc(B, ldb, ii, j)), elc(A, lda, i, ii)));
  } else {
    for (int k = i + 1; k < m; ++k) temp2 = rn_add(temp2, rn_mul(elc(B, ldb, k, j), elc(A, lda, k, i)));
    c = rn_add(rn_add(elc(C, ldc, i, j), rn_mul(temp1, elc(A, lda, i, i))), rn_mul(alpha, temp2));
    for (int ii = i - 1; ii >= 0; --ii) c = rn_add(c, rn_mul(rn_mul(alpha, elc(B, ldb, ii, j)), elc(A, lda, i, ii)));
  }
  return c;
}

}  // namespace gb
