// The element steps of DGETRI (SRC/dgetri.f:169-262) and of the upper
// triangular inverse it starts with (SRC/dtrtri.f:149-196,
// SRC/dtrti2.f:128-160), written once for host and device.  Each function
// computes what one GPU thread computes (one element, one row, or one small
// diagonal block), in the reference loop order with every operation
// separately rounded, so that the CPU tests can compose them with the
// oracle's DGEMM and compare the result bit for bit with the oracle's DGETRI.
#pragma once
#include <cstddef>

#include "latrs_seq.h"   // GB_HD, rn_*

namespace gb {

// One element (i, c) of B := A*B for the upper triangle A (m x m, non-unit)
// of BLAS/SRC/dtrmm.f:271-283 with ALPHA = 1: the diagonal term first, then
// the terms of rows k = i+1..m-1 in increasing k.  B0 is the block before the
// product (the reference reads B(k, c) before it is overwritten).
GB_HD inline double trmm_lun_elem(int i, int c, int m, const double* A, int lda, const double* B0, int ldb0) {
  const double* b = B0 + (size_t)c * ldb0;
  double v = rn_mul(b[i], A[(size_t)i + (size_t)i * lda]);
  for (int k = i + 1; k < m; ++k) v = rn_add(v, rn_mul(b[k], A[(size_t)i + (size_t)k * lda]));
  return v;
}

// Row i of B := ALPHA*B*inv(T) (BLAS/SRC/dtrsm.f:333-367) for the n x n
// triangle T (upper non-unit, or lower unit), B with n columns.
GB_HD inline void trsm_rn_row(int i, int upper, int nounit, int n, double alpha, const double* T, int ldt, double* B,
                              int ldb) {
  double* b = B + i;
  auto bb = [&](int col) -> double& { return b[(size_t)col * ldb]; };
  if (upper) {
    for (int j = 0; j < n; ++j) {
      bb(j) = rn_mul(alpha, bb(j));
      for (int k = 0; k < j; ++k) bb(j) = rn_sub(bb(j), rn_mul(T[(size_t)k + (size_t)j * ldt], bb(k)));
      if (nounit) bb(j) = rn_div(bb(j), T[(size_t)j + (size_t)j * ldt]);
    }
  } else {
    for (int j = n - 1; j >= 0; --j) {
      bb(j) = rn_mul(alpha, bb(j));
      for (int k = j + 1; k < n; ++k) bb(j) = rn_sub(bb(j), rn_mul(T[(size_t)k + (size_t)j * ldt], bb(k)));
      if (nounit) bb(j) = rn_div(bb(j), T[(size_t)j + (size_t)j * ldt]);
    }
  }
}

// DTRTI2('U', 'N') of an n x n block (SRC/dtrti2.f:128-143 with DTRMV,
// BLAS/SRC/dtrmv.f:226-235, and DSCAL).
GB_HD inline void trti2_upper_seq(int n, double* A, int lda) {
  auto a = [&](int i, int j) -> double& { return A[(size_t)i + (size_t)j * lda]; };
  for (int j = 0; j < n; ++j) {
    a(j, j) = rn_div(1.0, a(j, j));
    const double ajj = -a(j, j);
    double* x = &a(0, j);
    for (int jj = 0; jj < j; ++jj) {
      const double temp = x[jj];
      for (int i = 0; i < jj; ++i) x[i] = rn_add(x[i], rn_mul(temp, a(i, jj)));
      x[jj] = rn_mul(x[jj], a(jj, jj));
    }
    if (ajj != 1.0)
      for (int i = 0; i < j; ++i) x[i] = rn_mul(ajj, x[i]);
  }
}

// Row i of the unblocked DGETRI step for column j (dgetri.f:221-229): the
// DGEMV A(:, j) += sum_{jj > j} (-WORK(jj)) * A(:, jj), jj increasing.
GB_HD inline void getri_gemv_row(int i, int j, int n, double* A, int lda, const double* work) {
  double v = A[(size_t)i + (size_t)j * lda];
  for (int jj = j + 1; jj < n; ++jj) v = rn_add(v, rn_mul(rn_mul(-1.0, work[jj]), A[(size_t)i + (size_t)jj * lda]));
  A[(size_t)i + (size_t)j * lda] = v;
}

// Row i of the column interchanges that end DGETRI (dgetri.f:255-260):
// columns j and IPIV(j) swapped for j = N-1 down to 1.
GB_HD inline void getri_swap_row(int i, int n, double* A, int lda, const int* ipiv) {
  for (int j = n - 2; j >= 0; --j) {
    const int jp = ipiv[j] - 1;
    if (jp != j) {
      const double t = A[(size_t)i + (size_t)j * lda];
      A[(size_t)i + (size_t)j * lda] = A[(size_t)i + (size_t)jp * lda];
      A[(size_t)i + (size_t)jp * lda] = t;
    }
  }
}

}  // namespace gb
