// Kernels of DGECON on the GPU (SRC/dgecon.f:166-252): the DLATRS
// (SRC/dlatrs.f:264-847) triangular solves with overflow protection and the
// DRSCL (SRC/drscl.f:105-133) rescaling, for one vector in device memory.
//
// DLATRS runs in three parts: CNORM (column sums of the off-diagonal
// part, once per triangle, over all columns in parallel), the plan (TSCAL,
// the growth bound, the choice between a plain DTRSV and the careful
// solve), then either the library's triangular solve or the careful column
// sweep.  The plan, the careful sweep and DGECON's rescaling step are
// sequential recurrences; each runs as a one-thread kernel over the shared
// host/device code of latrs_seq.h, which the CPU tests check bit for bit
// against the oracle.
#pragma once
#include "latrs_seq.h"
#include "refine_kernels.cuh"

namespace gb {

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

// ------------------------------------------------------------- sweeps
__global__ void __launch_bounds__(1)
latrs_plan_kernel(int upper, int notran, int nounit, int n, const double* __restrict__ A, int lda,
                  const double* __restrict__ x, double* __restrict__ cnorm, LatrsPlan* __restrict__ plan) {
  latrs_plan_seq(upper, notran, nounit, n, A, lda, x, cnorm, plan);
}

__global__ void __launch_bounds__(1)
latrs_careful_kernel(int upper, int notran, int nounit, int n, const double* __restrict__ A, int lda,
                     double* __restrict__ x, double* __restrict__ cnorm, LatrsPlan* __restrict__ plan) {
  latrs_careful_seq(upper, notran, nounit, n, A, lda, x, cnorm, plan);
}

// *stop = 1 when DGECON's estimate stops with RCOND = 0 (dgecon.f:236).
__global__ void __launch_bounds__(1)
gecon_rescale_kernel(int n, double* __restrict__ x, const LatrsPlan* __restrict__ pl,
                     const LatrsPlan* __restrict__ pu, int* __restrict__ stop) {
  if (gecon_rescale_seq(n, x, pl->scale, pu->scale)) *stop = 1;
}

}  // namespace gb

namespace gb {

// ------------------------------------------------------------- DGESVX
// DGEEQU (SRC/dgeequ.f): row maxima R(i) = MAX_j |A(i,j)| (one thread per
// row, columns in order), column maxima C(j) = MAX_i |A(i,j)|*R(i) (one
// warp per column); maxima are order-free, so these equal the reference's.
__global__ void geequ_rowmax_kernel(const double* __restrict__ A, int lda, int m, int n, double* __restrict__ r) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= m) return;
  double v = 0.0;
  for (int j = 0; j < n; ++j) v = fmax(v, fabs(A[(size_t)i + (size_t)j * lda]));
  r[i] = v;
}

__global__ void __launch_bounds__(256)
geequ_colmax_kernel(const double* __restrict__ A, int lda, int m, int n, const double* __restrict__ r,
                    double* __restrict__ c) {
  const int j = blockIdx.x * 8 + (threadIdx.x >> 5), lane = threadIdx.x & 31;
  if (j >= n) return;
  const double* col = A + (size_t)j * lda;
  double v = 0.0;
  for (int i = lane; i < m; i += 32) v = fmax(v, __dmul_rn(fabs(col[i]), r[i]));
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, off));
  if (lane == 0) c[j] = v;
}

// What DGEEQU / the FACT = 'F' check report back: condition numbers of the
// scalings, AMAX and INFO.
struct EquStat {
  double rowcnd, colcnd, amax;
  int info;
};

// DGEEQU's two finishing steps on one thread (the R step, then, when it
// found no zero row, the C maxima must already be in c).  step 0: rows;
// step 1: columns.
__global__ void __launch_bounds__(1) equ_finish_kernel(int step, int m, int n, double* __restrict__ s,
                                                       EquStat* __restrict__ st) {
  double smax = 0.0;
  if (step == 0) {
    st->info = equ_finish_seq(m, s, 0, &st->rowcnd, &smax);
    st->amax = smax;
  } else {
    st->info = equ_finish_seq(n, s, m, &st->colcnd, &smax);
  }
}

// FACT = 'F': MIN(s) <= 0 check and the condition number of given R or C.
__global__ void __launch_bounds__(1) scalings_cnd_kernel(int n, const double* __restrict__ s, double* __restrict__ cnd,
                                                         int* __restrict__ bad) {
  *bad = scalings_cnd_seq(n, s, cnd);
}

// A(i,j) := C(j)*A(i,j), R(i)*A(i,j) or (C(j)*R(i))*A(i,j) (DLAQGE,
// SRC/dlaqge.f:159-186; also the right-hand-side scalings of DGESVX and
// the unscaling of X, with c = NULL).
__global__ void scale_rows_cols_kernel(double* __restrict__ A, int lda, int m, int n, const double* __restrict__ r,
                                       const double* __restrict__ c) {
  const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (size_t)m * n) return;
  const int j = (int)(e / m), i = (int)(e - (size_t)j * m);
  double* p = A + (size_t)i + (size_t)j * lda;
  if (c && r) *p = __dmul_rn(__dmul_rn(c[j], r[i]), *p);
  else if (c) *p = __dmul_rn(c[j], *p);
  else *p = __dmul_rn(r[i], *p);
}

// max |A(i,j)| over i <= min(m-1, j) (DLANTR('M','U','N'), SRC/dlantr.f:173-182)
// or over the whole m x n block (DLANGE('M')), NaN propagating: a NaN sets
// *nanflag, otherwise the bit patterns of |a| are maximised.
__global__ void max_abs_tri_kernel(const double* __restrict__ A, int lda, int m, int n, int upper,
                                   unsigned long long* __restrict__ bits, int* __restrict__ nanflag) {
  const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (size_t)m * n) return;
  const int j = (int)(e / m), i = (int)(e - (size_t)j * m);
  if (upper && i > j) return;
  const double v = A[(size_t)i + (size_t)j * lda];
  if (v != v) { *nanflag = 1; return; }
  atomicMax(bits, (unsigned long long)__double_as_longlong(fabs(v)));
}

// FERR(j) := FERR(j) / cnd (dgesvx.f:566-585).
__global__ void div_by_kernel(double* __restrict__ v, int n, double cnd) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) v[i] = __ddiv_rn(v[i], cnd);
}

}  // namespace gb

#include "getri_seq.h"

namespace gb {

// ------------------------------------------------------------- DGETRI
// First zero on the diagonal (DTRTRI's INFO, SRC/dtrtri.f:134-139): the
// smallest such index, 1-based, by an order-free atomicMin.
__global__ void first_zero_diag_kernel(const double* __restrict__ A, int lda, int n, int* __restrict__ first) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n && A[(size_t)i + (size_t)i * lda] == 0.0) atomicMin(first, i + 1);
}

// B := A*B (DTRMM left, upper, non-unit, ALPHA = 1) from the copy B0.
__global__ void trmm_lun_kernel(int m, int ncols, const double* __restrict__ A, int lda, const double* __restrict__ B0,
                                int ldb0, double* __restrict__ B, int ldb) {
  const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (size_t)m * ncols) return;
  const int c = (int)(e / m), i = (int)(e - (size_t)c * m);
  B[(size_t)i + (size_t)c * ldb] = trmm_lun_elem(i, c, m, A, lda, B0, ldb0);
}

// B := ALPHA*B*inv(T), one thread per row of B.
__global__ void trsm_rn_kernel(int m, int upper, int nounit, int n, double alpha, const double* __restrict__ T,
                               int ldt, double* __restrict__ B, int ldb) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < m) trsm_rn_row(i, upper, nounit, n, alpha, T, ldt, B, ldb);
}

// DTRTI2 of one diagonal block (at most the block size), on one thread.
__global__ void __launch_bounds__(1) trti2_upper_kernel(int n, double* __restrict__ A, int lda) {
  trti2_upper_seq(n, A, lda);
}

// WORK(:, c) = the strictly lower part of column j0 + c, which is then zeroed
// (dgetri.f:222-226, 236-241); rows <= j0 + c of WORK are left as they are.
__global__ void getri_take_l_kernel(int n, int j0, int jb, double* __restrict__ A, int lda, double* __restrict__ W,
                                    int ldw) {
  const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (size_t)n * jb) return;
  const int c = (int)(e / n), i = (int)(e - (size_t)c * n);
  const int jj = j0 + c;
  if (i <= jj) return;
  double* a = A + (size_t)i + (size_t)jj * lda;
  W[(size_t)i + (size_t)c * ldw] = *a;
  *a = 0.0;
}

__global__ void getri_gemv_kernel(int n, int j, double* __restrict__ A, int lda, const double* __restrict__ w) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) getri_gemv_row(i, j, n, A, lda, w);
}

__global__ void getri_swap_kernel(int n, double* __restrict__ A, int lda, const int* __restrict__ ipiv) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) getri_swap_row(i, n, A, lda, ipiv);
}

}  // namespace gb
