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
