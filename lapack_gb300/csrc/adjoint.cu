// Adjoint of X = A^{-1} B reusing the stored LU factors and IPIV:
//   gB = A^{-T} gX   (DGETRS('T'), SRC/dgetrs.f:199-217, on the stored factors)
//   gA = -gB X^T     (DGEMM('N','T', alpha=-1, gB, X, beta=0), BLAS/SRC/dgemm.f:363-383)
// The rank-nrhs product writes every element of gA exactly once (n^2 doubles
// out, n*nrhs doubles in per operand), so it is bound by the HBM write of gA;
// each element folds its nrhs products in the reference order (l = 1..K,
// C(i,j) = C(i,j) + (-X(j,l)) * gB(i,l) starting from zero).
#include "../../include/lapack_gb300.h"
#include "common.cuh"
#include "driver.h"
#include "prof.h"

namespace gb {
namespace {

constexpr int kAdjRows = 64;     // rows of gA per CTA tile (64 threads x 4 columns each)
constexpr int kAdjCols = 64;
constexpr int kAdjMaxRhs = 16;

template <bool EXACT>
__global__ void __launch_bounds__(256)
rank_update_neg_kernel(int n, int nrhs, const double* __restrict__ GB, int ldgb, const double* __restrict__ X, int ldx,
                       double* __restrict__ GA, int ldga) {
  __shared__ double gbs[kAdjMaxRhs][kAdjRows];
  __shared__ double xs[kAdjMaxRhs][kAdjCols];
  const int i0 = blockIdx.x * kAdjRows, j0 = blockIdx.y * kAdjCols;
  const int tid = threadIdx.x;
  for (int e = tid; e < nrhs * kAdjRows; e += 256) {
    const int q = e / kAdjRows, r = e - q * kAdjRows;
    gbs[q][r] = (i0 + r < n) ? GB[(size_t)(i0 + r) + (size_t)q * ldgb] : 0.0;
  }
  for (int e = tid; e < nrhs * kAdjCols; e += 256) {
    const int q = e / kAdjCols, c = e - q * kAdjCols;
    xs[q][c] = (j0 + c < n) ? X[(size_t)(j0 + c) + (size_t)q * ldx] : 0.0;
  }
  __syncthreads();
  const int r = tid & 63, cg = tid >> 6;       // 4 column groups of 16 columns
  if (i0 + r >= n) return;
#pragma unroll 4
  for (int cc = 0; cc < kAdjCols / 4; ++cc) {
    const int c = cg * (kAdjCols / 4) + cc;
    if (j0 + c >= n) break;
    double acc = 0.0;
    for (int q = 0; q < nrhs; ++q) acc = fmadd<EXACT>(-xs[q][c], gbs[q][r], acc);
    GA[(size_t)(i0 + r) + (size_t)(j0 + c) * ldga] = acc;
  }
}

}  // namespace

int adjoint_dev(int n, int nrhs, const double* dLU, int ldlu, const int* dIpiv, const double* dX, int ldx,
                const double* dGX, int ldgx, double* dGB, int ldgb, double* dGA, int ldga, cudaStream_t s) {
  if (n <= 0 || nrhs <= 0) return 0;
  if (nrhs > kAdjMaxRhs) return (int)cudaErrorInvalidValue;
  // gB := gX, then the transposed solve in place
  GB_CUDA_TRY(cudaMemcpy2DAsync(dGB, sizeof(double) * ldgb, dGX, sizeof(double) * ldgx, sizeof(double) * n, nrhs,
                                cudaMemcpyDeviceToDevice, s));
  int rc = getrs_dev<double>('T', n, nrhs, dLU, ldlu, dIpiv, nullptr, dGB, ldgb, s);
  if (rc) return rc;
  if (dGA) {
    dim3 grid((n + kAdjRows - 1) / kAdjRows, (n + kAdjCols - 1) / kAdjCols);
    prof_begin(kProfOther, s);
    if (options().exact)
      GB_LAUNCH(rank_update_neg_kernel<true><<<grid, 256, 0, s>>>(n, nrhs, dGB, ldgb, dX, ldx, dGA, ldga));
    else
      GB_LAUNCH(rank_update_neg_kernel<false><<<grid, 256, 0, s>>>(n, nrhs, dGB, ldgb, dX, ldx, dGA, ldga));
    prof_end(kProfOther, s, 2.0 * n * (double)n * nrhs, 8.0 * ((double)n * n + 2.0 * n * nrhs));
  }
  return (int)cudaGetLastError();
}

}  // namespace gb

extern "C" {

int gb300_dgesv_adjoint_dev(int n, int nrhs, const double* dLU, int ldlu, const int* dIpiv, const double* dX, int ldx,
                            const double* dGX, int ldgx, double* dGB, int ldgb, double* dGA, int ldga, void* stream) {
  if (n < 0) return -1;
  if (nrhs < 0 || nrhs > 16) return -2;
  if (ldlu < (n > 1 ? n : 1)) return -4;
  if (ldx < (n > 1 ? n : 1)) return -7;
  if (ldgx < (n > 1 ? n : 1)) return -9;
  if (ldgb < (n > 1 ? n : 1)) return -11;
  if (dGA && ldga < (n > 1 ? n : 1)) return -13;
  cudaStream_t s = (cudaStream_t)stream;
  int rc = gb::adjoint_dev(n, nrhs, dLU, ldlu, dIpiv, dX, ldx, dGX, ldgx, dGB, ldgb, dGA, ldga, s);
  if (!rc) rc = (int)cudaStreamSynchronize(s);
  return rc;
}

// Uniform-size batch: matrices and vectors packed contiguously with strides
// (in elements) between consecutive systems.
int gb300_dgesv_adjoint_batched_dev(int batch, int n, int nrhs, const double* dLU, long long stride_lu,
                                    const int* dIpiv, long long stride_ipiv, const double* dX, long long stride_x,
                                    const double* dGX, long long stride_gx, double* dGB, long long stride_gb,
                                    double* dGA, long long stride_ga, void* stream) {
  if (batch < 0) return -1;
  if (n < 0) return -2;
  if (nrhs < 0 || nrhs > 16) return -3;
  cudaStream_t s = (cudaStream_t)stream;
  for (int b = 0; b < batch; ++b) {
    int rc = gb::adjoint_dev(n, nrhs, dLU + b * stride_lu, n, dIpiv + b * stride_ipiv, dX + b * stride_x, n,
                             dGX + b * stride_gx, n, dGB + b * stride_gb, n, dGA ? dGA + b * stride_ga : nullptr, n, s);
    if (rc) return rc;
  }
  return (int)cudaStreamSynchronize(s);
}

}  // extern "C"
