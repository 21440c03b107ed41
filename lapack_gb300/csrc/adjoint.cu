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
                       double* __restrict__ GA, int ldga, long long sgb = 0, long long sx = 0, long long sga = 0) {
  GB += blockIdx.z * sgb;     // system of a batch
  X += blockIdx.z * sx;
  GA += blockIdx.z * sga;
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

// Batched preparation of the transposed solve: each CTA replays its
// system's IPIV (staged in shared memory first) into the row permutation,
// and copies its gX into the contiguous work array.
__global__ void __launch_bounds__(1024)
adj_prep_kernel(int n, int nrhs, const int* __restrict__ ipiv, long long sip, const double* __restrict__ GX,
                long long sgx, double* __restrict__ W, int* __restrict__ perm, int* __restrict__ status) {
  extern __shared__ int adj_sh[];
  int* lab = adj_sh;           // [n]
  int* piv = adj_sh + n;       // [n]
  const int b = blockIdx.x;
  ipiv += b * sip;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    lab[i] = i;
    piv[i] = ipiv[i];
  }
  const double* gx = GX + b * sgx;
  double* w = W + (size_t)b * n * nrhs;
  for (size_t e = threadIdx.x; e < (size_t)n * nrhs; e += blockDim.x) w[e] = gx[e];
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int i = 0; i < n; ++i) {
      const int p = piv[i] - 1;
      if (p < 0 || p >= n) {
        atomicCAS(status, kStatusOk, kStatusCapacity);
        continue;
      }
      if (p != i) { const int t = lab[i]; lab[i] = lab[p]; lab[p] = t; }
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < n; i += blockDim.x) perm[(size_t)b * n + i] = lab[i];
}

// gB(perm[r], :) = W(r, :) for every system: x = P^T w.
__global__ void adj_scatter_kernel(int n, int nrhs, int batch, const double* __restrict__ W, const int* __restrict__ perm,
                                   double* __restrict__ GB, long long sgb) {
  const size_t per = (size_t)n * nrhs;
  const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= per * batch) return;
  const int b = (int)(e / per);
  const size_t k = e - (size_t)b * per;
  const int q = (int)(k / n), r = (int)(k - (size_t)q * n);
  GB[b * sgb + perm[(size_t)b * n + r] + (size_t)q * n] = W[e];
}

}  // namespace

// Uniform-size batch with every matrix and vector of leading dimension n:
// one preparation launch, two batched transposed solves (all systems'
// block chains in flight together), one scatter, one rank update.
int adjoint_batched_dev(int batch, int n, int nrhs, const double* dLU, long long slu, const int* dIpiv, long long sip,
                        const double* dX, long long sx, const double* dGX, long long sgx, double* dGB, long long sgb,
                        double* dGA, long long sga, cudaStream_t s) {
  if (batch <= 0 || n <= 0 || nrhs <= 0) return 0;
  if (nrhs > kAdjMaxRhs) return (int)cudaErrorInvalidValue;
  int dev = 0, optin = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  const size_t smem = 2 * sizeof(int) * (size_t)n;
  int* status = device_status_word();
  if (!status) return (int)cudaErrorMemoryAllocation;
  if ((long long)smem > optin) {
    // IPIV of a system too long for one CTA's shared memory: system by system
    for (int b = 0; b < batch; ++b) {
      int rc = adjoint_dev(n, nrhs, dLU + b * slu, n, dIpiv + b * sip, dX + b * sx, n, dGX + b * sgx, n, dGB + b * sgb,
                           n, dGA ? dGA + b * sga : nullptr, n, s);
      if (rc) return rc;
    }
    return 0;
  }
  static bool attr[64] = {false};
  if (!attr[dev]) {
    GB_CUDA_TRY(cudaFuncSetAttribute(adj_prep_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, optin));
    attr[dev] = true;
  }
  const size_t per = (size_t)n * nrhs;
  DevScratch ws(sizeof(double) * per * batch + sizeof(int) * (size_t)n * batch, s);
  if (!ws.p) return (int)cudaErrorMemoryAllocation;
  double* W = ws.as<double>();
  int* perm = reinterpret_cast<int*>(W + per * batch);
  prof_begin(kProfOther, s);
  GB_LAUNCH(adj_prep_kernel<<<batch, 1024, smem, s>>>(n, nrhs, dIpiv, sip, dGX, sgx, W, perm, status));
  prof_end(kProfOther, s, 0.0, (double)batch * (8.0 * 2.0 * per + 8.0 * n));
  // U^T w = gX, then L^T w = w
  int rc = trsv_batched_dev<double>(false, true, n, nrhs, dLU, n, slu, W, n, (long long)per, batch, s);
  if (!rc) rc = trsv_batched_dev<double>(true, true, n, nrhs, dLU, n, slu, W, n, (long long)per, batch, s);
  if (rc) return rc;
  const size_t tot = per * batch;
  GB_LAUNCH(adj_scatter_kernel<<<(unsigned)((tot + 255) / 256), 256, 0, s>>>(n, nrhs, batch, W, perm, dGB, sgb));
  if (dGA) {
    dim3 grid((n + kAdjRows - 1) / kAdjRows, (n + kAdjCols - 1) / kAdjCols, batch);
    prof_begin(kProfOther, s);
    if (options().exact)
      GB_LAUNCH(rank_update_neg_kernel<true><<<grid, 256, 0, s>>>(n, nrhs, dGB, n, dX, n, dGA, n, sgb, sx, sga));
    else
      GB_LAUNCH(rank_update_neg_kernel<false><<<grid, 256, 0, s>>>(n, nrhs, dGB, n, dX, n, dGA, n, sgb, sx, sga));
    prof_end(kProfOther, s, 2.0 * batch * n * (double)n * nrhs, 8.0 * batch * ((double)n * n + 2.0 * n * nrhs));
  }
  return (int)cudaGetLastError();
}

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
  int rc = gb::adjoint_batched_dev(batch, n, nrhs, dLU, stride_lu, dIpiv, stride_ipiv, dX, stride_x, dGX, stride_gx, dGB,
                                   stride_gb, dGA, stride_ga, s);
  if (rc) return rc;
  return (int)cudaStreamSynchronize(s);
}

}  // extern "C"
