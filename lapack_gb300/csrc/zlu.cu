// Complex LU on the GPU: ZGETRF (SRC/zgetrf.f:144-225) with the recursive
// panel ZGETRF2 (SRC/zgetrf2.f:154-272), ZGETRS (SRC/zgetrs.f:157-223).
//
// The schedules (block loop, panel recursion, solve sequence) are the
// host-side templates of zlu_seq.h; here each of their steps is one kernel
// launch on the caller's stream: ZLASWP and ZTRSM with one thread per column,
// the ZGEMM update with one thread per element, the pivot step of a panel
// column on one thread.  Every thread runs the shared per-thread function
// in the reference loop order with separately rounded operations, so the
// factors, IPIV, INFO and solutions equal the reference's bit for bit (the
// CPU tests run the same schedules and functions against the oracle).  This
// is the correctness-first form of the complex path: no tiling and no
// tensor cores yet.
#include "common.cuh"
#include "driver.h"
#include "zlu_seq.h"

#include <climits>

namespace gb {

namespace {

unsigned zblocks(size_t n, int per = 128) { return (unsigned)((n + per - 1) / per); }

__global__ void __launch_bounds__(1) zcol_kernel(int m, zdc* __restrict__ a, int* __restrict__ ipiv, int gcol,
                                                 int* __restrict__ info) {
  if (zgetrf2_col(m, a, ipiv)) atomicMin(info, gcol);
}

__global__ void zlaswp_kernel(int ncols, zdc* __restrict__ A, int lda, int k1, int k2, const int* __restrict__ ipiv,
                              int incx) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j < ncols) zlaswp_col(A + (size_t)j * lda, k1, k2, ipiv, incx);
}

__global__ void ztrsm_kernel(int upper, int trans, int unit, int m, int ncols, const zdc* __restrict__ A, int lda,
                             zdc* __restrict__ B, int ldb) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j < ncols) ztrsm_left_col(upper, trans, unit, m, A, lda, B + (size_t)j * ldb);
}

__global__ void zgemm_kernel(int m, int n, int k, const zdc* __restrict__ A, int lda, const zdc* __restrict__ B,
                             int ldb, zdc* __restrict__ C, int ldc) {
  const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (size_t)m * n) return;
  const int j = (int)(e / m), i = (int)(e - (size_t)j * m);
  zgemm_nn_elem(i, j, k, A, lda, B, ldb, C, ldc);
}

__global__ void zipiv_add_kernel(int* __restrict__ ipiv, int cnt, int off) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < cnt) ipiv[i] += off;
}

// The backend of the zlu_seq.h schedules: one launch per step.  `info` is a
// device int holding INT_MAX until a zero pivot records its global column.
struct GpuZOps {
  cudaStream_t s;
  int* info;
  int col(int m, zdc* a, int* ipiv, int gcol) {
    GB_LAUNCH(zcol_kernel<<<1, 1, 0, s>>>(m, a, ipiv, gcol, info));
    return (int)cudaGetLastError();
  }
  int laswp(int ncols, zdc* A, int lda, int k1, int k2, const int* ipiv, int incx) {
    if (ncols <= 0 || k2 < k1) return 0;
    GB_LAUNCH(zlaswp_kernel<<<zblocks(ncols), 128, 0, s>>>(ncols, A, lda, k1, k2, ipiv, incx));
    return (int)cudaGetLastError();
  }
  int trsm(int upper, int trans, int unit, int m, int ncols, const zdc* A, int lda, zdc* B, int ldb) {
    if (m <= 0 || ncols <= 0) return 0;
    GB_LAUNCH(ztrsm_kernel<<<zblocks(ncols), 128, 0, s>>>(upper, trans, unit, m, ncols, A, lda, B, ldb));
    return (int)cudaGetLastError();
  }
  int gemm(int m, int n, int k, const zdc* A, int lda, const zdc* B, int ldb, zdc* C, int ldc) {
    if (m <= 0 || n <= 0 || k <= 0) return 0;   // ZGEMM's quick return (BETA = ONE)
    GB_LAUNCH(zgemm_kernel<<<zblocks((size_t)m * n, 256), 256, 0, s>>>(m, n, k, A, lda, B, ldb, C, ldc));
    return (int)cudaGetLastError();
  }
  int ipiv_add(int* ipiv, int cnt, int off) {
    if (cnt <= 0) return 0;
    GB_LAUNCH(zipiv_add_kernel<<<zblocks(cnt), 128, 0, s>>>(ipiv, cnt, off));
    return (int)cudaGetLastError();
  }
};

}  // namespace

int zgetrf_dev(int m, int n, zdc* dA, int lda, int* dIpiv, int nb, int* info, cudaStream_t s) {
  *info = 0;
  if (m <= 0 || n <= 0) return 0;
  DevScratch ib(sizeof(int), s);
  if (!ib.p) return (int)cudaErrorMemoryAllocation;
  const int none = INT_MAX;
  GB_CUDA_TRY(cudaMemcpyAsync(ib.p, &none, sizeof(int), cudaMemcpyHostToDevice, s));
  GpuZOps ops{s, ib.as<int>()};
  int rc = zgetrf_sched(ops, m, n, dA, lda, dIpiv, nb);
  if (rc) return rc;
  int h = none;
  GB_CUDA_TRY(cudaMemcpyAsync(&h, ib.p, sizeof(int), cudaMemcpyDeviceToHost, s));
  GB_CUDA_TRY(cudaStreamSynchronize(s));
  *info = (h == none) ? 0 : h;
  return 0;
}

int zgetrs_dev(int trans, int n, int nrhs, const zdc* dA, int lda, const int* dIpiv, zdc* dB, int ldb,
               cudaStream_t s) {
  GpuZOps ops{s, nullptr};
  return zgetrs_sched(ops, trans, n, nrhs, dA, lda, dIpiv, dB, ldb);
}

}  // namespace gb
