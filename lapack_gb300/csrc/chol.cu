// Cholesky on the GPU: xPOTRF (SRC/dpotrf.f:131-207) with the recursive
// panel xPOTRF2 (SRC/dpotrf2.f), xPOTRS (SRC/dpotrs.f), and the DSPOSV
// mixed-precision refinement (SRC/dsposv.f:237-420).
//
// The factorization follows the reference's left-looking block order: for
// each block column, a DSYRK of the diagonal block with the columns to its
// left, DPOTRF2 of the diagonal block, then the DGEMM and DTRSM of the
// block below (lower) or to the right (upper).  Every step is one kernel
// whose threads each compute one element, one row or one column through
// the shared host/device functions of potrf_seq.h (checked against the
// oracle on the CPU); the diagonal blocks (at most NB = 64 columns) are
// factored on one thread.  The solves use the library's triangular solve
// kernels.  DSPOSV mirrors DSGESV: FP32 Cholesky and solves, FP64 residual
// with the reference's DSYMM order, the same convergence test, the FP64
// fallback.
#include "driver.h"
#include "prof.h"
#include "potrf_seq.h"
#include "solve_kernels.cuh"

#include <algorithm>

namespace gb {

namespace {

unsigned nblocks(size_t n, int per = 256) { return (unsigned)((n + per - 1) / per); }

constexpr int kCholNb = 64;   // ILAENV(1, 'xPOTRF')

// DSYRK of the jb x jb diagonal block: one thread per element of its triangle.
template <typename T>
__global__ void syrk_tri_kernel(int upper, int jb, int k, const T* __restrict__ Aop, int lda, T* __restrict__ C,
                                int ldc) {
  const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (size_t)jb * jb) return;
  const int j = (int)(e / jb), i = (int)(e - (size_t)j * jb);
  if (upper ? (i > j) : (i < j)) return;
  syrk_elem(upper, i, j, k, T(-1), Aop, lda, C, ldc);
}

template <typename T>
__global__ void __launch_bounds__(1) potrf2_kernel(int upper, int n, T* __restrict__ A, int lda, int* __restrict__ info) {
  *info = potrf2_seq(upper, n, A, lda);
}

// DPOTRF's DGEMM update of an m x ncols block: one thread per element.
template <typename T>
__global__ void gemm_chol_kernel(int upper, int m, int ncols, int k, const T* __restrict__ A, int lda,
                                 const T* __restrict__ B, int ldb, T* __restrict__ C, int ldc) {
  const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (size_t)m * ncols) return;
  const int j = (int)(e / m), i = (int)(e - (size_t)j * m);
  gemm_chol_elem(upper, i, j, k, T(-1), A, lda, B, ldb, C, ldc);
}

template <typename T>
__global__ void trsm_rltn_kernel(int rows, int n, const T* __restrict__ A, int lda, T* __restrict__ B, int ldb) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < rows) trsm_rltn_row(i, n, A, lda, B, ldb);
}

template <typename T>
__global__ void trsm_lutn_kernel(int cols, int m, const T* __restrict__ A, int lda, T* __restrict__ B, int ldb) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j < cols) trsm_lutn_col(j, m, A, lda, B, ldb);
}

// DLANSY('I') row sums (one thread per row, the reference's order).
__global__ void lansy_rows_kernel(int upper, int n, const double* __restrict__ A, int lda, double* __restrict__ rows) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) rows[i] = lansy_row_sum(upper, i, n, A, lda);
}

// DLAT2S (SRC/dlat2s.f:128-158): the first element of the triangle, in
// column order, outside [-RMAX, RMAX] (as a column-major index, atomicMin),
// then the conversion of the triangle; the caller falls back when one is
// found, so the elements after it need not stay untouched.
__global__ void lat2s_first_kernel(int upper, int n, const double* __restrict__ A, int lda,
                                   unsigned long long* __restrict__ first) {
  const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (size_t)n * n) return;
  const int j = (int)(e / n), i = (int)(e - (size_t)j * n);
  if (upper ? (i > j) : (i < j)) return;
  const double v = A[(size_t)i + (size_t)j * lda];
  const double rmax = 3.4028234663852886e38;   // SLAMCH('O')
  if (v < -rmax || v > rmax) atomicMin(first, (unsigned long long)e);
}
__global__ void lat2s_kernel(int upper, int n, const double* __restrict__ A, int lda, float* __restrict__ S, int lds) {
  const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (size_t)n * n) return;
  const int j = (int)(e / n), i = (int)(e - (size_t)j * n);
  if (upper ? (i > j) : (i < j)) return;
  S[(size_t)i + (size_t)j * lds] = (float)A[(size_t)i + (size_t)j * lda];
}

// R := R - A*X for symmetric A (DSYMM('L', uplo, alpha = -1, beta = 1)):
// one thread per element, in place (each thread reads only its own R).
__global__ void symm_residual_kernel(int upper, int n, int nrhs, const double* __restrict__ A, int lda,
                                     const double* __restrict__ X, int ldx, double* __restrict__ R, int ldr) {
  const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (size_t)n * nrhs) return;
  const int j = (int)(e / n), i = (int)(e - (size_t)j * n);
  R[(size_t)i + (size_t)j * ldr] = symm_l_elem(upper, i, j, n, -1.0, A, lda, X, ldx, R, ldr);
}

}  // namespace

template <typename T>
int potrf_dev(bool upper, int n, T* A, int lda, int nb, int* info, cudaStream_t s) {
  *info = 0;
  if (n <= 0) return 0;
  DevScratch ib(sizeof(int), s);
  if (!ib.p) return (int)cudaErrorMemoryAllocation;
  int* dinfo = ib.as<int>();
  const int up = upper ? 1 : 0;
  auto diag_factor = [&](int off, int jb) -> int {
    GB_LAUNCH(potrf2_kernel<T><<<1, 1, 0, s>>>(up, jb, A + off + (size_t)off * lda, lda, dinfo));
    int h = 0;
    GB_CUDA_TRY(cudaMemcpyAsync(&h, dinfo, sizeof(int), cudaMemcpyDeviceToHost, s));
    GB_CUDA_TRY(cudaStreamSynchronize(s));
    if (h) *info = h + off;
    return 0;
  };
  if (nb <= 1 || nb >= n) return diag_factor(0, n);
  for (int j = 0; j < n; j += nb) {
    const int jb = std::min(nb, n - j);
    T* d = A + j + (size_t)j * lda;
    if (j > 0) {
      const T* aop = upper ? A + (size_t)j * lda : A + j;
      GB_LAUNCH(syrk_tri_kernel<T><<<nblocks((size_t)jb * jb), 256, 0, s>>>(up, jb, j, aop, lda, d, lda));
    }
    int rc = diag_factor(j, jb);
    if (rc || *info) return rc;
    const int rest = n - j - jb;
    if (rest <= 0) continue;
    if (!upper) {
      T* c = A + (j + jb) + (size_t)j * lda;
      if (j > 0)
        GB_LAUNCH(gemm_chol_kernel<T><<<nblocks((size_t)rest * jb), 256, 0, s>>>(0, rest, jb, j, A + j + jb, lda,
                                                                                  A + j, lda, c, lda));
      GB_LAUNCH(trsm_rltn_kernel<T><<<nblocks(rest), 256, 0, s>>>(rest, jb, d, lda, c, lda));
    } else {
      T* c = A + j + (size_t)(j + jb) * lda;
      if (j > 0)
        GB_LAUNCH(gemm_chol_kernel<T><<<nblocks((size_t)jb * rest), 256, 0, s>>>(
            1, jb, rest, j, A + (size_t)j * lda, lda, A + (size_t)(j + jb) * lda, lda, c, lda));
      GB_LAUNCH(trsm_lutn_kernel<T><<<nblocks(rest), 256, 0, s>>>(rest, jb, d, lda, c, lda));
    }
  }
  return (int)cudaGetLastError();
}
template int potrf_dev<double>(bool, int, double*, int, int, int*, cudaStream_t);
template int potrf_dev<float>(bool, int, float*, int, int, int*, cudaStream_t);

template <typename T>
int potrs_dev(bool upper, int n, int nrhs, const T* A, int lda, T* B, int ldb, cudaStream_t s) {
  // SRC/dpotrs.f:167-181: U**T U X = B or L L**T X = B
  if (n <= 0 || nrhs <= 0) return 0;
  int rc;
  if (upper) {
    if ((rc = trsm_left_dev<T>(true, true, false, n, nrhs, A, lda, B, ldb, s))) return rc;
    return trsm_left_dev<T>(true, false, false, n, nrhs, A, lda, B, ldb, s);
  }
  if ((rc = trsm_left_dev<T>(false, false, false, n, nrhs, A, lda, B, ldb, s))) return rc;
  return trsm_left_dev<T>(false, true, false, n, nrhs, A, lda, B, ldb, s);
}
template int potrs_dev<double>(bool, int, int, const double*, int, double*, int, cudaStream_t);
template int potrs_dev<float>(bool, int, int, const float*, int, float*, int, cudaStream_t);

int dsposv_dev(bool upper, int n, int nrhs, double* dA, int lda, const double* dB, int ldb, double* dX, int ldx,
               int* iter, int* info, cudaStream_t s) {
  const int itermax = 30;
  *iter = 0;
  *info = 0;
  if (n == 0) return 0;
  const int up = upper ? 1 : 0;
  const size_t nn = (size_t)n * n, nr = (size_t)n * nrhs;
  size_t bytes = 0;
  auto carve = [&](size_t b) { size_t off = bytes; bytes += (b + 255) / 256 * 256; return off; };
  const size_t o_sa = carve(sizeof(float) * nn), o_sx = carve(sizeof(float) * nr), o_r = carve(sizeof(double) * nr),
               o_rows = carve(sizeof(double) * n), o_anrm = carve(sizeof(double)),
               o_first = carve(sizeof(unsigned long long)), o_flags = carve(sizeof(int) * 4);
  DevScratch ws(bytes, s);
  if (!ws.p) return (int)cudaErrorMemoryAllocation;
  char* base = ws.as<char>();
  float* SA = reinterpret_cast<float*>(base + o_sa);
  float* SX = reinterpret_cast<float*>(base + o_sx);
  double* R = reinterpret_cast<double*>(base + o_r);
  double* rows = reinterpret_cast<double*>(base + o_rows);
  double* anrm = reinterpret_cast<double*>(base + o_anrm);
  unsigned long long* first = reinterpret_cast<unsigned long long*>(base + o_first);
  int* flags = reinterpret_cast<int*>(base + o_flags);   // [0] overflow, [1] notconv
  int hflags[2];
  int rc, sinfo = 0;
  auto residual = [&]() -> int {
    if (nrhs == 0) { hflags[0] = hflags[1] = 0; return 0; }
    GB_CUDA_TRY(cudaMemcpy2DAsync(R, sizeof(double) * (size_t)n, dB, sizeof(double) * (size_t)ldb,
                                  sizeof(double) * (size_t)n, nrhs, cudaMemcpyDeviceToDevice, s));
    prof_begin(kProfResidual, s);
    GB_LAUNCH(symm_residual_kernel<<<nblocks(nr), 256, 0, s>>>(up, n, nrhs, dA, lda, dX, ldx, R, n));
    prof_end(kProfResidual, s, 2.0 * n * (double)n * nrhs, 8.0 * ((double)n * n / 2 + 3.0 * n * nrhs));
    GB_LAUNCH(ir_check_kernel<<<nrhs, 256, 0, s>>>(dX, ldx, R, n, n, anrm, flags + 1, nullptr));
    GB_CUDA_TRY(cudaMemcpyAsync(hflags, flags, sizeof(int) * 2, cudaMemcpyDeviceToHost, s));
    GB_CUDA_TRY(cudaStreamSynchronize(s));
    return 0;
  };

  GB_CUDA_TRY(cudaMemsetAsync(flags, 0, sizeof(int) * 4, s));
  GB_CUDA_TRY(cudaMemsetAsync(first, 0xff, sizeof(unsigned long long), s));
  // ANRM = DLANSY('I'), SX = DLAG2S(B), SA = DLAT2S(A)
  GB_LAUNCH(lansy_rows_kernel<<<nblocks(n), 256, 0, s>>>(up, n, dA, lda, rows));
  GB_LAUNCH(max_nan_kernel<double><<<1, 1024, 0, s>>>(rows, n, anrm));
  if (nr > 0) GB_LAUNCH(dlag2s_kernel<<<nblocks(nr), 256, 0, s>>>(dB, ldb, SX, n, n, nrhs, flags));
  GB_LAUNCH(lat2s_first_kernel<<<nblocks(nn), 256, 0, s>>>(up, n, dA, lda, first));
  GB_LAUNCH(lat2s_kernel<<<nblocks(nn), 256, 0, s>>>(up, n, dA, lda, SA, n));
  {
    unsigned long long hf = 0;
    GB_CUDA_TRY(cudaMemcpyAsync(hflags, flags, sizeof(int), cudaMemcpyDeviceToHost, s));
    GB_CUDA_TRY(cudaMemcpyAsync(&hf, first, sizeof(hf), cudaMemcpyDeviceToHost, s));
    GB_CUDA_TRY(cudaStreamSynchronize(s));
    if (hflags[0] || hf != ~0ull) { *iter = -2; goto fallback; }
  }
  // SPOTRF with ILAENV's block size 64 (the LU's FP32 block size is a
  // different, tuned quantity)
  if ((rc = potrf_dev<float>(upper, n, SA, n, kCholNb, &sinfo, s))) return rc;
  if (sinfo != 0) { *iter = -3; goto fallback; }
  if ((rc = potrs_dev<float>(upper, n, nrhs, SA, n, SX, n, s))) return rc;
  if (nr > 0) GB_LAUNCH(slag2d_kernel<<<nblocks(nr), 256, 0, s>>>(SX, n, dX, ldx, n, nrhs));
  if ((rc = residual())) return rc;
  if (hflags[1] == 0) { *iter = 0; return 0; }
  for (int it = 1; it <= itermax; ++it) {
    GB_CUDA_TRY(cudaMemsetAsync(flags, 0, sizeof(int) * 2, s));
    GB_LAUNCH(dlag2s_kernel<<<nblocks(nr), 256, 0, s>>>(R, n, SX, n, n, nrhs, flags));
    if ((rc = potrs_dev<float>(upper, n, nrhs, SA, n, SX, n, s))) return rc;
    GB_LAUNCH(lag2d_axpy_kernel<<<nblocks(nr), 256, 0, s>>>(SX, n, dX, ldx, n, nrhs));
    if ((rc = residual())) return rc;
    if (hflags[0]) { *iter = -2; goto fallback; }
    if (hflags[1] == 0) { *iter = it; return 0; }
  }
  *iter = -itermax - 1;
fallback:
  // FP64 DPOTRF on A in place (ILAENV's block size, as DPOTRF uses), X = B,
  // DPOTRS (SRC/dsposv.f:405-418)
  if ((rc = potrf_dev<double>(upper, n, dA, lda, kCholNb, info, s))) return rc;
  if (*info != 0) return 0;
  if (nr > 0) GB_LAUNCH(copy_cols_kernel<double><<<nblocks(nr), 256, 0, s>>>(dB, ldb, dX, ldx, n, nrhs));
  return potrs_dev<double>(upper, n, nrhs, dA, lda, dX, ldx, s);
}

}  // namespace gb
