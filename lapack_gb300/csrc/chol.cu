// Cholesky on the GPU: xPOTRF (SRC/dpotrf.f:131-207) with the recursive
// panel xPOTRF2 (SRC/dpotrf2.f), xPOTRS (SRC/dpotrs.f), and the DSPOSV
// mixed-precision refinement (SRC/dsposv.f:237-420).
//
// The factorization follows the reference's left-looking block order: for
// each block column, a DSYRK of the diagonal block with the columns to its
// left, DPOTRF2 of the diagonal block, then the DGEMM and DTRSM of the
// block below (lower) or to the right (upper).  The DGEMM -- the O(n^3)
// part -- and the DSYRK of the diagonal block run on the tiled update kernel
// in the reference's per-element orders, with separately rounded products
// in exact mode and fused multiply-adds otherwise (the DSYRK stores one
// triangle and, in the lower form, skips the terms whose A(J,L) is zero, as
// BLAS/SRC/dsyrk.f:313-320 does).  The DTRSM (one thread per row or
// column, staged in shared memory) and the diagonal blocks' DPOTRF2 (at
// most NB = 64 columns, one CTA over shared memory, each recursion step's
// rows and elements spread over its threads) compute every element through
// the operations of the shared host/device functions of potrf_seq.h
// (checked against the oracle on the CPU).  The solves use the library's
// triangular solve kernels.  DSPOSV mirrors DSGESV: FP32 Cholesky and solves, FP64 residual
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

// DPOTRF2 of a diagonal block.  On the GPU a block of up to 64 x 64 is
// staged in shared memory and factored by the whole CTA (potrf2_par: the
// rows or columns of each DTRSM and the elements of each DSYRK spread over
// the threads, the recursion's order per element unchanged), then written
// back; a larger one is factored by one thread in place.
constexpr int kPotrf2Threads = 256;
#ifdef __CUDA_ARCH__
struct CtaSync {
  __device__ void operator()() const { __syncthreads(); }
};
#endif
template <typename T>
__global__ void __launch_bounds__(kPotrf2Threads) potrf2_kernel(int upper, int n, T* __restrict__ A, int lda,
                                                                int* __restrict__ info) {
#ifdef __CUDA_ARCH__
  if (n <= 64) {
    __shared__ T D[64 * 64];
    for (int e = threadIdx.x; e < n * n; e += kPotrf2Threads) {
      const int c = e / n, r = e - c * n;
      D[r + c * n] = A[(size_t)r + (size_t)c * lda];
    }
    __syncthreads();
    const int r = potrf2_par(upper, n, D, n, (int)threadIdx.x, kPotrf2Threads, CtaSync{});
    if (threadIdx.x == 0) *info = r;
    __syncthreads();
    for (int e = threadIdx.x; e < n * n; e += kPotrf2Threads) {
      const int c = e / n, r = e - c * n;
      A[(size_t)r + (size_t)c * lda] = D[r + c * n];
    }
    return;
  }
#endif
  if (blockIdx.x == 0 && threadIdx.x == 0) *info = potrf2_seq(upper, n, A, lda);
}

// dst(c, r) = src(r, c) for an rows x cols block: the transposed operand of
// DPOTRF's DGEMM update, which the tiled update kernel reads untransposed.
template <typename T>
__global__ void transpose_kernel(int rows, int cols, const T* __restrict__ src, int lds, T* __restrict__ dst,
                                 int ldd) {
  const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (size_t)rows * cols) return;
  const int c = (int)(e / rows), r = (int)(e - (size_t)c * rows);
  dst[(size_t)c + (size_t)r * ldd] = src[(size_t)r + (size_t)c * lds];
}

// The DTRSM of the block below (lower: one thread per row of B) or to the
// right (upper: one thread per column).  On the GPU each thread's row or
// column of B (and, in FP32, the diagonal block, n <= 64) is staged in shared memory
// (stride 65: a warp's 32 rows or columns fall in different banks) and the
// solve runs over restrict-qualified copies, so the loads of a step can be
// issued ahead of its updates; the operations and their order are those of
// trsm_rltn_row / trsm_lutn_col.  64 threads per CTA.
constexpr int kCholTrsmThreads = 64;
constexpr int kCholTrsmLd = 65;
// the diagonal block is staged too in FP32 (2 x 16.6 KB); in FP64 only B
// (33 KB), the diagonal block read through the L1 cache
template <typename T>
constexpr bool kStageA = sizeof(T) == 4;
template <typename T>
__global__ void __launch_bounds__(kCholTrsmThreads) trsm_rltn_kernel(int rows, int n, const T* __restrict__ A,
                                                                     int lda, T* __restrict__ B, int ldb) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
#ifdef __CUDA_ARCH__
  if (n <= 64) {
    __shared__ T As[kStageA<T> ? kCholTrsmLd * 64 : 1];   // As[j + k * 65] = A(j, k)
    __shared__ T Bs[kCholTrsmLd * 64];                    // Bs[t + k * 65] = B(i, k)
    if constexpr (kStageA<T>) {
      for (int e = threadIdx.x; e < n * n; e += kCholTrsmThreads) {
        const int k = e / n, j = e - k * n;
        As[j + k * kCholTrsmLd] = A[(size_t)j + (size_t)k * lda];
      }
      __syncthreads();
    }
    if (i >= rows) return;
    T* __restrict__ b = Bs + threadIdx.x;
    const T* __restrict__ a = kStageA<T> ? As : A;
    const int la = kStageA<T> ? kCholTrsmLd : lda;
    for (int k = 0; k < n; ++k) b[k * kCholTrsmLd] = B[(size_t)i + (size_t)k * ldb];
    for (int k = 0; k < n; ++k) {                         // BLAS/SRC/dtrsm.f:389-403
      const T bk = rn_div(b[k * kCholTrsmLd], a[k + (size_t)k * la]);
      b[k * kCholTrsmLd] = bk;
#pragma unroll 4
      for (int j = k + 1; j < n; ++j)
        b[j * kCholTrsmLd] = rn_sub(b[j * kCholTrsmLd], rn_mul(a[j + (size_t)k * la], bk));
    }
    for (int k = 0; k < n; ++k) B[(size_t)i + (size_t)k * ldb] = b[k * kCholTrsmLd];
    return;
  }
#endif
  if (i < rows) trsm_rltn_row(i, n, A, lda, B, ldb);
}

template <typename T>
__global__ void __launch_bounds__(kCholTrsmThreads) trsm_lutn_kernel(int cols, int m, const T* __restrict__ A,
                                                                     int lda, T* __restrict__ B, int ldb) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
#ifdef __CUDA_ARCH__
  if (m <= 64) {
    __shared__ T As[kStageA<T> ? kCholTrsmLd * 64 : 1];   // As[k + i * 65] = A(k, i)
    __shared__ T Bs[kCholTrsmLd * 64];                    // Bs[t * 65 + k] = B(k, j)
    if constexpr (kStageA<T>) {
      for (int e = threadIdx.x; e < m * m; e += kCholTrsmThreads) {
        const int c = e / m, r = e - c * m;
        As[r + c * kCholTrsmLd] = A[(size_t)r + (size_t)c * lda];
      }
      __syncthreads();
    }
    if (j >= cols) return;
    T* __restrict__ b = Bs + threadIdx.x * kCholTrsmLd;
    const T* __restrict__ a = kStageA<T> ? As : A;
    const int la = kStageA<T> ? kCholTrsmLd : lda;
    for (int k = 0; k < m; ++k) b[k] = B[(size_t)k + (size_t)j * ldb];
    for (int i = 0; i < m; ++i) {                         // BLAS/SRC/dtrsm.f:306-316
      T temp = b[i];
      for (int k = 0; k < i; ++k) temp = rn_sub(temp, rn_mul(a[k + (size_t)i * la], b[k]));
      b[i] = rn_div(temp, a[i + (size_t)i * la]);
    }
    for (int k = 0; k < m; ++k) B[(size_t)k + (size_t)j * ldb] = b[k];
    return;
  }
#endif
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
    GB_LAUNCH(potrf2_kernel<T><<<1, kPotrf2Threads, 0, s>>>(up, jb, A + off + (size_t)off * lda, lda, dinfo));
    int h = 0;
    GB_CUDA_TRY(cudaMemcpyAsync(&h, dinfo, sizeof(int), cudaMemcpyDeviceToHost, s));
    GB_CUDA_TRY(cudaStreamSynchronize(s));
    if (h) *info = h + off;
    return 0;
  };
  if (nb <= 1 || nb >= n) return diag_factor(0, n);
  // the transposed jb x j operand of the DGEMM update (at most nb x n)
  DevScratch tb(sizeof(T) * (size_t)nb * n, s);
  if (!tb.p) return (int)cudaErrorMemoryAllocation;
  T* Tt = tb.as<T>();
  for (int j = 0; j < n; j += nb) {
    const int jb = std::min(nb, n - j);
    T* d = A + j + (size_t)j * lda;
    int rc = 0;
    if (j > 0) {
      // the block's left (L) or upper (U) neighbour transposed, for the DSYRK
      // and the DGEMM: L: A(j:j+jb, 0:j)^T (j x jb); U: A(0:j, j:j+jb)^T (jb x j)
      if (!upper) {
        GB_LAUNCH(transpose_kernel<T><<<nblocks((size_t)jb * j), 256, 0, s>>>(jb, j, A + j, lda, Tt, j));
        rc = syrk_ordered_dev<T>(false, jb, j, A + j, lda, Tt, j, d, lda, s);
      } else {
        GB_LAUNCH(transpose_kernel<T><<<nblocks((size_t)j * jb), 256, 0, s>>>(j, jb, A + (size_t)j * lda, lda, Tt,
                                                                                 jb));
        rc = syrk_ordered_dev<T>(true, jb, j, Tt, jb, A + (size_t)j * lda, lda, d, lda, s);
      }
      if (rc) return rc;
    }
    rc = diag_factor(j, jb);
    if (rc || *info) return rc;
    const int rest = n - j - jb;
    if (rest <= 0) continue;
    const unsigned tg = nblocks(rest, kCholTrsmThreads);
    // the DGEMM update on the tiled update kernel, in the reference's
    // per-element order (dgemm.f: 'N','T' products subtracted in turn for L,
    // 'T','N' products summed then subtracted for U), then the DTRSM
    if (!upper) {
      T* c = A + (j + jb) + (size_t)j * lda;
      if (j > 0) {
        // C(rest x jb) -= A(j+jb:n, 0:j) * A(j:j+jb, 0:j)^T
        rc = gemm_ordered_dev<T>(false, rest, jb, j, A + j + jb, lda, Tt, j, c, lda, s);
        if (rc) return rc;
      }
      GB_LAUNCH(trsm_rltn_kernel<T><<<tg, kCholTrsmThreads, 0, s>>>(rest, jb, d, lda, c, lda));
    } else {
      T* c = A + j + (size_t)(j + jb) * lda;
      if (j > 0) {
        // C(jb x rest) -= A(0:j, j:j+jb)^T * A(0:j, j+jb:n)
        rc = gemm_ordered_dev<T>(true, jb, rest, j, Tt, jb, A + (size_t)(j + jb) * lda, lda, c, lda, s);
        if (rc) return rc;
      }
      GB_LAUNCH(trsm_lutn_kernel<T><<<tg, kCholTrsmThreads, 0, s>>>(rest, jb, d, lda, c, lda));
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
