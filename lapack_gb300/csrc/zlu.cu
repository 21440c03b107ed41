// Complex LU on the GPU: ZGETRF / CGETRF (SRC/zgetrf.f:144-225) with the
// recursive panel xGETRF2 (SRC/zgetrf2.f:154-272), ZGETRS / CGETRS
// (SRC/zgetrs.f:157-223), and the mixed-precision ZCGESV
// (SRC/zcgesv.f:259-448).
//
// The schedules (block loop, panel recursion, solve sequence, refinement
// loop) are the host-side templates of zlu_seq.h; here each of their steps
// is one kernel launch on the caller's stream: the ZGEMM update on shared-
// memory tiles and the pivot step of a panel column on one CTA (both in
// zlu_tiles.cu), ZLASWP and ZTRSM with one thread per column, the
// conversions with one thread per element, ZLANGE with one thread per row
// and its maximum on one thread, the convergence test with one thread per
// right-hand side.  Every element is computed in the reference loop order
// with separately rounded operations, so the results equal the reference's
// bit for bit (the CPU tests run the same schedules and functions against
// the oracle).  No tensor cores: the complex FMA units carry the update.
#include "common.cuh"
#include "driver.h"
#include "zlu_seq.h"

#include <climits>

namespace gb {

// zlu_tiles.cu: the tiled ZGEMM update (C -= A*B) and the pivot step of one
// panel column (a zero pivot records INFO = gcol by atomicMin).
template <typename R>
int zgemm_tile_dev(int m, int n, int k, const cpx<R>* A, int lda, const cpx<R>* B, int ldb, cpx<R>* C, int ldc,
                   cudaStream_t s);
template <typename R>
int zcol_cta_dev(int m, cpx<R>* a, int* ipiv, int gcol, int* info, cudaStream_t s);
// One CTA per column of a ZTRSM; false (nothing launched) for 'T'/'C' lower.
template <typename R>
bool ztrsm_cta_dev(int upper, int trans, int unit, int m, int ncols, const cpx<R>* A, int lda, cpx<R>* B, int ldb,
                   cudaStream_t s, int* rc);

namespace {

unsigned zblocks(size_t n, int per = 128) { return (unsigned)((n + per - 1) / per); }

template <typename R>
__global__ void zlaswp_kernel(int ncols, cpx<R>* __restrict__ A, int lda, int k1, int k2, const int* __restrict__ ipiv,
                              int incx) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j < ncols) zlaswp_col(A + (size_t)j * lda, k1, k2, ipiv, incx);
}

template <typename R>
__global__ void ztrsm_kernel(int upper, int trans, int unit, int m, int ncols, const cpx<R>* __restrict__ A, int lda,
                             cpx<R>* __restrict__ B, int ldb) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j < ncols) ztrsm_left_col(upper, trans, unit, m, A, lda, B + (size_t)j * ldb);
}

// The same for a triangle of order m <= 32 (the panel recursion's ZTRSM):
// on the GPU the triangle and each thread's column are staged in shared
// memory first (one round of global loads), so the solve's steps wait on
// shared memory, not on reloads of the column it has just stored.  32
// threads per CTA; the operations are those of ztrsm_left_col.
constexpr int kZtrsmSmall = 32;
template <typename R>
__global__ void __launch_bounds__(kZtrsmSmall) ztrsm_small_kernel(int upper, int trans, int unit, int m, int ncols,
                                                                  const cpx<R>* __restrict__ A, int lda,
                                                                  cpx<R>* __restrict__ B, int ldb) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
#ifdef __CUDA_ARCH__
  __shared__ cpx<R> As[kZtrsmSmall * kZtrsmSmall];
  __shared__ cpx<R> Bs[kZtrsmSmall * (kZtrsmSmall + 1)];
  for (int e = threadIdx.x; e < m * m; e += kZtrsmSmall) {
    const int c = e / m, r = e - c * m;
    As[r + c * kZtrsmSmall] = A[(size_t)r + (size_t)c * lda];
  }
  cpx<R>* b = Bs + threadIdx.x * (kZtrsmSmall + 1);
  if (j < ncols)
    for (int i = 0; i < m; ++i) b[i] = B[(size_t)i + (size_t)j * ldb];
  __syncthreads();
  if (j < ncols) {
    ztrsm_left_col(upper, trans, unit, m, As, kZtrsmSmall, b);
    for (int i = 0; i < m; ++i) B[(size_t)i + (size_t)j * ldb] = b[i];
  }
#else
  if (j < ncols) ztrsm_left_col(upper, trans, unit, m, A, lda, B + (size_t)j * ldb);
#endif
}

__global__ void zipiv_add_kernel(int* __restrict__ ipiv, int cnt, int off) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < cnt) ipiv[i] += off;
}

__global__ void zlange_rows_kernel(int n, const zdc* __restrict__ A, int lda, double* __restrict__ rows) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) rows[i] = zlange_row(i, n, A, lda);
}

__global__ void __launch_bounds__(1) zlange_max_kernel(int n, const double* __restrict__ rows,
                                                       double* __restrict__ out) {
  *out = zlange_max(n, rows);
}

__global__ void zlag2c_kernel(int m, int ncols, const zdc* __restrict__ A, int lda, cfc* __restrict__ S, int lds,
                              int* __restrict__ overflow) {
  const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (size_t)m * ncols) return;
  const int j = (int)(e / m), i = (int)(e - (size_t)j * m);
  if (!zlag2c_elem(A[(size_t)i + (size_t)j * lda], S + (size_t)i + (size_t)j * lds)) *overflow = 1;
}

__global__ void zlag2z_kernel(int m, int ncols, const cfc* __restrict__ S, int lds, zdc* __restrict__ X, int ldx,
                              int add) {
  const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (size_t)m * ncols) return;
  const int j = (int)(e / m), i = (int)(e - (size_t)j * m);
  zlag2z_elem(S[(size_t)i + (size_t)j * lds], X + (size_t)i + (size_t)j * ldx, add != 0);
}

__global__ void zcheck_kernel(int n, int nrhs, const zdc* __restrict__ X, int ldx, const zdc* __restrict__ R, int ldr,
                              double cte, int* __restrict__ notconv) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j < nrhs && zcgesv_col_notconv(n, X + (size_t)j * ldx, R + (size_t)j * ldr, cte)) *notconv = 1;
}

// Device words the backend keeps: [0] INFO (INT_MAX until a zero pivot),
// [1] conversion overflow, [2] not converged; then ANRM and the row sums.
struct ZWords {
  int* info;
  int* flags;       // flags[0] overflow, flags[1] notconv
  double* anrm;
  double* rows;     // n row sums (ZCGESV only)
};

// The backend of the zlu_seq.h schedules: one launch per step.
struct GpuZOps {
  cudaStream_t s;
  ZWords w;
  int info_reset() {
    const int none = INT_MAX;
    return (int)cudaMemcpyAsync(w.info, &none, sizeof(int), cudaMemcpyHostToDevice, s);
  }
  int info_read(int* out) {
    int h = INT_MAX;
    GB_CUDA_TRY(cudaMemcpyAsync(&h, w.info, sizeof(int), cudaMemcpyDeviceToHost, s));
    GB_CUDA_TRY(cudaStreamSynchronize(s));
    *out = (h == INT_MAX) ? 0 : h;
    return 0;
  }
  template <typename R>
  int col(int m, cpx<R>* a, int* ipiv, int gcol) {
    return zcol_cta_dev<R>(m, a, ipiv, gcol, w.info, s);
  }
  template <typename R>
  int laswp(int ncols, cpx<R>* A, int lda, int k1, int k2, const int* ipiv, int incx) {
    if (ncols <= 0 || k2 < k1) return 0;
    GB_LAUNCH(zlaswp_kernel<R><<<zblocks(ncols, 64), 64, 0, s>>>(ncols, A, lda, k1, k2, ipiv, incx));
    return (int)cudaGetLastError();
  }
  template <typename R>
  int trsm(int upper, int trans, int unit, int m, int ncols, const cpx<R>* A, int lda, cpx<R>* B, int ldb) {
    if (m <= 0 || ncols <= 0) return 0;
    // long columns (ZGETRS): a CTA per column; the panel's and the block
    // row's short ones (m <= NB): a thread per column
    int rc = 0;
    if (m > 128 && ztrsm_cta_dev<R>(upper, trans, unit, m, ncols, A, lda, B, ldb, s, &rc)) return rc;
    if (m <= kZtrsmSmall) {
      const unsigned g = zblocks(ncols, kZtrsmSmall);
      GB_LAUNCH(ztrsm_small_kernel<R><<<g, kZtrsmSmall, 0, s>>>(upper, trans, unit, m, ncols, A, lda, B, ldb));
      return (int)cudaGetLastError();
    }
    GB_LAUNCH(ztrsm_kernel<R><<<zblocks(ncols, 64), 64, 0, s>>>(upper, trans, unit, m, ncols, A, lda, B, ldb));
    return (int)cudaGetLastError();
  }
  template <typename R>
  int gemm(int m, int n, int k, const cpx<R>* A, int lda, const cpx<R>* B, int ldb, cpx<R>* C, int ldc) {
    if (m <= 0 || n <= 0 || k <= 0) return 0;   // ZGEMM's quick return (BETA = ONE)
    return zgemm_tile_dev<R>(m, n, k, A, lda, B, ldb, C, ldc, s);
  }
  int ipiv_add(int* ipiv, int cnt, int off) {
    if (cnt <= 0) return 0;
    GB_LAUNCH(zipiv_add_kernel<<<zblocks(cnt), 128, 0, s>>>(ipiv, cnt, off));
    return (int)cudaGetLastError();
  }
  int lange_inf(int n, const zdc* A, int lda, double* anrm) {
    GB_LAUNCH(zlange_rows_kernel<<<zblocks(n), 128, 0, s>>>(n, A, lda, w.rows));
    GB_LAUNCH(zlange_max_kernel<<<1, 1, 0, s>>>(n, w.rows, w.anrm));
    GB_CUDA_TRY(cudaMemcpyAsync(anrm, w.anrm, sizeof(double), cudaMemcpyDeviceToHost, s));
    GB_CUDA_TRY(cudaStreamSynchronize(s));
    return 0;
  }
  int flags_reset() { return (int)cudaMemsetAsync(w.flags, 0, 2 * sizeof(int), s); }
  int flags_read(int* ovf, int* nc) {
    int h[2] = {0, 0};
    GB_CUDA_TRY(cudaMemcpyAsync(h, w.flags, sizeof(h), cudaMemcpyDeviceToHost, s));
    GB_CUDA_TRY(cudaStreamSynchronize(s));
    *ovf = h[0];
    *nc = h[1];
    return 0;
  }
  int lag2c(int m, int ncols, const zdc* A, int lda, cfc* S, int lds) {
    if (m <= 0 || ncols <= 0) return 0;
    GB_LAUNCH(zlag2c_kernel<<<zblocks((size_t)m * ncols, 256), 256, 0, s>>>(m, ncols, A, lda, S, lds, w.flags));
    return (int)cudaGetLastError();
  }
  int lag2z(int m, int ncols, const cfc* S, int lds, zdc* X, int ldx, bool add) {
    if (m <= 0 || ncols <= 0) return 0;
    GB_LAUNCH(zlag2z_kernel<<<zblocks((size_t)m * ncols, 256), 256, 0, s>>>(m, ncols, S, lds, X, ldx, add ? 1 : 0));
    return (int)cudaGetLastError();
  }
  int copy(int m, int ncols, const zdc* B, int ldb, zdc* R, int ldr) {
    if (m <= 0 || ncols <= 0) return 0;
    return (int)cudaMemcpy2DAsync(R, sizeof(zdc) * (size_t)ldr, B, sizeof(zdc) * (size_t)ldb, sizeof(zdc) * (size_t)m,
                                  ncols, cudaMemcpyDeviceToDevice, s);
  }
  int check(int n, int nrhs, const zdc* X, int ldx, const zdc* R, int ldr, double cte) {
    if (nrhs <= 0) return 0;
    GB_LAUNCH(zcheck_kernel<<<zblocks(nrhs), 128, 0, s>>>(n, nrhs, X, ldx, R, ldr, cte, w.flags + 1));
    return (int)cudaGetLastError();
  }
};

}  // namespace

template <typename R>
int zgetrf_dev(int m, int n, cpx<R>* dA, int lda, int* dIpiv, int nb, int* info, cudaStream_t s) {
  *info = 0;
  if (m <= 0 || n <= 0) return 0;
  DevScratch ib(sizeof(int), s);
  if (!ib.p) return (int)cudaErrorMemoryAllocation;
  GpuZOps ops{s, ZWords{ib.as<int>(), nullptr, nullptr, nullptr}};
  return zgetrf_full(ops, m, n, dA, lda, dIpiv, nb, info);
}
template int zgetrf_dev<double>(int, int, zdc*, int, int*, int, int*, cudaStream_t);
template int zgetrf_dev<float>(int, int, cfc*, int, int*, int, int*, cudaStream_t);

template <typename R>
int zgetrs_dev(int trans, int n, int nrhs, const cpx<R>* dA, int lda, const int* dIpiv, cpx<R>* dB, int ldb,
               cudaStream_t s) {
  GpuZOps ops{s, ZWords{nullptr, nullptr, nullptr, nullptr}};
  return zgetrs_sched(ops, trans, n, nrhs, dA, lda, dIpiv, dB, ldb);
}
template int zgetrs_dev<double>(int, int, int, const zdc*, int, const int*, zdc*, int, cudaStream_t);
template int zgetrs_dev<float>(int, int, int, const cfc*, int, const int*, cfc*, int, cudaStream_t);

int zcgesv_dev(int n, int nrhs, zdc* dA, int lda, int* dIpiv, const zdc* dB, int ldb, zdc* dX, int ldx, int* iter,
               int* info, cudaStream_t s) {
  *iter = 0;
  *info = 0;
  if (n <= 0) return 0;
  size_t bytes = 0;
  auto carve = [&](size_t b) { size_t off = bytes; bytes += (b + 255) / 256 * 256; return off; };
  const size_t nn = (size_t)n * n, nr = (size_t)n * (size_t)(nrhs > 0 ? nrhs : 1);
  const size_t o_sa = carve(sizeof(cfc) * nn), o_sx = carve(sizeof(cfc) * nr), o_r = carve(sizeof(zdc) * nr),
               o_rows = carve(sizeof(double) * (size_t)n), o_anrm = carve(sizeof(double)),
               o_words = carve(sizeof(int) * 4);
  DevScratch ws(bytes, s);
  if (!ws.p) return (int)cudaErrorMemoryAllocation;
  char* base = ws.as<char>();
  int* words = reinterpret_cast<int*>(base + o_words);
  GpuZOps ops{s, ZWords{words, words + 1, reinterpret_cast<double*>(base + o_anrm),
                        reinterpret_cast<double*>(base + o_rows)}};
  return zcgesv_sched(ops, n, nrhs, dA, lda, dIpiv, dB, ldb, dX, ldx, reinterpret_cast<cfc*>(base + o_sa),
                      reinterpret_cast<cfc*>(base + o_sx), reinterpret_cast<zdc*>(base + o_r), iter, info);
}

}  // namespace gb
