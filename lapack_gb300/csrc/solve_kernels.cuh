// Kernels of the solve phase (DGETRS) and of the mixed-precision refinement
// driver (DSGESV): row permutations, blocked triangular solves, norms,
// precision conversions and the FP64 residual.
#pragma once
#include "common.cuh"

namespace gb {

// ---------------------------------------------------------------------------
// IPIV -> permutation.  DLASWP (SRC/dlaswp.f:138-183) applies the
// interchanges one after another; the net effect on rows lo..lo+span-1 is a
// permutation, computed here by replaying the swaps on row labels.  After
// the replay, position r holds original row perm[r] (a gather index).  One
// CTA; `lab` is shared memory when the window fits, global scratch
// otherwise.  An IPIV entry outside the window is reported through `status`
// and skipped (the reference would index out of bounds).
template <bool SHARED>
__global__ void __launch_bounds__(1024)
ipiv_to_perm_kernel(const int* __restrict__ ipiv, int k1, int k2, int incx, int lo, int span,
                    int* __restrict__ perm_out, int* __restrict__ lab_global, int* __restrict__ status) {
  extern __shared__ int lab_sh[];
  int* lab = SHARED ? lab_sh : lab_global;
  for (int i = threadIdx.x; i < span; i += blockDim.x) lab[i] = lo + i;
  __syncthreads();
  if (threadIdx.x == 0) {
    int i1, i2, inc, ix;
    if (incx > 0) { i1 = k1; i2 = k2; inc = 1; ix = k1; }
    else { i1 = k2; i2 = k1; inc = -1; ix = k1 + (k1 - k2) * incx; }
    for (int i = i1;; i += inc) {
      int p = ipiv[ix - 1];
      int a = i - 1 - lo, b = p - 1 - lo;
      if (a >= 0 && a < span && b >= 0 && b < span) {
        if (a != b) { int t = lab[a]; lab[a] = lab[b]; lab[b] = t; }
      } else {
        atomicCAS(status, kStatusOk, kStatusCapacity);
      }
      ix += incx;
      if (i == i2) break;
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < span; i += blockDim.x) perm_out[i] = lab[i];
}

// W(r, s) = B(perm[r], s)  (gather), or W(perm[r], s) = B(r, s)  (scatter).
template <typename T, bool SCATTER>
__global__ void perm_rows_kernel(const T* __restrict__ B, int ldb, T* __restrict__ W, int ldw,
                                 const int* __restrict__ perm, int perm_base, int n, int ncols) {
  size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  size_t total = (size_t)n * ncols;
  if (e >= total) return;
  int c = (int)(e / n), r = (int)(e - (size_t)c * n);
  int p = perm[r] - perm_base;
  if (SCATTER) W[(size_t)p + (size_t)c * ldw] = B[(size_t)r + (size_t)c * ldb];
  else W[(size_t)r + (size_t)c * ldw] = B[(size_t)p + (size_t)c * ldb];
}

template <typename T>
__global__ void copy_cols_kernel(const T* __restrict__ S, int lds, T* __restrict__ D, int ldd, int m, int ncols) {
  size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (size_t)m * ncols) return;
  int c = (int)(e / m), r = (int)(e - (size_t)c * m);
  D[(size_t)r + (size_t)c * ldd] = S[(size_t)r + (size_t)c * lds];
}

// ---------------------------------------------------------------------------
// Blocked triangular solve with several right-hand sides, X := op(T)^{-1} X,
// for the four DGETRS cases (SRC/dgetrs.f:187-217 calling
// BLAS/SRC/dtrsm.f:272-329).  The matrix is cut into 64-row blocks; CTAs
// take blocks in solve order from a ticket counter.  A CTA streams the
// 64 x 64 tiles of its block row (prefetched with cp.async, double
// buffered, independent of any dependency), folds in each source block's
// solution as soon as that block's flag is released, then solves its
// diagonal block with one warp per right-hand side (two rows per lane,
// shuffle broadcast, no block barriers), writes its solution and releases
// its own flag.  Every wait is bounded.  FORWARD: blocks in increasing order
// (L, or U^T); otherwise decreasing (U, or L^T).  TRANS reads T(k, r) for
// element (r, k).  In increasing / decreasing order of k each element
// receives its updates in the reference loop order (N cases and U^T); the
// L^T case would fold k in decreasing order where the reference folds in
// increasing order, so exact mode solves L^T with trsv_lt_exact_kernel.
constexpr int kSolveBS = 64;
constexpr int kSolveRQ = 4;   // right-hand sides per pass (256 threads = 64 rows x 4)
constexpr int kSolveLd = kSolveBS + 1;
template <typename T>
constexpr int kTrsvSmem = 2 * kSolveBS * kSolveLd * (int)sizeof(T);   // 33 KB (float) / 66.6 KB (double)



template <typename T, bool EXACT, bool FORWARD, bool UNIT, bool TRANS>
__global__ void __launch_bounds__(256)
trsv_blocked_kernel(const T* __restrict__ A, int lda, int n, T* __restrict__ X, int ldx, int nrhs,
                    int* __restrict__ flags, unsigned* __restrict__ ticket, int* __restrict__ status) {
  extern __shared__ __align__(16) unsigned char trsv_smem[];
  T* tiles = reinterpret_cast<T*>(trsv_smem);     // [2][64][65]: raw column-major copies
  __shared__ T xsrc[2][kSolveBS][kSolveRQ];
  __shared__ T xs[kSolveBS][kSolveRQ];
  __shared__ unsigned t_s;
  __shared__ int ok_s;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int r = tid & 63, q = tid >> 6;
  const int nblk = (n + kSolveBS - 1) / kSolveBS;
  if (tid == 0) { t_s = atomicAdd(ticket, 1u); ok_s = 1; }
  __syncthreads();
  const int t = (int)t_s;
  const int bi = FORWARD ? t : nblk - 1 - t;
  const int r0 = bi * kSolveBS;
  const int nr = min(kSolveBS, n - r0);
  const int nsrc = FORWARD ? bi : nblk - 1 - bi;

  // raw copy of the stored block behind op(T)(r0.., c0..): rows r0.., cols c0..
  // (non-transposed) or rows c0.., cols r0.. (transposed); element (rr, cc)
  // of the stored block lands at tile[cc * 65 + rr]
  auto issue_tile = [&](int bj, T* dst) {
    const int c0 = bj * kSolveBS;
    const int nc = min(kSolveBS, n - c0);
    const int srow = TRANS ? c0 : r0, scol = TRANS ? r0 : c0;
    const int nsr = TRANS ? nc : nr, nsc = TRANS ? nr : nc;
    for (int e = tid; e < kSolveBS * kSolveBS; e += 256) {
      const int cc = e >> 6, rr = e & 63;
      if (rr < nsr && cc < nsc) cp_async_elem(dst + cc * kSolveLd + rr, A + (size_t)(srow + rr) + (size_t)(scol + cc) * lda);
    }
  };
  // op(T)(row rr of this block, column kk of the source block)
  auto op_elem = [&](const T* tl, int rr, int kk) -> T { return TRANS ? tl[rr * kSolveLd + kk] : tl[kk * kSolveLd + rr]; };

  for (int q0 = 0; q0 < nrhs && ok_s; q0 += kSolveRQ) {
    const int nq = min(kSolveRQ, nrhs - q0);
    const bool active = (r < nr) && (q < nq);
    T acc = active ? X[(size_t)(r0 + r) + (size_t)(q0 + q) * ldx] : T(0);
    if (nsrc > 0) issue_tile(FORWARD ? 0 : nblk - 1, tiles);
    cp_async_commit();
    for (int step = 0; step < nsrc; ++step) {
      const int bj = FORWARD ? step : nblk - 1 - step;
      const int c0 = bj * kSolveBS;
      const int nc = min(kSolveBS, n - c0);
      const int buf = step & 1;
      // warp 0: wait for block bj's solution (every lane acquires), read it
      if (warp == 0) {
        int okw = 1;
        if (q0 == 0) {
          unsigned spins = 0;
          while (ld_acquire_s32(flags + bj) == 0) {
            if (++spins > kSpinLimit || *(volatile int*)status != kStatusOk) {
              atomicCAS(status, kStatusOk, kStatusFlagTimeout);
              okw = 0;
              break;
            }
          }
        }
        okw = __all_sync(0xffffffffu, okw);
        if (!okw) {
          if (lane == 0) ok_s = 0;
        } else {
          for (int e = lane; e < kSolveBS * kSolveRQ; e += 32) {
            const int cc = e % kSolveBS, qq = e / kSolveBS;
            xsrc[buf][cc][qq] = (cc < nc && qq < nq) ? ldcg(X + (size_t)(c0 + cc) + (size_t)(q0 + qq) * ldx) : T(0);
          }
        }
      }
      cp_async_wait<0>();
      __syncthreads();
      if (!ok_s) break;
      // prefetch the next tile into the other buffer while this one is used
      if (step + 1 < nsrc) issue_tile(FORWARD ? step + 1 : nblk - 2 - step, tiles + (buf ^ 1) * kSolveBS * kSolveLd);
      cp_async_commit();
      const T* tl = tiles + buf * kSolveBS * kSolveLd;
      if (active) {
        if (FORWARD) {
          for (int kk = 0; kk < nc; ++kk) acc = fnmadd<EXACT>(op_elem(tl, r, kk), xsrc[buf][kk][q], acc);
        } else {
          for (int kk = nc - 1; kk >= 0; --kk) acc = fnmadd<EXACT>(op_elem(tl, r, kk), xsrc[buf][kk][q], acc);
        }
      }
    }
    cp_async_wait<0>();
    __syncthreads();
    if (!ok_s) break;
    // diagonal block: stage it in buffer 0, one warp per right-hand side
    issue_tile(bi, tiles);
    cp_async_commit();
    xs[r][q] = acc;
    cp_async_wait<0>();
    __syncthreads();
    if (warp < nq) {
      const T* D = tiles;
      const int qq = warp;
      T x0 = lane < nr ? xs[lane][qq] : T(0);
      T x1 = lane + 32 < nr ? xs[lane + 32][qq] : T(0);
      if (FORWARD) {
        for (int k = 0; k < nr; ++k) {
          const bool hi = k >= 32;
          T xk = hi ? x1 : x0;
          if (!UNIT) {
            if ((k & 31) == lane) {
              xk = xk / op_elem(D, k, k);
              if (hi) x1 = xk; else x0 = xk;
            }
          }
          xk = __shfl_sync(0xffffffffu, xk, k & 31);
          if (lane > k && lane < nr) x0 = fnmadd<EXACT>(op_elem(D, lane, k), xk, x0);
          if (lane + 32 > k && lane + 32 < nr) x1 = fnmadd<EXACT>(op_elem(D, lane + 32, k), xk, x1);
        }
      } else {
        for (int k = nr - 1; k >= 0; --k) {
          const bool hi = k >= 32;
          T xk = hi ? x1 : x0;
          if (!UNIT) {
            if ((k & 31) == lane) {
              xk = xk / op_elem(D, k, k);
              if (hi) x1 = xk; else x0 = xk;
            }
          }
          xk = __shfl_sync(0xffffffffu, xk, k & 31);
          if (lane < k) x0 = fnmadd<EXACT>(op_elem(D, lane, k), xk, x0);
          if (lane + 32 < k) x1 = fnmadd<EXACT>(op_elem(D, lane + 32, k), xk, x1);
        }
      }
      if (lane < nr) X[(size_t)(r0 + lane) + (size_t)(q0 + qq) * ldx] = x0;
      if (lane + 32 < nr) X[(size_t)(r0 + lane + 32) + (size_t)(q0 + qq) * ldx] = x1;
    }
    __syncthreads();
  }
  __threadfence();
  __syncthreads();
  if (tid == 0) st_release_s32(flags + bi, ok_s ? 1 : -1);
}

// X := L^{-T} X in the reference order, for exact mode: DTRSM('L','L','T',
// diag) (BLAS/SRC/dtrsm.f:317-328) forms each X(i) as one dot product,
// TEMP = X(i) - sum_{k=i+1..n} L(k,i) X(k) folded in increasing k, after every
// X(k), k > i, is final.  That order is one dependent chain per right-hand
// side, so one thread solves one right-hand side.
template <typename T, bool UNIT>
__global__ void __launch_bounds__(64)
trsv_lt_exact_kernel(const T* __restrict__ A, int lda, int n, T* __restrict__ X, int ldx, int nrhs) {
  const int j = blockIdx.x * 64 + threadIdx.x;
  if (j >= nrhs) return;
  T* x = X + (size_t)j * ldx;
  for (int i = n - 1; i >= 0; --i) {
    const T* col = A + (size_t)i * lda;
    T temp = x[i];
    for (int k = i + 1; k < n; ++k) temp = fnmadd<true>(col[k], x[k], temp);
    if (!UNIT) temp = temp / col[i];
    x[i] = temp;
  }
}

// Raises the dynamic shared-memory limit of one instantiation (needed for
// the 66.6 KB double tiles); returns the CUDA status of the attribute call.
template <typename T, bool EXACT, bool FORWARD, bool UNIT, bool TRANS>
cudaError_t trsv_set_smem() {
  return cudaFuncSetAttribute(trsv_blocked_kernel<T, EXACT, FORWARD, UNIT, TRANS>,
                              cudaFuncAttributeMaxDynamicSharedMemorySize, kTrsvSmem<T>);
}

// ---------------------------------------------------------------------------
// DLANGE('I') (SRC/dlange.f:173-189): row absolute sums in column order,
// then the maximum with NaN propagation.  One thread per row keeps the
// reference summation order; 32 independent loads are kept in flight.
template <typename T>
__global__ void __launch_bounds__(64)
row_abs_sum_kernel(const T* __restrict__ A, int lda, int m, int n, T* __restrict__ rowsum) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= m) return;
  const T* p = A + i;
  T s = 0;
  int j = 0;
  for (; j + 32 <= n; j += 32) {
    T v[32];
#pragma unroll
    for (int u = 0; u < 32; ++u) v[u] = p[(size_t)(j + u) * lda];
#pragma unroll
    for (int u = 0; u < 32; ++u) s = s + (v[u] < 0 ? -v[u] : v[u]);
  }
  for (; j < n; ++j) {
    T v = p[(size_t)j * lda];
    s = s + (v < 0 ? -v : v);
  }
  rowsum[i] = s;
}

// Chunked row sums: part[s][i] = sum of |A(i, l)| over chunk s of the columns.
static __global__ void __launch_bounds__(64)
row_abs_sum_split_kernel(const double* __restrict__ A, int lda, int m, int n, int chunk, double* __restrict__ part) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= m) return;
  const int l0 = blockIdx.y * chunk, l1 = min(n, l0 + chunk);
  const double* p = A + i;
  double s = 0;
  int j = l0;
  for (; j + 16 <= l1; j += 16) {
    double v[16];
#pragma unroll
    for (int u = 0; u < 16; ++u) v[u] = p[(size_t)(j + u) * lda];
#pragma unroll
    for (int u = 0; u < 16; ++u) s = s + fabs(v[u]);
  }
  for (; j < l1; ++j) s = s + fabs(p[(size_t)j * lda]);
  part[(size_t)blockIdx.y * m + i] = s;
}
static __global__ void fold_partials_kernel(const double* __restrict__ part, int nsplit, int m, double* __restrict__ out) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= m) return;
  double s = 0;
  for (int k = 0; k < nsplit; ++k) s = s + part[(size_t)k * m + i];
  out[i] = s;
}

template <typename T>
__global__ void __launch_bounds__(1024)
max_nan_kernel(const T* __restrict__ x, int m, T* __restrict__ out) {
  __shared__ T red[32];
  __shared__ int nan_s;
  if (threadIdx.x == 0) nan_s = 0;
  __syncthreads();
  T v = 0;
  int hasnan = 0;
  for (int i = threadIdx.x; i < m; i += blockDim.x) {
    T t = x[i];
    if (t != t) hasnan = 1;
    else if (t > v) v = t;
  }
  if (hasnan) nan_s = 1;
  for (int off = 16; off > 0; off >>= 1) { T o = __shfl_xor_sync(0xffffffffu, v, off); v = o > v ? o : v; }
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x < 32) {
    v = (threadIdx.x < (blockDim.x + 31) / 32) ? red[threadIdx.x] : T(0);
    for (int off = 16; off > 0; off >>= 1) { T o = __shfl_xor_sync(0xffffffffu, v, off); v = o > v ? o : v; }
    if (threadIdx.x == 0) *out = nan_s ? T(NAN) : v;
  }
}

// DLAG2S (SRC/dlag2s.f:135-146): FP64 -> FP32, flag = 1 if any |a| > FLT_MAX
// (a NaN passes, as in the reference).
static __global__ void dlag2s_kernel(const double* __restrict__ A, int lda, float* __restrict__ S, int lds, int m, int n,
                              int* __restrict__ overflow) {
  size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (size_t)m * n) return;
  int c = (int)(e / m), r = (int)(e - (size_t)c * m);
  double v = A[(size_t)r + (size_t)c * lda];
  const double rmax = 3.4028234663852886e38;
  if (v < -rmax || v > rmax) *overflow = 1;
  S[(size_t)r + (size_t)c * lds] = (float)v;
}

// DLANGE('I') row sums and DLAG2S in one pass over A (SRC/dlange.f:173-189,
// SRC/dlag2s.f:135-146): thread i of the grid owns row i of the column chunk
// blockIdx.y, converts every element to FP32 (flagging |a| > SLAMCH('O')) and
// sums |a| in column order; part[chunk][i] receives the chunk's sum.  Loads
// of 16 columns are issued together.
static __global__ void __launch_bounds__(128)
dlag2s_rowsum_kernel(const double* __restrict__ A, int lda, int m, int n, int chunk, float* __restrict__ S, int lds,
                     double* __restrict__ part, int* __restrict__ overflow, bool accumulate = false) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= m) return;
  const int l0 = blockIdx.y * chunk, l1 = min(n, l0 + chunk);
  // |a|, the overflow test |a| > SLAMCH('O') (false for NaN) and the
  // rounding to FP32 on the bit pattern with integer operations: the FP64
  // units, a few per SM on this GPU, are left with the sum
  constexpr unsigned long long kAbs = 0x7FFFFFFFFFFFFFFFull;
  constexpr unsigned long long kRmaxBits = 0x47EFFFFFE0000000ull;   // 3.4028234663852886e38
  constexpr unsigned long long kInfBits = 0x7FF0000000000000ull;
  const double* p = A + i;
  float* q = S + i;
  // accumulate: continue the row sums of the columns before (one running
  // sum per row in column order, the columns arriving in chunks)
  double s = accumulate ? part[(size_t)blockIdx.y * m + i] : 0.0;
  bool ovf = false;
  int j = l0;
  for (; j + 16 <= l1; j += 16) {
    double v[16];
#pragma unroll
    for (int u = 0; u < 16; ++u) v[u] = p[(size_t)(j + u) * lda];
#pragma unroll
    for (int u = 0; u < 16; ++u) {
      const unsigned long long bits = (unsigned long long)__double_as_longlong(v[u]);
      const unsigned long long ab = bits & kAbs;
      s = s + __longlong_as_double((long long)ab);
      ovf |= (ab > kRmaxBits) & (ab <= kInfBits);
      q[(size_t)(j + u) * lds] = __uint_as_float(f64_bits_to_f32_bits_rn(bits));
    }
  }
  for (; j < l1; ++j) {
    const unsigned long long bits = (unsigned long long)__double_as_longlong(p[(size_t)j * lda]);
    const unsigned long long ab = bits & kAbs;
    s = s + __longlong_as_double((long long)ab);
    ovf |= (ab > kRmaxBits) & (ab <= kInfBits);
    q[(size_t)j * lds] = __uint_as_float(f64_bits_to_f32_bits_rn(bits));
  }
  part[(size_t)blockIdx.y * m + i] = s;
  if (ovf) *overflow = 1;
}

// SLAG2D (SRC/slag2d.f:123-128).
static __global__ void slag2d_kernel(const float* __restrict__ S, int lds, double* __restrict__ A, int lda, int m, int n) {
  size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (size_t)m * n) return;
  int c = (int)(e / m), r = (int)(e - (size_t)c * m);
  A[(size_t)r + (size_t)c * lda] = (double)S[(size_t)r + (size_t)c * lds];
}

// SLAG2D followed by DAXPY with alpha = 1 (SRC/dsgesv.f:373-377):
// X(:,j) := X(:,j) + double(SX(:,j)).
static __global__ void lag2d_axpy_kernel(const float* __restrict__ S, int lds, double* __restrict__ X, int ldx, int n, int nrhs) {
  size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (size_t)n * nrhs) return;
  int c = (int)(e / n), r = (int)(e - (size_t)c * n);
  X[(size_t)r + (size_t)c * ldx] = X[(size_t)r + (size_t)c * ldx] + (double)S[(size_t)r + (size_t)c * lds];
}

// R = B - A*X in FP64 (DLACPY + DGEMM('N','N', alpha=-1, beta=1),
// SRC/dsgesv.f:328-332): one thread per row, columns folded in increasing
// order as the reference DGEMM does; up to 16 right-hand sides per pass so
// A is read once for nrhs <= 16.  X chunks are staged in shared memory.
constexpr int kResidRows = 64;
constexpr int kResidMaxRhs = 16;
template <bool EXACT>
__global__ void __launch_bounds__(kResidRows)
residual_kernel(const double* __restrict__ A, int lda, const double* __restrict__ X, int ldx,
                const double* __restrict__ B, int ldb, double* __restrict__ R, int ldr, int n, int nrhs) {
  __shared__ double xs[32][kResidMaxRhs];
  const int i = blockIdx.x * kResidRows + threadIdx.x;
  for (int q0 = 0; q0 < nrhs; q0 += kResidMaxRhs) {
    const int nq = min(kResidMaxRhs, nrhs - q0);
    double acc[kResidMaxRhs];
#pragma unroll
    for (int q = 0; q < kResidMaxRhs; ++q) acc[q] = (i < n && q < nq) ? B[(size_t)i + (size_t)(q0 + q) * ldb] : 0.0;
    for (int l0 = 0; l0 < n; l0 += 32) {
      const int nl = min(32, n - l0);
      __syncthreads();
      for (int e = threadIdx.x; e < 32 * kResidMaxRhs; e += kResidRows) {
        int l = e % 32, q = e / 32;
        xs[l][q] = (l < nl && q < nq) ? X[(size_t)(l0 + l) + (size_t)(q0 + q) * ldx] : 0.0;
      }
      __syncthreads();
      if (i < n) {
        double a[32];
#pragma unroll
        for (int u = 0; u < 32; ++u) a[u] = (u < nl) ? A[(size_t)i + (size_t)(l0 + u) * lda] : 0.0;
#pragma unroll
        for (int u = 0; u < 32; ++u) {
          if (u < nl) {
#pragma unroll
            for (int q = 0; q < kResidMaxRhs; ++q)
              if (q < nq) acc[q] = fnmadd<EXACT>(xs[u][q], a[u], acc[q]);
          }
        }
      }
    }
    if (i < n) {
#pragma unroll
      for (int q = 0; q < kResidMaxRhs; ++q)
        if (q < nq) R[(size_t)i + (size_t)(q0 + q) * ldr] = acc[q];
    }
  }
}


// Split-column form of the FP64 residual for the default (fused) mode.  On
// GB300 one dependent DFMA chain per row cannot fill the FP64 pipe, so the
// columns are cut into `nsplit` chunks: partial[s][q][i] is the sum over
// chunk s of A(i,l)*X(l,q), and residual_reduce_kernel folds the chunks in
// fixed order s = 0..nsplit-1 (deterministic run to run).
template <int RQ>
__global__ void __launch_bounds__(kResidRows)
residual_partial_kernel(const double* __restrict__ A, int lda, const double* __restrict__ X, int ldx, int n,
                        int nrhs, int q0, int chunk, double* __restrict__ partial) {
  __shared__ double xs[32][RQ];
  const int i = blockIdx.x * kResidRows + threadIdx.x;
  const int s = blockIdx.y;
  const int l_beg = s * chunk, l_end = min(n, l_beg + chunk);
  const int nq = min(RQ, nrhs - q0);
  double acc[RQ];
#pragma unroll
  for (int q = 0; q < RQ; ++q) acc[q] = 0.0;
  for (int l0 = l_beg; l0 < l_end; l0 += 32) {
    const int nl = min(32, l_end - l0);
    __syncthreads();
    for (int e = threadIdx.x; e < 32 * RQ; e += kResidRows) {
      int l = e % 32, q = e / 32;
      xs[l][q] = (l < nl && q < nq) ? X[(size_t)(l0 + l) + (size_t)(q0 + q) * ldx] : 0.0;
    }
    __syncthreads();
    if (i < n) {
      double a[32];
#pragma unroll
      for (int u = 0; u < 32; ++u) a[u] = (u < nl) ? A[(size_t)i + (size_t)(l0 + u) * lda] : 0.0;
#pragma unroll
      for (int u = 0; u < 32; ++u)
#pragma unroll
        for (int q = 0; q < RQ; ++q) acc[q] = fma(a[u], xs[u][q], acc[q]);
    }
  }
  if (i < n) {
#pragma unroll
    for (int q = 0; q < RQ; ++q)
      if (q < nq) partial[((size_t)s * RQ + q) * n + i] = acc[q];
  }
}

template <int RQ>
__global__ void residual_reduce_kernel(const double* __restrict__ partial, int nsplit, const double* __restrict__ B,
                                       int ldb, double* __restrict__ R, int ldr, int n, int nrhs, int q0) {
  size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int nq = min(RQ, nrhs - q0);
  if (e >= (size_t)n * nq) return;
  int q = (int)(e / n), i = (int)(e - (size_t)q * n);
  double sum = 0.0;
  for (int s = 0; s < nsplit; ++s) sum += partial[((size_t)s * RQ + q) * n + i];
  R[(size_t)i + (size_t)(q0 + q) * ldr] = B[(size_t)i + (size_t)(q0 + q) * ldb] - sum;
}

// Convergence test of SRC/dsgesv.f:337-342 for every right-hand side:
// XNRM = |X(IDAMAX(X(:,j)),j)|, RNRM likewise, not converged when
// RNRM > XNRM*CTE with CTE = ||A||_inf * eps * sqrt(n).  One CTA per
// right-hand side; `notconv` counts the failing ones.  With `nonfinite`
// (the library's NaN guard, off by default) a NaN or infinity in X or R
// sets *nonfinite instead of letting the NaN pass the test.
static __global__ void __launch_bounds__(256)
ir_check_kernel(const double* __restrict__ X, int ldx, const double* __restrict__ R, int ldr, int n,
                const double* __restrict__ anrm, int* __restrict__ notconv, double* __restrict__ norms_out,
                int* __restrict__ nonfinite = nullptr) {
  __shared__ Cand<double> red[2][8];
  const int j = blockIdx.x, tid = threadIdx.x;
  Cand<double> bx{0, -1, -1}, br{0, -1, -1};
  bool bad = false;
  for (int i = tid; i < n; i += 256) {
    const double xv = X[(size_t)i + (size_t)j * ldx], rv = R[(size_t)i + (size_t)j * ldr];
    Cand<double> cx = make_cand(xv, i, 0);
    Cand<double> cr = make_cand(rv, i, 0);
    if (cand_better(cx, bx)) bx = cx;
    if (cand_better(cr, br)) br = cr;
    bad |= !isfinite(xv) || !isfinite(rv);
  }
  if (nonfinite && __syncthreads_or(bad) && tid == 0) *nonfinite = 1;
  bx = warp_best(bx);
  br = warp_best(br);
  if ((tid & 31) == 0) { red[0][tid >> 5] = bx; red[1][tid >> 5] = br; }
  __syncthreads();
  if (tid == 0) {
    for (int w = 1; w < 8; ++w) {
      if (cand_better(red[0][w], red[0][0])) red[0][0] = red[0][w];
      if (cand_better(red[1][w], red[1][0])) red[1][0] = red[1][w];
    }
    int ix = red[0][0].row, ir = red[1][0].row;
    double xv = ix >= 0 ? X[(size_t)ix + (size_t)j * ldx] : 0.0;
    double rv = ir >= 0 ? R[(size_t)ir + (size_t)j * ldr] : 0.0;
    double xnrm = fabs(xv), rnrm = fabs(rv);
    const double eps = 1.1102230246251565e-16;
    double cte = (*anrm) * eps * sqrt((double)n) * 1.0;
    if (rnrm > xnrm * cte) atomicAdd(notconv, 1);
    if (norms_out) { norms_out[2 * j] = xnrm; norms_out[2 * j + 1] = rnrm; }
  }
}


// DLAG2S stop-at-first-overflow (SRC/dlag2s.f:137-144): the first pass finds
// the smallest column-major index with |a| > FLT_MAX, the second converts
// only the elements before it.
static __global__ void first_overflow_kernel(const double* __restrict__ A, int lda, int m, int n,
                                      unsigned long long* __restrict__ first) {
  size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (size_t)m * n) return;
  int c = (int)(e / m), r = (int)(e - (size_t)c * m);
  double v = A[(size_t)r + (size_t)c * lda];
  const double rmax = 3.4028234663852886e38;
  if (v < -rmax || v > rmax) atomicMin(first, (unsigned long long)e);
}
static __global__ void lag2s_upto_kernel(const double* __restrict__ A, int lda, float* __restrict__ S, int lds, int m, int n,
                                  const unsigned long long* __restrict__ first) {
  size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (size_t)m * n || e >= *first) return;
  int c = (int)(e / m), r = (int)(e - (size_t)c * m);
  S[(size_t)r + (size_t)c * lds] = (float)A[(size_t)r + (size_t)c * lda];
}

// DLANGE('1') column sums (SRC/dlange.f:155-163) in row order: a 32 x 32
// tile is staged through shared memory so each thread folds one column's
// values in increasing row order.
template <typename T>
__global__ void __launch_bounds__(1024)
col_abs_sum_kernel(const T* __restrict__ A, int lda, int m, int n, T* __restrict__ colsum) {
  __shared__ T tile[32][33];
  const int c0 = blockIdx.x * 32;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  T s = 0;
  for (int r0 = 0; r0 < m; r0 += 32) {
    int r = r0 + tx, c = c0 + ty;
    tile[ty][tx] = (r < m && c < n) ? A[(size_t)r + (size_t)c * lda] : T(0);
    __syncthreads();
    if (ty == 0) {
      int nr = min(32, m - r0);
      for (int k = 0; k < nr; ++k) { T v = tile[tx][k]; s = s + (v < 0 ? -v : v); }
    }
    __syncthreads();
  }
  if (ty == 0 && c0 + tx < n) colsum[c0 + tx] = s;
}

// max |a| with NaN propagation (DLANGE 'M', SRC/dlange.f:141-152).
template <typename T>
__global__ void max_abs_kernel(const T* __restrict__ A, int lda, int m, int n, unsigned long long* __restrict__ bits,
                               int* __restrict__ nanflag) {
  size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (size_t)m * n) return;
  int c = (int)(e / m), r = (int)(e - (size_t)c * m);
  double v = (double)A[(size_t)r + (size_t)c * lda];
  if (v != v) { *nanflag = 1; return; }
  v = fabs(v);
  atomicMax(bits, (unsigned long long)__double_as_longlong(v));
}
static __global__ void sumsq_scaled_kernel(const double* __restrict__ A, int lda, int m, int n,
                                    const unsigned long long* __restrict__ bits, double* __restrict__ acc) {
  size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (size_t)m * n) return;
  int c = (int)(e / m), r = (int)(e - (size_t)c * m);
  double scale = __longlong_as_double((long long)*bits);
  if (!(scale > 0) || isinf(scale)) return;
  double v = A[(size_t)r + (size_t)c * lda] / scale;
  atomicAdd(acc, v * v);
}

}  // namespace gb
