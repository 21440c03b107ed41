// Trailing-matrix update C := C - A*B on the CUDA cores (DFMA for FP64,
// FFMA for the FP32 form), the DGEMM('N','N', alpha=-1, beta=1) call of
// SRC/dgetrf.f:212-216.  Column-major operands.
//
// Each thread keeps a TM x TN block of C in registers, loaded from C before
// the K loop, and folds the K products into it in increasing k -- the
// per-element order of the reference loop (BLAS/SRC/dgemm.f:337-341).  With
// EXACT the product and the subtraction round separately, as the reference
// computes them; otherwise they fuse into one FMA.
//
// On GB300 the FP64 units retire about two DFMA per clock per SM, so the
// FP64 form is compute-bound for any K here and needs no tensor path (the
// f64 mma.sync measured slower than DFMA on this part).
#pragma once
#include "common.cuh"

namespace gb {

// SUM_FIRST: the products are summed from zero in increasing k and the sum
// subtracted from C once (the 'T','N' form of BLAS/SRC/dgemm.f:348-360 with
// ALPHA = -1, BETA = 1) instead of each product subtracted in turn.
// TRI: 1 stores only the elements on or below the diagonal of C, 2 only
// those on or above it (DSYRK's triangle).  SKIPZ: a term whose B element is
// zero is skipped (BLAS/SRC/dsyrk.f:313-320, IF (A(J,L).NE.ZERO)).
template <typename T, int BM, int BN, int BK, int TM, int TN, bool EXACT, bool SUM_FIRST = false, int TRI = 0,
          bool SKIPZ = false>
__global__ void __launch_bounds__((BM / TM) * (BN / TN), 1)
gemm_nn_update_kernel(int M, int N, int K, const T* __restrict__ A, int lda,
                      const T* __restrict__ B, int ldb, T* __restrict__ C, int ldc) {
  constexpr int NT = (BM / TM) * (BN / TN);
  constexpr int TX = BM / TM;          // threads along M
  __shared__ __align__(16) T As[2][BK][BM];
  __shared__ __align__(16) T Bs[2][BK][BN];
  const int tid = threadIdx.x;
  const int tx = tid % TX, ty = tid / TX;
  const int m0 = blockIdx.x * BM, n0 = blockIdx.y * BN;
  if ((TRI == 1 && m0 + BM <= n0) || (TRI == 2 && m0 >= n0 + BN)) return;   // tile outside the triangle

  T acc[TM][TN];
#pragma unroll
  for (int j = 0; j < TN; ++j) {
    int n = n0 + ty + j * (BN / TN);
#pragma unroll
    for (int i = 0; i < TM; ++i) {
      int m = m0 + tx + i * TX;
      acc[i][j] = (!SUM_FIRST && m < M && n < N) ? C[(size_t)m + (size_t)n * ldc] : T(0);
    }
  }

  constexpr int A_PER = (BM * BK) / NT;
  constexpr int B_PER = (BK * BN) / NT;
  static_assert(A_PER * NT == BM * BK && B_PER * NT == BK * BN, "tile/thread mismatch");
  T ra[A_PER], rb[B_PER];

  auto load_global = [&](int k0) {
#pragma unroll
    for (int s = 0; s < A_PER; ++s) {
      int e = tid + s * NT;
      int mm = e % BM, kk = e / BM;
      int m = m0 + mm, k = k0 + kk;
      ra[s] = (m < M && k < K) ? A[(size_t)m + (size_t)k * lda] : T(0);
    }
#pragma unroll
    for (int s = 0; s < B_PER; ++s) {
      int e = tid + s * NT;
      int kk = e % BK, nn = e / BK;
      int k = k0 + kk, n = n0 + nn;
      rb[s] = (k < K && n < N) ? B[(size_t)k + (size_t)n * ldb] : T(0);
    }
  };
  auto store_shared = [&](int buf) {
#pragma unroll
    for (int s = 0; s < A_PER; ++s) {
      int e = tid + s * NT;
      As[buf][e / BM][e % BM] = ra[s];
    }
#pragma unroll
    for (int s = 0; s < B_PER; ++s) {
      int e = tid + s * NT;
      Bs[buf][e % BK][e / BK] = rb[s];
    }
  };

  const int nk = (K + BK - 1) / BK;
  if (nk == 0) return;
  load_global(0);
  store_shared(0);
  __syncthreads();
  for (int t = 0; t < nk; ++t) {
    const int buf = t & 1;
    if (t + 1 < nk) load_global((t + 1) * BK);
    const int kmax = min(BK, K - t * BK);
    for (int kk = 0; kk < kmax; ++kk) {
      T a[TM], b[TN];
#pragma unroll
      for (int i = 0; i < TM; ++i) a[i] = As[buf][kk][tx + i * TX];
#pragma unroll
      for (int j = 0; j < TN; ++j) b[j] = Bs[buf][kk][ty + j * (BN / TN)];
#pragma unroll
      for (int i = 0; i < TM; ++i)
#pragma unroll
        for (int j = 0; j < TN; ++j) {
          const T r = SUM_FIRST ? fmadd<EXACT>(a[i], b[j], acc[i][j]) : fnmadd<EXACT>(a[i], b[j], acc[i][j]);
          acc[i][j] = (SKIPZ && b[j] == T(0)) ? acc[i][j] : r;
        }
    }
    if (t + 1 < nk) {
      store_shared(buf ^ 1);
      __syncthreads();
    }
  }
#pragma unroll
  for (int j = 0; j < TN; ++j) {
    int n = n0 + ty + j * (BN / TN);
#pragma unroll
    for (int i = 0; i < TM; ++i) {
      int m = m0 + tx + i * TX;
      if (m < M && n < N && (TRI != 1 || m >= n) && (TRI != 2 || m <= n)) {
        T* pc = C + (size_t)m + (size_t)n * ldc;
        if constexpr (SUM_FIRST) *pc = fnmadd<EXACT>(T(1), acc[i][j], *pc);   // C - sum, one rounding
        else *pc = acc[i][j];
      }
    }
  }
}

}  // namespace gb
