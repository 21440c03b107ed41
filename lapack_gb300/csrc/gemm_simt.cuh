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

template <typename T, int BM, int BN, int BK, int TM, int TN, bool EXACT>
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

  T acc[TM][TN];
#pragma unroll
  for (int j = 0; j < TN; ++j) {
    int n = n0 + ty + j * (BN / TN);
#pragma unroll
    for (int i = 0; i < TM; ++i) {
      int m = m0 + tx + i * TX;
      acc[i][j] = (m < M && n < N) ? C[(size_t)m + (size_t)n * ldc] : T(0);
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
        for (int j = 0; j < TN; ++j) acc[i][j] = fnmadd<EXACT>(a[i], b[j], acc[i][j]);
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
      if (m < M && n < N) C[(size_t)m + (size_t)n * ldc] = acc[i][j];
    }
  }
}

}  // namespace gb
