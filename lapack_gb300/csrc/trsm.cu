// Triangular solves with many right-hand sides for the LU: the block row
// of U, U12 = L11^{-1} A12 (SRC/dgetrf.f:204 and SRC/dgetrf2.f:240 calling
// BLAS/SRC/dtrsm.f:290-300, unit lower, left side, no transpose).  Kept in
// a translation unit of its own: the fully unrolled solves are the slowest
// code to compile.
#include "driver.h"
#include "prof.h"
#include "lu_kernels.cuh"

namespace gb {

// ------------------------------------------------------------------- TRSM
template <typename T, bool EXACT, int LPC>
static int launch_trsm_leaf_l(const T* L, int ldl, T* B, int ldb, int k, int ncols, cudaStream_t s) {
  static bool attr[64] = {false};
  int dev = 0;
  cudaGetDevice(&dev);
  if (!attr[dev]) {
    GB_CUDA_TRY(cudaFuncSetAttribute(trsm_llnu_leaf_kernel<T, EXACT, LPC>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     trsm_leaf_smem<T>(kTrsmLeafMax, LPC)));
    attr[dev] = true;
  }
  constexpr int cpb = kTrsmThreads / LPC;
  const int grid = (ncols + cpb - 1) / cpb;
  GB_LAUNCH(trsm_llnu_leaf_kernel<T, EXACT, LPC><<<grid, kTrsmThreads, trsm_leaf_smem<T>(k, LPC), s>>>(L, ldl, B, ldb,
                                                                                                     k, ncols));
  return 0;
}

// lanes per column follow the height of L: one 8-row block per lane and step
template <typename T, bool EXACT>
static int launch_trsm_leaf(const T* L, int ldl, T* B, int ldb, int k, int ncols, cudaStream_t s) {
  prof_begin(kProfTrsm, s);
  if (k > 64) return launch_trsm_leaf_l<T, EXACT, 16>(L, ldl, B, ldb, k, ncols, s);
  if (k > 32) return launch_trsm_leaf_l<T, EXACT, 8>(L, ldl, B, ldb, k, ncols, s);
  return launch_trsm_leaf_l<T, EXACT, 4>(L, ldl, B, ldb, k, ncols, s);
}

// One-launch solve for 64 < k <= KMAX: LPC lanes per column, 16 when the
// columns are few (short chain), 4 when they are many (less staging).
template <typename T, bool EXACT, int KMAX, int LPC>
static int launch_trsm_tri_k(const T* L, int ldl, T* B, int ldb, int k, int ncols, cudaStream_t s) {
  static bool attr[64] = {false};
  int dev = 0;
  cudaGetDevice(&dev);
  constexpr int smem = trsm_tri_smem<T, KMAX, LPC>();
  if (!attr[dev]) {
    GB_CUDA_TRY(cudaFuncSetAttribute(trsm_llnu_tri_kernel<T, EXACT, KMAX, LPC>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
    attr[dev] = true;
  }
  constexpr int cpb = kTrsmThreads / LPC;
  const int grid = (ncols + cpb - 1) / cpb;
  GB_LAUNCH(trsm_llnu_tri_kernel<T, EXACT, KMAX, LPC><<<grid, kTrsmThreads, smem, s>>>(L, ldl, B, ldb, k, ncols));
  return 0;
}

template <typename T, bool EXACT, int KMAX>
static int launch_trsm_tri(const T* L, int ldl, T* B, int ldb, int k, int ncols, cudaStream_t s) {
  prof_begin(kProfTrsm, s);
  // 256 rows: 16 lanes per column keep a lane's 16 rows in registers (the
  // fully unrolled solve of fewer lanes exceeds the unroller's limit)
  constexpr int kWide = KMAX > 128 ? 16 : 4;
  int rc = ncols <= 2048 ? launch_trsm_tri_k<T, EXACT, KMAX, 16>(L, ldl, B, ldb, k, ncols, s)
                         : launch_trsm_tri_k<T, EXACT, KMAX, kWide>(L, ldl, B, ldb, k, ncols, s);
  prof_end(kProfTrsm, s, (double)k * k * ncols, sizeof(T) * ((double)k * k + 2.0 * k * ncols));
  return rc;
}

// B := L^{-1} B, L unit lower k x k: one leaf launch up to 128 rows (4 to
// 16 lanes per column, 8-row blocks); with one_launch, the packed-triangle
// kernel for 64 < k <= 256 (FP32) or 128 (FP64), whose several lanes per
// column suit the wide block row of U; GEMM for the coupling beyond.
// one_launch = false keeps to the leaf kernel and the GEMM (the panel's
// solves, which run beside the trailing update).
template <typename T>
int trsm_llnu_dev(int k, int ncols, const T* L, int ldl, T* B, int ldb, cudaStream_t s, int gemm_mode,
                  bool one_launch) {
  if (k <= 0 || ncols <= 0) return 0;
  if (one_launch && k > kLeafMax && k <= (sizeof(T) == 4 ? 256 : 128)) {
    int rc;
    if (k <= 128)
      rc = options().exact ? launch_trsm_tri<T, true, 128>(L, ldl, B, ldb, k, ncols, s)
                           : launch_trsm_tri<T, false, 128>(L, ldl, B, ldb, k, ncols, s);
    else if constexpr (sizeof(T) == 4)
      rc = options().exact ? launch_trsm_tri<T, true, 256>(L, ldl, B, ldb, k, ncols, s)
                           : launch_trsm_tri<T, false, 256>(L, ldl, B, ldb, k, ncols, s);
    else
      rc = (int)cudaErrorInvalidValue;
    if (rc) return rc;
    return (int)cudaGetLastError();
  }
  if (k <= kTrsmLeafMax) {
    int rc = options().exact ? launch_trsm_leaf<T, true>(L, ldl, B, ldb, k, ncols, s)
                             : launch_trsm_leaf<T, false>(L, ldl, B, ldb, k, ncols, s);
    if (rc) return rc;
    prof_end(kProfTrsm, s, (double)k * k * ncols, sizeof(T) * ((double)k * k + 2.0 * k * ncols));
    return (int)cudaGetLastError();
  }
  const int kone = (one_launch ? (sizeof(T) == 4 ? 256 : 128) : kTrsmLeafMax);   // largest single solve
  int k1 = ((k / 2) + kLeafMax - 1) / kLeafMax * kLeafMax;
  if (k1 > kone) k1 = kone;
  if (k1 >= k) k1 = kLeafMax;
  int rc = trsm_llnu_dev<T>(k1, ncols, L, ldl, B, ldb, s, gemm_mode, one_launch);
  if (rc) return rc;
  rc = gemm_update_dev<T>(k - k1, ncols, k1, L + k1, ldl, B, ldb, B + k1, ldb, s, gemm_mode);
  if (rc) return rc;
  return trsm_llnu_dev<T>(k - k1, ncols, L + k1 + (size_t)k1 * ldl, ldl, B + k1, ldb, s, gemm_mode, one_launch);
}
template int trsm_llnu_dev<double>(int, int, const double*, int, double*, int, cudaStream_t, int, bool);
template int trsm_llnu_dev<float>(int, int, const float*, int, float*, int, cudaStream_t, int, bool);


}  // namespace gb

namespace gb {

// ---------------------------------------------------------------------------
// Inverse X = L^{-1} of a unit lower triangular k x k matrix (k <= 512), in
// 64-row blocks.  (1) Each diagonal block is inverted by one CTA, thread j
// forward-substituting unit vector e_j in registers; blocks above the
// diagonal are zeroed.  (2) One CTA per block column J computes, for
// I = J+1, ..., X_IJ = -X_II * (sum_{K=J}^{I-1} L_IK X_KJ) with 64 x 64
// products in shared memory.  Used in the default (BF16x3) mode to form the
// block row of U as one product L11^{-1} A12.
constexpr int kInvB = 64;
constexpr int kInvLd = kInvB + 1;

template <typename T>
static __global__ void __launch_bounds__(kInvB)
unit_lower_diag_inv_kernel(const T* __restrict__ L, int ldl, int k, T* __restrict__ X, int ldx) {
  __shared__ T D[kInvB * kInvLd];
  const int bI = blockIdx.x, r0 = bI * kInvB, nb = min(kInvB, k - r0);
  const int j = threadIdx.x;
  for (int e = j; e < kInvB * kInvB; e += kInvB) {
    const int r = e & 63, c = e >> 6;
    D[r * kInvLd + c] = (r < nb && c < nb) ? L[(size_t)(r0 + r) + (size_t)(r0 + c) * ldl] : T(0);
  }
  // zero the blocks of X above the diagonal in this block column
  for (int r = j; r < r0; r += kInvB)
    for (int c = 0; c < nb; ++c) X[(size_t)r + (size_t)(r0 + c) * ldx] = T(0);
  __syncthreads();
  T x[kInvB];
#pragma unroll
  for (int i = 0; i < kInvB; ++i) {
    T s = T(0);
#pragma unroll
    for (int q = 0; q < i; ++q) s = fma(D[i * kInvLd + q], x[q], s);
    x[i] = (i < j) ? T(0) : ((i == j ? T(1) : T(0)) - s);
  }
  if (j < nb) {
#pragma unroll
    for (int i = 0; i < kInvB; ++i)
      if (i < nb) X[(size_t)(r0 + i) + (size_t)(r0 + j) * ldx] = x[i];
  }
}

// C (64 x 64, ld kInvLd, shared) = alpha * A * B + (accumulate ? C : 0) for
// 64 x 64 shared operands; 256 threads, a 4 x 4 block each.
template <typename T>
__device__ __forceinline__ void inv_block_mm(const T* A, const T* B, T* C, bool accumulate, T alpha) {
  const int tid = threadIdx.x, tr = (tid & 15) * 4, tc = (tid >> 4) * 4;
  T acc[4][4];
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int b = 0; b < 4; ++b) acc[a][b] = T(0);
  for (int q = 0; q < kInvB; ++q) {
    T av[4], bv[4];
#pragma unroll
    for (int a = 0; a < 4; ++a) av[a] = A[(tr + a) * kInvLd + q];
#pragma unroll
    for (int b = 0; b < 4; ++b) bv[b] = B[q * kInvLd + tc + b];
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
      for (int b = 0; b < 4; ++b) acc[a][b] = fma(av[a], bv[b], acc[a][b]);
  }
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int b = 0; b < 4; ++b) {
      T* c = C + (tr + a) * kInvLd + tc + b;
      *c = (accumulate ? *c : T(0)) + alpha * acc[a][b];
    }
}

template <typename T>
static __global__ void __launch_bounds__(256)
unit_lower_offdiag_inv_kernel(const T* __restrict__ L, int ldl, int k, T* __restrict__ X, int ldx) {
  extern __shared__ __align__(16) unsigned char inv_smem[];
  T* Xc = reinterpret_cast<T*>(inv_smem);          // [nblk][64][65]: X_KJ of this block column
  const int nblk = (k + kInvB - 1) / kInvB;
  T* Lt = Xc + (size_t)nblk * kInvB * kInvLd;      // L_IK
  T* Tt = Lt + kInvB * kInvLd;                     // running sum
  T* Dt = Tt + kInvB * kInvLd;                     // X_II
  const int J = blockIdx.x, tid = threadIdx.x;
  auto load_block = [&](const T* src, int lds, int I, int K, T* dst) {
    const int r0 = I * kInvB, c0 = K * kInvB, nr = min(kInvB, k - r0), nc = min(kInvB, k - c0);
    for (int e = tid; e < kInvB * kInvB; e += 256) {
      const int r = e & 63, c = e >> 6;
      dst[r * kInvLd + c] = (r < nr && c < nc) ? src[(size_t)(r0 + r) + (size_t)(c0 + c) * lds] : T(0);
    }
  };
  load_block(X, ldx, J, J, Xc + (size_t)J * kInvB * kInvLd);
  for (int I = J + 1; I < nblk; ++I) {
    for (int K = J; K < I; ++K) {
      __syncthreads();
      load_block(L, ldl, I, K, Lt);
      __syncthreads();
      inv_block_mm(Lt, Xc + (size_t)K * kInvB * kInvLd, Tt, K > J, T(1));
    }
    __syncthreads();
    load_block(X, ldx, I, I, Dt);
    __syncthreads();
    T* XI = Xc + (size_t)I * kInvB * kInvLd;
    inv_block_mm(Dt, Tt, XI, false, T(-1));
    __syncthreads();
    const int r0 = I * kInvB, c0 = J * kInvB, nr = min(kInvB, k - r0), nc = min(kInvB, k - c0);
    for (int e = tid; e < kInvB * kInvB; e += 256) {
      const int r = e & 63, c = e >> 6;
      if (r < nr && c < nc) X[(size_t)(r0 + r) + (size_t)(c0 + c) * ldx] = XI[r * kInvLd + c];
    }
  }
}

template <typename T>
int unit_lower_inverse_dev(int k, const T* L, int ldl, T* X, int ldx, cudaStream_t s) {
  if (k <= 0) return 0;
  const int nblk = (k + kInvB - 1) / kInvB;
  if (nblk > 8) return (int)cudaErrorInvalidValue;
  prof_begin(kProfTrsm, s);
  GB_LAUNCH(unit_lower_diag_inv_kernel<T><<<nblk, kInvB, 0, s>>>(L, ldl, k, X, ldx));
  if (nblk > 1) {
    const int smem = (int)(sizeof(T) * (size_t)(nblk + 3) * kInvB * kInvLd);
    static bool attr[64] = {false};
    int dev = 0;
    cudaGetDevice(&dev);
    if (!attr[dev]) {
      int optin = 0;
      cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
      GB_CUDA_TRY(cudaFuncSetAttribute(unit_lower_offdiag_inv_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       optin));
      attr[dev] = true;
    }
    GB_LAUNCH(unit_lower_offdiag_inv_kernel<T><<<nblk - 1, 256, smem, s>>>(L, ldl, k, X, ldx));
  }
  prof_end(kProfTrsm, s, (double)k * k * k / 3.0, sizeof(T) * 2.0 * k * k);
  return (int)cudaGetLastError();
}
template int unit_lower_inverse_dev<float>(int, const float*, int, float*, int, cudaStream_t);

}  // namespace gb
