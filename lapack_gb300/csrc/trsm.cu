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
template <typename T, bool EXACT, int KMAX>
static int launch_trsm_leaf_k(int grid, const T* L, int ldl, T* B, int ldb, int k, int ncols, cudaStream_t s) {
  static bool attr[64] = {false};
  int dev = 0;
  cudaGetDevice(&dev);
  if (!attr[dev]) {
    GB_CUDA_TRY(cudaFuncSetAttribute(trsm_llnu_leaf_kernel<T, EXACT, KMAX>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     trsm_leaf_smem<T, KMAX>()));
    attr[dev] = true;
  }
  GB_LAUNCH(trsm_llnu_leaf_kernel<T, EXACT, KMAX><<<grid, kTrsmThreads, trsm_leaf_smem<T, KMAX>(), s>>>(L, ldl, B, ldb,
                                                                                                     k, ncols));
  return 0;
}

// the unrolled solve is sized to the leaf: 16, 32 or 64 rows
template <typename T, bool EXACT>
static int launch_trsm_leaf(int grid, const T* L, int ldl, T* B, int ldb, int k, int ncols, cudaStream_t s) {
  prof_begin(kProfTrsm, s);
  int rc;
  if (k <= 16) rc = launch_trsm_leaf_k<T, EXACT, 16>(grid, L, ldl, B, ldb, k, ncols, s);
  else if (k <= 32) rc = launch_trsm_leaf_k<T, EXACT, 32>(grid, L, ldl, B, ldb, k, ncols, s);
  else rc = launch_trsm_leaf_k<T, EXACT, 64>(grid, L, ldl, B, ldb, k, ncols, s);
  return rc;
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

// B := L^{-1} B, L unit lower k x k: leaves of at most 64 rows, one launch
// up to 256 rows (FP32) or 128 rows (FP64), GEMM for the coupling beyond.
// one_launch = false keeps to the leaf kernel and the GEMM (small shared
// memory footprint: the panel's solves run beside the trailing update).
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
  if (k <= kLeafMax) {
    int grid = (ncols + kTrsmCols - 1) / kTrsmCols;
    int rc = options().exact ? launch_trsm_leaf<T, true>(grid, L, ldl, B, ldb, k, ncols, s)
                             : launch_trsm_leaf<T, false>(grid, L, ldl, B, ldb, k, ncols, s);
    if (rc) return rc;
    prof_end(kProfTrsm, s, (double)k * k * ncols, sizeof(T) * ((double)k * k + 2.0 * k * ncols));
    return (int)cudaGetLastError();
  }
  const int kone = (one_launch ? (sizeof(T) == 4 ? 256 : 128) : kLeafMax);   // largest single solve
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
