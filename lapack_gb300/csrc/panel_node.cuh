// One node of the recursive panel factorization, fused into one launch:
// U12 = L11^{-1} A12 (SRC/dgetrf2.f:240, BLAS/SRC/dtrsm.f:290-300) and
// A22 := A22 - A21 * U12 (SRC/dgetrf2.f:247, BLAS/SRC/dgemm.f:337-341) for
// a node whose halves are at most 64 columns wide.
//
// The two steps of the node used to be two dependent launches: a one- or
// two-CTA triangular solve whose k-step chain is pure latency, then the
// update over all rows.  Here every CTA solves the (at most 64 x 64) U12
// itself from shared memory while its loads of A21 and A22 are in flight,
// then updates its 128 rows of A22 with it.  The CTA that arrives last at
// the node counter (all CTAs have then read A12) writes U12 over A12 and
// resets the counter for the next node: no CTA waits on another.
//
// Arithmetic order: the solve is that of trsm_llnu_leaf_kernel (row i of
// column c updated by x_k * L(i, k) for k ascending, solve_unit_lower_cols)
// and the update folds k in increasing order into C as
// gemm_nn_update_kernel does, so the node's result is bitwise that of the
// two separate launches, in the exact mode too.
#pragma once
#include <algorithm>

#include "common.cuh"
#include "driver.h"
#include "lu_kernels.cuh"
#include "prof.h"

namespace gb {

constexpr int kNodeThreads = 256;
constexpr int kNodeBM = 128;        // rows of A22 per CTA
constexpr int kNodeUCols = 64;      // widest right half (four lanes per column in the solve)
constexpr int kNodeMaxK = 64;       // widest left half

// L11 by columns (ldt x ldt), U12 by columns (64 x ldx), A21 tile (k x 128)
template <typename T>
__host__ __device__ constexpr int node_smem(int k) {
  return (trsm_ldt(k) * trsm_ldt(k) + trsm_ldx<T>(k) * kNodeUCols + k * kNodeBM) * (int)sizeof(T);
}

// A11 points at the node's top-left element; the node covers rows [0, M)
// and columns [0, k + nc) from there: L11 = A11(0:k, 0:k), A12 = A11(0:k,
// k:k+nc), A21 = A11(k:M, 0:k), A22 = A11(k:M, k:k+nc).  Grid: max(1,
// ceil((M-k)/128)) CTAs.  *node_count is zero on entry and on exit.
// TN = columns of A22 per thread (16 threads along the columns).
template <typename T, bool EXACT, int TN>
__global__ void __launch_bounds__(kNodeThreads)
panel_node_kernel(T* __restrict__ A11, int lda, int M, int k, int nc, int* __restrict__ node_count) {
  constexpr int TM = kNodeBM / 16;               // update: rows per thread (8)
  static_assert(16 * TN <= kNodeUCols, "right half wider than 64 columns");
  extern __shared__ __align__(16) unsigned char node_smem_raw[];
  const int ldt = trsm_ldt(k), ldu = trsm_ldx<T>(k);
  T* Lt = reinterpret_cast<T*>(node_smem_raw);   // Lt[j * ldt + i] = L(i, j)
  T* Us = Lt + ldt * ldt;                        // Us[c * ldu + i] = A12(i, c), then U12
  T* As = Us + ldu * kNodeUCols;                 // As[l * 128 + r] = A21(m0 + r, l)
  const int tid = threadIdx.x;
  const int m0 = blockIdx.x * kNodeBM;           // first row of this CTA's A22 block (below k)
  const int M2 = M - k;                          // rows of A21 / A22

  // (1) L11 and A12 into shared memory (cp.async group 1)
  stage_cols_async<T, kNodeThreads>(A11, lda, k, k, Lt, ldt, tid);
  stage_cols_async<T, kNodeThreads>(A11 + (size_t)k * lda, lda, k, nc, Us, ldu, tid);
  cp_async_commit();
  // (2) the A21 tile (group 2, zero beyond M2), in flight during the solve
  if (m0 < M2) {
    for (int e = tid; e < k * kNodeBM; e += kNodeThreads) {
      const int l = e / kNodeBM, r = e - l * kNodeBM;
      const bool ok = m0 + r < M2;
      const T* src = A11 + (size_t)(k + (ok ? m0 + r : 0)) + (size_t)l * lda;
      cp_async_elem_zfill(As + l * kNodeBM + r, src, ok);
    }
  }
  cp_async_commit();
  // (3) this thread's block of A22: rows 4 tx .. 4 tx + 3 and 64 + 4 tx ..
  // 64 + 4 tx + 3 (two 16-byte shared-memory vectors of A21 per k), columns
  // ty, ty + 16, ...
  const int tx = tid & 15, ty = tid >> 4;
  auto row_of = [&](int i) { return (i < 4 ? 4 * tx + i : 64 + 4 * tx + (i - 4)); };
  T acc[TM][TN];
  auto load_acc = [&]() {
#pragma unroll
    for (int j = 0; j < TN; ++j) {
      const int c = ty + 16 * j;
#pragma unroll
      for (int i = 0; i < TM; ++i) {
        const int r = m0 + row_of(i);
        acc[i][j] = (r < M2 && c < nc) ? A11[(size_t)(k + r) + (size_t)(k + c) * lda] : T(0);
      }
    }
  };
  load_acc();                                    // its latency hides behind the solve
  cp_async_wait<1>();                            // group 1: L11 and A12
  __syncthreads();
  // every CTA has read A12 once it passes the counter; the last one writes U12
  __shared__ int last_s;
  if (tid == 0) {
    __threadfence();
    const int prev = atomicAdd(node_count, 1);
    last_s = (prev == (int)gridDim.x - 1);
  }
  // (4) U12 = L11^{-1} A12 in shared memory, four lanes per column
  solve_unit_lower_cols<T, EXACT, 4>(Lt, ldt, Us, ldu, k, nc, tid);
  cp_async_wait<0>();                            // group 2: the A21 tile
  __syncthreads();
  if (last_s) {
    const int warp = tid >> 5, lane = tid & 31;
    for (int c = warp; c < nc; c += kNodeThreads / 32)
      for (int r = lane; r < k; r += 32) A11[(size_t)r + (size_t)(k + c) * lda] = Us[c * ldu + r];
    if (tid == 0) *node_count = 0;
  }
  if (m0 >= M2) return;

  // (5) A22 block -= A21 block * U12, k ascending
  static_assert(TM == 8, "two 4-row groups per thread");
  for (int l = 0; l < k; ++l) {
    T a[TM], b[TN];
    const T* ar = As + l * kNodeBM + 4 * tx;
    if constexpr (sizeof(T) == 4) {
      const float4 p = *reinterpret_cast<const float4*>(ar), q = *reinterpret_cast<const float4*>(ar + 64);
      a[0] = p.x; a[1] = p.y; a[2] = p.z; a[3] = p.w; a[4] = q.x; a[5] = q.y; a[6] = q.z; a[7] = q.w;
    } else {
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const double2 p = *reinterpret_cast<const double2*>(ar + 64 * h),
                      q = *reinterpret_cast<const double2*>(ar + 64 * h + 2);
        a[4 * h] = p.x; a[4 * h + 1] = p.y; a[4 * h + 2] = q.x; a[4 * h + 3] = q.y;
      }
    }
#pragma unroll
    for (int j = 0; j < TN; ++j) b[j] = Us[(ty + 16 * j) * ldu + l];
#pragma unroll
    for (int i = 0; i < TM; ++i)
#pragma unroll
      for (int j = 0; j < TN; ++j) acc[i][j] = fnmadd<EXACT>(a[i], b[j], acc[i][j]);
  }
#pragma unroll
  for (int j = 0; j < TN; ++j) {
    const int c = ty + 16 * j;
#pragma unroll
    for (int i = 0; i < TM; ++i) {
      const int r = m0 + row_of(i);
      if (r < M2 && c < nc) A11[(size_t)(k + r) + (size_t)(k + c) * lda] = acc[i][j];
    }
  }
}

// ------------------------------------------------------- fused panel node
template <typename T, bool EXACT, int TN>
static int launch_node_k(T* A11, int lda, int M, int k, int nc, int* node_count, cudaStream_t s) {
  static bool attr[64] = {false};
  int dev = 0;
  cudaGetDevice(&dev);
  if (!attr[dev]) {
    GB_CUDA_TRY(cudaFuncSetAttribute(panel_node_kernel<T, EXACT, TN>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     node_smem<T>(kNodeMaxK)));
    attr[dev] = true;
  }
  const int grid = std::max(1, (M - k + kNodeBM - 1) / kNodeBM);
  GB_LAUNCH(panel_node_kernel<T, EXACT, TN><<<grid, kNodeThreads, node_smem<T>(k), s>>>(A11, lda, M, k, nc, node_count));
  return 0;
}

template <typename T, bool EXACT>
static int launch_node(T* A11, int lda, int M, int k, int nc, int* node_count, cudaStream_t s) {
  if (nc <= 16) return launch_node_k<T, EXACT, 1>(A11, lda, M, k, nc, node_count, s);
  if (nc <= 32) return launch_node_k<T, EXACT, 2>(A11, lda, M, k, nc, node_count, s);
  return launch_node_k<T, EXACT, 4>(A11, lda, M, k, nc, node_count, s);
}

template <typename T>
int panel_node_dev(T* A11, int lda, int M, int k, int nc, int* node_count, cudaStream_t s) {
  if (k <= 0 || nc <= 0) return 0;
  if (k > kNodeMaxK || nc > kNodeUCols || M < k || !node_count) return (int)cudaErrorInvalidValue;
  prof_begin(kProfTrsm, s);
  const int rc = options().exact ? launch_node<T, true>(A11, lda, M, k, nc, node_count, s)
                                 : launch_node<T, false>(A11, lda, M, k, nc, node_count, s);
  if (rc) return rc;
  prof_end(kProfTrsm, s, (double)k * k * nc + 2.0 * (double)(M - k) * nc * k,
           sizeof(T) * ((double)k * k + 2.0 * k * nc + (double)(M - k) * k + 2.0 * (double)(M - k) * nc));
  return (int)cudaGetLastError();
}
}  // namespace gb
