// Host orchestration of DGETRF / SGETRF and DGETRS / SGETRS on one GPU.
//
// DGETRF (SRC/dgetrf.f:174-219) is a blocked right-looking LU: for each
// block column of width NB, factor the panel (SRC/dgetrf2.f, here a
// recursion whose leaves of width <= 64 are the cooperative panel kernel),
// apply its interchanges to the other columns, form the block row of U with
// a triangular solve, then update the trailing matrix with one GEMM.
#include <vector>

#include "driver.h"
#include "prof.h"
#include "gemm_simt.cuh"
#include "lu_kernels.cuh"
#include "panel_cluster.cuh"
#include "solve_kernels.cuh"
#include "trsv_stream.cuh"

#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <mutex>

namespace gb {

// ----------------------------------------------------------------- options
static int env_int(const char* name, int dflt) {
  const char* v = getenv(name);
  return (v && *v) ? atoi(v) : dflt;
}

Options& options() {
  static Options o = [] {
    Options x;
    x.exact = env_int("LAPACK_GB300_EXACT", 0) != 0;
    x.nb_f64 = std::max(1, env_int("LAPACK_GB300_NB64", 64));
    x.nb_f32 = std::max(1, env_int("LAPACK_GB300_NB32", 256));
    x.panel_ctas_f64 = env_int("LAPACK_GB300_PANEL_CTAS64", 0);
    x.panel_ctas_f32 = env_int("LAPACK_GB300_PANEL_CTAS32", 0);
    x.cluster_panel = env_int("LAPACK_GB300_CLUSTER_PANEL", 2);
    x.lookahead = env_int("LAPACK_GB300_LOOKAHEAD", 1);
    x.trsv_inv = env_int("LAPACK_GB300_TRSV_INV", 1);
    x.gemm_ws = env_int("LAPACK_GB300_GEMM_WS", 1);
    x.gemm_tiles = std::max(0, env_int("LAPACK_GB300_GEMM_TILES", 4));
    x.ir_nan_guard = env_int("LAPACK_GB300_IR_NAN_GUARD", 0);
    x.panel_fuse = env_int("LAPACK_GB300_PANEL_FUSE", 1);
    x.feed = env_int("LAPACK_GB300_FEED", 1);
    x.feed_lazy = env_int("LAPACK_GB300_FEED_LAZY", 0);
    x.pool_keep = env_int("LAPACK_GB300_POOL_KEEP", 1);
    x.feed_catchup = env_int("LAPACK_GB300_FEED_CATCHUP", 8);
    const char* mm = getenv("LAPACK_GB300_MIXED");
    if (mm && strcmp(mm, "fp32") == 0) x.mixed_mode = kMixedFp32;
    if (mm && strcmp(mm, "bf16x3") == 0) x.mixed_mode = kMixedBf16x3;
    const char* sm = getenv("LAPACK_GB300_SGETRF");
    if (sm && strcmp(sm, "bf16x3") == 0) x.sgetrf_mode = kMixedBf16x3;
    return x;
  }();
  return o;
}

int device_sm_count() {
  int dev = 0;
  cudaGetDevice(&dev);
  static int cache[64] = {0};
  if (dev < 64 && cache[dev]) return cache[dev];
  int n = 0;
  cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
  if (dev < 64) cache[dev] = n;
  return n;
}

// The scratch comes from the device's default stream-ordered pool.  By
// default the pool hands its memory back to the driver at every
// synchronisation, so each call would map its gigabytes again (and a pool
// growing while host->device copies run waits for them); with option
// pool_keep the pool keeps what it has grown to for the process (a
// property of this process's pool, nothing on the device).
static void keep_pool_memory() {
  static bool done[64] = {false};
  int dev = 0;
  if (!options().pool_keep || cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64 || done[dev]) return;
  done[dev] = true;
  cudaMemPool_t pool;
  if (cudaDeviceGetDefaultMemPool(&pool, dev) != cudaSuccess) {
    cudaGetLastError();
    return;
  }
  unsigned long long keep = ~0ull;
  if (cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep) != cudaSuccess) cudaGetLastError();
}

DevScratch::DevScratch(size_t bytes, cudaStream_t st) : s(st) {
  keep_pool_memory();
  if (bytes && cudaMallocAsync(&p, bytes, st) != cudaSuccess) p = nullptr;
}
DevScratch::~DevScratch() {
  if (p) cudaFreeAsync(p, s);
}

int check_status(int* dStatus, cudaStream_t s) {
  int h = 0;
  if (cudaMemcpyAsync(&h, dStatus, sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess) return -1;
  if (cudaStreamSynchronize(s) != cudaSuccess) return -1;
  return h;
}

// Per-device status word written by kernels whose bounded waits ran out.
int* device_status_word() {
  static std::mutex mu;
  static int* words[64] = {nullptr};
  int dev = 0;
  cudaGetDevice(&dev);
  std::lock_guard<std::mutex> lk(mu);
  if (!words[dev]) {
    int* p = nullptr;
    if (cudaMalloc(&p, sizeof(int)) != cudaSuccess) return nullptr;
    cudaMemset(p, 0, sizeof(int));
    cudaDeviceSynchronize();
    // keep stream-ordered scratch cached between calls instead of returning it to the OS
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
      uint64_t thr = UINT64_MAX;
      cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
      // scratch freed on one stream is not reused on another by inserting a
      // wait between the two (the look-ahead streams must stay independent)
      int no = 0;
      cudaMemPoolSetAttribute(pool, cudaMemPoolReuseAllowInternalDependencies, &no);
    }
    words[dev] = p;
  }
  return words[dev];
}

// ------------------------------------------------------------------- GEMM
template <>
int gemm_update_dev<double>(int M, int N, int K, const double* A, int lda, const double* B, int ldb, double* C,
                            int ldc, cudaStream_t s, int) {
  if (M <= 0 || N <= 0 || K <= 0) return 0;
  dim3 grid((M + 127) / 128, (N + 63) / 64);
  prof_begin(kProfGemmF64, s);
  if (options().exact)
    GB_LAUNCH(gemm_nn_update_kernel<double, 128, 64, 16, 8, 4, true><<<grid, 256, 0, s>>>(M, N, K, A, lda, B, ldb, C, ldc));
  else
    GB_LAUNCH(gemm_nn_update_kernel<double, 128, 64, 16, 8, 4, false><<<grid, 256, 0, s>>>(M, N, K, A, lda, B, ldb, C, ldc));
  prof_end(kProfGemmF64, s, 2.0 * M * N * (double)K, 8.0 * ((double)M * K + (double)K * N + 2.0 * M * N));
  return (int)cudaGetLastError();
}

template <>
int gemm_update_dev<float>(int M, int N, int K, const float* A, int lda, const float* B, int ldb, float* C, int ldc,
                           cudaStream_t s, int mode) {
  if (M <= 0 || N <= 0 || K <= 0) return 0;
  if (mode == kMixedBf16x3) return gemm_bf16x3_dev(M, N, K, A, lda, B, ldb, C, ldc, s);
  prof_begin(kProfGemmF32, s);
  const bool ex = options().exact;
  // tile width follows N: the narrow updates of the panel recursion (N <= 64)
  // get 128 x 16/32/64 tiles instead of computing mostly padding
  if (N <= 16) {
    dim3 grid((M + 127) / 128, (N + 15) / 16);
    if (ex) GB_LAUNCH(gemm_nn_update_kernel<float, 128, 16, 16, 4, 2, true><<<grid, 256, 0, s>>>(M, N, K, A, lda, B, ldb, C, ldc));
    else GB_LAUNCH(gemm_nn_update_kernel<float, 128, 16, 16, 4, 2, false><<<grid, 256, 0, s>>>(M, N, K, A, lda, B, ldb, C, ldc));
  } else if (N <= 32) {
    dim3 grid((M + 127) / 128, (N + 31) / 32);
    if (ex) GB_LAUNCH(gemm_nn_update_kernel<float, 128, 32, 8, 4, 4, true><<<grid, 256, 0, s>>>(M, N, K, A, lda, B, ldb, C, ldc));
    else GB_LAUNCH(gemm_nn_update_kernel<float, 128, 32, 8, 4, 4, false><<<grid, 256, 0, s>>>(M, N, K, A, lda, B, ldb, C, ldc));
  } else if (N <= 64) {
    dim3 grid((M + 127) / 128, (N + 63) / 64);
    if (ex) GB_LAUNCH(gemm_nn_update_kernel<float, 128, 64, 8, 4, 8, true><<<grid, 256, 0, s>>>(M, N, K, A, lda, B, ldb, C, ldc));
    else GB_LAUNCH(gemm_nn_update_kernel<float, 128, 64, 8, 4, 8, false><<<grid, 256, 0, s>>>(M, N, K, A, lda, B, ldb, C, ldc));
  } else {
    dim3 grid((M + 127) / 128, (N + 127) / 128);
    if (ex) GB_LAUNCH(gemm_nn_update_kernel<float, 128, 128, 8, 8, 8, true><<<grid, 256, 0, s>>>(M, N, K, A, lda, B, ldb, C, ldc));
    else GB_LAUNCH(gemm_nn_update_kernel<float, 128, 128, 8, 8, 8, false><<<grid, 256, 0, s>>>(M, N, K, A, lda, B, ldb, C, ldc));
  }
  prof_end(kProfGemmF32, s, 2.0 * M * N * (double)K, 4.0 * ((double)M * K + (double)K * N + 2.0 * M * N));
  return (int)cudaGetLastError();
}


// C -= A*B in the reference DGEMM orders (the Cholesky factorization's
// updates, SRC/dpotrf.f): sum_first false, each product subtracted from C in
// increasing k ('N','T' form, BLAS/SRC/dgemm.f:367-383); true, the products
// summed from zero in increasing k and the sum subtracted once ('T','N'
// form, dgemm.f:348-360).  Products separately rounded in exact mode, fused
// into one FMA otherwise (as the LU's updates).
// BK: the K depth staged per round.  The thin tiles run one or two CTAs per
// SM with a K of up to the matrix order, so each element's K chain waits on
// the next round's global loads unless a round covers many k: deeper rounds
// for the 16 x 16 and 8 x 8 tiles (within 48 KB of shared memory); 16 for
// the 128 x 64 and 32 x 32 tiles (deeper measured slower there).
template <typename T, int BM, int BN, int BK, int TM, int TN, bool SF, int TRI, bool SKIPZ>
static void launch_update_tile(int M, int N, int K, const T* A, int lda, const T* B, int ldb, T* C, int ldc,
                               cudaStream_t s) {
  dim3 grid((M + BM - 1) / BM, (N + BN - 1) / BN);
  if (options().exact)
    GB_LAUNCH(gemm_nn_update_kernel<T, BM, BN, BK, TM, TN, true, SF, TRI, SKIPZ>
              <<<grid, (BM / TM) * (BN / TN), 0, s>>>(M, N, K, A, lda, B, ldb, C, ldc));
  else
    GB_LAUNCH(gemm_nn_update_kernel<T, BM, BN, BK, TM, TN, false, SF, TRI, SKIPZ>
              <<<grid, (BM / TM) * (BN / TN), 0, s>>>(M, N, K, A, lda, B, ldb, C, ldc));
}

// The tile is the largest of 128 x 64 (M at least 128: the upper form's
// M = NB = 64 would leave half of it padding), 32 x 32 and 16 x 16 that
// still gives every SM a CTA: the Cholesky's updates are thin (N or M = NB =
// 64) with a long K, so the CTA count, not the per-CTA reuse, limits them
// (a 64 x 64 tile measured slower than 32 x 32 for these shapes).  The
// per-element order does not depend on the tile.
template <typename T, bool SF>
static void launch_update_by_size(int M, int N, int K, const T* A, int lda, const T* B, int ldb, T* C, int ldc,
                                  cudaStream_t s) {
  const long sms = device_sm_count();
  auto ctas = [&](int bm, int bn) { return (long)((M + bm - 1) / bm) * ((N + bn - 1) / bn); };
  constexpr int bk16 = sizeof(T) == 4 ? 128 : 64;
  if (M >= 128 && ctas(128, 64) >= sms)
    launch_update_tile<T, 128, 64, 16, 8, 4, SF, 0, false>(M, N, K, A, lda, B, ldb, C, ldc, s);
  else if (ctas(32, 32) >= sms)
    launch_update_tile<T, 32, 32, 16, 2, 2, SF, 0, false>(M, N, K, A, lda, B, ldb, C, ldc, s);
  else
    launch_update_tile<T, 16, 16, bk16, 1, 1, SF, 0, false>(M, N, K, A, lda, B, ldb, C, ldc, s);
}

template <typename T>
int gemm_ordered_dev(bool sum_first, int M, int N, int K, const T* A, int lda, const T* B, int ldb, T* C, int ldc,
                   cudaStream_t s) {
  if (M <= 0 || N <= 0 || K <= 0) return 0;
  prof_begin(sizeof(T) == 8 ? kProfGemmF64 : kProfGemmF32, s);
  if (sum_first) launch_update_by_size<T, true>(M, N, K, A, lda, B, ldb, C, ldc, s);
  else launch_update_by_size<T, false>(M, N, K, A, lda, B, ldb, C, ldc, s);
  prof_end(sizeof(T) == 8 ? kProfGemmF64 : kProfGemmF32, s, 2.0 * M * N * (double)K,
           sizeof(T) * ((double)M * K + (double)K * N + 2.0 * M * N));
  return (int)cudaGetLastError();
}
// DSYRK of the Cholesky's diagonal block in the reference orders, with the
// other operand transposed: lower ('L','N', dsyrk.f:313-320) C -= A*B on and
// below the diagonal, each product subtracted in turn, terms with a zero B
// element skipped; upper ('U','T', dsyrk.f:327-339) the products summed and
// the sum subtracted, on and above the diagonal.  8 x 8 tiles of 64 threads
// (one element each): the n x n block (n <= 64) with a K of up to the order
// of the matrix is spread over as many SMs as it has tiles in its triangle.
template <typename T>
int syrk_ordered_dev(bool upper, int n, int K, const T* A, int lda, const T* B, int ldb, T* C, int ldc, cudaStream_t s) {
  if (n <= 0 || K <= 0) return 0;
  if (upper) launch_update_tile<T, 8, 8, 128, 1, 1, true, 2, false>(n, n, K, A, lda, B, ldb, C, ldc, s);
  else launch_update_tile<T, 8, 8, 128, 1, 1, false, 1, true>(n, n, K, A, lda, B, ldb, C, ldc, s);
  return (int)cudaGetLastError();
}
template int syrk_ordered_dev<double>(bool, int, int, const double*, int, const double*, int, double*, int, cudaStream_t);
template int syrk_ordered_dev<float>(bool, int, int, const float*, int, const float*, int, float*, int, cudaStream_t);
template int gemm_ordered_dev<double>(bool, int, int, int, const double*, int, const double*, int, double*, int,
                                    cudaStream_t);
template int gemm_ordered_dev<float>(bool, int, int, int, const float*, int, const float*, int, float*, int,
                                   cudaStream_t);

// ------------------------------------------------------------------ panel
template <typename T>
struct PanelCtx {
  PanelScratch<T> ps;
  int* status;
  int max_optin;
  size_t words_bytes;    // candidate words + pair count, zeroed before each leaf
  int* perm = nullptr;    // optional running row permutation (gather index), updated with every leaf
  // Look-ahead: each leaf writes its pair list into the next slot of the
  // block column's log and applies it at once only to the columns
  // [imm_lo, imm_hi) (the block column); the rest is replayed later.
  bool logging = false;
  int imm_lo = 0, imm_hi = 0;
  int* log_dst = nullptr;
  int* log_src = nullptr;
  int* log_cnt = nullptr;   // [kMaxLogSlots], zeroed before the block column
  PairLogArgs log{};
  int* node_count = nullptr;   // arrival counter of the fused panel-node kernel (zero between launches)
};

template <typename T, bool EXACT>
static int launch_leaf(T* P, int lda, int M, int JB, int row0, int* ipiv, int* info, PanelCtx<T>& cx,
                       cudaStream_t s) {
  const int nsm = device_sm_count();
  // CTAs taking part in the panel: all SMs for FP64 (its FMA rate is low, the
  // rank-1 updates need every SM); fewer for FP32, where the per-column grid
  // barrier dominates and a smaller grid synchronises faster
  const Options& opt = options();
  int gmax = sizeof(T) == 8 ? opt.panel_ctas_f64 : opt.panel_ctas_f32;
  if (gmax <= 0 || gmax > nsm) gmax = nsm;
  int R = std::max(32, (M + gmax - 1) / gmax);
  int G = (M + R - 1) / R;
  size_t smem = (size_t)JB * R * sizeof(T) + (size_t)R * sizeof(int) + 16;
  auto kern = leaf_panel_kernel<T, EXACT>;
  static int dyn_cap_dev[64] = {0};
  int dev = 0;
  cudaGetDevice(&dev);
  if (!dyn_cap_dev[dev]) {
    cudaFuncAttributes fa;
    GB_CUDA_TRY(cudaFuncGetAttributes(&fa, (const void*)kern));
    const int cap = cx.max_optin - (int)fa.sharedSizeBytes;
    GB_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, cap));
    dyn_cap_dev[dev] = cap;
  }
  const int dyn_cap = dyn_cap_dev[dev];
  if ((long long)smem > dyn_cap) return 1000 + kStatusCapacity;   // panel taller than the GPU's shared memory holds
  int occ = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, kPanelThreads, smem);
  if (occ * nsm < G) return 1000 + kStatusCapacity;
  if (G > device_sm_count()) return 1000 + kStatusCapacity;   // scratch is sized for one CTA per SM
  GB_CUDA_TRY(cudaMemsetAsync(cx.ps.word, 0, cx.words_bytes, s));
  PanelScratch<T> ps = cx.ps;
  int* status = cx.status;
  void* args[] = {&P, &lda, &M, &JB, &R, &row0, &ipiv, &info, &ps, &status};
  prof_begin(kProfPanel, s);
  int rc = (int)cudaLaunchCooperativeKernel((void*)kern, G, kPanelThreads, args, smem, s);
  count_launch();
  // algorithmic work of the leaf: M x JB panel read and written once,
  // sum over columns of the rank-1 updates
  prof_end(kProfPanel, s, (double)M * JB * JB, 2.0 * sizeof(T) * (double)M * JB);
  return rc;
}

// A leaf's interchanges on the columns [lo, c0) and [c1, hi).
template <typename T>
static int laswp_pairs(T* A, int lda, int lo, int hi, int c0, int c1, int ntop, PanelCtx<T>& cx, cudaStream_t s,
                       int* perm) {
  T* Ab = A + (size_t)lo * lda;
  const int ncols = hi - lo;
  c0 -= lo;
  c1 -= lo;
  int warps = c0 + (ncols - c1) + (perm ? 1 : 0);
  if (warps <= 0) return 0;
  int blocks = (warps * 32 + 255) / 256;
  prof_begin(kProfLaswp, s);
  GB_LAUNCH(laswp_pairs_kernel<T><<<blocks, 256, 0, s>>>(Ab, lda, ncols, c0, c1, cx.ps.pair_dst, cx.ps.pair_src,
                                                cx.ps.pair_count, ntop, perm));
  prof_end(kProfLaswp, s, 0.0, 2.0 * sizeof(T) * 2.0 * ntop * warps);
  return (int)cudaGetLastError();
}

// A block column's logged interchanges on the columns [a0, a1) and [b0, b1).
template <typename T>
static int laswp_log(T* A, int lda, int a0, int a1, int b0, int b1, const PanelCtx<T>& cx, int* perm,
                     cudaStream_t s) {
  a1 = std::max(a0, a1);
  b1 = std::max(b0, b1);
  const int warps = (a1 - a0) + (b1 - b0) + (perm ? 1 : 0);
  if (warps <= 0 || cx.log.nslots == 0) return 0;
  int rows = 0;
  for (int q = 0; q < cx.log.nslots; ++q) rows += 2 * cx.log.ntop[q];
  prof_begin(kProfLaswp, s);
  GB_LAUNCH(laswp_log_kernel<T><<<(warps * 32 + 255) / 256, 256, 0, s>>>(A, lda, a0, a1, b0, b1, cx.log_dst,
                                                                        cx.log_src, cx.log_cnt, cx.log, perm));
  prof_end(kProfLaswp, s, 0.0, 2.0 * sizeof(T) * (double)rows * warps);
  return (int)cudaGetLastError();
}

// ---- cluster leaf (FP32): availability, width and launch

// Optional cycle counters of the push leaf's column steps (one buffer per
// device, null while off).
static bool g_leaf_phase_on = false;
static unsigned long long* g_leaf_phase[64] = {nullptr};
static unsigned long long* leaf_phase_buffer() {
  int dev = 0;
  if (!g_leaf_phase_on || cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return nullptr;
  if (!g_leaf_phase[dev]) {
    void* p = nullptr;
    if (cudaMalloc(&p, 8 * sizeof(unsigned long long)) != cudaSuccess) return nullptr;
    cudaMemset(p, 0, 8 * sizeof(unsigned long long));
    g_leaf_phase[dev] = static_cast<unsigned long long*>(p);
  }
  return g_leaf_phase[dev];
}
struct ClusterCaps {
  bool ok = false;
  int dyn_cap = 0;
};

template <bool EXACT, bool PUSH = false>
static ClusterCaps cluster_caps() {
  static ClusterCaps caps[64];
  static bool done[64] = {false};
  int dev = 0;
  cudaGetDevice(&dev);
  if (!done[dev]) {
    done[dev] = true;
    const void* kern = PUSH ? (const void*)leaf_panel_cluster_push_kernel<EXACT, 64>
                            : (const void*)leaf_panel_cluster_kernel<EXACT, 64>;
    cudaFuncAttributes fa;
    int optin = 0;
    if (cudaFuncGetAttributes(&fa, (const void*)kern) == cudaSuccess &&
        cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) == cudaSuccess) {
      const int cap = optin - (int)fa.sharedSizeBytes;
      if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, cap) == cudaSuccess &&
          cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) == cudaSuccess) {
        cudaLaunchConfig_t cfg = {};
        cudaLaunchAttribute at[1];
        at[0].id = cudaLaunchAttributeClusterDimension;
        at[0].val.clusterDim.x = kClusterCtas;
        at[0].val.clusterDim.y = 1;
        at[0].val.clusterDim.z = 1;
        cfg.gridDim = dim3(kClusterCtas);
        cfg.blockDim = dim3(kClusterThreads);
        cfg.dynamicSmemBytes = cap;
        cfg.attrs = at;
        cfg.numAttrs = 1;
        int nclusters = 0;
        if (cudaOccupancyMaxActiveClusters(&nclusters, kern, &cfg) == cudaSuccess && nclusters >= 1) {
          caps[dev].ok = true;
          caps[dev].dyn_cap = cap;
        }
      }
    }
    cudaGetLastError();   // clear any error from an unsupported query
  }
  return caps[dev];
}

// Leaf plan of the FP32 cluster path for an M-row panel: the register
// kernel (kind 1) with 32-column leaves up to M = 16384 and 16-column leaves
// up to M = 32768 (64 row values per thread), else the shared-memory cluster
// kernel (kind 2) with the widest leaf of 64, 32, 24, 16 or 8 columns that
// fits; 0 when neither applies.  Returns the leaf width.
template <typename T>
static int cluster_leaf_width(int M, int* kind) {
  *kind = 0;
  if (sizeof(T) != 4 || options().cluster_panel == 0) return 0;
  const bool push = options().cluster_panel == 3;
  ClusterCaps c = options().exact ? (push ? cluster_caps<true, true>() : cluster_caps<true>())
                                  : (push ? cluster_caps<false, true>() : cluster_caps<false>());
  if (!c.ok) return 0;
  long long R = (M + kClusterCtas - 1) / kClusterCtas;
  if (options().cluster_panel >= 2) R = leaf_push_rows((int)R);
  if (options().cluster_panel == 1) {
    if (R <= 2 * kClusterThreads) { *kind = 1; return 32; }
    if (R <= 4 * kClusterThreads) { *kind = 1; return 16; }
  }
  // 64, 32, 24, 16 or 8 columns (widths between 32 and 64 would split a
  // 64-column block into unequal leaves)
  for (int lw : {64, 32, 24, 16, 8})
    if ((long long)(lw + 1) * R * 4 + 16 <= c.dyn_cap) { *kind = 2; return lw; }
  return 0;
}

template <bool EXACT, int JB>
static int launch_leaf_cluster_reg(float* P, int lda, int M, int jb, int row0, int* ipiv, int* info,
                                   PanelCtx<float>& cx, cudaStream_t s) {
  static bool attr[64] = {false};
  int dev = 0;
  cudaGetDevice(&dev);
  if (!attr[dev]) {
    GB_CUDA_TRY(cudaFuncSetAttribute(leaf_panel_cluster_reg_kernel<EXACT, JB>,
                                     cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
    attr[dev] = true;
  }
  const int R = (M + kClusterCtas - 1) / kClusterCtas;
  if (R > (64 / JB) * kClusterThreads || jb > JB) return 1000 + kStatusCapacity;
  // with the interchange log the pair count is this leaf's slot of the
  // block column's counters, zeroed with them before the block column
  if (!cx.logging) GB_CUDA_TRY(cudaMemsetAsync(cx.ps.pair_count, 0, sizeof(int), s));
  cudaLaunchConfig_t cfg = {};
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = kClusterCtas;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.gridDim = dim3(kClusterCtas);
  cfg.blockDim = dim3(kClusterThreads);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = s;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  prof_begin(kProfPanel, s);
  int rc = (int)cudaLaunchKernelEx(&cfg, leaf_panel_cluster_reg_kernel<EXACT, JB>, P, lda, M, jb, R, row0, ipiv, info,
                                   cx.ps.pair_dst, cx.ps.pair_src, cx.ps.pair_count, cx.status);
  count_launch();
  prof_end(kProfPanel, s, (double)M * jb * jb, 2.0 * 4.0 * (double)M * jb);
  return rc;
}

template <bool EXACT, int JBT, bool PUSH>
static int launch_leaf_cluster_w(float* P, int lda, int M, int JB, int R, size_t smem, int row0, int* ipiv, int* info,
                                 PanelCtx<float>& cx, cudaStream_t s, int dyn_cap) {
  static bool attr[64] = {false};
  int dev = 0;
  cudaGetDevice(&dev);
  const void* kern = PUSH ? (const void*)leaf_panel_cluster_push_kernel<EXACT, JBT>
                          : (const void*)leaf_panel_cluster_kernel<EXACT, JBT>;
  if (!attr[dev]) {
    GB_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, dyn_cap));
    GB_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
    attr[dev] = true;
  }
  cudaLaunchConfig_t cfg = {};
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = kClusterCtas;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.gridDim = dim3(kClusterCtas);
  cfg.blockDim = dim3(kClusterThreads);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  // with the interchange log, the leaf also applies its interchanges to the
  // rest of its block column
  int a0 = 0, a1 = 0, b0 = 0, b1 = 0;
  if (cx.logging) {
    a0 = cx.imm_lo;
    a1 = row0;
    b0 = row0 + JB;
    b1 = cx.imm_hi;
  }
  if constexpr (PUSH)
    return (int)cudaLaunchKernelEx(&cfg, leaf_panel_cluster_push_kernel<EXACT, JBT>, P, lda, M, JB, R, row0, ipiv,
                                   info, cx.ps.pair_dst, cx.ps.pair_src, cx.ps.pair_count, cx.status, a0, a1, b0, b1,
                                   leaf_phase_buffer());
  else
    return (int)cudaLaunchKernelEx(&cfg, leaf_panel_cluster_kernel<EXACT, JBT>, P, lda, M, JB, R, row0, ipiv, info,
                                   cx.ps.pair_dst, cx.ps.pair_src, cx.ps.pair_count, cx.status, a0, a1, b0, b1);
}

template <bool EXACT, bool PUSH>
static int launch_leaf_cluster_p(float* P, int lda, int M, int JB, int row0, int* ipiv, int* info,
                                 PanelCtx<float>& cx, cudaStream_t s) {
  ClusterCaps c = cluster_caps<EXACT, PUSH>();
  const int R = (M + kClusterCtas - 1) / kClusterCtas;
  const int Rs = leaf_push_rows(R);      // both shared-memory leaves pad their rows
  size_t smem = (size_t)JB * Rs * 4 + (size_t)Rs * 4 + 16;
  if (!c.ok || (long long)smem > c.dyn_cap || JB > 64) return 1000 + kStatusCapacity;
  // with the interchange log the pair count is this leaf's slot of the
  // block column's counters, zeroed with them before the block column
  if (!cx.logging) GB_CUDA_TRY(cudaMemsetAsync(cx.ps.pair_count, 0, sizeof(int), s));
  prof_begin(kProfPanel, s);
  int rc;
  if (JB <= 8) rc = launch_leaf_cluster_w<EXACT, 8, PUSH>(P, lda, M, JB, R, smem, row0, ipiv, info, cx, s, c.dyn_cap);
  else if (JB <= 16)
    rc = launch_leaf_cluster_w<EXACT, 16, PUSH>(P, lda, M, JB, R, smem, row0, ipiv, info, cx, s, c.dyn_cap);
  else if (JB <= 32)
    rc = launch_leaf_cluster_w<EXACT, 32, PUSH>(P, lda, M, JB, R, smem, row0, ipiv, info, cx, s, c.dyn_cap);
  else rc = launch_leaf_cluster_w<EXACT, 64, PUSH>(P, lda, M, JB, R, smem, row0, ipiv, info, cx, s, c.dyn_cap);
  count_launch();
  prof_end(kProfPanel, s, (double)M * JB * JB, 2.0 * 4.0 * (double)M * JB);
  return rc;
}

// The shared-memory cluster leaf: the push exchange (option cluster_panel
// 3) or the cluster-barrier exchange (2).
template <bool EXACT>
static int launch_leaf_cluster(float* P, int lda, int M, int JB, int row0, int* ipiv, int* info,
                               PanelCtx<float>& cx, cudaStream_t s) {
  if (options().cluster_panel == 3) return launch_leaf_cluster_p<EXACT, true>(P, lda, M, JB, row0, ipiv, info, cx, s);
  return launch_leaf_cluster_p<EXACT, false>(P, lda, M, JB, row0, ipiv, info, cx, s);
}

// Left width of a recursion split of w > leaf columns: halves above 64
// columns (the internal updates stay <= 64 wide or a multiple of 64 deep),
// whole leaves, about half on the left, within 64 columns (e.g. 24 + 24 + 16
// instead of four leaves of 16).
static inline int split_cols(int w, int leaf) {
  int n1;
  if (w > 64) {
    n1 = (w / 2 + 7) / 8 * 8;
  } else {
    const int nleaf = (w + leaf - 1) / leaf;
    n1 = leaf * ((nleaf + 1) / 2);
  }
  if (n1 >= w || n1 <= 0) n1 = w / 2;
  return n1;
}

// DGETRF2-shaped recursion on the panel of columns [c0, c0+w), rows [c0, m).
// Each leaf applies its interchanges to every other column of the matrix
// (left: the DLASWP of SRC/dgetrf.f:193, right: SRC/dgetrf2.f:236 and
// SRC/dgetrf.f:199), so the recursion never re-applies them.
template <typename T>
static int getrf_rec(T* A, int lda, int m, int n, int c0, int w, int* ipiv, int* info, PanelCtx<T>& cx,
                     cudaStream_t s, int gemm_mode) {
  int ckind = 0;
  const int clw = cluster_leaf_width<T>(m - c0, &ckind);
  const int leaf = clw ? clw : kLeafMax;
  if (w <= leaf) {
    T* P = A + c0 + (size_t)c0 * lda;
    int rc;
    if (cx.logging) {
      const int sl = cx.log.nslots;
      if (sl >= kMaxLogSlots) return 1000 + kStatusCapacity;
      cx.ps.pair_dst = cx.log_dst + (size_t)sl * 2 * kLeafMax;
      cx.ps.pair_src = cx.log_src + (size_t)sl * 2 * kLeafMax;
      cx.ps.pair_count = cx.log_cnt + sl;
      cx.log.ntop[sl] = w;
      cx.log.nslots = sl + 1;
    }
    if constexpr (sizeof(T) == 4) {
      const bool ex = options().exact;
      if (ckind == 1 && clw == 32)
        rc = ex ? launch_leaf_cluster_reg<true, 32>(P, lda, m - c0, w, c0, ipiv + c0, info, cx, s)
                : launch_leaf_cluster_reg<false, 32>(P, lda, m - c0, w, c0, ipiv + c0, info, cx, s);
      else if (ckind == 1)
        rc = ex ? launch_leaf_cluster_reg<true, 16>(P, lda, m - c0, w, c0, ipiv + c0, info, cx, s)
                : launch_leaf_cluster_reg<false, 16>(P, lda, m - c0, w, c0, ipiv + c0, info, cx, s);
      else if (ckind == 2)
        rc = ex ? launch_leaf_cluster<true>(P, lda, m - c0, w, c0, ipiv + c0, info, cx, s)
                : launch_leaf_cluster<false>(P, lda, m - c0, w, c0, ipiv + c0, info, cx, s);
      else
        rc = options().exact ? launch_leaf<T, true>(P, lda, m - c0, w, c0, ipiv + c0, info, cx, s)
                             : launch_leaf<T, false>(P, lda, m - c0, w, c0, ipiv + c0, info, cx, s);
    } else {
      rc = options().exact ? launch_leaf<T, true>(P, lda, m - c0, w, c0, ipiv + c0, info, cx, s)
                           : launch_leaf<T, false>(P, lda, m - c0, w, c0, ipiv + c0, info, cx, s);
    }
    if (rc) return rc;
    if (cx.logging && sizeof(T) == 4 && ckind == 2) return 0;   // applied inside the cluster leaf
    if (cx.logging) return laswp_pairs<T>(A, lda, cx.imm_lo, cx.imm_hi, c0, c0 + w, w, cx, s, nullptr);
    return laswp_pairs<T>(A, lda, 0, n, c0, c0 + w, w, cx, s, cx.perm);
  }
  const int n1 = split_cols(w, leaf);
  int rc = getrf_rec<T>(A, lda, m, n, c0, n1, ipiv, info, cx, s, gemm_mode);
  if (rc) return rc;
  T* A11 = A + c0 + (size_t)c0 * lda;
  // narrow updates inside the panel (64 columns or fewer) run on the FP32
  // FMA kernel: one launch, no operand split, K <= 64 would be padded to a
  // full BF16 K block anyway
  const int gm = (gemm_mode == kMixedBf16x3 && w - n1 <= 64) ? kMixedFp32 : gemm_mode;
  if (options().panel_fuse && n1 <= 64 && w - n1 <= 64 && (sizeof(T) == 8 || gm == kMixedFp32)) {
    // the solve and the narrow update of this node in one launch (same arithmetic)
    rc = panel_node_dev<T>(A11, lda, m - c0, n1, w - n1, cx.node_count, s);
  } else {
    rc = trsm_llnu_dev<T>(n1, w - n1, A11, lda, A11 + (size_t)n1 * lda, lda, s, gm, false);
    if (rc) return rc;
    rc = gemm_update_dev<T>(m - c0 - n1, w - n1, n1, A11 + n1, lda, A11 + (size_t)n1 * lda, lda,
                            A11 + n1 + (size_t)n1 * lda, lda, s, gm);
  }
  if (rc) return rc;
  return getrf_rec<T>(A, lda, m, n, c0 + n1, w - n1, ipiv, info, cx, s, gemm_mode);
}

// Leaves the recursion of getrf_rec makes for the block column [c0, c0+w).
template <typename T>
static int count_leaves(int m, int c0, int w) {
  int ckind = 0;
  const int clw = cluster_leaf_width<T>(m - c0, &ckind);
  const int leaf = clw ? clw : kLeafMax;
  if (w <= leaf) return 1;
  const int n1 = split_cols(w, leaf);
  return count_leaves<T>(m, c0, n1) + count_leaves<T>(m, c0 + n1, w - n1);
}

// Per-device second stream (highest priority) and events of the look-ahead
// schedule.  The mutex is held while one factorization queues its work.
struct LookaheadRes {
  std::mutex mu;
  bool ok = false, tried = false;
  cudaStream_t sp = nullptr;
  cudaEvent_t fork = nullptr, P[2] = {nullptr, nullptr}, L[2] = {nullptr, nullptr};
};

static LookaheadRes* lookahead_res() {
  static LookaheadRes res[64];
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return nullptr;
  LookaheadRes& r = res[dev];
  std::lock_guard<std::mutex> lk(r.mu);
  if (!r.tried) {
    r.tried = true;
    int lo = 0, hi = 0;
    bool ok = cudaDeviceGetStreamPriorityRange(&lo, &hi) == cudaSuccess &&
              cudaStreamCreateWithPriority(&r.sp, cudaStreamNonBlocking, hi) == cudaSuccess;
    const unsigned fl = cudaEventDisableTiming;
    ok = ok && cudaEventCreateWithFlags(&r.fork, fl) == cudaSuccess;
    for (int i = 0; i < 2 && ok; ++i)
      ok = cudaEventCreateWithFlags(&r.P[i], fl) == cudaSuccess && cudaEventCreateWithFlags(&r.L[i], fl) == cudaSuccess;
    r.ok = ok;
    cudaGetLastError();
  }
  return r.ok ? &r : nullptr;
}

// U12 = L11^{-1} A12 for the columns [c_beg, c_end) of the block row of
// block column j (SRC/dgetrf.f:204).  With linv (the BF16x3 mode, the
// inverse of L11 formed once per block column by form_linv) as one BF16x3
// product, else by substitution.  Both schedules (look-ahead or not) use
// the same method for every column, so they compute the same.
template <typename T>
static int block_row_u(T* dA, int lda, int j, int jb, int c_beg, int c_end, const T* linv, cudaStream_t s,
                       int gemm_mode) {
  if (c_end <= c_beg) return 0;
  T* Ajj = dA + j + (size_t)j * lda;
  T* U = dA + j + (size_t)c_beg * lda;
  if constexpr (sizeof(T) == 4) {
    if (linv) return gemm_bf16x3_dev(jb, c_end - c_beg, jb, linv, jb, U, lda, U, lda, s, true);
  }
  return trsm_llnu_dev<T>(jb, c_end - c_beg, Ajj, lda, U, lda, s, gemm_mode);
}

// The U rows of the block column next to j (the look-ahead's critical
// path: the next panel waits for them).  In the BF16x3 mode they come from
// FP32 substitution in the one-launch 128-row solves (no L11^{-1} to form
// first: the inverse, which the wider rest of the block row uses, is formed
// after the next panel has been released); otherwise as block_row_u.  Both
// schedules (look-ahead or not) use this for the next block column and
// block_row_u for the rest, so they compute the same.
template <typename T>
static int next_block_row_u(T* dA, int lda, int j, int jb, int c_beg, int c_end, bool linv_mode, cudaStream_t s,
                            int gemm_mode) {
  if (c_end <= c_beg) return 0;
  if (!linv_mode) return block_row_u<T>(dA, lda, j, jb, c_beg, c_end, nullptr, s, gemm_mode);
  T* Ajj = dA + j + (size_t)j * lda;
  return trsm_llnu_dev<T>(jb, c_end - c_beg, Ajj, lda, dA + j + (size_t)c_beg * lda, lda, s, kMixedFp32, false);
}

template <typename T>
static int form_linv(T* dA, int lda, int j, int jb, T* linv, cudaStream_t s) {
  if constexpr (sizeof(T) == 4) {
    if (linv) return unit_lower_inverse_dev<T>(jb, dA + j + (size_t)j * lda, lda, linv, jb, s);
  }
  return 0;
}

static __global__ void iota_kernel(int* p, int n) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) p[i] = i;
}

// Host events marking the end of each look-ahead step while columns are
// fed in: the host keeps at most two steps ahead of the device, so that
// the chunks it finds arrived are taken in as early as the device can use
// them (a chunk taken in late is first brought up to date column block by
// column block).
struct StepEvents {
  cudaEvent_t e[4] = {nullptr, nullptr, nullptr, nullptr};
  bool ok = true;
  StepEvents() {
    for (auto& x : e) ok = ok && cudaEventCreateWithFlags(&x, cudaEventDisableTiming) == cudaSuccess;
  }
  ~StepEvents() {
    for (auto& x : e)
      if (x) cudaEventDestroy(x);
  }
};

// Optional timeline of the fed factorization (gb300_feed_trace): timing
// events on the factorization's stream at each step's end (kind 0) and
// after each chunk is taken in and brought up to date (kind 1, with the
// step it joined at), read back as milliseconds after the first.
struct FeedTrace {
  bool on = false;
  std::vector<cudaEvent_t> ev;
  std::vector<int> kind, idx, aux;
  void add(int k, int i, int a, cudaStream_t s) {
    cudaEvent_t e = nullptr;
    if (cudaEventCreate(&e) != cudaSuccess) return;
    cudaEventRecord(e, s);
    ev.push_back(e);
    kind.push_back(k);
    idx.push_back(i);
    aux.push_back(a);
  }
  void clear() {
    for (auto e : ev) cudaEventDestroy(e);
    ev.clear();
    kind.clear();
    idx.clear();
    aux.clear();
  }
};
static FeedTrace g_feed_trace;

void feed_trace_mark(int kind, int idx, int aux, cudaStream_t s) {
  if (g_feed_trace.on) g_feed_trace.add(kind, idx, aux, s);
}

template <typename T>
int getrf_dev(int m, int n, T* dA, int lda, int* dIpiv, int* dInfo, cudaStream_t s, int gemm_mode, int nb,
              int* dPerm, const ColumnFeed* feed) {
  GB_CUDA_TRY(cudaMemsetAsync(dInfo, 0, sizeof(int), s));
  if (m <= 0 || n <= 0) return 0;
  if (feed && (!dPerm || sizeof(T) != 4 || feed->nchunks < 1 || feed->cols[0] != 0 ||
               feed->cols[feed->nchunks] != n))
    return (int)cudaErrorInvalidValue;
  if (dPerm) GB_LAUNCH(iota_kernel<<<(m + 255) / 256, 256, 0, s>>>(dPerm, m));
  const int nsm = device_sm_count();
  int dev = 0;
  cudaGetDevice(&dev);
  int optin = 0;
  cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  const int G = nsm;
  size_t bytes = 0;
  auto carve = [&](size_t b) { size_t off = bytes; bytes += (b + 255) / 256 * 256; return off; };
  size_t o_word = carve(sizeof(unsigned long long) * 2 * G + sizeof(int));   // words, then the pair count
  size_t o_abs = carve(sizeof(T) * 2 * G);
  size_t o_clab = carve(sizeof(int) * 2 * G);
  size_t o_crow = carve(sizeof(T) * 2 * G * kLeafMax);
  size_t o_rowk = carve(sizeof(T) * 2 * kLeafMax);
  size_t o_rkl = carve(sizeof(int) * 2);
  size_t o_pd = carve(sizeof(int) * 2 * kLeafMax);
  size_t o_psrc = carve(sizeof(int) * 2 * kLeafMax);
  // look-ahead: two block-column logs (pair lists of up to kMaxLogSlots leaves)
  const size_t log_ints = (size_t)kMaxLogSlots * 2 * kLeafMax;
  size_t o_log = carve(sizeof(int) * 4 * log_ints);
  size_t o_lcnt = carve(sizeof(int) * 2 * kMaxLogSlots);
  const int nb_inv = std::min(std::max(nb, 1), 512);   // L11^{-1} up to 512 x 512 (BF16x3 mode)
  size_t o_linv = carve(sizeof(T) * (size_t)nb_inv * nb_inv);
  size_t o_node = carve(sizeof(int));
  DevScratch ws(bytes, s);
  if (!ws.p) return (int)cudaErrorMemoryAllocation;
  char* base = ws.as<char>();
  PanelCtx<T> cx;
  cx.ps.word = reinterpret_cast<unsigned long long*>(base + o_word);
  cx.ps.pair_count = reinterpret_cast<int*>(base + o_word + sizeof(unsigned long long) * 2 * G);
  cx.ps.absval = reinterpret_cast<T*>(base + o_abs);
  cx.ps.cand_label = reinterpret_cast<int*>(base + o_clab);
  cx.ps.cand_row = reinterpret_cast<T*>(base + o_crow);
  cx.ps.row_k = reinterpret_cast<T*>(base + o_rowk);
  cx.ps.row_k_label = reinterpret_cast<int*>(base + o_rkl);
  cx.ps.pair_dst = reinterpret_cast<int*>(base + o_pd);
  cx.ps.pair_src = reinterpret_cast<int*>(base + o_psrc);
  cx.words_bytes = sizeof(unsigned long long) * 2 * G + sizeof(int);
  cx.perm = dPerm;
  cx.status = device_status_word();
  cx.max_optin = optin;
  if (!cx.status) return (int)cudaErrorMemoryAllocation;
  cx.node_count = reinterpret_cast<int*>(base + o_node);
  GB_CUDA_TRY(cudaMemsetAsync(cx.node_count, 0, sizeof(int), s));

  const int mn = std::min(m, n);
  if (nb < 1) nb = 1;

  // Look-ahead schedule (FP32 cluster leaves, two or more block columns):
  // block column k is factored on the second stream sp while the user
  // stream s finishes the trailing update of block column k-1; s then
  // applies column k's interchanges, forms U and updates the next block
  // column first (event L), so that sp can start on it, and the rest of
  // the trailing matrix after.  The work per element and its order are
  // those of the one-stream loop below.
  bool la = sizeof(T) == 4 && options().lookahead != 0 && mn > nb;
  if (la) {
    int ck = 0;
    la = cluster_leaf_width<T>(m, &ck) != 0;
    for (int j = 0; la && j < mn; j += nb)
      la = count_leaves<T>(m, j, std::min(nb, mn - j)) <= kMaxLogSlots;
  }
  // inverse of the block column's unit lower triangle (BF16x3 mode only:
  // the exact and FP32 modes keep the substitution of SRC/dgetrf.f:204)
  T* linv = (sizeof(T) == 4 && gemm_mode == kMixedBf16x3 && !options().exact && nb <= 512)
                ? reinterpret_cast<T*>(base + o_linv)
                : nullptr;
  LookaheadRes* lr = la ? lookahead_res() : nullptr;
  // Fed columns: [0, win) are in the matrix and current; chunk nq is next.
  // Chunks taken in together form the pending slab [win, pend_end): their
  // rows are reordered at once by the interchanges made so far (the gather
  // in admit), every later step's interchanges reach them with the rest of
  // the matrix, and block column by block column, in order, they get the U
  // rows and trailing updates of the block columns already factored -- a
  // few block columns per step, so the catch-up runs beside the panels
  // instead of holding them up -- until they are current and join the
  // window.  Per element these are the operations of the right-looking
  // loop in its order (an interchange of a later block column moves whole
  // rows of L and of the slab alike), so the result does not depend on
  // when a chunk arrived.
  int win = feed ? 0 : n, nq = 0;
  int pend_end = win, pend_k = 0;   // pending slab, brought up to date through block column pend_k - 1
  // fed columns with the look-ahead: every block column's L11^{-1}, for the catch-up
  DevScratch linv_keep((feed && lr && linv) ? sizeof(T) * (size_t)((mn + nb - 1) / nb) * nb * nb : 0, s);
  T* linv_hist = linv_keep.as<T>();
  if (feed && lr && linv && !linv_hist) return (int)cudaErrorMemoryAllocation;
  // chunks [nq, qend) become the pending slab (none pending), after the
  // interchanges of block columns 0..kdone-1
  auto take_in = [&](int qend, int kdone) -> int {
    if (qend <= nq || pend_end > win) return 0;
    for (int q = nq; q < qend; ++q) {
      GB_CUDA_TRY(cudaStreamWaitEvent(s, feed->ready[q], 0));
      const int rc = feed->admit(q, kdone > 0 ? dPerm : nullptr, s);
      if (rc) return rc;
      if (feed->rejected(q)) return kFeedStop;
    }
    pend_end = feed->cols[qend];
    pend_k = 0;
    nq = qend;
    return 0;
  };
  // block columns pend_k..kto-1 on the pending slab; it joins the window once current at step k_now
  auto catch_up = [&](int kto, int k_now) -> int {
    if (pend_end <= win) return 0;
    const int c0 = win, c1 = pend_end;
    for (int kk = pend_k, jj = pend_k * nb; kk < kto; ++kk, jj += nb) {
      const int jjb = std::min(nb, std::min(m, n) - jj), jj2 = jj + jjb;
      const T* lv = linv_hist ? linv_hist + (size_t)kk * nb * nb : nullptr;
      T* Ajj = dA + jj + (size_t)jj * lda;
      int rc = block_row_u<T>(dA, lda, jj, jjb, c0, c1, lv, s, gemm_mode);
      if (!rc && jj2 < m)
        rc = gemm_update_dev<T>(m - jj2, c1 - c0, jjb, Ajj + jjb, lda, dA + jj + (size_t)c0 * lda, lda,
                                dA + jj2 + (size_t)c0 * lda, lda, s, gemm_mode);
      if (rc) return rc;
    }
    pend_k = std::max(pend_k, kto);
    if (pend_k >= k_now) {
      if (g_feed_trace.on)
        for (int q = 0; q < feed->nchunks; ++q)
          if (feed->cols[q] >= c0 && feed->cols[q] < c1) g_feed_trace.add(1, q, k_now, s);
      win = pend_end;
    }
    return 0;
  };
  // the first chunk index whose columns reach `col`
  auto chunk_reaching = [&](int col) {
    int q = nq;
    while (q < feed->nchunks && feed->cols[q] < col) ++q;
    return q;
  };
  // chunks landed so far, from nq on
  auto chunks_landed = [&]() {
    int q = nq;
    while (q < feed->nchunks && cudaEventQuery(feed->ready[q]) == cudaSuccess) ++q;
    cudaGetLastError();   // (a not-ready query leaves no error behind)
    return q;
  };
  // everything the step after the next needs, and (eagerly) whatever landed
  auto take_in_now = [&](int need, int k_now) -> int {
    int rc = 0;
    if (win < need) {
      rc = catch_up(k_now, k_now);
      if (!rc && win < need) {
        int qend = chunk_reaching(need);
        if (options().feed_lazy == 0) qend = std::max(qend, chunks_landed());
        rc = take_in(qend, k_now);
        if (!rc) rc = catch_up(k_now, k_now);
      }
    }
    return rc;
  };
  if (feed && !lr) {
    // no look-ahead schedule: take every chunk in before the factorization
    const int rc = take_in_now(n, 0);
    if (rc) return rc;
  }
  if (lr) {
    std::lock_guard<std::mutex> lk(lr->mu);
    cudaStream_t sp = lr->sp;
    int* logs = reinterpret_cast<int*>(base + o_log);
    int* lcnt = reinterpret_cast<int*>(base + o_lcnt);
    // room for the BF16 hi/lo split of the largest A21 (m rows, nb columns)
    const bool split_a21 = sizeof(T) == 4 && gemm_mode == kMixedBf16x3;
    DevScratch a21buf(split_a21 ? bf16x3_split_bytes(m, nb) : 0, s);
    if (split_a21 && !a21buf.p) return (int)cudaErrorMemoryAllocation;
    StepEvents steps;
    if (feed) {
      if (!steps.ok) return (int)cudaErrorMemoryAllocation;
      // the first two block columns before anything starts
      const int rc = take_in_now(std::min(n, 2 * nb), 0);
      if (rc) return rc;
    }
    GB_CUDA_TRY(cudaEventRecord(lr->fork, s));
    GB_CUDA_TRY(cudaStreamWaitEvent(sp, lr->fork, 0));
    int k = 0;
    for (int j = 0; j < mn; j += nb, ++k) {
      const int jb = std::min(nb, mn - j);
      const int b = k & 1;
      if (feed && k >= 2) GB_CUDA_TRY(cudaEventSynchronize(steps.e[(k - 2) & 3]));
      if (k > 0) GB_CUDA_TRY(cudaStreamWaitEvent(sp, lr->L[b ^ 1], 0));
      cx.logging = true;
      cx.imm_lo = j;
      cx.imm_hi = j + jb;
      cx.log_dst = logs + (size_t)(2 * b) * log_ints;
      cx.log_src = logs + (size_t)(2 * b + 1) * log_ints;
      cx.log_cnt = lcnt + b * kMaxLogSlots;
      cx.log.nslots = 0;
      GB_CUDA_TRY(cudaMemsetAsync(cx.log_cnt, 0, sizeof(int) * kMaxLogSlots, sp));
      if (g_feed_trace.on) g_feed_trace.add(6, k, 0, sp);   // panel k starts
      int rc = getrf_rec<T>(dA, lda, m, n, j, jb, dIpiv, dInfo, cx, sp, gemm_mode);
      if (rc) return rc;
      if (g_feed_trace.on) g_feed_trace.add(7, k, 0, sp);   // panel k done
      GB_CUDA_TRY(cudaEventRecord(lr->P[b], sp));
      GB_CUDA_TRY(cudaStreamWaitEvent(s, lr->P[b], 0));
      const int j2 = j + jb;
      const int nb2 = j2 < mn ? std::min(nb, mn - j2) : 0;   // next block column
      T* Ajj = dA + j + (size_t)j * lda;
      T* lv = linv_hist ? linv_hist + (size_t)k * nb * nb : linv;
      // the BF16 split of A21, made once for both updates of this block column
      // (stream s orders it after the previous column's updates that read the buffer)
      const bool presplit = a21buf.p && j2 < m;
      Bf16SplitA a21;
      if (presplit) {
        if constexpr (sizeof(T) == 4) rc = bf16x3_split_a_dev(m - j2, jb, Ajj + jb, lda, a21buf.p, &a21, s);
        if (rc) return rc;
      }
      auto update = [&](int ncols, int coff) -> int {
        if constexpr (sizeof(T) == 4) {
          if (presplit)
            return gemm_bf16x3_dev(m - j2, ncols, jb, Ajj + jb, lda, Ajj + (size_t)coff * lda, lda,
                                   Ajj + jb + (size_t)coff * lda, lda, s, false, &a21);
        }
        return gemm_update_dev<T>(m - j2, ncols, jb, Ajj + jb, lda, Ajj + (size_t)coff * lda, lda,
                                  Ajj + jb + (size_t)coff * lda, lda, s, gemm_mode);
      };
      // next block column first
      if (nb2 > 0) {
        rc = laswp_log<T>(dA, lda, j2, j2 + nb2, 0, 0, cx, nullptr, s);
        if (!rc) rc = next_block_row_u<T>(dA, lda, j, jb, j2, j2 + nb2, lv != nullptr, s, gemm_mode);
        if (!rc && j2 < m) rc = update(nb2, jb);
        if (rc) return rc;
      }
      GB_CUDA_TRY(cudaEventRecord(lr->L[b], s));
      if (g_feed_trace.on) g_feed_trace.add(5, k, 0, s);    // next block column ready for panel k+1
      // L11^{-1} for the rest of the block row, off the next panel's path
      rc = form_linv<T>(dA, lda, j, jb, lv, s);
      if (rc) return rc;
      const int c2 = j2 + nb2;
      if (feed) {
        // the columns the next step needs (the block column after the next
        // one), current before this block column's interchanges reach them;
        // then landed chunks, a few block columns of catch-up per step
        rc = take_in_now(std::min(n, c2 + nb), k);
        if (!rc && options().feed_lazy != 1) {
          // feed_lazy 2 (a test setting) takes the next chunk in every step, landed or not
          if (pend_end <= win)
            rc = take_in(options().feed_lazy == 2 ? std::min(feed->nchunks, nq + 1) : chunks_landed(), k);
          const int budget = options().feed_catchup;   // block columns per step, 0: all at once
          if (!rc) rc = catch_up(budget > 0 ? std::min(k, pend_k + budget) : k, k);
        }
        if (rc) return rc;
      }
      // then the columns left of the block column and the rest of the
      // trailing matrix (the pending slab takes the interchanges too)
      rc = laswp_log<T>(dA, lda, 0, j, c2, std::max(win, pend_end), cx, cx.perm, s);
      if (!rc && c2 < win) {
        rc = block_row_u<T>(dA, lda, j, jb, c2, win, lv, s, gemm_mode);
        if (!rc && j2 < m) rc = update(win - c2, c2 - j);
      }
      if (rc) return rc;
      if (feed) GB_CUDA_TRY(cudaEventRecord(steps.e[k & 3], s));
      if (g_feed_trace.on) g_feed_trace.add(0, k, win, s);
    }
    // columns right of min(m, n) still outside (wide matrices)
    if (feed) {
      const int rc = take_in_now(n, k);
      if (rc) return rc;
    }
    return (int)cudaGetLastError();
  }

  for (int j = 0; j < mn; j += nb) {
    const int jb = std::min(nb, mn - j);
    int rc = getrf_rec<T>(dA, lda, m, n, j, jb, dIpiv, dInfo, cx, s, gemm_mode);
    if (rc) return rc;
    if (j + jb < n) {
      T* Ajj = dA + j + (size_t)j * lda;
      const int j2 = j + jb;
      const int c2 = j2 + (j2 < mn ? std::min(nb, mn - j2) : 0);   // next block column, then the rest
      rc = form_linv<T>(dA, lda, j, jb, linv, s);
      if (!rc) rc = next_block_row_u<T>(dA, lda, j, jb, j2, std::min(c2, n), linv != nullptr, s, gemm_mode);
      if (!rc) rc = block_row_u<T>(dA, lda, j, jb, c2, n, linv, s, gemm_mode);
      if (rc) return rc;
      if (j + jb < m) {
        rc = gemm_update_dev<T>(m - j - jb, n - j - jb, jb, Ajj + jb, lda, Ajj + (size_t)jb * lda, lda,
                                Ajj + jb + (size_t)jb * lda, lda, s, gemm_mode);
        if (rc) return rc;
      }
    }
  }
  return (int)cudaGetLastError();
}
template int getrf_dev<double>(int, int, double*, int, int*, int*, cudaStream_t, int, int, int*, const ColumnFeed*);
template int getrf_dev<float>(int, int, float*, int, int*, int*, cudaStream_t, int, int, int*, const ColumnFeed*);

// ------------------------------------------------------------- permutation
int ipiv_perm_dev(const int* dIpiv, int k1, int k2, int incx, int lo, int span, int* dPerm, cudaStream_t s) {
  if (span <= 0) return 0;
  int* status = device_status_word();
  if (!status) return (int)cudaErrorMemoryAllocation;
  int dev = 0, optin = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  size_t smem = (size_t)span * sizeof(int);
  if ((long long)smem <= optin - 1024) {
    static bool attr[64] = {false};
    if (!attr[dev]) {
      cudaFuncSetAttribute(ipiv_to_perm_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin - 1024);
      attr[dev] = true;
    }
    GB_LAUNCH(ipiv_to_perm_kernel<true><<<1, 1024, smem, s>>>(dIpiv, k1, k2, incx, lo, span, dPerm, nullptr, status));
  } else {
    DevScratch lab(smem, s);
    if (!lab.p) return (int)cudaErrorMemoryAllocation;
    GB_LAUNCH(ipiv_to_perm_kernel<false><<<1, 1024, 0, s>>>(dIpiv, k1, k2, incx, lo, span, dPerm, lab.as<int>(), status));
  }
  return (int)cudaGetLastError();
}

// ------------------------------------------------------------------- DLASWP
// General DLASWP (SRC/dlaswp.f) on device memory.  The caller names the row
// window [lo, lo+span) that holds rows K1..K2 and every IPIV target; the
// interchanges are replayed into a permutation of that window, the window
// is gathered out, then copied back.  Rows are 1-based in IPIV.
template <typename T>
int laswp_dev(int ncols, T* dA, int lda, int k1, int k2, const int* dIpiv, int incx, int lo, int span,
              cudaStream_t s) {
  if (ncols <= 0 || incx == 0 || span <= 0) return 0;
  DevScratch perm(sizeof(int) * (size_t)span, s);
  DevScratch tmp(sizeof(T) * (size_t)span * ncols, s);
  if (!perm.p || !tmp.p) return (int)cudaErrorMemoryAllocation;
  int rc = ipiv_perm_dev(dIpiv, k1, k2, incx, lo, span, perm.as<int>(), s);
  if (rc) return rc;
  size_t tot = (size_t)span * ncols;
  unsigned blocks = (unsigned)((tot + 255) / 256);
  GB_LAUNCH(perm_rows_kernel<T, false><<<blocks, 256, 0, s>>>(dA, lda, tmp.as<T>(), span, perm.as<int>(), 0, span, ncols));
  GB_LAUNCH(copy_cols_kernel<T><<<blocks, 256, 0, s>>>(tmp.as<T>(), span, dA + lo, lda, span, ncols));
  return (int)cudaGetLastError();
}
template int laswp_dev<double>(int, double*, int, int, int, const int*, int, int, int, cudaStream_t);
template int laswp_dev<float>(int, float*, int, int, int, const int*, int, int, int, cudaStream_t);

// ------------------------------------------------------------------- GETRS
template <typename T, bool EXACT, bool FORWARD, bool UNIT, bool TRANS>
static int launch_trsv(const T* A, int lda, int n, T* X, int ldx, int nrhs, cudaStream_t s, bool inv_diag,
                       int nbatch = 1, long long sA = 0, long long sX = 0, bool dtrsv_order = false) {
  const int nblk = (n + kSolveBS - 1) / kSolveBS;
  int dev = 0;
  cudaGetDevice(&dev);
  if constexpr (!EXACT) {
    // streaming solve: the publication array (sentinel-filled, all bits
    // set), then the ticket
    const size_t pub_bytes = ((size_t)n * nrhs * nbatch * sizeof(T) + 255) / 256 * 256;
    DevScratch ctl(pub_bytes + 256, s);
    if (!ctl.p) return (int)cudaErrorMemoryAllocation;
    T* pub = ctl.as<T>();
    unsigned* ticket = reinterpret_cast<unsigned*>(ctl.as<char>() + pub_bytes);
    GB_CUDA_TRY(cudaMemsetAsync(pub, 0xFF, pub_bytes, s));
    GB_CUDA_TRY(cudaMemsetAsync(ticket, 0, sizeof(unsigned), s));
    // inverted diagonal blocks only for the FP32 solves
    if constexpr (sizeof(T) != 4) inv_diag = false;
    static bool set_inv[64] = {false}, set_sub[64] = {false};
    bool& set = inv_diag ? set_inv[dev] : set_sub[dev];
    auto kern = trsv_stream_kernel<T, FORWARD, UNIT, TRANS, false>;
    int smem = ts_smem_bytes<T, false>();
    if constexpr (sizeof(T) == 4) {
      if (inv_diag) {
        kern = trsv_stream_kernel<T, FORWARD, UNIT, TRANS, true>;
        smem = ts_smem_bytes<T, true>();
      }
    }
    if (!set) {
      GB_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
      set = true;
    }
    prof_begin(kProfTrsv, s);
    GB_LAUNCH(kern<<<(unsigned)nblk * (unsigned)nbatch, kTsThreads, smem, s>>>(A, lda, n, X, ldx, nrhs, pub, ticket,
                                                                             device_status_word(), sA, sX, nbatch));
    prof_end(kProfTrsv, s, (double)nbatch * n * n * nrhs,
             (double)nbatch * sizeof(T) * (0.5 * n * (double)n + 2.0 * n * nrhs));
    return (int)cudaGetLastError();
  }
  if (nbatch > 1) {
    for (int b = 0; b < nbatch; ++b) {
      int rc = launch_trsv<T, EXACT, FORWARD, UNIT, TRANS>(A + b * sA, lda, n, X + b * sX, ldx, nrhs, s, inv_diag,
                                                           1, 0, 0, dtrsv_order);
      if (rc) return rc;
    }
    return 0;
  }
  if constexpr (TRANS && !FORWARD) {
    // L^T in exact mode: DTRSM folds each element's sum in increasing k,
    // which the blocked kernel's backward order does not; DTRSV folds it in
    // decreasing k (BLAS/SRC/dtrsv.f:296-303), which the blocked kernel does
    if (!dtrsv_order) {
      prof_begin(kProfTrsv, s);
      GB_LAUNCH(trsv_lt_exact_kernel<T, UNIT><<<(unsigned)((nrhs + 63) / 64), 64, 0, s>>>(A, lda, n, X, ldx, nrhs));
      prof_end(kProfTrsv, s, (double)n * n * nrhs, sizeof(T) * (0.5 * n * (double)n + 2.0 * n * nrhs));
      return (int)cudaGetLastError();
    }
  }
  DevScratch ctl(sizeof(int) * (size_t)(nblk + 1), s);
  if (!ctl.p) return (int)cudaErrorMemoryAllocation;
  GB_CUDA_TRY(cudaMemsetAsync(ctl.p, 0, sizeof(int) * (size_t)(nblk + 1), s));
  int* flags = ctl.as<int>();
  unsigned* ticket = reinterpret_cast<unsigned*>(flags + nblk);
  static bool smem_set[64] = {false};
  if (!smem_set[dev]) {
    GB_CUDA_TRY((trsv_set_smem<T, EXACT, FORWARD, UNIT, TRANS>()));
    smem_set[dev] = true;
  }
  prof_begin(kProfTrsv, s);
  GB_LAUNCH(trsv_blocked_kernel<T, EXACT, FORWARD, UNIT, TRANS><<<nblk, 256, kTrsvSmem<T>, s>>>(A, lda, n, X, ldx, nrhs, flags, ticket,
                                                                        device_status_word()));
  prof_end(kProfTrsv, s, (double)n * n * nrhs, sizeof(T) * (0.5 * n * (double)n + 2.0 * n * nrhs));
  return (int)cudaGetLastError();
}

template <typename T, bool EXACT>
static int getrs_impl(char trans, int n, int nrhs, const T* dA, int lda, const int* dPerm, T* dB, int ldb,
                      cudaStream_t s, bool inv) {
  DevScratch w(sizeof(T) * (size_t)n * nrhs, s);
  if (!w.p) return (int)cudaErrorMemoryAllocation;
  T* W = w.as<T>();
  size_t tot = (size_t)n * nrhs;
  unsigned blocks = (unsigned)((tot + 255) / 256);
  int rc;
  if (trans == 'N') {
    GB_LAUNCH(perm_rows_kernel<T, false><<<blocks, 256, 0, s>>>(dB, ldb, W, n, dPerm, 0, n, nrhs));
    if ((rc = launch_trsv<T, EXACT, true, true, false>(dA, lda, n, W, n, nrhs, s, inv))) return rc;
    if ((rc = launch_trsv<T, EXACT, false, false, false>(dA, lda, n, W, n, nrhs, s, inv))) return rc;
    GB_LAUNCH(copy_cols_kernel<T><<<blocks, 256, 0, s>>>(W, n, dB, ldb, n, nrhs));
  } else {
    GB_LAUNCH(copy_cols_kernel<T><<<blocks, 256, 0, s>>>(dB, ldb, W, n, n, nrhs));
    if ((rc = launch_trsv<T, EXACT, true, false, true>(dA, lda, n, W, n, nrhs, s, inv))) return rc;
    if ((rc = launch_trsv<T, EXACT, false, true, true>(dA, lda, n, W, n, nrhs, s, inv))) return rc;
    GB_LAUNCH(perm_rows_kernel<T, true><<<blocks, 256, 0, s>>>(W, n, dB, ldb, dPerm, 0, n, nrhs));
  }
  return (int)cudaGetLastError();
}

template <typename T>
int getrs_dev(char trans, int n, int nrhs, const T* dA, int lda, const int* dIpiv, const int* dPerm, T* dB, int ldb,
              cudaStream_t s, bool inv_diag) {
  if (n <= 0 || nrhs <= 0) return 0;
  DevScratch permbuf(dPerm ? 0 : sizeof(int) * (size_t)n, s);
  if (!dPerm) {
    if (!permbuf.p) return (int)cudaErrorMemoryAllocation;
    int rc = ipiv_perm_dev(dIpiv, 1, n, 1, 0, n, permbuf.as<int>(), s);
    if (rc) return rc;
    dPerm = permbuf.as<int>();
  }
  char t = (trans == 'n' || trans == 'N') ? 'N' : 'T';
  return options().exact ? getrs_impl<T, true>(t, n, nrhs, dA, lda, dPerm, dB, ldb, s, false)
                         : getrs_impl<T, false>(t, n, nrhs, dA, lda, dPerm, dB, ldb, s, inv_diag);
}
template int getrs_dev<double>(char, int, int, const double*, int, const int*, const int*, double*, int, cudaStream_t,
                               bool);
template int getrs_dev<float>(char, int, int, const float*, int, const int*, const int*, float*, int, cudaStream_t,
                              bool);

// op(T) X = B for a batch of systems of one size (T unit lower L or upper U
// of stored LU factors), X overwritten in place; strides in elements.
template <typename T>
int trsv_batched_dev(bool lower, bool trans, int n, int nrhs, const T* dA, int lda, long long sA, T* dX, int ldx,
                     long long sX, int nbatch, cudaStream_t s, bool dtrsv_order) {
  if (n <= 0 || nrhs <= 0 || nbatch <= 0) return 0;
  // solve order: forward for L and for U^T, backward for U and for L^T
  const bool ex = options().exact;
  if (!trans) {
    if (lower)
      return ex ? launch_trsv<T, true, true, true, false>(dA, lda, n, dX, ldx, nrhs, s, false, nbatch, sA, sX)
                : launch_trsv<T, false, true, true, false>(dA, lda, n, dX, ldx, nrhs, s, false, nbatch, sA, sX);
    return ex ? launch_trsv<T, true, false, false, false>(dA, lda, n, dX, ldx, nrhs, s, false, nbatch, sA, sX)
              : launch_trsv<T, false, false, false, false>(dA, lda, n, dX, ldx, nrhs, s, false, nbatch, sA, sX);
  }
  if (lower)
    return ex ? launch_trsv<T, true, false, true, true>(dA, lda, n, dX, ldx, nrhs, s, false, nbatch, sA, sX,
                                                        dtrsv_order)
              : launch_trsv<T, false, false, true, true>(dA, lda, n, dX, ldx, nrhs, s, false, nbatch, sA, sX);
  return ex ? launch_trsv<T, true, true, false, true>(dA, lda, n, dX, ldx, nrhs, s, false, nbatch, sA, sX)
            : launch_trsv<T, false, true, false, true>(dA, lda, n, dX, ldx, nrhs, s, false, nbatch, sA, sX);
}
template int trsv_batched_dev<double>(bool, bool, int, int, const double*, int, long long, double*, int, long long,
                                      int, cudaStream_t, bool);

// op(T) X = B for nrhs right-hand sides with any UPLO / TRANS / DIAG of the
// triangle T (DTRSM('L', ...), BLAS/SRC/dtrsm.f:272-329): exact mode in the
// DTRSM loop order, otherwise the streaming solve.
template <typename T>
int trsm_left_dev(bool upper, bool trans, bool unit, int n, int nrhs, const T* dA, int lda, T* dB, int ldb,
                  cudaStream_t s) {
  if (n <= 0 || nrhs <= 0) return 0;
  const bool ex = options().exact;
#define GB_TRSM(FWD, UN, TR)                                                                           \
  return ex ? launch_trsv<T, true, FWD, UN, TR>(dA, lda, n, dB, ldb, nrhs, s, false)                   \
            : launch_trsv<T, false, FWD, UN, TR>(dA, lda, n, dB, ldb, nrhs, s, false)
  // solve order: forward for L and for U^T, backward for U and for L^T
  if (!trans) {
    if (!upper) { if (unit) GB_TRSM(true, true, false); else GB_TRSM(true, false, false); }
    if (unit) GB_TRSM(false, true, false);
    GB_TRSM(false, false, false);
  }
  if (upper) { if (unit) GB_TRSM(true, true, true); else GB_TRSM(true, false, true); }
  if (unit) GB_TRSM(false, true, true);
  GB_TRSM(false, false, true);
#undef GB_TRSM
}
template int trsm_left_dev<double>(bool, bool, bool, int, int, const double*, int, double*, int, cudaStream_t);
template int trsm_left_dev<float>(bool, bool, bool, int, int, const float*, int, float*, int, cudaStream_t);

// DTRSV (BLAS/SRC/dtrsv.f, INCX = 1) on one device vector for any UPLO,
// TRANS, DIAG, in every mode with the reference's operations: each element's
// sum in the DTRSV loop order and a true division by the diagonal.  DLATRS
// relies on this: its growth bound admits the plain solve for values near
// underflow, where a reciprocal of the diagonal can overflow although the
// quotient does not.
int dtrsv_dev(bool upper, bool trans, bool unit, int n, const double* dA, int lda, double* dX, cudaStream_t s) {
  if (n <= 0) return 0;
  // solve order: forward for L and for U^T, backward for U and for L^T
#define GB_TRSV(FWD, UN, TR) \
  return launch_trsv<double, true, FWD, UN, TR>(dA, lda, n, dX, n, 1, s, false, 1, 0, 0, true)
  if (!trans) {
    if (!upper) { if (unit) GB_TRSV(true, true, false); else GB_TRSV(true, false, false); }
    if (unit) GB_TRSV(false, true, false);
    GB_TRSV(false, false, false);
  }
  if (upper) { if (unit) GB_TRSV(true, true, true); else GB_TRSV(true, false, true); }
  if (unit) GB_TRSV(false, true, true);
  GB_TRSV(false, false, true);
#undef GB_TRSV
}

}  // namespace gb

extern "C" {
int gb300_feed_trace(int on) {
  const int old = gb::g_feed_trace.on;
  gb::g_feed_trace.clear();
  gb::g_feed_trace.on = on != 0;
  return old;
}
// Up to cap records of the last look-ahead factorizations: kind (0 step end,
// 1 chunk taken in, 2 chunk landed and converted, 3 start of the copies, 5
// next block column ready, 6 panel start, 7 panel end),
// index (step or chunk), aux (columns in the window, or the step a chunk
// joined at), milliseconds after the first record.
int gb300_feed_trace_read(int* kind, int* idx, int* aux, double* ms, int cap) {
  auto& t = gb::g_feed_trace;
  if (t.ev.empty()) return 0;
  if (cudaEventSynchronize(t.ev.back()) != cudaSuccess) return -1;
  const int n = std::min<int>(cap, (int)t.ev.size());
  for (int i = 0; i < n; ++i) {
    float f = 0;
    cudaEventElapsedTime(&f, t.ev[0], t.ev[i]);
    kind[i] = t.kind[i];
    idx[i] = t.idx[i];
    aux[i] = t.aux[i];
    ms[i] = f;
  }
  return n;
}
int gb300_leaf_profile(int on) {
  const int old = gb::g_leaf_phase_on;
  gb::g_leaf_phase_on = on != 0;
  return old;
}
int gb300_leaf_profile_read(unsigned long long* cycles) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return -1;
  for (int i = 0; i < 6; ++i) cycles[i] = 0;
  if (!gb::g_leaf_phase[dev]) return 0;
  if (cudaMemcpy(cycles, gb::g_leaf_phase[dev], 6 * sizeof(unsigned long long), cudaMemcpyDeviceToHost) != cudaSuccess)
    return -1;
  cudaMemset(gb::g_leaf_phase[dev], 0, 8 * sizeof(unsigned long long));
  return 0;
}
}  // extern "C"
