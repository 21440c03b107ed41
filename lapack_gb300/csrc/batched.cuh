// Batched DGESV / SGESV on many independent systems of uneven size
// (n <= 512, nrhs <= 4) in one persistent launch.  No single reference
// routine: each system is DGETRF (SRC/dgetrf.f) followed by DGETRS('N')
// (SRC/dgetrs.f), i.e. DGESV (SRC/dgesv.f:148-173), with the same pivot
// rule, scaling rule and per-element update order as the single-system
// path.
//
// CTAs take systems from an atomic queue in the order given by `order`
// (largest first, for load balance).  Per system, a blocked right-looking LU
// with panel width nb (from the per-size-bucket table):
//   panel   rows j..n-1, columns j..j+nb-1 staged in shared memory and
//           factored column by column (block-wide IDAMAX reduction);
//   swaps   the panel's interchanges applied to the other columns as one
//           gather over the touched rows;
//   TRSM    U12 = L11^{-1} A12, one thread per column in registers;
//   update  A22 -= A21 * U12 in tiles, U12 chunks staged in shared memory.
// Then the solve: the permutation applied to B, and both triangular solves
// with one warp per right-hand side (rows spread over the lanes, the solved
// value broadcast by shuffle).  The trailing matrix lives in global memory
// (each system is at most 2 MB in FP64, mostly L2-resident while a CTA
// works on it).
#pragma once
#include "common.cuh"

namespace gb {

constexpr int kBatThreads = 256;
constexpr int kBatMaxN = 512;
constexpr int kBatMaxNb = 64;               // panel width cap (FP64 is limited to 32 by shared memory)
constexpr int kBatMaxRhs = 4;
constexpr int kBatBuckets = kBatMaxN / 64;   // size buckets of 64 rows
constexpr int kBatUChunk = 64;               // U12 columns staged per chunk

// panel [cap][512] + U12 chunk [cap][kBatUChunk] + B [4][512] + labels and pairs
template <typename T>
constexpr size_t batched_smem_bytes(int cap) {
  return sizeof(T) * ((size_t)cap * kBatMaxN + (size_t)cap * kBatUChunk + (size_t)kBatMaxN * kBatMaxRhs) +
         sizeof(int) * (4 * kBatMaxNb + kBatMaxN) + 64;
}
template <typename T>
constexpr int batched_cap() { return sizeof(T) == 8 ? 32 : 64; }

template <typename T>
struct BatchArgs {
  int batch;
  const int* n;
  const int* nrhs;
  T* const* A;
  const int* lda;
  int* const* ipiv;
  T* const* B;
  const int* ldb;
  int* info;
  const int* order;        // processing order (largest systems first)
  unsigned* queue;         // zeroed before the launch
  const int* nb_table;     // panel width per 64-row size bucket (each <= cap)
  int cap;                 // panel width the shared memory is laid out for (32 or 64)
  int solve;               // 0: factor only (DGETRF), 1: factor + solve (DGESV)
};

// Block-wide IDAMAX over x[0..len) of a shared-memory column: returns the
// index (first maximum, NaN only when first) to every thread.
template <typename T>
__device__ __forceinline__ int block_iamax(const T* x, int len, Cand<T>* red) {
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  Cand<T> best;
  best.absval = 0; best.row = -1; best.cls = -1;
  for (int i = tid; i < len; i += kBatThreads) {
    Cand<T> c = make_cand(x[i], i, 0);
    if (cand_better(c, best)) best = c;
  }
  best = warp_best(best);
  if (lane == 0) red[warp] = best;
  __syncthreads();
  if (warp == 0) {
    Cand<T> c = lane < kBatThreads / 32 ? red[lane] : Cand<T>{0, -1, -1};
    c = warp_best(c);
    if (lane == 0) red[kBatThreads / 32] = c;
  }
  __syncthreads();
  const int r = red[kBatThreads / 32].row;
  return r < 0 ? 0 : r;
}

// Shared-memory layout, sized for the widest panel `cap`:
// [panel cap x 512][U12 chunk cap x 64][B 4 x 512][labels 512][pairs 2 x 128]
template <typename T>
__device__ __forceinline__ T* bat_panel(unsigned char* smem) { return reinterpret_cast<T*>(smem); }
template <typename T>
__device__ __forceinline__ T* bat_uchunk(unsigned char* smem, int cap) {
  return bat_panel<T>(smem) + (size_t)cap * kBatMaxN;
}
template <typename T>
__device__ __forceinline__ T* bat_rhs(unsigned char* smem, int cap) {
  return bat_uchunk<T>(smem, cap) + (size_t)cap * kBatUChunk;
}
template <typename T>
__device__ __forceinline__ int* bat_labels(unsigned char* smem, int cap) {
  return reinterpret_cast<int*>(bat_rhs<T>(smem, cap) + (size_t)kBatMaxN * kBatMaxRhs);
}

template <typename T, bool EXACT>
__device__ void batched_getrf_one(int n, T* __restrict__ A, int lda, int* __restrict__ ipiv, int* __restrict__ info,
                                  int nb, int cap, unsigned char* smem) {
  const int tid = threadIdx.x;
  T* P = bat_panel<T>(smem);                                // panel [nb][M]
  T* U = bat_uchunk<T>(smem, cap);                          // U12 chunk [nb][kBatUChunk]
  int* lab = bat_labels<T>(smem, cap);                      // [kBatMaxN]
  int* pd = lab + kBatMaxN;                                 // pair dst [2nb]
  int* ps = pd + 2 * kBatMaxNb;                             // pair src [2nb]
  __shared__ Cand<T> red[kBatThreads / 32 + 1];
  __shared__ int npairs_s;
  int first_zero = 0;
  for (int j = 0; j < n; j += nb) {
    const int jb = min(nb, n - j);
    const int M = n - j;
    // 1. stage the panel and factor it column by column
    batched_copy<8, kBatThreads, T>(
        jb * M, tid, [&](int e) { const int c = e / M, r = e - c * M; return A[(size_t)(j + r) + (size_t)(j + c) * lda]; },
        [&](int e, T v) { const int c = e / M, r = e - c * M; P[c * M + r] = v; });
    for (int r = tid; r < M; r += kBatThreads) lab[r] = r;
    __syncthreads();
    for (int k = 0; k < jb; ++k) {
      const int p = k + block_iamax<T>(P + k * M + k, M - k, red);
      const T pv = P[k * M + p];
      if (tid == 0) {
        ipiv[j + k] = j + p + 1;
        if (pv == T(0) && first_zero == 0) first_zero = j + k + 1;
      }
      if (pv == T(0) && first_zero == 0) first_zero = j + k + 1;
      if (p != k) {
        for (int c = tid; c < jb; c += kBatThreads) {
          const T t = P[c * M + k];
          P[c * M + k] = P[c * M + p];
          P[c * M + p] = t;
        }
        if (tid == 0) { const int t = lab[k]; lab[k] = lab[p]; lab[p] = t; }
      }
      __syncthreads();
      const bool scale = pv != T(0);
      const bool recip = (pv < 0 ? -pv : pv) >= Lim<T>::sfmin();
      const T rp = T(1) / pv;
      for (int r = k + 1 + tid; r < M; r += kBatThreads) {
        const T v = P[k * M + r];
        const T l = scale ? (recip ? v * rp : v / pv) : v;
        P[k * M + r] = l;
        for (int c = k + 1; c < jb; ++c) P[c * M + r] = fnmadd<EXACT>(l, P[c * M + k], P[c * M + r]);
      }
      __syncthreads();
    }
    // write the factored panel back
    for (int e = tid; e < jb * M; e += kBatThreads) {
      const int c = e / M, r = e - c * M;
      A[(size_t)(j + r) + (size_t)(j + c) * lda] = P[c * M + r];
    }
    // 2. interchanges of the other columns as a gather over the moved rows
    if (tid == 0) {
      int np = 0;
      for (int r = 0; r < M && np < 2 * kBatMaxNb; ++r)
        if (lab[r] != r) { pd[np] = j + r; ps[np] = j + lab[r]; ++np; }
      npairs_s = np;
    }
    __syncthreads();
    const int np = npairs_s;
    if (np > 0) {
      for (int c = tid; c < n; c += kBatThreads) {
        if (c >= j && c < j + jb) continue;
        T v[2 * kBatMaxNb];
#pragma unroll 8
        for (int i = 0; i < np; ++i) v[i] = A[(size_t)ps[i] + (size_t)c * lda];
#pragma unroll 8
        for (int i = 0; i < np; ++i) A[(size_t)pd[i] + (size_t)c * lda] = v[i];
      }
    }
    __syncthreads();
    const int ncol = n - j - jb;
    if (ncol <= 0) continue;
    // 3. U12 = L11^{-1} A12 (L11 = top jb rows of the panel), per column in registers
    for (int c = tid; c < ncol; c += kBatThreads) {
      T x[kBatMaxNb];
      T* col = A + (size_t)j + (size_t)(j + jb + c) * lda;
#pragma unroll
      for (int i = 0; i < kBatMaxNb; ++i) x[i] = i < jb ? col[i] : T(0);
#pragma unroll
      for (int kk = 0; kk < kBatMaxNb - 1; ++kk) {
        if (kk < jb - 1) {
#pragma unroll
          for (int i = kk + 1; i < kBatMaxNb; ++i)
            if (i < jb) x[i] = fnmadd<EXACT>(x[kk], P[kk * M + i], x[i]);
        }
      }
#pragma unroll
      for (int i = 0; i < kBatMaxNb; ++i)
        if (i < jb) col[i] = x[i];
    }
    __syncthreads();
    // 4. A22 -= A21 * U12 in chunks of kBatUChunk columns; A21 = panel rows jb..M-1
    const int mrows = M - jb;
    for (int cb = 0; cb < ncol; cb += kBatUChunk) {
      const int cw = min(kBatUChunk, ncol - cb);
      batched_copy<8, kBatThreads, T>(
          jb * cw, tid,
          [&](int e) { const int c = e / jb, r = e - c * jb; return A[(size_t)(j + r) + (size_t)(j + jb + cb + c) * lda]; },
          [&](int e, T v) { const int c = e / jb, r = e - c * jb; U[r * kBatUChunk + c] = v; });
      __syncthreads();
      // each thread: 4 rows x 4 columns of the chunk per pass
      const int tiles_r = (mrows + 3) / 4, tiles_c = (cw + 3) / 4;
      for (int t = tid; t < tiles_r * tiles_c; t += kBatThreads) {
        const int tr = t % tiles_r, tc = t / tiles_r;
        const int r0 = tr * 4, c0 = tc * 4;
        T acc[4][4];
#pragma unroll
        for (int a = 0; a < 4; ++a)
#pragma unroll
          for (int b = 0; b < 4; ++b) {
            const int r = r0 + a, c = c0 + b;
            acc[a][b] = (r < mrows && c < cw) ? A[(size_t)(j + jb + r) + (size_t)(j + jb + cb + c) * lda] : T(0);
          }
        for (int kk = 0; kk < jb; ++kk) {
          T av[4], bv[4];
#pragma unroll
          for (int a = 0; a < 4; ++a) av[a] = (r0 + a < mrows) ? P[kk * M + jb + r0 + a] : T(0);
#pragma unroll
          for (int b = 0; b < 4; ++b) bv[b] = U[kk * kBatUChunk + c0 + b];
#pragma unroll
          for (int a = 0; a < 4; ++a)
#pragma unroll
            for (int b = 0; b < 4; ++b) acc[a][b] = fnmadd<EXACT>(av[a], bv[b], acc[a][b]);
        }
#pragma unroll
        for (int a = 0; a < 4; ++a)
#pragma unroll
          for (int b = 0; b < 4; ++b) {
            const int r = r0 + a, c = c0 + b;
            if (r < mrows && c < cw) A[(size_t)(j + jb + r) + (size_t)(j + jb + cb + c) * lda] = acc[a][b];
          }
      }
      __syncthreads();
    }
  }
  if (tid == 0) *info = first_zero;
  __syncthreads();
}

// X := A^{-1} B with the factors of batched_getrf_one: the interchanges
// (IPIV replayed in order) and the two triangular solves, one warp per
// right-hand side.  The factors are staged in 32-column chunks into the
// panel buffer so the sequential steps read shared memory, not L2.  The
// per-element order is the reference one (BLAS/SRC/dtrsm.f:278-300).
constexpr int kBatSolveChunk = 32;

template <typename T, bool EXACT>
__device__ void batched_getrs_one(int n, int nrhs, const T* __restrict__ A, int lda, const int* __restrict__ ipiv,
                                  T* __restrict__ B, int ldb, unsigned char* smem, int cap) {
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  T* Lc = bat_panel<T>(smem);                               // [kBatSolveChunk][n] chunk of factors (cap >= 32)
  T* Bs = bat_rhs<T>(smem, cap);                            // [nrhs][kBatMaxN]
  for (int e = tid; e < n * nrhs; e += kBatThreads) {
    const int q = e / n, r = e - q * n;
    Bs[q * kBatMaxN + r] = B[(size_t)r + (size_t)q * ldb];
  }
  __syncthreads();
  if (warp < nrhs && lane == 0) {
    T* x = Bs + warp * kBatMaxN;
    for (int i = 0; i < n; ++i) {
      const int p = ipiv[i] - 1;
      if (p != i) { const T t = x[i]; x[i] = x[p]; x[p] = t; }
    }
  }
  __syncthreads();
  // L (unit lower): columns k0..k0+31 staged, rows k0..n-1
  for (int k0 = 0; k0 < n; k0 += kBatSolveChunk) {
    const int kw = min(kBatSolveChunk, n - k0), rows = n - k0;
    batched_copy<8, kBatThreads, T>(
        kw * rows, tid,
        [&](int e) { const int c = e / rows, r = e - c * rows; return A[(size_t)(k0 + r) + (size_t)(k0 + c) * lda]; },
        [&](int e, T v) { const int c = e / rows, r = e - c * rows; Lc[c * rows + r] = v; });
    __syncthreads();
    if (warp < nrhs) {
      T* x = Bs + warp * kBatMaxN;
      for (int c = 0; c < kw; ++c) {
        const T xk = x[k0 + c];
        for (int r = c + 1 + lane; r < rows; r += 32) x[k0 + r] = fnmadd<EXACT>(xk, Lc[c * rows + r], x[k0 + r]);
        __syncwarp();
      }
    }
    __syncthreads();
  }
  // U (non-unit upper): chunks from the bottom, rows 0..k1-1
  for (int k1 = n; k1 > 0; k1 -= kBatSolveChunk) {
    const int k0 = max(0, k1 - kBatSolveChunk), kw = k1 - k0, rows = k1;
    batched_copy<8, kBatThreads, T>(
        kw * rows, tid,
        [&](int e) { const int c = e / rows, r = e - c * rows; return A[(size_t)r + (size_t)(k0 + c) * lda]; },
        [&](int e, T v) { const int c = e / rows, r = e - c * rows; Lc[c * rows + r] = v; });
    __syncthreads();
    if (warp < nrhs) {
      T* x = Bs + warp * kBatMaxN;
      for (int c = kw - 1; c >= 0; --c) {
        const int k = k0 + c;
        if (lane == 0) x[k] = x[k] / Lc[c * rows + k];
        __syncwarp();
        const T xk = x[k];
        for (int r = lane; r < k; r += 32) x[r] = fnmadd<EXACT>(xk, Lc[c * rows + r], x[r]);
        __syncwarp();
      }
    }
    __syncthreads();
  }
  for (int e = tid; e < n * nrhs; e += kBatThreads) {
    const int q = e / n, r = e - q * n;
    B[(size_t)r + (size_t)q * ldb] = Bs[q * kBatMaxN + r];
  }
  __syncthreads();
}

template <typename T, bool EXACT>
__global__ void __launch_bounds__(kBatThreads)
batched_gesv_kernel(BatchArgs<T> a) {
  extern __shared__ __align__(16) unsigned char bat_smem[];
  __shared__ int sys_s;
  for (;;) {
    if (threadIdx.x == 0) {
      const unsigned t = atomicAdd(a.queue, 1u);
      sys_s = t < (unsigned)a.batch ? a.order[t] : -1;
    }
    __syncthreads();
    const int s = sys_s;
    __syncthreads();
    if (s < 0) break;
    const int n = a.n[s];
    if (n <= 0 || n > kBatMaxN) {
      if (threadIdx.x == 0) a.info[s] = n > kBatMaxN ? -1 : 0;
      continue;
    }
    const int nb = min(max(a.nb_table[(n - 1) / 64], 1), a.cap);
    batched_getrf_one<T, EXACT>(n, a.A[s], a.lda[s], a.ipiv[s], a.info + s, nb, a.cap, bat_smem);
    __syncthreads();
    if (a.solve && a.info[s] == 0 && a.nrhs[s] > 0)
      batched_getrs_one<T, EXACT>(n, min(a.nrhs[s], kBatMaxRhs), a.A[s], a.lda[s], a.ipiv[s], a.B[s], a.ldb[s],
                                  bat_smem, a.cap);
  }
}

// The per-bucket panel widths, passed by value.
struct BucketTable { int nb[kBatBuckets]; };
static __global__ void batched_set_table_kernel(int* __restrict__ tab, BucketTable t) {
  if (threadIdx.x < kBatBuckets) tab[threadIdx.x] = t.nb[threadIdx.x];
}

// Counting sort of the systems by n, largest first.
static __global__ void batched_hist_kernel(int batch, const int* __restrict__ n, int* __restrict__ hist) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < batch) atomicAdd(hist + min(max(n[i], 0), kBatMaxN + 1), 1);
}
static __global__ void batched_scan_kernel(int* __restrict__ hist) {
  // exclusive scan from the largest size down (single thread: 514 entries)
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    int run = 0;
    for (int v = kBatMaxN + 1; v >= 0; --v) { const int c = hist[v]; hist[v] = run; run += c; }
  }
}
static __global__ void batched_place_kernel(int batch, const int* __restrict__ n, int* __restrict__ cursor,
                                            int* __restrict__ order) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < batch) order[atomicAdd(cursor + min(max(n[i], 0), kBatMaxN + 1), 1)] = i;
}

}  // namespace gb
