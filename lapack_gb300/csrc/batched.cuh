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

// Threads per CTA and CTAs per SM: two CTAs of 256 threads (eight warps)
// per SM, 128 registers per thread; a 32-column FP32 panel (83 KB of
// shared memory per CTA) or a 16-column FP64 one (94 KB).  Two systems per
// SM overlap their per-column latencies: one 512-thread FP32 CTA per SM with
// a 64-column panel was 1.7x slower, four 128-thread ones 1.07x; one FP64
// CTA per SM 1.2x.
template <typename T>
constexpr int bat_threads() { return 256; }
template <typename T>
constexpr int bat_ctas_per_sm() { return 2; }
constexpr int kBatMaxN = 512;
constexpr int kBatMaxNb = 64;               // panel width cap (FP64 is limited to 32 by shared memory)
constexpr int kBatMaxRhs = 4;
constexpr int kBatBuckets = kBatMaxN / 64;   // size buckets of 64 rows
// U12 columns staged per chunk: the block-row solve takes eight columns per warp
template <typename T>
constexpr int bat_uchunk_cols() { return bat_threads<T>() / 32 * 8; }
constexpr int kBatUStride = 64 + 8;          // row stride of the staged chunk (spreads the solve's lanes over the banks)
constexpr int kBatDefer = 4;                 // panel columns whose rank-1 updates are applied together
static_assert(bat_uchunk_cols<float>() + 8 <= kBatUStride && bat_uchunk_cols<double>() + 8 <= kBatUStride,
              "the staged U12 chunk fits its row stride");
static_assert(bat_threads<float>() >= kBatMaxNb && bat_threads<double>() >= kBatMaxNb,
              "the pivot-row step takes one thread per panel column");

// panel [cap][512] + two U12 chunks [cap][kBatUStride] + B [4][512] + labels and pairs
template <typename T>
constexpr size_t batched_smem_bytes(int cap) {
  return sizeof(T) * ((size_t)cap * kBatMaxN + 2 * (size_t)cap * kBatUStride + (size_t)kBatMaxN * kBatMaxRhs) +
         sizeof(int) * (4 * kBatMaxNb + kBatMaxN) + 64;
}
template <typename T>
constexpr int batched_cap() { return sizeof(T) == 8 ? 16 : 32; }

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
  unsigned long long* phase;   // per-phase SM cycles summed over CTAs (kBatPhases), or null
};

// Phases of the per-system work whose cycles the optional instrumentation
// sums (thread 0 of every CTA, clock64 differences).
enum : int { kBatPhQueue = 0, kBatPhStage, kBatPhPanel, kBatPhSwap, kBatPhTrsm, kBatPhUpdate, kBatPhSolve, kBatPhases };
struct BatPhaseClock {
  unsigned long long* out;
  long long t0;
  __device__ __forceinline__ explicit BatPhaseClock(unsigned long long* o) : out(threadIdx.x == 0 ? o : nullptr) {
    t0 = out ? clock64() : 0;
  }
  __device__ __forceinline__ void mark(int ph) {
    if (out) {
      const long long now = clock64();
      atomicAdd(out + ph, (unsigned long long)(now - t0));
      t0 = now;
    }
  }
};

// 16-byte shared-memory vector of T and its unpacking.
template <typename T> struct Vec16;
template <> struct Vec16<float> {
  using type = float4;
  __device__ __forceinline__ static void unpack(const float4& v, float* o) { o[0] = v.x; o[1] = v.y; o[2] = v.z; o[3] = v.w; }
};
template <> struct Vec16<double> {
  using type = double2;
  __device__ __forceinline__ static void unpack(const double2& v, double* o) { o[0] = v.x; o[1] = v.y; }
};

// Shared-memory layout, sized for the widest panel `cap`:
// [panel cap x 512][U12 chunk cap x kBatUStride][B 4 x 512][labels 512][pairs 2 x 128]
// Copies a rows x cols block element (r, c) from src(r, c) to dst(r, c, v):
// warp w takes columns w, w + NT/32, ..., its lanes the rows, 32 bytes of
// loads per lane in flight before the stores (no index division per element).
template <int NT, typename T, typename Src, typename Dst>
__device__ __forceinline__ void colwise_copy(int rows, int cols, int tid, Src src, Dst dst) {
  constexpr int U = 32 / (int)sizeof(T);
  const int warp = tid >> 5, lane = tid & 31;
  for (int c = warp; c < cols; c += NT / 32)
    for (int r0 = 0; r0 < rows; r0 += 32 * U) {
      T v[U];
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const int r = r0 + lane + 32 * u;
        if (r < rows) v[u] = src(r, c);
      }
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const int r = r0 + lane + 32 * u;
        if (r < rows) dst(r, c, v[u]);
      }
    }
}

template <typename T>
__device__ __forceinline__ T* bat_panel(unsigned char* smem) { return reinterpret_cast<T*>(smem); }
template <typename T>
__device__ __forceinline__ T* bat_uchunk(unsigned char* smem, int cap) {
  return bat_panel<T>(smem) + (size_t)cap * kBatMaxN;
}
template <typename T>
__device__ __forceinline__ T* bat_rhs(unsigned char* smem, int cap) {
  return bat_uchunk<T>(smem, cap) + 2 * (size_t)cap * kBatUStride;
}
template <typename T>
__device__ __forceinline__ int* bat_labels(unsigned char* smem, int cap) {
  return reinterpret_cast<int*>(bat_rhs<T>(smem, cap) + (size_t)kBatMaxN * kBatMaxRhs);
}

template <typename T, bool EXACT>
__device__ void batched_getrf_one(int n, T* __restrict__ A, int lda, int* __restrict__ ipiv, int* __restrict__ info,
                                  int nb, int cap, unsigned char* smem, BatPhaseClock& clk) {
  constexpr int kBatThreads = bat_threads<T>();
  const int tid = threadIdx.x;
  T* P = bat_panel<T>(smem);                                // panel [nb][M]
  T* const Ubuf = bat_uchunk<T>(smem, cap);                 // two U12 chunks [nb][kBatUStride]
  int* lab = bat_labels<T>(smem, cap);                      // [kBatMaxN]
  int* pd = lab + kBatMaxN;                                 // pair dst [2nb]
  int* ps = pd + 2 * kBatMaxNb;                             // pair src [2nb]
  __shared__ Cand<T> red[kBatThreads / 32 + 1];
  __shared__ int npairs_s;
  // pivot rows of the columns whose updates are still pending (slot k % kBatDefer)
  __shared__ T uh[kBatDefer * kBatMaxNb];
  int first_zero = 0;
  for (int j = 0; j < n; j += nb) {
    const int jb = min(nb, n - j);
    const int M = n - j;
    const int Mp = (M + 3) & ~3;          // panel column stride: 16-byte aligned columns
    // 1. stage the panel and factor it column by column
    colwise_copy<kBatThreads, T>(
        M, jb, tid, [&](int r, int c) { return A[(size_t)(j + r) + (size_t)(j + c) * lda]; },
        [&](int r, int c, T v) { P[c * Mp + r] = v; });
    for (int r = tid; r < M; r += kBatThreads) lab[r] = r;
    __syncthreads();
    clk.mark(kBatPhStage);
    // Column by column, with the rank-1 updates of a group of kBatDefer
    // columns deferred: column k+1 receives the group's pending updates at
    // once (its values are the next pivot candidates, searched during that
    // update), the columns after it receive them every kBatDefer columns in
    // one pass.  Every element still receives its updates in increasing k
    // (the order of SRC/dgetrf2.f), so the factors are those of the
    // column-by-column loop.  Per column: one CTA-wide reduction of the
    // candidates, one barrier after the interchange.
    Cand<T> mine{0, -1, -1};
    for (int r = tid; r < M; r += kBatThreads) {
      const Cand<T> c = make_cand(P[r], r, 0);
      if (cand_better(c, mine)) mine = c;
    }
    for (int k = 0; k < jb; ++k) {
      const int s_slot = k % kBatDefer, kfirst = k - s_slot;
      // 1. the pivot: warp winners, then every thread reduces the warps'
      mine = warp_best(mine);
      if ((tid & 31) == 0) red[tid >> 5] = mine;
      __syncthreads();
      Cand<T> best = red[0];
#pragma unroll
      for (int w = 1; w < kBatThreads / 32; ++w)
        if (cand_better(red[w], best)) best = red[w];
      const int p = best.row < 0 ? k : best.row;
      // 2. the pivot row brought up to date (the group's pending updates on
      //    its columns after k+1) becomes row k of U and the pending-update
      //    row of this column; the old row k moves to p as it stands (its
      //    multipliers and pending updates travel with it)
      //    (threads 0..63, one column each: every read of the two rows
      //    before any write, separated by a barrier of those 64 threads)
      if (tid < kBatMaxNb) {
        const int c = tid;
        T v = T(0), old_k = T(0);
        if (c < jb) {
          v = P[c * Mp + p];
          if (c > k)
            for (int d = 0; d < s_slot; ++d) v = fnmadd<EXACT>(P[(kfirst + d) * Mp + p], uh[d * kBatMaxNb + c], v);
          old_k = P[c * Mp + k];
        }
        asm volatile("bar.sync 1, %0;" ::"n"(kBatMaxNb) : "memory");
        if (c < jb) {
          uh[s_slot * kBatMaxNb + c] = v;
          if (p != k) P[c * Mp + p] = old_k;
          P[c * Mp + k] = v;
        }
        if (c == 0 && p != k) { const int t = lab[k]; lab[k] = lab[p]; lab[p] = t; }
      }
      __syncthreads();
      const T pv = P[k * Mp + k];
      if (tid == 0) ipiv[j + k] = j + p + 1;
      if (pv == T(0) && first_zero == 0) first_zero = j + k + 1;
      // 3. scale column k, update column k+1 (and search it), flush the
      //    group's updates into the later columns every kBatDefer columns
      const bool scale = pv != T(0);
      const bool recip = (pv < 0 ? -pv : pv) >= Lim<T>::sfmin();
      const T rp = T(1) / pv;
      const bool flush = s_slot == kBatDefer - 1;
      mine = Cand<T>{0, -1, -1};
      for (int r = k + 1 + tid; r < M; r += kBatThreads) {
        const T v = P[k * Mp + r];
        T l = v;
        if (scale) l = recip ? v * rp : v / pv;
        P[k * Mp + r] = l;
        T ld[kBatDefer];
#pragma unroll
        for (int d = 0; d < kBatDefer; ++d) ld[d] = d < s_slot ? P[(kfirst + d) * Mp + r] : (d == s_slot ? l : T(0));
        if (k + 1 < jb) {
          T t = P[(k + 1) * Mp + r];
#pragma unroll
          for (int d = 0; d < kBatDefer; ++d)
            if (d <= s_slot) t = fnmadd<EXACT>(ld[d], uh[d * kBatMaxNb + k + 1], t);
          P[(k + 1) * Mp + r] = t;
          const Cand<T> c = make_cand(t, r, k + 1);
          if (cand_better(c, mine)) mine = c;
        }
        if (flush) {
          for (int c = k + 2; c < jb; ++c) {
            T t = P[c * Mp + r];
#pragma unroll
            for (int d = 0; d < kBatDefer; ++d) t = fnmadd<EXACT>(ld[d], uh[d * kBatMaxNb + c], t);
            P[c * Mp + r] = t;
          }
        }
      }
    }
    // (no update is left pending: the last column's k+1 step covers the
    // panel's final column)
    __syncthreads();
    clk.mark(kBatPhPanel);
    // write the factored panel back
    colwise_copy<kBatThreads, T>(
        M, jb, tid, [&](int r, int c) { return P[c * Mp + r]; },
        [&](int r, int c, T v) { A[(size_t)(j + r) + (size_t)(j + c) * lda] = v; });
    // 2. interchanges of the other columns as a gather over the moved rows
    // (at most 2 jb rows moved; their order in the list does not matter:
    // every source is read before any destination is written)
    if (tid == 0) npairs_s = 0;
    __syncthreads();
    for (int r = tid; r < M; r += kBatThreads) {
      if (lab[r] != r) {
        const int slot = atomicAdd(&npairs_s, 1);
        if (slot < 2 * kBatMaxNb) {
          pd[slot] = j + r;
          ps[slot] = j + lab[r];
        }
      }
    }
    __syncthreads();
    const int np = min(npairs_s, 2 * kBatMaxNb);
    if (np > 0) {
      // a warp moves kG columns at a time, the lanes over the moved rows
      // (np <= 128): all kG columns' sources are loaded before any of their
      // destinations is written, so the loads of a round are in flight together
      const int warp = tid >> 5, lane = tid & 31;
      constexpr int kPer = 2 * kBatMaxNb / 32, kG = sizeof(T) == 4 ? 4 : 2, kW = kBatThreads / 32;
      for (int c0 = warp * kG; c0 < n; c0 += kW * kG) {
        T v[kG][kPer];
#pragma unroll
        for (int g = 0; g < kG; ++g) {
          const int c = c0 + g;
          const bool live = c < n && (c < j || c >= j + jb);
#pragma unroll
          for (int q = 0; q < kPer; ++q) {
            const int i = lane + 32 * q;
            if (live && i < np) v[g][q] = A[(size_t)c * lda + ps[i]];
          }
        }
        __syncwarp();
#pragma unroll
        for (int g = 0; g < kG; ++g) {
          const int c = c0 + g;
          const bool live = c < n && (c < j || c >= j + jb);
#pragma unroll
          for (int q = 0; q < kPer; ++q) {
            const int i = lane + 32 * q;
            if (live && i < np) A[(size_t)c * lda + pd[i]] = v[g][q];
          }
        }
      }
    }
    __syncthreads();
    clk.mark(kBatPhSwap);
    const int ncol = n - j - jb;
    if (ncol <= 0) continue;
    // 3 + 4. per chunk of bat_uchunk_cols columns of the block row: stage A12 in
    //    shared memory, U12 = L11^{-1} A12 there (SRC/dgetrf.f:204), write
    //    U12 back, then A22 -= A21 * U12 (SRC/dgetrf.f:212-216) with U12 read
    //    from shared memory.  The triangular solve: warp w takes columns
    //    8w..8w+7, the four lane groups of eight the rows of one residue mod
    //    4, one step per column kk of L11 (every element gets its updates in
    //    increasing kk, the order of BLAS/SRC/dtrsm.f:290-300).
    //    The chunks alternate between two buffers: the next chunk's A12
    //    (final once the interchanges are done; the current chunk's update
    //    writes only rows below the block row) is loaded with cp.async while
    //    the current chunk is written back and updated.
    constexpr int kUChunk = bat_uchunk_cols<T>();
    auto prefetch = [&](int cb, T* dst) {
      const int cw = min(kUChunk, ncol - cb);
      for (int e = tid; e < jb * cw; e += kBatThreads) {
        const int c = e / jb, r = e - c * jb;
        cp_async_elem_zfill(dst + r * kBatUStride + c, A + (size_t)(j + r) + (size_t)(j + jb + cb + c) * lda, true);
      }
      cp_async_commit();
    };
    prefetch(0, Ubuf);
    for (int cb = 0, it = 0; cb < ncol; cb += kUChunk, ++it) {
      const int cw = min(kUChunk, ncol - cb);
      T* U = Ubuf + (size_t)(it & 1) * cap * kBatUStride;
      cp_async_wait<0>();
      __syncthreads();
      {
        const int lane = tid & 31, c = 8 * (tid >> 5) + (lane & 7), q = lane >> 3;
        const bool live = c < cw;
        for (int kk = 0; kk + 1 < jb; ++kk) {
          if (live) {
            const T xk = U[kk * kBatUStride + c];
            const int i0 = kk + 1 + ((q - (kk + 1)) & 3);
            for (int i = i0; i < jb; i += 4)
              U[i * kBatUStride + c] = fnmadd<EXACT>(xk, P[kk * Mp + i], U[i * kBatUStride + c]);
          }
          __syncwarp();
        }
      }
      __syncthreads();
      if (cb + kUChunk < ncol) prefetch(cb + kUChunk, Ubuf + (size_t)((it + 1) & 1) * cap * kBatUStride);
      colwise_copy<kBatThreads, T>(
          jb, cw, tid, [&](int r, int c) { return U[r * kBatUStride + c]; },
          [&](int r, int c, T v) { A[(size_t)(j + r) + (size_t)(j + jb + cb + c) * lda] = v; });
      clk.mark(kBatPhTrsm);
      // each thread: a 4 x 4 tile of the chunk per pass, its operands read
      // from shared memory with 16-byte loads.  Tile rows start at the
      // aligned row jb & ~3 of the panel; rows above jb (part of U) and
      // columns past the chunk are computed but not stored.
      constexpr int VE = 16 / (int)sizeof(T);               // elements per 16-byte load
      using V = typename Vec16<T>::type;
      const int rb = jb & ~3;
      const int tiles_r = (M - rb + 3) / 4, tiles_c = (cw + 3) / 4;
      for (int t = tid; t < tiles_r * tiles_c; t += kBatThreads) {
        const int tr = t % tiles_r, tc = t / tiles_r;
        const int r0 = rb + tr * 4, c0 = tc * 4;          // panel row, chunk column
        T acc[4][4];
#pragma unroll
        for (int a = 0; a < 4; ++a)
#pragma unroll
          for (int b = 0; b < 4; ++b) {
            const int r = r0 + a, c = c0 + b;
            acc[a][b] = (r >= jb && r < M && c < cw) ? A[(size_t)(j + r) + (size_t)(j + jb + cb + c) * lda] : T(0);
          }
        for (int kk = 0; kk < jb; ++kk) {
          T av[4], bv[4];
          const V* pa = reinterpret_cast<const V*>(P + (size_t)kk * Mp + r0);
          const V* pb = reinterpret_cast<const V*>(U + (size_t)kk * kBatUStride + c0);
#pragma unroll
          for (int qv = 0; qv < 4 / VE; ++qv) {
            Vec16<T>::unpack(pa[qv], av + qv * VE);
            Vec16<T>::unpack(pb[qv], bv + qv * VE);
          }
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
            if (r >= jb && r < M && c < cw) A[(size_t)(j + r) + (size_t)(j + jb + cb + c) * lda] = acc[a][b];
          }
      }
      __syncthreads();
      clk.mark(kBatPhUpdate);
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

// x[r] -= xk * l[r] for the rows r = r0, r0 + 32, ... below rend (one lane's
// share of a column step): the loads of four rows are issued before their
// updates, one update per element as in the loop form.
template <bool EXACT, typename T>
__device__ __forceinline__ void axpy_rows(T xk, const T* __restrict__ l, T* __restrict__ x, int r0, int rend) {
  int r = r0;
  for (; r + 96 < rend; r += 128) {
    const T l0 = l[r], l1 = l[r + 32], l2 = l[r + 64], l3 = l[r + 96];
    const T x0 = x[r], x1 = x[r + 32], x2 = x[r + 64], x3 = x[r + 96];
    x[r] = fnmadd<EXACT>(xk, l0, x0);
    x[r + 32] = fnmadd<EXACT>(xk, l1, x1);
    x[r + 64] = fnmadd<EXACT>(xk, l2, x2);
    x[r + 96] = fnmadd<EXACT>(xk, l3, x3);
  }
  for (; r < rend; r += 32) x[r] = fnmadd<EXACT>(xk, l[r], x[r]);
}

template <typename T, bool EXACT>
__device__ void batched_getrs_one(int n, int nrhs, const T* __restrict__ A, int lda, const int* __restrict__ ipiv,
                                  T* __restrict__ B, int ldb, unsigned char* smem, int cap) {
  constexpr int kBatThreads = bat_threads<T>();
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  T* Lc = bat_panel<T>(smem);                               // [sc][n] chunk of factors, sc <= cap
  const int sc = min(kBatSolveChunk, cap);
  T* Bs = bat_rhs<T>(smem, cap);                            // [nrhs][kBatMaxN]
  colwise_copy<kBatThreads, T>(
      n, nrhs, tid, [&](int r, int q) { return B[(size_t)r + (size_t)q * ldb]; },
      [&](int r, int q, T v) { Bs[q * kBatMaxN + r] = v; });
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
  for (int k0 = 0; k0 < n; k0 += sc) {
    const int kw = min(sc, n - k0), rows = n - k0;
    colwise_copy<kBatThreads, T>(
        rows, kw, tid, [&](int r, int c) { return A[(size_t)(k0 + r) + (size_t)(k0 + c) * lda]; },
        [&](int r, int c, T v) { Lc[c * rows + r] = v; });
    __syncthreads();
    if (warp < nrhs) {
      T* __restrict__ x = Bs + warp * kBatMaxN + k0;
      for (int c = 0; c < kw; ++c) {
        const T xk = x[c];
        axpy_rows<EXACT>(xk, Lc + c * rows, x, c + 1 + lane, rows);
        __syncwarp();
      }
    }
    __syncthreads();
  }
  // U (non-unit upper): chunks from the bottom, rows 0..k1-1
  for (int k1 = n; k1 > 0; k1 -= sc) {
    const int k0 = max(0, k1 - sc), kw = k1 - k0, rows = k1;
    colwise_copy<kBatThreads, T>(
        rows, kw, tid, [&](int r, int c) { return A[(size_t)r + (size_t)(k0 + c) * lda]; },
        [&](int r, int c, T v) { Lc[c * rows + r] = v; });
    __syncthreads();
    if (warp < nrhs) {
      T* __restrict__ x = Bs + warp * kBatMaxN;
      for (int c = kw - 1; c >= 0; --c) {
        const int k = k0 + c;
        const T xk = x[k] / Lc[c * rows + k];    // every lane divides the same operands
        __syncwarp();
        if (lane == 0) x[k] = xk;
        axpy_rows<EXACT>(xk, Lc + c * rows, x, lane, k);
        __syncwarp();
      }
    }
    __syncthreads();
  }
  colwise_copy<kBatThreads, T>(
      n, nrhs, tid, [&](int r, int q) { return Bs[q * kBatMaxN + r]; },
      [&](int r, int q, T v) { B[(size_t)r + (size_t)q * ldb] = v; });
  __syncthreads();
}

template <typename T, bool EXACT>
__global__ void __launch_bounds__(bat_threads<T>(), bat_ctas_per_sm<T>())
batched_gesv_kernel(BatchArgs<T> a) {
  extern __shared__ __align__(16) unsigned char bat_smem[];
  __shared__ int sys_s;
  BatPhaseClock clk(a.phase);
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
    clk.mark(kBatPhQueue);
    batched_getrf_one<T, EXACT>(n, a.A[s], a.lda[s], a.ipiv[s], a.info + s, nb, a.cap, bat_smem, clk);
    __syncthreads();
    if (a.solve && a.info[s] == 0 && a.nrhs[s] > 0)
      batched_getrs_one<T, EXACT>(n, min(a.nrhs[s], kBatMaxRhs), a.A[s], a.lda[s], a.ipiv[s], a.B[s], a.ldb[s],
                                  bat_smem, a.cap);
    clk.mark(kBatPhSolve);
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
