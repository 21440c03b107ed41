// Kernels of the blocked LU factorization and of the solves, templated on
// the element type (double for the D routines, float for the S routines).
#pragma once
#include "common.cuh"

namespace gb {

constexpr int kPanelThreads = 256;
constexpr int kLeafMax = 64;      // widest panel the cooperative leaf kernel factors

// Global scratch of one leaf-panel launch (sized for G CTAs and JB <= 64).
// Per column k, CTA g publishes its pivot candidate in word[k&1][g]: the
// upper 32 bits an order-preserving key of the candidate (see cand_key), the
// lower 32 bits its row (25 bits) and the column sequence number k+1
// (7 bits).  For double the key cannot hold |a| exactly, so |a| itself goes
// to absval[k&1][g] before the word is released.  Readers poll the words
// (acquire) until every sequence number reads k+1: that poll is both the
// grid barrier and the candidate exchange.
template <typename T>
struct PanelScratch {
  unsigned long long* word;   // [2][G], zeroed before the launch
  T* absval;                  // [2][G]   (double only)
  int* cand_label;            // [2][G]
  T* cand_row;                // [2][G][kLeafMax]
  T* row_k;                   // [2][kLeafMax]
  int* row_k_label;           // [2]
  int* pair_dst;              // [2*kLeafMax] global 0-based destination rows
  int* pair_src;              // [2*kLeafMax] global 0-based source rows
  int* pair_count;            // number of valid pairs beyond the JB top rows, zeroed before the launch
};

// 32-bit key, larger is better, that orders candidates as cand_better does
// on class and |value| (row ties are broken separately): 0 = NaN elsewhere,
// 1 + bits(|v|) for an ordinary value (float; for double the high word of
// |v|, refined by absval), 0xFFFFFFFF = leading NaN.
template <typename T>
__device__ __forceinline__ unsigned cand_key(const Cand<T>& c) {
  if (c.cls == 2) return 0xFFFFFFFFu;
  if (c.cls <= 0) return 0u;
  if constexpr (sizeof(T) == 4) return __float_as_uint((float)c.absval) + 1u;
  else return (unsigned)(__double_as_longlong((double)c.absval) >> 32) + 1u;
}

// Copies JB <= 64 elements with 16-byte accesses (all loads issued before
// the stores); both pointers 16-byte aligned, the tail past JB is copied too
// (the buffers hold kLeafMax elements).
template <typename T, bool SRC_GLOBAL_CG>
__device__ __forceinline__ void copy_row64(T* __restrict__ dst, const T* __restrict__ src) {
  constexpr int NV = kLeafMax * (int)sizeof(T) / 16;
  const uint4* s4 = reinterpret_cast<const uint4*>(src);
  uint4* d4 = reinterpret_cast<uint4*>(dst);
  uint4 v[NV];
#pragma unroll
  for (int i = 0; i < NV; ++i) v[i] = SRC_GLOBAL_CG ? __ldcg(s4 + i) : s4[i];
#pragma unroll
  for (int i = 0; i < NV; ++i) d4[i] = v[i];
}

__device__ __forceinline__ void st_release_u64(unsigned long long* p, unsigned long long v) {
  asm volatile("st.release.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ unsigned long long ld_acquire_u64(const unsigned long long* p) {
  unsigned long long v;
  asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}

// Leaf panel factorization, DGETRF2 semantics (SRC/dgetrf2.f:170-265) on an
// M x JB panel (JB <= 64) whose top-left element is row `row0` of the
// matrix.  The panel is spread over the co-resident CTAs of a cooperative
// grid, R consecutive rows per CTA held in shared memory (column-major tile).
// Per column k, warp 0 of every CTA finds the CTA's best candidate among its
// rows >= k (IDAMAX order), publishes it with its whole row, passes the grid
// barrier, reduces the G published candidates to the same winner, fetches
// the winning row and performs the row interchange in shared memory; then
// all threads scale the column below the pivot (reciprocal when
// |pivot| >= sfmin, else division) and apply the rank-1 update to the rest of
// their rows.  Two block-wide barriers per column.  The interchanges of
// whole panel rows are summarised at the end as (dst, src) row pairs.
template <typename T, bool EXACT>
__global__ void __launch_bounds__(kPanelThreads)
leaf_panel_kernel(T* __restrict__ P, int lda, int M, int JB, int R, int row0,
                  int* __restrict__ ipiv, int* __restrict__ info, PanelScratch<T> w,
                  int* __restrict__ status) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* tile = reinterpret_cast<T*>(smem_raw);                       // [JB][R]
  int* label = reinterpret_cast<int*>(tile + (size_t)JB * R);     // [R]
  __shared__ __align__(16) T urow[kLeafMax];
  __shared__ __align__(16) T rowk_s[kLeafMax];
  __shared__ __align__(16) T stage_c[kLeafMax];
  __shared__ __align__(16) T stage_k[kLeafMax];
  __shared__ int win_label_s, rowk_label_s;
  __shared__ T pv_s;
  __shared__ int ok_s;

  const int G = gridDim.x, b = blockIdx.x, tid = threadIdx.x;
  const int lane = tid & 31, warp = tid >> 5;
  const int rbeg = b * R;
  const int nrows = max(0, min(M, rbeg + R) - rbeg);

  if (nrows > 0)
    batched_copy<8, kPanelThreads, T>(
        JB * nrows, tid,
        [&](int e) { const int c = e / nrows, r = e - c * nrows; return P[(size_t)(rbeg + r) + (size_t)c * lda]; },
        [&](int e, T v) { const int c = e / nrows, r = e - c * nrows; tile[c * R + r] = v; });
  for (int r = tid; r < nrows; r += kPanelThreads) label[r] = rbeg + r;
  if (tid == 0) ok_s = 1;
  __syncthreads();

  for (int k = 0; k < JB; ++k) {
    const int par = k & 1;
    if (warp == 0) {
      // 1. the CTA's candidate among its rows >= k
      Cand<T> best;
      best.absval = 0; best.row = -1; best.cls = -1;
      for (int r = max(0, k - rbeg) + lane; r < nrows; r += 32) {
        Cand<T> c = make_cand(tile[k * R + r], rbeg + r, k);
        if (cand_better(c, best)) best = c;
      }
      best = warp_best(best);
      const bool own_k = (k >= rbeg && k < rbeg + nrows);
      const unsigned seq = (unsigned)(k + 1);
      // 2. lane 0 alone writes what this CTA publishes for column k (its
      //    candidate row, row k if it owns it) and then releases the word
      // the warp gathers the rows from the column-major tile into staging
      if (best.row >= 0)
        for (int c = lane; c < kLeafMax; c += 32) stage_c[c] = c < JB ? tile[c * R + (best.row - rbeg)] : T(0);
      if (own_k)
        for (int c = lane; c < kLeafMax; c += 32) stage_k[c] = c < JB ? tile[c * R + (k - rbeg)] : T(0);
      __syncwarp();
      if (lane == 0) {
        if (best.row >= 0) {
          copy_row64<T, false>(w.cand_row + ((size_t)par * G + b) * kLeafMax, stage_c);
          w.cand_label[par * G + b] = label[best.row - rbeg];
        }
        if (own_k) {
          copy_row64<T, false>(w.row_k + par * kLeafMax, stage_k);
          w.row_k_label[par] = label[k - rbeg];
        }
        if constexpr (sizeof(T) == 8) w.absval[par * G + b] = best.absval;
        const unsigned rowbits = (unsigned)(best.row < 0 ? 0x1FFFFFF : best.row) & 0x1FFFFFFu;
        const unsigned long long wv =
            ((unsigned long long)cand_key(best) << 32) | ((unsigned long long)rowbits << 7) | (unsigned long long)seq;
        st_release_u64(w.word + par * G + b, wv);
      }
      // 3. poll every CTA's word for this column (lane L acquires CTAs L,
      //    L+32, ...): the poll is the grid barrier and the candidate exchange
      Cand<T> cb;
      cb.absval = 0; cb.row = -1; cb.cls = -1;
      int cw = -1;
      int okb = 1;
      for (int g = lane; g < G; g += 32) {
        unsigned long long wv = 0;
        unsigned spins = 0;
        for (;;) {
          wv = ld_acquire_u64(w.word + par * G + g);
          if ((unsigned)(wv & 0x7Fu) == seq) break;
          if (++spins > kSpinLimit || *(volatile int*)status != kStatusOk) {
            atomicCAS(status, kStatusOk, kStatusBarrierTimeout);
            okb = 0;
            break;
          }
        }
        if (!okb) break;
        const unsigned key = (unsigned)(wv >> 32);
        const int row = (int)((wv >> 7) & 0x1FFFFFFu);
        if (row == 0x1FFFFFF) continue;            // that CTA has no rows >= k
        Cand<T> cc;
        cc.row = row;
        if (key == 0xFFFFFFFFu) { cc.cls = 2; cc.absval = 0; }
        else if (key == 0u) { cc.cls = 0; cc.absval = 0; }
        else {
          cc.cls = 1;
          if constexpr (sizeof(T) == 4) cc.absval = __uint_as_float(key - 1u);
          else cc.absval = ldcg(w.absval + par * G + g);
        }
        if (cw < 0 || cand_better(cc, cb)) { cb = cc; cw = g; }
      }
      okb = __all_sync(0xffffffffu, okb);
      if (!okb) {
        if (lane == 0) ok_s = 0;
      } else {
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
          Cand<T> o = shfl_cand(cb, off);
          int ow = __shfl_xor_sync(0xffffffffu, cw, off);
          if (ow >= 0 && (cw < 0 || cand_better(o, cb))) { cb = o; cw = ow; }
        }
        const int prow = cb.row;
        const int kown = k / R;                      // CTA holding row k
        // 4. the lane that acquired the winner's word reads its row; the lane
        //    that acquired row k's owner reads row k (needed by the CTA that
        //    holds the pivot row)
        if (lane == (cw & 31)) {
          copy_row64<T, true>(urow, w.cand_row + ((size_t)par * G + cw) * kLeafMax);
          win_label_s = ldcg(w.cand_label + par * G + cw);
        }
        const bool own_p = (prow >= rbeg && prow < rbeg + nrows);
        if (own_p && prow != k && lane == (kown & 31)) {
          copy_row64<T, true>(rowk_s, w.row_k + par * kLeafMax);
          rowk_label_s = ldcg(w.row_k_label + par);
        }
        __syncwarp();
        const T pv = urow[k];
        if (lane == 0) {
          pv_s = pv;
          if (b == 0) {
            ipiv[k] = row0 + prow + 1;
            if (pv == T(0) && *info == 0) *info = row0 + k + 1;
          }
        }
        // 5. interchange rows k and prow (whole panel rows)
        if (prow != k) {
          if (own_k) {
            const int lk = k - rbeg;
            for (int c = lane; c < JB; c += 32) tile[c * R + lk] = urow[c];
            if (lane == 0) label[lk] = win_label_s;
          }
          if (own_p) {
            const int lp = prow - rbeg;
            for (int c = lane; c < JB; c += 32) tile[c * R + lp] = rowk_s[c];
            if (lane == 0) label[lp] = rowk_label_s;
          }
        }
      }
    }
    __syncthreads();
    if (!ok_s) break;
    // 5. scale the column below the pivot and update the rest of each row
    const T pv = pv_s;
    if (pv != T(0)) {
      const bool recip = (pv < 0 ? -pv : pv) >= Lim<T>::sfmin();
      const T rp = T(1) / pv;
      for (int r = max(0, k + 1 - rbeg) + tid; r < nrows; r += kPanelThreads) {
        const T v = tile[k * R + r];
        const T l = recip ? v * rp : v / pv;
        tile[k * R + r] = l;
        for (int c = k + 1; c < JB; ++c) tile[c * R + r] = fnmadd<EXACT>(l, urow[c], tile[c * R + r]);
      }
    } else {
      // zero pivot: the column stays unscaled; the update uses it as is
      for (int r = max(0, k + 1 - rbeg) + tid; r < nrows; r += kPanelThreads) {
        const T l = tile[k * R + r];
        for (int c = k + 1; c < JB; ++c) tile[c * R + r] = fnmadd<EXACT>(l, urow[c], tile[c * R + r]);
      }
    }
    __syncthreads();
  }
  // write the factored rows back and summarise the interchanges
  for (int e = tid; e < JB * nrows; e += kPanelThreads) {
    int c = e / nrows, r = e - c * nrows;
    P[(size_t)(rbeg + r) + (size_t)c * lda] = tile[c * R + r];
  }
  for (int r = tid; r < nrows; r += kPanelThreads) {
    int g = rbeg + r;
    if (g < JB) {
      w.pair_dst[g] = row0 + g;
      w.pair_src[g] = row0 + label[r];
    } else if (label[r] != g) {
      int slot = JB + atomicAdd(w.pair_count, 1);
      if (slot < 2 * kLeafMax) {
        w.pair_dst[slot] = row0 + g;
        w.pair_src[slot] = row0 + label[r];
      } else {
        atomicCAS(status, kStatusOk, kStatusCapacity);
      }
    }
  }
}

// Applies a leaf's row interchanges, given as (dst, src) pairs, to the
// columns [0, c_skip0) and [c_skip1, ncols): every column reads all its
// source elements before writing any destination (a permutation applied as
// a gather).  One warp per column.
template <typename T>
__global__ void __launch_bounds__(256)
laswp_pairs_kernel(T* __restrict__ A, int lda, int ncols, int c_skip0, int c_skip1,
                   const int* __restrict__ pair_dst, const int* __restrict__ pair_src,
                   const int* __restrict__ pair_count_ext, int ntop, int* __restrict__ perm) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  const int nleft = c_skip0, nright = ncols - c_skip1;
  const int np = ntop + *pair_count_ext;
  if (perm && warp == nleft + nright) {
    // the same gather on the running row permutation of the factorization
    constexpr int kMaxPer = (2 * kLeafMax + 31) / 32;
    int v[kMaxPer];
#pragma unroll
    for (int s = 0; s < kMaxPer; ++s) {
      int i = lane + 32 * s;
      if (i < np) v[s] = perm[pair_src[i]];
    }
    __syncwarp();
#pragma unroll
    for (int s = 0; s < kMaxPer; ++s) {
      int i = lane + 32 * s;
      if (i < np) perm[pair_dst[i]] = v[s];
    }
    return;
  }
  if (warp >= nleft + nright) return;
  const int col = warp < nleft ? warp : c_skip1 + (warp - nleft);
  T* Ac = A + (size_t)col * lda;
  constexpr int kMaxPer = (2 * kLeafMax + 31) / 32;
  T v[kMaxPer];
#pragma unroll
  for (int s = 0; s < kMaxPer; ++s) {
    int i = lane + 32 * s;
    if (i < np) v[s] = Ac[pair_src[i]];
  }
  __syncwarp();
#pragma unroll
  for (int s = 0; s < kMaxPer; ++s) {
    int i = lane + 32 * s;
    if (i < np) Ac[pair_dst[i]] = v[s];
  }
}

// Row interchanges of a whole block column, kept as the ordered list of its
// leaves' (dst, src) pair lists, replayed later on the columns outside the
// block column.  This is the DLASWP of SRC/dgetrf.f:193 (columns left of
// the panel) and SRC/dgetrf.f:199 (columns right of it), deferred so that
// the next panel can be factored while those columns are still being
// updated.  Slot s holds ntop[s] + counts[s] pairs at dst/src + s*2*kLeafMax.
constexpr int kMaxLogSlots = 64;

struct PairLogArgs {
  int nslots;
  int ntop[kMaxLogSlots];
};

// Replays the logged pair lists, in order, on the columns [a0, a1) and
// [b0, b1) (one warp per column) and, when perm is given, on the running
// row permutation (one extra warp).
template <typename T>
__global__ void __launch_bounds__(256)
laswp_log_kernel(T* __restrict__ A, int lda, int a0, int a1, int b0, int b1, const int* __restrict__ log_dst,
                 const int* __restrict__ log_src, const int* __restrict__ counts, PairLogArgs la,
                 int* __restrict__ perm) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  const int na = a1 - a0, nbc = b1 - b0;
  constexpr int kMaxPer = (2 * kLeafMax + 31) / 32;
  if (perm && warp == na + nbc) {
    for (int s = 0; s < la.nslots; ++s) {
      const int* dst = log_dst + (size_t)s * 2 * kLeafMax;
      const int* src = log_src + (size_t)s * 2 * kLeafMax;
      const int np = min(la.ntop[s] + counts[s], 2 * kLeafMax);
      int v[kMaxPer];
#pragma unroll
      for (int q = 0; q < kMaxPer; ++q) {
        int i = lane + 32 * q;
        if (i < np) v[q] = perm[src[i]];
      }
      __syncwarp();
#pragma unroll
      for (int q = 0; q < kMaxPer; ++q) {
        int i = lane + 32 * q;
        if (i < np) perm[dst[i]] = v[q];
      }
      __syncwarp();
    }
    return;
  }
  if (warp >= na + nbc) return;
  const int col = warp < na ? a0 + warp : b0 + (warp - na);
  T* Ac = A + (size_t)col * lda;
  for (int s = 0; s < la.nslots; ++s) {
    const int* dst = log_dst + (size_t)s * 2 * kLeafMax;
    const int* src = log_src + (size_t)s * 2 * kLeafMax;
    const int np = min(la.ntop[s] + counts[s], 2 * kLeafMax);
    T v[kMaxPer];
#pragma unroll
    for (int q = 0; q < kMaxPer; ++q) {
      int i = lane + 32 * q;
      if (i < np) v[q] = Ac[src[i]];
    }
    __syncwarp();
#pragma unroll
    for (int q = 0; q < kMaxPer; ++q) {
      int i = lane + 32 * q;
      if (i < np) Ac[dst[i]] = v[q];
    }
    __syncwarp();
  }
}

// Forward substitution X := L^{-1} X for a unit lower triangular L (k x k)
// and nc columns of X kept column-major in shared memory (element (i, c) at
// X[c * ldx + i], ldx a multiple of 16 bytes, rows allocated up to k
// rounded up to 8), LPC adjacent lanes per column, in blocks of 8 rows.
// Lane `sub` of a column owns the row blocks I with I % LPC == sub; at step
// J the owner of block J solves its 8 x 8 diagonal block in registers, and
// after a warp barrier every lane subtracts L(I, J) x_J from each of its
// blocks I > J.  Blocks of X and columns of L (Lt[j * ldt + i] = L(i, j),
// ldt a multiple of 8) move in 16-byte vectors.  The loops over the blocks
// are real loops: their unrolled bodies are a few hundred instructions
// that stay in the instruction cache (a fully unrolled 64-row solve is
// thousands of straight-line instructions fetched once per launch, which
// cost more than the arithmetic).  Per element the updates run in
// increasing j, x_i := x_i - x_j * L(i, j), the order of
// BLAS/SRC/dtrsm.f:290-300.  Rows i >= k of the padded blocks hold whatever
// shared memory holds and are never stored.  Every thread of the block
// calls this (tid < LPC * ncolumns-per-block); lanes of columns >= nc only
// keep the warp barriers.
template <typename T>
__device__ __forceinline__ void ld8_shared(const T* __restrict__ p, T (&v)[8]) {
  if constexpr (sizeof(T) == 4) {
    const float4 a = reinterpret_cast<const float4*>(p)[0], b = reinterpret_cast<const float4*>(p)[1];
    v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w; v[4] = b.x; v[5] = b.y; v[6] = b.z; v[7] = b.w;
  } else {
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const double2 q = reinterpret_cast<const double2*>(p)[u];
      v[2 * u] = q.x;
      v[2 * u + 1] = q.y;
    }
  }
}
template <typename T>
__device__ __forceinline__ void st8_shared(T* __restrict__ p, const T (&v)[8]) {
  if constexpr (sizeof(T) == 4) {
    reinterpret_cast<float4*>(p)[0] = make_float4(v[0], v[1], v[2], v[3]);
    reinterpret_cast<float4*>(p)[1] = make_float4(v[4], v[5], v[6], v[7]);
  } else {
#pragma unroll
    for (int u = 0; u < 4; ++u) reinterpret_cast<double2*>(p)[u] = make_double2(v[2 * u], v[2 * u + 1]);
  }
}

template <typename T, bool EXACT, int LPC>
__device__ __forceinline__ void solve_unit_lower_cols(const T* __restrict__ Lt, int ldt, T* __restrict__ X, int ldx,
                                                      int k, int nc, int tid) {
  static_assert(LPC == 4 || LPC == 8 || LPC == 16, "lanes per column: 4, 8 or 16");
  const int col = tid / LPC, sub = tid % LPC;
  const bool act = col < nc;
  const int nblk = (k + 7) / 8;
  T* xc = X + (size_t)(act ? col : 0) * ldx;
  for (int J = 0; J < nblk; ++J) {
    const int j0 = 8 * J;
    T xj[8];
    if (act && J % LPC == sub) {
      // the diagonal block
      ld8_shared<T>(xc + j0, xj);
#pragma unroll
      for (int jj = 0; jj < 7; ++jj) {
        T l[8];
        ld8_shared<T>(Lt + (size_t)(j0 + jj) * ldt + j0, l);
#pragma unroll
        for (int ii = jj + 1; ii < 8; ++ii) xj[ii] = fnmadd<EXACT>(xj[jj], l[ii], xj[ii]);
      }
      st8_shared<T>(xc + j0, xj);
    }
    __syncwarp();
    if (act) {
      ld8_shared<T>(xc + j0, xj);
      // this lane's blocks below J: the first I > J with I % LPC == sub
      for (int I = J + 1 + ((sub - J - 1) & (LPC - 1)); I < nblk; I += LPC) {
        const int i0 = 8 * I;
        T xi[8];
        ld8_shared<T>(xc + i0, xi);
#pragma unroll
        for (int jj = 0; jj < 8; ++jj) {
          T l[8];
          ld8_shared<T>(Lt + (size_t)(j0 + jj) * ldt + i0, l);
#pragma unroll
          for (int ii = 0; ii < 8; ++ii) xi[ii] = fnmadd<EXACT>(xj[jj], l[ii], xi[ii]);
        }
        st8_shared<T>(xc + i0, xi);
      }
    }
    __syncwarp();
  }
}

// Leading dimensions of the staged blocks: L by columns (k rounded up to
// 8) and the columns of X, padded by 16 bytes so that neighbouring columns
// start in different banks.
__host__ __device__ constexpr int trsm_ldt(int k) { return (k + 7) / 8 * 8; }
template <typename T>
__host__ __device__ constexpr int trsm_ldx(int k) { return trsm_ldt(k) + 16 / (int)sizeof(T); }

// B := L^{-1} B for a unit lower triangular L (k x k, k <= kTrsmLeafMax)
// and B of k rows (the panel's U12 = L11^{-1} A12, SRC/dgetrf2.f:240): L
// and this CTA's 256 / LPC columns of B are staged in shared memory by
// cp.async, then solved LPC lanes per column (solve_unit_lower_cols).
// More lanes per column for taller L: more warps share the k-step chain.
constexpr int kTrsmThreads = 256;
constexpr int kTrsmLeafMax = 128;

template <typename T>
__host__ __device__ constexpr int trsm_leaf_smem(int k, int lpc) {
  return (trsm_ldt(k) * trsm_ldt(k) + trsm_ldx<T>(k) * (kTrsmThreads / lpc)) * (int)sizeof(T);
}

template <typename T, bool EXACT, int LPC>
__global__ void __launch_bounds__(kTrsmThreads)
trsm_llnu_leaf_kernel(const T* __restrict__ L, int ldl, T* __restrict__ B, int ldb, int k, int ncols) {
  constexpr int CPB = kTrsmThreads / LPC;                   // columns per CTA
  extern __shared__ __align__(16) unsigned char trsm_smem[];
  const int ldt = trsm_ldt(k), ldx = trsm_ldx<T>(k);
  T* Lt = reinterpret_cast<T*>(trsm_smem);                  // Lt[j * ldt + i] = L(i, j)
  T* Bs = Lt + ldt * ldt;                                   // Bs[c * ldx + i] = B(i, c0 + c)
  const int tid = threadIdx.x;
  const int c0 = blockIdx.x * CPB;
  const int nc = min(CPB, ncols - c0);
  stage_cols_async<T, kTrsmThreads>(L, ldl, k, k, Lt, ldt, tid);
  stage_cols_async<T, kTrsmThreads>(B + (size_t)c0 * ldb, ldb, k, nc, Bs, ldx, tid);
  cp_async_commit();
  cp_async_wait<0>();
  __syncthreads();
  solve_unit_lower_cols<T, EXACT, LPC>(Lt, ldt, Bs, ldx, k, nc, tid);
  __syncthreads();
  const int warp = tid >> 5, lane = tid & 31;
  for (int c = warp; c < nc; c += kTrsmThreads / 32)
    for (int r = lane; r < k; r += 32) B[(size_t)r + (size_t)(c0 + c) * ldb] = Bs[c * ldx + r];
}

// The same solve for k up to KMAX = 128 or 256 in one launch (the block
// row of U: k = NB = 256).  The strictly lower triangle of L is kept packed
// in shared memory (column j's rows j+1.. at tri_off(j); 130 KB for 256
// FP32 rows), staged with cp.async; LPC lanes share a column, lane s holding
// rows s, s+LPC, ... in registers; per k the lane holding row k broadcasts
// it and every lane updates its rows below k, in the reference order
// (BLAS/SRC/dtrsm.f:296-298).  More lanes per column shorten the chain of
// the k steps (the look-ahead's 256-column solve); fewer cost less staging
// per column (the wide solve of the rest of the block row).
template <int KMAX>
__host__ __device__ constexpr int tri_off(int j) {
  return j * (2 * KMAX - j - 1) / 2;
}

template <typename T, int KMAX, int LPC>
constexpr int trsm_tri_smem() {
  return (KMAX * (KMAX - 1) / 2 + KMAX * (kTrsmThreads / LPC + 1)) * (int)sizeof(T);
}

template <typename T, bool EXACT, int KMAX, int LPC>
__global__ void __launch_bounds__(kTrsmThreads, 1)
trsm_llnu_tri_kernel(const T* __restrict__ L, int ldl, T* __restrict__ B, int ldb, int k, int ncols) {
  constexpr int RPL = KMAX / LPC;                        // rows per lane
  constexpr int CPB = kTrsmThreads / LPC;                // columns per CTA
  constexpr int BLD = CPB + 1;
  extern __shared__ __align__(16) unsigned char trsm_smem[];
  T* Lp = reinterpret_cast<T*>(trsm_smem);
  T* Bs = Lp + KMAX * (KMAX - 1) / 2;                    // [KMAX][CPB + 1]
  const int tid = threadIdx.x, lane = tid & 31;
  const int c0 = blockIdx.x * CPB;
  const int nc = min(CPB, ncols - c0);
  for (int j = 0; j < k - 1; ++j) {
    const int off = tri_off<KMAX>(j);
    for (int i = j + 1 + tid; i < k; i += kTrsmThreads) cp_async_elem(Lp + off + (i - j - 1), L + (size_t)i + (size_t)j * ldl);
  }
  for (int e = tid; e < k * nc; e += kTrsmThreads) {
    const int c = e / k, r = e - c * k;
    cp_async_elem(Bs + r * BLD + c, B + (size_t)r + (size_t)(c0 + c) * ldb);
  }
  cp_async_commit();
  cp_async_wait<0>();
  __syncthreads();
  const int col = tid / LPC, sub = tid % LPC;
  const int gbase = lane & ~(LPC - 1);
  // sliding window: during block kb (steps kb*LPC .. kb*LPC+LPC-1) x[t]
  // holds row sub + LPC*(t + kb); the block's rows leave through x[0] when
  // the block ends.  Only one block of steps is unrolled, so the code stays
  // small enough for the instruction cache.
  T x[RPL];
#pragma unroll
  for (int t = 0; t < RPL; ++t) {
    const int i = sub + LPC * t;
    x[t] = (col < nc && i < k) ? Bs[i * BLD + col] : T(0);
  }
  for (int kb = 0; kb < RPL; ++kb) {
    const int kbase = kb * LPC;
#pragma unroll
    for (int kk = 0; kk < LPC; ++kk) {
      const int kcur = kbase + kk;
      if (kcur < k - 1) {
        const T xk = __shfl_sync(0xffffffffu, x[0], gbase | kk);
        const T* Lc = Lp + tri_off<KMAX>(kcur) - kcur - 1;   // Lc[i] = L(i, kcur) for i > kcur
#pragma unroll
        for (int t = 0; t < RPL; ++t) {
          const int i = sub + LPC * (t + kb);
          if (i > kcur && i < k) x[t] = fnmadd<EXACT>(xk, Lc[i], x[t]);
        }
      }
    }
    {
      const int i = sub + kbase;
      if (col < nc && i < k) Bs[i * BLD + col] = x[0];
    }
#pragma unroll
    for (int t = 0; t < RPL - 1; ++t) x[t] = x[t + 1];
    x[RPL - 1] = T(0);
  }
  __syncthreads();
  for (int e = tid; e < k * nc; e += kTrsmThreads) {
    const int c = e / k, r = e - c * k;
    B[(size_t)r + (size_t)(c0 + c) * ldb] = Bs[r * BLD + c];
  }
}

}  // namespace gb
