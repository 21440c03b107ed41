// Kernels of the blocked LU factorization and of the solves, templated on
// the element type (double for the D routines, float for the S routines).
#pragma once
#include "common.cuh"

namespace gb {

constexpr int kPanelThreads = 256;
constexpr int kLeafMax = 64;      // widest panel the cooperative leaf kernel factors

// Global scratch of one leaf-panel launch (sized for G CTAs and JB <= 64).
template <typename T>
struct PanelScratch {
  Cand<T>* cand;       // [2][G]
  int* cand_label;     // [2][G]
  T* cand_row;         // [2][G][kLeafMax]
  T* row_k;            // [2][kLeafMax]
  int* row_k_label;    // [2]
  unsigned* counter;   // grid-barrier counter, zeroed before the launch
  int* pair_dst;       // [2*kLeafMax] global 0-based destination rows
  int* pair_src;       // [2*kLeafMax] global 0-based source rows
  int* pair_count;     // number of valid pairs
};

// Leaf panel factorization, DGETRF2 semantics (SRC/dgetrf2.f:170-265) on an
// M x JB panel (JB <= 64) whose top-left element is row `row0` of the
// matrix.  The panel is spread over the co-resident CTAs of a cooperative
// grid, R consecutive rows per CTA held in shared memory.  For each column:
// every CTA finds its best candidate (IDAMAX order), publishes it together
// with its whole row, one grid barrier, then every CTA picks the same winner,
// swaps, scales (reciprocal when |pivot| >= sfmin, else divides) and applies
// the rank-1 update to its rows.  The interchanges of whole panel rows are
// summarised at the end as (dst, src) row pairs for the other columns.
template <typename T, bool EXACT>
__global__ void __launch_bounds__(kPanelThreads)
leaf_panel_kernel(T* __restrict__ P, int lda, int M, int JB, int R, int row0,
                  int* __restrict__ ipiv, int* __restrict__ info, PanelScratch<T> w,
                  int* __restrict__ status) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* tile = reinterpret_cast<T*>(smem_raw);                       // [JB][R]
  int* label = reinterpret_cast<int*>(tile + (size_t)JB * R);     // [R]
  __shared__ T urow[kLeafMax];
  __shared__ Cand<T> red[kPanelThreads / 32];
  __shared__ int redw[kPanelThreads / 32];
  __shared__ Cand<T> win_s;
  __shared__ int win_cta_s;

  const int G = gridDim.x, b = blockIdx.x, tid = threadIdx.x;
  const int lane = tid & 31, warp = tid >> 5;
  const int rbeg = b * R;
  const int nrows = max(0, min(M, rbeg + R) - rbeg);

  for (int e = tid; e < JB * nrows; e += kPanelThreads) {
    int c = e / nrows, r = e - c * nrows;
    tile[c * R + r] = P[(size_t)(rbeg + r) + (size_t)c * lda];
  }
  for (int r = tid; r < nrows; r += kPanelThreads) label[r] = rbeg + r;
  __syncthreads();

  bool ok = true;
  for (int k = 0; k < JB && ok; ++k) {
    const int par = k & 1;
    // 1. local candidate among owned rows >= k
    Cand<T> best;
    best.absval = 0; best.row = -1; best.cls = -1;
    for (int r = tid; r < nrows; r += kPanelThreads) {
      int g = rbeg + r;
      if (g >= k) {
        Cand<T> c = make_cand(tile[k * R + r], g, k);
        if (cand_better(c, best)) best = c;
      }
    }
    best = warp_best(best);
    if (lane == 0) red[warp] = best;
    __syncthreads();
    if (warp == 0) {
      Cand<T> c = (lane < kPanelThreads / 32) ? red[lane] : Cand<T>{0, -1, -1};
      c = warp_best(c);
      if (lane == 0) {
        win_s = c;
        w.cand[par * G + b] = c;
      }
    }
    __syncthreads();
    if (win_s.row >= 0) {
      int lr = win_s.row - rbeg;
      for (int c = tid; c < JB; c += kPanelThreads) w.cand_row[((size_t)par * G + b) * kLeafMax + c] = tile[c * R + lr];
      if (tid == 0) w.cand_label[par * G + b] = label[lr];
    }
    if (k >= rbeg && k < rbeg + nrows) {
      int lk = k - rbeg;
      for (int c = tid; c < JB; c += kPanelThreads) w.row_k[par * kLeafMax + c] = tile[c * R + lk];
      if (tid == 0) w.row_k_label[par] = label[lk];
    }
    // 2. one grid barrier per column
    ok = grid_barrier(w.counter, (unsigned)k, status);
    if (!ok) break;
    // 3. every CTA reduces the same G candidates to the same winner
    Cand<T> cb;
    cb.absval = 0; cb.row = -1; cb.cls = -1;
    int cw = -1;
    for (int g = tid; g < G; g += kPanelThreads) {
      Cand<T> cc;
      cc.absval = ldcg(&w.cand[par * G + g].absval);
      cc.row = ldcg(&w.cand[par * G + g].row);
      cc.cls = ldcg(&w.cand[par * G + g].cls);
      if (cc.row >= 0 && (cw < 0 || cand_better(cc, cb))) { cb = cc; cw = g; }
    }
    // warp reduction carrying the CTA index
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
      Cand<T> o = shfl_cand(cb, off);
      int ow = __shfl_xor_sync(0xffffffffu, cw, off);
      if (ow >= 0 && (cw < 0 || cand_better(o, cb))) { cb = o; cw = ow; }
    }
    if (lane == 0) { red[warp] = cb; redw[warp] = cw; }
    __syncthreads();
    if (warp == 0) {
      Cand<T> c = (lane < kPanelThreads / 32) ? red[lane] : Cand<T>{0, -1, -1};
      int cwi = (lane < kPanelThreads / 32) ? redw[lane] : -1;
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) {
        Cand<T> o = shfl_cand(c, off);
        int ow = __shfl_xor_sync(0xffffffffu, cwi, off);
        if (ow >= 0 && (cwi < 0 || cand_better(o, c))) { c = o; cwi = ow; }
      }
      if (lane == 0) { win_s = c; win_cta_s = cwi; }
    }
    __syncthreads();
    const int wcta = win_cta_s;
    const int prow = win_s.row;
    const T* wrow = w.cand_row + ((size_t)par * G + wcta) * kLeafMax;
    for (int c = tid; c < JB; c += kPanelThreads) urow[c] = ldcg(wrow + c);
    __syncthreads();
    const T pv = urow[k];
    if (b == 0 && tid == 0) {
      ipiv[k] = row0 + prow + 1;
      if (pv == T(0) && *info == 0) *info = row0 + k + 1;
    }
    // 4. interchange rows k and prow (whole panel rows)
    if (prow != k) {
      if (k >= rbeg && k < rbeg + nrows) {
        int lk = k - rbeg;
        for (int c = tid; c < JB; c += kPanelThreads) tile[c * R + lk] = urow[c];
        if (tid == 0) label[lk] = ldcg(w.cand_label + par * G + wcta);
      }
      if (prow >= rbeg && prow < rbeg + nrows) {
        int lp = prow - rbeg;
        const T* rk = w.row_k + par * kLeafMax;
        for (int c = tid; c < JB; c += kPanelThreads) tile[c * R + lp] = ldcg(rk + c);
        if (tid == 0) label[lp] = ldcg(w.row_k_label + par);
      }
    }
    __syncthreads();
    // 5. scale the column below the pivot and update the rest of the panel
    if (pv != T(0)) {
      const bool recip = (pv < 0 ? -pv : pv) >= Lim<T>::sfmin();
      const T rp = T(1) / pv;
      const int r0 = max(0, k + 1 - rbeg);
      for (int r = r0 + tid; r < nrows; r += kPanelThreads) {
        T v = tile[k * R + r];
        tile[k * R + r] = recip ? v * rp : v / pv;
      }
    }
    __syncthreads();
    {
      const int r0 = max(0, k + 1 - rbeg);
      const int nr = nrows - r0;
      const int nc = JB - k - 1;
      if (nr > 0 && nc > 0) {
        for (int e = tid; e < nr * nc; e += kPanelThreads) {
          int cc = e / nr, r = r0 + (e - cc * nr);
          int c = k + 1 + cc;
          tile[c * R + r] = fnmadd<EXACT>(tile[k * R + r], urow[c], tile[c * R + r]);
        }
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
                   const int* __restrict__ pair_count_ext, int ntop) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  const int nleft = c_skip0, nright = ncols - c_skip1;
  if (warp >= nleft + nright) return;
  const int col = warp < nleft ? warp : c_skip1 + (warp - nleft);
  const int np = ntop + *pair_count_ext;
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

// B := L^{-1} B for a unit lower triangular L (k x k, k <= 64) and B of k
// rows; one CTA per slab of BC columns of B (BC = 64 for float, 16 for
// double, keeping static shared memory under 48 KB).  Forward substitution
// in the reference order (BLAS/SRC/dtrsm.f:290-300): for each k, rows below
// k get B(i,j) - B(k,j)*A(i,k).
template <typename T>
struct TrsmSlab { static constexpr int BC = sizeof(T) == 8 ? 16 : 64; };

template <typename T, bool EXACT>
__global__ void __launch_bounds__(256)
trsm_llnu_leaf_kernel(const T* __restrict__ L, int ldl, T* __restrict__ B, int ldb, int k, int ncols) {
  constexpr int BC = TrsmSlab<T>::BC;
  constexpr int RG = 256 / BC;              // row groups
  __shared__ T Ls[kLeafMax][kLeafMax];
  __shared__ T Bs[kLeafMax][BC + 1];
  const int tid = threadIdx.x;
  const int c0 = blockIdx.x * BC;
  const int nc = min(BC, ncols - c0);
  for (int e = tid; e < k * k; e += 256) {
    int c = e / k, r = e - c * k;
    Ls[r][c] = L[(size_t)r + (size_t)c * ldl];
  }
  for (int e = tid; e < k * nc; e += 256) {
    int c = e / k, r = e - c * k;
    Bs[r][c] = B[(size_t)r + (size_t)(c0 + c) * ldb];
  }
  __syncthreads();
  const int c = tid % BC;
  const int rq = tid / BC;
  for (int kk = 0; kk < k - 1; ++kk) {
    if (c < nc) {
      T bk = Bs[kk][c];
      for (int r = kk + 1 + rq; r < k; r += RG) Bs[r][c] = fnmadd<EXACT>(bk, Ls[r][kk], Bs[r][c]);
    }
    __syncthreads();
  }
  for (int e = tid; e < k * nc; e += 256) {
    int cc = e / k, r = e - cc * k;
    B[(size_t)r + (size_t)(c0 + cc) * ldb] = Bs[r][cc];
  }
}

}  // namespace gb
