// Leaf panel factorization of the FP32 LU on one thread-block cluster.
//
// The grid-wide leaf kernel exchanges one pivot candidate per column
// through L2, which on GB300 costs a few microseconds per column (several
// dependent L2 round trips across the two dies).  Here the M x JB panel is
// spread over the CTAs of ONE cluster (16 CTAs, one per SM, all in one GPC),
// each holding R rows in shared memory; candidates, the pivot row and row k
// are exchanged through distributed shared memory with one hardware cluster
// barrier per column.  Same semantics as leaf_panel_kernel (DGETRF2 on the
// panel, SRC/dgetrf2.f:170-265): IDAMAX pivot order, reciprocal-or-divide
// scaling, rank-1 updates in increasing k, interchanges of whole panel rows
// summarised as (dst, src) pairs.
//
// Pivot order as one 64-bit key, larger wins: the upper word is cand_key
// (class and |a|), the lower word ~row, so equal |a| goes to the smaller row
// as IDAMAX's strict '>' does.  The search for column k+1 is folded into the
// rank-1 update of column k.
#pragma once
#include <cooperative_groups.h>

#include "lu_kernels.cuh"

namespace gb {

constexpr int kClusterCtas = 16;
constexpr int kClusterThreads = 512;

struct ClusterSlot {
  unsigned long long key;
  int label;
  int row_k_label;
  float row[kLeafMax];
  float row_k[kLeafMax];
};

__device__ __forceinline__ unsigned long long pack_key(float v, int row, int first_row) {
  Cand<float> c = make_cand(v, row, first_row);
  return ((unsigned long long)cand_key(c) << 32) | (unsigned long long)(0xFFFFFFFFu - (unsigned)row);
}

// Warp maximum of 64-bit keys: the maximum upper word, then the maximum
// lower word among the lanes that hold it (two redux instructions).
__device__ __forceinline__ unsigned long long warp_max_u64(unsigned long long v) {
  const unsigned hi = (unsigned)(v >> 32);
  const unsigned mhi = __reduce_max_sync(0xffffffffu, hi);
  const unsigned mlo = __reduce_max_sync(0xffffffffu, hi == mhi ? (unsigned)v : 0u);
  return ((unsigned long long)mhi << 32) | mlo;
}

// JBT: the leaf-width capacity (8, 16, 32 or 64), so the rank-1 update's
// column loop is unrolled; JB <= JBT is the actual width.
template <bool EXACT, int JBT>
__global__ void __launch_bounds__(kClusterThreads, 1)
leaf_panel_cluster_kernel(float* __restrict__ P, int lda, int M, int JB, int R, int row0, int* __restrict__ ipiv,
                          int* __restrict__ info, int* __restrict__ pair_dst, int* __restrict__ pair_src,
                          int* __restrict__ pair_count, int* __restrict__ status, int swap_a0, int swap_a1,
                          int swap_b0, int swap_b1) {
  namespace cg = cooperative_groups;
  cg::cluster_group cluster = cg::this_cluster();
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float* tile = reinterpret_cast<float*>(smem_raw);                        // [JB][R]
  int* label = reinterpret_cast<int*>(tile + (size_t)JB * R);              // [R]
  __shared__ ClusterSlot slot[2];
  __shared__ __align__(16) float urow[kLeafMax];
  __shared__ __align__(16) float rowk_s[kLeafMax];
  __shared__ unsigned long long wbest[kClusterThreads / 32];
  __shared__ float pv_s;
  __shared__ int win_label_s, rowk_label_s, prow_s;

  const int b = (int)cluster.block_rank(), G = (int)cluster.num_blocks();
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int rbeg = b * R;
  const int nrows = max(0, min(M, rbeg + R) - rbeg);

  // stage the CTA's rows: every element an asynchronous copy, all in flight
  // at once (the panel streams from L2/HBM at the SM's bandwidth)
  for (int c = 0; c < JB; ++c)
    for (int r = tid; r < nrows; r += kClusterThreads)
      cp_async_elem(tile + c * R + r, P + (size_t)(rbeg + r) + (size_t)c * lda);
  cp_async_commit();
  for (int r = tid; r < nrows; r += kClusterThreads) label[r] = rbeg + r;
  cp_async_wait<0>();
  __syncthreads();
  // candidates for column 0
  unsigned long long mykey = 0;
  for (int r = tid; r < nrows; r += kClusterThreads) {
    unsigned long long kk = pack_key(tile[r], rbeg + r, 0);
    mykey = kk > mykey ? kk : mykey;
  }

  for (int k = 0; k < JB; ++k) {
    const int par = k & 1;
    // 1. this CTA's best candidate for column k
    mykey = warp_max_u64(mykey);
    if (lane == 0) wbest[warp] = mykey;
    __syncthreads();
    if (warp == 0) {
      unsigned long long kk = lane < kClusterThreads / 32 ? wbest[lane] : 0ull;
      kk = warp_max_u64(kk);
      ClusterSlot& sl = slot[par];
      if (lane == 0) sl.key = kk;
      if (kk != 0ull) {
        const int lr = (int)(0xFFFFFFFFu - (unsigned)(kk & 0xFFFFFFFFull)) - rbeg;
        for (int c = lane; c < JB; c += 32) sl.row[c] = tile[c * R + lr];
        if (lane == 0) sl.label = label[lr];
      }
      if (k >= rbeg && k < rbeg + nrows) {
        for (int c = lane; c < JB; c += 32) sl.row_k[c] = tile[c * R + (k - rbeg)];
        if (lane == 0) sl.row_k_label = label[k - rbeg];
      }
    }
    // 2. one cluster barrier per column (release / acquire on shared::cluster)
    cluster.sync();
    // 3. every CTA reduces the G keys to the same winner and fetches rows
    if (warp == 0) {
      int prow;
      bool own_p;
      if constexpr (JBT <= 16) {
        // one round trip: lanes q and q+16 read CTA q's key, label and one half
        // each of its candidate row (and of row k, from the CTA holding it)
        constexpr int H = JBT / 2;
        const int q = lane & 15, half = lane >> 4;
        const ClusterSlot* qs = cluster.map_shared_rank(&slot[par], q < G ? q : 0);
        const bool holds_k = q == k / R;
        unsigned long long kk = 0ull;
        int qlabel = 0, klabel = 0;
        float hrow[H], hrowk[H];
        if (q < G) {
          kk = qs->key;
          qlabel = qs->label;
  #pragma unroll
          for (int j = 0; j < H; ++j) {
            const int c = half * H + j;
            hrow[j] = c < JB ? qs->row[c] : 0.0f;
          }
          if (holds_k) {
            klabel = qs->row_k_label;
  #pragma unroll
            for (int j = 0; j < H; ++j) {
              const int c = half * H + j;
              hrowk[j] = c < JB ? qs->row_k[c] : 0.0f;
            }
          }
        }
        const unsigned long long wk = warp_max_u64(kk);
        const int wc = __ffsll(__ballot_sync(0xffffffffu, kk == wk && lane < G)) - 1;   // CTA holding it
        const int prow_ = (int)(0xFFFFFFFFu - (unsigned)(wk & 0xFFFFFFFFull));
        if (q == wc) {
  #pragma unroll
          for (int j = 0; j < H; ++j) {
            const int c = half * H + j;
            if (c < JB) urow[c] = hrow[j];
          }
          if (half == 0) win_label_s = qlabel;
        }
        const bool own_p_ = (prow_ >= rbeg && prow_ < rbeg + nrows);
        if (own_p_ && prow_ != k && holds_k) {
  #pragma unroll
          for (int j = 0; j < H; ++j) {
            const int c = half * H + j;
            if (c < JB) rowk_s[c] = hrowk[j];
          }
          if (half == 0) rowk_label_s = klabel;
        }
        prow = prow_;
        own_p = own_p_;
      } else {
        // key round trip, then the winner's row (and row k for the pivot's owner)
        unsigned long long kk = 0ull;
        if (lane < G) kk = cluster.map_shared_rank(&slot[par], lane)->key;
        const unsigned long long wk = warp_max_u64(kk);
        const int wc = __ffsll(__ballot_sync(0xffffffffu, kk == wk && lane < G)) - 1;   // CTA holding it
        prow = (int)(0xFFFFFFFFu - (unsigned)(wk & 0xFFFFFFFFull));
        const ClusterSlot* ws = cluster.map_shared_rank(&slot[par], wc);
        for (int c = lane; c < JB; c += 32) urow[c] = ws->row[c];
        if (lane == 0) win_label_s = ws->label;
        own_p = (prow >= rbeg && prow < rbeg + nrows);
        if (own_p && prow != k) {
          const ClusterSlot* ks = cluster.map_shared_rank(&slot[par], k / R);
          for (int c = lane; c < JB; c += 32) rowk_s[c] = ks->row_k[c];
          if (lane == 0) rowk_label_s = ks->row_k_label;
        }
      }
      __syncwarp();
      if (lane == 0) {
        prow_s = prow;
        pv_s = urow[k];
        if (b == 0) {
          ipiv[k] = row0 + prow + 1;
          if (urow[k] == 0.0f && *info == 0) *info = row0 + k + 1;
        }
      }
      __syncwarp();
      if (prow != k) {
        if (k >= rbeg && k < rbeg + nrows) {
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
    __syncthreads();
    // 4. scale column k below the pivot, rank-1 update of each row, and the
    //    candidate search of column k+1 on the updated values
    const float pv = pv_s;
    const bool scale = pv != 0.0f;
    const bool recip = fabsf(pv) >= Lim<float>::sfmin();
    const float rp = 1.0f / pv;
    mykey = 0;
    // the panel rows and the pivot row never overlap in shared memory
    float* __restrict__ tl = tile;
    const float* __restrict__ ur = urow;
    if (R <= 2 * kClusterThreads) {
      // one or two rows per thread
      for (int r = max(0, k + 1 - rbeg) + tid; r < nrows; r += kClusterThreads) {
        const float v = tile[k * R + r];
        const float l = scale ? (recip ? v * rp : v / pv) : v;
        tile[k * R + r] = l;
        // four columns at a time: all loads before any store (the compiler
        // cannot see that rows c*R and (c+1)*R differ)
        int c = k + 1;
        for (; c + 3 < JB; c += 4) {
          float* p0 = tl + c * R + r;
          const float t0 = p0[0], t1 = p0[R], t2 = p0[2 * R], t3 = p0[3 * R];
          const float u0 = ur[c], u1 = ur[c + 1], u2 = ur[c + 2], u3 = ur[c + 3];
          const float n0 = fnmadd<EXACT>(l, u0, t0), n1 = fnmadd<EXACT>(l, u1, t1);
          const float n2 = fnmadd<EXACT>(l, u2, t2), n3 = fnmadd<EXACT>(l, u3, t3);
          p0[0] = n0;
          p0[R] = n1;
          p0[2 * R] = n2;
          p0[3 * R] = n3;
        }
        for (; c < JB; ++c) tl[c * R + r] = fnmadd<EXACT>(l, ur[c], tl[c * R + r]);
        if (k + 1 < JB) {
          unsigned long long kk = pack_key(tile[(k + 1) * R + r], rbeg + r, k + 1);
          mykey = kk > mykey ? kk : mykey;
        }
      }
      continue;
    }
    // three or more rows per thread: rows r, r+512, r+1024, r+1536 are
    // updated together, so their shared-memory read-modify-writes overlap
    for (int r0 = max(0, k + 1 - rbeg) + tid; r0 < nrows; r0 += 4 * kClusterThreads) {
      int rr[4];
      bool act[4];
      float l[4], nk[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        rr[i] = r0 + i * kClusterThreads;
        act[i] = rr[i] < nrows;
        const float v = act[i] ? tl[k * R + rr[i]] : 0.0f;
        l[i] = scale ? (recip ? v * rp : v / pv) : v;
        if (act[i]) tl[k * R + rr[i]] = l[i];
        nk[i] = 0.0f;
      }
      if (k + 1 < JB) {
        // column k+1 first: its new values are the next pivot candidates
        const float uc = ur[k + 1];
#pragma unroll
        for (int i = 0; i < 4; ++i)
          if (act[i]) {
            float* __restrict__ pc = tl + (k + 1) * R + rr[i];
            nk[i] = fnmadd<EXACT>(l[i], uc, *pc);
            *pc = nk[i];
          }
      }
#pragma unroll 2
      for (int c = k + 2; c < JB; ++c) {
        const float uc = ur[c];
#pragma unroll
        for (int i = 0; i < 4; ++i)
          if (act[i]) {
            float* __restrict__ pc = tl + c * R + rr[i];
            *pc = fnmadd<EXACT>(l[i], uc, *pc);
          }
      }
      if (k + 1 < JB) {
#pragma unroll
        for (int i = 0; i < 4; ++i)
          if (act[i]) {
            unsigned long long kk = pack_key(nk[i], rbeg + rr[i], k + 1);
            mykey = kk > mykey ? kk : mykey;
          }
      }
    }
  }
  // no CTA may exit while others can still read its shared memory
  cluster.sync();
  for (int c = 0; c < JB; ++c)
    for (int r = tid; r < nrows; r += kClusterThreads) P[(size_t)(rbeg + r) + (size_t)c * lda] = tile[c * R + r];
  for (int r = tid; r < nrows; r += kClusterThreads) {
    int g = rbeg + r;
    if (g < JB) {
      pair_dst[g] = row0 + g;
      pair_src[g] = row0 + label[r];
    } else if (label[r] != g) {
      int s = JB + atomicAdd(pair_count, 1);
      if (s < 2 * kLeafMax) {
        pair_dst[s] = row0 + g;
        pair_src[s] = row0 + label[r];
      } else {
        atomicCAS(status, kStatusOk, kStatusCapacity);
      }
    }
  }
  // The leaf's interchanges on the matrix columns [swap_a0, swap_a1) and
  // [swap_b0, swap_b1) (the rest of its block column when the other columns
  // get them later from the log): once every CTA has written its pairs, CTA
  // b's warps take columns b*16+w, +256, ...; one warp per column gathers
  // all source rows before writing any destination.
  const int na = max(0, swap_a1 - swap_a0), nb = max(0, swap_b1 - swap_b0);
  if (na + nb > 0) {
    __threadfence();
    cluster.sync();
    float* Am = P - (size_t)row0 - (size_t)row0 * lda;
    const int np = min(JB + *(volatile int*)pair_count, 2 * kLeafMax);
    constexpr int kPer = (2 * kLeafMax + 31) / 32;
    for (int idx = b * (kClusterThreads / 32) + warp; idx < na + nb; idx += G * (kClusterThreads / 32)) {
      const int col = idx < na ? swap_a0 + idx : swap_b0 + (idx - na);
      float* Ac = Am + (size_t)col * lda;
      float v[kPer];
#pragma unroll
      for (int q = 0; q < kPer; ++q) {
        const int i = lane + 32 * q;
        if (i < np) v[q] = Ac[__ldcg(pair_src + i)];
      }
      __syncwarp();
#pragma unroll
      for (int q = 0; q < kPer; ++q) {
        const int i = lane + 32 * q;
        if (i < np) Ac[__ldcg(pair_dst + i)] = v[q];
      }
    }
  }
}

}  // namespace gb

namespace gb {

// Register-resident form of the cluster leaf: each thread owns RPT rows of
// its CTA (local rows t, t+512, ...) and keeps their JB values in registers
// for the whole leaf (JB * RPT = 64), so the rank-1 updates never touch
// shared memory.  Only the published candidate row, row k and the pivot row
// travel through (distributed) shared memory.  Column indices that depend on
// k are resolved with unrolled selects so the row arrays stay in registers.
template <bool EXACT, int JB>
__global__ void __launch_bounds__(kClusterThreads, 1)
leaf_panel_cluster_reg_kernel(float* __restrict__ P, int lda, int M, int jb, int R, int row0, int* __restrict__ ipiv,
                              int* __restrict__ info, int* __restrict__ pair_dst, int* __restrict__ pair_src,
                              int* __restrict__ pair_count, int* __restrict__ status) {
  namespace cg = cooperative_groups;
  constexpr int RPT = 64 / JB;
  cg::cluster_group cluster = cg::this_cluster();
  __shared__ ClusterSlot slot[2];
  __shared__ __align__(16) float urow[kLeafMax];
  __shared__ __align__(16) float rowk_s[kLeafMax];
  __shared__ unsigned long long wbest[kClusterThreads / 32];
  __shared__ float pv_s;
  __shared__ int win_label_s, rowk_label_s, prow_s;

  const int b = (int)cluster.block_rank(), G = (int)cluster.num_blocks();
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int rbeg = b * R;
  const int nrows = max(0, min(M, rbeg + R) - rbeg);

  float a[RPT][JB];
  int lab[RPT];
#pragma unroll
  for (int i = 0; i < RPT; ++i) {
    const int r = tid + i * kClusterThreads;
    lab[i] = rbeg + r;
#pragma unroll
    for (int c = 0; c < JB; ++c) a[i][c] = (r < nrows && c < jb) ? P[(size_t)(rbeg + r) + (size_t)c * lda] : 0.0f;
  }
  unsigned long long mykey = 0;
#pragma unroll
  for (int i = 0; i < RPT; ++i) {
    const int r = tid + i * kClusterThreads;
    if (r < nrows) {
      const unsigned long long kk = pack_key(a[i][0], rbeg + r, 0);
      mykey = kk > mykey ? kk : mykey;
    }
  }

  for (int k = 0; k < jb; ++k) {
    const int par = k & 1;
    // 1. the CTA's best candidate, known to every warp
    mykey = warp_max_u64(mykey);
    if (lane == 0) wbest[warp] = mykey;
    __syncthreads();
    unsigned long long ck = lane < kClusterThreads / 32 ? wbest[lane] : 0ull;
    ck = warp_max_u64(ck);
    ClusterSlot& sl = slot[par];
    if (tid == 0) sl.key = ck;
    // the owner of that row publishes it; the owner of row k publishes row k
    const int cand_local = ck ? (int)(0xFFFFFFFFu - (unsigned)(ck & 0xFFFFFFFFull)) - rbeg : -1;
    const int k_local = (k >= rbeg && k < rbeg + nrows) ? k - rbeg : -1;
#pragma unroll
    for (int i = 0; i < RPT; ++i) {
      const int r = tid + i * kClusterThreads;
      if (r == cand_local) {
#pragma unroll
        for (int c = 0; c < JB; ++c) sl.row[c] = a[i][c];
        sl.label = lab[i];
      }
      if (r == k_local) {
#pragma unroll
        for (int c = 0; c < JB; ++c) sl.row_k[c] = a[i][c];
        sl.row_k_label = lab[i];
      }
    }
    // 2. one cluster barrier per column
    cluster.sync();
    // 3. winner and rows, fetched through distributed shared memory
    if (warp == 0) {
      unsigned long long kk = 0ull;
      if (lane < G) kk = cluster.map_shared_rank(&slot[par], lane)->key;
      const unsigned long long wk = warp_max_u64(kk);
      const int wc = __ffsll(__ballot_sync(0xffffffffu, kk == wk && lane < G)) - 1;
      const int prow = (int)(0xFFFFFFFFu - (unsigned)(wk & 0xFFFFFFFFull));
      const ClusterSlot* ws = cluster.map_shared_rank(&slot[par], wc);
      if (lane < JB) urow[lane] = ws->row[lane];
      if (lane == 0) win_label_s = ws->label;
      const bool own_p = (prow >= rbeg && prow < rbeg + nrows);
      if (own_p && prow != k) {
        const ClusterSlot* ks = cluster.map_shared_rank(&slot[par], k / R);
        if (lane < JB) rowk_s[lane] = ks->row_k[lane];
        if (lane == 0) rowk_label_s = ks->row_k_label;
      }
      __syncwarp();
      if (lane == 0) {
        prow_s = prow;
        pv_s = urow[k];
        if (b == 0) {
          ipiv[k] = row0 + prow + 1;
          if (urow[k] == 0.0f && *info == 0) *info = row0 + k + 1;
        }
      }
    }
    __syncthreads();
    // 4. interchange rows k and prow in the owners' registers
    const int prow = prow_s;
    const int p_local = (prow >= rbeg && prow < rbeg + nrows) ? prow - rbeg : -1;
    if (prow != k) {
#pragma unroll
      for (int i = 0; i < RPT; ++i) {
        const int r = tid + i * kClusterThreads;
        if (r == k_local) {
#pragma unroll
          for (int c = 0; c < JB; ++c) a[i][c] = urow[c];
          lab[i] = win_label_s;
        }
        if (r == p_local) {
#pragma unroll
          for (int c = 0; c < JB; ++c) a[i][c] = rowk_s[c];
          lab[i] = rowk_label_s;
        }
      }
    }
    // 5. scale, rank-1 update and the candidate search of column k+1
    const float pv = pv_s;
    const bool scale = pv != 0.0f;
    const bool recip = fabsf(pv) >= Lim<float>::sfmin();
    const float rp = 1.0f / pv;
    // the pivot row in registers for 16-wide leaves; 32-wide leaves read it
    // from shared memory (broadcast) to stay within 128 registers per thread
    constexpr bool kURegs = JB <= 16;
    float u[kURegs ? JB : 1];
    if constexpr (kURegs) {
#pragma unroll
      for (int c = 0; c < JB; ++c) u[c] = urow[c];
    }
    mykey = 0;
#pragma unroll
    for (int i = 0; i < RPT; ++i) {
      const int r = tid + i * kClusterThreads;
      if (r < nrows && rbeg + r > k) {
        float v = 0.0f;
#pragma unroll
        for (int c = 0; c < JB; ++c)
          if (c == k) v = a[i][c];
        const float l = scale ? (recip ? v * rp : v / pv) : v;
#pragma unroll
        for (int c = 0; c < JB; ++c) {
          if (c == k) a[i][c] = l;
          else if (c > k) a[i][c] = fnmadd<EXACT>(l, kURegs ? u[kURegs ? c : 0] : urow[c], a[i][c]);
        }
        if (k + 1 < jb) {
          float nx = 0.0f;
#pragma unroll
          for (int c = 0; c < JB; ++c)
            if (c == k + 1) nx = a[i][c];
          const unsigned long long kk = pack_key(nx, rbeg + r, k + 1);
          mykey = kk > mykey ? kk : mykey;
        }
      }
    }
  }
  // no CTA may exit while others can still read its shared memory
  cluster.sync();
#pragma unroll
  for (int i = 0; i < RPT; ++i) {
    const int r = tid + i * kClusterThreads;
    if (r < nrows) {
#pragma unroll
      for (int c = 0; c < JB; ++c)
        if (c < jb) P[(size_t)(rbeg + r) + (size_t)c * lda] = a[i][c];
      const int g = rbeg + r;
      if (g < jb) {
        pair_dst[g] = row0 + g;
        pair_src[g] = row0 + lab[i];
      } else if (lab[i] != g) {
        int s = jb + atomicAdd(pair_count, 1);
        if (s < 2 * kLeafMax) {
          pair_dst[s] = row0 + g;
          pair_src[s] = row0 + lab[i];
        } else {
          atomicCAS(status, kStatusOk, kStatusCapacity);
        }
      }
    }
  }
}

}  // namespace gb
