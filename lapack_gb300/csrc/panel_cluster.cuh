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
constexpr int kDefer = 4;   // columns whose rank-1 updates the cluster leaf applies together

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

// Step 5 of a leaf column on the CTA's tile (stride Rp, a multiple of four):
// scale column k below the pivot, bring column k+1 up to date (the next
// pivot candidates, whose best key is returned) and, every kDefer columns,
// apply the group's kDefer pending updates to the later columns; in the
// order of DGETRF2's right-looking rank-1 updates per element
// (SRC/dgetrf2.f:217-265).  Groups of four rows with 16-byte accesses; rows
// at or above k and the padding rows after the CTA's last row keep their
// values.
template <bool EXACT>
__device__ __forceinline__ unsigned long long leaf_update_quads(float* __restrict__ tl, int Rp, int k, int JB,
                                                              int rbeg, int nrows, int kfirst, int s_slot,
                                                              const float (*uh)[kLeafMax], float pv) {
  const int tid = threadIdx.x;
  const bool scale = pv != 0.0f;
  const bool recip = fabsf(pv) >= Lim<float>::sfmin();
  const float rp = 1.0f / pv;
  const bool flush = s_slot == kDefer - 1;
  unsigned long long mykey = 0;
  const int r_lo = k + 1 - rbeg;       // first local row below the diagonal
  const int nq = (nrows + 3) >> 2;
  for (int q = max(0, r_lo) / 4 + tid; q < nq; q += kClusterThreads) {
    const int r0 = 4 * q;
    bool act[4];
#pragma unroll
    for (int e = 0; e < 4; ++e) act[e] = (r0 + e >= r_lo) && (r0 + e < nrows);
    float4 v = *reinterpret_cast<const float4*>(tl + (size_t)k * Rp + r0);
    float l[4] = {v.x, v.y, v.z, v.w};
    if (scale) {
      if (recip) {
#pragma unroll
        for (int e = 0; e < 4; ++e) l[e] = act[e] ? l[e] * rp : l[e];
      } else {
#pragma unroll
        for (int e = 0; e < 4; ++e) l[e] = act[e] ? l[e] / pv : l[e];
      }
      *reinterpret_cast<float4*>(tl + (size_t)k * Rp + r0) = make_float4(l[0], l[1], l[2], l[3]);
    }
    float ld[kDefer][4];
#pragma unroll
    for (int d = 0; d < kDefer; ++d) {
      if (d < s_slot) {
        const float4 w = *reinterpret_cast<const float4*>(tl + (size_t)(kfirst + d) * Rp + r0);
        ld[d][0] = w.x; ld[d][1] = w.y; ld[d][2] = w.z; ld[d][3] = w.w;
      } else {
#pragma unroll
        for (int e = 0; e < 4; ++e) ld[d][e] = d == s_slot ? l[e] : 0.0f;
      }
    }
    if (k + 1 < JB) {
      const float4 w = *reinterpret_cast<const float4*>(tl + (size_t)(k + 1) * Rp + r0);
      float t[4] = {w.x, w.y, w.z, w.w};
#pragma unroll
      for (int d = 0; d < kDefer; ++d) {
        if (d <= s_slot) {
          const float u = uh[d][k + 1];
#pragma unroll
          for (int e = 0; e < 4; ++e) t[e] = act[e] ? fnmadd<EXACT>(ld[d][e], u, t[e]) : t[e];
        }
      }
      *reinterpret_cast<float4*>(tl + (size_t)(k + 1) * Rp + r0) = make_float4(t[0], t[1], t[2], t[3]);
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        if (act[e]) {
          const unsigned long long kk = pack_key(t[e], rbeg + r0 + e, k + 1);
          mykey = kk > mykey ? kk : mykey;
        }
      }
    }
    if (flush) {
#pragma unroll 4
      for (int c = k + 2; c < JB; ++c) {
        float* pc = tl + (size_t)c * Rp + r0;
        const float4 w = *reinterpret_cast<const float4*>(pc);
        float t[4] = {w.x, w.y, w.z, w.w};
#pragma unroll
        for (int d = 0; d < kDefer; ++d) {
          const float u = uh[d][c];
#pragma unroll
          for (int e = 0; e < 4; ++e) t[e] = act[e] ? fnmadd<EXACT>(ld[d][e], u, t[e]) : t[e];
        }
        *reinterpret_cast<float4*>(pc) = make_float4(t[0], t[1], t[2], t[3]);
      }
    }
  }
  return mykey;
}

__host__ __device__ constexpr int leaf_push_rows(int R) {
  return ((R + 3) / 4 % 2 == 0) ? (R + 3) / 4 * 4 + 4 : (R + 3) / 4 * 4;
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
  const int Rp = leaf_push_rows(R);                                        // padded row stride
  float* tile = reinterpret_cast<float*>(smem_raw);                        // [JB][Rp]
  int* label = reinterpret_cast<int*>(tile + (size_t)JB * Rp);             // [Rp]
  __shared__ ClusterSlot slot[2];
  __shared__ __align__(16) float urow[kLeafMax];
  __shared__ __align__(16) float rowk_s[kLeafMax];
  __shared__ unsigned long long wbest[kClusterThreads / 32];
  __shared__ float pv_s;
  __shared__ int win_label_s, rowk_label_s, prow_s;
  // pivot rows of the columns whose updates are still pending (slot k % kDefer)
  __shared__ __align__(16) float uh[kDefer][kLeafMax];

  const int b = (int)cluster.block_rank(), G = (int)cluster.num_blocks();
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int rbeg = b * R;
  const int nrows = max(0, min(M, rbeg + R) - rbeg);

  // stage the CTA's rows: every element an asynchronous copy, all in flight
  // at once (the panel streams from L2/HBM at the SM's bandwidth)
  for (int c = 0; c < JB; ++c)
    for (int r = tid; r < nrows; r += kClusterThreads)
      cp_async_elem(tile + c * Rp + r, P + (size_t)(rbeg + r) + (size_t)c * lda);
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
    // updates of columns kfirst .. k-1 (slots 0 .. s_slot-1) to the columns
    // after k+... are still pending in the tile (see step 6)
    const int s_slot = k % kDefer, kfirst = k - s_slot;
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
        // the candidate row is published up to date: its columns after k get
        // the pending updates, in column order (it may become row k of U)
        const int lr = (int)(0xFFFFFFFFu - (unsigned)(kk & 0xFFFFFFFFull)) - rbeg;
        for (int c = lane; c < JB; c += 32) {
          float v = tile[c * Rp + lr];
          if (c > k)
            for (int d = 0; d < s_slot; ++d) v = fnmadd<EXACT>(tile[(kfirst + d) * Rp + lr], uh[d][c], v);
          sl.row[c] = v;
        }
        if (lane == 0) sl.label = label[lr];
      }
      if (k >= rbeg && k < rbeg + nrows) {
        for (int c = lane; c < JB; c += 32) sl.row_k[c] = tile[c * Rp + (k - rbeg)];
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
      // row k becomes the (up-to-date) pivot row even without an interchange;
      // the row it displaces moves with its multipliers and still pending
      // updates, which step 6 applies at its new place
      if (k >= rbeg && k < rbeg + nrows) {
        const int lk = k - rbeg;
        for (int c = lane; c < JB; c += 32) tile[c * Rp + lk] = urow[c];
        if (lane == 0 && prow != k) label[lk] = win_label_s;
      }
      if (prow != k && own_p) {
        const int lp = prow - rbeg;
        for (int c = lane; c < JB; c += 32) tile[c * Rp + lp] = rowk_s[c];
        if (lane == 0) label[lp] = rowk_label_s;
      }
      for (int c = lane; c < JB; c += 32) uh[s_slot][c] = urow[c];
    }
    __syncthreads();
    // 6. scale column k below the pivot; column k+1 receives the pending
    //    updates and this column's at once (its values are the next pivot
    //    candidates); every kDefer columns the later columns receive the
    //    group's kDefer updates in one pass
    mykey = leaf_update_quads<EXACT>(tile, Rp, k, JB, rbeg, nrows, kfirst, s_slot, uh, pv_s);
  }
  // no CTA may exit while others can still read its shared memory
  cluster.sync();
  for (int c = 0; c < JB; ++c)
    for (int r = tid; r < nrows; r += kClusterThreads) P[(size_t)(rbeg + r) + (size_t)c * lda] = tile[c * Rp + r];
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

// ---------------------------------------------------------------------------
// Push form of the cluster leaf: the same factorization as
// leaf_panel_cluster_kernel, with the per-column exchange done by remote
// asynchronous stores instead of a cluster barrier and remote loads.  For
// column k every CTA sends its candidate (key, label and the candidate row,
// brought up to date) into a receive slot of every CTA of the cluster with
// st.async, which also counts the bytes on the receiver's mbarrier; the CTA
// holding row k sends that row the same way.  Each CTA then waits on its own
// mbarrier for the G + 1 messages of the column and picks the winner from
// the G keys itself (all CTAs reach the same winner).  One remote store
// latency per column replaces the barrier and the two dependent remote
// round trips.  Receive slots alternate by column parity: a CTA sends the
// messages of column k+2 only after it has received every CTA's message of
// column k+1, and each CTA sends that only after it has read its slots of
// column k, so a slot is never overwritten while it is being read; each
// CTA re-arms the barrier of a parity as soon as it has read that column.
template <int JBT>
struct PushMsg {
  unsigned long long key;
  int label;
  int pad;
  float row[JBT];
};

__device__ __forceinline__ uint32_t cl_smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ uint32_t cl_mapa(uint32_t addr, int rank) {
  uint32_t r;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(addr), "r"(rank));
  return r;
}
__device__ __forceinline__ void cl_st_async_v4(uint32_t raddr, uint4 v, uint32_t rbar) {
  asm volatile("st.async.shared::cluster.mbarrier::complete_tx::bytes.v4.b32 [%0], {%1, %2, %3, %4}, [%5];"
               ::"r"(raddr), "r"(v.x), "r"(v.y), "r"(v.z), "r"(v.w), "r"(rbar)
               : "memory");
}
__device__ __forceinline__ void cl_arm(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(cl_smem_u32(bar)), "r"(bytes)
               : "memory");
}
// Bounded wait (acquire at cluster scope: the remote stores are released by
// their complete-tx); returns false when it ran out.
__device__ __forceinline__ bool cl_wait(uint64_t* bar, uint32_t parity) {
  const uint32_t a = cl_smem_u32(bar);
  for (unsigned spins = 0; spins < kSpinLimit; ++spins) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.acquire.cluster.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(a), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

template <bool EXACT, int JBT>
__global__ void __launch_bounds__(kClusterThreads, 1)
leaf_panel_cluster_push_kernel(float* __restrict__ P, int lda, int M, int JB, int R, int row0, int* __restrict__ ipiv,
                               int* __restrict__ info, int* __restrict__ pair_dst, int* __restrict__ pair_src,
                               int* __restrict__ pair_count, int* __restrict__ status, int swap_a0, int swap_a1,
                               int swap_b0, int swap_b1, unsigned long long* __restrict__ phase) {
  namespace cg = cooperative_groups;
  cg::cluster_group cluster = cg::this_cluster();
  using Msg = PushMsg<JBT>;
  static_assert(sizeof(Msg) % 16 == 0, "message of whole 16-byte vectors");
  extern __shared__ __align__(16) unsigned char smem_raw[];
  // rows of the tile padded to a multiple of four (the update works on
  // groups of four rows with 16-byte shared-memory accesses) and to an odd
  // number of such groups, so that the lanes of a warp reading one row
  // across the columns spread over eight banks instead of one
  const int Rp = leaf_push_rows(R);
  float* tile = reinterpret_cast<float*>(smem_raw);                        // [JB][Rp]
  int* label = reinterpret_cast<int*>(tile + (size_t)JB * Rp);             // [Rp]
  __shared__ __align__(16) Msg recv[2][kClusterCtas];                      // candidates of column k, by parity
  __shared__ __align__(16) Msg recv_k[2];                                  // row k of column k, by parity
  __shared__ __align__(16) Msg out_s;                                      // this CTA's candidate message
  __shared__ __align__(16) Msg outk_s;                                     // row k, when this CTA holds it
  __shared__ __align__(8) uint64_t full[2];
  __shared__ unsigned long long wbest[kClusterThreads / 32];
  __shared__ float pv_s;
  __shared__ __align__(16) float uh[kDefer][kLeafMax];

  const int b = (int)cluster.block_rank(), G = (int)cluster.num_blocks();
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int rbeg = b * R;
  const int nrows = max(0, min(M, rbeg + R) - rbeg);
  // a message is its 16-byte header and the row's JB values, whole vectors
  const int nvec = 1 + (JB + 3) / 4;
  const uint32_t tx_per_col = (uint32_t)((G + 1) * nvec * 16);
  // this lane's first vector of the push (destination d0, vector v0) and
  // the step of 32 vectors in destinations and vectors
  const int d0 = lane / nvec, v0 = lane - d0 * nvec, q32 = 32 / nvec, r32 = 32 - q32 * nvec;

  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(cl_smem_u32(&full[0])));
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(cl_smem_u32(&full[1])));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    cl_arm(&full[0], tx_per_col);
    if (JB > 1) cl_arm(&full[1], tx_per_col);
  }
  for (int c = 0; c < JB; ++c)
    for (int r = tid; r < nrows; r += kClusterThreads)
      cp_async_elem(tile + c * Rp + r, P + (size_t)(rbeg + r) + (size_t)c * lda);
  cp_async_commit();
  for (int r = tid; r < nrows; r += kClusterThreads) label[r] = rbeg + r;
  cp_async_wait<0>();
  // every CTA's barriers are initialised and armed before any message flies
  cluster.sync();
  unsigned long long mykey = 0;
  for (int r = tid; r < nrows; r += kClusterThreads) {
    unsigned long long kk = pack_key(tile[r], rbeg + r, 0);
    mykey = kk > mykey ? kk : mykey;
  }
  bool timed_out = false;
  // optional cycle counts of the column steps (CTA 0, thread 0): [0] the
  // CTA reduction, [1] the message and its push, [2] the wait, [3] the
  // interchange, [4] the barrier after it, [5] the update
  const bool timing = phase != nullptr && b == 0 && tid == 0;
  long long ph[6] = {0, 0, 0, 0, 0, 0};
  long long tc = timing ? clock64() : 0;
  auto mark = [&](int i) {
    if (timing) {
      const long long now = clock64();
      ph[i] += now - tc;
      tc = now;
    }
  };

  for (int k = 0; k < JB; ++k) {
    const int par = k & 1;
    const int s_slot = k % kDefer, kfirst = k - s_slot;
    const int k_cta = k / R;
    // 1. this CTA's best candidate for column k
    mykey = warp_max_u64(mykey);
    if (lane == 0) wbest[warp] = mykey;
    __syncthreads();
    mark(0);
    if (warp == 0) {
      unsigned long long kk = lane < kClusterThreads / 32 ? wbest[lane] : 0ull;
      kk = warp_max_u64(kk);
      // 2 + 3. the message: key, label and the candidate row with the
      //    group's pending updates applied to its columns after k, staged
      //    in shared memory, then pushed to every CTA of the cluster with
      //    consecutive lanes covering one destination's vectors (few
      //    destinations per store instruction); the CTA holding row k
      //    sends that row as it stands
      if (lane == 0) out_s.key = kk;
      if (kk != 0ull) {
        const int lr = (int)(0xFFFFFFFFu - (unsigned)(kk & 0xFFFFFFFFull)) - rbeg;
        for (int c = lane; c < JB; c += 32) {
          float v = tile[c * Rp + lr];
          if (c > k)
            for (int d = 0; d < s_slot; ++d) v = fnmadd<EXACT>(tile[(kfirst + d) * Rp + lr], uh[d][c], v);
          out_s.row[c] = v;
        }
        if (lane == 0) out_s.label = label[lr];
      }
      const bool holds_k = (b == k_cta);
      const int lk0 = k - rbeg;
      if (holds_k) {
        for (int c = lane; c < JB; c += 32) outk_s.row[c] = tile[c * Rp + lk0];
        if (lane == 0) outk_s.label = label[lk0];
      }
      __syncwarp();
      {
        const uint32_t bar_l = cl_smem_u32(&full[par]);
        const uint4* src = reinterpret_cast<const uint4*>(&out_s);
        const uint32_t slot_l = cl_smem_u32(&recv[par][b]);
        // vector i = lane + 32 j of the G * nvec is vector v of CTA d; (d, v)
        // stepped without a division
        for (int d = d0, v = v0; d < G; d += q32, v += r32) {
          if (v >= nvec) { v -= nvec; ++d; }
          if (d >= G) break;
          cl_st_async_v4(cl_mapa(slot_l + 16u * v, d), src[v], cl_mapa(bar_l, d));
        }
        if (holds_k) {
          const uint4* srck = reinterpret_cast<const uint4*>(&outk_s);
          const uint32_t slotk_l = cl_smem_u32(&recv_k[par]);
          for (int d = d0, v = v0; d < G; d += q32, v += r32) {
            if (v >= nvec) { v -= nvec; ++d; }
            if (d >= G) break;
            cl_st_async_v4(cl_mapa(slotk_l + 16u * v, d), srck[v], cl_mapa(bar_l, d));
          }
        }
      }
      mark(1);
      // 4. wait for the G candidates and row k of this column (every lane
      //    of the warp acquires the remote stores it is about to read)
      // After one wait has run out the CTA waits no more: it finishes the
      // leaf on whatever it holds (the status word tells the host).
      const bool ok = timed_out ? false : __all_sync(0xffffffffu, cl_wait(&full[par], (uint32_t)((k >> 1) & 1)));
      if (!ok && !timed_out) {
        timed_out = true;
        if (lane == 0) atomicCAS(status, kStatusOk, kStatusFlagTimeout);
      }
      mark(2);
      // the winner (every CTA reaches the same), its row into the pending
      // pivot rows and, where this CTA holds them, into row k; the old row
      // k into the pivot's place
      unsigned long long ck = lane < G ? recv[par][lane].key : 0ull;
      const unsigned long long wk = warp_max_u64(ck);
      const int wc = __ffsll(__ballot_sync(0xffffffffu, ck == wk && lane < G)) - 1;
      const int prow = (int)(0xFFFFFFFFu - (unsigned)(wk & 0xFFFFFFFFull));
      const Msg& wm = recv[par][wc < 0 ? 0 : wc];
      const bool own_p = (prow >= rbeg && prow < rbeg + nrows) && prow != k;
      const bool own_k = (k >= rbeg && k < rbeg + nrows);
      const int lp = prow - rbeg;
      for (int c = lane; c < JB; c += 32) {
        const float u = wm.row[c];
        uh[s_slot][c] = u;
        if (own_k) tile[c * Rp + lk0] = u;
        if (own_p) tile[c * Rp + lp] = recv_k[par].row[c];
      }
      if (lane == 0) {
        const float pv = wm.row[k];
        if (own_k && prow != k) label[lk0] = wm.label;
        if (own_p) label[lp] = recv_k[par].label;
        pv_s = pv;
        if (b == 0) {
          ipiv[k] = row0 + prow + 1;
          if (pv == 0.0f && *info == 0) *info = row0 + k + 1;
        }
        // the slots of this parity are read: re-arm for column k + 2
        if (k + 2 < JB) cl_arm(&full[par], tx_per_col);
      }
      mark(3);
    }
    __syncthreads();
    mark(4);
    // 5. scale column k, update column k+1 (the next candidates) and, every
    //    kDefer columns, the later columns
    mykey = leaf_update_quads<EXACT>(tile, Rp, k, JB, rbeg, nrows, kfirst, s_slot, uh, pv_s);
    mark(5);
  }
  if (timing)
    for (int i = 0; i < 6; ++i) atomicAdd(phase + i, (unsigned long long)ph[i]);
  // the columns left over after the last flush (JB not a multiple of kDefer)
  // were finished column by column above; no CTA leaves while another may
  // still read it in the interchange step below
  cluster.sync();
  for (int c = 0; c < JB; ++c)
    for (int r = tid; r < nrows; r += kClusterThreads) P[(size_t)(rbeg + r) + (size_t)c * lda] = tile[c * Rp + r];
  for (int r = tid; r < nrows; r += kClusterThreads) {
    int g = rbeg + r;
    if (g < JB) {
      pair_dst[g] = row0 + g;
      pair_src[g] = row0 + label[r];
    } else if (label[r] != g) {
      int sl = JB + atomicAdd(pair_count, 1);
      if (sl < 2 * kLeafMax) {
        pair_dst[sl] = row0 + g;
        pair_src[sl] = row0 + label[r];
      } else {
        atomicCAS(status, kStatusOk, kStatusCapacity);
      }
    }
  }
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
