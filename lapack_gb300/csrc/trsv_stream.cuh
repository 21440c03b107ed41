// Streaming blocked triangular solve with several right-hand sides,
// X := op(T)^{-1} X, for the four DGETRS cases (SRC/dgetrs.f:187-217 calling
// BLAS/SRC/dtrsm.f:272-329) in the default (fused multiply-add) mode.
//
// The matrix is cut into 64-row blocks that CTAs take in solve order from a
// ticket counter.  A solved block is published by storing its values into a
// publication array that was filled with a sentinel bit pattern before the
// launch; each value is one aligned store, so a reader that sees a
// non-sentinel value sees the final one, and no flag, fence or counter sits
// between a block's solution and its readers.  (A NaN result is published
// as a NaN of another payload; arithmetic never produces the sentinel.)
//
// A CTA
//   * stages its diagonal block and the coupling tile to the block solved
//     just before it (the link) in shared memory before it waits for
//     anything; with INV it also forms the inverse Dinv of the diagonal
//     block and M = Dinv * (coupling tile);
//   * folds every other source block into per-warp partial sums, issuing a
//     column group's matrix loads before it polls that group's solution
//     values (split over warps by column groups for op = N, by rows for
//     op = T);
//   * INV: y = Dinv (b - partial sums) is ready before the link arrives;
//     the link costs one 64 x 64 matrix-vector product, x = y - M x_link.
//     Otherwise the link tile is folded like the others and the diagonal
//     block is solved by warp-synchronous substitution (non-unit diagonals
//     as products with reciprocals formed in the prologue).
// The summation order differs from the reference loop order, so the exact
// mode keeps trsv_blocked_kernel.  Every wait is bounded.
#pragma once
#include "common.cuh"

namespace gb {

constexpr int kTsBS = 64;
constexpr int kTsRQ = 4;            // right-hand sides per group
constexpr int kTsThreads = 256;     // 8 warps
constexpr int kTsLd = kTsBS + 1;

template <typename T>
struct TsBits;
template <>
struct TsBits<float> {
  static constexpr unsigned kSentinel = 0xFFFFFFFFu;
  static constexpr unsigned kNaN = 0x7FC00000u;
};
template <>
struct TsBits<double> {
  static constexpr unsigned long long kSentinel = 0xFFFFFFFFFFFFFFFFull;
  static constexpr unsigned long long kNaN = 0x7FF8000000000000ull;
};

template <typename T, bool INV>
constexpr int ts_smem_bytes() {
  // diagonal block, link tile, Dinv and M (INV), per-warp partials,
  // right-hand side / y, per-warp link values, reciprocal diagonal
  return (int)sizeof(T) * ((INV ? 4 : 2) * kTsBS * kTsLd + 8 * kTsBS * kTsRQ + kTsBS * kTsRQ +
                           8 * kTsBS * kTsRQ + kTsBS);
}

// relaxed (single-copy atomic) load and store of one published value
__device__ __forceinline__ float ts_ld_pub(const float* p) {
  unsigned v;
  asm volatile("ld.relaxed.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return __uint_as_float(v);
}
__device__ __forceinline__ double ts_ld_pub(const double* p) {
  unsigned long long v;
  asm volatile("ld.relaxed.gpu.global.b64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return __longlong_as_double((long long)v);
}
__device__ __forceinline__ bool ts_is_sentinel(float v) { return __float_as_uint(v) == TsBits<float>::kSentinel; }
__device__ __forceinline__ bool ts_is_sentinel(double v) {
  return (unsigned long long)__double_as_longlong(v) == TsBits<double>::kSentinel;
}
__device__ __forceinline__ void ts_st_pub(float* p, float v) {
  unsigned b = (v != v) ? TsBits<float>::kNaN : __float_as_uint(v);
  asm volatile("st.relaxed.gpu.global.b32 [%0], %1;" ::"l"(p), "r"(b) : "memory");
}
__device__ __forceinline__ void ts_st_pub(double* p, double v) {
  unsigned long long b = (v != v) ? TsBits<double>::kNaN : (unsigned long long)__double_as_longlong(v);
  asm volatile("st.relaxed.gpu.global.b64 [%0], %1;" ::"l"(p), "l"(b) : "memory");
}

// Inverse of the nr x nr triangular block D (lower when LOWER), padded to
// the identity beyond nr; one thread per column j, the column's entries
// kept in registers (entries on the zero side of the diagonal are zero).
template <typename T, bool LOWER, bool UNIT>
__device__ __forceinline__ void ts_invert(const T* D, T* Dinv, int nr) {
  const int j = threadIdx.x;
  if (j >= kTsBS) return;
  T x[kTsBS];
  if (LOWER) {
#pragma unroll
    for (int i = 0; i < kTsBS; ++i) {
      T s = T(0);
#pragma unroll
      for (int k = 0; k < i; ++k) s = fma(D[i * kTsLd + k], x[k], s);
      const T d = (UNIT || i >= nr) ? T(1) : D[i * kTsLd + i];
      const T rhs = (i == j) ? T(1) : T(0);
      x[i] = (i < j) ? T(0) : (rhs - s) / d;
    }
  } else {
#pragma unroll
    for (int i = kTsBS - 1; i >= 0; --i) {
      T s = T(0);
#pragma unroll
      for (int k = i + 1; k < kTsBS; ++k) s = fma(D[i * kTsLd + k], x[k], s);
      const T d = (UNIT || i >= nr) ? T(1) : D[i * kTsLd + i];
      const T rhs = (i == j) ? T(1) : T(0);
      x[i] = (i > j) ? T(0) : (rhs - s) / d;
    }
  }
#pragma unroll
  for (int i = 0; i < kTsBS; ++i) Dinv[i * kTsLd + j] = x[i];
}

// Reads NV published values per lane (entries with use[i] false read as 0),
// re-reading until none is the sentinel.  False when the wait runs out or
// another kernel reported an error.
template <typename T, int NV>
__device__ __forceinline__ bool ts_poll(T (&v)[NV], const T* const (&p)[NV], const bool (&use)[NV],
                                        int* status) {
  unsigned spins = 0;
  for (;;) {
    bool miss = false;
#pragma unroll
    for (int i = 0; i < NV; ++i) {
      v[i] = use[i] ? ts_ld_pub(p[i]) : T(0);
      miss |= use[i] && ts_is_sentinel(v[i]);
    }
    if (!__any_sync(0xffffffffu, miss)) return true;
    ++spins;
    if (__any_sync(0xffffffffu, spins > kSpinLimit || *(volatile int*)status != kStatusOk)) {
      if ((threadIdx.x & 31) == 0) atomicCAS(status, kStatusOk, kStatusFlagTimeout);
      return false;
    }
  }
}

template <typename T, bool FORWARD, bool UNIT, bool TRANS, bool INV>
__global__ void __launch_bounds__(kTsThreads)
trsv_stream_kernel(const T* __restrict__ A, int lda, int n, T* __restrict__ X, int ldx, int nrhs, T* __restrict__ pub,
                   unsigned* __restrict__ ticket, int* __restrict__ status, long long sA, long long sX, int nbatch) {
  extern __shared__ __align__(16) unsigned char ts_smem[];
  T* D = reinterpret_cast<T*>(ts_smem);                 // [64][65] op(T) diagonal block, row-major
  T* Lt = D + kTsBS * kTsLd;                            // [64][65] op(T) link tile, row-major
  T* Dinv = Lt + kTsBS * kTsLd;                         // [64][65] (INV)
  T* M = Dinv + kTsBS * kTsLd;                          // [64][65] Dinv * Lt (INV)
  T* red = D + (INV ? 4 : 2) * kTsBS * kTsLd;           // [8][64][RQ] per-warp partial sums (op = N)
  T* rv = red + 8 * kTsBS * kTsRQ;                      // [64][RQ] b - folded sources
  T* xl = rv + kTsBS * kTsRQ;                           // [8][64][RQ] link values, one copy per warp
  T* rdiag = xl + 8 * kTsBS * kTsRQ;                    // [64] reciprocal diagonal (substitution)
  __shared__ unsigned t_s;
  __shared__ int ok_s;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int nblk = (n + kTsBS - 1) / kTsBS;
  if (tid == 0) { t_s = atomicAdd(ticket, 1u); ok_s = 1; }
  __syncthreads();
  // a batch of independent systems shares the ticket counter, block-major:
  // ticket -> (block t in solve order, system), so the resident CTAs work on
  // the first blocks of every system at once and each system's chain of
  // blocks overlaps the others'; a block waits only on smaller tickets (the
  // earlier blocks of its own system)
  const int sys = (int)(t_s % (unsigned)nbatch);
  const int t = (int)(t_s / (unsigned)nbatch);
  A += sys * sA;
  X += sys * sX;
  pub += (size_t)sys * n * nrhs;
  const int bi = FORWARD ? t : nblk - 1 - t;
  const int r0 = bi * kTsBS;
  const int nr = min(kTsBS, n - r0);
  const int nsrc = t;                                  // sources in solve order: tickets 0 .. t-1
  auto src_block = [&](int s) { return FORWARD ? s : nblk - 1 - s; };
  const int cl = nsrc > 0 ? src_block(nsrc - 1) * kTsBS : 0;   // link block's first column
  const int ncl = nsrc > 0 ? min(kTsBS, n - cl) : 0;

  // ---- prologue: diagonal block (identity beyond nr) and link tile, op orientation
  for (int e = tid; e < kTsBS * kTsBS; e += kTsThreads) {
    const int a = e & 63, b = e >> 6;        // a runs along stored columns: coalesced
    const int i = TRANS ? b : a, j = TRANS ? a : b;
    D[i * kTsLd + j] = (i < nr && j < nr) ? (TRANS ? A[(size_t)(r0 + j) + (size_t)(r0 + i) * lda]
                                                   : A[(size_t)(r0 + i) + (size_t)(r0 + j) * lda])
                                          : (i == j ? T(1) : T(0));
    if (nsrc > 0)
      Lt[i * kTsLd + j] = (i < nr && j < ncl) ? (TRANS ? A[(size_t)(cl + j) + (size_t)(r0 + i) * lda]
                                                       : A[(size_t)(r0 + i) + (size_t)(cl + j) * lda])
                                              : T(0);
  }
  __syncthreads();
  if (!INV && !UNIT && tid < kTsBS) rdiag[tid] = T(1) / D[tid * kTsLd + tid];
  if (INV) {
    ts_invert<T, FORWARD, UNIT>(D, Dinv, nr);
    __syncthreads();
    if (nsrc > 0) {
      // M = Dinv * Lt: thread -> row tid/4, columns tid%4 + 4k
      const int i = tid >> 2, c = tid & 3;
      T m[16];
#pragma unroll
      for (int k = 0; k < 16; ++k) m[k] = T(0);
      for (int l = 0; l < kTsBS; ++l) {
        const T d = Dinv[i * kTsLd + l];
#pragma unroll
        for (int k = 0; k < 16; ++k) m[k] = fma(d, Lt[l * kTsLd + c + 4 * k], m[k]);
      }
#pragma unroll
      for (int k = 0; k < 16; ++k) M[i * kTsLd + c + 4 * k] = m[k];
    }
  }
  __syncthreads();
  // sources folded into partial sums: all, or all but the link with INV
  const int nbulk = INV ? max(nsrc - 1, 0) : nsrc;

  for (int q0 = 0; q0 < nrhs; q0 += kTsRQ) {
    const int nq = min(kTsRQ, nrhs - q0);
    const T* pq = pub + (size_t)q0 * n;               // published values of this group, leading dimension n
    bool okw = true;
    if (!TRANS) {
      // ---- op = N: warp w takes the column groups G = w, w+8, ... of CG
      // columns; lane holds rows lane and lane+32 of the block
      constexpr int CG = sizeof(T) == 4 ? 32 : 16;
      constexpr int GPS = kTsBS / CG;
      T acc0[kTsRQ], acc1[kTsRQ];
#pragma unroll
      for (int q = 0; q < kTsRQ; ++q) { acc0[q] = T(0); acc1[q] = T(0); }
      for (int G = warp; G < GPS * nbulk; G += 8) {
        const int s = G / GPS, h = G % GPS;
        const int c0 = src_block(s) * kTsBS + h * CG;
        const int nc = min(CG, n - c0);
        if (nc <= 0) continue;
        const bool link = !INV && s == nsrc - 1;
        T a0[CG], a1[CG];
        if (!link) {
          const T* Ac = A + (size_t)r0 + (size_t)c0 * lda;
#pragma unroll
          for (int j = 0; j < CG; ++j) {
            a0[j] = (j < nc && lane < nr) ? Ac[lane + (size_t)j * lda] : T(0);
            a1[j] = (j < nc && lane + 32 < nr) ? Ac[lane + 32 + (size_t)j * lda] : T(0);
          }
        } else {
#pragma unroll
          for (int j = 0; j < CG; ++j) {
            a0[j] = Lt[lane * kTsLd + h * CG + j];
            a1[j] = Lt[(lane + 32) * kTsLd + h * CG + j];
          }
        }
        T xv[kTsRQ];
        const T* ptr[kTsRQ];
        bool use[kTsRQ];
#pragma unroll
        for (int q = 0; q < kTsRQ; ++q) {
          ptr[q] = pq + (size_t)q * n + c0 + lane;
          use[q] = lane < nc && q < nq;
        }
        if (!(okw = ts_poll<T, kTsRQ>(xv, ptr, use, status))) break;
#pragma unroll
        for (int q = 0; q < kTsRQ; ++q) {
          if (q < nq) {
#pragma unroll
            for (int j = 0; j < CG; ++j) {
              const T xj = __shfl_sync(0xffffffffu, xv[q], j);
              acc0[q] = fma(a0[j], xj, acc0[q]);
              acc1[q] = fma(a1[j], xj, acc1[q]);
            }
          }
        }
      }
      if (!okw) ok_s = 0;
#pragma unroll
      for (int q = 0; q < kTsRQ; ++q) {
        red[(warp * kTsBS + lane) * kTsRQ + q] = acc0[q];
        red[(warp * kTsBS + lane + 32) * kTsRQ + q] = acc1[q];
      }
      __syncthreads();
      {
        const int row = tid >> 2, q = tid & 3;
        T v = T(0);
        if (row < nr && q < nq) {
          T sum = T(0);
#pragma unroll
          for (int w = 0; w < 8; ++w) sum += red[(w * kTsBS + row) * kTsRQ + q];
          v = X[(size_t)(r0 + row) + (size_t)(q0 + q) * ldx] - sum;
        }
        rv[row * kTsRQ + q] = v;
      }
    } else {
      // ---- op = T: warp w holds rows 8w .. 8w+7 of op(T)'s block row; lanes
      // run along the source columns (stored rows, contiguous)
      T acc[8][kTsRQ];
#pragma unroll
      for (int i = 0; i < 8; ++i)
#pragma unroll
        for (int q = 0; q < kTsRQ; ++q) acc[i][q] = T(0);
      const int rb = warp * 8;
      for (int s = 0; s < nbulk; ++s) {
        const int c0 = src_block(s) * kTsBS;
        const int nc = min(kTsBS, n - c0);
        const bool link = !INV && s == nsrc - 1;
        T a[2][8];
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          const int cc = h * 32 + lane;
#pragma unroll
          for (int i = 0; i < 8; ++i)
            a[h][i] = link ? Lt[(rb + i) * kTsLd + cc]
                           : ((cc < nc && rb + i < nr) ? A[(size_t)(c0 + cc) + (size_t)(r0 + rb + i) * lda] : T(0));
        }
        T xv[2 * kTsRQ];
        const T* ptr[2 * kTsRQ];
        bool use[2 * kTsRQ];
#pragma unroll
        for (int h = 0; h < 2; ++h)
#pragma unroll
          for (int q = 0; q < kTsRQ; ++q) {
            ptr[h * kTsRQ + q] = pq + (size_t)q * n + c0 + h * 32 + lane;
            use[h * kTsRQ + q] = h * 32 + lane < nc && q < nq;
          }
        if (!(okw = ts_poll<T, 2 * kTsRQ>(xv, ptr, use, status))) break;
#pragma unroll
        for (int q = 0; q < kTsRQ; ++q)
          if (q < nq)
#pragma unroll
            for (int i = 0; i < 8; ++i) {
              acc[i][q] = fma(a[0][i], xv[q], acc[i][q]);
              acc[i][q] = fma(a[1][i], xv[kTsRQ + q], acc[i][q]);
            }
      }
      if (!okw && lane == 0) ok_s = 0;
#pragma unroll
      for (int i = 0; i < 8; ++i)
#pragma unroll
        for (int q = 0; q < kTsRQ; ++q) {
          T v = acc[i][q];
#pragma unroll
          for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
          const int row = rb + i;
          if (lane == 0)
            rv[row * kTsRQ + q] = (row < nr && q < nq) ? X[(size_t)(r0 + row) + (size_t)(q0 + q) * ldx] - v : T(0);
        }
    }
    __syncthreads();
    if (!ok_s) break;

    // ---- diagonal block
    if (INV) {
      // y = Dinv * rv, then x = y - M * x_link: thread -> row tid/4, a
      // quarter of the columns, sums combined over the four lanes of a row
      const int row = tid >> 2, part = tid & 3;
      T y[kTsRQ];
#pragma unroll
      for (int q = 0; q < kTsRQ; ++q) {
        T sum = T(0);
        if (q < nq) {
#pragma unroll
          for (int j = 0; j < 16; ++j) sum = fma(Dinv[row * kTsLd + part * 16 + j], rv[(part * 16 + j) * kTsRQ + q], sum);
        }
        sum += __shfl_xor_sync(0xffffffffu, sum, 1);
        sum += __shfl_xor_sync(0xffffffffu, sum, 2);
        y[q] = sum;
      }
      if (nsrc > 0) {
        // every warp reads the link block's values itself and keeps a copy
        T v[2 * kTsRQ];
        const T* ptr[2 * kTsRQ];
        bool use[2 * kTsRQ];
#pragma unroll
        for (int h = 0; h < 2; ++h)
#pragma unroll
          for (int q = 0; q < kTsRQ; ++q) {
            ptr[h * kTsRQ + q] = pq + (size_t)q * n + cl + h * 32 + lane;
            use[h * kTsRQ + q] = h * 32 + lane < ncl && q < nq;
          }
        okw = ts_poll<T, 2 * kTsRQ>(v, ptr, use, status);
        T* xw = xl + warp * kTsBS * kTsRQ;
#pragma unroll
        for (int h = 0; h < 2; ++h)
#pragma unroll
          for (int q = 0; q < kTsRQ; ++q) xw[(h * 32 + lane) * kTsRQ + q] = v[h * kTsRQ + q];
        __syncwarp();
#pragma unroll
        for (int q = 0; q < kTsRQ; ++q) {
          T sum = T(0);
          if (q < nq) {
#pragma unroll
            for (int j = 0; j < 16; ++j) sum = fma(M[row * kTsLd + part * 16 + j], xw[(part * 16 + j) * kTsRQ + q], sum);
          }
          sum += __shfl_xor_sync(0xffffffffu, sum, 1);
          sum += __shfl_xor_sync(0xffffffffu, sum, 2);
          y[q] -= sum;
        }
      }
      if (okw && part == 0 && row < nr) {
#pragma unroll
        for (int q = 0; q < kTsRQ; ++q)
          if (q < nq) {
            X[(size_t)(r0 + row) + (size_t)(q0 + q) * ldx] = y[q];
            ts_st_pub(pub + (size_t)(q0 + q) * n + r0 + row, y[q]);
          }
      }
      if (!okw) ok_s = 0;
    } else if (warp < nq) {
      const int qq = warp;
      T x0 = lane < nr ? rv[lane * kTsRQ + qq] : T(0);
      T x1 = lane + 32 < nr ? rv[(lane + 32) * kTsRQ + qq] : T(0);
      if (FORWARD) {
        for (int k = 0; k < nr; ++k) {
          const bool hi = k >= 32;
          T xk = hi ? x1 : x0;
          if (!UNIT && (k & 31) == lane) {
            xk = xk * rdiag[k];
            if (hi) x1 = xk; else x0 = xk;
          }
          xk = __shfl_sync(0xffffffffu, xk, k & 31);
          if (lane > k && lane < nr) x0 = fma(-D[lane * kTsLd + k], xk, x0);
          if (lane + 32 > k && lane + 32 < nr) x1 = fma(-D[(lane + 32) * kTsLd + k], xk, x1);
        }
      } else {
        for (int k = nr - 1; k >= 0; --k) {
          const bool hi = k >= 32;
          T xk = hi ? x1 : x0;
          if (!UNIT && (k & 31) == lane) {
            xk = xk * rdiag[k];
            if (hi) x1 = xk; else x0 = xk;
          }
          xk = __shfl_sync(0xffffffffu, xk, k & 31);
          if (lane < k) x0 = fma(-D[lane * kTsLd + k], xk, x0);
          if (lane + 32 < k) x1 = fma(-D[(lane + 32) * kTsLd + k], xk, x1);
        }
      }
      T* pw = pub + (size_t)(q0 + qq) * n + r0;
      if (lane < nr) {
        X[(size_t)(r0 + lane) + (size_t)(q0 + qq) * ldx] = x0;
        ts_st_pub(pw + lane, x0);
      }
      if (lane + 32 < nr) {
        X[(size_t)(r0 + lane + 32) + (size_t)(q0 + qq) * ldx] = x1;
        ts_st_pub(pw + lane + 32, x1);
      }
    }
    __syncthreads();
    if (!ok_s) break;
  }
}

}  // namespace gb
