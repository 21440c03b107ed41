// The two steps of the complex LU that carry its time, as CTA-wide kernels:
//
// * the ZGEMM('N','N') update C := C - A*B (SRC/zgetrf.f:214-218,
//   SRC/zgetrf2.f:251, ZCGESV's residual) on shared-memory tiles.  Each
//   thread keeps TM x TN elements of C in registers and folds the K terms
//   into them in increasing L as BLAS/SRC/zgemm.f:326-340 does: TEMP =
//   ALPHA*B(L,J) (formed once per tile element when B is staged), C(I,J) =
//   C(I,J) + TEMP*A(I,L), every real operation separately rounded -- the
//   per-element order of zgemm_nn_elem, so the bits are the same.
// * the triangular solve of one long column (ZGETRS) on one CTA;
// * the pivot step of one panel column (SRC/zgetrf2.f:176-211): IZAMAX as
//   independent reductions over the CTA's threads (zamax_part and its
//   combination, the result izamax_seq gives), the interchange by one
//   thread, then the column scaled by the reciprocal of the pivot (or
//   divided by it below SFMIN) with one element per thread.
//
// Templated on the component type (COMPLEX*16 and COMPLEX).
#include "common.cuh"
#include "driver.h"
#include "zlu_seq.h"

#include <algorithm>

namespace gb {

namespace {

template <typename R, int BM, int BN, int BK, int TM, int TN>
__global__ void __launch_bounds__((BM / TM) * (BN / TN))
zgemm_tile_kernel(int M, int N, int K, const cpx<R>* __restrict__ A, int lda, const cpx<R>* __restrict__ B, int ldb,
                  cpx<R>* __restrict__ C, int ldc) {
  constexpr int NT = (BM / TM) * (BN / TN);
  constexpr int TX = BM / TM;
  __shared__ cpx<R> As[BK][BM];
  __shared__ cpx<R> Ts[BK][BN];   // TEMP = ALPHA*B(L, J)
  const int tid = threadIdx.x, tx = tid % TX, ty = tid / TX;
  const int m0 = blockIdx.x * BM, n0 = blockIdx.y * BN;
  const cpx<R> zero = zmk(R(0), R(0)), alpha = zmk(R(-1), R(0));
  cpx<R> acc[TM][TN];
#pragma unroll
  for (int j = 0; j < TN; ++j) {
    const int n = n0 + ty + j * (BN / TN);
#pragma unroll
    for (int i = 0; i < TM; ++i) {
      const int m = m0 + tx + i * TX;
      acc[i][j] = (m < M && n < N) ? C[(size_t)m + (size_t)n * ldc] : zero;
    }
  }
  for (int k0 = 0; k0 < K; k0 += BK) {
    for (int e = tid; e < BM * BK; e += NT) {
      const int mm = e % BM, kk = e / BM, m = m0 + mm, k = k0 + kk;
      As[kk][mm] = (m < M && k < K) ? A[(size_t)m + (size_t)k * lda] : zero;
    }
    for (int e = tid; e < BK * BN; e += NT) {
      const int kk = e % BK, nn = e / BK, k = k0 + kk, n = n0 + nn;
      Ts[kk][nn] = (k < K && n < N) ? zmul(alpha, B[(size_t)k + (size_t)n * ldb]) : zero;
    }
    __syncthreads();
    const int kmax = min(BK, K - k0);   // no term beyond K: adding a zero product could flip a -0
    for (int kk = 0; kk < kmax; ++kk) {
      cpx<R> a[TM], t[TN];
#pragma unroll
      for (int i = 0; i < TM; ++i) a[i] = As[kk][tx + i * TX];
#pragma unroll
      for (int j = 0; j < TN; ++j) t[j] = Ts[kk][ty + j * (BN / TN)];
#pragma unroll
      for (int i = 0; i < TM; ++i)
#pragma unroll
        for (int j = 0; j < TN; ++j) acc[i][j] = zadd(acc[i][j], zmul(t[j], a[i]));
    }
    __syncthreads();
  }
#pragma unroll
  for (int j = 0; j < TN; ++j) {
    const int n = n0 + ty + j * (BN / TN);
#pragma unroll
    for (int i = 0; i < TM; ++i) {
      const int m = m0 + tx + i * TX;
      if (m < M && n < N) C[(size_t)m + (size_t)n * ldc] = acc[i][j];
    }
  }
}

template <typename R, int BM, int BN, int TM, int TN>
void launch_ztile(int m, int n, int k, const cpx<R>* A, int lda, const cpx<R>* B, int ldb, cpx<R>* C, int ldc,
                  cudaStream_t s) {
  dim3 grid((m + BM - 1) / BM, (n + BN - 1) / BN);
  GB_LAUNCH(zgemm_tile_kernel<R, BM, BN, 8, TM, TN><<<grid, (BM / TM) * (BN / TN), 0, s>>>(m, n, k, A, lda, B, ldb,
                                                                                          C, ldc));
}

constexpr int kZcolThreads = 256;

template <typename R>
__global__ void __launch_bounds__(kZcolThreads) zcol_cta_kernel(int m, cpx<R>* __restrict__ a, int* __restrict__ ipiv,
                                                                int gcol, int* __restrict__ info) {
  const int tid = threadIdx.x;
  if (m == 1) {
    if (tid == 0) {
      *ipiv = 1;
      if (zis0(a[0])) atomicMin(info, gcol);
    }
    return;
  }
  constexpr int kWarps = kZcolThreads / 32;
  __shared__ ZamaxPart<R> part[kWarps];
  __shared__ int p_s, mode_s;      // pivot row (1-based); 0 zero pivot, 1 no scaling, 2 multiply, 3 divide
  __shared__ cpx<R> r_s;
  const int lane = tid & 31, warp = tid >> 5;
  // the parts combined within each warp by shuffles, then the warps' by warp
  // 0 (the combination is associative, commutative and idempotent: a lane
  // past the end combines with its own value)
  auto warp_combine = [&](ZamaxPart<R> p) {
    for (int off = 16; off > 0; off >>= 1) {
      ZamaxPart<R> o;
      o.nan = __shfl_down_sync(0xffffffffu, p.nan, off);
      o.inf = __shfl_down_sync(0xffffffffu, p.inf, off);
      o.over = __shfl_down_sync(0xffffffffu, p.over, off);
      o.val = __shfl_down_sync(0xffffffffu, p.val, off);
      o.idx = __shfl_down_sync(0xffffffffu, p.idx, off);
      p = zamax_combine(p, o);
    }
    return p;
  };
  ZamaxPart<R> mine = warp_combine(zamax_part(m, a, tid, kZcolThreads));
  if (lane == 0) part[warp] = mine;
  __syncthreads();
  if (warp == 0) {
    mine = warp_combine(part[lane < kWarps ? lane : 0]);
    if (lane == 0) part[0] = mine;
  }
  __syncthreads();
  const ZamaxPart<R> all = part[0];
  int sidx = kZamaxNone;
  if (all.nan == kZamaxNone && all.inf == kZamaxNone && all.over != kZamaxNone) {
    // the scaled pass from the first overflowing sum
    __shared__ R sv[kWarps];
    __shared__ int si[kWarps];
    R v;
    int i;
    zamax_scaled_part(m, a, all.over, tid, kZcolThreads, &v, &i);
    for (int off = 16; off > 0; off >>= 1)
      zamax_pick(v, i, __shfl_down_sync(0xffffffffu, v, off), __shfl_down_sync(0xffffffffu, i, off));
    if (lane == 0) { sv[warp] = v; si[warp] = i; }
    __syncthreads();
    v = sv[0];
    i = si[0];
    for (int w = 1; w < kWarps; ++w) zamax_pick(v, i, sv[w], si[w]);
    sidx = i;
  }
  if (tid == 0) {
    const int p = zamax_result(all, sidx);
    *ipiv = p;
    p_s = p;
    if (zis0(a[p - 1])) {
      atomicMin(info, gcol);
      mode_s = 0;
    } else {
      if (p != 1) {
        const cpx<R> t = a[0];
        a[0] = a[p - 1];
        a[p - 1] = t;
      }
      if (zhypot(a[0].re, a[0].im) >= CpxLim<R>::tiny) {   // ABS(A(1,1)) >= SFMIN
        const cpx<R> r = zdiv(zmk(R(1), R(0)), a[0]);
        r_s = r;
        mode_s = (r.re == R(1) && r.im == R(0)) ? 1 : 2;    // ZSCAL's ZA = ONE quick return
      } else {
        r_s = a[0];
        mode_s = 3;
      }
    }
  }
  __syncthreads();
  const int mode = mode_s;
  if (mode < 2) return;
  const cpx<R> r = r_s;
  for (int i = 1 + tid; i < m; i += kZcolThreads) a[i] = (mode == 2) ? zmul(r, a[i]) : zdiv(a[i], r);
}

// One column b of ZTRSM('L', UPLO, TRANSA, DIAG), ALPHA = ONE, per CTA, for
// the three forms whose every element can follow the reference order with
// the rows spread over the threads (thread i % 256 owns row i and applies
// every operation on it, one barrier per k):
//  'N' lower / upper (BLAS/SRC/ztrsm.f:277-300): step k divides B(k) by
//   A(k,k), then each later (lower) or earlier (upper) row subtracts
//   B(k)*A(i,k) -- row i receives its terms in the reference's k order;
//  'T' / 'C' upper (ztrsm.f:302-318): row i's running TEMP is kept in B(i)
//   and receives A(k,i)*B(k) (conjugated for 'C') as soon as B(k) is final,
//   k ascending as in the reference's dot loop, then the division.
// ('T' / 'C' lower sums its terms in k ascending while the rows finish in
// k descending: it stays on one thread per column.)  The column is staged
// in shared memory when it fits (smem != 0), else worked on in place.
constexpr int kZtrsmThreads = 256;
template <typename R>
__global__ void __launch_bounds__(kZtrsmThreads) ztrsm_cta_kernel(int upper, int trans, int unit, int m,
                                                                  const cpx<R>* __restrict__ A, int lda,
                                                                  cpx<R>* __restrict__ B, int ldb, int smem) {
  extern __shared__ __align__(16) unsigned char ztrsm_raw[];
  constexpr int NT = kZtrsmThreads;
  cpx<R>* bg = B + (size_t)blockIdx.x * ldb;
  cpx<R>* b = smem ? reinterpret_cast<cpx<R>*>(ztrsm_raw) : bg;
  const int tid = threadIdx.x;
  const cpx<R> one = zmk(R(1), R(0));
  auto a = [&](int i, int j) -> cpx<R> { return A[(size_t)i + (size_t)j * lda]; };
  for (int i = tid; i < m; i += NT) b[i] = zmul(one, bg[i]);   // ALPHA*B
  const bool cj = trans == 2;
  auto first_after = [&](int k) { return k + 1 + ((tid - (k + 1)) % NT + NT) % NT; };   // first row > k of this thread
  if (trans == 0 && !upper) {
    for (int k = 0; k < m; ++k) {
      if (!unit && tid == k % NT) b[k] = zdiv(b[k], a(k, k));
      __syncthreads();
      const cpx<R> bk = b[k];
      for (int i = first_after(k); i < m; i += NT) b[i] = zsub(b[i], zmul(bk, a(i, k)));
    }
  } else if (trans == 0) {
    for (int k = m - 1; k >= 0; --k) {
      if (!unit && tid == k % NT) b[k] = zdiv(b[k], a(k, k));
      __syncthreads();
      const cpx<R> bk = b[k];
      for (int i = tid; i < k; i += NT) b[i] = zsub(b[i], zmul(bk, a(i, k)));
    }
  } else {
    for (int k = 0; k < m; ++k) {
      if (!unit && tid == k % NT) b[k] = zdiv(b[k], cj ? zconj(a(k, k)) : a(k, k));
      __syncthreads();
      const cpx<R> bk = b[k];
      for (int i = first_after(k); i < m; i += NT) b[i] = zsub(b[i], zmul(cj ? zconj(a(k, i)) : a(k, i), bk));
    }
  }
  if (smem) {
    __syncthreads();
    for (int i = tid; i < m; i += NT) bg[i] = b[i];
  }
}

}  // namespace

// The tile is the largest of 64 x 32, 32 x 32 and 16 x 16 that gives every
// SM a CTA (the panel's updates are thin); the per-element order does not
// depend on it.
template <typename R>
int zgemm_tile_dev(int m, int n, int k, const cpx<R>* A, int lda, const cpx<R>* B, int ldb, cpx<R>* C, int ldc,
                   cudaStream_t s) {
  if (m <= 0 || n <= 0 || k <= 0) return 0;
  const long sms = device_sm_count();
  auto ctas = [&](int bm, int bn) { return (long)((m + bm - 1) / bm) * ((n + bn - 1) / bn); };
  if (ctas(64, 32) >= sms) launch_ztile<R, 64, 32, 4, 2>(m, n, k, A, lda, B, ldb, C, ldc, s);
  else if (ctas(32, 32) >= sms) launch_ztile<R, 32, 32, 2, 2>(m, n, k, A, lda, B, ldb, C, ldc, s);
  else launch_ztile<R, 16, 16, 1, 1>(m, n, k, A, lda, B, ldb, C, ldc, s);
  return (int)cudaGetLastError();
}
template int zgemm_tile_dev<double>(int, int, int, const zdc*, int, const zdc*, int, zdc*, int, cudaStream_t);
template int zgemm_tile_dev<float>(int, int, int, const cfc*, int, const cfc*, int, cfc*, int, cudaStream_t);

// false when the form is 'T' / 'C' lower (the caller keeps one thread per
// column for it)
template <typename R>
bool ztrsm_cta_dev(int upper, int trans, int unit, int m, int ncols, const cpx<R>* A, int lda, cpx<R>* B, int ldb,
                   cudaStream_t s, int* rc) {
  *rc = 0;
  if (trans != 0 && !upper) return false;
  constexpr int kMaxSmem = 96 * 1024;
  static bool attr[64] = {false};
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 64 && !attr[dev]) {
    *rc = (int)cudaFuncSetAttribute(ztrsm_cta_kernel<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, kMaxSmem);
    if (*rc) return true;
    attr[dev] = true;
  }
  const size_t bytes = sizeof(cpx<R>) * (size_t)m;
  const int smem = bytes <= (size_t)kMaxSmem ? (int)bytes : 0;
  GB_LAUNCH(ztrsm_cta_kernel<R><<<ncols, kZtrsmThreads, smem, s>>>(upper, trans, unit, m, A, lda, B, ldb, smem));
  *rc = (int)cudaGetLastError();
  return true;
}
template bool ztrsm_cta_dev<double>(int, int, int, int, int, const zdc*, int, zdc*, int, cudaStream_t, int*);
template bool ztrsm_cta_dev<float>(int, int, int, int, int, const cfc*, int, cfc*, int, cudaStream_t, int*);

template <typename R>
int zcol_cta_dev(int m, cpx<R>* a, int* ipiv, int gcol, int* info, cudaStream_t s) {
  GB_LAUNCH(zcol_cta_kernel<R><<<1, kZcolThreads, 0, s>>>(m, a, ipiv, gcol, info));
  return (int)cudaGetLastError();
}
template int zcol_cta_dev<double>(int, zdc*, int*, int, int*, cudaStream_t);
template int zcol_cta_dev<float>(int, cfc*, int*, int, int*, cudaStream_t);

}  // namespace gb
