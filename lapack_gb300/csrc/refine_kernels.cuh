// Kernels of DGERFS on the GPU (SRC/dgerfs.f:186-424): the residual
// R = B - op(A) X together with the componentwise bound W = |B| + |op(A)||X|,
// the backward error BERR, the forward-error weights, and the DLACN2
// (SRC/dlacn2.f:134-263) 1-norm estimator steps, all on device vectors.
//
// Every launch works on a list of right-hand-side columns (ColList): the
// reference refines one column at a time and stops each one on its own
// test, so the columns still refining, or still inside the estimator, are
// handed to each pass together and each column sees exactly the arithmetic
// it would see alone.
#pragma once
#include "common.cuh"

namespace gb {

constexpr int kRfsMaxList = 64;
struct ColList {
  int n;                   // entries used
  int c[kRfsMaxList];      // column index of entry t
};

// DLACN2 reverse-communication state of one column: ISAVE(1..3) and EST.
struct LacnState {
  double est;
  int kase;
  int jump;   // ISAVE(1)
  int j;      // ISAVE(2), 1-based
  int iter;   // ISAVE(3)
};

// ---------------------------------------------------------------- residual
// Reference order (BLAS/SRC/dgemv.f:256-311 as DGERFS calls it, then the W
// loops of SRC/dgerfs.f:343-366), every product separately rounded.
// 'N': R(i) = B(i) + sum_j (-X(j))*A(i,j) folded in j order; W(i) = |B(i)| +
// sum_j |A(i,j)|*|X(j)| in j order.  'T': R(k) = B(k) + (-1)*(sum_i A(i,k)X(i))
// and W(k) = |B(k)| + (sum_i |A(i,k)||X(i)|), sums in i order.
// One thread per output element, blockIdx.y = list entry.
template <bool TRANS>
__global__ void __launch_bounds__(128)
rfs_resid_exact_kernel(const double* __restrict__ A, int lda, const double* __restrict__ B, int ldb,
                       const double* __restrict__ X, int ldx, double* __restrict__ R, double* __restrict__ W, int ldr,
                       int n, ColList cols) {
  const int i = blockIdx.x * 128 + threadIdx.x;
  const int c = cols.c[blockIdx.y];
  if (i >= n) return;
  const double* x = X + (size_t)c * ldx;
  const double bi = B[(size_t)i + (size_t)c * ldb];
  double r, w;
  if (!TRANS) {
    r = bi;
    w = fabs(bi);
    for (int j = 0; j < n; ++j) {
      const double a = A[(size_t)i + (size_t)j * lda], xj = x[j];
      r = __dadd_rn(r, __dmul_rn(-xj, a));
      w = __dadd_rn(w, __dmul_rn(fabs(a), fabs(xj)));
    }
  } else {
    const double* a = A + (size_t)i * lda;
    double t = 0.0, sw = 0.0;
    for (int l = 0; l < n; ++l) {
      t = __dadd_rn(t, __dmul_rn(a[l], x[l]));
      sw = __dadd_rn(sw, __dmul_rn(fabs(a[l]), fabs(x[l])));
    }
    r = __dadd_rn(bi, -t);
    w = __dadd_rn(fabs(bi), sw);
  }
  R[(size_t)i + (size_t)c * ldr] = r;
  W[(size_t)i + (size_t)c * ldr] = w;
}

// 'N', default mode: one thread per row of A, four list entries per block
// (blockIdx.z), columns of A cut into blockIdx.y chunks whose partial sums
// of A*X and |A|*|X| are folded in fixed chunk order by rfs_resid_fold_kernel
// (deterministic run to run).  X chunks are staged in shared memory.
constexpr int kRfsRows = 64;
constexpr int kRfsRq = 4;
__global__ void __launch_bounds__(kRfsRows)
rfs_resid_partial_n_kernel(const double* __restrict__ A, int lda, const double* __restrict__ X, int ldx, int n,
                           int chunk, ColList cols, double* __restrict__ P) {
  __shared__ double xs[32][kRfsRq];
  const int i = blockIdx.x * kRfsRows + threadIdx.x;
  const int s = blockIdx.y, t0 = blockIdx.z * kRfsRq;
  const int nq = min(kRfsRq, cols.n - t0);
  const int l_beg = s * chunk, l_end = min(n, l_beg + chunk);
  double ax[kRfsRq], aw[kRfsRq];
#pragma unroll
  for (int q = 0; q < kRfsRq; ++q) ax[q] = aw[q] = 0.0;
  for (int l0 = l_beg; l0 < l_end; l0 += 32) {
    const int nl = min(32, l_end - l0);
    __syncthreads();
    for (int e = threadIdx.x; e < 32 * kRfsRq; e += kRfsRows) {
      const int l = e % 32, q = e / 32;
      xs[l][q] = (l < nl && q < nq) ? X[(size_t)(l0 + l) + (size_t)cols.c[t0 + q] * ldx] : 0.0;
    }
    __syncthreads();
    if (i < n) {
      double a[32];
#pragma unroll
      for (int u = 0; u < 32; ++u) a[u] = (u < nl) ? A[(size_t)i + (size_t)(l0 + u) * lda] : 0.0;
#pragma unroll
      for (int u = 0; u < 32; ++u)
#pragma unroll
        for (int q = 0; q < kRfsRq; ++q) {
          ax[q] = fma(a[u], xs[u][q], ax[q]);
          aw[q] = fma(fabs(a[u]), fabs(xs[u][q]), aw[q]);
        }
    }
  }
  if (i < n) {
    const int L = cols.n;
#pragma unroll
    for (int q = 0; q < kRfsRq; ++q)
      if (q < nq) {
        P[(((size_t)s * L + t0 + q) * 2 + 0) * n + i] = ax[q];
        P[(((size_t)s * L + t0 + q) * 2 + 1) * n + i] = aw[q];
      }
  }
}

__global__ void rfs_resid_fold_kernel(const double* __restrict__ P, int nsplit, const double* __restrict__ B, int ldb,
                                      double* __restrict__ R, double* __restrict__ W, int ldr, int n, ColList cols) {
  const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int L = cols.n;
  if (e >= (size_t)n * L) return;
  const int t = (int)(e / n), i = (int)(e - (size_t)t * n);
  double sx = 0.0, sw = 0.0;
  for (int s = 0; s < nsplit; ++s) {
    sx += P[(((size_t)s * L + t) * 2 + 0) * n + i];
    sw += P[(((size_t)s * L + t) * 2 + 1) * n + i];
  }
  const int c = cols.c[t];
  const double b = B[(size_t)i + (size_t)c * ldb];
  R[(size_t)i + (size_t)c * ldr] = b - sx;
  W[(size_t)i + (size_t)c * ldr] = fabs(b) + sw;
}

// 'T', default mode: one warp per column k of A (eight per block), four list
// entries per block (blockIdx.y); rows of X staged 256 at a time in shared
// memory, lane partial sums folded by a fixed shuffle tree.
__global__ void __launch_bounds__(256)
rfs_resid_t_kernel(const double* __restrict__ A, int lda, const double* __restrict__ B, int ldb,
                   const double* __restrict__ X, int ldx, double* __restrict__ R, double* __restrict__ W, int ldr,
                   int n, ColList cols) {
  __shared__ double xs[kRfsRq][256];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int k = blockIdx.x * 8 + warp;
  const int t0 = blockIdx.y * kRfsRq;
  const int nq = min(kRfsRq, cols.n - t0);
  double ax[kRfsRq], aw[kRfsRq];
#pragma unroll
  for (int q = 0; q < kRfsRq; ++q) ax[q] = aw[q] = 0.0;
  const double* a = A + (size_t)min(k, n - 1) * lda;
  for (int i0 = 0; i0 < n; i0 += 256) {
    const int ni = min(256, n - i0);
    __syncthreads();
#pragma unroll
    for (int q = 0; q < kRfsRq; ++q)
      xs[q][threadIdx.x] = (q < nq && threadIdx.x < ni) ? X[(size_t)(i0 + threadIdx.x) + (size_t)cols.c[t0 + q] * ldx]
                                                        : 0.0;
    __syncthreads();
    if (k < n) {
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        const int ii = lane + 32 * u;
        const double av = (ii < ni) ? a[i0 + ii] : 0.0;
#pragma unroll
        for (int q = 0; q < kRfsRq; ++q) {
          ax[q] = fma(av, xs[q][ii], ax[q]);
          aw[q] = fma(fabs(av), fabs(xs[q][ii]), aw[q]);
        }
      }
    }
  }
  if (k >= n) return;
#pragma unroll
  for (int q = 0; q < kRfsRq; ++q)
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
      ax[q] += __shfl_xor_sync(0xffffffffu, ax[q], off);
      aw[q] += __shfl_xor_sync(0xffffffffu, aw[q], off);
    }
  if (lane < nq) {
    double sx = ax[0], sw = aw[0];
#pragma unroll
    for (int q = 1; q < kRfsRq; ++q)
      if (lane == q) { sx = ax[q]; sw = aw[q]; }
    const int c = cols.c[t0 + lane];
    const double b = B[(size_t)k + (size_t)c * ldb];
    R[(size_t)k + (size_t)c * ldr] = b - sx;
    W[(size_t)k + (size_t)c * ldr] = fabs(b) + sw;
  }
}

// ------------------------------------------------------ backward error
// BERR = max_i |R(i)| / W(i), with (|R(i)| + SAFE1) / (W(i) + SAFE1) where
// W(i) <= SAFE2 (SRC/dgerfs.f:368-382).  A NaN ratio never replaces the
// running maximum, as in the reference's S = MAX(S, ...) with S >= 0.
__device__ __forceinline__ double block_max_256(double v, double* red) {
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, off));
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  double m = red[0];
#pragma unroll
  for (int w = 1; w < 8; ++w) m = fmax(m, red[w]);
  __syncthreads();
  return m;
}

__global__ void __launch_bounds__(256)
rfs_berr_kernel(const double* __restrict__ R, const double* __restrict__ W, int ldr, int n, double safe1,
                double safe2, ColList cols, double* __restrict__ berr) {
  __shared__ double red[8];
  const int c = cols.c[blockIdx.x];
  const double* r = R + (size_t)c * ldr;
  const double* w = W + (size_t)c * ldr;
  double s = 0.0;
  for (int i = threadIdx.x; i < n; i += 256) {
    const double wi = w[i], ar = fabs(r[i]);
    const double q = (wi > safe2) ? __ddiv_rn(ar, wi) : __ddiv_rn(__dadd_rn(ar, safe1), __dadd_rn(wi, safe1));
    s = fmax(s, q);
  }
  s = block_max_256(s, red);
  if (threadIdx.x == 0) berr[c] = s;
}

// W(i) = |R(i)| + NZ*EPS*W(i), plus SAFE1 where W(i) <= SAFE2
// (SRC/dgerfs.f:412-420), for every listed column.
__global__ void rfs_ferr_weights_kernel(const double* __restrict__ R, double* __restrict__ W, int ldr, int n,
                                        double nzeps, double safe1, double safe2, ColList cols) {
  const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (size_t)n * cols.n) return;
  const int t = (int)(e / n), i = (int)(e - (size_t)t * n);
  const size_t o = (size_t)i + (size_t)cols.c[t] * ldr;
  const double wi = W[o];
  const double v = __dadd_rn(fabs(R[o]), __dmul_rn(nzeps, wi));
  W[o] = (wi > safe2) ? v : __dadd_rn(v, safe1);
}

// ------------------------------------------------------ column movement
// D(:, t) = S(:, c_t) (times W(:, c_t) when W is given): the listed columns
// packed side by side for one multi-right-hand-side DGETRS.
__global__ void rfs_gather_kernel(const double* __restrict__ S, int lds, const double* __restrict__ W, int ldw,
                                  double* __restrict__ D, int ldd, int n, ColList cols, int t_base) {
  const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (size_t)n * cols.n) return;
  const int t = (int)(e / n), i = (int)(e - (size_t)t * n);
  const int c = cols.c[t];
  double v = S[(size_t)i + (size_t)c * lds];
  if (W) v = __dmul_rn(W[(size_t)i + (size_t)c * ldw], v);
  D[(size_t)i + (size_t)(t_base + t) * ldd] = v;
}

// S(:, c_t) = D(:, t) (times W(:, c_t) when W is given), or, with `add`,
// S(:, c_t) = S(:, c_t) + D(:, t) (the DAXPY of SRC/dgerfs.f:393).
__global__ void rfs_scatter_kernel(const double* __restrict__ D, int ldd, const double* __restrict__ W, int ldw,
                                   double* __restrict__ S, int lds, int n, ColList cols, int t_base, int add) {
  const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (size_t)n * cols.n) return;
  const int t = (int)(e / n), i = (int)(e - (size_t)t * n);
  const int c = cols.c[t];
  double v = D[(size_t)i + (size_t)(t_base + t) * ldd];
  if (W) v = __dmul_rn(W[(size_t)i + (size_t)c * ldw], v);
  double* dst = S + (size_t)i + (size_t)c * lds;
  *dst = add ? __dadd_rn(*dst, v) : v;
}

// ------------------------------------------------------ DLACN2 steps
// DASUM in the reference order (EXACT: one sequential sum) or as a fixed
// tree over the block (otherwise).  Every thread gets the result.
template <bool EXACT>
__device__ double block_asum(const double* x, int n, double* red) {
  double s = 0.0;
  if (EXACT) {
    if (threadIdx.x == 0)
      for (int i = 0; i < n; ++i) s = __dadd_rn(s, fabs(x[i]));
  } else {
    for (int i = threadIdx.x; i < n; i += 256) s += fabs(x[i]);
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
  }
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  double t = red[0];
  if (!EXACT) {
#pragma unroll
    for (int w = 1; w < 8; ++w) t += red[w];
  }
  __syncthreads();
  return t;
}

// IDAMAX (BLAS/SRC/idamax.f) over x, 1-based, as a block reduction with the
// first-maximum and leading-NaN rules.
__device__ int block_idamax(const double* x, int n, Cand<double>* red) {
  Cand<double> best;
  best.absval = 0;
  best.row = -1;
  best.cls = -1;
  for (int i = threadIdx.x; i < n; i += 256) {
    Cand<double> c = make_cand(x[i], i, 0);
    if (cand_better(c, best)) best = c;
  }
  best = warp_best(best);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = best;
  __syncthreads();
  Cand<double> b = red[0];
#pragma unroll
  for (int w = 1; w < 8; ++w)
    if (cand_better(red[w], b)) b = red[w];
  __syncthreads();
  return b.row + 1;
}

// One DLACN2 call for each listed column (one CTA each): consumes the
// product the previous call asked for (in X) and leaves the next request in
// X and KASE, or KASE = 0 with the estimate in EST.  The branch taken is
// uniform over the CTA.
template <bool EXACT>
__global__ void __launch_bounds__(256)
lacn2_step_kernel(int n, double* __restrict__ Xe, int ldx, double* __restrict__ V, int* __restrict__ Isgn,
                  LacnState* __restrict__ st, ColList cols) {
  __shared__ double red[8];
  __shared__ Cand<double> cred[8];
  const int c = cols.c[blockIdx.x];
  double* x = Xe + (size_t)c * ldx;
  double* v = V + (size_t)c * n;
  int* isgn = Isgn + (size_t)c * n;
  LacnState S = st[c];
  const int itmax = 5;
  bool go50 = false, go120 = false;
  __syncthreads();
  if (S.kase == 0) {
    const double inv = __ddiv_rn(1.0, (double)n);
    for (int i = threadIdx.x; i < n; i += 256) x[i] = inv;
    S.kase = 1;
    S.jump = 1;
  } else if (S.jump == 1) {
    if (n == 1) {
      if (threadIdx.x == 0) v[0] = x[0];
      S.est = fabs(x[0]);
      S.kase = 0;
    } else {
      S.est = block_asum<EXACT>(x, n, red);
      for (int i = threadIdx.x; i < n; i += 256) {
        const double sg = x[i] >= 0.0 ? 1.0 : -1.0;
        x[i] = sg;
        isgn[i] = (int)sg;
      }
      S.kase = 2;
      S.jump = 2;
    }
  } else if (S.jump == 2) {
    S.j = block_idamax(x, n, cred);
    S.iter = 2;
    go50 = true;
  } else if (S.jump == 3) {
    for (int i = threadIdx.x; i < n; i += 256) v[i] = x[i];
    const double estold = S.est;
    S.est = block_asum<EXACT>(x, n, red);
    int diff = 0;
    for (int i = threadIdx.x; i < n; i += 256) diff |= ((x[i] >= 0.0 ? 1 : -1) != isgn[i]);
    const int changed = __syncthreads_or(diff);
    if (!changed || S.est <= estold) {
      go120 = true;
    } else {
      for (int i = threadIdx.x; i < n; i += 256) {
        const double sg = x[i] >= 0.0 ? 1.0 : -1.0;
        x[i] = sg;
        isgn[i] = (int)sg;
      }
      S.kase = 2;
      S.jump = 4;
    }
  } else if (S.jump == 4) {
    const int jlast = S.j;
    S.j = block_idamax(x, n, cred);
    if (x[jlast - 1] != fabs(x[S.j - 1]) && S.iter < itmax) {
      S.iter += 1;
      go50 = true;
    } else {
      go120 = true;
    }
  } else {   // jump 5
    const double temp = __dmul_rn(2.0, __ddiv_rn(block_asum<EXACT>(x, n, red), (double)(3 * n)));
    if (temp > S.est) {
      for (int i = threadIdx.x; i < n; i += 256) v[i] = x[i];
      S.est = temp;
    }
    S.kase = 0;
  }
  __syncthreads();   // every read of x above precedes the writes below
  if (go50) {
    for (int i = threadIdx.x; i < n; i += 256) x[i] = (i == S.j - 1) ? 1.0 : 0.0;
    S.kase = 1;
    S.jump = 3;
  } else if (go120) {
    const double den = (double)(n - 1);
    for (int i = threadIdx.x; i < n; i += 256) {
      const double m = __dadd_rn(1.0, __ddiv_rn((double)i, den));
      x[i] = (i & 1) ? -m : m;
    }
    S.kase = 1;
    S.jump = 5;
  }
  if (threadIdx.x == 0) st[c] = S;
}

// FERR(c) = EST / max_i |X(i, c)| when that maximum is not zero
// (SRC/dgerfs.f:453-459).
__global__ void __launch_bounds__(256)
rfs_ferr_finish_kernel(const double* __restrict__ X, int ldx, int n, const LacnState* __restrict__ st,
                       ColList cols, double* __restrict__ ferr) {
  __shared__ double red[8];
  const int c = cols.c[blockIdx.x];
  const double* x = X + (size_t)c * ldx;
  double m = 0.0;
  for (int i = threadIdx.x; i < n; i += 256) m = fmax(m, fabs(x[i]));
  m = block_max_256(m, red);
  if (threadIdx.x == 0) ferr[c] = (m != 0.0) ? __ddiv_rn(st[c].est, m) : st[c].est;
}

}  // namespace gb
