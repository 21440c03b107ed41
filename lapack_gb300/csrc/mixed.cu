// DSGESV on the GPU (SRC/dsgesv.f:243-429): FP32 LU of a converted copy of
// A, FP32 solves, FP64 residual / update / convergence test on the device,
// ITERMAX = 30 refinement steps, then the FP64 DGETRF/DGETRS fallback with
// the reference's ITER codes (-2 conversion overflow, -3 FP32 LU singular,
// -31 no convergence).
#include "driver.h"
#include "prof.h"
#include "solve_kernels.cuh"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

namespace gb {

// DLANGE('I') into a device double: exact mode sums each row in column order
// (SRC/dlange.f:173-189); otherwise the columns are cut into chunks whose
// partial row sums are folded in fixed order (deterministic, more parallel).
static int row_abs_sums(int m, int n, const double* dA, int lda, double* d_out, cudaStream_t s) {
  const int nsplit = options().exact ? 1 : std::max(1, std::min(16, n / 512));
  const int chunk = (n + nsplit - 1) / nsplit;
  DevScratch buf(sizeof(double) * (size_t)m * (nsplit + 1), s);
  if (!buf.p) return (int)cudaErrorMemoryAllocation;
  double* part = buf.as<double>();
  double* rows = part + (size_t)m * nsplit;
  if (nsplit == 1) {
    GB_LAUNCH(row_abs_sum_kernel<double><<<(m + 63) / 64, 64, 0, s>>>(dA, lda, m, n, rows));
  } else {
    dim3 g((m + 63) / 64, nsplit);
    GB_LAUNCH(row_abs_sum_split_kernel<<<g, 64, 0, s>>>(dA, lda, m, n, chunk, part));
    GB_LAUNCH(fold_partials_kernel<<<(m + 255) / 256, 256, 0, s>>>(part, nsplit, m, rows));
  }
  GB_LAUNCH(max_nan_kernel<double><<<1, 1024, 0, s>>>(rows, m, d_out));
  return (int)cudaGetLastError();
}

double dlange_inf_dev(int m, int n, const double* dA, int lda, cudaStream_t s, int* err) {
  *err = 0;
  if (m <= 0 || n <= 0) return 0.0;
  DevScratch buf(sizeof(double), s);
  if (!buf.p) { *err = (int)cudaErrorMemoryAllocation; return 0.0; }
  if ((*err = row_abs_sums(m, n, dA, lda, buf.as<double>(), s))) return 0.0;
  double h = 0;
  cudaMemcpyAsync(&h, buf.as<double>(), sizeof(double), cudaMemcpyDeviceToHost, s);
  if (cudaStreamSynchronize(s) != cudaSuccess) *err = (int)cudaGetLastError();
  return h;
}

static int residual(int n, int nrhs, const double* A, int lda, const double* X, int ldx, const double* B, int ldb,
                    double* R, int ldr, cudaStream_t s) {
  unsigned grid = (unsigned)((n + kResidRows - 1) / kResidRows);
  prof_begin(kProfResidual, s);
  if (options().exact) {
    // the reference order: one sequential sum per row (SRC/dsgesv.f:328-332)
    GB_LAUNCH(residual_kernel<true><<<grid, kResidRows, 0, s>>>(A, lda, X, ldx, B, ldb, R, ldr, n, nrhs));
  } else {
    // enough independent chains to keep the FP64 pipe busy: ~16 column
    // chunks of >= 256 columns; right-hand sides in passes of 1, 2 or 4
    int nsplit = std::max(1, std::min(16, n / 256));
    int chunk = ((n + nsplit - 1) / nsplit + 31) / 32 * 32;
    nsplit = (n + chunk - 1) / chunk;
    const int rq = nrhs >= 4 ? 4 : (nrhs >= 2 ? 2 : 1);
    DevScratch part(sizeof(double) * (size_t)nsplit * rq * n, s);
    if (!part.p) return (int)cudaErrorMemoryAllocation;
    for (int q0 = 0; q0 < nrhs; q0 += rq) {
      dim3 g2(grid, nsplit);
      size_t tot = (size_t)n * std::min(rq, nrhs - q0);
      unsigned gr = (unsigned)((tot + 255) / 256);
      double* P = part.as<double>();
      if (rq == 4) {
        GB_LAUNCH(residual_partial_kernel<4><<<g2, kResidRows, 0, s>>>(A, lda, X, ldx, n, nrhs, q0, chunk, P));
        GB_LAUNCH(residual_reduce_kernel<4><<<gr, 256, 0, s>>>(P, nsplit, B, ldb, R, ldr, n, nrhs, q0));
      } else if (rq == 2) {
        GB_LAUNCH(residual_partial_kernel<2><<<g2, kResidRows, 0, s>>>(A, lda, X, ldx, n, nrhs, q0, chunk, P));
        GB_LAUNCH(residual_reduce_kernel<2><<<gr, 256, 0, s>>>(P, nsplit, B, ldb, R, ldr, n, nrhs, q0));
      } else {
        GB_LAUNCH(residual_partial_kernel<1><<<g2, kResidRows, 0, s>>>(A, lda, X, ldx, n, nrhs, q0, chunk, P));
        GB_LAUNCH(residual_reduce_kernel<1><<<gr, 256, 0, s>>>(P, nsplit, B, ldb, R, ldr, n, nrhs, q0));
      }
    }
  }
  prof_end(kProfResidual, s, 2.0 * n * (double)n * nrhs, 8.0 * ((double)n * n + 3.0 * n * nrhs));
  return (int)cudaGetLastError();
}

static unsigned blocks_for(size_t n) { return (unsigned)((n + 255) / 256); }

int dlag2s_dev(int m, int n, const double* dA, int lda, float* dS, int lds, long long* first, cudaStream_t s) {
  *first = -1;
  if (m <= 0 || n <= 0) return 0;
  DevScratch f(sizeof(unsigned long long), s);
  if (!f.p) return (int)cudaErrorMemoryAllocation;
  GB_CUDA_TRY(cudaMemsetAsync(f.p, 0xff, sizeof(unsigned long long), s));
  size_t tot = (size_t)m * n;
  GB_LAUNCH(first_overflow_kernel<<<blocks_for(tot), 256, 0, s>>>(dA, lda, m, n, f.as<unsigned long long>()));
  GB_LAUNCH(lag2s_upto_kernel<<<blocks_for(tot), 256, 0, s>>>(dA, lda, dS, lds, m, n, f.as<unsigned long long>()));
  unsigned long long h = 0;
  GB_CUDA_TRY(cudaMemcpyAsync(&h, f.p, sizeof(h), cudaMemcpyDeviceToHost, s));
  GB_CUDA_TRY(cudaStreamSynchronize(s));
  *first = (h == ~0ull) ? -1 : (long long)h;
  return 0;
}

int slag2d_dev(int m, int n, const float* dS, int lds, double* dA, int lda, cudaStream_t s) {
  if (m <= 0 || n <= 0) return 0;
  GB_LAUNCH(slag2d_kernel<<<blocks_for((size_t)m * n), 256, 0, s>>>(dS, lds, dA, lda, m, n));
  return (int)cudaGetLastError();
}

int dlange_dev(int which, int m, int n, const double* dA, int lda, double* out, cudaStream_t s) {
  *out = 0.0;
  if (m <= 0 || n <= 0) return 0;
  if (which == 2) {
    int err = 0;
    *out = dlange_inf_dev(m, n, dA, lda, s, &err);
    return err;
  }
  size_t tot = (size_t)m * n;
  if (which == 1) {
    DevScratch cs(sizeof(double) * ((size_t)n + 1), s);
    if (!cs.p) return (int)cudaErrorMemoryAllocation;
    GB_LAUNCH(col_abs_sum_kernel<double><<<(n + 31) / 32, 1024, 0, s>>>(dA, lda, m, n, cs.as<double>()));
    GB_LAUNCH(max_nan_kernel<double><<<1, 1024, 0, s>>>(cs.as<double>(), n, cs.as<double>() + n));
    GB_CUDA_TRY(cudaMemcpyAsync(out, cs.as<double>() + n, sizeof(double), cudaMemcpyDeviceToHost, s));
    GB_CUDA_TRY(cudaStreamSynchronize(s));
    return 0;
  }
  DevScratch w(32, s);
  if (!w.p) return (int)cudaErrorMemoryAllocation;
  GB_CUDA_TRY(cudaMemsetAsync(w.p, 0, 32, s));
  unsigned long long* bits = w.as<unsigned long long>();
  int* nanflag = reinterpret_cast<int*>(w.as<char>() + 8);
  double* acc = reinterpret_cast<double*>(w.as<char>() + 16);
  GB_LAUNCH(max_abs_kernel<double><<<blocks_for(tot), 256, 0, s>>>(dA, lda, m, n, bits, nanflag));
  if (which == 3) GB_LAUNCH(sumsq_scaled_kernel<<<blocks_for(tot), 256, 0, s>>>(dA, lda, m, n, bits, acc));
  unsigned long long hb = 0;
  int hn = 0;
  double ha = 0;
  GB_CUDA_TRY(cudaMemcpyAsync(&hb, bits, 8, cudaMemcpyDeviceToHost, s));
  GB_CUDA_TRY(cudaMemcpyAsync(&hn, nanflag, 4, cudaMemcpyDeviceToHost, s));
  GB_CUDA_TRY(cudaMemcpyAsync(&ha, acc, 8, cudaMemcpyDeviceToHost, s));
  GB_CUDA_TRY(cudaStreamSynchronize(s));
  double mx;
  memcpy(&mx, &hb, 8);
  if (hn) { *out = NAN; return 0; }
  if (which == 0) { *out = mx; return 0; }
  *out = (mx > 0 && !std::isinf(mx)) ? mx * std::sqrt(ha) : mx;   // Frobenius by scaled sum of squares
  return 0;
}


// Streams of the host-pointer DSGESV, per host thread and device: one for
// the host->device copies, one for the conversions of the landed chunks;
// and a pinned word per chunk receiving the overflow flag after its
// conversion.
struct FeedStreams {
  cudaStream_t copy[64] = {};
  cudaStream_t conv[64] = {};
  int* flag_words = nullptr;
  int nwords = 0;
  ~FeedStreams() {
    if (flag_words) cudaFreeHost(flag_words);
  }
};

static FeedStreams* feed_streams(int nchunks) {
  thread_local FeedStreams fs;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return nullptr;
  if (!fs.copy[dev] && cudaStreamCreateWithFlags(&fs.copy[dev], cudaStreamNonBlocking) != cudaSuccess) return nullptr;
  if (!fs.conv[dev] && cudaStreamCreateWithFlags(&fs.conv[dev], cudaStreamNonBlocking) != cudaSuccess) return nullptr;
  if (fs.nwords < nchunks) {
    if (fs.flag_words) cudaFreeHost(fs.flag_words);
    fs.flag_words = nullptr;
    fs.nwords = 0;
    if (cudaHostAlloc(&fs.flag_words, sizeof(int) * (size_t)nchunks, cudaHostAllocMapped) != cudaSuccess) return nullptr;
    fs.nwords = nchunks;
  }
  return &fs;
}

// dst(i, c) = src(perm[i], c) (perm null: src(i, c)): the rows of a landed
// chunk in the order of the interchanges made before it was taken in, and
// the copy back.  Kernels rather than device-to-device memcpy: a memcpy
// would queue on the copy engines behind the host->device chunks.
static __global__ void gather_rows_kernel(const float* __restrict__ src, int lds, const int* __restrict__ perm, int m,
                                          float* __restrict__ dst, int ldd) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < m) dst[(size_t)i + (size_t)blockIdx.y * ldd] = src[(size_t)(perm ? perm[i] : i) + (size_t)blockIdx.y * lds];
}

// *word = *flag, word in mapped host memory (the chunk's overflow verdict,
// read by the host after the conversion's event; no copy engine involved)
static __global__ void flag_to_host_kernel(const int* __restrict__ flag, volatile int* word) { *word = *flag; }

// Events of one host-pointer call, destroyed with it (a pending event is
// released once it completes).
struct EventSet {
  std::vector<cudaEvent_t> e;
  bool ok = true;
  explicit EventSet(int k) : e(k, nullptr) {
    for (auto& x : e) ok = ok && cudaEventCreateWithFlags(&x, cudaEventDisableTiming) == cudaSuccess;
  }
  ~EventSet() {
    for (auto& x : e)
      if (x) cudaEventDestroy(x);
  }
};

// The host-pointer DSGESV up to the FP32 factorization.  B, then A in
// column chunks go to the device on the copy stream; each landed chunk is
// converted on the conversion stream (DLAG2S and its DLANGE row sums: the
// chunks are the row-sum split, so the folded norm is that of one pass, or
// in exact mode 2048-column chunks continuing one running sum per row); the
// FP32 factorization on s takes every chunk in as it is converted.  Returns
// 0 (SA factored, its INFO in flags[2]), 1 (an entry overflows FP32: ITER =
// -2) or a CUDA error; on return s is ordered after every copy and
// conversion.
static int fed_sgetrf(int n, int nrhs, double* dA, int lda, double* dB, int ldb, const HostOperands& h, float* SA,
                      float* SX, double* part, double* rows, double* anrm, int nsplit, int chunk, int* flags,
                      int* dIpiv, int* perm, cudaStream_t s) {
  const Options& opt = options();
  const int cw = opt.exact ? std::min(n, 2048) : chunk;
  std::vector<int> cols;
  for (int c0 = 0; c0 < n; c0 += cw) cols.push_back(c0);
  cols.push_back(n);
  const int Q = (int)cols.size() - 1;
  FeedStreams* fs = feed_streams(Q);
  if (!fs) return (int)cudaErrorMemoryAllocation;
  int dev = 0;
  cudaGetDevice(&dev);
  cudaStream_t cp = fs->copy[dev], cv = fs->conv[dev];
  int* words = fs->flag_words;
  int* words_dev = nullptr;
  GB_CUDA_TRY(cudaHostGetDevicePointer(reinterpret_cast<void**>(&words_dev), words, 0));
  // events: [0, Q) chunk converted, Q start, Q+1 B landed; evl: chunk landed
  EventSet ev(Q + 2), evl(Q);
  if (!ev.ok || !evl.ok) return (int)cudaErrorMemoryAllocation;
  DevScratch tmp(sizeof(float) * (size_t)n * cw, s);
  if (!tmp.p) return (int)cudaErrorMemoryAllocation;
  {
    // grow the pool now by what the catch-ups' operand splits take (A21
    // and a slab of U rows in BF16 hi/lo), not while the copies run
    DevScratch pre(2 * bf16x3_split_bytes(n, opt.nb_f32), s);
    if (!pre.p) return (int)cudaErrorMemoryAllocation;
  }
  for (int q = 0; q < Q; ++q) words[q] = 0;
  // the copies follow whatever s queued before (the buffers, the flags reset)
  feed_trace_mark(3, 0, 0, s);
  GB_CUDA_TRY(cudaEventRecord(ev.e[Q], s));
  GB_CUDA_TRY(cudaStreamWaitEvent(cp, ev.e[Q], 0));
  GB_CUDA_TRY(cudaStreamWaitEvent(cv, ev.e[Q], 0));
  prof_begin(kProfCopyH2D, cp);
  GB_CUDA_TRY(cudaMemcpy2DAsync(dB, sizeof(double) * ldb, h.b, sizeof(double) * h.ldb, sizeof(double) * n, nrhs,
                                cudaMemcpyHostToDevice, cp));
  GB_CUDA_TRY(cudaEventRecord(ev.e[Q + 1], cp));
  for (int q = 0; q < Q; ++q) {
    const int c0 = cols[q], c1 = cols[q + 1];
    GB_CUDA_TRY(cudaMemcpy2DAsync(dA + (size_t)c0 * lda, sizeof(double) * lda, h.a + (size_t)c0 * h.lda,
                                  sizeof(double) * h.lda, sizeof(double) * n, c1 - c0, cudaMemcpyHostToDevice, cp));
    GB_CUDA_TRY(cudaEventRecord(evl.e[q], cp));
    GB_CUDA_TRY(cudaStreamWaitEvent(cv, evl.e[q], 0));
    dim3 g((n + 127) / 128, 1);
    GB_LAUNCH(dlag2s_rowsum_kernel<<<g, 128, 0, cv>>>(dA + (size_t)c0 * lda, lda, n, c1 - c0, c1 - c0,
                                                      SA + (size_t)c0 * n, n, opt.exact ? part : part + (size_t)q * n,
                                                      flags, opt.exact && q > 0));
    GB_LAUNCH(flag_to_host_kernel<<<1, 1, 0, cv>>>(flags, words_dev + q));
    GB_CUDA_TRY(cudaEventRecord(ev.e[q], cv));
    feed_trace_mark(2, q, 0, cv);
  }
  prof_end(kProfCopyH2D, cp, 0.0, 8.0 * (double)n * (n + nrhs));
  // SX = DLAG2S(B) once B has landed
  GB_CUDA_TRY(cudaStreamWaitEvent(s, ev.e[Q + 1], 0));
  GB_LAUNCH(dlag2s_kernel<<<blocks_for((size_t)n * nrhs), 256, 0, s>>>(dB, ldb, SX, n, n, nrhs, flags));
  ColumnFeed feed;
  feed.nchunks = Q;
  feed.cols = cols.data();
  feed.ready = ev.e.data();
  feed.admit = [&](int q, const int* pm, cudaStream_t st) -> int {
    if (!pm) return 0;   // no interchanges yet
    const int c0 = cols[q], nc = cols[q + 1] - c0;
    dim3 g((n + 255) / 256, nc);
    GB_LAUNCH(gather_rows_kernel<<<g, 256, 0, st>>>(SA + (size_t)c0 * n, n, pm, n, tmp.as<float>(), n));
    GB_LAUNCH(gather_rows_kernel<<<g, 256, 0, st>>>(tmp.as<float>(), n, nullptr, n, SA + (size_t)c0 * n, n));
    return (int)cudaGetLastError();
  };
  feed.rejected = [&](int q) -> bool {
    if (cudaEventSynchronize(ev.e[q]) != cudaSuccess) return true;
    return words[q] != 0;
  };
  int rc = getrf_dev<float>(n, n, SA, n, dIpiv, flags + 2, s, opt.mixed_mode, opt.nb_f32, perm, &feed);
  // s after every chunk's conversion (and so every copy)
  const cudaError_t jrc = cudaStreamWaitEvent(s, ev.e[Q - 1], 0);
  if (rc == kFeedStop) return 1;
  if (rc) return rc;
  if (jrc != cudaSuccess) return (int)jrc;
  GB_LAUNCH(fold_partials_kernel<<<(n + 255) / 256, 256, 0, s>>>(part, nsplit, n, rows));
  GB_LAUNCH(max_nan_kernel<double><<<1, 1024, 0, s>>>(rows, n, anrm));
  return (int)cudaGetLastError();
}

int dsgesv_dev(int n, int nrhs, double* dA, int lda, int* dIpiv, const double* dB, int ldb, double* dX, int ldx,
               int* iter, int* info, cudaStream_t s, const HostOperands* host) {
  const int itermax = 30;
  *iter = 0;
  *info = 0;
  if (n == 0) return 0;
  const Options& opt = options();
  // device scratch: SA (n x n FP32), SX (n x nrhs FP32), R (n x nrhs FP64),
  // the gather permutation, ||A||_inf, flags
  size_t nn = (size_t)n * n, nr = (size_t)n * nrhs;
  size_t bytes = 0;
  auto carve = [&](size_t b) { size_t off = bytes; bytes += (b + 255) / 256 * 256; return off; };
  size_t o_sa = carve(sizeof(float) * nn);
  size_t o_sx = carve(sizeof(float) * nr);
  size_t o_r = carve(sizeof(double) * nr);
  size_t o_perm = carve(sizeof(int) * n);
  size_t o_anrm = carve(sizeof(double));
  size_t o_flags = carve(sizeof(int) * 4);     // [0] overflow, [1] notconv, [2] sgetrf info
  DevScratch ws(bytes, s);
  if (!ws.p) return (int)cudaErrorMemoryAllocation;
  char* base = ws.as<char>();
  float* SA = reinterpret_cast<float*>(base + o_sa);
  float* SX = reinterpret_cast<float*>(base + o_sx);
  double* R = reinterpret_cast<double*>(base + o_r);
  int* perm = reinterpret_cast<int*>(base + o_perm);
  double* anrm = reinterpret_cast<double*>(base + o_anrm);
  int* flags = reinterpret_cast<int*>(base + o_flags);
  int hflags[4];
  int rc;
  // row sums of DLANGE('I'): exact mode one running sum per row in column
  // order, otherwise column chunks folded in fixed order
  const int nsplit = opt.exact ? 1 : std::max(1, std::min(16, n / 512));
  const int chunk = (n + nsplit - 1) / nsplit;
  DevScratch buf(sizeof(double) * (size_t)n * (nsplit + 1), s);
  if (!buf.p) return (int)cudaErrorMemoryAllocation;
  double* part = buf.as<double>();
  double* rows = part + (size_t)n * nsplit;

  GB_CUDA_TRY(cudaMemsetAsync(flags, 0, sizeof(int) * 4, s));
  if (host) {
    // copies, conversion and SGETRF overlapped; the overflow test of
    // DLAG2S(B) and DLAG2S(A) and the SGETRF INFO are read after
    rc = fed_sgetrf(n, nrhs, dA, lda, const_cast<double*>(dB), ldb, *host, SA, SX, part, rows, anrm, nsplit,
                    chunk, flags, dIpiv, perm, s);
    if (rc > 1) return rc;
    GB_CUDA_TRY(cudaMemcpyAsync(hflags, flags, sizeof(int) * 3, cudaMemcpyDeviceToHost, s));
    GB_CUDA_TRY(cudaStreamSynchronize(s));
    if (rc == 1 || hflags[0]) { *iter = -2; goto fallback; }
    if (hflags[2] != 0) { *iter = -3; goto fallback; }
  } else {
    // SX = DLAG2S(B)
    GB_LAUNCH(dlag2s_kernel<<<blocks_for(nr), 256, 0, s>>>(dB, ldb, SX, n, n, nrhs, flags));
    // ANRM = DLANGE('I') (kept on the device for the convergence test) and
    // SA = DLAG2S(A), in one pass over A; exact mode sums each row in column
    // order, otherwise column chunks are folded in fixed order
    dim3 g((n + 127) / 128, nsplit);
    GB_LAUNCH(dlag2s_rowsum_kernel<<<g, 128, 0, s>>>(dA, lda, n, n, chunk, SA, n, part, flags));
    GB_LAUNCH(fold_partials_kernel<<<(n + 255) / 256, 256, 0, s>>>(part, nsplit, n, rows));
    GB_LAUNCH(max_nan_kernel<double><<<1, 1024, 0, s>>>(rows, n, anrm));
    GB_CUDA_TRY(cudaMemcpyAsync(hflags, flags, sizeof(int), cudaMemcpyDeviceToHost, s));
    GB_CUDA_TRY(cudaStreamSynchronize(s));
    if (hflags[0]) { *iter = -2; goto fallback; }
    // SGETRF(SA)
    // the factorization also returns the gather permutation the solves reuse
    rc = getrf_dev<float>(n, n, SA, n, dIpiv, flags + 2, s, opt.mixed_mode, opt.nb_f32, perm);
    if (rc) return rc;
    GB_CUDA_TRY(cudaMemcpyAsync(hflags + 2, flags + 2, sizeof(int), cudaMemcpyDeviceToHost, s));
    GB_CUDA_TRY(cudaStreamSynchronize(s));
    if (hflags[2] != 0) { *iter = -3; goto fallback; }
  }
  // SX = SA^{-1} SX, X = SLAG2D(SX), R = B - A X
  if ((rc = getrs_dev<float>('N', n, nrhs, SA, n, dIpiv, perm, SX, n, s, opt.trsv_inv != 0))) return rc;
  GB_LAUNCH(slag2d_kernel<<<blocks_for(nr), 256, 0, s>>>(SX, n, dX, ldx, n, nrhs));
  if ((rc = residual(n, nrhs, dA, lda, dX, ldx, dB, ldb, R, n, s))) return rc;
  // the NaN guard (option ir_nan_guard) reports a non-finite X or R in
  // flags[0], the overflow flag, so it ends the refinement as DLAG2S would
  GB_LAUNCH(ir_check_kernel<<<nrhs, 256, 0, s>>>(dX, ldx, R, n, n, anrm, flags + 1, nullptr,
                                                 opt.ir_nan_guard ? flags : nullptr));
  GB_CUDA_TRY(cudaMemcpyAsync(hflags, flags, sizeof(int) * 2, cudaMemcpyDeviceToHost, s));
  GB_CUDA_TRY(cudaStreamSynchronize(s));
  if (hflags[0]) { *iter = -2; goto fallback; }
  if (hflags[1] == 0) { *iter = 0; return 0; }
  for (int it = 1; it <= itermax; ++it) {
    GB_CUDA_TRY(cudaMemsetAsync(flags, 0, sizeof(int) * 2, s));
    GB_LAUNCH(dlag2s_kernel<<<blocks_for(nr), 256, 0, s>>>(R, n, SX, n, n, nrhs, flags));
    if ((rc = getrs_dev<float>('N', n, nrhs, SA, n, dIpiv, perm, SX, n, s, opt.trsv_inv != 0))) return rc;
    GB_LAUNCH(lag2d_axpy_kernel<<<blocks_for(nr), 256, 0, s>>>(SX, n, dX, ldx, n, nrhs));
    if ((rc = residual(n, nrhs, dA, lda, dX, ldx, dB, ldb, R, n, s))) return rc;
    GB_LAUNCH(ir_check_kernel<<<nrhs, 256, 0, s>>>(dX, ldx, R, n, n, anrm, flags + 1, nullptr,
                                                   opt.ir_nan_guard ? flags : nullptr));
    GB_CUDA_TRY(cudaMemcpyAsync(hflags, flags, sizeof(int) * 2, cudaMemcpyDeviceToHost, s));
    GB_CUDA_TRY(cudaStreamSynchronize(s));
    if (hflags[0]) { *iter = -2; goto fallback; }
    if (hflags[1] == 0) { *iter = it; return 0; }
  }
  *iter = -itermax - 1;
fallback:
  // FP64 DGETRF on A in place, X = B, DGETRS (SRC/dsgesv.f:415-429)
  rc = getrf_dev<double>(n, n, dA, lda, dIpiv, flags + 3, s, 0, opt.nb_f64);
  if (rc) return rc;
  GB_CUDA_TRY(cudaMemcpyAsync(hflags + 3, flags + 3, sizeof(int), cudaMemcpyDeviceToHost, s));
  GB_CUDA_TRY(cudaStreamSynchronize(s));
  *info = hflags[3];
  if (*info != 0) return 0;
  GB_LAUNCH(copy_cols_kernel<double><<<blocks_for(nr), 256, 0, s>>>(dB, ldb, dX, ldx, n, nrhs));
  return getrs_dev<double>('N', n, nrhs, dA, lda, dIpiv, nullptr, dX, ldx, s);
}

}  // namespace gb
