// Internal host-side interface of the GB300 LU solve library.
#pragma once
#include <cuda_runtime.h>
#include <cstddef>
#include <functional>

namespace gb {

// How the FP32 factorization inside DSGESV computes its trailing updates.
enum MixedMode : int {
  kMixedBf16x3 = 0,   // tcgen05 BF16 tensor cores, hi*hi + hi*lo + lo*hi, FP32 accumulation
  kMixedFp32 = 1,     // FFMA on the CUDA cores (the SGETRF arithmetic)
};

struct Options {
  bool exact = false;       // separately rounded products (bitwise reference order)
  int nb_f64 = 64;          // outer block size of the FP64 factorization
  int nb_f32 = 256;         // outer block size of the FP32 factorization
  int mixed_mode = kMixedBf16x3;
  int sgetrf_mode = kMixedFp32;   // sgetrf_ itself: plain FP32 by default
  int panel_ctas_f64 = 0;         // CTAs of the cooperative panel (0: all SMs)
  int panel_ctas_f32 = 0;
  int cluster_panel = 2;          // FP32 leaves on one thread-block cluster: 2 shared-memory kernel with cluster
                                  // barriers, 3 the same with a pushed exchange, 1 register kernel, 0 off
  int lookahead = 1;              // FP32 cluster path: factor the next block column beside the trailing update
  int trsv_inv = 1;               // DSGESV's FP32 solves: diagonal blocks applied as their inverses
  int gemm_ws = 1;                // BF16x3 update: 1 warp-specialised multi-tile kernel, 0 one tile per CTA
  int gemm_tiles = 4;             // tiles per CTA of the warp-specialised update (0: one CTA per SM)
  int ir_nan_guard = 0;           // DSGESV: a non-finite iterate or residual ends the refinement (ITER = -2)
  int panel_fuse = 1;             // panel recursion: a node with halves <= 64 columns as one fused launch
  int feed = 1;                   // host-pointer DSGESV: copy A in column chunks beside the FP32 factorization
  int feed_lazy = 0;              // test settings: 1 take a chunk in only when needed, 2 one chunk every step
  int pool_keep = 1;              // the stream-ordered pool keeps its memory between calls (set at first use)
  int feed_catchup = 8;           // block columns of catch-up a pending chunk gets per step
};
Options& options();          // process-wide; initialised from LAPACK_GB300_* environment variables

int device_sm_count();

// Scratch device memory, stream ordered (cudaMallocAsync / cudaFreeAsync).
struct DevScratch {
  void* p = nullptr;
  cudaStream_t s = nullptr;
  DevScratch() = default;
  DevScratch(size_t bytes, cudaStream_t st);
  ~DevScratch();
  DevScratch(const DevScratch&) = delete;
  DevScratch& operator=(const DevScratch&) = delete;
  template <typename T> T* as() const { return static_cast<T*>(p); }
};

// Columns of the matrix that reach the device while it is being factored
// (the host-pointer DSGESV copies A in column chunks beside the FP32
// factorization).  Chunk q covers columns [cols[q], cols[q+1]) and is in
// the matrix, in the original row order, once event ready[q] has
// completed.  When the factorization takes chunk q in, it calls
// admit(q, dPerm, s), which queues on s the reordering of the chunk's rows
// by the gather permutation of the interchanges so far, and then
// rejected(q), which may block until the chunk's data are known and
// returns true when they cannot be factored (DSGESV: an entry overflows
// FP32); the factorization then returns kFeedStop.
struct ColumnFeed {
  int nchunks = 0;
  const int* cols = nullptr;             // nchunks + 1 column boundaries
  const cudaEvent_t* ready = nullptr;    // nchunks events
  std::function<int(int, const int*, cudaStream_t)> admit;
  std::function<bool(int)> rejected;
};
constexpr int kFeedStop = 2000;
// A timing mark for the optional timeline of fed factorizations (no-op unless on).
void feed_trace_mark(int kind, int idx, int aux, cudaStream_t s);

// Device-pointer routines.  Return 0 or a CUDA / status error code; the
// LAPACK INFO goes to the device int *dInfo.  All work is queued on `s`.
// dPerm (optional, m ints): receives the gather permutation of P*A.
// feed (FP32, needs dPerm): columns arriving during the factorization.
template <typename T>
int getrf_dev(int m, int n, T* dA, int lda, int* dIpiv, int* dInfo, cudaStream_t s, int gemm_mode, int nb,
              int* dPerm = nullptr, const ColumnFeed* feed = nullptr);
template <typename T>
int getrs_dev(char trans, int n, int nrhs, const T* dA, int lda, const int* dIpiv, const int* dPerm,
              T* dB, int ldb, cudaStream_t s, bool inv_diag = false);   // inv_diag: diagonal blocks by their inverses
// X = L^{-1} for a unit lower triangular k x k L (k <= 512), FP32.
template <typename T>
int unit_lower_inverse_dev(int k, const T* L, int ldl, T* X, int ldx, cudaStream_t s);
// op(T) X = B for nbatch systems of one size, T the unit lower (lower) or
// upper triangle of stored LU factors; strides between systems in elements.
// dtrsv_order: in exact mode, each element's sum in the DTRSV loop order
// (BLAS/SRC/dtrsv.f) rather than the DTRSM order of DGETRS.
template <typename T>
int trsv_batched_dev(bool lower, bool trans, int n, int nrhs, const T* dA, int lda, long long sA, T* dX, int ldx,
                     long long sX, int nbatch, cudaStream_t s, bool dtrsv_order = false);
// op(T) X = B, T a triangle of dA (any UPLO / TRANS / DIAG), nrhs columns.
template <typename T>
int trsm_left_dev(bool upper, bool trans, bool unit, int n, int nrhs, const T* dA, int lda, T* dB, int ldb,
                  cudaStream_t s);
// Cholesky on device memory (SRC/dpotrf.f with block size nb); *info host.
template <typename T>
int potrf_dev(bool upper, int n, T* dA, int lda, int nb, int* info, cudaStream_t s);
template <typename T>
int potrs_dev(bool upper, int n, int nrhs, const T* dA, int lda, T* dB, int ldb, cudaStream_t s);
// DSPOSV on device memory; *iter and *info are host outputs.
int dsposv_dev(bool upper, int n, int nrhs, double* dA, int lda, const double* dB, int ldb, double* dX, int ldx,
               int* iter, int* info, cudaStream_t s);
// Complex LU (xGETRF with block size nb, xGETRF2 panels) and xGETRS
// (trans 0 = 'N', 1 = 'T', 2 = 'C') on device memory, for COMPLEX*16
// (R = double) and COMPLEX (R = float); elements are (re, im) pairs.  ZCGESV
// on device memory.  *info and *iter are host outputs.
template <typename R> struct cpx;
template <typename R>
int zgetrf_dev(int m, int n, cpx<R>* dA, int lda, int* dIpiv, int nb, int* info, cudaStream_t s);
template <typename R>
int zgetrs_dev(int trans, int n, int nrhs, const cpx<R>* dA, int lda, const int* dIpiv, cpx<R>* dB, int ldb,
               cudaStream_t s);
int zcgesv_dev(int n, int nrhs, cpx<double>* dA, int lda, int* dIpiv, const cpx<double>* dB, int ldb,
               cpx<double>* dX, int ldx, int* iter, int* info, cudaStream_t s);
// DTRSV on one device vector (X has n elements, unit stride).
int dtrsv_dev(bool upper, bool trans, bool unit, int n, const double* dA, int lda, double* dX, cudaStream_t s);
// DLATRS (SRC/dlatrs.f) on one device vector: *scale (host) receives SCALE;
// dCnorm (n doubles) is read when normin_y, else computed.
int dlatrs_dev(bool upper, bool trans, bool unit, bool normin_y, int n, const double* dA, int lda, double* dX,
               double* scale, double* dCnorm, cudaStream_t s);
// Gather permutation of a factorization: position r of P*A holds row perm[r].
int ipiv_perm_dev(const int* dIpiv, int k1, int k2, int incx, int lo, int span, int* dPerm, cudaStream_t s);
template <typename T>
int laswp_dev(int ncols, T* dA, int lda, int k1, int k2, const int* dIpiv, int incx, int lo, int span,
              cudaStream_t s);
template <typename T>
int gemm_update_dev(int M, int N, int K, const T* A, int lda, const T* B, int ldb, T* C, int ldc,
                    cudaStream_t s, int gemm_mode);
// One node of the panel recursion in one launch (k, nc <= 64): U12 =
// L11^{-1} A12 and A22 -= A21 U12, bitwise as trsm_llnu_dev + the FFMA / DFMA
// update.  *node_count: a zeroed device int, left zeroed.
template <typename T>
int panel_node_dev(T* A11, int lda, int M, int k, int nc, int* node_count, cudaStream_t s);
template <typename T>
int trsm_llnu_dev(int k, int ncols, const T* L, int ldl, T* B, int ldb, cudaStream_t s, int gemm_mode,
                  bool one_launch = true);   // false: leaf kernel + GEMM only (small shared memory)

// The BF16 hi/lo split of an update's A operand (M x Kp bf16 each, K-major),
// made once by bf16x3_split_a_dev and passed to several updates that share A.
struct Bf16SplitA {
  const void* hi = nullptr;
  const void* lo = nullptr;
  int M = 0, Kp = 0;
};
// Bytes one split of an M x K operand takes (hi and lo, 256-byte aligned).
size_t bf16x3_split_bytes(int M, int K);
// Splits A (M x K, column-major) into buf (bf16x3_split_bytes(M, K) bytes).
int bf16x3_split_a_dev(int M, int K, const float* A, int lda, void* buf, Bf16SplitA* out, cudaStream_t s);
// BF16x3 tensor-core update C -= A*B for FP32 operands (tcgen05); with
// a_pre the A operand's split is taken from there instead of made here.
int gemm_bf16x3_dev(int M, int N, int K, const float* A, int lda, const float* B, int ldb, float* C, int ldc,
                    cudaStream_t s, bool overwrite = false,   // overwrite: C = A*B
                    const Bf16SplitA* a_pre = nullptr);

// Host operands of the host-pointer DSGESV: dsgesv_dev copies them into
// dA / dB itself, A in column chunks on a second stream while the FP32
// factorization takes the chunks in as they land.
struct HostOperands {
  const double* a;
  int lda;
  const double* b;
  int ldb;
};
// C -= A*B in the reference DGEMM orders: sum_first false, each product
// subtracted in turn ('N','T'); true, the products summed and the sum
// subtracted once ('T','N').  Products separately rounded in exact mode,
// fused otherwise.  Tiled (the Cholesky factorization's updates).
template <typename T>
int gemm_ordered_dev(bool sum_first, int M, int N, int K, const T* A, int lda, const T* B, int ldb, T* C, int ldc,
                   cudaStream_t s);
// DSYRK of an n x n diagonal block (the other operand given transposed, B =
// op(A)^T): lower C -= A*B on and below the diagonal with dsyrk.f's zero
// skip, upper C -= (A*B summed first) on and above it.  Rounding as
// gemm_ordered_dev.  Tiled.
template <typename T>
int syrk_ordered_dev(bool upper, int n, int K, const T* A, int lda, const T* B, int ldb, T* C, int ldc, cudaStream_t s);
// DSGESV on device memory.  *iter and *info are host outputs.  With host,
// dA and dB are filled from host->a and host->b first.
int dsgesv_dev(int n, int nrhs, double* dA, int lda, int* dIpiv, const double* dB, int ldb, double* dX, int ldx,
               int* iter, int* info, cudaStream_t s, const HostOperands* host = nullptr);
// DGECON on device memory: *rcond and *info are host outputs.
int dgecon_dev(char norm, int n, const double* LU, int lda, double anorm, double* rcond, int* info, cudaStream_t s);
// DGESVX on device memory after its argument checks (for FACT = 'F' the
// caller passes ROWCND / COLCND of the given scalings).  *equed, *rcond,
// *rpvgrw (WORK(1)) and *info are host values; R, C, FERR, BERR device arrays.
int dgesvx_dev(char fact, char trans, int n, int nrhs, double* A, int lda, double* AF, int ldaf, int* ipiv,
               char* equed, double* R, double* C, double* B, int ldb, double* X, int ldx, double rowcnd,
               double colcnd, double* rcond, double* ferr, double* berr, double* rpvgrw, int* info, cudaStream_t s);
// MIN(s) <= 0 test (returns 1) and MAX(min,SMLNUM)/MIN(max,BIGNUM) of device scalings.
int scalings_cnd_dev(int n, const double* s_dev, double* cnd, cudaStream_t s, int* err);
// DGETRI on device memory: DTRTRI in blocks of nb_trtri, the inv(A)*L loop
// in blocks of nb (the workspace-limited value); *info is a host output.
int dgetri_dev(int n, double* A, int lda, const int* ipiv, int nb_trtri, int nb, int* info, cudaStream_t s);
// DGERFS on device memory; FERR/BERR are device arrays of nrhs doubles.
int dgerfs_dev(char trans, int n, int nrhs, const double* A, int lda, const double* AF, int ldaf, const int* ipiv,
               const double* B, int ldb, double* X, int ldx, double* ferr, double* berr, cudaStream_t s);
double dlange_inf_dev(int m, int n, const double* dA, int lda, cudaStream_t s, int* err);
// DLANGE on device memory: which = 0 'M', 1 '1', 2 'I', 3 'F'.  *out is a
// host double, valid after the stream synchronises.
int dlange_dev(int which, int m, int n, const double* dA, int lda, double* out, cudaStream_t s);
// DLAG2S with the reference's stop-at-first-overflow semantics; *first
// (host) receives the column-major index of the first overflow or -1.
int dlag2s_dev(int m, int n, const double* dA, int lda, float* dS, int lds, long long* first, cudaStream_t s);
int slag2d_dev(int m, int n, const float* dS, int lds, double* dA, int lda, cudaStream_t s);

// gB = A^{-T} gX, gA = -gB X^T from the stored factors (gA skipped if null).
int adjoint_dev(int n, int nrhs, const double* dLU, int ldlu, const int* dIpiv, const double* dX, int ldx,
                const double* dGX, int ldgx, double* dGB, int ldgb, double* dGA, int ldga, cudaStream_t s);

// Kernel launch status of the last failing bounded wait, 0 if none.
int check_status(int* dStatus, cudaStream_t s);
int* device_status_word();

}  // namespace gb
