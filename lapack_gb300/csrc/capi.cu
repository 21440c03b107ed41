// C ABI of the library: the LAPACK Fortran-ABI routines (host pointers, the
// library stages data through GPU memory inside each call) and the gb300_*
// device-pointer entry points.
#include "../../include/lapack_gb300.h"
#include "driver.h"
#include "latrs_seq.h"
#include "prof.h"
#include "zlu_seq.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <vector>

using gb::DevScratch;
using gb::options;

namespace {

// ------------------------------------------------------------ xerbla_
std::mutex g_xerbla_mu;
int g_xerbla_capture = 0;
char g_xerbla_name[16] = {0};
int g_xerbla_info = 0;

bool lsame(char a, char b) { return (a | 0x20) == (b | 0x20); }

void call_xerbla(const char* name, int info) {
  lapack_int i = info;
  xerbla_(name, &i, strlen(name));
}

// Per-host-thread non-blocking stream for the host-pointer routines.
cudaStream_t thread_stream() {
  thread_local cudaStream_t s = nullptr;
  thread_local int dev_of_s = -1;
  int dev = 0;
  cudaGetDevice(&dev);
  if (!s || dev_of_s != dev) {
    cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
    dev_of_s = dev;
  }
  return s;
}

// A device failure inside a LAPACK-ABI routine has no reference INFO code;
// it is reported on stderr and as INFO = -1000 - code.
void device_failure(const char* name, int code, lapack_int* info) {
  fprintf(stderr, "lapack_gb300: %s failed on the GPU (status %d: %s)\n", name, code,
          code > 0 && code < 1000 ? cudaGetErrorString((cudaError_t)code) : "bounded wait or capacity");
  if (info) *info = -1000 - code;
}

int finish(cudaStream_t s) {
  cudaError_t e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return (int)e;
  int st = gb::check_status(gb::device_status_word(), s);
  if (st != 0) {
    int zero = 0;
    cudaMemcpy(gb::device_status_word(), &zero, sizeof(int), cudaMemcpyHostToDevice);
    return 1000 + st;
  }
  return 0;
}

template <typename T>
int h2d(T* d, int ldd, const T* h, int ldh, int m, int n, cudaStream_t s) {
  if (m <= 0 || n <= 0) return 0;
  return (int)cudaMemcpy2DAsync(d, sizeof(T) * (size_t)ldd, h, sizeof(T) * (size_t)ldh, sizeof(T) * (size_t)m, n,
                                cudaMemcpyHostToDevice, s);
}
template <typename T>
int d2h(T* h, int ldh, const T* d, int ldd, int m, int n, cudaStream_t s) {
  if (m <= 0 || n <= 0) return 0;
  return (int)cudaMemcpy2DAsync(h, sizeof(T) * (size_t)ldh, d, sizeof(T) * (size_t)ldd, sizeof(T) * (size_t)m, n,
                                cudaMemcpyDeviceToHost, s);
}

inline int ld_dev(int m) { return std::max(1, (m + 31) / 32 * 32); }

// Device copies of the operands of the host-pointer solve routines live in
// one buffer per host thread and device, grown on demand and kept for the
// next call (freed when the thread exits).  Keeping it matters beyond the
// cost of allocating: a host->device copy into device memory the GPU has
// not touched before runs several times slower than into memory it has.
struct HostWorkspace {
  char* p[64] = {};
  size_t bytes[64] = {};
  ~HostWorkspace() {
    for (int d = 0; d < 64; ++d)
      if (p[d] && cudaSetDevice(d) == cudaSuccess) cudaFree(p[d]);
  }
};

char* host_workspace(size_t bytes, cudaStream_t s) {
  thread_local HostWorkspace w;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return nullptr;
  if (w.bytes[dev] < bytes) {
    if (w.p[dev]) {
      cudaStreamSynchronize(s);
      cudaFree(w.p[dev]);
      w.p[dev] = nullptr;
      w.bytes[dev] = 0;
    }
    void* q = nullptr;
    if (cudaMalloc(&q, bytes) != cudaSuccess) {
      cudaGetLastError();
      return nullptr;
    }
    w.p[dev] = static_cast<char*>(q);
    w.bytes[dev] = bytes;
  }
  return w.p[dev];
}

// Consecutive 256-byte aligned pieces of one buffer.
struct Carve {
  size_t off = 0;
  char* base = nullptr;
  size_t add(size_t b) {
    size_t o = off;
    off += (b + 255) / 256 * 256;
    return o;
  }
  template <typename T>
  T* at(size_t o) const { return reinterpret_cast<T*>(base + o); }
};

// ------------------------------------------------------------ GETRF
template <typename T>
void getrf_host(const char* name, const lapack_int* m, const lapack_int* n, T* a, const lapack_int* lda,
                lapack_int* ipiv, lapack_int* info, int nb, int gemm_mode) {
  *info = 0;
  if (*m < 0) *info = -1;
  else if (*n < 0) *info = -2;
  else if (*lda < std::max(1, *m)) *info = -4;
  if (*info != 0) { call_xerbla(name, -*info); return; }
  if (*m == 0 || *n == 0) return;
  cudaStream_t s = thread_stream();
  const int M = *m, N = *n, ld = ld_dev(M), mn = std::min(M, N);
  Carve cv;
  const size_t oA = cv.add(sizeof(T) * (size_t)ld * N), oP = cv.add(sizeof(int) * (mn + 1));
  cv.base = host_workspace(cv.off, s);
  if (!cv.base) { device_failure(name, (int)cudaErrorMemoryAllocation, info); return; }
  T* dA = cv.at<T>(oA);
  int* dP = cv.at<int>(oP);
  int* dInfo = dP + mn;
  int rc = h2d(dA, ld, a, *lda, M, N, s);
  if (!rc) rc = gb::getrf_dev<T>(M, N, dA, ld, dP, dInfo, s, gemm_mode, nb);
  if (!rc) rc = d2h(a, *lda, dA, ld, M, N, s);
  if (!rc) rc = (int)cudaMemcpyAsync(ipiv, dP, sizeof(int) * mn, cudaMemcpyDeviceToHost, s);
  int hinfo = 0;
  if (!rc) rc = (int)cudaMemcpyAsync(&hinfo, dInfo, sizeof(int), cudaMemcpyDeviceToHost, s);
  if (!rc) rc = finish(s);
  if (rc) { device_failure(name, rc, info); return; }
  *info = hinfo;
}

// ------------------------------------------------------------ GETRS
template <typename T>
void getrs_host(const char* name, const char* trans, const lapack_int* n, const lapack_int* nrhs, const T* a,
                const lapack_int* lda, const lapack_int* ipiv, T* b, const lapack_int* ldb, lapack_int* info) {
  *info = 0;
  const bool notran = lsame(*trans, 'N');
  if (!notran && !lsame(*trans, 'T') && !lsame(*trans, 'C')) *info = -1;
  else if (*n < 0) *info = -2;
  else if (*nrhs < 0) *info = -3;
  else if (*lda < std::max(1, *n)) *info = -5;
  else if (*ldb < std::max(1, *n)) *info = -8;
  if (*info != 0) { call_xerbla(name, -*info); return; }
  if (*n == 0 || *nrhs == 0) return;
  cudaStream_t s = thread_stream();
  const int N = *n, R = *nrhs, ld = ld_dev(N);
  Carve cv;
  const size_t oA = cv.add(sizeof(T) * (size_t)ld * N), oB = cv.add(sizeof(T) * (size_t)ld * R),
               oP = cv.add(sizeof(int) * N);
  cv.base = host_workspace(cv.off, s);
  if (!cv.base) { device_failure(name, (int)cudaErrorMemoryAllocation, info); return; }
  T* dA = cv.at<T>(oA);
  T* dB = cv.at<T>(oB);
  int* dP = cv.at<int>(oP);
  int rc = h2d(dA, ld, a, *lda, N, N, s);
  if (!rc) rc = h2d(dB, ld, b, *ldb, N, R, s);
  if (!rc) rc = (int)cudaMemcpyAsync(dP, ipiv, sizeof(int) * N, cudaMemcpyHostToDevice, s);
  if (!rc) rc = gb::getrs_dev<T>(notran ? 'N' : 'T', N, R, dA, ld, dP, nullptr, dB, ld, s);
  if (!rc) rc = d2h(b, *ldb, dB, ld, N, R, s);
  if (!rc) rc = finish(s);
  if (rc) device_failure(name, rc, info);
}

// ------------------------------------------------------------ GESV
template <typename T>
void gesv_host(const char* name, const lapack_int* n, const lapack_int* nrhs, T* a, const lapack_int* lda,
               lapack_int* ipiv, T* b, const lapack_int* ldb, lapack_int* info, int nb, int gemm_mode) {
  *info = 0;
  if (*n < 0) *info = -1;
  else if (*nrhs < 0) *info = -2;
  else if (*lda < std::max(1, *n)) *info = -4;
  else if (*ldb < std::max(1, *n)) *info = -7;
  if (*info != 0) { call_xerbla(name, -*info); return; }
  if (*n == 0) return;
  cudaStream_t s = thread_stream();
  const int N = *n, R = *nrhs, ld = ld_dev(N);
  Carve cv;
  const size_t oA = cv.add(sizeof(T) * (size_t)ld * N), oB = cv.add(sizeof(T) * (size_t)ld * std::max(R, 1)),
               oP = cv.add(sizeof(int) * (N + 1));
  cv.base = host_workspace(cv.off, s);
  if (!cv.base) { device_failure(name, (int)cudaErrorMemoryAllocation, info); return; }
  T* dA = cv.at<T>(oA);
  T* dB = cv.at<T>(oB);
  int* dP = cv.at<int>(oP);
  int* dInfo = dP + N;
  int hinfo = 0;
  int rc = h2d(dA, ld, a, *lda, N, N, s);
  if (!rc) rc = h2d(dB, ld, b, *ldb, N, R, s);
  if (!rc) rc = gb::getrf_dev<T>(N, N, dA, ld, dP, dInfo, s, gemm_mode, nb);
  if (!rc) rc = (int)cudaMemcpyAsync(&hinfo, dInfo, sizeof(int), cudaMemcpyDeviceToHost, s);
  if (!rc) rc = finish(s);
  if (!rc && hinfo == 0 && R > 0)   // SRC/dgesv.f:166: solve only for a nonsingular U
    rc = gb::getrs_dev<T>('N', N, R, dA, ld, dP, nullptr, dB, ld, s);
  if (!rc) rc = d2h(a, *lda, dA, ld, N, N, s);
  if (!rc && hinfo == 0) rc = d2h(b, *ldb, dB, ld, N, R, s);
  if (!rc) rc = (int)cudaMemcpyAsync(ipiv, dP, sizeof(int) * N, cudaMemcpyDeviceToHost, s);
  if (!rc) rc = finish(s);
  if (rc) { device_failure(name, rc, info); return; }
  *info = hinfo;
}

// ------------------------------------------------------------ LASWP
template <typename T>
void laswp_host(const lapack_int* n, T* a, const lapack_int* lda, const lapack_int* k1, const lapack_int* k2,
                const lapack_int* ipiv, const lapack_int* incx) {
  // DLASWP has no argument checks and no INFO (SRC/dlaswp.f:136-150)
  const int inc = *incx;
  if (inc == 0 || *n <= 0) return;
  const int K1 = *k1, K2 = *k2;
  if (K2 < K1) return;
  // the row window touched: rows K1..K2 and every interchange target
  int lo = K1, hi = K2;
  for (int i = K1; i <= K2; ++i) {
    int p = ipiv[K1 - 1 + (i - K1) * std::abs(inc)];
    lo = std::min(lo, p);
    hi = std::max(hi, p);
  }
  if (lo < 1) return;   // the reference would index before A(1,.)
  const int span = hi - lo + 1, N = *n, LDA = *lda;
  const int nidx = K1 + (K2 - K1) * std::abs(inc);
  cudaStream_t s = thread_stream();
  // the device copy holds rows lo..hi only, so IPIV is re-based to that window
  std::vector<int> shifted(ipiv, ipiv + nidx);
  for (auto& v : shifted) v -= (lo - 1);
  DevScratch dA(sizeof(T) * (size_t)span * N, s), dP(sizeof(int) * (size_t)nidx, s);
  if (!dA.p || !dP.p) { device_failure("DLASWP", (int)cudaErrorMemoryAllocation, nullptr); return; }
  int rc = h2d(dA.as<T>(), span, a + (lo - 1), LDA, span, N, s);
  if (!rc) rc = (int)cudaMemcpyAsync(dP.p, shifted.data(), sizeof(int) * nidx, cudaMemcpyHostToDevice, s);
  if (!rc) rc = gb::laswp_dev<T>(N, dA.as<T>(), span, K1 - (lo - 1), K2 - (lo - 1), dP.as<int>(), inc, 0, span, s);
  if (!rc) rc = d2h(a + (lo - 1), LDA, dA.as<T>(), span, span, N, s);
  if (!rc) rc = finish(s);
  if (rc) device_failure("DLASWP", rc, nullptr);
}

}  // namespace

namespace {
// ------------------------------------------------------------ POTRF / POTRS / POSV
template <typename T>
void potrf_host(const char* name, const char* uplo, const lapack_int* n, T* a, const lapack_int* lda,
                lapack_int* info) {
  // SRC/dpotrf.f:131-145
  *info = 0;
  const bool upper = lsame(*uplo, 'U');
  if (!upper && !lsame(*uplo, 'L')) *info = -1;
  else if (*n < 0) *info = -2;
  else if (*lda < std::max(1, *n)) *info = -4;
  if (*info != 0) { call_xerbla(name, -*info); return; }
  if (*n == 0) return;
  cudaStream_t s = thread_stream();
  const int N = *n, ld = ld_dev(N);
  DevScratch dA(sizeof(T) * (size_t)ld * N, s);
  if (!dA.p) { device_failure(name, (int)cudaErrorMemoryAllocation, info); return; }
  int inf = 0;
  int rc = h2d(dA.as<T>(), ld, a, *lda, N, N, s);
  if (!rc) rc = gb::potrf_dev<T>(upper, N, dA.as<T>(), ld, 64, &inf, s);
  if (!rc) rc = d2h(a, *lda, dA.as<T>(), ld, N, N, s);
  if (!rc) rc = finish(s);
  if (rc) { device_failure(name, rc, info); return; }
  *info = inf;
}
template <typename T>
void potrs_host(const char* name, const char* uplo, const lapack_int* n, const lapack_int* nrhs, const T* a,
                const lapack_int* lda, T* b, const lapack_int* ldb, lapack_int* info) {
  // SRC/dpotrs.f:146-165
  *info = 0;
  const bool upper = lsame(*uplo, 'U');
  if (!upper && !lsame(*uplo, 'L')) *info = -1;
  else if (*n < 0) *info = -2;
  else if (*nrhs < 0) *info = -3;
  else if (*lda < std::max(1, *n)) *info = -5;
  else if (*ldb < std::max(1, *n)) *info = -7;
  if (*info != 0) { call_xerbla(name, -*info); return; }
  if (*n == 0 || *nrhs == 0) return;
  cudaStream_t s = thread_stream();
  const int N = *n, R = *nrhs, ld = ld_dev(N);
  DevScratch dA(sizeof(T) * (size_t)ld * N, s), dB(sizeof(T) * (size_t)ld * R, s);
  if (!dA.p || !dB.p) { device_failure(name, (int)cudaErrorMemoryAllocation, info); return; }
  int rc = h2d(dA.as<T>(), ld, a, *lda, N, N, s);
  if (!rc) rc = h2d(dB.as<T>(), ld, b, *ldb, N, R, s);
  if (!rc) rc = gb::potrs_dev<T>(upper, N, R, dA.as<T>(), ld, dB.as<T>(), ld, s);
  if (!rc) rc = d2h(b, *ldb, dB.as<T>(), ld, N, R, s);
  if (!rc) rc = finish(s);
  if (rc) device_failure(name, rc, info);
}
}  // namespace

// ------------------------------------------------------------ complex LU
// COMPLEX*16 / COMPLEX arrays are (re, im) pairs; xGETRF uses ILAENV's block
// size 64, as the reference does.
template <typename R>
void zgetrf_host(const char* name, const lapack_int* m, const lapack_int* n, void* a, const lapack_int* lda,
                 lapack_int* ipiv, lapack_int* info, int nb = 64) {
  // SRC/zgetrf.f:144-157 (nb = 1: xGETRF2 alone, SRC/zgetrf2.f:154-170)
  using C = gb::cpx<R>;
  *info = 0;
  if (*m < 0) *info = -1;
  else if (*n < 0) *info = -2;
  else if (*lda < std::max(1, *m)) *info = -4;
  if (*info != 0) { call_xerbla(name, -*info); return; }
  if (*m == 0 || *n == 0) return;
  cudaStream_t s = thread_stream();
  const int M = *m, N = *n, ld = ld_dev(M), mn = std::min(M, N);
  DevScratch dA(sizeof(C) * (size_t)ld * N, s), dP(sizeof(int) * mn, s);
  if (!dA.p || !dP.p) { device_failure(name, (int)cudaErrorMemoryAllocation, info); return; }
  C* ha = static_cast<C*>(a);
  int inf = 0;
  int rc = h2d(dA.as<C>(), ld, ha, *lda, M, N, s);
  if (!rc) rc = gb::zgetrf_dev<R>(M, N, dA.as<C>(), ld, dP.as<int>(), nb, &inf, s);
  if (!rc) rc = d2h(ha, *lda, dA.as<C>(), ld, M, N, s);
  if (!rc) rc = (int)cudaMemcpyAsync(ipiv, dP.p, sizeof(int) * mn, cudaMemcpyDeviceToHost, s);
  if (!rc) rc = finish(s);
  if (rc) { device_failure(name, rc, info); return; }
  *info = inf;
}

template <typename R>
void zgetrs_host(const char* name, const char* trans, const lapack_int* n, const lapack_int* nrhs, const void* a,
                 const lapack_int* lda, const lapack_int* ipiv, void* b, const lapack_int* ldb, lapack_int* info) {
  // SRC/zgetrs.f:157-177
  using C = gb::cpx<R>;
  *info = 0;
  const bool notran = lsame(*trans, 'N'), tr = lsame(*trans, 'T'), cj = lsame(*trans, 'C');
  if (!notran && !tr && !cj) *info = -1;
  else if (*n < 0) *info = -2;
  else if (*nrhs < 0) *info = -3;
  else if (*lda < std::max(1, *n)) *info = -5;
  else if (*ldb < std::max(1, *n)) *info = -8;
  if (*info != 0) { call_xerbla(name, -*info); return; }
  if (*n == 0 || *nrhs == 0) return;
  cudaStream_t s = thread_stream();
  const int N = *n, R_ = *nrhs, ld = ld_dev(N);
  DevScratch dA(sizeof(C) * (size_t)ld * N, s), dB(sizeof(C) * (size_t)ld * R_, s), dP(sizeof(int) * N, s);
  if (!dA.p || !dB.p || !dP.p) { device_failure(name, (int)cudaErrorMemoryAllocation, info); return; }
  C* hb = static_cast<C*>(b);
  int rc = h2d(dA.as<C>(), ld, static_cast<const C*>(a), *lda, N, N, s);
  if (!rc) rc = h2d(dB.as<C>(), ld, static_cast<const C*>(hb), *ldb, N, R_, s);
  if (!rc) rc = (int)cudaMemcpyAsync(dP.p, ipiv, sizeof(int) * N, cudaMemcpyHostToDevice, s);
  if (!rc) rc = gb::zgetrs_dev<R>(notran ? 0 : (tr ? 1 : 2), N, R_, dA.as<C>(), ld, dP.as<int>(), dB.as<C>(), ld, s);
  if (!rc) rc = d2h(hb, *ldb, dB.as<C>(), ld, N, R_, s);
  if (!rc) rc = finish(s);
  if (rc) device_failure(name, rc, info);
}

template <typename R>
void zgesv_host(const char* name, const lapack_int* n, const lapack_int* nrhs, void* a, const lapack_int* lda,
                lapack_int* ipiv, void* b, const lapack_int* ldb, lapack_int* info) {
  // SRC/zgesv.f:148-177: the solve only when the factorization succeeded
  using C = gb::cpx<R>;
  *info = 0;
  if (*n < 0) *info = -1;
  else if (*nrhs < 0) *info = -2;
  else if (*lda < std::max(1, *n)) *info = -4;
  else if (*ldb < std::max(1, *n)) *info = -7;
  if (*info != 0) { call_xerbla(name, -*info); return; }
  if (*n == 0) return;
  cudaStream_t s = thread_stream();
  const int N = *n, R_ = *nrhs, ld = ld_dev(N);
  DevScratch dA(sizeof(C) * (size_t)ld * N, s), dB(sizeof(C) * (size_t)ld * std::max(R_, 1), s),
      dP(sizeof(int) * N, s);
  if (!dA.p || !dB.p || !dP.p) { device_failure(name, (int)cudaErrorMemoryAllocation, info); return; }
  C* ha = static_cast<C*>(a);
  C* hb = static_cast<C*>(b);
  int inf = 0;
  int rc = h2d(dA.as<C>(), ld, ha, *lda, N, N, s);
  if (!rc) rc = h2d(dB.as<C>(), ld, static_cast<const C*>(hb), *ldb, N, R_, s);
  if (!rc) rc = gb::zgetrf_dev<R>(N, N, dA.as<C>(), ld, dP.as<int>(), 64, &inf, s);
  if (!rc && inf == 0) rc = gb::zgetrs_dev<R>(0, N, R_, dA.as<C>(), ld, dP.as<int>(), dB.as<C>(), ld, s);
  if (!rc) rc = d2h(ha, *lda, dA.as<C>(), ld, N, N, s);
  if (!rc) rc = (int)cudaMemcpyAsync(ipiv, dP.p, sizeof(int) * N, cudaMemcpyDeviceToHost, s);
  if (!rc && inf == 0) rc = d2h(hb, *ldb, dB.as<C>(), ld, N, R_, s);
  if (!rc) rc = finish(s);
  if (rc) { device_failure(name, rc, info); return; }
  *info = inf;
}

extern "C" {

__attribute__((weak)) void xerbla_(const char* srname, const lapack_int* info, size_t len) {
  char nm[16] = {0};
  size_t l = std::min<size_t>(len, 15);
  memcpy(nm, srname, l);
  while (l > 0 && nm[l - 1] == ' ') nm[--l] = 0;
  {
    std::lock_guard<std::mutex> lk(g_xerbla_mu);
    memcpy(g_xerbla_name, nm, 16);
    g_xerbla_info = *info;
    if (g_xerbla_capture) return;
  }
  // SRC/xerbla.f:86-88
  printf(" ** On entry to %s parameter number %2d had an illegal value\n", nm, *info);
  fflush(stdout);
  exit(0);
}

void gb300_xerbla_capture(int on) {
  std::lock_guard<std::mutex> lk(g_xerbla_mu);
  g_xerbla_capture = on;
  g_xerbla_info = 0;
  g_xerbla_name[0] = 0;
}

int gb300_xerbla_last(char* name, int cap) {
  std::lock_guard<std::mutex> lk(g_xerbla_mu);
  if (name && cap > 0) snprintf(name, (size_t)cap, "%s", g_xerbla_name);
  return g_xerbla_info;
}

const char* gb300_version(void) { return "lapack_gb300 0.1 (sm_103a)"; }

void dgetrf_(const lapack_int* m, const lapack_int* n, double* a, const lapack_int* lda, lapack_int* ipiv,
             lapack_int* info) {
  getrf_host<double>("DGETRF", m, n, a, lda, ipiv, info, options().nb_f64, 0);
}
void sgetrf_(const lapack_int* m, const lapack_int* n, float* a, const lapack_int* lda, lapack_int* ipiv,
             lapack_int* info) {
  getrf_host<float>("SGETRF", m, n, a, lda, ipiv, info, options().nb_f32, options().sgetrf_mode);
}
// DGETRF2 is the unblocked recursive panel routine of the reference; on the
// GPU it runs the same recursion without an outer blocking loop.
void dgetrf2_(const lapack_int* m, const lapack_int* n, double* a, const lapack_int* lda, lapack_int* ipiv,
              lapack_int* info) {
  getrf_host<double>("DGETRF2", m, n, a, lda, ipiv, info, std::max(1, std::min(*m, *n)), 0);
}
void sgetrf2_(const lapack_int* m, const lapack_int* n, float* a, const lapack_int* lda, lapack_int* ipiv,
              lapack_int* info) {
  getrf_host<float>("SGETRF2", m, n, a, lda, ipiv, info, std::max(1, std::min(*m, *n)), options().sgetrf_mode);
}
void dgetrs_(const char* trans, const lapack_int* n, const lapack_int* nrhs, const double* a, const lapack_int* lda,
             const lapack_int* ipiv, double* b, const lapack_int* ldb, lapack_int* info, size_t) {
  getrs_host<double>("DGETRS", trans, n, nrhs, a, lda, ipiv, b, ldb, info);
}
void sgetrs_(const char* trans, const lapack_int* n, const lapack_int* nrhs, const float* a, const lapack_int* lda,
             const lapack_int* ipiv, float* b, const lapack_int* ldb, lapack_int* info, size_t) {
  getrs_host<float>("SGETRS", trans, n, nrhs, a, lda, ipiv, b, ldb, info);
}
void dgesv_(const lapack_int* n, const lapack_int* nrhs, double* a, const lapack_int* lda, lapack_int* ipiv,
            double* b, const lapack_int* ldb, lapack_int* info) {
  gesv_host<double>("DGESV ", n, nrhs, a, lda, ipiv, b, ldb, info, options().nb_f64, 0);
}
void sgesv_(const lapack_int* n, const lapack_int* nrhs, float* a, const lapack_int* lda, lapack_int* ipiv,
            float* b, const lapack_int* ldb, lapack_int* info) {
  gesv_host<float>("SGESV ", n, nrhs, a, lda, ipiv, b, ldb, info, options().nb_f32, options().sgetrf_mode);
}
void dlaswp_(const lapack_int* n, double* a, const lapack_int* lda, const lapack_int* k1, const lapack_int* k2,
             const lapack_int* ipiv, const lapack_int* incx) {
  laswp_host<double>(n, a, lda, k1, k2, ipiv, incx);
}
void slaswp_(const lapack_int* n, float* a, const lapack_int* lda, const lapack_int* k1, const lapack_int* k2,
             const lapack_int* ipiv, const lapack_int* incx) {
  laswp_host<float>(n, a, lda, k1, k2, ipiv, incx);
}

void dsgesv_(const lapack_int* n, const lapack_int* nrhs, double* a, const lapack_int* lda, lapack_int* ipiv,
             const double* b, const lapack_int* ldb, double* x, const lapack_int* ldx, double*, float*,
             lapack_int* iter, lapack_int* info) {
  *info = 0;
  *iter = 0;
  if (*n < 0) *info = -1;
  else if (*nrhs < 0) *info = -2;
  else if (*lda < std::max(1, *n)) *info = -4;
  else if (*ldb < std::max(1, *n)) *info = -7;
  else if (*ldx < std::max(1, *n)) *info = -9;
  if (*info != 0) { call_xerbla("DSGESV", -*info); return; }
  if (*n == 0) return;
  cudaStream_t s = thread_stream();
  const int N = *n, R = *nrhs, ld = ld_dev(N);
  Carve cv;
  const size_t oA = cv.add(sizeof(double) * (size_t)ld * N), oB = cv.add(sizeof(double) * (size_t)ld * std::max(R, 1)),
               oX = cv.add(sizeof(double) * (size_t)ld * std::max(R, 1)), oP = cv.add(sizeof(int) * N);
  cv.base = host_workspace(cv.off, s);
  if (!cv.base) { device_failure("DSGESV", (int)cudaErrorMemoryAllocation, info); return; }
  double* dA = cv.at<double>(oA);
  double* dB = cv.at<double>(oB);
  double* dX = cv.at<double>(oX);
  int* dP = cv.at<int>(oP);
  int it = 0, inf = 0;
  int rc;
  if (gb::options().feed) {
    // A and B are copied inside: A in column chunks that the FP32
    // factorization takes in as they land
    const gb::HostOperands host{a, *lda, b, *ldb};
    rc = gb::dsgesv_dev(N, R, dA, ld, dP, dB, ld, dX, ld, &it, &inf, s, &host);
  } else {
    gb::prof_begin(gb::kProfCopyH2D, s);
    rc = h2d(dA, ld, a, *lda, N, N, s);
    if (!rc) rc = h2d(dB, ld, b, *ldb, N, R, s);
    gb::prof_end(gb::kProfCopyH2D, s, 0.0, 8.0 * (double)N * (N + R));
    if (!rc) rc = gb::dsgesv_dev(N, R, dA, ld, dP, dB, ld, dX, ld, &it, &inf, s);
  }
  if (!rc) rc = finish(s);
  // A is returned unchanged when ITER >= 0 and holds the FP64 LU otherwise
  gb::prof_begin(gb::kProfCopyD2H, s);
  if (!rc && it < 0) rc = d2h(a, *lda, dA, ld, N, N, s);
  if (!rc && inf == 0) rc = d2h(x, *ldx, dX, ld, N, R, s);
  if (!rc) rc = (int)cudaMemcpyAsync(ipiv, dP, sizeof(int) * N, cudaMemcpyDeviceToHost, s);
  gb::prof_end(gb::kProfCopyD2H, s, 0.0, 8.0 * (double)N * ((it < 0 ? N : 0) + R) + 4.0 * N);
  if (!rc) rc = finish(s);
  if (rc) { device_failure("DSGESV", rc, info); return; }
  *iter = it;
  *info = inf;
}

void dgerfs_(const char* trans, const lapack_int* n, const lapack_int* nrhs, const double* a, const lapack_int* lda,
             const double* af, const lapack_int* ldaf, const lapack_int* ipiv, const double* b, const lapack_int* ldb,
             double* x, const lapack_int* ldx, double* ferr, double* berr, double*, lapack_int*, lapack_int* info,
             size_t) {
  // argument checks of SRC/dgerfs.f:239-261
  *info = 0;
  const bool notran = lsame(*trans, 'N');
  if (!notran && !lsame(*trans, 'T') && !lsame(*trans, 'C')) *info = -1;
  else if (*n < 0) *info = -2;
  else if (*nrhs < 0) *info = -3;
  else if (*lda < std::max(1, *n)) *info = -5;
  else if (*ldaf < std::max(1, *n)) *info = -7;
  else if (*ldb < std::max(1, *n)) *info = -10;
  else if (*ldx < std::max(1, *n)) *info = -12;
  if (*info != 0) { call_xerbla("DGERFS", -*info); return; }
  if (*n == 0 || *nrhs == 0) {
    for (int j = 0; j < *nrhs; ++j) ferr[j] = berr[j] = 0.0;
    return;
  }
  cudaStream_t s = thread_stream();
  const int N = *n, R = *nrhs, ld = ld_dev(N);
  DevScratch dA(sizeof(double) * (size_t)ld * N, s), dAF(sizeof(double) * (size_t)ld * N, s),
      dB(sizeof(double) * (size_t)ld * R, s), dX(sizeof(double) * (size_t)ld * R, s),
      dE(sizeof(double) * 2 * (size_t)R, s), dP(sizeof(int) * N, s);
  if (!dA.p || !dAF.p || !dB.p || !dX.p || !dE.p || !dP.p) {
    device_failure("DGERFS", (int)cudaErrorMemoryAllocation, info);
    return;
  }
  double* dF = dE.as<double>();
  int rc = h2d(dA.as<double>(), ld, a, *lda, N, N, s);
  if (!rc) rc = h2d(dAF.as<double>(), ld, af, *ldaf, N, N, s);
  if (!rc) rc = h2d(dB.as<double>(), ld, b, *ldb, N, R, s);
  if (!rc) rc = h2d(dX.as<double>(), ld, x, *ldx, N, R, s);
  if (!rc) rc = (int)cudaMemcpyAsync(dP.p, ipiv, sizeof(int) * N, cudaMemcpyHostToDevice, s);
  if (!rc) rc = gb::dgerfs_dev(notran ? 'N' : 'T', N, R, dA.as<double>(), ld, dAF.as<double>(), ld, dP.as<int>(),
                               dB.as<double>(), ld, dX.as<double>(), ld, dF, dF + R, s);
  if (!rc) rc = d2h(x, *ldx, dX.as<double>(), ld, N, R, s);
  if (!rc) rc = (int)cudaMemcpyAsync(ferr, dF, sizeof(double) * R, cudaMemcpyDeviceToHost, s);
  if (!rc) rc = (int)cudaMemcpyAsync(berr, dF + R, sizeof(double) * R, cudaMemcpyDeviceToHost, s);
  if (!rc) rc = finish(s);
  if (rc) device_failure("DGERFS", rc, info);
}

void dgecon_(const char* norm, const lapack_int* n, const double* a, const lapack_int* lda, const double* anorm,
             double* rcond, double*, lapack_int*, lapack_int* info, size_t) {
  // argument checks of SRC/dgecon.f:183-195
  *info = 0;
  const bool onenrm = *norm == '1' || lsame(*norm, 'O');
  if (!onenrm && !lsame(*norm, 'I')) *info = -1;
  else if (*n < 0) *info = -2;
  else if (*lda < std::max(1, *n)) *info = -4;
  else if (*anorm < 0.0) *info = -5;
  if (*info != 0) { call_xerbla("DGECON", -*info); return; }
  if (*n == 0 || *anorm == 0.0 || *anorm != *anorm || *anorm > 1.7976931348623157e308) {
    int inf = 0;
    gb::dgecon_dev(onenrm ? '1' : 'I', *n, nullptr, std::max(1, *n), *anorm, rcond, &inf, nullptr);
    *info = inf;
    return;
  }
  cudaStream_t s = thread_stream();
  const int N = *n, ld = ld_dev(N);
  DevScratch dA(sizeof(double) * (size_t)ld * N, s);
  if (!dA.p) { device_failure("DGECON", (int)cudaErrorMemoryAllocation, info); return; }
  int inf = 0;
  int rc = h2d(dA.as<double>(), ld, a, *lda, N, N, s);
  if (!rc) rc = gb::dgecon_dev(onenrm ? '1' : 'I', N, dA.as<double>(), ld, *anorm, rcond, &inf, s);
  if (!rc) rc = finish(s);
  if (rc) { device_failure("DGECON", rc, info); return; }
  *info = inf;
}

namespace {
int latrs_args(char uplo, char trans, char diag, char normin, int n, int lda) {
  // argument checks of SRC/dlatrs.f:287-306
  if (!lsame(uplo, 'U') && !lsame(uplo, 'L')) return -1;
  if (!lsame(trans, 'N') && !lsame(trans, 'T') && !lsame(trans, 'C')) return -2;
  if (!lsame(diag, 'N') && !lsame(diag, 'U')) return -3;
  if (!lsame(normin, 'Y') && !lsame(normin, 'N')) return -4;
  if (n < 0) return -5;
  if (lda < std::max(1, n)) return -7;
  return 0;
}
}  // namespace

void dlatrs_(const char* uplo, const char* trans, const char* diag, const char* normin, const lapack_int* n,
             const double* a, const lapack_int* lda, double* x, double* scale, double* cnorm, lapack_int* info, size_t,
             size_t, size_t, size_t) {
  *info = latrs_args(*uplo, *trans, *diag, *normin, *n, *lda);
  if (*info != 0) { call_xerbla("DLATRS", -*info); return; }
  *scale = 1.0;
  if (*n == 0) return;
  cudaStream_t s = thread_stream();
  const int N = *n, ld = ld_dev(N);
  DevScratch dA(sizeof(double) * (size_t)ld * N, s), dV(sizeof(double) * 2 * (size_t)N, s);
  if (!dA.p || !dV.p) { device_failure("DLATRS", (int)cudaErrorMemoryAllocation, info); return; }
  double* dX = dV.as<double>();
  double* dC = dX + N;
  const bool normin_y = lsame(*normin, 'Y');
  int rc = h2d(dA.as<double>(), ld, a, *lda, N, N, s);
  if (!rc) rc = (int)cudaMemcpyAsync(dX, x, sizeof(double) * N, cudaMemcpyHostToDevice, s);
  if (!rc && normin_y) rc = (int)cudaMemcpyAsync(dC, cnorm, sizeof(double) * N, cudaMemcpyHostToDevice, s);
  if (!rc) rc = gb::dlatrs_dev(lsame(*uplo, 'U'), !lsame(*trans, 'N'), lsame(*diag, 'U'), normin_y, N,
                               dA.as<double>(), ld, dX, scale, dC, s);
  if (!rc) rc = (int)cudaMemcpyAsync(x, dX, sizeof(double) * N, cudaMemcpyDeviceToHost, s);
  if (!rc) rc = (int)cudaMemcpyAsync(cnorm, dC, sizeof(double) * N, cudaMemcpyDeviceToHost, s);
  if (!rc) rc = finish(s);
  if (rc) device_failure("DLATRS", rc, info);
}

namespace {
// DGESVX argument checks (SRC/dgesvx.f:375-430); for FACT = 'F' also the
// condition numbers of the given scalings.  Returns INFO (0 or negative).
int gesvx_args(char fact, char trans, int n, int nrhs, int lda, int ldaf, char equed, const double* r,
               const double* c, int ldb, int ldx, bool host_scalings, double* rowcnd, double* colcnd,
               cudaStream_t s, int* err) {
  const bool nofact = lsame(fact, 'N'), equil = lsame(fact, 'E');
  bool rowequ = false, colequ = false;
  if (!nofact && !equil) {
    rowequ = lsame(equed, 'R') || lsame(equed, 'B');
    colequ = lsame(equed, 'C') || lsame(equed, 'B');
  }
  *err = 0;
  if (!nofact && !equil && !lsame(fact, 'F')) return -1;
  if (!lsame(trans, 'N') && !lsame(trans, 'T') && !lsame(trans, 'C')) return -2;
  if (n < 0) return -3;
  if (nrhs < 0) return -4;
  if (lda < std::max(1, n)) return -6;
  if (ldaf < std::max(1, n)) return -8;
  if (lsame(fact, 'F') && !(rowequ || colequ || lsame(equed, 'N'))) return -10;
  if (rowequ) {
    const int bad = host_scalings ? gb::scalings_cnd_seq(n, r, rowcnd) : gb::scalings_cnd_dev(n, r, rowcnd, s, err);
    if (*err) return 0;
    if (bad) return -11;
  }
  if (colequ) {
    const int bad = host_scalings ? gb::scalings_cnd_seq(n, c, colcnd) : gb::scalings_cnd_dev(n, c, colcnd, s, err);
    if (*err) return 0;
    if (bad) return -12;
  }
  if (ldb < std::max(1, n)) return -14;
  if (ldx < std::max(1, n)) return -16;
  return 0;
}
}  // namespace

void dgesvx_(const char* fact, const char* trans, const lapack_int* n, const lapack_int* nrhs, double* a,
             const lapack_int* lda, double* af, const lapack_int* ldaf, lapack_int* ipiv, char* equed, double* r,
             double* c, double* b, const lapack_int* ldb, double* x, const lapack_int* ldx, double* rcond,
             double* ferr, double* berr, double* work, lapack_int*, lapack_int* info, size_t, size_t, size_t) {
  double rowcnd = 1.0, colcnd = 1.0;
  int err = 0;
  *info = gesvx_args(*fact, *trans, *n, *nrhs, *lda, *ldaf, *equed, r, c, *ldb, *ldx, true, &rowcnd, &colcnd,
                     nullptr, &err);
  if (*info != 0) { call_xerbla("DGESVX", -*info); return; }
  const bool factored = lsame(*fact, 'F'), equil = lsame(*fact, 'E');
  const int N = *n, R = *nrhs, ld = ld_dev(N);
  cudaStream_t s = thread_stream();
  const size_t nn = (size_t)ld * std::max(N, 1), nr = (size_t)ld * std::max(R, 1);
  DevScratch dA(sizeof(double) * nn, s), dAF(sizeof(double) * nn, s), dB(sizeof(double) * nr, s),
      dX(sizeof(double) * nr, s), dV(sizeof(double) * (2 * (size_t)std::max(N, 1) + 2 * (size_t)std::max(R, 1)), s),
      dP(sizeof(int) * std::max(N, 1), s);
  if (!dA.p || !dAF.p || !dB.p || !dX.p || !dV.p || !dP.p) {
    device_failure("DGESVX", (int)cudaErrorMemoryAllocation, info);
    return;
  }
  double* dR = dV.as<double>();
  double* dC = dR + std::max(N, 1);
  double* dF = dC + std::max(N, 1);
  double* dBe = dF + std::max(R, 1);
  int rc = h2d(dA.as<double>(), ld, a, *lda, N, N, s);
  if (!rc) rc = h2d(dB.as<double>(), ld, b, *ldb, N, R, s);
  if (!rc && N > 0) rc = (int)cudaMemcpyAsync(dR, r, sizeof(double) * N, cudaMemcpyHostToDevice, s);
  if (!rc && N > 0) rc = (int)cudaMemcpyAsync(dC, c, sizeof(double) * N, cudaMemcpyHostToDevice, s);
  if (!rc && factored) rc = h2d(dAF.as<double>(), ld, af, *ldaf, N, N, s);
  if (!rc && factored && N > 0) rc = (int)cudaMemcpyAsync(dP.p, ipiv, sizeof(int) * N, cudaMemcpyHostToDevice, s);
  char eq = factored ? *equed : 'N';
  double rcnd = 0.0, rpv = 1.0;
  int inf = 0;
  if (!rc) rc = gb::dgesvx_dev(*fact, lsame(*trans, 'N') ? 'N' : 'T', N, R, dA.as<double>(), ld, dAF.as<double>(),
                               ld, dP.as<int>(), &eq, dR, dC, dB.as<double>(), ld, dX.as<double>(), ld, rowcnd,
                               colcnd, &rcnd, dF, dBe, &rpv, &inf, s);
  if (!rc) rc = finish(s);
  if (!rc && equil) rc = d2h(a, *lda, dA.as<double>(), ld, N, N, s);
  if (!rc && !factored) rc = d2h(af, *ldaf, dAF.as<double>(), ld, N, N, s);
  if (!rc && !factored && N > 0) rc = (int)cudaMemcpyAsync(ipiv, dP.p, sizeof(int) * N, cudaMemcpyDeviceToHost, s);
  if (!rc && equil && N > 0) rc = (int)cudaMemcpyAsync(r, dR, sizeof(double) * N, cudaMemcpyDeviceToHost, s);
  if (!rc && equil && N > 0) rc = (int)cudaMemcpyAsync(c, dC, sizeof(double) * N, cudaMemcpyDeviceToHost, s);
  // B comes back in every case: it is scaled before the factorization
  // (SRC/dgesvx.f:492-508, before DGETRF at :515), so a singular U leaves it
  // scaled as well
  const bool solved = inf == 0 || inf == N + 1;
  if (!rc) rc = d2h(b, *ldb, dB.as<double>(), ld, N, R, s);
  if (!rc && solved) rc = d2h(x, *ldx, dX.as<double>(), ld, N, R, s);
  if (!rc && solved && R > 0) rc = (int)cudaMemcpyAsync(ferr, dF, sizeof(double) * R, cudaMemcpyDeviceToHost, s);
  if (!rc && solved && R > 0) rc = (int)cudaMemcpyAsync(berr, dBe, sizeof(double) * R, cudaMemcpyDeviceToHost, s);
  if (!rc) rc = finish(s);
  if (rc) { device_failure("DGESVX", rc, info); return; }
  if (!factored) *equed = eq;
  *rcond = rcnd;
  work[0] = rpv;
  *info = inf;
}

void dgetri_(const lapack_int* n, double* a, const lapack_int* lda, const lapack_int* ipiv, double* work,
             const lapack_int* lwork, lapack_int* info) {
  // SRC/dgetri.f:169-197: workspace query and argument checks; NB is the
  // library's FP64 block size (64 by default, ILAENV's value)
  *info = 0;
  int nb = options().nb_f64;
  const int N = *n;
  work[0] = (double)std::max(1, N * nb);
  const bool lquery = (*lwork == -1);
  if (N < 0) *info = -1;
  else if (*lda < std::max(1, N)) *info = -3;
  else if (*lwork < std::max(1, N) && !lquery) *info = -6;
  if (*info != 0) { call_xerbla("DGETRI", -*info); return; }
  if (lquery || N == 0) return;
  int iws = N;
  if (nb > 1 && nb < N) {
    iws = std::max(N * nb, 1);
    if (*lwork < iws) nb = *lwork / N;   // dgetri.f:203-210 (NBMIN = 2 below)
  }
  const int nb_run = (nb < 2) ? 1 : nb;
  cudaStream_t s = thread_stream();
  const int ld = ld_dev(N);
  DevScratch dA(sizeof(double) * (size_t)ld * N, s), dP(sizeof(int) * N, s);
  if (!dA.p || !dP.p) { device_failure("DGETRI", (int)cudaErrorMemoryAllocation, info); return; }
  int inf = 0;
  int rc = h2d(dA.as<double>(), ld, a, *lda, N, N, s);
  if (!rc) rc = (int)cudaMemcpyAsync(dP.p, ipiv, sizeof(int) * N, cudaMemcpyHostToDevice, s);
  if (!rc) rc = gb::dgetri_dev(N, dA.as<double>(), ld, dP.as<int>(), options().nb_f64, nb_run, &inf, s);
  if (!rc && inf == 0) rc = d2h(a, *lda, dA.as<double>(), ld, N, N, s);
  if (!rc) rc = finish(s);
  if (rc) { device_failure("DGETRI", rc, info); return; }
  *info = inf;
  if (inf == 0) work[0] = (double)iws;
}

void dpotrf_(const char* uplo, const lapack_int* n, double* a, const lapack_int* lda, lapack_int* info, size_t) {
  potrf_host<double>("DPOTRF", uplo, n, a, lda, info);
}
void spotrf_(const char* uplo, const lapack_int* n, float* a, const lapack_int* lda, lapack_int* info, size_t) {
  potrf_host<float>("SPOTRF", uplo, n, a, lda, info);
}
void dpotrs_(const char* uplo, const lapack_int* n, const lapack_int* nrhs, const double* a, const lapack_int* lda,
             double* b, const lapack_int* ldb, lapack_int* info, size_t) {
  potrs_host<double>("DPOTRS", uplo, n, nrhs, a, lda, b, ldb, info);
}
void spotrs_(const char* uplo, const lapack_int* n, const lapack_int* nrhs, const float* a, const lapack_int* lda,
             float* b, const lapack_int* ldb, lapack_int* info, size_t) {
  potrs_host<float>("SPOTRS", uplo, n, nrhs, a, lda, b, ldb, info);
}
void dposv_(const char* uplo, const lapack_int* n, const lapack_int* nrhs, double* a, const lapack_int* lda,
            double* b, const lapack_int* ldb, lapack_int* info, size_t) {
  // SRC/dposv.f:130-165
  *info = 0;
  const bool upper = lsame(*uplo, 'U');
  if (!upper && !lsame(*uplo, 'L')) *info = -1;
  else if (*n < 0) *info = -2;
  else if (*nrhs < 0) *info = -3;
  else if (*lda < std::max(1, *n)) *info = -5;
  else if (*ldb < std::max(1, *n)) *info = -7;
  if (*info != 0) { call_xerbla("DPOSV ", -*info); return; }
  if (*n == 0) return;
  cudaStream_t s = thread_stream();
  const int N = *n, R = *nrhs, ld = ld_dev(N);
  DevScratch dA(sizeof(double) * (size_t)ld * N, s), dB(sizeof(double) * (size_t)ld * std::max(R, 1), s);
  if (!dA.p || !dB.p) { device_failure("DPOSV", (int)cudaErrorMemoryAllocation, info); return; }
  int inf = 0;
  int rc = h2d(dA.as<double>(), ld, a, *lda, N, N, s);
  if (!rc) rc = h2d(dB.as<double>(), ld, b, *ldb, N, R, s);
  if (!rc) rc = gb::potrf_dev<double>(upper, N, dA.as<double>(), ld, 64, &inf, s);
  if (!rc && inf == 0) rc = gb::potrs_dev<double>(upper, N, R, dA.as<double>(), ld, dB.as<double>(), ld, s);
  if (!rc) rc = d2h(a, *lda, dA.as<double>(), ld, N, N, s);
  if (!rc && inf == 0) rc = d2h(b, *ldb, dB.as<double>(), ld, N, R, s);
  if (!rc) rc = finish(s);
  if (rc) { device_failure("DPOSV", rc, info); return; }
  *info = inf;
}
void dsposv_(const char* uplo, const lapack_int* n, const lapack_int* nrhs, double* a, const lapack_int* lda,
             const double* b, const lapack_int* ldb, double* x, const lapack_int* ldx, double*, float*,
             lapack_int* iter, lapack_int* info, size_t) {
  // SRC/dsposv.f:209-232
  *info = 0;
  *iter = 0;
  const bool upper = lsame(*uplo, 'U');
  if (!upper && !lsame(*uplo, 'L')) *info = -1;
  else if (*n < 0) *info = -2;
  else if (*nrhs < 0) *info = -3;
  else if (*lda < std::max(1, *n)) *info = -5;
  else if (*ldb < std::max(1, *n)) *info = -7;
  else if (*ldx < std::max(1, *n)) *info = -9;
  if (*info != 0) { call_xerbla("DSPOSV", -*info); return; }
  if (*n == 0) return;
  cudaStream_t s = thread_stream();
  const int N = *n, R = *nrhs, ld = ld_dev(N);
  DevScratch dA(sizeof(double) * (size_t)ld * N, s), dB(sizeof(double) * (size_t)ld * std::max(R, 1), s),
      dX(sizeof(double) * (size_t)ld * std::max(R, 1), s);
  if (!dA.p || !dB.p || !dX.p) { device_failure("DSPOSV", (int)cudaErrorMemoryAllocation, info); return; }
  int it = 0, inf = 0;
  int rc = h2d(dA.as<double>(), ld, a, *lda, N, N, s);
  if (!rc) rc = h2d(dB.as<double>(), ld, b, *ldb, N, R, s);
  if (!rc) rc = gb::dsposv_dev(upper, N, R, dA.as<double>(), ld, dB.as<double>(), ld, dX.as<double>(), ld, &it, &inf,
                               s);
  if (!rc) rc = finish(s);
  // A holds the FP64 factor when the refinement fell back (ITER < 0)
  if (!rc && it < 0) rc = d2h(a, *lda, dA.as<double>(), ld, N, N, s);
  if (!rc && inf == 0) rc = d2h(x, *ldx, dX.as<double>(), ld, N, R, s);
  if (!rc) rc = finish(s);
  if (rc) { device_failure("DSPOSV", rc, info); return; }
  *iter = it;
  *info = inf;
}

// ---------------------------------------------------------------- complex LU
void zgetrf_(const lapack_int* m, const lapack_int* n, void* a, const lapack_int* lda, lapack_int* ipiv,
             lapack_int* info) {
  zgetrf_host<double>("ZGETRF", m, n, a, lda, ipiv, info);
}
void cgetrf_(const lapack_int* m, const lapack_int* n, void* a, const lapack_int* lda, lapack_int* ipiv,
             lapack_int* info) {
  zgetrf_host<float>("CGETRF", m, n, a, lda, ipiv, info);
}
void zgetrf2_(const lapack_int* m, const lapack_int* n, void* a, const lapack_int* lda, lapack_int* ipiv,
              lapack_int* info) {
  zgetrf_host<double>("ZGETRF2", m, n, a, lda, ipiv, info, 1);
}
void cgetrf2_(const lapack_int* m, const lapack_int* n, void* a, const lapack_int* lda, lapack_int* ipiv,
              lapack_int* info) {
  zgetrf_host<float>("CGETRF2", m, n, a, lda, ipiv, info, 1);
}
void zgetrs_(const char* trans, const lapack_int* n, const lapack_int* nrhs, const void* a, const lapack_int* lda,
             const lapack_int* ipiv, void* b, const lapack_int* ldb, lapack_int* info, size_t) {
  zgetrs_host<double>("ZGETRS", trans, n, nrhs, a, lda, ipiv, b, ldb, info);
}
void cgetrs_(const char* trans, const lapack_int* n, const lapack_int* nrhs, const void* a, const lapack_int* lda,
             const lapack_int* ipiv, void* b, const lapack_int* ldb, lapack_int* info, size_t) {
  zgetrs_host<float>("CGETRS", trans, n, nrhs, a, lda, ipiv, b, ldb, info);
}
void zgesv_(const lapack_int* n, const lapack_int* nrhs, void* a, const lapack_int* lda, lapack_int* ipiv, void* b,
            const lapack_int* ldb, lapack_int* info) {
  zgesv_host<double>("ZGESV ", n, nrhs, a, lda, ipiv, b, ldb, info);
}
void cgesv_(const lapack_int* n, const lapack_int* nrhs, void* a, const lapack_int* lda, lapack_int* ipiv, void* b,
            const lapack_int* ldb, lapack_int* info) {
  zgesv_host<float>("CGESV ", n, nrhs, a, lda, ipiv, b, ldb, info);
}
void zcgesv_(const lapack_int* n, const lapack_int* nrhs, void* a, const lapack_int* lda, lapack_int* ipiv,
             const void* b, const lapack_int* ldb, void* x, const lapack_int* ldx, void*, void*, double*,
             lapack_int* iter, lapack_int* info) {
  // SRC/zcgesv.f:259-292
  using gb::zdc;
  *info = 0;
  *iter = 0;
  if (*n < 0) *info = -1;
  else if (*nrhs < 0) *info = -2;
  else if (*lda < std::max(1, *n)) *info = -4;
  else if (*ldb < std::max(1, *n)) *info = -7;
  else if (*ldx < std::max(1, *n)) *info = -9;
  if (*info != 0) { call_xerbla("ZCGESV", -*info); return; }
  if (*n == 0) return;
  cudaStream_t s = thread_stream();
  const int N = *n, R = *nrhs, ld = ld_dev(N);
  DevScratch dA(sizeof(zdc) * (size_t)ld * N, s), dB(sizeof(zdc) * (size_t)ld * std::max(R, 1), s),
      dX(sizeof(zdc) * (size_t)ld * std::max(R, 1), s), dP(sizeof(int) * N, s);
  if (!dA.p || !dB.p || !dX.p || !dP.p) { device_failure("ZCGESV", (int)cudaErrorMemoryAllocation, info); return; }
  zdc* ha = static_cast<zdc*>(a);
  int it = 0, inf = 0;
  int rc = h2d(dA.as<zdc>(), ld, ha, *lda, N, N, s);
  if (!rc) rc = h2d(dB.as<zdc>(), ld, static_cast<const zdc*>(b), *ldb, N, R, s);
  if (!rc) rc = gb::zcgesv_dev(N, R, dA.as<zdc>(), ld, dP.as<int>(), dB.as<zdc>(), ld, dX.as<zdc>(), ld, &it, &inf, s);
  // A holds the COMPLEX*16 factors when the refinement fell back (ITER < 0)
  if (!rc && it < 0) rc = d2h(ha, *lda, dA.as<zdc>(), ld, N, N, s);
  if (!rc) rc = (int)cudaMemcpyAsync(ipiv, dP.p, sizeof(int) * N, cudaMemcpyDeviceToHost, s);
  if (!rc && inf == 0) rc = d2h(static_cast<zdc*>(x), *ldx, dX.as<zdc>(), ld, N, R, s);
  if (!rc) rc = finish(s);
  if (rc) { device_failure("ZCGESV", rc, info); return; }
  *iter = it;
  *info = inf;
}

void dlag2s_(const lapack_int* m, const lapack_int* n, const double* a, const lapack_int* lda, float* sa,
             const lapack_int* ldsa, lapack_int* info) {
  // SRC/dlag2s.f:135-146: no argument checks; conversion in column order
  // stops at the first |a| > SLAMCH('O') with INFO = 1, leaving later
  // elements of SA untouched.
  *info = 0;
  if (*m <= 0 || *n <= 0) return;
  cudaStream_t s = thread_stream();
  const int M = *m, N = *n, ld = ld_dev(M);
  DevScratch dA(sizeof(double) * (size_t)ld * N, s), dS(sizeof(float) * (size_t)ld * N, s);
  if (!dA.p || !dS.p) { device_failure("DLAG2S", (int)cudaErrorMemoryAllocation, info); return; }
  long long first = -1;
  int rc = h2d(dA.as<double>(), ld, a, *lda, M, N, s);
  if (!rc) rc = h2d(dS.as<float>(), ld, sa, *ldsa, M, N, s);   // keeps the untouched tail on overflow
  if (!rc) rc = gb::dlag2s_dev(M, N, dA.as<double>(), ld, dS.as<float>(), ld, &first, s);
  if (!rc) rc = d2h(sa, *ldsa, dS.as<float>(), ld, M, N, s);
  if (!rc) rc = finish(s);
  if (rc) { device_failure("DLAG2S", rc, info); return; }
  *info = first >= 0 ? 1 : 0;
}
void slag2d_(const lapack_int* m, const lapack_int* n, const float* sa, const lapack_int* ldsa, double* a,
             const lapack_int* lda, lapack_int* info) {
  *info = 0;
  if (*m <= 0 || *n <= 0) return;
  cudaStream_t s = thread_stream();
  const int M = *m, N = *n, ld = ld_dev(M);
  DevScratch dA(sizeof(double) * (size_t)ld * N, s), dS(sizeof(float) * (size_t)ld * N, s);
  if (!dA.p || !dS.p) { device_failure("SLAG2D", (int)cudaErrorMemoryAllocation, info); return; }
  int rc = h2d(dS.as<float>(), ld, sa, *ldsa, M, N, s);
  if (!rc) rc = gb::slag2d_dev(M, N, dS.as<float>(), ld, dA.as<double>(), ld, s);
  if (!rc) rc = d2h(a, *lda, dA.as<double>(), ld, M, N, s);
  if (!rc) rc = finish(s);
  if (rc) device_failure("SLAG2D", rc, info);
}

double dlamch_(const char* c, size_t) {
  switch (*c | 0x20) {
    case 'e': return 1.1102230246251565e-16;
    case 's': return 2.2250738585072014e-308;
    case 'o': return 1.7976931348623157e308;
    case 'p': return 2.220446049250313e-16;
    case 'b': return 2.0;
    case 'u': return 2.2250738585072014e-308;
    case 'n': return 53.0;
    case 'r': return 1.0;
    case 'm': return -1021.0;
    case 'l': return 1024.0;
    default: return 0.0;
  }
}
float slamch_(const char* c, size_t) {
  switch (*c | 0x20) {
    case 'e': return 5.96046448e-08f;
    case 's': return 1.17549435e-38f;
    case 'o': return 3.40282347e38f;
    case 'p': return 1.1920929e-07f;
    case 'b': return 2.0f;
    case 'u': return 1.17549435e-38f;
    case 'n': return 24.0f;
    case 'r': return 1.0f;
    case 'm': return -125.0f;
    case 'l': return 128.0f;
    default: return 0.0f;
  }
}

double dlange_(const char* norm, const lapack_int* m, const lapack_int* n, const double* a, const lapack_int* lda,
               double* work, size_t) {
  (void)work;
  if (std::min(*m, *n) <= 0) return 0.0;
  int which;
  if (lsame(*norm, 'M')) which = 0;
  else if (lsame(*norm, 'O') || *norm == '1') which = 1;
  else if (lsame(*norm, 'I')) which = 2;
  else if (lsame(*norm, 'F') || lsame(*norm, 'E')) which = 3;
  else return 0.0;
  cudaStream_t s = thread_stream();
  const int M = *m, N = *n, ld = ld_dev(M);
  DevScratch dA(sizeof(double) * (size_t)ld * N, s);
  if (!dA.p) { device_failure("DLANGE", (int)cudaErrorMemoryAllocation, nullptr); return 0.0; }
  double v = 0.0;
  int err = h2d(dA.as<double>(), ld, a, *lda, M, N, s);
  if (!err) err = gb::dlange_dev(which, M, N, dA.as<double>(), ld, &v, s);
  if (!err) err = finish(s);
  if (err) device_failure("DLANGE", err, nullptr);
  return v;
}

// ------------------------------------------------------ device entry points
int gb300_dgetrf_dev(int m, int n, double* dA, int lda, int* dIpiv, int* info, void* stream) {
  if (m < 0) return -1;
  if (n < 0) return -2;
  if (lda < std::max(1, m)) return -4;
  cudaStream_t s = (cudaStream_t)stream;
  DevScratch di(sizeof(int), s);
  if (!di.p) return (int)cudaErrorMemoryAllocation;
  int rc = gb::getrf_dev<double>(m, n, dA, lda, dIpiv, di.as<int>(), s, 0, options().nb_f64);
  int h = 0;
  if (!rc) rc = (int)cudaMemcpyAsync(&h, di.p, sizeof(int), cudaMemcpyDeviceToHost, s);
  if (!rc) rc = finish(s);
  if (info) *info = h;
  return rc;
}
int gb300_sgetrf_dev(int m, int n, float* dA, int lda, int* dIpiv, int* info, void* stream) {
  if (m < 0) return -1;
  if (n < 0) return -2;
  if (lda < std::max(1, m)) return -4;
  cudaStream_t s = (cudaStream_t)stream;
  DevScratch di(sizeof(int), s);
  if (!di.p) return (int)cudaErrorMemoryAllocation;
  int rc = gb::getrf_dev<float>(m, n, dA, lda, dIpiv, di.as<int>(), s, options().sgetrf_mode, options().nb_f32);
  int h = 0;
  if (!rc) rc = (int)cudaMemcpyAsync(&h, di.p, sizeof(int), cudaMemcpyDeviceToHost, s);
  if (!rc) rc = finish(s);
  if (info) *info = h;
  return rc;
}
int gb300_dgetrs_dev(char trans, int n, int nrhs, const double* dA, int lda, const int* dIpiv, double* dB, int ldb,
                     void* stream) {
  if (!lsame(trans, 'N') && !lsame(trans, 'T') && !lsame(trans, 'C')) return -1;
  if (n < 0) return -2;
  if (nrhs < 0) return -3;
  if (lda < std::max(1, n)) return -5;
  if (ldb < std::max(1, n)) return -8;
  cudaStream_t s = (cudaStream_t)stream;
  int rc = gb::getrs_dev<double>(lsame(trans, 'N') ? 'N' : 'T', n, nrhs, dA, lda, dIpiv, nullptr, dB, ldb, s);
  if (!rc) rc = finish(s);
  return rc;
}
int gb300_sgetrs_dev(char trans, int n, int nrhs, const float* dA, int lda, const int* dIpiv, float* dB, int ldb,
                     void* stream) {
  if (!lsame(trans, 'N') && !lsame(trans, 'T') && !lsame(trans, 'C')) return -1;
  if (n < 0) return -2;
  if (nrhs < 0) return -3;
  if (lda < std::max(1, n)) return -5;
  if (ldb < std::max(1, n)) return -8;
  cudaStream_t s = (cudaStream_t)stream;
  int rc = gb::getrs_dev<float>(lsame(trans, 'N') ? 'N' : 'T', n, nrhs, dA, lda, dIpiv, nullptr, dB, ldb, s);
  if (!rc) rc = finish(s);
  return rc;
}
int gb300_dgesv_dev(int n, int nrhs, double* dA, int lda, int* dIpiv, double* dB, int ldb, int* info, void* stream) {
  if (n < 0) return -1;
  if (nrhs < 0) return -2;
  if (lda < std::max(1, n)) return -4;
  if (ldb < std::max(1, n)) return -7;
  int h = 0;
  int rc = gb300_dgetrf_dev(n, n, dA, lda, dIpiv, &h, stream);
  if (!rc && h == 0 && n > 0 && nrhs > 0) rc = gb300_dgetrs_dev('N', n, nrhs, dA, lda, dIpiv, dB, ldb, stream);
  if (info) *info = h;
  return rc;
}
int gb300_dsgesv_dev(int n, int nrhs, double* dA, int lda, int* dIpiv, const double* dB, int ldb, double* dX,
                     int ldx, int* iter, int* info, void* stream) {
  if (n < 0) return -1;
  if (nrhs < 0) return -2;
  if (lda < std::max(1, n)) return -4;
  if (ldb < std::max(1, n)) return -7;
  if (ldx < std::max(1, n)) return -9;
  cudaStream_t s = (cudaStream_t)stream;
  int it = 0, inf = 0;
  int rc = gb::dsgesv_dev(n, nrhs, dA, lda, dIpiv, dB, ldb, dX, ldx, &it, &inf, s);
  if (!rc) rc = finish(s);
  if (iter) *iter = it;
  if (info) *info = inf;
  return rc;
}

int gb300_dgecon_dev(char norm, int n, const double* dA, int lda, double anorm, double* rcond, int* info,
                     void* stream) {
  const bool onenrm = norm == '1' || lsame(norm, 'O');
  if (!onenrm && !lsame(norm, 'I')) return -1;
  if (n < 0) return -2;
  if (lda < std::max(1, n)) return -4;
  if (anorm < 0.0) return -5;
  cudaStream_t s = (cudaStream_t)stream;
  double r = 0.0;
  int inf = 0;
  int rc = gb::dgecon_dev(onenrm ? '1' : 'I', n, dA, lda, anorm, &r, &inf, s);
  if (!rc) rc = finish(s);
  if (rcond) *rcond = r;
  if (info) *info = inf;
  return rc;
}

int gb300_dlatrs_dev(char uplo, char trans, char diag, char normin, int n, const double* dA, int lda, double* dX,
                     double* scale, double* dCnorm, void* stream) {
  const int bad = latrs_args(uplo, trans, diag, normin, n, lda);
  if (bad) return bad;
  cudaStream_t s = (cudaStream_t)stream;
  double sc = 1.0;
  int rc = gb::dlatrs_dev(lsame(uplo, 'U'), !lsame(trans, 'N'), lsame(diag, 'U'), lsame(normin, 'Y'), n, dA, lda, dX,
                          &sc, dCnorm, s);
  if (!rc) rc = finish(s);
  if (scale) *scale = sc;
  return rc;
}

int gb300_dgesvx_dev(char fact, char trans, int n, int nrhs, double* dA, int lda, double* dAF, int ldaf, int* dIpiv,
                     char* equed, double* dR, double* dC, double* dB, int ldb, double* dX, int ldx, double* rcond,
                     double* dFerr, double* dBerr, double* rpvgrw, int* info, void* stream) {
  cudaStream_t s = (cudaStream_t)stream;
  double rowcnd = 1.0, colcnd = 1.0;
  int err = 0;
  const int bad = gesvx_args(fact, trans, n, nrhs, lda, ldaf, *equed, dR, dC, ldb, ldx, false, &rowcnd, &colcnd, s,
                             &err);
  if (err) return err;
  if (bad) return bad;
  double rc_ = 0.0, rp = 1.0;
  int inf = 0;
  int rc = gb::dgesvx_dev(fact, lsame(trans, 'N') ? 'N' : 'T', n, nrhs, dA, lda, dAF, ldaf, dIpiv, equed, dR, dC, dB,
                          ldb, dX, ldx, rowcnd, colcnd, &rc_, dFerr, dBerr, &rp, &inf, s);
  if (!rc) rc = finish(s);
  if (rcond) *rcond = rc_;
  if (rpvgrw) *rpvgrw = rp;
  if (info) *info = inf;
  return rc;
}

int gb300_dgetri_dev(int n, double* dA, int lda, const int* dIpiv, int* info, void* stream) {
  if (n < 0) return -1;
  if (lda < std::max(1, n)) return -3;
  cudaStream_t s = (cudaStream_t)stream;
  int inf = 0;
  int rc = gb::dgetri_dev(n, dA, lda, dIpiv, options().nb_f64, options().nb_f64, &inf, s);
  if (!rc) rc = finish(s);
  if (info) *info = inf;
  return rc;
}

int gb300_dpotrf_dev(char uplo, int n, double* dA, int lda, int* info, void* stream) {
  if (!lsame(uplo, 'U') && !lsame(uplo, 'L')) return -1;
  if (n < 0) return -2;
  if (lda < std::max(1, n)) return -4;
  cudaStream_t s = (cudaStream_t)stream;
  int inf = 0;
  int rc = gb::potrf_dev<double>(lsame(uplo, 'U'), n, dA, lda, 64, &inf, s);
  if (!rc) rc = finish(s);
  if (info) *info = inf;
  return rc;
}
int gb300_dpotrs_dev(char uplo, int n, int nrhs, const double* dA, int lda, double* dB, int ldb, void* stream) {
  if (!lsame(uplo, 'U') && !lsame(uplo, 'L')) return -1;
  if (n < 0) return -2;
  if (nrhs < 0) return -3;
  if (lda < std::max(1, n)) return -5;
  if (ldb < std::max(1, n)) return -7;
  cudaStream_t s = (cudaStream_t)stream;
  int rc = gb::potrs_dev<double>(lsame(uplo, 'U'), n, nrhs, dA, lda, dB, ldb, s);
  if (!rc) rc = finish(s);
  return rc;
}
int gb300_dsposv_dev(char uplo, int n, int nrhs, double* dA, int lda, const double* dB, int ldb, double* dX, int ldx,
                     int* iter, int* info, void* stream) {
  if (!lsame(uplo, 'U') && !lsame(uplo, 'L')) return -1;
  if (n < 0) return -2;
  if (nrhs < 0) return -3;
  if (lda < std::max(1, n)) return -5;
  if (ldb < std::max(1, n)) return -7;
  if (ldx < std::max(1, n)) return -9;
  cudaStream_t s = (cudaStream_t)stream;
  int it = 0, inf = 0;
  int rc = gb::dsposv_dev(lsame(uplo, 'U'), n, nrhs, dA, lda, dB, ldb, dX, ldx, &it, &inf, s);
  if (!rc) rc = finish(s);
  if (iter) *iter = it;
  if (info) *info = inf;
  return rc;
}

int gb300_zgetrf_dev(int m, int n, void* dA, int lda, int* dIpiv, int* info, void* stream) {
  if (m < 0) return -1;
  if (n < 0) return -2;
  if (lda < std::max(1, m)) return -4;
  cudaStream_t s = (cudaStream_t)stream;
  int inf = 0;
  int rc = gb::zgetrf_dev<double>(m, n, static_cast<gb::zdc*>(dA), lda, dIpiv, 64, &inf, s);
  if (!rc) rc = finish(s);
  if (info) *info = inf;
  return rc;
}
int gb300_zgetrs_dev(char trans, int n, int nrhs, const void* dA, int lda, const int* dIpiv, void* dB, int ldb,
                     void* stream) {
  const bool notran = lsame(trans, 'N'), tr = lsame(trans, 'T');
  if (!notran && !tr && !lsame(trans, 'C')) return -1;
  if (n < 0) return -2;
  if (nrhs < 0) return -3;
  if (lda < std::max(1, n)) return -5;
  if (ldb < std::max(1, n)) return -8;
  cudaStream_t s = (cudaStream_t)stream;
  int rc = gb::zgetrs_dev<double>(notran ? 0 : (tr ? 1 : 2), n, nrhs, static_cast<const gb::zdc*>(dA), lda, dIpiv,
                                  static_cast<gb::zdc*>(dB), ldb, s);
  if (!rc) rc = finish(s);
  return rc;
}
int gb300_zgesv_dev(int n, int nrhs, void* dA, int lda, int* dIpiv, void* dB, int ldb, int* info, void* stream) {
  if (n < 0) return -1;
  if (nrhs < 0) return -2;
  if (lda < std::max(1, n)) return -4;
  if (ldb < std::max(1, n)) return -7;
  cudaStream_t s = (cudaStream_t)stream;
  int inf = 0;
  int rc = gb::zgetrf_dev<double>(n, n, static_cast<gb::zdc*>(dA), lda, dIpiv, 64, &inf, s);
  if (!rc && inf == 0)
    rc = gb::zgetrs_dev<double>(0, n, nrhs, static_cast<const gb::zdc*>(dA), lda, dIpiv, static_cast<gb::zdc*>(dB),
                                ldb, s);
  if (!rc) rc = finish(s);
  if (info) *info = inf;
  return rc;
}
int gb300_zcgesv_dev(int n, int nrhs, void* dA, int lda, int* dIpiv, const void* dB, int ldb, void* dX, int ldx,
                     int* iter, int* info, void* stream) {
  if (n < 0) return -1;
  if (nrhs < 0) return -2;
  if (lda < std::max(1, n)) return -4;
  if (ldb < std::max(1, n)) return -7;
  if (ldx < std::max(1, n)) return -9;
  cudaStream_t s = (cudaStream_t)stream;
  int it = 0, inf = 0;
  int rc = gb::zcgesv_dev(n, nrhs, static_cast<gb::zdc*>(dA), lda, dIpiv, static_cast<const gb::zdc*>(dB), ldb,
                          static_cast<gb::zdc*>(dX), ldx, &it, &inf, s);
  if (!rc) rc = finish(s);
  if (iter) *iter = it;
  if (info) *info = inf;
  return rc;
}

int gb300_dgerfs_dev(char trans, int n, int nrhs, const double* dA, int lda, const double* dAF, int ldaf,
                     const int* dIpiv, const double* dB, int ldb, double* dX, int ldx, double* dFerr, double* dBerr,
                     void* stream) {
  if (!lsame(trans, 'N') && !lsame(trans, 'T') && !lsame(trans, 'C')) return -1;
  if (n < 0) return -2;
  if (nrhs < 0) return -3;
  if (lda < std::max(1, n)) return -5;
  if (ldaf < std::max(1, n)) return -7;
  if (ldb < std::max(1, n)) return -10;
  if (ldx < std::max(1, n)) return -12;
  cudaStream_t s = (cudaStream_t)stream;
  int rc = gb::dgerfs_dev(lsame(trans, 'N') ? 'N' : 'T', n, nrhs, dA, lda, dAF, ldaf, dIpiv, dB, ldb, dX, ldx, dFerr,
                          dBerr, s);
  if (!rc) rc = finish(s);
  return rc;
}

int gb300_dgemm_update_dev(int m, int n, int k, const double* dA, int lda, const double* dB, int ldb, double* dC,
                           int ldc, void* stream) {
  if (m < 0) return -1;
  if (n < 0) return -2;
  if (k < 0) return -3;
  if (lda < std::max(1, m)) return -5;
  if (ldb < std::max(1, k)) return -7;
  if (ldc < std::max(1, m)) return -9;
  cudaStream_t s = (cudaStream_t)stream;
  int rc = gb::gemm_update_dev<double>(m, n, k, dA, lda, dB, ldb, dC, ldc, s, 0);
  if (!rc) rc = finish(s);
  return rc;
}
int gb300_sgemm_update_dev(int mode, int m, int n, int k, const float* dA, int lda, const float* dB, int ldb,
                           float* dC, int ldc, void* stream) {
  if (m < 0) return -2;
  if (n < 0) return -3;
  if (k < 0) return -4;
  if (lda < std::max(1, m)) return -6;
  if (ldb < std::max(1, k)) return -8;
  if (ldc < std::max(1, m)) return -10;
  cudaStream_t s = (cudaStream_t)stream;
  int rc = gb::gemm_update_dev<float>(m, n, k, dA, lda, dB, ldb, dC, ldc, s,
                                      mode == 0 ? gb::kMixedBf16x3 : gb::kMixedFp32);
  if (!rc) rc = finish(s);
  return rc;
}

int gb300_set_option(const char* name, int value) {
  gb::Options& o = options();
  int old;
  if (!strcmp(name, "exact")) { old = o.exact; o.exact = value != 0; }
  else if (!strcmp(name, "nb64")) { old = o.nb_f64; o.nb_f64 = std::max(1, value); }
  else if (!strcmp(name, "nb32")) { old = o.nb_f32; o.nb_f32 = std::max(1, value); }
  else if (!strcmp(name, "mixed")) { old = o.mixed_mode; o.mixed_mode = value; }
  else if (!strcmp(name, "sgetrf")) { old = o.sgetrf_mode; o.sgetrf_mode = value; }
  else if (!strcmp(name, "panel_ctas64")) { old = o.panel_ctas_f64; o.panel_ctas_f64 = value; }
  else if (!strcmp(name, "panel_ctas32")) { old = o.panel_ctas_f32; o.panel_ctas_f32 = value; }
  else if (!strcmp(name, "cluster_panel")) { old = o.cluster_panel; o.cluster_panel = value; }
  else if (!strcmp(name, "lookahead")) { old = o.lookahead; o.lookahead = value; }
  else if (!strcmp(name, "trsv_inv")) { old = o.trsv_inv; o.trsv_inv = value; }
  else if (!strcmp(name, "gemm_ws")) { old = o.gemm_ws; o.gemm_ws = value; }
  else if (!strcmp(name, "panel_fuse")) { old = o.panel_fuse; o.panel_fuse = value; }
  else if (!strcmp(name, "feed")) { old = o.feed; o.feed = value; }
  else if (!strcmp(name, "feed_lazy")) { old = o.feed_lazy; o.feed_lazy = value; }
  else if (!strcmp(name, "pool_keep")) { old = o.pool_keep; o.pool_keep = value; }
  else if (!strcmp(name, "feed_catchup")) { old = o.feed_catchup; o.feed_catchup = std::max(0, value); }
  else if (!strcmp(name, "gemm_tiles")) { old = o.gemm_tiles; o.gemm_tiles = std::max(0, value); }
  else if (!strcmp(name, "ir_nan_guard")) { old = o.ir_nan_guard; o.ir_nan_guard = value != 0; }
  else return -1;
  return old;
}
int gb300_get_option(const char* name) {
  gb::Options& o = options();
  if (!strcmp(name, "exact")) return o.exact;
  if (!strcmp(name, "nb64")) return o.nb_f64;
  if (!strcmp(name, "nb32")) return o.nb_f32;
  if (!strcmp(name, "mixed")) return o.mixed_mode;
  if (!strcmp(name, "sgetrf")) return o.sgetrf_mode;
  if (!strcmp(name, "panel_ctas64")) return o.panel_ctas_f64;
  if (!strcmp(name, "panel_ctas32")) return o.panel_ctas_f32;
  if (!strcmp(name, "cluster_panel")) return o.cluster_panel;
  if (!strcmp(name, "lookahead")) return o.lookahead;
  if (!strcmp(name, "trsv_inv")) return o.trsv_inv;
  if (!strcmp(name, "gemm_ws")) return o.gemm_ws;
  if (!strcmp(name, "panel_fuse")) return o.panel_fuse;
  if (!strcmp(name, "feed")) return o.feed;
  if (!strcmp(name, "feed_lazy")) return o.feed_lazy;
  if (!strcmp(name, "pool_keep")) return o.pool_keep;
  if (!strcmp(name, "feed_catchup")) return o.feed_catchup;
  if (!strcmp(name, "gemm_tiles")) return o.gemm_tiles;
  if (!strcmp(name, "ir_nan_guard")) return o.ir_nan_guard;
  return -1;
}
int gb300_status(int clear) {
  int* w = gb::device_status_word();
  if (!w) return -1;
  int h = 0;
  cudaMemcpy(&h, w, sizeof(int), cudaMemcpyDeviceToHost);
  if (clear) cudaMemset(w, 0, sizeof(int));
  return h;
}

}  // extern "C"
