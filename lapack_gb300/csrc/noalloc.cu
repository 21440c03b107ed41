// gb300_dgetrs_noalloc: DGETRS on device memory without allocating.
//
// Who needs it: a caller that may not allocate GPU memory at the point of the
// solve -- a serving process that reserved its whole device-memory budget at
// start-up and hands the rest to its own pool, a latency-critical loop where
// cudaMalloc/cudaMallocAsync could synchronise or stall, or code running
// inside an allocator callback.  The ordinary gb300_dgetrs_dev takes its
// scratch (row permutation, solve workspace, block flags) from the
// stream-ordered allocator; this variant takes it from one fixed array that
// is part of the library's device image.
//
// The array below (kNoAllocBytes, about 1.1 MB) is reserved on every GPU that
// loads the library and stays there until the process exits.  It bounds the
// problem size: n <= kNoAllocMaxN and n * nrhs <= kNoAllocMaxElems; larger
// calls are rejected with an error code and do nothing.
//
// Every call uses the same array and leaves its last contents there; the
// parts that must start at zero (block flags, ticket, status) are cleared at
// the start of each call.  Two calls whose work overlaps on the GPU (for
// example on two streams) race on the array and give wrong results: issue
// them one after another.
//
// On the first call on a device the library looks up the array's device
// address (cudaGetSymbolAddress) with that device current and sets the
// shared-memory attributes of the kernels it launches; make that first call
// before any stream capture.  Every call reads the kernels' status word back
// and waits for its stream before it returns.  No cudaMalloc, cudaFree or
// allocating library routine is called.
//
// The solution agrees with gb300_dgetrs_dev's to rounding: both solve with
// the same factors, but this variant always uses the blocked solve kernel in
// its default (FMA) form and does not follow the exact-mode option.
#include "../../include/lapack_gb300.h"
#include "common.cuh"
#include "prof.h"
#include "solve_kernels.cuh"

#include <cstdint>
#include <mutex>

namespace gb {
namespace {

constexpr int kNoAllocMaxN = 16384;
constexpr int kNoAllocMaxElems = 131072;          // n * nrhs
constexpr int kNoAllocMaxBlocks = (kNoAllocMaxN + kSolveBS - 1) / kSolveBS;
// layout: [W: doubles][perm: ints][flags: blocks+1 ints][status int]
constexpr size_t kOffW = 0;
constexpr size_t kOffPerm = kOffW + sizeof(double) * (size_t)kNoAllocMaxElems;
constexpr size_t kOffFlags = kOffPerm + sizeof(int) * (size_t)kNoAllocMaxN;
constexpr size_t kOffStatus = kOffFlags + sizeof(int) * (size_t)(kNoAllocMaxBlocks + 1);
constexpr size_t kNoAllocBytes = (kOffStatus + sizeof(int) + 255) / 256 * 256;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

struct DeviceSetup {
  unsigned char* base = nullptr;   // device address of g_noalloc_scratch
  bool done = false;
};
std::mutex g_setup_mu;
DeviceSetup g_setup[64];

// Once per device, with that device current: the array's device address and
// the shared-memory attributes of the permutation and solve kernels.
int setup_device(unsigned char** base) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return (int)e;
  if (dev < 0 || dev >= 64) return (int)cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lk(g_setup_mu);
  if (!g_setup[dev].done) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return (int)e;
    e = cudaFuncSetAttribute(ipiv_to_perm_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)(sizeof(int) * kNoAllocMaxN));
    if (e != cudaSuccess) return (int)e;
    if ((e = trsv_set_smem<double, false, true, true, false>()) != cudaSuccess) return (int)e;
    if ((e = trsv_set_smem<double, false, false, false, false>()) != cudaSuccess) return (int)e;
    if ((e = trsv_set_smem<double, false, true, false, true>()) != cudaSuccess) return (int)e;
    if ((e = trsv_set_smem<double, false, false, true, true>()) != cudaSuccess) return (int)e;
    g_setup[dev].base = static_cast<unsigned char*>(p);
    g_setup[dev].done = true;
  }
  *base = g_setup[dev].base;
  return 0;
}

template <bool FORWARD, bool UNIT, bool TRANS>
int launch_solve(const double* A, int lda, int n, double* W, int nrhs, int* flags, int* status, cudaStream_t s) {
  const int nblk = (n + kSolveBS - 1) / kSolveBS;
  unsigned* ticket = reinterpret_cast<unsigned*>(flags + nblk);
  GB_CUDA_TRY(cudaMemsetAsync(flags, 0, sizeof(int) * (size_t)(nblk + 1), s));
  GB_LAUNCH(trsv_blocked_kernel<double, false, FORWARD, UNIT, TRANS>
            <<<nblk, 256, kTrsvSmem<double>, s>>>(A, lda, n, W, n, nrhs, flags, ticket, status));
  return 0;
}

}  // namespace
}  // namespace gb

extern "C" int gb300_dgetrs_noalloc(char trans, int n, int nrhs, const double* dA, int lda, const int* dIpiv,
                                    double* dB, int ldb, void* stream) {
  using namespace gb;
  const char t = (char)(trans | 0x20);
  if (t != 'n' && t != 't' && t != 'c') return -1;
  if (n < 0) return -2;
  if (nrhs < 0) return -3;
  if (lda < (n > 1 ? n : 1)) return -5;
  if (ldb < (n > 1 ? n : 1)) return -8;
  if (n > kNoAllocMaxN || (long long)n * nrhs > kNoAllocMaxElems) return -100;   // beyond the fixed scratch
  unsigned char* base = nullptr;
  int rc = setup_device(&base);
  if (rc) return rc;
  if (n == 0 || nrhs == 0) return 0;
  cudaStream_t s = (cudaStream_t)stream;
  double* W = reinterpret_cast<double*>(base + kOffW);
  int* perm = reinterpret_cast<int*>(base + kOffPerm);
  int* flags = reinterpret_cast<int*>(base + kOffFlags);
  int* status = reinterpret_cast<int*>(base + kOffStatus);
  GB_CUDA_TRY(cudaMemsetAsync(status, 0, sizeof(int), s));
  GB_LAUNCH(ipiv_to_perm_kernel<true><<<1, 1024, sizeof(int) * (size_t)n, s>>>(dIpiv, 1, n, 1, 0, n, perm, nullptr,
                                                                             status));
  const size_t tot = (size_t)n * nrhs;
  const unsigned blocks = (unsigned)((tot + 255) / 256);
  if (t == 'n') {
    GB_LAUNCH(perm_rows_kernel<double, false><<<blocks, 256, 0, s>>>(dB, ldb, W, n, perm, 0, n, nrhs));
    if ((rc = launch_solve<true, true, false>(dA, lda, n, W, nrhs, flags, status, s))) return rc;
    if ((rc = launch_solve<false, false, false>(dA, lda, n, W, nrhs, flags, status, s))) return rc;
    GB_LAUNCH(copy_cols_kernel<double><<<blocks, 256, 0, s>>>(W, n, dB, ldb, n, nrhs));
  } else {
    GB_LAUNCH(copy_cols_kernel<double><<<blocks, 256, 0, s>>>(dB, ldb, W, n, n, nrhs));
    if ((rc = launch_solve<true, false, true>(dA, lda, n, W, nrhs, flags, status, s))) return rc;
    if ((rc = launch_solve<false, true, true>(dA, lda, n, W, nrhs, flags, status, s))) return rc;
    GB_LAUNCH(perm_rows_kernel<double, true><<<blocks, 256, 0, s>>>(W, n, dB, ldb, perm, 0, n, nrhs));
  }
  int hstatus = 0;
  GB_CUDA_TRY(cudaMemcpyAsync(&hstatus, status, sizeof(int), cudaMemcpyDeviceToHost, s));
  GB_CUDA_TRY(cudaStreamSynchronize(s));
  return hstatus ? 1000 + hstatus : 0;
}
