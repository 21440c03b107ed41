// Shared device helpers for the GB300 LU solve library (sm_103a).
#pragma once
#include "fp_convert.h"
#include <cuda_runtime.h>
#include <cstdint>
#include <cstdio>

#include "prof.h"

namespace gb {

// Error status words written by kernels whose waits are bounded.  A wait
// that runs out sets the status and the kernel returns instead of hanging.
enum : int {
  kStatusOk = 0,
  kStatusBarrierTimeout = 1,
  kStatusFlagTimeout = 2,
  kStatusCapacity = 3,
};

// A spin of at most this many polls, with a ~256 ns sleep between polls,
// ends a wait after roughly one to two seconds.
constexpr unsigned kSpinLimit = 1u << 22;

__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ int ld_acquire_s32(const int* p) {
  int v;
  asm volatile("ld.acquire.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release_s32(int* p, int v) {
  asm volatile("st.release.gpu.global.s32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Copies `total` elements, element e from src(e) to dst(e), with NT threads:
// each thread issues U independent loads into registers before storing, so
// the copy pays one memory latency per U elements instead of one per element.
template <int U, int NT, typename T, typename Src, typename Dst>
__device__ __forceinline__ void batched_copy(int total, int tid, Src src, Dst dst) {
  for (int e0 = tid; e0 < total; e0 += U * NT) {
    T v[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int e = e0 + u * NT;
      if (e < total) v[u] = src(e);
    }
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int e = e0 + u * NT;
      if (e < total) dst(e, v[u]);
    }
  }
}

// Loads of data written by other CTAs of the same launch go through L2.
template <typename T>
__device__ __forceinline__ T ldcg(const T* p) { return __ldcg(p); }

// Grid-wide barrier for cooperatively launched (co-resident) grids.
// `counter` is monotonic within one launch and starts at zero; barrier
// number `gen` (0-based) completes when it reaches (gen+1)*gridDim.x.
// Bounded: on timeout, or when another CTA already reported an error,
// it records the status and returns false.
__device__ __forceinline__ bool grid_barrier(unsigned* counter, unsigned gen, int* status) {
  __syncthreads();
  __shared__ int ok_s;
  if (threadIdx.x == 0) {
    __threadfence();
    atomicAdd(counter, 1u);
    const unsigned target = (gen + 1u) * gridDim.x;
    unsigned spins = 0;
    int ok = 1;
    while (ld_acquire_u32(counter) < target) {
      if (++spins > kSpinLimit || *(volatile int*)status != kStatusOk) {
        atomicCAS(status, kStatusOk, kStatusBarrierTimeout);
        ok = 0;
        break;
      }
      __nanosleep(64);
    }
    __threadfence();
    ok_s = ok;
  }
  __syncthreads();
  return ok_s != 0;
}

// c - a*b with (EXACT) a separately rounded product, as the reference
// Fortran computes C + (-b)*a without contraction, or (otherwise) one fused
// multiply-add.
template <bool EXACT>
__device__ __forceinline__ double fnmadd(double a, double b, double c) {
  if constexpr (EXACT) return __dsub_rn(c, __dmul_rn(a, b));
  else return fma(-a, b, c);
}
template <bool EXACT>
__device__ __forceinline__ float fnmadd(float a, float b, float c) {
  if constexpr (EXACT) return __fsub_rn(c, __fmul_rn(a, b));
  else return fmaf(-a, b, c);
}
template <bool EXACT>
__device__ __forceinline__ double fmadd(double a, double b, double c) {
  if constexpr (EXACT) return __dadd_rn(c, __dmul_rn(a, b));
  else return fma(a, b, c);
}
template <bool EXACT>
__device__ __forceinline__ float fmadd(float a, float b, float c) {
  if constexpr (EXACT) return __fadd_rn(c, __fmul_rn(a, b));
  else return fmaf(a, b, c);
}

template <typename T> struct Lim;
template <> struct Lim<double> {
  static __host__ __device__ constexpr double sfmin() { return 2.2250738585072014e-308; }
};
template <> struct Lim<float> {
  static __host__ __device__ constexpr float sfmin() { return 1.17549435e-38f; }
};

// Pivot candidate ordering that reproduces IxAMAX (BLAS/SRC/idamax.f:93-123)
// as a parallel reduction: larger |x| wins, ties go to the smaller row, a NaN
// wins only when it is the first element of the search (cls 2) and is
// otherwise never chosen (cls 0).
template <typename T>
struct Cand {
  T absval;
  int row;   // panel-local row, -1 for "no candidate"
  int cls;   // 2: leading NaN, 1: ordinary value, 0: NaN elsewhere, -1: none
};

template <typename T>
__device__ __forceinline__ bool cand_better(const Cand<T>& a, const Cand<T>& b) {
  if (a.cls != b.cls) return a.cls > b.cls;
  if (a.cls == 1 && a.absval != b.absval) return a.absval > b.absval;
  return a.row < b.row && a.row >= 0;
}

template <typename T>
__device__ __forceinline__ Cand<T> make_cand(T v, int row, int first_row) {
  Cand<T> c;
  c.row = row;
  if (v != v) {
    c.cls = (row == first_row) ? 2 : 0;
    c.absval = 0;
  } else {
    c.cls = 1;
    c.absval = v < 0 ? -v : v;
  }
  return c;
}

template <typename T>
__device__ __forceinline__ Cand<T> shfl_cand(const Cand<T>& c, int src_lane_xor) {
  Cand<T> o;
  o.absval = __shfl_xor_sync(0xffffffffu, c.absval, src_lane_xor);
  o.row = __shfl_xor_sync(0xffffffffu, c.row, src_lane_xor);
  o.cls = __shfl_xor_sync(0xffffffffu, c.cls, src_lane_xor);
  return o;
}

template <typename T>
__device__ __forceinline__ Cand<T> warp_best(Cand<T> c) {
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    Cand<T> o = shfl_cand(c, off);
    if (cand_better(o, c)) c = o;
  }
  return c;
}

// Asynchronous 4- or 8-byte global -> shared copies (cp.async, L1-cached).
template <typename T>
__device__ __forceinline__ void cp_async_elem(T* smem_dst, const T* gsrc) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(smem_dst);
  if constexpr (sizeof(T) == 8)
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(d), "l"(gsrc) : "memory");
  else
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(d), "l"(gsrc) : "memory");
}
// The same with zero fill: `valid` false writes zeros and reads nothing
// (gsrc must still be a mapped address).
template <typename T>
__device__ __forceinline__ void cp_async_elem_zfill(T* smem_dst, const T* gsrc, bool valid) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(smem_dst);
  const int n = valid ? (int)sizeof(T) : 0;
  if constexpr (sizeof(T) == 8)
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;" ::"r"(d), "l"(gsrc), "r"(n) : "memory");
  else
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;" ::"r"(d), "l"(gsrc), "r"(n) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }

// Stages a rows x cols column-major block (leading dimension ld) into shared
// memory at dst[c * ldd + r] with cp.async: warp w takes columns w, w + NT/32,
// ..., its lanes consecutive rows (coalesced reads, no index division).
// The caller commits and waits.
template <typename T, int NT>
__device__ __forceinline__ void stage_cols_async(const T* __restrict__ src, int ld, int rows, int cols,
                                                 T* __restrict__ dst, int ldd, int tid) {
  const int warp = tid >> 5, lane = tid & 31;
  for (int c = warp; c < cols; c += NT / 32) {
    const T* s = src + (size_t)c * ld;
    T* d = dst + (size_t)c * ldd;
    for (int r = lane; r < rows; r += 32) cp_async_elem(d + r, s + r);
  }
}


}  // namespace gb

// Launches a kernel of this library and counts it.
#define GB_LAUNCH(...)        \
  do {                        \
    __VA_ARGS__;              \
    ::gb::count_launch();     \
  } while (0)

#define GB_CUDA_TRY(expr)                                                         \
  do {                                                                            \
    cudaError_t _e = (expr);                                                      \
    if (_e != cudaSuccess) {                                                      \
      fprintf(stderr, "lapack_gb300: CUDA error %s at %s:%d (%s)\n",              \
              cudaGetErrorString(_e), __FILE__, __LINE__, #expr);                 \
      return (int)_e;                                                             \
    }                                                                             \
  } while (0)
