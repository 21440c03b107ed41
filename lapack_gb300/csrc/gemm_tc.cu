// Trailing-matrix update of the FP32 factorization on the BF16 tensor cores
// (tcgen05, sm_103a): C := C - A*B for FP32 column-major A (M x K), B (K x N),
// C (M x N), the SGEMM('N','N', alpha=-1, beta=1) call of SRC/sgetrf.f (or,
// with overwrite, C := A*B, which may alias B: B is split before C is
// written), as
// split-BF16x3 products: with a = ah + al and b = bh + bl (ah = bf16(a),
// al = bf16(a - ah)), a*b ~ ah*bh + ah*bl + al*bh, the three products
// accumulated in FP32 in tensor memory.
//
// Two steps per call:
//  1. split kernels write ah/al and bh/bl as K-major bf16 arrays (row r holds
//     K contiguous values, K padded with zeros to a multiple of 64);
//  2. an MMA kernel: by default the warp-specialised multi-tile kernel
//     described before gemm_bf16x3_ws_kernel below; where C cannot be moved
//     by TMA (C or its column stride not 16-byte aligned, M not a multiple
//     of 4) the one-tile kernel: one CTA per 128 x 128 tile of C.  Per 64-wide K block
//     one thread issues the four TMA loads (128B-swizzled tiles) on an
//     mbarrier, then twelve tcgen05.mma (M=128, N=128, K=16, three products x
//     four K steps) into a 128-column TMEM accumulator, and commits them to a
//     second mbarrier.  The four warps then read the accumulator with
//     tcgen05.ld (warp w owns TMEM lanes 32w..32w+31 = tile rows) and apply
//     C -= acc with coalesced column accesses.  64 KB of shared memory per CTA
//     lets three CTAs share an SM so one CTA's epilogue overlaps another's
//     loads and MMAs.
// Every mbarrier wait is bounded; on timeout the kernel records a status,
// skips the epilogue and still frees its TMEM.
#include "driver.h"
#include "prof.h"
#include "common.cuh"

#include <cuda.h>
#include <cuda_bf16.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <mutex>

namespace gb {
namespace {

constexpr int kTcBM = 128;
constexpr int kTcBN = 128;
constexpr int kTcBK = 64;                      // one 128-byte swizzle row of bf16
constexpr int kTcThreads = 128;
constexpr int kTileBytesA = kTcBM * kTcBK * 2;  // 16 KB
constexpr int kTileBytesB = kTcBN * kTcBK * 2;  // 16 KB
constexpr int kStageBytes = 2 * kTileBytesA + 2 * kTileBytesB;   // hi + lo of A and B
constexpr int kTcSmem = kStageBytes + 1024;    // + alignment slack for the 1024-byte swizzle atoms
constexpr uint32_t kTmemCols = 128;

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
// Bounded parity wait; returns false after ~kSpinLimit polls.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
  const uint32_t a = smem_u32(bar);
  for (unsigned spins = 0; spins < kSpinLimit; ++spins) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(a), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, int x, int y, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];"
      ::"r"(smem_u32(dst)), "l"(map), "r"(x), "r"(y), "r"(smem_u32(bar))
      : "memory");
}

// Shared-memory matrix descriptor of a K-major, 128B-swizzled bf16 tile whose
// rows are 128 bytes and whose 8-row swizzle atoms are 1024 bytes apart.
__device__ __forceinline__ uint64_t smem_desc_sw128(uint32_t addr) {
  uint64_t d = 0;
  d |= (uint64_t)((addr >> 4) & 0x3FFF);           // start address
  d |= (uint64_t)(16 >> 4) << 16;                   // leading byte offset (unused for swizzled K-major)
  d |= (uint64_t)(1024 >> 4) << 32;                 // stride byte offset: next 8-row group
  d |= (uint64_t)1 << 46;                           // descriptor version for tcgen05
  d |= (uint64_t)2 << 61;                           // 128-byte swizzle
  return d;
}

// Instruction descriptor, kind::f16: D = F32, A = B = BF16, both K-major, M x N.
__host__ __device__ constexpr uint32_t idesc_bf16_f32(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void mma_bf16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n"
      ::"r"(tmem_d), "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate));
}

__device__ __forceinline__ void tmem_ld_32cols(uint32_t taddr, float (&v)[32]) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, "
      "%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]),
        "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
        "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

// 32 consecutive columns of row m of C (zero outside the matrix).
__device__ __forceinline__ void load_c_chunk(const float* __restrict__ C, int ldc, int M, int N, int m, int n_beg,
                                             float (&out)[32]) {
#pragma unroll
  for (int j = 0; j < 32; ++j) {
    const int n = n_beg + j;
    out[j] = (m < M && n < N) ? __ldg(C + (size_t)m + (size_t)n * ldc) : 0.f;
  }
}

__global__ void __launch_bounds__(kTcThreads)
gemm_bf16x3_kernel(const __grid_constant__ CUtensorMap tm_ah, const __grid_constant__ CUtensorMap tm_al,
                   const __grid_constant__ CUtensorMap tm_bh, const __grid_constant__ CUtensorMap tm_bl,
                   float* __restrict__ C, int ldc, int M, int N, int nkb, int* __restrict__ status, int overwrite) {
  extern __shared__ unsigned char tc_smem_raw[];
  __shared__ __align__(8) uint64_t bar_load;
  __shared__ __align__(8) uint64_t bar_mma;
  __shared__ uint32_t tmem_slot;
  __shared__ int ok_s;

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int m0 = blockIdx.x * kTcBM, n0 = blockIdx.y * kTcBN;
  // 1024-byte aligned stage: [ah | al | bh | bl]
  const uint32_t raw = smem_u32(tc_smem_raw);
  unsigned char* stage = tc_smem_raw + (((raw + 1023u) & ~1023u) - raw);
  unsigned char* s_ah = stage;
  unsigned char* s_al = stage + kTileBytesA;
  unsigned char* s_bh = stage + 2 * kTileBytesA;
  unsigned char* s_bl = stage + 2 * kTileBytesA + kTileBytesB;

  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_slot)),
                 "r"(kTmemCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (tid == 0) {
    mbar_init(&bar_load, 1);
    mbar_init(&bar_mma, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    ok_s = 1;
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = tmem_slot;
  const int m = m0 + warp * 32 + lane;
  // the first C chunk is fetched while the tensor cores work
  float cpre[32];
  if (!overwrite) load_c_chunk(C, ldc, M, N, m, n0, cpre);

  if (tid == 0) {
    const uint32_t idesc = idesc_bf16_f32(kTcBM, kTcBN);
    const uint32_t a_hi = smem_u32(s_ah), a_lo = smem_u32(s_al), b_hi = smem_u32(s_bh), b_lo = smem_u32(s_bl);
    for (int kb = 0; kb < nkb; ++kb) {
      mbar_expect_tx(&bar_load, kStageBytes);
      tma_load_2d(s_ah, &tm_ah, kb * kTcBK, m0, &bar_load);
      tma_load_2d(s_al, &tm_al, kb * kTcBK, m0, &bar_load);
      tma_load_2d(s_bh, &tm_bh, kb * kTcBK, n0, &bar_load);
      tma_load_2d(s_bl, &tm_bl, kb * kTcBK, n0, &bar_load);
      if (!mbar_wait(&bar_load, kb & 1)) {
        atomicCAS(status, kStatusOk, kStatusFlagTimeout);
        ok_s = 0;
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
#pragma unroll
      for (int kk = 0; kk < kTcBK / 16; ++kk) {
        const uint32_t off = kk * 32;   // 16 bf16 along K = 32 bytes inside the swizzled row
        const uint64_t dah = smem_desc_sw128(a_hi + off), dal = smem_desc_sw128(a_lo + off);
        const uint64_t dbh = smem_desc_sw128(b_hi + off), dbl = smem_desc_sw128(b_lo + off);
        const uint32_t acc0 = (kb > 0 || kk > 0) ? 1u : 0u;
        mma_bf16(tmem, dal, dbh, idesc, acc0);   // small terms first
        mma_bf16(tmem, dah, dbl, idesc, 1u);
        mma_bf16(tmem, dah, dbh, idesc, 1u);
      }
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                       smem_u32(&bar_mma))
                   : "memory");
      // single-stage buffer: the next K block's loads wait for these MMAs
      if (!mbar_wait(&bar_mma, kb & 1)) {
        atomicCAS(status, kStatusOk, kStatusFlagTimeout);
        ok_s = 0;
        break;
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");

  if (ok_s && nkb > 0) {
    // warp w reads TMEM lanes 32w..32w+31 = rows m0 + 32w + lane of the tile;
    // C is read a 32-column chunk ahead of the subtraction (all loads of a
    // chunk issued before any store)
    const uint32_t lane_base = tmem + ((uint32_t)(warp * 32) << 16);
    float nxt[32];
#pragma unroll
    for (int j = 0; j < 32; ++j) nxt[j] = cpre[j];
#pragma unroll 1
    for (int c0 = 0; c0 < kTcBN; c0 += 32) {
      float cur[32];
#pragma unroll
      for (int j = 0; j < 32; ++j) cur[j] = nxt[j];
      if (!overwrite && c0 + 32 < kTcBN) load_c_chunk(C, ldc, M, N, m, n0 + c0 + 32, nxt);
      float v[32];
      tmem_ld_32cols(lane_base + (uint32_t)c0, v);
      if (m < M) {
#pragma unroll
        for (int j = 0; j < 32; ++j) {
          const int n = n0 + c0 + j;
          if (n < N) C[(size_t)m + (size_t)n * ldc] = overwrite ? v[j] : cur[j] - v[j];
        }
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols));
  }
}

// ---------------------------------------------------------------------------
// Warp-specialised form of the same update, several tiles per CTA.
//
// One CTA per SM (224 KB of shared memory) walks tiles t = blockIdx.x +
// i * gridDim.x.  Roles:
//   warp 0  operand producer: TMA loads of ah, al, bh, bl per 64-wide K block
//           into a two-stage ring (64 KB per stage);
//   warp 1  MMA issuer: twelve tcgen05.mma per K block into one of two
//           128-column TMEM accumulators (tile i uses accumulator i & 1), so
//           the next tile's products run while the epilogue drains this one;
//   warp 6  C producer: TMA loads of the C tile in two 128 x 64 halves into a
//           ring of three 32 KB buffers, issued as soon as a buffer is free,
//           so C streams from HBM ahead of the epilogue;
//   warps 2-5 epilogue: warp w owns TMEM lanes 32(w%4)..+31 (tile rows) and
//           the matching 32-row quadrant of each C buffer; it reads the
//           accumulator with tcgen05.ld, forms C - acc in shared memory and
//           writes its quadrant back with a TMA store.
// Every mbarrier wait is bounded.  A wait that runs out records the status
// and raises a CTA-wide abort flag; every role then leaves its loop, the
// producers wait (bounded) for their copies in flight, and TMEM is freed.
constexpr int kWsStages = 2;
constexpr int kWsCBufs = 3;
constexpr int kWsCHalfCols = 64;
constexpr int kWsCHalfBytes = kTcBM * kWsCHalfCols * 4;    // 32 KB
constexpr int kWsCQuadBytes = 32 * kWsCHalfCols * 4;        // 8 KB: 32 rows x 64 columns
constexpr int kWsThreads = 224;
constexpr int kWsSmem = kWsStages * kStageBytes + kWsCBufs * kWsCHalfBytes + 1024;
constexpr uint32_t kWsTmemCols = 256;

struct WsBars {
  uint64_t full[kWsStages], empty[kWsStages];
  uint64_t acc_full[2], acc_empty[2];
  uint64_t c_full[kWsCBufs], c_empty[kWsCBufs];
  uint64_t mma_done;
};

// Bounded wait that also gives up when another role has raised the abort
// flag; returns false then (and sets the flag itself on a timeout).
__device__ __forceinline__ bool ws_wait(uint64_t* bar, uint32_t parity, volatile int* abort_flag, int* status) {
  const uint32_t a = smem_u32(bar);
  for (unsigned spins = 0; spins < kSpinLimit; ++spins) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(a), "r"(parity)
        : "memory");
    if (done) return true;
    if ((spins & 255u) == 255u && *abort_flag) return false;
  }
  *abort_flag = 1;
  atomicCAS(status, kStatusOk, kStatusFlagTimeout);
  return false;
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ void tma_load_2d_hint(void* dst, const CUtensorMap* map, int x, int y, uint64_t* bar,
                                                 uint64_t policy) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes.L2::cache_hint"
      " [%0], [%1, {%2, %3}], [%4], %5;"
      ::"r"(smem_u32(dst)), "l"(map), "r"(x), "r"(y), "r"(smem_u32(bar)), "l"(policy)
      : "memory");
}

__device__ __forceinline__ void tma_store_2d_hint(const CUtensorMap* map, int x, int y, const void* src,
                                                  uint64_t policy) {
  asm volatile(
      "cp.async.bulk.tensor.2d.global.shared::cta.bulk_group.L2::cache_hint [%0, {%1, %2}], [%3], %4;"
      ::"l"(map), "r"(x), "r"(y), "r"(smem_u32(src)), "l"(policy)
      : "memory");
}

__global__ void __launch_bounds__(kWsThreads, 1)
gemm_bf16x3_ws_kernel(const __grid_constant__ CUtensorMap tm_ah, const __grid_constant__ CUtensorMap tm_al,
                      const __grid_constant__ CUtensorMap tm_bh, const __grid_constant__ CUtensorMap tm_bl,
                      const __grid_constant__ CUtensorMap tm_c, int M, int N, int tiles_m, int ntiles,
                      int tiles_per_cta, int nkb, int* __restrict__ status, int overwrite) {
  extern __shared__ unsigned char ws_smem_raw[];
  __shared__ WsBars bars;
  __shared__ uint32_t tmem_slot;
  __shared__ volatile int abort_s;

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const uint32_t raw = smem_u32(ws_smem_raw);
  unsigned char* base = ws_smem_raw + (((raw + 1023u) & ~1023u) - raw);
  unsigned char* stage0 = base;                                          // kWsStages x [ah | al | bh | bl]
  float* cbuf0 = reinterpret_cast<float*>(base + kWsStages * kStageBytes);  // kWsCBufs x 4 quadrants

  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_slot)),
                 "r"(kWsTmemCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (tid == 0) {
    for (int i = 0; i < kWsStages; ++i) {
      mbar_init(&bars.full[i], 1);
      mbar_init(&bars.empty[i], 1);
    }
    for (int i = 0; i < 2; ++i) {
      mbar_init(&bars.acc_full[i], 1);
      mbar_init(&bars.acc_empty[i], 4);     // lane 0 of each epilogue warp
    }
    for (int i = 0; i < kWsCBufs; ++i) {
      mbar_init(&bars.c_full[i], 1);
      mbar_init(&bars.c_empty[i], 4);       // each epilogue warp after its store has read the buffer
    }
    mbar_init(&bars.mma_done, 1);
    abort_s = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = tmem_slot;
  int* st = status;

  if (warp == 0) {
    // ---------------------------------------------------- operand producer
    if (lane == 0) {
      uint64_t keep;
      asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(keep));
      uint32_t it = 0;
      bool ok = true;
      for (int i = 0; i < tiles_per_cta && ok; ++i) {
        const int t = blockIdx.x + i * gridDim.x;
        if (t >= ntiles) break;
        const int m0 = (t % tiles_m) * kTcBM, n0 = (t / tiles_m) * kTcBN;
        for (int kb = 0; kb < nkb; ++kb, ++it) {
          const int s = (int)(it % kWsStages);
          const uint32_t u = it / kWsStages;
          if (!ws_wait(&bars.empty[s], (u & 1u) ^ 1u, &abort_s, st)) { ok = false; break; }
          unsigned char* sb = stage0 + (size_t)s * kStageBytes;
          mbar_expect_tx(&bars.full[s], kStageBytes);
          tma_load_2d_hint(sb, &tm_ah, kb * kTcBK, m0, &bars.full[s], keep);
          tma_load_2d_hint(sb + kTileBytesA, &tm_al, kb * kTcBK, m0, &bars.full[s], keep);
          tma_load_2d_hint(sb + 2 * kTileBytesA, &tm_bh, kb * kTcBK, n0, &bars.full[s], keep);
          tma_load_2d_hint(sb + 2 * kTileBytesA + kTileBytesB, &tm_bl, kb * kTcBK, n0, &bars.full[s], keep);
        }
      }
      if (!ok) {
        // copies in flight land before the CTA may exit
        for (uint32_t j = (it > (uint32_t)kWsStages ? it - kWsStages : 0u); j < it; ++j) {
          volatile int never = 0;
          ws_wait(&bars.full[j % kWsStages], (j / kWsStages) & 1u, &never, st);
        }
      }
    }
  } else if (warp == 6) {
    // ------------------------------------------------------------ C producer
    if (lane == 0) {
      uint64_t stream_pol;
      asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(stream_pol));
      uint32_t cit = 0;
      bool ok = true;
      for (int i = 0; i < tiles_per_cta && ok; ++i) {
        const int t = blockIdx.x + i * gridDim.x;
        if (t >= ntiles) break;
        const int m0 = (t % tiles_m) * kTcBM, n0 = (t / tiles_m) * kTcBN;
        for (int h = 0; h < 2; ++h, ++cit) {
          const int b = (int)(cit % kWsCBufs);
          const uint32_t u = cit / kWsCBufs;
          if (!ws_wait(&bars.c_empty[b], (u & 1u) ^ 1u, &abort_s, st)) { ok = false; break; }
          if (overwrite) {
            mbar_arrive(&bars.c_full[b]);
          } else {
            float* cb = cbuf0 + (size_t)b * (kWsCHalfBytes / 4);
            mbar_expect_tx(&bars.c_full[b], kWsCHalfBytes);
#pragma unroll
            for (int q = 0; q < 4; ++q)
              tma_load_2d_hint(cb + q * (kWsCQuadBytes / 4), &tm_c, m0 + 32 * q, n0 + h * kWsCHalfCols,
                               &bars.c_full[b], stream_pol);
          }
        }
      }
      if (!ok && !overwrite) {
        for (uint32_t j = (cit > (uint32_t)kWsCBufs ? cit - kWsCBufs : 0u); j < cit; ++j) {
          volatile int never = 0;
          ws_wait(&bars.c_full[j % kWsCBufs], (j / kWsCBufs) & 1u, &never, st);
        }
      }
    }
  } else if (warp == 1) {
    // ------------------------------------------------------------ MMA issuer
    if (lane == 0) {
      const uint32_t idesc = idesc_bf16_f32(kTcBM, kTcBN);
      uint32_t it = 0, tl = 0;
      bool ok = true;
      for (int i = 0; i < tiles_per_cta && ok; ++i, ++tl) {
        const int t = blockIdx.x + i * gridDim.x;
        if (t >= ntiles) break;
        const int a = (int)(tl & 1u);
        const uint32_t ua = tl >> 1;
        if (!ws_wait(&bars.acc_empty[a], (ua & 1u) ^ 1u, &abort_s, st)) { ok = false; break; }
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const uint32_t acc = tmem + (uint32_t)(a * kTcBN);
        for (int kb = 0; kb < nkb; ++kb, ++it) {
          const int s = (int)(it % kWsStages);
          const uint32_t u = it / kWsStages;
          if (!ws_wait(&bars.full[s], u & 1u, &abort_s, st)) { ok = false; break; }
          asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
          const uint32_t sb = smem_u32(stage0 + (size_t)s * kStageBytes);
          const uint32_t a_hi = sb, a_lo = sb + kTileBytesA, b_hi = sb + 2 * kTileBytesA,
                         b_lo = sb + 2 * kTileBytesA + kTileBytesB;
#pragma unroll
          for (int kk = 0; kk < kTcBK / 16; ++kk) {
            const uint32_t off = kk * 32;
            const uint64_t dah = smem_desc_sw128(a_hi + off), dal = smem_desc_sw128(a_lo + off);
            const uint64_t dbh = smem_desc_sw128(b_hi + off), dbl = smem_desc_sw128(b_lo + off);
            const uint32_t acc0 = (kb > 0 || kk > 0) ? 1u : 0u;
            mma_bf16(acc, dal, dbh, idesc, acc0);   // small terms first
            mma_bf16(acc, dah, dbl, idesc, 1u);
            mma_bf16(acc, dah, dbh, idesc, 1u);
          }
          asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                           smem_u32(&bars.empty[s]))
                       : "memory");
        }
        if (!ok) break;
        asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                         smem_u32(&bars.acc_full[a]))
                     : "memory");
      }
      // every MMA issued has completed before TMEM is freed
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                       smem_u32(&bars.mma_done))
                   : "memory");
      volatile int never = 0;
      ws_wait(&bars.mma_done, 0, &never, st);
    }
  } else {
    // -------------------------------------------------------------- epilogue
    const int q = warp & 3;                      // TMEM lane quadrant = tile rows 32q..32q+31
    uint64_t stream_pol;
    asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(stream_pol));
    uint32_t cit = 0, tl = 0;
    for (int i = 0; i < tiles_per_cta; ++i, ++tl) {
      const int t = blockIdx.x + i * gridDim.x;
      if (t >= ntiles) break;
      const int m0 = (t % tiles_m) * kTcBM, n0 = (t / tiles_m) * kTcBN;
      const int a = (int)(tl & 1u);
      const uint32_t ua = tl >> 1;
      bool ok = ws_wait(&bars.acc_full[a], ua & 1u, &abort_s, st);
      if (!__all_sync(0xffffffffu, ok)) break;
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint32_t lane_base = tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(a * kTcBN);
      bool fail = false;
      for (int h = 0; h < 2; ++h, ++cit) {
        const int b = (int)(cit % kWsCBufs);
        const uint32_t u = cit / kWsCBufs;
        ok = ws_wait(&bars.c_full[b], u & 1u, &abort_s, st);
        if (!__all_sync(0xffffffffu, ok)) { fail = true; break; }
        float* cq = cbuf0 + (size_t)b * (kWsCHalfBytes / 4) + q * (kWsCQuadBytes / 4);   // [64 cols][32 rows]
#pragma unroll
        for (int j = 0; j < 2; ++j) {
          float v[32];
          tmem_ld_32cols(lane_base + (uint32_t)(h * kWsCHalfCols + j * 32), v);
#pragma unroll
          for (int c = 0; c < 32; ++c) {
            float* p = cq + (j * 32 + c) * 32 + lane;
            *p = overwrite ? v[c] : *p - v[c];
          }
        }
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncwarp();
        if (lane == 0) {
          // quadrants wholly outside C are not stored (the loads there only
          // filled zeros); partial ones are clipped by the tensor map
          if (m0 + 32 * q < M && n0 + h * kWsCHalfCols < N) {
            tma_store_2d_hint(&tm_c, m0 + 32 * q, n0 + h * kWsCHalfCols, cq, stream_pol);
            asm volatile("cp.async.bulk.commit_group;" ::: "memory");
            asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
          }
          mbar_arrive(&bars.c_empty[b]);
        }
        __syncwarp();
      }
      if (fail) break;
      // this warp's reads of accumulator a are complete
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      __syncwarp();
      if (lane == 0) mbar_arrive(&bars.acc_empty[a]);
    }
    if (lane == 0) asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");
    __syncwarp();
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 1) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kWsTmemCols));
  }
}

// A (M x K, column-major) -> ah/al [M][Kp] row-major bf16 (K contiguous),
// through a 32 x 32 shared-memory transpose; zero for k >= K.
__global__ void __launch_bounds__(256)
split_a_kernel(const float* __restrict__ A, int lda, int M, int K, int Kp, __nv_bfloat16* __restrict__ ah,
               __nv_bfloat16* __restrict__ al) {
  __shared__ float t[32][33];
  const int m0 = blockIdx.x * 32, k0 = blockIdx.y * 32;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;   // 32 x 8
  for (int i = ty; i < 32; i += 8) {
    int m = m0 + tx, k = k0 + i;
    t[i][tx] = (m < M && k < K) ? A[(size_t)m + (size_t)k * lda] : 0.f;
  }
  __syncthreads();
  for (int i = ty; i < 32; i += 8) {
    int m = m0 + i, k = k0 + tx;
    if (m < M && k < Kp) {
      float x = t[tx][i];
      __nv_bfloat16 h = __float2bfloat16_rn(x);
      __nv_bfloat16 l = __float2bfloat16_rn(x - __bfloat162float(h));
      ah[(size_t)m * Kp + k] = h;
      al[(size_t)m * Kp + k] = l;
    }
  }
}

// B (K x N, column-major: K contiguous per column) -> bh/bl [N][Kp].
__global__ void __launch_bounds__(256)
split_b_kernel(const float* __restrict__ B, int ldb, int K, int N, int Kp, __nv_bfloat16* __restrict__ bh,
               __nv_bfloat16* __restrict__ bl) {
  size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (size_t)N * Kp) return;
  int n = (int)(e / Kp), k = (int)(e - (size_t)n * Kp);
  float x = k < K ? B[(size_t)k + (size_t)n * ldb] : 0.f;
  __nv_bfloat16 h = __float2bfloat16_rn(x);
  __nv_bfloat16 l = __float2bfloat16_rn(x - __bfloat162float(h));
  bh[e] = h;
  bl[e] = l;
}

PFN_cuTensorMapEncodeTiled_v12000 get_encode() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  });
  return fn;
}

// 2D map over a row-major bf16 array [rows][Kp], box 64 (K) x box_rows.
bool make_map(CUtensorMap* map, const void* base, int rows, int Kp, int box_rows) {
  auto enc = get_encode();
  if (!enc) return false;
  cuuint64_t dims[2] = {(cuuint64_t)Kp, (cuuint64_t)rows};
  cuuint64_t strides[1] = {(cuuint64_t)Kp * 2};
  cuuint32_t box[2] = {(cuuint32_t)kTcBK, (cuuint32_t)box_rows};
  cuuint32_t estr[2] = {1, 1};
  CUresult r = enc(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(base), dims, strides, box, estr,
                   CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                   CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS;
}

// 2D map over a column-major fp32 matrix (rows contiguous), box 32 rows x 64
// columns: one epilogue warp's quadrant of a C half-tile.
bool make_map_c(CUtensorMap* map, const float* base, int M, int N, int ldc) {
  auto enc = get_encode();
  if (!enc) return false;
  cuuint64_t dims[2] = {(cuuint64_t)M, (cuuint64_t)N};
  cuuint64_t strides[1] = {(cuuint64_t)ldc * 4};
  cuuint32_t box[2] = {32u, (cuuint32_t)kWsCHalfCols};
  cuuint32_t estr[2] = {1, 1};
  CUresult r = enc(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<float*>(base), dims, strides, box, estr,
                   CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                   CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS;
}

}  // namespace



size_t bf16x3_split_bytes(int M, int K) {
  const int Kp = (K + kTcBK - 1) / kTcBK * kTcBK;
  return 2 * (((size_t)M * Kp * 2 + 255) / 256 * 256);
}

int bf16x3_split_a_dev(int M, int K, const float* A, int lda, void* buf, Bf16SplitA* out, cudaStream_t s) {
  const int Kp = (K + kTcBK - 1) / kTcBK * kTcBK;
  const size_t half = ((size_t)M * Kp * 2 + 255) / 256 * 256;
  __nv_bfloat16* ah = static_cast<__nv_bfloat16*>(buf);
  __nv_bfloat16* al = reinterpret_cast<__nv_bfloat16*>(static_cast<char*>(buf) + half);
  out->hi = ah;
  out->lo = al;
  out->M = M;
  out->Kp = Kp;
  if (M <= 0 || K <= 0) return 0;
  prof_begin(kProfOther, s);
  dim3 ga((M + 31) / 32, (Kp + 31) / 32);
  GB_LAUNCH(split_a_kernel<<<ga, 256, 0, s>>>(A, lda, M, K, Kp, ah, al));
  prof_end(kProfOther, s, 0.0, 4.0 * (double)M * K + 4.0 * (double)M * Kp);
  return (int)cudaGetLastError();
}

int gemm_bf16x3_dev(int M, int N, int K, const float* A, int lda, const float* B, int ldb, float* C, int ldc,
                    cudaStream_t s, bool overwrite, const Bf16SplitA* a_pre) {
  if (M <= 0 || N <= 0 || K <= 0) return 0;
  const int Kp = (K + kTcBK - 1) / kTcBK * kTcBK;
  if (a_pre && (a_pre->M != M || a_pre->Kp != Kp)) return (int)cudaErrorInvalidValue;
  const size_t bytes_a = a_pre ? 0 : (size_t)M * Kp * 2, bytes_b = (size_t)N * Kp * 2;
  auto up = [](size_t b) { return (b + 255) / 256 * 256; };
  DevScratch ws(2 * up(bytes_a) + 2 * up(bytes_b), s);
  if (!ws.p) return (int)cudaErrorMemoryAllocation;
  char* base = ws.as<char>();
  const __nv_bfloat16* ah = a_pre ? static_cast<const __nv_bfloat16*>(a_pre->hi) : reinterpret_cast<__nv_bfloat16*>(base);
  const __nv_bfloat16* al =
      a_pre ? static_cast<const __nv_bfloat16*>(a_pre->lo) : reinterpret_cast<__nv_bfloat16*>(base + up(bytes_a));
  __nv_bfloat16* bh = reinterpret_cast<__nv_bfloat16*>(base + 2 * up(bytes_a));
  __nv_bfloat16* bl = reinterpret_cast<__nv_bfloat16*>(base + 2 * up(bytes_a) + up(bytes_b));

  // the operand splits are their own class; the update class brackets the
  // tensor-core kernel alone (the roofline's per-launch time)
  prof_begin(kProfOther, s);
  if (!a_pre) {
    dim3 ga((M + 31) / 32, (Kp + 31) / 32);
    GB_LAUNCH(split_a_kernel<<<ga, 256, 0, s>>>(A, lda, M, K, Kp, const_cast<__nv_bfloat16*>(ah),
                                                const_cast<__nv_bfloat16*>(al)));
  }
  size_t nb = (size_t)N * Kp;
  GB_LAUNCH(split_b_kernel<<<(unsigned)((nb + 255) / 256), 256, 0, s>>>(B, ldb, K, N, Kp, bh, bl));
  prof_end(kProfOther, s, 0.0, (a_pre ? 0.0 : 4.0 * (double)M * K + 4.0 * (double)M * Kp) +
                                   4.0 * (double)N * K + 4.0 * (double)N * Kp);

  CUtensorMap m_ah, m_al, m_bh, m_bl;
  if (!make_map(&m_ah, ah, M, Kp, kTcBM) || !make_map(&m_al, al, M, Kp, kTcBM) ||
      !make_map(&m_bh, bh, N, Kp, kTcBN) || !make_map(&m_bl, bl, N, Kp, kTcBN))
    return (int)cudaErrorInvalidValue;
  int dev = 0;
  cudaGetDevice(&dev);
  static bool attr[64] = {false};
  if (dev >= 0 && dev < 64 && !attr[dev]) {
    GB_CUDA_TRY(cudaFuncSetAttribute(gemm_bf16x3_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kTcSmem));
    GB_CUDA_TRY(cudaFuncSetAttribute(gemm_bf16x3_ws_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kWsSmem));
    attr[dev] = true;
  }
  prof_begin(kProfGemmBf16x3, s);
  const int tiles_m = (M + kTcBM - 1) / kTcBM, tiles_n = (N + kTcBN - 1) / kTcBN;
  // the warp-specialised kernel stores C by TMA: C and its column stride
  // must be 16-byte aligned, and so must the end of each column (a TMA
  // store clips the box at the matrix edge in 16-byte units: with M not a
  // multiple of 4 it would also write the rows after M in the last unit)
  CUtensorMap m_c;
  const bool use_ws = options().gemm_ws != 0 && ((uintptr_t)C % 16) == 0 && ((size_t)ldc * 4) % 16 == 0 &&
                      M % 4 == 0 && make_map_c(&m_c, C, M, N, ldc);
  if (use_ws) {
    const int ntiles = tiles_m * tiles_n;
    int tpc = options().gemm_tiles, grid;
    if (tpc <= 0) {
      grid = std::min(ntiles, device_sm_count());
      tpc = (ntiles + grid - 1) / grid;
    } else {
      grid = (ntiles + tpc - 1) / tpc;
    }
    GB_LAUNCH(gemm_bf16x3_ws_kernel<<<grid, kWsThreads, kWsSmem, s>>>(m_ah, m_al, m_bh, m_bl, m_c, M, N, tiles_m,
                                                                      ntiles, tpc, Kp / kTcBK, device_status_word(),
                                                                      overwrite ? 1 : 0));
  } else {
    dim3 grid(tiles_m, tiles_n);
    GB_LAUNCH(gemm_bf16x3_kernel<<<grid, kTcThreads, kTcSmem, s>>>(m_ah, m_al, m_bh, m_bl, C, ldc, M, N, Kp / kTcBK,
                                                                   device_status_word(), overwrite ? 1 : 0));
  }
  prof_end(kProfGemmBf16x3, s, 2.0 * M * N * (double)K,
           4.0 * ((double)M * K + (double)K * N + (overwrite ? 1.0 : 2.0) * M * N));
  return (int)cudaGetLastError();
}

}  // namespace gb
