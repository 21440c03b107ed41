// Launch counter, per-kernel-class event timing, and the FP64/FP32
// arithmetic peak probes used as roofline denominators.
#include "common.cuh"
#include "prof.h"
#include "../../include/lapack_gb300.h"

#include <cooperative_groups.h>

#include <atomic>
#include <mutex>
#include <vector>

namespace gb {

static std::atomic<long long> g_launches{0};
static bool g_prof = false;
static unsigned g_mask = ~0u;
static std::mutex g_mu;
struct Rec { cudaEvent_t a, b; int kind; double flops, bytes; };
static std::vector<Rec> g_recs;
static std::vector<cudaEvent_t> g_free_events;
static cudaEvent_t g_pending[kProfKinds];

static cudaEvent_t get_event() {
  if (!g_free_events.empty()) { cudaEvent_t e = g_free_events.back(); g_free_events.pop_back(); return e; }
  cudaEvent_t e;
  cudaEventCreate(&e);
  return e;
}

void count_launch(int n) { g_launches.fetch_add(n, std::memory_order_relaxed); }
bool prof_on() { return g_prof; }

void prof_begin(int kind, cudaStream_t s) {
  if (!g_prof || !((g_mask >> kind) & 1u)) return;
  std::lock_guard<std::mutex> lk(g_mu);
  cudaEvent_t e = get_event();
  cudaEventRecord(e, s);
  g_pending[kind] = e;
}

void prof_end(int kind, cudaStream_t s, double flops, double bytes) {
  if (!g_prof || !((g_mask >> kind) & 1u)) return;
  std::lock_guard<std::mutex> lk(g_mu);
  cudaEvent_t e = get_event();
  cudaEventRecord(e, s);
  g_recs.push_back({g_pending[kind], e, kind, flops, bytes});
}

// FMA-chain probes: 8 independent chains per thread, long enough that the
// launch is compute bound; each FMA counts two flops.
template <typename T>
__global__ void probe_fma_kernel(T* out, int iters, T a, T b) {
  T x0 = threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
      x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
    }
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}

// FP64 tensor-core (DMMA) probes: each warp keeps four independent
// accumulator tiles and issues mma.sync back to back.  SHAPE 0 is
// m8n8k4 (512 flop per instruction), SHAPE 1 is m16n8k16 (4096 flop).
template <int SHAPE>
__global__ void probe_dmma_kernel(double* out, int iters) {
  const double a0 = 1.0 + 1e-9 * threadIdx.x, b0 = 1.0 - 1e-9 * threadIdx.x;
  if constexpr (SHAPE == 0) {
    double c[4][2] = {};
    for (int i = 0; i < iters; ++i) {
#pragma unroll
      for (int t = 0; t < 4; ++t)
        asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};"
                     : "+d"(c[t][0]), "+d"(c[t][1])
                     : "d"(a0), "d"(b0));
    }
    double acc = 0;
#pragma unroll
    for (int t = 0; t < 4; ++t) acc += c[t][0] + c[t][1];
    out[blockIdx.x * blockDim.x + threadIdx.x] = acc;
  } else {
    double c[4][4] = {};
    for (int i = 0; i < iters; ++i) {
#pragma unroll
      for (int t = 0; t < 4; ++t)
        asm volatile("mma.sync.aligned.m16n8k16.row.col.f64.f64.f64.f64 {%0,%1,%2,%3}, "
                     "{%4,%5,%6,%7,%8,%9,%10,%11}, {%12,%13,%14,%15}, {%0,%1,%2,%3};"
                     : "+d"(c[t][0]), "+d"(c[t][1]), "+d"(c[t][2]), "+d"(c[t][3])
                     : "d"(a0), "d"(a0), "d"(a0), "d"(a0), "d"(a0), "d"(a0), "d"(a0), "d"(a0), "d"(b0), "d"(b0),
                       "d"(b0), "d"(b0));
    }
    double acc = 0;
#pragma unroll
    for (int t = 0; t < 4; ++t) acc += c[t][0] + c[t][1] + c[t][2] + c[t][3];
    out[blockIdx.x * blockDim.x + threadIdx.x] = acc;
  }
}

// Cluster exchange probe: every iteration is the skeleton of one column of
// the cluster panel leaf without its arithmetic: a CTA-wide barrier, warp 0
// of every CTA pushes a 16-byte message into every CTA of the cluster with
// st.async (counted on the receiver's mbarrier), waits for the G messages
// of the iteration, then a second CTA-wide barrier.  mode 1 replaces the
// push and wait by one cluster barrier.  Waits are bounded; on a timeout
// *bad is set and the probe stops waiting.
__global__ void __launch_bounds__(512, 1) probe_cluster_kernel(int iters, int mode, int* bad) {
  namespace cg = cooperative_groups;
  cg::cluster_group cluster = cg::this_cluster();
  __shared__ __align__(16) uint4 slots[2][16];
  __shared__ __align__(8) uint64_t full[2];
  __shared__ int sink;
  const int b = (int)cluster.block_rank(), G = (int)cluster.num_blocks();
  const int tid = threadIdx.x, lane = tid & 31;
  const uint32_t tx = (uint32_t)(G * 16);
  if (tid == 0) {
    for (int i = 0; i < 2; ++i) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"((uint32_t)__cvta_generic_to_shared(&full[i])));
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    for (int i = 0; i < 2; ++i)
      asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(
                       (uint32_t)__cvta_generic_to_shared(&full[i])),
                   "r"(tx)
                   : "memory");
    sink = 0;
  }
  cluster.sync();
  bool timed_out = false;
  for (int it = 0; it < iters; ++it) {
    const int par = it & 1;
    __syncthreads();
    if (mode == 1) {
      cluster.sync();
    } else if (tid < 32) {
      const uint32_t bar_l = (uint32_t)__cvta_generic_to_shared(&full[par]);
      const uint32_t slot_l = (uint32_t)__cvta_generic_to_shared(&slots[par][b]);
      if (lane < G) {
        uint32_t ra, rb;
        asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(ra) : "r"(slot_l), "r"(lane));
        asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(rb) : "r"(bar_l), "r"(lane));
        asm volatile("st.async.shared::cluster.mbarrier::complete_tx::bytes.v4.b32 [%0], {%1, %2, %3, %4}, [%5];"
                     ::"r"(ra), "r"(it), "r"(b), "r"(0), "r"(0), "r"(rb)
                     : "memory");
      }
      bool ok = true;
      if (!timed_out) {
        ok = false;
        for (unsigned spins = 0; spins < kSpinLimit && !ok; ++spins) {
          uint32_t done;
          asm volatile(
              "{\n .reg .pred p;\n mbarrier.try_wait.parity.acquire.cluster.shared::cta.b64 p, [%1], %2;\n"
              " selp.u32 %0, 1, 0, p;\n}\n"
              : "=r"(done)
              : "r"(bar_l), "r"((uint32_t)((it >> 1) & 1))
              : "memory");
          ok = done != 0;
        }
      }
      ok = __all_sync(0xffffffffu, ok);
      if (!ok && !timed_out) {
        timed_out = true;
        if (lane == 0) atomicExch(bad, 1);
      }
      if (lane == 0) {
        sink += (int)slots[par][(b + 1) % G].x;
        if (it + 2 < iters)
          asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar_l), "r"(tx) : "memory");
      }
    }
    __syncthreads();
  }
  cluster.sync();
  if (tid == 0 && sink == -1) atomicExch(bad, 2);
}

}  // namespace gb

extern "C" {

long long gb300_launch_count(void) { return gb::g_launches.load(); }

unsigned gb300_prof_mask(unsigned mask) {
  unsigned old = gb::g_mask;
  gb::g_mask = mask;
  return old;
}

int gb300_prof_enable(int on) {
  int old = gb::g_prof;
  gb::g_prof = on != 0;
  return old;
}

void gb300_prof_reset(void) {
  std::lock_guard<std::mutex> lk(gb::g_mu);
  for (auto& r : gb::g_recs) { gb::g_free_events.push_back(r.a); gb::g_free_events.push_back(r.b); }
  gb::g_recs.clear();
}

int gb300_prof_read(int kind, double* ms, double* flops, double* bytes, long long* launches) {
  std::lock_guard<std::mutex> lk(gb::g_mu);
  double t = 0, f = 0, by = 0;
  long long n = 0;
  for (auto& r : gb::g_recs) {
    if (r.kind != kind) continue;
    if (cudaEventSynchronize(r.b) != cudaSuccess) return -1;
    float x = 0;
    cudaEventElapsedTime(&x, r.a, r.b);
    t += x; f += r.flops; by += r.bytes; ++n;
  }
  if (ms) *ms = t;
  if (flops) *flops = f;
  if (bytes) *bytes = by;
  if (launches) *launches = n;
  return 0;
}

// Measured arithmetic throughput of this GPU in TFLOP/s: which = 0 FP64
// FMA (DFMA), 1 FP32 FMA (FFMA), 2 FP64 tensor core mma.sync m8n8k4,
// 3 FP64 tensor core mma.sync m16n8k16.  A few tens of milliseconds of work.
double gb300_probe_peak(int which) {
  if (which < 0 || which > 3) return -1.0;
  int dev = 0, nsm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  const int blocks = nsm * 4, threads = 256;
  const int iters = which == 0 ? 2000 : which == 1 ? 20000 : which == 2 ? 1000 : 200;
  void* out = nullptr;
  if (cudaMalloc(&out, sizeof(double) * blocks * threads) != cudaSuccess) return -1.0;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  float best = 1e30f;
  for (int rep = 0; rep < 3; ++rep) {
    cudaEventRecord(e0);
    if (which == 0) gb::probe_fma_kernel<double><<<blocks, threads>>>((double*)out, iters, 0.999999, 1e-7);
    else if (which == 1) gb::probe_fma_kernel<float><<<blocks, threads>>>((float*)out, iters, 0.999999f, 1e-7f);
    else if (which == 2) gb::probe_dmma_kernel<0><<<blocks, threads>>>((double*)out, iters);
    else gb::probe_dmma_kernel<1><<<blocks, threads>>>((double*)out, iters);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    if (rep > 0 && ms < best) best = ms;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  double flops;
  if (which <= 1) flops = 2.0 * 64.0 * iters * (double)blocks * threads;
  else flops = (which == 2 ? 512.0 : 4096.0) * 4.0 * iters * (double)blocks * (threads / 32);
  return flops / (best * 1e-3) / 1e12;
}

// Microseconds per iteration of the cluster exchange probe (see
// probe_cluster_kernel): mode 0 pushed messages, 1 cluster barrier; ctas is
// the cluster size (2 to 16).  Negative on an error or a timed-out wait.
double gb300_probe_cluster_exchange(int ctas, int mode, int iters) {
  if (ctas < 1 || ctas > 16 || iters < 1) return -1.0;
  int* bad = nullptr;
  if (cudaMalloc(&bad, sizeof(int)) != cudaSuccess) return -1.0;
  cudaMemset(bad, 0, sizeof(int));
  if (cudaFuncSetAttribute(gb::probe_cluster_kernel, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) !=
      cudaSuccess) {
    cudaFree(bad);
    return -1.0;
  }
  cudaLaunchConfig_t cfg = {};
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = ctas;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.gridDim = dim3(ctas);
  cfg.blockDim = dim3(512);
  cfg.attrs = at;
  cfg.numAttrs = 1;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  double best = 1e30;
  for (int rep = 0; rep < 3; ++rep) {
    cudaEventRecord(e0);
    cudaLaunchKernelEx(&cfg, gb::probe_cluster_kernel, iters, mode, bad);
    cudaEventRecord(e1);
    if (cudaEventSynchronize(e1) != cudaSuccess) { best = -1.0; break; }
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    if (ms < best) best = ms;
  }
  int hbad = 0;
  cudaMemcpy(&hbad, bad, sizeof(int), cudaMemcpyDeviceToHost);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(bad);
  if (hbad || best < 0) return -1.0;
  return best * 1e3 / iters;
}

}  // extern "C"
