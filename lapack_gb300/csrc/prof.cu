// Launch counter, per-kernel-class event timing, and the FP64/FP32
// arithmetic peak probes used as roofline denominators.
#include "prof.h"
#include "../../include/lapack_gb300.h"

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

}  // extern "C"
