// Host side of the batched uneven-size solver: ordering (counting sort by
// size, largest first), the persistent launch, the per-bucket panel-width
// table and its autotuner.  The launch sequence never synchronises with the
// host, so it can be captured into a CUDA graph.
#include "../../include/lapack_gb300.h"
#include "batched.cuh"
#include "driver.h"
#include "prof.h"

#include <algorithm>
#include <mutex>

namespace gb {
namespace {

std::mutex g_tab_mu;
// optional per-phase cycle counters of the batched kernel (one per device)
bool g_phase_on = false;
unsigned long long* g_phase[64] = {nullptr};

unsigned long long* phase_buffer() {
  int dev = 0;
  if (!g_phase_on || cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return nullptr;
  if (!g_phase[dev]) {
    void* p = nullptr;
    if (cudaMalloc(&p, sizeof(unsigned long long) * kBatPhases) != cudaSuccess) return nullptr;
    cudaMemset(p, 0, sizeof(unsigned long long) * kBatPhases);
    g_phase[dev] = static_cast<unsigned long long*>(p);
  }
  return g_phase[dev];
}
int g_nb_table[2][kBatBuckets] = {
    {16, 16, 16, 16, 16, 16, 16, 16},   // double (capacity 16)
    {16, 32, 32, 32, 32, 32, 32, 32},   // float (capacity 32)
};

template <typename T, bool EXACT>
int launch_batched(BatchArgs<T> a, cudaStream_t s) {
  const int cap = batched_cap<T>();
  const size_t smem = batched_smem_bytes<T>(cap);
  static bool attr[64] = {false};
  int dev = 0;
  cudaGetDevice(&dev);
  if (!attr[dev]) {
    GB_CUDA_TRY(cudaFuncSetAttribute(batched_gesv_kernel<T, EXACT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)smem));
    attr[dev] = true;
  }
  int occ = 0;
  GB_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, batched_gesv_kernel<T, EXACT>, bat_threads<T>(), smem));
  const int grid = std::max(1, std::min(a.batch, device_sm_count() * std::max(1, occ)));
  a.cap = cap;
  prof_begin(kProfOther, s);
  GB_LAUNCH(batched_gesv_kernel<T, EXACT><<<grid, bat_threads<T>(), smem, s>>>(a));
  prof_end(kProfOther, s, 0.0, 0.0);
  return (int)cudaGetLastError();
}

}  // namespace

template <typename T>
int gesv_vbatched_dev(int batch, const int* d_n, const int* d_nrhs, T* const* dA, const int* d_lda, int* const* dIpiv,
                      T* const* dB, const int* d_ldb, int* d_info, int solve, cudaStream_t s) {
  if (batch <= 0) return 0;
  const int dt = sizeof(T) == 8 ? 0 : 1;
  size_t bytes = 0;
  auto carve = [&](size_t b) { size_t off = bytes; bytes += (b + 255) / 256 * 256; return off; };
  const size_t o_order = carve(sizeof(int) * (size_t)batch);
  const size_t o_hist = carve(sizeof(int) * (kBatMaxN + 2));
  const size_t o_queue = carve(sizeof(unsigned));
  const size_t o_tab = carve(sizeof(int) * kBatBuckets);
  DevScratch ws(bytes, s);
  if (!ws.p) return (int)cudaErrorMemoryAllocation;
  char* base = ws.as<char>();
  int* order = reinterpret_cast<int*>(base + o_order);
  int* hist = reinterpret_cast<int*>(base + o_hist);
  unsigned* queue = reinterpret_cast<unsigned*>(base + o_queue);
  int* tab = reinterpret_cast<int*>(base + o_tab);
  int htab[kBatBuckets];
  {
    std::lock_guard<std::mutex> lk(g_tab_mu);
    std::copy(g_nb_table[dt], g_nb_table[dt] + kBatBuckets, htab);
  }
  // the table goes to the device by value, as a kernel parameter, so no
  // host buffer has to outlive an asynchronous (or graph-captured) call
  GB_CUDA_TRY(cudaMemsetAsync(hist, 0, sizeof(int) * (kBatMaxN + 2), s));
  const unsigned g = (unsigned)((batch + 255) / 256);
  GB_LAUNCH(batched_hist_kernel<<<g, 256, 0, s>>>(batch, d_n, hist));
  GB_LAUNCH(batched_scan_kernel<<<1, 32, 0, s>>>(hist));
  GB_LAUNCH(batched_place_kernel<<<g, 256, 0, s>>>(batch, d_n, hist, order));
  GB_LAUNCH(batched_set_table_kernel<<<1, kBatBuckets, 0, s>>>(tab, BucketTable{{htab[0], htab[1], htab[2], htab[3],
                                                                                   htab[4], htab[5], htab[6], htab[7]}}));
  GB_CUDA_TRY(cudaMemsetAsync(queue, 0, sizeof(unsigned), s));
  BatchArgs<T> a{batch, d_n, d_nrhs, dA, d_lda, dIpiv, dB, d_ldb, d_info, order, queue, tab, 0, solve, phase_buffer()};
  return options().exact ? launch_batched<T, true>(a, s) : launch_batched<T, false>(a, s);
}
template int gesv_vbatched_dev<double>(int, const int*, const int*, double* const*, const int*, int* const*,
                                       double* const*, const int*, int*, int, cudaStream_t);
template int gesv_vbatched_dev<float>(int, const int*, const int*, float* const*, const int*, int* const*,
                                      float* const*, const int*, int*, int, cudaStream_t);

void set_batched_table(int dt, const int* tab) {
  std::lock_guard<std::mutex> lk(g_tab_mu);
  const int cap = dt == 0 ? batched_cap<double>() : batched_cap<float>();
  for (int b = 0; b < kBatBuckets; ++b) g_nb_table[dt][b] = std::min(std::max(tab[b], 1), cap);
}
void get_batched_table(int dt, int* tab) {
  std::lock_guard<std::mutex> lk(g_tab_mu);
  std::copy(g_nb_table[dt], g_nb_table[dt] + kBatBuckets, tab);
}

}  // namespace gb

extern "C" {

int gb300_dgesv_vbatched_dev(int batch, const int* d_n, const int* d_nrhs, double* const* dA_array, const int* d_lda,
                             int* const* dIpiv_array, double* const* dB_array, const int* d_ldb, int* d_info,
                             void* stream) {
  if (batch < 0) return -1;
  return gb::gesv_vbatched_dev<double>(batch, d_n, d_nrhs, dA_array, d_lda, dIpiv_array, dB_array, d_ldb, d_info, 1,
                                       (cudaStream_t)stream);
}
int gb300_sgesv_vbatched_dev(int batch, const int* d_n, const int* d_nrhs, float* const* dA_array, const int* d_lda,
                             int* const* dIpiv_array, float* const* dB_array, const int* d_ldb, int* d_info,
                             void* stream) {
  if (batch < 0) return -1;
  return gb::gesv_vbatched_dev<float>(batch, d_n, d_nrhs, dA_array, d_lda, dIpiv_array, dB_array, d_ldb, d_info, 1,
                                      (cudaStream_t)stream);
}
int gb300_dgetrf_vbatched_dev(int batch, const int* d_n, double* const* dA_array, const int* d_lda,
                              int* const* dIpiv_array, int* d_info, void* stream) {
  if (batch < 0) return -1;
  return gb::gesv_vbatched_dev<double>(batch, d_n, nullptr, dA_array, d_lda, dIpiv_array, nullptr, nullptr, d_info,
                                       0, (cudaStream_t)stream);
}
int gb300_vbatched_set_nb(int dtype, const int* table) {
  if (dtype != 0 && dtype != 1) return -1;
  gb::set_batched_table(dtype, table);
  return 0;
}
int gb300_vbatched_profile(int on) {
  const int old = gb::g_phase_on;
  gb::g_phase_on = on != 0;
  return old;
}
int gb300_vbatched_profile_read(unsigned long long* cycles) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return -1;
  for (int i = 0; i < gb::kBatPhases; ++i) cycles[i] = 0;
  if (!gb::g_phase[dev]) return 0;
  if (cudaMemcpy(cycles, gb::g_phase[dev], sizeof(unsigned long long) * gb::kBatPhases, cudaMemcpyDeviceToHost) !=
      cudaSuccess)
    return -1;
  cudaMemset(gb::g_phase[dev], 0, sizeof(unsigned long long) * gb::kBatPhases);
  return 0;
}
int gb300_vbatched_get_nb(int dtype, int* table) {
  if (dtype != 0 && dtype != 1) return -1;
  gb::get_batched_table(dtype, table);
  return 0;
}

}  // extern "C"
