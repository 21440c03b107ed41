"""A CPU stand-in for running simple CUDA sources of the library in tests.

Kernels whose launches are one-dimensional and whose threads touch disjoint
data (no shared memory, no barriers, shared words only updated by atomicMin
or identical stores) compute the same on the CPU when their blocks and
threads run one after another.  `translate` rewrites every
`kernel<<<grid, block, smem, stream>>>(args)` of such a source into a call of
a sequential launcher; `EMU` stands in for the CUDA runtime calls those
sources make (copies, memsets, synchronisation, stream-ordered scratch as
host memory); `build` compiles the result with g++ into a shared library."""
import os
import re
import subprocess

EMU = r"""
#pragma once
// CPU stand-in for the CUDA runtime calls and kernel launches of a simple source.
#include <cstddef>
#include <cstdlib>
#include <cstring>
#include <cstdio>
#define __global__
#define __launch_bounds__(...)
struct dim3 { unsigned x, y, z; };
static thread_local dim3 blockIdx, threadIdx, blockDim;
typedef void* cudaStream_t;
typedef int cudaError_t;
enum { cudaSuccess = 0, cudaErrorMemoryAllocation = 2 };
enum cudaMemcpyKind { cudaMemcpyHostToDevice, cudaMemcpyDeviceToHost, cudaMemcpyDeviceToDevice };
template <typename T> static inline T atomicMin(T* p, T v) { T o = *p; if (v < o) *p = v; return o; }
template <typename T> static inline T atomicMax(T* p, T v) { T o = *p; if (v > o) *p = v; return o; }
static inline cudaError_t cudaMemcpyAsync(void* d, const void* s, size_t n, cudaMemcpyKind, cudaStream_t) {
  memmove(d, s, n); return cudaSuccess; }
static inline cudaError_t cudaMemcpy2DAsync(void* d, size_t dp, const void* s, size_t sp, size_t w, size_t h,
                                            cudaMemcpyKind, cudaStream_t) {
  for (size_t r = 0; r < h; ++r) memmove((char*)d + r * dp, (const char*)s + r * sp, w);
  return cudaSuccess; }
static inline cudaError_t cudaMemsetAsync(void* d, int v, size_t n, cudaStream_t) { memset(d, v, n); return cudaSuccess; }
static inline cudaError_t cudaStreamSynchronize(cudaStream_t) { return cudaSuccess; }
static inline cudaError_t cudaGetLastError() { return cudaSuccess; }
static inline const char* cudaGetErrorString(cudaError_t) { return "emulated"; }
#define GB_LAUNCH(...) do { __VA_ARGS__; } while (0)
#define GB_CUDA_TRY(expr) do { cudaError_t _e = (expr); if (_e != cudaSuccess) return (int)_e; } while (0)
namespace emu {
template <typename K, typename... A>
void launch(K kernel, unsigned grid, unsigned block, int, cudaStream_t, A... args) {
  blockDim = dim3{block, 1, 1};
  for (unsigned b = 0; b < grid; ++b)
    for (unsigned t = 0; t < block; ++t) {
      blockIdx = dim3{b, 0, 0};
      threadIdx = dim3{t, 0, 0};
      kernel(args...);
    }
}
}  // namespace emu
namespace gb {
struct DevScratch {
  void* p = nullptr;
  DevScratch(size_t bytes, cudaStream_t) { p = calloc(1, bytes ? bytes : 1); }
  ~DevScratch() { free(p); }
  DevScratch(const DevScratch&) = delete;
  DevScratch& operator=(const DevScratch&) = delete;
  template <typename T> T* as() const { return static_cast<T*>(p); }
};
}  // namespace gb
"""



def translate(src, drop_includes=("common.cuh", "driver.h"), min_launches=1):
    """`src` with its launches made sequential and the named includes
    replaced by the stand-in."""
    for inc in drop_includes:
        src = src.replace(f'#include "{inc}"\n', "")
    src = '#include "emu_cuda.h"\n' + src
    launch = re.compile(r"(\w+(?:<\w+>)?)<<<(.*?)>>>\(")
    out, n = launch.subn(lambda m: f"emu::launch({m.group(1)}, {m.group(2)}, ", src)
    assert n >= min_launches, n
    assert "<<<" not in out
    return out


def build(tmp_dir, name, source, include_dirs):
    """Compile `source` (with the stand-in header beside it) into
    tmp_dir/lib<name>.so; returns its path."""
    with open(os.path.join(tmp_dir, "emu_cuda.h"), "w") as f:
        f.write(EMU)
    cpp = os.path.join(tmp_dir, name + ".cpp")
    with open(cpp, "w") as f:
        f.write(source)
    so = os.path.join(tmp_dir, "lib" + name + ".so")
    cmd = ["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fPIC", "-shared", "-I", tmp_dir]
    for d in include_dirs:
        cmd += ["-I", d]
    r = subprocess.run(cmd + [cpp, "-o", so], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]
    return so
