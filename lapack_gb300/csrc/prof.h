// Launch accounting and optional per-kernel-class CUDA-event timing.
#pragma once
#include <cuda_runtime.h>

namespace gb {

enum ProfKind : int {
  kProfGemmF64 = 0,     // FP64 trailing update (DFMA)
  kProfGemmF32 = 1,     // FP32 trailing update (FFMA)
  kProfGemmBf16x3 = 2,  // FP32 trailing update on BF16 tensor cores
  kProfPanel = 3,       // cooperative leaf panel
  kProfLaswp = 4,       // row interchanges
  kProfTrsm = 5,        // TRSM leaves in the factorization
  kProfTrsv = 6,        // blocked triangular solves (GETRS)
  kProfResidual = 7,    // FP64 residual of the refinement
  kProfOther = 8,
  kProfCopyH2D = 9,     // host-to-device operand copies of the host-pointer routines
  kProfCopyD2H = 10,    // device-to-host result copies of the host-pointer routines
  kProfKinds = 11,
};

// Counts one kernel launch of this library.
void count_launch(int n = 1);
bool prof_on();
// Brackets one launch on stream s with events when profiling is on;
// `flops` / `bytes` are the algorithmic work of the launch.
void prof_begin(int kind, cudaStream_t s);
void prof_end(int kind, cudaStream_t s, double flops, double bytes);

}  // namespace gb
