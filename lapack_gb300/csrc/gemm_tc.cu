// BF16x3 tensor-core trailing update for the FP32 factorization (tcgen05).
#include "driver.h"

namespace gb {

int gemm_bf16x3_dev(int, int, int, const float*, int, const float*, int, float*, int, cudaStream_t) {
  return (int)cudaErrorNotSupported;
}

}  // namespace gb
