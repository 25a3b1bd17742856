// tcgen05 BF16 assignment (placeholder until the tensor-core kernel lands).
#include "common.cuh"
#include "kernels.h"

namespace kmgb {

bool bf16_tc_supported(int d) {
  (void)d;
  return false;
}

float assign_bf16_gamma(int d) {
  (void)d;
  return 0.0f;
}

cudaError_t launch_assign_bf16(const void*, long long, const void*, long long, const AssignArgs&,
                               cudaStream_t) {
  return cudaErrorNotSupported;
}

}  // namespace kmgb
