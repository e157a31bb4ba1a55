// FP32 instantiations of the sequential-walk kernels.
#include "eb_walk.cuh"

namespace ss {
void *sr_kernel_f32(int V, int NV, bool seg) {
  return seg ? sr_ptr<float, float, true>(V, NV) : sr_ptr<float, float, false>(V, NV);
}
}  // namespace ss
