// FP16-storage instantiations of the sequential-walk kernels.
#include "eb_walk.cuh"

namespace ss {
void *sr_kernel_f16(int V, int NV, bool seg, bool out_f32) {
  if (seg) return sr_ptr<__half, float, true>(V, NV);
  return out_f32 ? sr_ptr<__half, float, false>(V, NV) : sr_ptr<__half, __half, false>(V, NV);
}
}  // namespace ss
