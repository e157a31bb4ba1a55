// BF16-storage instantiations of the sequential-walk kernels.
#include "eb_walk.cuh"

namespace ss {
void *sr_kernel_bf16(int V, int NV, bool seg, bool out_f32) {
  if (seg) return sr_ptr<__nv_bfloat16, float, true>(V, NV);
  return out_f32 ? sr_ptr<__nv_bfloat16, float, false>(V, NV) : sr_ptr<__nv_bfloat16, __nv_bfloat16, false>(V, NV);
}
}  // namespace ss
