// BF16-storage instantiations of the sequential-walk kernels.
#include "eb_g4.cuh"

namespace ss {
void *sr_kernel_bf16(int V, int NV, bool seg, bool out_f32) {
  if (seg) return sr_ptr<__nv_bfloat16, float, true>(V, NV);
  return out_f32 ? sr_ptr<__nv_bfloat16, float, false>(V, NV) : sr_ptr<__nv_bfloat16, __nv_bfloat16, false>(V, NV);
}
void *g4_kernel_bf16(int V, int NV, bool out_f32) {
  return out_f32 ? g4_ptr<__nv_bfloat16, float>(V, NV) : g4_ptr<__nv_bfloat16, __nv_bfloat16>(V, NV);
}
}  // namespace ss
