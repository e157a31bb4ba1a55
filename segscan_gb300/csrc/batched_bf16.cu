// BF16-storage instantiations of the batched SpMM kernel.
#include "batched.cuh"
namespace ss {
void *batched_kernel_bf16(int V, int NV, bool out_f32) {
  return out_f32 ? batched_ptr<__nv_bfloat16, float>(V, NV) : batched_ptr<__nv_bfloat16, __nv_bfloat16>(V, NV);
}
}  // namespace ss
