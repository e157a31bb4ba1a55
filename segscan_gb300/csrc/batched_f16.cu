// FP16-storage instantiations of the batched SpMM kernel.
#include "batched.cuh"
namespace ss {
void *batched_kernel_f16(int V, int NV, bool out_f32) {
  return out_f32 ? batched_ptr<__half, float>(V, NV) : batched_ptr<__half, __half>(V, NV);
}
}  // namespace ss
