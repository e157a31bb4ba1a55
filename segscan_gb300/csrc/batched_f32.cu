// FP32 instantiations of the batched SpMM kernel.
#include "batched.cuh"
namespace ss {
void *batched_kernel_f32(int V, int NV) { return batched_ptr<float, float>(V, NV); }
}  // namespace ss
