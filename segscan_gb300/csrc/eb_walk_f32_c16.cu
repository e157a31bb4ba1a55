// FP32 values and B with a 16-bit C: the ebsr walk rounds its FP32 sums to
// the output type in its stores (no separate cast pass over C).
#include "eb_walk.cuh"

namespace ss {
void *sr_kernel_f32_c16(int V, int NV, int c_dtype) {
  if (c_dtype == SS_BF16) return sr_ptr<float, __nv_bfloat16, false>(V, NV);
  if (c_dtype == SS_F16) return sr_ptr<float, __half, false>(V, NV);
  return nullptr;
}
}  // namespace ss
