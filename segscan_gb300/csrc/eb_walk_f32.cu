// FP32 instantiations of the sequential-walk kernels.
#include "eb_g4.cuh"

namespace ss {
void *sr_kernel_f32(int V, int NV, bool seg) {
  return seg ? sr_ptr<float, float, true>(V, NV) : sr_ptr<float, float, false>(V, NV);
}
void *g4_kernel_f32(int V, int NV, int c_dtype) {
  if (c_dtype == SS_F32) return g4_ptr<float, float>(V, NV);
  return g4_kernel_f32_c16(V, NV, c_dtype);
}
}  // namespace ss
