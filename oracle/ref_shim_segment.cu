// Exposes the reference's host segment_coo loop as a C ABI (see
// ref_shim_spmm.cu).  TEST INFRASTRUCTURE ONLY.  A separate translation unit
// because new-cg/include/utils/check.cuh and test-cg/include/util/check.cuh
// share the include guard CHECK_.
#include "new-cg/include/utils/check.cuh"

extern "C" {
// segment_coo_sequencial (new-cg/include/utils/check.cuh:44-52):
// dst[index[i], :] += src[i, :], FP32.
void ref_segment_coo_sequencial(const float *src, const int *index, int nnz,
                                int N, int dst_len, float *dst) {
  segment_coo_sequencial<float, int>(src, index, nnz, N, dst_len, dst);
}
}
