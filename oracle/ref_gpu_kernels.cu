// The reference's own SpMM kernels (test-cg/include/spmm/spmm_cg.cuh) and
// the dgSPARSE baseline kernels it includes (spmm.cuh), compiled for sm_103a into a device-only cubin with plain extern "C"
// entry names, so the tests (tests/ref_kernels.py) can check and time them
// on the same GPU as this library through the CUDA driver API.  MEASUREMENT INFRASTRUCTURE ONLY: built by
// `make ref` from the reference sources where they lie (REF=<checkout>),
// output in oracle/_ref/ (never committed); nothing here is product code.
//
// The reference kernels are __global__ templates.  Its headers are
// included with __global__ re-annotated as __device__ (the CUDA headers are
// included first, untouched), and each entry below is a __global__ wrapper
// that calls one instantiation with the reference's README-best static knobs
// for N = 64 (README.md:160-210):
//   ebpr (5,256,5,1,16): group 32, tile 32, float4
//   rbpr (3,256,3,1,2):  group 8,  tile 8,  float4
//   ebsr (4,256,4,1,1,16): CoarsenFactor 4, ThreadNz 1, group 16
//   rbsr (coarsen 4, tile 2^5): float4, tile 32
// The host side computes the launch geometry with the launchers' formulas
// (spmm_cg.cuh:176-197, 333-353, 553-566, 664-677).
#include <cuda_runtime.h>
#include <cuda_runtime_api.h>
#include <cooperative_groups.h>
#include <cusparse.h>
#include <cuda_fp16.h>
#include <math.h>
#include <stdio.h>
#include <string.h>
#include <algorithm>
#include <cassert>
#include <cstdlib>
#include <iostream>
#include <limits.h>
#include <memory>
#include <tuple>
#include <typeinfo>
#include <vector>
#pragma push_macro("__global__")
#undef __global__
#define __global__ __device__
#include "test-cg/include/spmm/spmm_cg.cuh"
#pragma pop_macro("__global__")

#define REF_ARGS_NNZ                                                                                    \
  const int M, const int N, const int K, const int nnz, const int *indptr, const int *indices,        \
      const float *data, const float *B, float *C
#define REF_ARGS const int M, const int N, const int K, const int *indptr, const int *indices, const float *data, \
                     const float *B, float *C

extern "C" {
__global__ void ref_ebpr_n64(REF_ARGS_NNZ) {
  csrspmm_parreduce_nnzbalance_cg_kernel<float4, 32, 32>(M, N, K, nnz, indptr, indices, data, B, C);
}
__global__ void ref_rbpr_n64(REF_ARGS) {
  csrspmm_parreduce_rowbalance_cg_kernel<float4, 8, 8>(M, N, K, indptr, indices, data, B, C);
}
__global__ void ref_ebsr_n64(REF_ARGS_NNZ) {
  csrspmm_rowcaching_nnzbalance_cg_kernel<4, 1, 16>(M, N, K, nnz, indptr, indices, data, B, C);
}
__global__ void ref_rbsr_n64(REF_ARGS) {
  csrspmm_seqreduce_rowbalance_cg_kernel<float4, 32>(M, N, K, indptr, indices, data, B, C);
}

// The dgSPARSE baseline kernels the reference compares its static tuples
// against (test-cg/include/spmm/spmm.cuh:17-637, README.md:212-260), with
// the access widths their launchers pick for N a multiple of 4 (float4 for
// ebpr/rbpr, spmm.cuh:172, 314) and the ebsr CoarsenFactor for N < 128 (1)
// and 128 <= N < 512 (2) with ThreadNz 1 (spmm.cuh:525-529).
__global__ void dg_ebpr_f4(REF_ARGS_NNZ) {
  csrspmm_parreduce_nnzbalance_kernel<float4>(M, N, K, nnz, indptr, indices, data, B, C);
}
__global__ void dg_rbpr_f4(REF_ARGS) {
  csrspmm_parreduce_rowbalance_kernel<float4>(M, N, K, indptr, indices, data, B, C);
}
__global__ void dg_ebsr_c1(REF_ARGS_NNZ) {
  csrspmm_rowcaching_nnzbalance_kernel<1, 1>(M, N, K, nnz, indptr, indices, data, B, C);
}
__global__ void dg_ebsr_c2(REF_ARGS_NNZ) {
  csrspmm_rowcaching_nnzbalance_kernel<2, 1>(M, N, K, nnz, indptr, indices, data, B, C);
}
__global__ void dg_rbsr(REF_ARGS) {
  csrspmm_seqreduce_rowbalance_kernel(M, N, K, indptr, indices, data, B, C);
}
}
