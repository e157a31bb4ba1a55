// The reference's segment_coo kernels (new-cg/include/segscan/segscan.cuh)
// compiled for sm_103a into a device-only cubin, launched through the
// driver API by the tests that compare against them.  MEASUREMENT
// INFRASTRUCTURE ONLY: built by `make -C oracle ref` from the reference
// sources where they lie; output in oracle/_ref/ (never committed).
//
// A separate translation unit from ref_gpu_kernels.cu: both reference
// headers declare an `extern __shared__ shared_mem` of different types.
// As there, the headers are included with __global__ re-annotated as
// __device__ and each entry is a __global__ wrapper around one
// instantiation:
//   segment_coo_sr<float, int, 4, 256, 4, 1, 1, 16> (segscan.cuh:817-866):
//     segscan_sr_kernel<float, int, CoarsenFactor 4, ThreadNz 1, group 16>
//   segment_coo_sorted_sr<float, int, 2, 4, 8, 2, 16>, the variant
//     new-cg/src/main.cu:54 runs (segscan.cuh:974-1008):
//     segscan_sr_sorted_kernel<float, int, CoarsenFactor 2, ThreadNz 4, DtileSize 8>
//   segment_coo<float, int, 5, 256, 5, 1, 16> (segscan.cuh:150-184,
//     new-cg/src/main.cu:50): segscan_kernel<float, int, float4, 32, 32>
//   segment_coo_new<float, int, 5, 256, 5, 2> (segscan.cuh:327-355,
//     new-cg/src/main.cu:51): segscan_new_kernel<float, int, float4, 32>
//   segment_coo_noshmem_sr<float, int, 4, 256, 4, 2, 1, 16> (:868-916,
//     main.cu:53): segscan_sr_noshmem_kernel<float, int, 4, 2, 16>
//   segment_coo_noshmem_lessatom_sr<float, int, 4, 256, 4, 1, 1, 16>
//     (:918-972, main.cu:54): segscan_sr_noshmem_lessatom_kernel<float, int, 4, 1, 16>
// segscan_sr_kernel reads index[] up to group_size - 1 entries past nnz
// (segscan.cuh:402, 459), segscan_kernel up to tile_size - 1 (:31) and
// segscan_new_kernel up to blockDim.x - 1 (:209); the caller pads the index
// buffer.
#include <cuda_runtime.h>
#include <cooperative_groups.h>
#include <cuda_fp16.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <algorithm>
#include <iostream>
#include <vector>
#pragma push_macro("__global__")
#undef __global__
#define __global__ __device__
#include "new-cg/include/segscan/segscan.cuh"
#pragma pop_macro("__global__")

extern "C" {
__global__ void ref_seg_sr_n64(const float *src, const int *index, const int nnz, const int N, float *dst) {
  segscan_sr_kernel<float, int, 4, 1, 16>(src, index, nnz, N, dst);
}
__global__ void ref_seg_sorted_sr(const float *src, const int *index, const int nnz, const int N, float *dst) {
  segscan_sr_sorted_kernel<float, int, 2, 4, 8>(src, index, nnz, N, dst);
}
__global__ void ref_seg_pr_f4(const float *src, const int *index, const int nnz, const int N, float *dst) {
  segscan_kernel<float, int, float4, 32, 32>(src, index, nnz, N, dst);
}
__global__ void ref_seg_new_f4(const float *src, const int *index, const int nnz, const int N, float *dst) {
  segscan_new_kernel<float, int, float4, 32>(src, index, nnz, N, dst);
}
__global__ void ref_seg_noshmem_n64(const float *src, const int *index, const int nnz, const int N, float *dst) {
  segscan_sr_noshmem_kernel<float, int, 4, 2, 16>(src, index, nnz, N, dst);
}
__global__ void ref_seg_lessatom_n64(const float *src, const int *index, const int nnz, const int N, float *dst) {
  segscan_sr_noshmem_lessatom_kernel<float, int, 4, 1, 16>(src, index, nnz, N, dst);
}
}
