// Exposes the reference's own host code for the SpMM path as a C ABI, so the
// tests can pin the oracle against it.  TEST INFRASTRUCTURE ONLY: built by
// `make ref` from the reference sources where they lie (REF=<checkout>),
// output in oracle/_ref/ (never committed).  Nothing here is product code.
//
// binary_search_segment_number is declared __device__ in the reference
// (test-cg/include/util/check.cuh:88-102).  The CUDA headers are included
// first, then __device__ is re-annotated as host+device for the reference
// headers only, so the very same source runs on the host.
#include <cuda_runtime.h>
#include <cuda_runtime_api.h>
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
#pragma push_macro("__device__")
#undef __device__
#define __device__ __location__(host) __location__(device)
#include "test-cg/include/util/check.cuh"
#include "test-cg/include/dataloader/dataloader.hpp"
#pragma pop_macro("__device__")

extern "C" {

// util::spmm_reference_host (check.cuh:139-158): C += A*B, FP32.
void ref_spmm_reference_host(int M, int N, int *indptr, int *indices,
                             float *vals, float *B, float *C) {
  util::spmm_reference_host<int, float>(M, N, indptr, indices, vals, B, C);
}

// binary_search_segment_number (check.cuh:88-102) for a list of elements.
void ref_row_ids(const int *indptr, int M, int nnz, const int *elems,
                 long long count, int *rows) {
  for (long long i = 0; i < count; i++)
    rows[i] = binary_search_segment_number<int>(indptr, M, nnz, elems[i]);
}

// transpose + compressedRow (dataloader.hpp:109-144), the way DataLoader
// (dataloader.hpp:170-183) builds A^T from A's COO rows and CSR columns.
void ref_transpose(int nrow, int ncol, int nnz, const int *coo_row,
                   const int *csr_col, int *t_indptr, int *t_indices) {
  std::vector<int> row(coo_row, coo_row + nnz), col(csr_col, csr_col + nnz);
  std::vector<int> row_t(nnz, 0), col_t(nnz, 0), rowptr_t;
  transpose<int>(ncol, row, col, row_t, col_t);
  compressedRow<int>(ncol, row_t, rowptr_t);
  for (int c = 0; c <= ncol; c++) t_indptr[c] = rowptr_t[c];
  for (int q = 0; q < nnz; q++) t_indices[q] = col_t[q];
  (void)nrow;
}

// read_mtx_file (dataloader.hpp:22-107): the reference's Matrix Market
// reader, pattern only.  First call with null outputs to get the sizes
// (nrow, ncol, nnz after its own processing), then with buffers of
// nrow + 1 and nnz entries.  Valid files only (the reference exit()s).
void ref_read_mtx(const char *path, int *nrow, int *ncol, int *nnz, int *indptr, int *indices) {
  int M = 0, K = 0, Z = 0;
  std::vector<int> ip, ix, coo;
  read_mtx_file(path, M, K, Z, ip, ix, coo);
  *nrow = M;
  *ncol = K;
  *nnz = Z;
  if (indptr)
    for (size_t i = 0; i < ip.size(); i++) indptr[i] = ip[i];
  if (indices)
    for (size_t i = 0; i < ix.size(); i++) indices[i] = ix[i];
}

}  // extern "C"
