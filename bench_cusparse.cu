// cuSPARSE CSR x dense SpMM as a comparison line for bench.py (measurement
// only; not part of the library).  It follows the reference's cuSPARSE call
// (test-cg/include/spmm/spmm.cuh:640-694): CSR A with int32 indices, B and C
// dense row-major FP32, C = A * B with CUSPARSE_SPMM_ALG_DEFAULT.  The handle,
// descriptors and workspace are created once (csp_create), each csp_run is
// one cusparseSpMM on the given stream, and csp_destroy releases all of
// them (the reference never frees its descriptors or buffer).
//
//   nvcc -gencode arch=compute_103a,code=sm_103a -O3 -shared -Xcompiler -fPIC \
//        -o _build/bench_cusparse.so bench_cusparse.cu -lcusparse
#include <cuda_runtime.h>
#include <cusparse.h>

namespace {
struct Line {
  cusparseHandle_t handle = nullptr;
  cusparseSpMatDescr_t A = nullptr;
  cusparseDnMatDescr_t B = nullptr, C = nullptr;
  void *buf = nullptr;
};

void release(Line *l) {
  if (l->A) cusparseDestroySpMat(l->A);
  if (l->B) cusparseDestroyDnMat(l->B);
  if (l->C) cusparseDestroyDnMat(l->C);
  if (l->buf) cudaFree(l->buf);
  if (l->handle) cusparseDestroy(l->handle);
  delete l;
}
}  // namespace

extern "C" {

// Returns 0 and a handle in *out, or the failing cuSPARSE status (a CUDA
// error e as 1000 + e).
int csp_create(void **out, int M, int K, int nnz, const int *indptr, const int *indices, const float *vals, int N,
               const float *B, float *C) {
  Line *l = new Line;
  const float alpha = 1.f, beta = 0.f;
  size_t bytes = 0;
  int st = cusparseCreate(&l->handle);
  if (!st)
    st = cusparseCreateCsr(&l->A, M, K, nnz, (void *)indptr, (void *)indices, (void *)vals, CUSPARSE_INDEX_32I,
                           CUSPARSE_INDEX_32I, CUSPARSE_INDEX_BASE_ZERO, CUDA_R_32F);
  if (!st) st = cusparseCreateDnMat(&l->B, K, N, N, (void *)B, CUDA_R_32F, CUSPARSE_ORDER_ROW);
  if (!st) st = cusparseCreateDnMat(&l->C, M, N, N, (void *)C, CUDA_R_32F, CUSPARSE_ORDER_ROW);
  if (!st)
    st = cusparseSpMM_bufferSize(l->handle, CUSPARSE_OPERATION_NON_TRANSPOSE, CUSPARSE_OPERATION_NON_TRANSPOSE,
                                 &alpha, l->A, l->B, &beta, l->C, CUDA_R_32F, CUSPARSE_SPMM_ALG_DEFAULT, &bytes);
  if (!st && bytes > 0) {
    const cudaError_t e = cudaMalloc(&l->buf, bytes);
    if (e != cudaSuccess) st = 1000 + (int)e;  // CUDA errors reported above cuSPARSE's status range
  }
  if (st) {
    release(l);
    return st;
  }
  *out = l;
  return 0;
}

int csp_run(void *h, void *stream) {
  Line *l = (Line *)h;
  const float alpha = 1.f, beta = 0.f;
  int st = cusparseSetStream(l->handle, (cudaStream_t)stream);
  if (st) return st;
  return cusparseSpMM(l->handle, CUSPARSE_OPERATION_NON_TRANSPOSE, CUSPARSE_OPERATION_NON_TRANSPOSE, &alpha, l->A,
                      l->B, &beta, l->C, CUDA_R_32F, CUSPARSE_SPMM_ALG_DEFAULT, l->buf);
}

void csp_destroy(void *h) {
  if (h) release((Line *)h);
}

}  // extern "C"
