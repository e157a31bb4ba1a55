// Row assignment, input validation and value gather.
#include <atomic>

#include "common.cuh"
#include "internal.h"

namespace ss {

// A device attribute of the current device, cached per device; `fallback`
// when it cannot be read.
static int device_attr(cudaDeviceAttr attr, std::atomic<int> (&cache)[64], int fallback) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return fallback;
  if (dev < 0 || dev >= 64) {
    int n = 0;
    return cudaDeviceGetAttribute(&n, attr, dev) == cudaSuccess && n > 0 ? n : fallback;
  }
  int n = cache[dev].load(std::memory_order_relaxed);
  if (n > 0) return n;
  if (cudaDeviceGetAttribute(&n, attr, dev) != cudaSuccess || n <= 0) return fallback;
  cache[dev].store(n, std::memory_order_relaxed);  // every thread stores the same value
  return n;
}

int sm_count() {
  static std::atomic<int> cache[64];  // 0 = not looked up yet
  return device_attr(cudaDevAttrMultiProcessorCount, cache, 1);
}

long long l2_bytes() {
  static std::atomic<int> cache[64];
  return device_attr(cudaDevAttrL2CacheSize, cache, 64 << 20);
}

// rows[i] = binary_search_segment_number(indptr, M, nnz, e) for e = elems[i]
// (test-cg/include/util/check.cuh:88-102), or for e = i when elems is null.
__global__ void row_ids_kernel(const int32_t *__restrict__ indptr, int M, const int32_t *__restrict__ elems,
                               int64_t count, int32_t *__restrict__ rows) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < count;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int e = elems ? elems[i] : (int)i;
    rows[i] = row_search(indptr, 1, M, e);
  }
}

// Flag bits: 1 indptr[0] != 0, 2 indptr[M] != nnz, 4 indptr decreasing,
// 8 column outside [0, ncol), 16 index not sorted, 32 index outside [0, dst_len).
__global__ void csr_validate_kernel(const int32_t *__restrict__ indptr, const int32_t *__restrict__ indices,
                                    int M, int K, int nnz, int32_t *flag) {
  int bad = 0;
  const int64_t tid = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  if (tid == 0) {
    if (indptr[0] != 0) bad |= 1;
    if (indptr[M] != nnz) bad |= 2;
  }
  for (int64_t r = tid; r < M; r += stride)
    if (indptr[r + 1] < indptr[r]) bad |= 4;
  for (int64_t p = tid; p < nnz; p += stride)
    if ((unsigned)indices[p] >= (unsigned)K) bad |= 8;
  if (bad) atomicOr(flag, bad);
}

__global__ void index_validate_kernel(const int32_t *__restrict__ index, int nnz, int dst_len, int32_t *flag) {
  int bad = 0;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < nnz; p += stride) {
    const int v = index[p];
    if ((unsigned)v >= (unsigned)dst_len) bad |= 32;
    if (p + 1 < nnz && index[p + 1] < v) bad |= 16;
  }
  if (bad) atomicOr(flag, bad);
}

template <typename T>
__global__ void gather_kernel(const T *__restrict__ in, const int32_t *__restrict__ perm, int n, T *__restrict__ out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    out[i] = (unsigned)perm[i] < (unsigned)n ? in[perm[i]] : T(0);
}

static int grid_for(int64_t n, int threads) {
  int64_t b = (n + threads - 1) / threads;
  const int64_t cap = (int64_t)sm_count() * 32;
  if (b > cap) b = cap;
  return b < 1 ? 1 : (int)b;
}

}  // namespace ss

using namespace ss;

extern "C" {

ss_status ss_row_ids(const int32_t *indptr, int M, int nnz, const int32_t *elems, int64_t count, int32_t *rows,
                     void *stream) {
  ss::NvtxRange nvtx_range("ss_row_ids");
  if (M < 1 || nnz < 0 || count < 0) return fail(SS_ERR_INVALID_ARG, "bad sizes (M %d nnz %d)", M, nnz);
  if (count == 0) return SS_OK;
  if (!indptr || !rows) return fail(SS_ERR_INVALID_ARG, "null pointer");
  row_ids_kernel<<<grid_for(count, 256), 256, 0, (cudaStream_t)stream>>>(indptr, M, elems, count, rows);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? SS_OK : cuda_fail(e, "row_ids launch");
}

ss_status ss_csr_validate(const ss_csr *A, int32_t *d_flag, void *stream) {
  if (!A || !d_flag || A->nrow < 0 || A->nnz < 0 || A->ncol < 0 || !A->indptr)
    return fail(SS_ERR_INVALID_ARG, "bad CSR descriptor");
  if (A->nnz > 0 && !A->indices) return fail(SS_ERR_INVALID_ARG, "indices is null");
  cudaStream_t s = (cudaStream_t)stream;
  cudaError_t e = cudaMemsetAsync(d_flag, 0, sizeof(int32_t), s);
  if (e != cudaSuccess) return cuda_fail(e, "clear flag");
  int64_t n = A->nrow > A->nnz ? A->nrow : A->nnz;
  csr_validate_kernel<<<grid_for(n + 1, 256), 256, 0, s>>>(A->indptr, A->indices, A->nrow, A->ncol, A->nnz, d_flag);
  e = cudaGetLastError();
  return e == cudaSuccess ? SS_OK : cuda_fail(e, "csr_validate launch");
}

ss_status ss_index_validate(const int32_t *index, int nnz, int dst_len, int32_t *d_flag, void *stream) {
  if (!d_flag || nnz < 0 || dst_len < 0 || (nnz > 0 && !index)) return fail(SS_ERR_INVALID_ARG, "bad arguments");
  cudaStream_t s = (cudaStream_t)stream;
  cudaError_t e = cudaMemsetAsync(d_flag, 0, sizeof(int32_t), s);
  if (e != cudaSuccess) return cuda_fail(e, "clear flag");
  if (nnz == 0) return SS_OK;
  index_validate_kernel<<<grid_for(nnz, 256), 256, 0, s>>>(index, nnz, dst_len, d_flag);
  e = cudaGetLastError();
  return e == cudaSuccess ? SS_OK : cuda_fail(e, "index_validate launch");
}

ss_status ss_gather_values(const void *values, int dtype, const int32_t *perm, int nnz, void *out, void *stream) {
  if (nnz < 0 || dtype < SS_F32 || dtype > SS_F16) return fail(SS_ERR_INVALID_ARG, "bad arguments");
  if (nnz == 0) return SS_OK;
  if (!values || !perm || !out) return fail(SS_ERR_INVALID_ARG, "null pointer");
  cudaStream_t s = (cudaStream_t)stream;
  if (dtype == SS_F32)
    gather_kernel<float><<<grid_for(nnz, 256), 256, 0, s>>>((const float *)values, perm, nnz, (float *)out);
  else
    gather_kernel<uint16_t><<<grid_for(nnz, 256), 256, 0, s>>>((const uint16_t *)values, perm, nnz, (uint16_t *)out);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? SS_OK : cuda_fail(e, "gather launch");
}

}  // extern "C"
