// SDDMM for the backward pass of C = A * B:
//   dvals[p] = dot(dC[i, :], B[k, :]) for every stored nonzero p = (i, k).
// No counterpart in the reference (it has no backward).
//
// A team of L lanes along N (V-wide vectors, like the SpMM gathers) owns a
// chunk of consecutive nonzeros; the chunk's first row comes from one
// binary search, later rows from walking indptr (rows only move forward),
// so dC rows are read once per row while B rows are gathered four at a
// time.  The team reduces each dot product with shuffles.  FP32 math.
#include "common.cuh"
#include "internal.h"

namespace ss {

constexpr int SDDMM_CHUNK = 128;  // nonzeros per team chunk
constexpr int SDDMM_U = 8;  // nonzeros per step

// Stores the U dot products reduced by butterfly_sum (common.cuh): the
// lanes holding a finished sum write it, to nonzero p0 + its index.
template <int U>
__device__ __forceinline__ void butterfly_store(float (&v)[U], int lane, int lanes, unsigned mask, float *out,
                                                int p0, int ce) {
  int base = 0;
  const float x = butterfly_sum<U>(v, lane, lanes, mask, base);
  if ((lane & (lanes / U - 1)) == 0 && p0 + base < ce) out[p0 + base] = x;
}

template <typename T, int V>
__global__ void __launch_bounds__(256) sddmm_kernel(int M, int K, int N, int nnz, const int32_t *__restrict__ indptr,
                                                    const int32_t *__restrict__ cols, const float *__restrict__ dC,
                                                    const T *__restrict__ B, float *__restrict__ out, int lanes,
                                                    int log2_lanes) {
  const int tid = threadIdx.x;
  const int lane = tid & (lanes - 1);
  const int team = (blockIdx.x * blockDim.x + tid) >> log2_lanes;
  const int teams = (gridDim.x * blockDim.x) >> log2_lanes;
  const unsigned wl = tid & 31;
  const unsigned mask = lanes >= 32 ? 0xffffffffu : (((1u << lanes) - 1u) << (wl & ~(unsigned)(lanes - 1)));
  const uint64_t keep = policy_keep(1.0f), strm = policy_stream();
  const int nchunks = (nnz + SDDMM_CHUNK - 1) / SDDMM_CHUNK;
  for (int chunk = team; chunk < nchunks; chunk += teams) {
    const int cs = chunk * SDDMM_CHUNK, ce = min(cs + SDDMM_CHUNK, nnz);
    int row = row_search(indptr, 1, M, cs);
    int next = __ldg(indptr + min(row + 1, M));
    for (int p0 = cs; p0 < ce; p0 += SDDMM_U) {
      float part[SDDMM_U];
      #pragma unroll
      for (int u = 0; u < SDDMM_U; u++) {
        const int p = p0 + u;
        part[u] = 0.f;
        if (p >= ce) continue;
        while (p >= next && row < M - 1) {  // rows only move forward inside a chunk
          row++;
          next = __ldg(indptr + row + 1);
        }
        const int c = ld_idx(cols + p, strm);
        if ((unsigned)c >= (unsigned)K) continue;
        for (int j0 = lane * V; j0 < N; j0 += lanes * V) {
          float g[V], b[V];
          load_vec<float, V>(dC + (int64_t)row * N + j0, g, keep);
          load_vec<T, V>(B + (int64_t)c * N + j0, b, keep);
          #pragma unroll
          for (int i = 0; i < V; i++) part[u] = fmaf(g[i], b[i], part[u]);
        }
      }
      if (lanes >= SDDMM_U) {
        butterfly_store<SDDMM_U>(part, lane, lanes, mask, out, p0, ce);
      } else {
        #pragma unroll
        for (int u = 0; u < SDDMM_U; u++) {
          float x = part[u];
          for (int off = lanes >> 1; off > 0; off >>= 1) x += __shfl_xor_sync(mask, x, off);
          if (lane == 0 && p0 + u < ce) out[p0 + u] = x;
        }
      }
    }
  }
}

template <typename T>
static void *sddmm_ptr(int V) {
  if (V == 1) return (void *)sddmm_kernel<T, 1>;
  if (V == 2) return (void *)sddmm_kernel<T, 2>;
  if (V == 4) return (void *)sddmm_kernel<T, 4>;
  return nullptr;
}

}  // namespace ss

using namespace ss;

extern "C" ss_status ss_sddmm(const ss_csr *A, int N, const float *dC, const void *B, float *dvals, void *stream) {
  ss::NvtxRange nvtx_range("ss_sddmm");
  if (!A || A->nrow < 0 || A->ncol < 0 || A->nnz < 0 || N < 0) return fail(SS_ERR_INVALID_ARG, "bad arguments");
  if (A->value_dtype < SS_F32 || A->value_dtype > SS_F16) return fail(SS_ERR_INVALID_ARG, "bad dtype");
  const int nnz = A->nnz;
  if (nnz == 0) return SS_OK;
  if (!A->indptr || !A->indices || !dC || !B || !dvals) return fail(SS_ERR_INVALID_ARG, "null pointer");
  if (N == 0) {
    cudaError_t e = cudaMemsetAsync(dvals, 0, (size_t)nnz * 4, (cudaStream_t)stream);
    return e == cudaSuccess ? SS_OK : cuda_fail(e, "sddmm zero");
  }
  // V: widest vector (<= 16 bytes of FP32 dC) dividing N; lanes cover N
  int V = 4;
  while (V > 1 && (N % V) != 0) V >>= 1;
  const int es = dtype_size(A->value_dtype);
  if (((uintptr_t)dC % (4 * V)) || ((uintptr_t)B % (es * V)))
    return fail(SS_ERR_ALIGNMENT, "dC/B not aligned to the %d-element vector access", V);
  int lanes = ceil_pow2(ceil_div(N, V));
  if (lanes > 32) lanes = 32;
  void *fn = A->value_dtype == SS_F32 ? sddmm_ptr<float>(V)
             : A->value_dtype == SS_BF16 ? sddmm_ptr<__nv_bfloat16>(V) : sddmm_ptr<__half>(V);
  const int threads = 256;
  const long long teams_needed = ((long long)nnz + SDDMM_CHUNK - 1) / SDDMM_CHUNK;
  long long blocks = (teams_needed * lanes + threads - 1) / threads;
  if (blocks > (long long)sm_count() * 16) blocks = (long long)sm_count() * 16;
  if (blocks < 1) blocks = 1;
  int log2_lanes = ilog2(lanes);
  int M = A->nrow, K = A->ncol, Nn = N, nz = nnz;
  const int32_t *ip = A->indptr, *ix = A->indices;
  void *args[] = {&M, &K, &Nn, &nz, &ip, &ix, &dC, &B, &dvals, &lanes, &log2_lanes};
  cudaError_t e = cudaLaunchKernel(fn, dim3((unsigned)blocks), dim3(threads), args, 0, (cudaStream_t)stream);
  return e == cudaSuccess ? SS_OK : cuda_fail(e, "sddmm launch");
}
