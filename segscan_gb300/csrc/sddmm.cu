// SDDMM for the backward pass of C = A * B:
//   dvals[p] = dot(dC[i, :], B[k, :]) for every stored nonzero p = (i, k).
// No counterpart in the reference (it has no backward).
//
// A team of L lanes along N (V-wide vectors, like the SpMM gathers) owns a
// chunk of consecutive nonzeros; the U dot products of a step are reduced
// across the lanes by a butterfly.  FP32 math.  Two kernels:
//  * teams narrower than a warp (N < 32 V): the chunk's first row from one
//    binary search, later rows followed along indptr (rows only move
//    forward), eight nonzeros per step; at 32 registers 64 warps per SM
//    stay resident;
//  * whole-warp teams (N >= 32 V): the rows come from a window of indptr
//    the 32 lanes hold one entry each (the row of position p is the
//    window's first row plus the number of lanes whose row start is <= p,
//    less one: one ballot, no dependent loads), four nonzeros per step whose
//    column indices were loaded during the previous step, dC and B slices
//    loaded together with 16-bit B kept packed until every load of the step
//    is issued, compile-time lane masks.
// B rows are gathered with an evict-last L2 policy; dC rows too when dC fits
// in half the L2, else evict-first (they are read once, row after row).
#include "common.cuh"
#include "eb_common.cuh"
#include "internal.h"

namespace ss {

constexpr int SDDMM_CHUNK = 128;  // nonzeros per team chunk
constexpr int SDDMM_U = 8;        // nonzeros per step, sub-warp teams
constexpr int SDDMM_WU = 4;       // nonzeros per step, whole-warp teams

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
__global__ void __launch_bounds__(256) sddmm_rows_kernel(int M, int K, int N, int nnz,
                                                         const int32_t *__restrict__ indptr,
                                                         const int32_t *__restrict__ cols, const float *__restrict__ dC,
                                                         const T *__restrict__ B, float *__restrict__ out, int lanes,
                                                         int log2_lanes, int dc_stream) {
  const int tid = threadIdx.x;
  const int lane = tid & (lanes - 1);
  const int team = (blockIdx.x * blockDim.x + tid) >> log2_lanes;
  const int teams = (gridDim.x * blockDim.x) >> log2_lanes;
  const unsigned wl = tid & 31;
  const unsigned mask = lanes >= 32 ? 0xffffffffu : (((1u << lanes) - 1u) << (wl & ~(unsigned)(lanes - 1)));
  const uint64_t keep = policy_keep(1.0f), strm = policy_stream();
  const uint64_t dc_pol = dc_stream ? strm : keep;
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
          load_vec<float, V>(dC + (int64_t)row * N + j0, g, dc_pol);
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

struct SddmmArgs {
  int M, K, N, nnz;
  int slices;     // column slices of 32 * V elements covering N
  int dc_stream;  // dC rows loaded evict-first (dC larger than half the L2)
  const int32_t *indptr, *cols;
  const float *dC;  // [M x N]
  const void *B;    // [K x N], the values' storage type
  float *out;       // [nnz]
};

// Whole-warp teams: lane masks and shuffle widths are compile-time
// constants; 64 registers, four blocks of 256 per SM.
template <typename T, int V>
__global__ void __launch_bounds__(256, 4) sddmm_warp_kernel(SddmmArgs a) {
  constexpr int U = SDDMM_WU;
  constexpr int L = 32;
  constexpr unsigned mask = 0xffffffffu;
  const int tid = threadIdx.x;
  const int lane = tid & 31;
  const int team = (blockIdx.x * blockDim.x + tid) >> 5;
  const int teams = (gridDim.x * blockDim.x) >> 5;
  const uint64_t keep = policy_keep(1.0f), strm = policy_stream();
  const uint64_t dc_pol = a.dc_stream ? strm : keep;
  const T *__restrict__ B = (const T *)a.B;
  const int nchunks = (a.nnz + SDDMM_CHUNK - 1) / SDDMM_CHUNK;
  for (int chunk = team; chunk < nchunks; chunk += teams) {
    const int cs = chunk * SDDMM_CHUNK, ce = min(cs + SDDMM_CHUNK, a.nnz);
    // the row holding cs (the last row starting at or before it), then the
    // window: lane l holds indptr[wb + l]
    int wb = max(min(group_lower_bound(a.indptr, a.M, cs + 1, lane, L, mask), a.M) - 1, 0);
    int win = __ldg(a.indptr + min(wb + lane, a.M));
    // row of position p >= the previous call's p, always in [0, M): an
    // indptr that does not start at 0 or decreases gives wrong rows but no
    // access outside dC
    auto row_of = [&](int p) -> int {
      for (;;) {
        const int cnt = __popc(group_ballot(mask, win <= p, L));
        if (cnt < L) return min(max(wb + cnt - 1, 0), a.M - 1);
        // every row start in the window is <= p: p's row is the last one or
        // later; slide the window to it (wb + L - 1 < M here, since indptr[M]
        // = nnz > p)
        wb += L - 1;
        win = __ldg(a.indptr + min(wb + lane, a.M));
      }
    };
    int col[U];
    #pragma unroll
    for (int u = 0; u < U; u++) col[u] = cs + u < ce ? ld_idx(a.cols + cs + u, strm) : -1;
    for (int p0 = cs; p0 < ce; p0 += U) {
      int row[U];
      bool ok[U];
      #pragma unroll
      for (int u = 0; u < U; u++) {
        row[u] = row_of(min(p0 + u, ce - 1));  // collective: every lane, every u
        ok[u] = p0 + u < ce && (unsigned)col[u] < (unsigned)a.K;
      }
      // the next step's columns, in flight while this step's rows are used
      int ncol[U];
      #pragma unroll
      for (int u = 0; u < U; u++) {
        const int q = p0 + U + u;
        ncol[u] = q < ce ? ld_idx(a.cols + q, strm) : -1;
      }
      float part[U];
      #pragma unroll
      for (int u = 0; u < U; u++) part[u] = 0.f;
      for (int s = 0; s < a.slices; s++) {
        const int j0 = (s * L + lane) * V;
        const bool act = j0 < a.N;
        float g[U][V];
        RawVec<T, V> braw[U];
        #pragma unroll
        for (int u = 0; u < U; u++) {
          zero_raw(braw[u]);
          #pragma unroll
          for (int i = 0; i < V; i++) g[u][i] = 0.f;
          if (ok[u] && act) {
            load_vec<float, V>(a.dC + (int64_t)row[u] * a.N + j0, g[u], dc_pol);
            load_raw<T, V>(B + (int64_t)col[u] * a.N + j0, braw[u], keep);
          }
        }
        #pragma unroll
        for (int u = 0; u < U; u++) {
          float b[V];
          unpack_raw(braw[u], b);
          #pragma unroll
          for (int i = 0; i < V; i++) part[u] = fmaf(g[u][i], b[i], part[u]);
        }
      }
      butterfly_store<U>(part, lane, L, mask, a.out, p0, ce);
      #pragma unroll
      for (int u = 0; u < U; u++) col[u] = ncol[u];
    }
  }
}

template <typename T>
static void *sddmm_ptr(int V, bool warp) {
  if (warp) {
    if (V == 1) return (void *)sddmm_warp_kernel<T, 1>;
    if (V == 2) return (void *)sddmm_warp_kernel<T, 2>;
    if (V == 4) return (void *)sddmm_warp_kernel<T, 4>;
  } else {
    if (V == 1) return (void *)sddmm_rows_kernel<T, 1>;
    if (V == 2) return (void *)sddmm_rows_kernel<T, 2>;
    if (V == 4) return (void *)sddmm_rows_kernel<T, 4>;
  }
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
  if (A->nrow < 1) return fail(SS_ERR_INVALID_ARG, "%d nonzeros in a matrix without rows", nnz);
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
  const bool warp = lanes == 32;
  void *fn = A->value_dtype == SS_F32 ? sddmm_ptr<float>(V, warp)
             : A->value_dtype == SS_BF16 ? sddmm_ptr<__nv_bfloat16>(V, warp) : sddmm_ptr<__half>(V, warp);
  const int threads = 256;
  const long long teams_needed = ((long long)nnz + SDDMM_CHUNK - 1) / SDDMM_CHUNK;
  long long blocks = (teams_needed * lanes + threads - 1) / threads;
  if (blocks > (long long)sm_count() * 16) blocks = (long long)sm_count() * 16;
  if (blocks < 1) blocks = 1;
  // dC is read row after row, each row's reuse served by L1: when it is
  // larger than half the L2, its lines are marked evict-first so that they
  // do not push out the gathered B rows; a smaller dC is kept like B
  const int dc_stream = (long long)A->nrow * N * 4 > l2_bytes() / 2;
  cudaError_t e;
  if (warp) {
    SddmmArgs a;
    a.M = A->nrow; a.K = A->ncol; a.N = N; a.nnz = nnz;
    a.slices = ceil_div(N, lanes * V);
    a.indptr = A->indptr; a.cols = A->indices; a.dC = dC; a.B = B; a.out = dvals;
    a.dc_stream = dc_stream;
    void *args[] = {&a};
    e = cudaLaunchKernel(fn, dim3((unsigned)blocks), dim3(threads), args, 0, (cudaStream_t)stream);
  } else {
    int log2_lanes = ilog2(lanes);
    int M = A->nrow, K = A->ncol, Nn = N, nz = nnz;
    const int32_t *ip = A->indptr, *ix = A->indices;
    int dcs = dc_stream;
    void *args[] = {&M, &K, &Nn, &nz, &ip, &ix, &dC, &B, &dvals, &lanes, &log2_lanes, &dcs};
    e = cudaLaunchKernel(fn, dim3((unsigned)blocks), dim3(threads), args, 0, (cudaStream_t)stream);
  }
  return e == cudaSuccess ? SS_OK : cuda_fail(e, "sddmm launch");
}
