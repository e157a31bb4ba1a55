// Fused backward of C = A * B, walked over the rows of A^T.
//
// No counterpart in the reference (it has no backward).  For a row k of A^T
// (a column of A) and each of its nonzeros q = (k, i), whose position in A
// is p = perm[q] and value a = values[p]:
//   dB[k, :]  = sum over the row's q, in order, of a * dC[i, :]
//   dvals[p]  = dot(dC[i, :], B[k, :])
// so one gather of the dC row serves both gradients: SDDMM followed by
// A^T * dC would gather a B row and then a dC row for every nonzero.
//
// A group of L lanes along N (lane l holds elements (j * L + l) * V .. + V -
// 1 for j < NV, so each gathered row is one contiguous request per j) owns a
// contiguous block of A^T rows: the rows that start inside its share of
// about nnz / groups positions, so the blocks hold similar numbers of
// nonzeros and no row is split.  It streams the block's nonzeros in order,
// four at a time, with their four dC rows and values in flight while the
// next four positions' indices and permutation entries load.  Row ends come
// from a window of t_indptr the lanes hold one entry each, and the B slice
// of the next row is loaded one row ahead, so a row change costs no round
// trip.  The four partial dot products are reduced across the lanes by a
// fixed butterfly (butterfly_sum); dB is summed in position order, with
// Kahan compensation when the row is longer than the threshold, so dB has
// the bits of the row-balanced sequential SpMM (rbsr) on A^T.  FP32 math.
#include "common.cuh"
#include "eb_common.cuh"
#include "internal.h"

namespace ss {

constexpr int BWD_U = 4;  // nonzeros (dC rows) in flight per group

struct BwdArgs {
  int K, M, N, nnz, kahan;
  int chunk;        // positions per group's share
  int groups;       // groups with a share (the last one takes the rest)
  const int32_t *t_indptr, *t_indices, *perm;
  const void *vals;  // A's values in A's order, or null (ones)
  const float *dC;   // [M x N]
  const void *B;     // [K x N], the values' storage type
  void *dB;          // [K x N]
  float *dvals;      // [nnz], A's order
  int lanes, log2_lanes;
};

// WARP: the group is a whole warp (32 lanes), so lane masks and shuffle
// widths are compile-time constants and warp collectives need no
// convergence handling.
template <typename T, typename TC, int V, int NV, bool WARP>
__global__ void __launch_bounds__(256, NV == 1 ? 4 : 1) fused_bwd_kernel(BwdArgs a) {
  const int tid = threadIdx.x;
  const int L = WARP ? 32 : a.lanes;
  const int lane = tid & (L - 1);
  const int group = (blockIdx.x * blockDim.x + tid) >> (WARP ? 5 : a.log2_lanes);
  const unsigned wl = tid & 31;
  const unsigned mask = WARP ? 0xffffffffu : L >= 32 ? 0xffffffffu : (((1u << L) - 1u) << (wl & ~(unsigned)(L - 1)));
  if (group >= a.groups) return;  // whole groups exit together
  const uint64_t keep = policy_keep(1.0f), strm = policy_stream();
  const T *B = (const T *)a.B;
  const T *vals = (const T *)a.vals;
  bool act[NV];
  #pragma unroll
  for (int j = 0; j < NV; j++) act[j] = (j * L + lane) * V < a.N;
  // the rows starting in [lo, hi)
  const long long lo = (long long)group * a.chunk;
  const int r_lo = group_lower_bound(a.t_indptr, a.K, (int)lo, lane, L, mask);
  const int r_hi = group == a.groups - 1
                       ? a.K
                       : group_lower_bound(a.t_indptr, a.K, (int)min(lo + a.chunk, (long long)a.nnz), lane, L, mask);
  if (r_lo >= r_hi) return;
  const int qe = __ldg(a.t_indptr + r_hi);

  // t_indptr[wb + l] held by lane l
  int wb = r_lo, win = __ldg(a.t_indptr + min(r_lo + lane, a.K));
  auto ptr_at = [&](int r) -> int {  // t_indptr[r], r >= wb
    if (r >= wb + L) {
      wb = r;
      win = __ldg(a.t_indptr + min(r + lane, a.K));
    }
    return __shfl_sync(mask, win, r - wb, L);
  };
  // B slice of row r, kept packed: 16-bit slices are widened only when the
  // row becomes current, so the prefetch one row ahead is not waited for
  auto load_b = [&](int r, RawVec<T, V> (&dst)[NV]) {
    #pragma unroll
    for (int j = 0; j < NV; j++) {
      zero_raw(dst[j]);
      if (act[j] && r < r_hi) load_raw<T, V>(B + (int64_t)r * a.N + (j * L + lane) * V, dst[j], strm);
    }
  };

  int k = r_lo;
  int sk = ptr_at(k), ek = ptr_at(k + 1);
  bool kahan = ek - sk > a.kahan;
  float bcur[NV][V], acc[NV][V], comp[NV][V];
  RawVec<T, V> bnext[NV];
  load_b(k, bnext);
  #pragma unroll
  for (int j = 0; j < NV; j++) unpack_raw(bnext[j], bcur[j]);
  load_b(k + 1, bnext);
  #pragma unroll
  for (int j = 0; j < NV; j++)
    #pragma unroll
    for (int i = 0; i < V; i++) { acc[j][i] = 0.f; comp[j][i] = 0.f; }
  // row k is done: its dB row stored, the next row set up
  auto next_row = [&]() {
    TC *dst = (TC *)a.dB + (int64_t)k * a.N;
    #pragma unroll
    for (int j = 0; j < NV; j++) {
      if (act[j]) store_vec<TC, V>(dst + (j * L + lane) * V, acc[j], strm);
      #pragma unroll
      for (int i = 0; i < V; i++) { acc[j][i] = 0.f; comp[j][i] = 0.f; }
      unpack_raw(bnext[j], bcur[j]);
    }
    k++;
    sk = ek;
    ek = ptr_at(k + 1);
    kahan = ek - sk > a.kahan;
    load_b(k + 1, bnext);
  };

  int row[BWD_U], pos[BWD_U];
  int q0 = sk;
  #pragma unroll
  for (int u = 0; u < BWD_U; u++) {
    row[u] = q0 + u < qe ? ld_idx(a.t_indices + q0 + u, strm) : -1;
    pos[u] = q0 + u < qe ? ld_idx(a.perm + q0 + u, strm) : -1;
  }
  for (; q0 < qe; q0 += BWD_U) {
    float av[BWD_U];
    float g[BWD_U][NV][V];
    RawVec<T, 1> araw[BWD_U];  // values loaded packed: widened after every gather is issued
    bool okv[BWD_U];
    #pragma unroll
    for (int u = 0; u < BWD_U; u++) {
      const bool ok = (unsigned)row[u] < (unsigned)a.M && (unsigned)pos[u] < (unsigned)a.nnz;
      okv[u] = ok;
      zero_raw(araw[u]);
      if (ok && vals) load_raw<T, 1>(vals + pos[u], araw[u], keep);
      #pragma unroll
      for (int j = 0; j < NV; j++) {
        if (ok && act[j]) {
          load_vec<float, V>(a.dC + (int64_t)row[u] * a.N + (j * L + lane) * V, g[u][j], keep);
        } else {
          #pragma unroll
          for (int i = 0; i < V; i++) g[u][j][i] = 0.f;
        }
      }
    }
    #pragma unroll
    for (int u = 0; u < BWD_U; u++) {
      float x[1];
      unpack_raw(araw[u], x);
      av[u] = okv[u] ? (vals ? x[0] : 1.f) : 0.f;
    }
    // the next four positions' indices, in flight while these are used
    int nrow[BWD_U], npos[BWD_U];
    #pragma unroll
    for (int u = 0; u < BWD_U; u++) {
      const int q = q0 + BWD_U + u;
      nrow[u] = q < qe ? ld_idx(a.t_indices + q, strm) : -1;
      npos[u] = q < qe ? ld_idx(a.perm + q, strm) : -1;
    }
    float part[BWD_U];
    #pragma unroll
    for (int u = 0; u < BWD_U; u++) {
      part[u] = 0.f;
      if (q0 + u >= qe) continue;
      while (q0 + u >= ek) next_row();  // rows that end here (empty ones too) are stored
      #pragma unroll
      for (int j = 0; j < NV; j++)
        #pragma unroll
        for (int i = 0; i < V; i++) part[u] = fmaf(g[u][j][i], bcur[j][i], part[u]);
      // one branch per nonzero on the row's (group-uniform) mode; the empty
      // asm keeps the compiler from computing both steps and selecting
      if (kahan) {
        asm volatile("");
        #pragma unroll
        for (int j = 0; j < NV; j++)
          #pragma unroll
          for (int i = 0; i < V; i++) kahan_fma(acc[j][i], comp[j][i], av[u], g[u][j][i]);
      } else {
        #pragma unroll
        for (int j = 0; j < NV; j++)
          #pragma unroll
          for (int i = 0; i < V; i++) acc[j][i] = fmaf(av[u], g[u][j][i], acc[j][i]);
      }
    }
    // the four dot products: reduced across the lanes, stored at A's positions
    if (L >= BWD_U) {
      int base = 0;
      const float x = butterfly_sum<BWD_U>(part, lane, L, mask, base);
      // the storing lane reads perm[q0 + base] again (just loaded, cached)
      // rather than indexing pos[] by a lane-dependent base, which would put
      // pos in local memory
      if ((lane & (L / BWD_U - 1)) == 0 && q0 + base < qe) {
        const int pb = __ldg(a.perm + q0 + base);
        if ((unsigned)pb < (unsigned)a.nnz) a.dvals[pb] = x;
      }
    } else {
      #pragma unroll
      for (int u = 0; u < BWD_U; u++) {
        float x = part[u];
        for (int off = L >> 1; off > 0; off >>= 1) x += __shfl_xor_sync(mask, x, off);
        if (lane == 0 && pos[u] >= 0 && pos[u] < a.nnz) a.dvals[pos[u]] = x;
      }
    }
    #pragma unroll
    for (int u = 0; u < BWD_U; u++) { row[u] = nrow[u]; pos[u] = npos[u]; }
  }
  // the last row with nonzeros and the empty rows after it
  while (k < r_hi) next_row();
}

template <typename T, typename TC, bool WARP>
static void *bwd_ptr_w(int V, int NV) {
  if (NV == 1) {
    if (V == 1) return (void *)fused_bwd_kernel<T, TC, 1, 1, WARP>;
    if (V == 2) return (void *)fused_bwd_kernel<T, TC, 2, 1, WARP>;
    if (V == 4) return (void *)fused_bwd_kernel<T, TC, 4, 1, WARP>;
  } else {
    if (V == 1) return (void *)fused_bwd_kernel<T, TC, 1, 2, WARP>;
    if (V == 2) return (void *)fused_bwd_kernel<T, TC, 2, 2, WARP>;
    if (V == 4) return (void *)fused_bwd_kernel<T, TC, 4, 2, WARP>;
  }
  return nullptr;
}

template <typename T, typename TC>
static void *bwd_ptr(int V, int NV, int lanes) {
  return lanes == 32 ? bwd_ptr_w<T, TC, true>(V, NV) : bwd_ptr_w<T, TC, false>(V, NV);
}

}  // namespace ss

using namespace ss;

extern "C" ss_status ss_spmm_backward(const ss_csr *AT, const int32_t *perm, const void *values, int N,
                                      const float *dC, const void *B, void *dB, int dB_dtype, float *dvals,
                                      int kahan_threshold, void *stream) {
  ss::NvtxRange nvtx_range("ss_spmm_backward");
  if (!AT || AT->nrow < 0 || AT->ncol < 0 || AT->nnz < 0 || N < 0) return fail(SS_ERR_INVALID_ARG, "bad arguments");
  const int dt = AT->value_dtype;
  if (dt < SS_F32 || dt > SS_F16) return fail(SS_ERR_INVALID_ARG, "value_dtype %d unknown", dt);
  if (dB_dtype != SS_F32 && dB_dtype != dt) return fail(SS_ERR_INVALID_ARG, "dB_dtype must be SS_F32 or the value dtype");
  const int K = AT->nrow, M = AT->ncol, nnz = AT->nnz;
  if (K == 0 || N == 0) return SS_OK;
  if (!AT->indptr || !dB || (nnz > 0 && (!AT->indices || !perm || !dC || !B || !dvals)))
    return fail(SS_ERR_INVALID_ARG, "null pointer");
  // V: widest vector (<= 16 bytes of FP32 dC) dividing N; lanes and NV cover N
  int V = 4;
  while (V > 1 && (N % V) != 0) V >>= 1;
  int lanes = ceil_pow2(ceil_div(N, V));
  if (lanes > 32) lanes = 32;
  const int NV = ceil_div(N, lanes * V);
  if (NV > 2)
    return fail(SS_ERR_UNSUPPORTED_KNOBS, "fused backward covers N <= %d here (got %d); use ss_sddmm and ss_spmm on A^T",
                64 * V, N);
  const int es = dtype_size(dt), cs = dtype_size(dB_dtype);
  if (((uintptr_t)dC % (4 * V)) || ((uintptr_t)B % (es * V)) || ((uintptr_t)dB % (cs * V)) ||
      ((uintptr_t)values % es) || ((uintptr_t)perm % 4))
    return fail(SS_ERR_ALIGNMENT, "dC / B / dB not aligned to the %d-element vector access", V);
  void *fn = nullptr;
  if (dt == SS_F32) fn = bwd_ptr<float, float>(V, NV, lanes);
  else if (dt == SS_BF16) fn = dB_dtype == SS_F32 ? bwd_ptr<__nv_bfloat16, float>(V, NV, lanes)
                                                  : bwd_ptr<__nv_bfloat16, __nv_bfloat16>(V, NV, lanes);
  else fn = dB_dtype == SS_F32 ? bwd_ptr<__half, float>(V, NV, lanes) : bwd_ptr<__half, __half>(V, NV, lanes);
  if (!fn) return fail(SS_ERR_UNSUPPORTED_KNOBS, "no fused backward kernel for V=%d NV=%d", V, NV);
  BwdArgs a;
  a.K = K; a.M = M; a.N = N; a.nnz = nnz;
  a.kahan = kahan_threshold > 0 ? kahan_threshold : 1024;
  a.t_indptr = AT->indptr; a.t_indices = AT->indices; a.perm = perm; a.vals = values;
  a.dC = dC; a.B = B; a.dB = dB; a.dvals = dvals;
  a.lanes = lanes; a.log2_lanes = ilog2(lanes);
  // shares of about nnz / (eight blocks per SM's groups) positions, at least 64
  const int threads = 256;
  const long long groups_per_block = threads / lanes;
  const long long target = (long long)sm_count() * 8 * groups_per_block;
  long long chunk = ((long long)nnz + target - 1) / target;
  if (chunk < 64) chunk = 64;
  long long groups = ((long long)nnz + chunk - 1) / chunk;
  if (groups < 1) groups = 1;
  a.chunk = (int)chunk;
  a.groups = (int)groups;
  const long long blocks = (groups + groups_per_block - 1) / groups_per_block;
  void *args[] = {&a};
  cudaError_t e = cudaLaunchKernel(fn, dim3((unsigned)blocks), dim3(threads), args, 0, (cudaStream_t)stream);
  return e == cudaSuccess ? SS_OK : cuda_fail(e, "fused backward launch");
}
