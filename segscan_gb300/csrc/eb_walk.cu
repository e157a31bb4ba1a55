// Element-balanced, sequential reduction: ebsr SpMM and the sequential
// segment_coo family.
//
// Reference counterparts: csrspmm_rowcaching_nnzbalance_cg_kernel
// (test-cg/include/spmm/spmm_cg.cuh:376-551) and segscan_sr_kernel /
// segscan_sr_noshmem_kernel / segscan_sr_noshmem_lessatom_kernel /
// segscan_sr_sorted_kernel (new-cg/include/segscan/segscan.cuh:357-815).
//
// A worker is a group of G lanes laid along N (lane l owns E = V*NV
// consecutive columns, so one gathered B row is a single contiguous request
// across the group).  The worker stages its chunk's (column, value, row)
// triples in shared memory, then walks them in order, gathering four B rows
// ahead of the multiply-adds and flushing a row whenever the row id changes
// (eb_common.cuh: owner store / head carry / zero gaps).
#include "eb_common.cuh"
#include "internal.h"

namespace ss {

constexpr int SR_UNROLL = 4;

template <typename T, typename TC, int V, int NV, bool SEG, bool KAHAN>
__device__ __forceinline__ void sr_chunk(const EbArgs &a, int chunk, int lane, unsigned mask,
                                         int *s_col, float *s_val, int *s_row, int col0,
                                         const bool (&act)[NV], uint64_t keep, uint64_t strm) {
  const T *__restrict__ B = (const T *)a.B;
  const T *__restrict__ vals = (const T *)a.vals;
  const int G = a.team_lanes;
  const bool is_max = SEG && a.reduce == SS_MAX;
  const float ident = is_max ? -INFINITY : 0.f;

  const ChunkInfo ci = chunk_info<SEG>(a, chunk);
  if (blockIdx.y == 0 && lane == 0) a.carry_rows[chunk] = ci.has_head ? ci.r_first : -1;
  if (!a.accumulate && !ci.has_head) zero_rows<TC, V, NV>(a, ci.prev_row + 1, ci.r_first - 1, col0, act, strm);

  int cur = ci.r_first;
  int cnt = 0;
  float acc[NV][V], comp[NV][V];
  #pragma unroll
  for (int j = 0; j < NV; j++)
    #pragma unroll
    for (int i = 0; i < V; i++) { acc[j][i] = ident; comp[j][i] = 0.f; }

  for (int sb = ci.cs; sb < ci.ce; sb += a.stage) {
    const int n = min(a.stage, ci.ce - sb);
    __syncwarp(mask);  // the previous stage has been consumed
    for (int i = lane; i < n; i += G) {
      const int p = sb + i;
      if (SEG) {
        s_col[i] = p;
        s_val[i] = 1.f;
      } else {
        int c = ld_idx(a.cols + p, strm);
        float v = load_val<T>(vals, p, strm);
        if ((unsigned)c >= (unsigned)a.K) { c = 0; v = 0.f; }
        s_col[i] = c;
        s_val[i] = v;
      }
      s_row[i] = chunk_row<SEG>(a, ci, p);
    }
    __syncwarp(mask);
    for (int q = 0; q < n; q += SR_UNROLL) {
      float b[SR_UNROLL][NV][V];
      #pragma unroll
      for (int u = 0; u < SR_UNROLL; u++) {
        const bool live = q + u < n;
        const int c = live ? s_col[q + u] : 0;
        #pragma unroll
        for (int j = 0; j < NV; j++) {
          if (live && act[j]) {
            load_vec<T, V>(B + (int64_t)c * a.N + col0 + j * V, b[u][j], SEG ? strm : keep);
          } else {
            #pragma unroll
            for (int i = 0; i < V; i++) b[u][j][i] = 0.f;
          }
        }
      }
      #pragma unroll
      for (int u = 0; u < SR_UNROLL; u++) {
        if (q + u >= n) break;
        const int r = s_row[q + u];
        const float v = s_val[q + u];
        if (r != cur) {
          flush_row<TC, V, NV>(a, ci, chunk, cur, acc, cnt, true, col0, act, strm);
          if (!a.accumulate) zero_rows<TC, V, NV>(a, cur + 1, r - 1, col0, act, strm);
          cur = r;
          cnt = 0;
          #pragma unroll
          for (int j = 0; j < NV; j++)
            #pragma unroll
            for (int i = 0; i < V; i++) { acc[j][i] = ident; comp[j][i] = 0.f; }
        }
        cnt++;
        #pragma unroll
        for (int j = 0; j < NV; j++)
          #pragma unroll
          for (int i = 0; i < V; i++) {
            if (is_max) acc[j][i] = fmaxf(acc[j][i], b[u][j][i]);
            else if (KAHAN) kahan_add(acc[j][i], comp[j][i], v * b[u][j][i]);
            else acc[j][i] = fmaf(v, b[u][j][i], acc[j][i]);
          }
      }
    }
  }
  const bool complete = row_ends_in_chunk<SEG>(a, ci, cur);
  flush_row<TC, V, NV>(a, ci, chunk, cur, acc, cnt, complete, col0, act, strm);
  if (!a.accumulate && ci.ce >= a.nnz) zero_rows<TC, V, NV>(a, cur + 1, a.M - 1, col0, act, strm);
}

template <typename T, typename TC, int V, int NV, bool SEG>
__global__ void __launch_bounds__(1024) eb_sr_kernel(EbArgs a) {
  extern __shared__ int4 smem_raw[];
  const int tid = threadIdx.x;
  const int lane = tid & (a.team_lanes - 1);
  const int wib = tid >> a.log2_team_lanes;
  const unsigned wl = tid & 31;
  const unsigned mask = a.team_lanes >= 32
                            ? 0xffffffffu
                            : (((1u << a.team_lanes) - 1u) << (wl & ~(unsigned)(a.team_lanes - 1)));
  int *s_col = reinterpret_cast<int *>(smem_raw) + (size_t)wib * a.stage * 3;
  float *s_val = reinterpret_cast<float *>(s_col + a.stage);
  int *s_row = s_col + 2 * a.stage;
  const int col0 = blockIdx.y * a.col_tile + lane * (V * NV);
  bool act[NV];
  #pragma unroll
  for (int j = 0; j < NV; j++) act[j] = col0 + j * V < a.N;
  const uint64_t keep = policy_keep(), strm = policy_stream();
  const bool kahan = a.chunk > a.kahan;
  const int stride = gridDim.x * a.workers_per_block;
  for (int chunk = blockIdx.x * a.workers_per_block + wib; chunk < a.num_chunks; chunk += stride) {
    if (kahan) sr_chunk<T, TC, V, NV, SEG, true>(a, chunk, lane, mask, s_col, s_val, s_row, col0, act, keep, strm);
    else sr_chunk<T, TC, V, NV, SEG, false>(a, chunk, lane, mask, s_col, s_val, s_row, col0, act, keep, strm);
  }
}

// ---------------------------------------------------------------------
// Launch
// ---------------------------------------------------------------------
template <typename T, typename TC, bool SEG>
static void *sr_ptr(int V, int NV) {
  if (NV == 1) {
    if (V == 1) return (void *)eb_sr_kernel<T, TC, 1, 1, SEG>;
    if (V == 2) return (void *)eb_sr_kernel<T, TC, 2, 1, SEG>;
    if (V == 4) return (void *)eb_sr_kernel<T, TC, 4, 1, SEG>;
    if constexpr (sizeof(T) == 2) if (V == 8) return (void *)eb_sr_kernel<T, TC, 8, 1, SEG>;
  } else {
    if (V == 1) return (void *)eb_sr_kernel<T, TC, 1, 2, SEG>;
    if (V == 2) return (void *)eb_sr_kernel<T, TC, 2, 2, SEG>;
    if (V == 4) return (void *)eb_sr_kernel<T, TC, 4, 2, SEG>;
    if constexpr (sizeof(T) == 2) if (V == 8) return (void *)eb_sr_kernel<T, TC, 8, 2, SEG>;
  }
  return nullptr;
}

EbArgs eb_base_args(const EbGeom &g, void *ws, int N);

static ss_status run_sr(void *fn, EbArgs &a, const EbGeom &g, cudaStream_t s, const char *what) {
  if (!fn) return fail(SS_ERR_UNSUPPORTED_KNOBS, "no %s kernel for V=%d NV=%d", what, g.cs.V, g.cs.NV);
  if (g.smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)g.smem);
    if (e != cudaSuccess) return cuda_fail(e, what);
  }
  dim3 grid(g.grid_x, g.cs.tiles, 1), block(g.block, 1, 1);
  void *args[] = {&a};
  cudaError_t err = cudaLaunchKernel(fn, grid, block, args, g.smem, s);
  if (err != cudaSuccess) return cuda_fail(err, what);
  return SS_OK;
}

ss_status launch_ebsr(const SpmmCall &c, const EbGeom &g, void *ws, cudaStream_t s) {
  EbArgs a = eb_base_args(g, ws, c.N);
  a.M = c.M; a.K = c.K; a.nnz = c.nnz;
  a.indptr = c.indptr; a.cols = c.indices; a.index = nullptr; a.vals = c.vals; a.B = c.B; a.C = c.C;
  a.accumulate = c.accumulate; a.reduce = SS_SUM; a.kahan = c.kahan_threshold;
  void *fn = nullptr;
  if (c.val_dtype == SS_F32) fn = sr_ptr<float, float, false>(g.cs.V, g.cs.NV);
  else if (c.val_dtype == SS_BF16)
    fn = c.c_dtype == SS_F32 ? sr_ptr<__nv_bfloat16, float, false>(g.cs.V, g.cs.NV)
                             : sr_ptr<__nv_bfloat16, __nv_bfloat16, false>(g.cs.V, g.cs.NV);
  else
    fn = c.c_dtype == SS_F32 ? sr_ptr<__half, float, false>(g.cs.V, g.cs.NV)
                             : sr_ptr<__half, __half, false>(g.cs.V, g.cs.NV);
  ss_status st = run_sr(fn, a, g, s, "ebsr launch");
  if (st != SS_OK) return st;
  return launch_fixup(carry_view(ws, g.num_chunks, c.N), g.num_chunks, c.N, c.M, c.C, c.c_dtype, SS_SUM, c.accumulate,
                      nullptr, c.nnz, s);
}

ss_status launch_seg_sr(const SegCall &c, const EbGeom &g, void *ws, cudaStream_t s) {
  EbArgs a = eb_base_args(g, ws, c.N);
  a.M = c.dst_len; a.K = c.nnz; a.nnz = c.nnz;
  a.indptr = nullptr; a.cols = nullptr; a.index = c.index; a.vals = nullptr; a.B = c.src; a.C = c.dst;
  a.accumulate = c.accumulate; a.reduce = c.reduce; a.kahan = c.kahan_threshold;
  void *fn = nullptr;
  if (c.src_dtype == SS_F32) fn = sr_ptr<float, float, true>(g.cs.V, g.cs.NV);
  else if (c.src_dtype == SS_BF16) fn = sr_ptr<__nv_bfloat16, float, true>(g.cs.V, g.cs.NV);
  else fn = sr_ptr<__half, float, true>(g.cs.V, g.cs.NV);
  ss_status st = run_sr(fn, a, g, s, "segment_coo sr launch");
  if (st != SS_OK) return st;
  return launch_fixup(carry_view(ws, g.num_chunks, c.N), g.num_chunks, c.N, c.dst_len, c.dst, SS_F32, c.reduce, c.accumulate,
                      c.index, c.nnz, s);
}

}  // namespace ss
