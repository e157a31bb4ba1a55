// Element-balanced, parallel reduction: ebpr SpMM and the shuffle-scan
// segment_coo family.
//
// Reference counterparts: csrspmm_parreduce_nnzbalance_cg_kernel
// (test-cg/include/spmm/spmm_cg.cuh:14-175), segscan_kernel and
// segscan_new_kernel (new-cg/include/segscan/segscan.cuh:7-148, 186-325).
//
// A worker is a tile of `tile` lanes, one nonzero per lane per step, times
// `colgroups` column groups (each lane of a group owns one V-wide slice of
// the column tile, as the reference's access_t does).  Each step multiplies
// `tile` consecutive nonzeros by their B slices and runs a segmented
// inclusive scan across the lanes (shuffles; rows are the segment keys).
// The last lane's segment carries into the next step in registers; every
// segment that ends inside the chunk is flushed once (eb_common.cuh), so
// there are no atomics.  The reference instead atomically adds every
// segment head into a pre-zeroed C.
#include "eb_common.cuh"
#include "internal.h"

namespace ss {

// Row of nonzero p from the staged row starts win[i] = indptr[r_first + i],
// i < nwin: the same upper_bound - 1 as row_search over [r_first + 1,
// r_last + 1), read from shared memory.
__device__ __forceinline__ int win_row(const int32_t *win, int nwin, int r_first, int p) {
  int lo = 1, hi = nwin - 1;
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (win[mid] <= p) lo = mid + 1; else hi = mid;
  }
  return r_first + hi - 1;
}

template <typename T, typename TC, int V, bool SEG>
__global__ void __launch_bounds__(1024) eb_pr_kernel(EbArgs a) {
  extern __shared__ int32_t pr_win[];  // [tile-lane sets of the block][a.stage] (SpMM)
  const T *__restrict__ B = (const T *)a.B;
  const T *__restrict__ vals = (const T *)a.vals;
  const int tile = a.team_lanes;
  const int tid = threadIdx.x;
  const int lane = tid & (tile - 1);
  const int cg = (tid >> a.log2_team_lanes) & (a.colgroups - 1);
  const int wib = tid >> (a.log2_team_lanes + a.log2_colgroups);
  const unsigned wl = tid & 31;
  const unsigned mask = tile >= 32 ? 0xffffffffu : (((1u << tile) - 1u) << (wl & ~(unsigned)(tile - 1)));
  const int col0 = blockIdx.y * a.col_tile + cg * V;
  bool act[1] = {col0 < a.N};
  const uint64_t keep = policy_keep(a.keep_frac), strm = policy_stream();
  const bool is_max = SEG && a.reduce == SS_MAX;
  const float ident = is_max ? -INFINITY : 0.f;
  const int stride = gridDim.x * a.workers_per_block;

  int32_t *win = pr_win + (size_t)(tid >> a.log2_team_lanes) * a.stage;
  const int W = a.stage;
  for (int chunk = blockIdx.x * a.workers_per_block + wib; chunk < a.num_chunks; chunk += stride) {
    const ChunkInfo ci = SEG ? chunk_info<SEG>(a, chunk) : chunk_info_group(a, chunk, lane, tile, mask);
    if (blockIdx.y == 0 && cg == 0 && lane == 0) a.carry_rows[chunk] = ci.has_head ? ci.r_first : -1;

    // running segment carried across steps; without a head row it starts as
    // the row before the chunk, so the first step zeroes the gap after it
    int run_row = ci.has_head ? ci.r_first : ci.prev_row;
    float run[1][V];
    int run_cnt = 0;
    #pragma unroll
    for (int i = 0; i < V; i++) run[0][i] = ident;

    // SpMM: a sliding window of row starts in shared memory, win[i] =
    // indptr[min(win_base + i, M)], refilled from the current row whenever a
    // step reaches past it; rows are searched there, not in global memory
    int win_base = -1;
    // the next step's column and value are loaded one step ahead
    int c_next = 0;
    float v_next = 0.f;
    if (!SEG && ci.cs + lane < ci.ce) {
      c_next = ld_idx(a.cols + ci.cs + lane, strm);
      v_next = load_val<T>(vals, ci.cs + lane, strm);
    }

    for (int sb = ci.cs; sb < ci.ce; sb += tile) {
      const int p = sb + lane;
      const bool live = p < ci.ce;
      const int nlive = min(tile, ci.ce - sb);
      int row = INT_MAX;
      float x[1][V];
      int cnt = 0;
      #pragma unroll
      for (int i = 0; i < V; i++) x[0][i] = ident;
      int c = 0;
      float v = 0.f;
      float b[V];
      if (SEG) {
        c = p;
        v = 1.f;
      } else {
        c = c_next;
        v = v_next;
        if ((unsigned)c >= (unsigned)a.K) { c = 0; v = 0.f; }
        if (live && act[0]) load_vec<T, V>(B + (int64_t)c * a.N + col0, b, keep);
        const int pn = p + tile;
        if (pn < ci.ce) {
          c_next = ld_idx(a.cols + pn, strm);
          v_next = load_val<T>(vals, pn, strm);
        }
        // window: must hold the start of the step's last row's successor
        const int plast = sb + nlive - 1;
        const int rs = max(run_row, ci.r_first);  // row of nonzero sb is at least this
        const bool stale = W > 0 && (win_base < 0 || rs < win_base ||
                                     (win[W - 1] <= plast && win_base + W - 1 < a.M));
        if (stale) {
          __syncwarp(mask);
          win_base = rs;
          for (int i = lane; i < W; i += tile) win[i] = __ldg(a.indptr + min(win_base + i, a.M));
          __syncwarp(mask);
        }
      }
      if (live) {
        if (SEG) {
          row = chunk_row<SEG>(a, ci, p);
        } else if (W > 0 && (p < win[W - 1] || win_base + W - 1 >= a.M) && win[0] <= p) {
          int lo = 1, hi = W - 1;  // first slot whose start is past p
          while (lo < hi) {
            const int mid = (lo + hi) >> 1;
            if (win[mid] <= p) lo = mid + 1; else hi = mid;
          }
          row = min(win_base + hi - 1, ci.r_last);
        } else {
          row = chunk_row<SEG>(a, ci, p);
        }
        if (SEG) {
          if (act[0]) load_vec<T, V>(B + (int64_t)c * a.N + col0, b, strm);
        }
        if (act[0]) {
          #pragma unroll
          for (int i = 0; i < V; i++) x[0][i] = is_max ? b[i] : v * b[i];
        }
        cnt = 1;
      }
      // the carried segment ended at the previous step's last lane
      if (run_cnt > 0 && __shfl_sync(mask, row, 0, tile) != run_row) {
        if (lane == 0) flush_row<TC, V, 1>(a, ci, chunk, run_row, run, run_cnt, true, col0, act, strm);
        run_cnt = 0;
        #pragma unroll
        for (int i = 0; i < V; i++) run[0][i] = ident;
      }
      // segmented inclusive scan over the tile (rows are the keys)
      for (int off = 1; off < tile; off <<= 1) {
        const int r2 = __shfl_up_sync(mask, row, off, tile);
        const int c2 = __shfl_up_sync(mask, cnt, off, tile);
        float x2[V];
        #pragma unroll
        for (int i = 0; i < V; i++) x2[i] = __shfl_up_sync(mask, x[0][i], off, tile);
        if (lane >= off && r2 == row) {
          cnt += c2;
          #pragma unroll
          for (int i = 0; i < V; i++) x[0][i] = is_max ? fmaxf(x[0][i], x2[i]) : x[0][i] + x2[i];
        }
      }
      // carry-in from the previous step (only the first segment can match)
      if (live && run_cnt > 0 && row == run_row) {
        cnt += run_cnt;
        #pragma unroll
        for (int i = 0; i < V; i++) x[0][i] = is_max ? fmaxf(x[0][i], run[0][i]) : x[0][i] + run[0][i];
      }
      int prev_r = __shfl_up_sync(mask, row, 1, tile);
      int next_r = __shfl_down_sync(mask, row, 1, tile);
      if (lane == 0) prev_r = run_row;
      const bool next_live = lane + 1 < nlive;
      if (live && row != prev_r && !a.accumulate)
        zero_rows<TC, V, 1>(a, prev_r + 1, row - 1, col0, act, strm);
      if (live && next_live && next_r != row)
        flush_row<TC, V, 1>(a, ci, chunk, row, x, cnt, true, col0, act, strm);
      // the last live lane's segment continues into the next step
      run_row = __shfl_sync(mask, row, nlive - 1, tile);
      run_cnt = __shfl_sync(mask, cnt, nlive - 1, tile);
      #pragma unroll
      for (int i = 0; i < V; i++) run[0][i] = __shfl_sync(mask, x[0][i], nlive - 1, tile);
    }
    if (lane == 0) {
      const bool complete = row_ends_in_chunk<SEG>(a, ci, run_row);
      flush_row<TC, V, 1>(a, ci, chunk, run_row, run, run_cnt, complete, col0, act, strm);
      if (!a.accumulate && ci.ce >= a.nnz) zero_rows<TC, V, 1>(a, run_row + 1, a.M - 1, col0, act, strm);
    }
  }
}

template <typename T, typename TC, bool SEG>
static void *pr_ptr(int V) {
  if (V == 1) return (void *)eb_pr_kernel<T, TC, 1, SEG>;
  if (V == 2) return (void *)eb_pr_kernel<T, TC, 2, SEG>;
  if (V == 4) return (void *)eb_pr_kernel<T, TC, 4, SEG>;
  if constexpr (sizeof(T) == 2) if (V == 8) return (void *)eb_pr_kernel<T, TC, 8, SEG>;
  return nullptr;
}

EbArgs eb_base_args(const EbGeom &g, void *ws, int N);

static ss_status run_pr(void *fn, EbArgs &a, const EbGeom &g, cudaStream_t s, const char *what) {
  if (!fn) return fail(SS_ERR_UNSUPPORTED_KNOBS, "no %s kernel for V=%d", what, g.cs.V);
  dim3 grid(g.grid_x, g.cs.tiles, 1), block(g.block, 1, 1);
  void *args[] = {&a};
  cudaError_t err = cudaLaunchKernel(fn, grid, block, args, g.smem, s);
  if (err != cudaSuccess) return cuda_fail(err, what);
  return SS_OK;
}

ss_status launch_ebpr(const SpmmCall &c, const EbGeom &g, void *ws, cudaStream_t s) {
  EbArgs a = eb_base_args(g, ws, c.N);
  a.M = c.M; a.K = c.K; a.nnz = c.nnz;
  a.indptr = c.indptr; a.cols = c.indices; a.index = nullptr; a.vals = c.vals; a.B = c.B; a.C = c.C;
  a.accumulate = c.accumulate; a.reduce = SS_SUM; a.kahan = c.kahan_threshold;
  a.keep_frac = l2_keep_fraction((size_t)c.K * c.N * dtype_size(c.val_dtype));
  void *fn;
  if (c.val_dtype == SS_F32) fn = pr_ptr<float, float, false>(g.cs.V);
  else if (c.val_dtype == SS_BF16)
    fn = c.c_dtype == SS_F32 ? pr_ptr<__nv_bfloat16, float, false>(g.cs.V)
                             : pr_ptr<__nv_bfloat16, __nv_bfloat16, false>(g.cs.V);
  else
    fn = c.c_dtype == SS_F32 ? pr_ptr<__half, float, false>(g.cs.V) : pr_ptr<__half, __half, false>(g.cs.V);
  ss_status st = run_pr(fn, a, g, s, "ebpr launch");
  if (st != SS_OK) return st;
  return launch_fixup(carry_view(ws, g.num_chunks, c.N, g.cs.tiles), g.num_chunks, c.N, c.M, c.C, c.c_dtype, SS_SUM, c.accumulate,
                      nullptr, c.nnz, s);
}

ss_status launch_seg_pr(const SegCall &c, const EbGeom &g, void *ws, cudaStream_t s) {
  EbArgs a = eb_base_args(g, ws, c.N);
  a.M = c.dst_len; a.K = c.nnz; a.nnz = c.nnz;
  a.indptr = nullptr; a.cols = nullptr; a.index = c.index; a.vals = nullptr; a.B = c.src; a.C = c.dst;
  a.accumulate = c.accumulate; a.reduce = c.reduce; a.kahan = c.kahan_threshold;
  void *fn;
  if (c.src_dtype == SS_F32) fn = pr_ptr<float, float, true>(g.cs.V);
  else if (c.src_dtype == SS_BF16) fn = pr_ptr<__nv_bfloat16, float, true>(g.cs.V);
  else fn = pr_ptr<__half, float, true>(g.cs.V);
  ss_status st = run_pr(fn, a, g, s, "segment_coo pr launch");
  if (st != SS_OK) return st;
  return launch_fixup(carry_view(ws, g.num_chunks, c.N, g.cs.tiles), g.num_chunks, c.N, c.dst_len, c.dst, SS_F32, c.reduce, c.accumulate,
                      c.index, c.nnz, s);
}

}  // namespace ss
