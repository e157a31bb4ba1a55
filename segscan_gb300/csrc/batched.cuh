// Batched SpMM: many independent CSR matrices in one persistent launch.
//
// No counterpart in the reference (its drivers launch one matrix at a time).
// A plan (host + device copies, built by ss_batch_plan) lists the matrices
// and numbers their work items: item i is chunk (i - item_begin[m]) of
// matrix m = item_mat[i], a chunk being thread_nz * G consecutive nonzeros
// of that matrix (its own knob, element-balanced), or, for a matrix planned
// row-balanced, a block of whole rows holding about that many nonzeros (each
// row then summed in order by one group, as rbsr sums it).  The persistent kernel runs one resident
// wave; every group takes the next item from a device counter (atomicAdd,
// no waiting on other groups) and walks it with the ebsr chunk walk
// (eb_walk.cuh) against that matrix's arrays.  Straddling rows go to the
// matrix's head/tail slots and the last of their chunks to finish
// assembles them (carry_arrive), so one launch does the whole step.
// Matrices without nonzeros get a zero-fill item.  The whole step (counter
// reset, walk) is stream-ordered and can be captured in a graph.
#pragma once
#include "eb_walk.cuh"

namespace ss {

struct BatchMat {
  const int32_t *indptr;
  const int32_t *indices;
  const void *vals;
  const void *B;
  void *C;
  int M, K, nnz;
  int chunk;          // element-balanced: nonzeros per item
  int num_chunks;     // items of this matrix (1 zero-fill item when nnz == 0)
  int item_begin;     // first item of this matrix
  int use_tma;
  int rows_per_item;  // row-balanced (> 0): whole rows per item, no row split
};

struct BatchHeader {
  int count, N, total_items, c_dtype, val_dtype;
  int V, NV, G, log2G, stage, col_tile, tiles, workers_per_block, block, grid, kahan;
  size_t smem;
  // device-side offsets (bytes from the plan base)
  size_t mats_off, item_mat_off, rows_off, heads_off, tails_off, counter_off;
  size_t dev_bytes;
};

template <typename T, typename TC, int V, int NV>
__global__ void __launch_bounds__(512, SS_SR_MIN_BLOCKS) batched_kernel(const char *plan, BatchHeader h,
                                                                         int *err) {
  extern __shared__ __align__(16) char smem_raw[];
  const BatchMat *mats = reinterpret_cast<const BatchMat *>(plan + h.mats_off);
  const int32_t *item_mat = reinterpret_cast<const int32_t *>(plan + h.item_mat_off);
  int32_t *rows_all = (int32_t *)(plan + h.rows_off);
  float *heads_all = (float *)(plan + h.heads_off);
  float *tails_all = (float *)(plan + h.tails_off);
  int *counter = (int *)(plan + h.counter_off);

  const int tid = threadIdx.x;
  const int G = h.G;
  const int lane = tid & (G - 1);
  const int wib = tid >> h.log2G;
  const unsigned wl = tid & 31;
  const unsigned mask = G >= 32 ? 0xffffffffu : (((1u << G) - 1u) << (wl & ~(unsigned)(G - 1)));
  const SrLayout L = sr_layout(h.stage, (int)sizeof(T));
  char *g = smem_raw + (size_t)wib * L.bytes;
  Stage st;
  st.bar = reinterpret_cast<uint64_t *>(g);
  st.col = reinterpret_cast<int32_t *>(g + L.col_off);
  st.val = g + L.val_off;
  st.info = reinterpret_cast<int32_t *>(g + L.info_off);
  st.win = reinterpret_cast<int32_t *>(g + L.win_off);
  st.phases = 0;
  st.tma = 0;
  if (lane == 0) {
    mbar_init(st.bar, 1);
    mbar_init(st.bar + 1, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncwarp(mask);
  const int col0 = blockIdx.y * h.col_tile + lane * (V * NV);
  bool act[NV];
  #pragma unroll
  for (int j = 0; j < NV; j++) act[j] = col0 + j * V < h.N;
  const uint64_t keep = policy_keep(1.0f), strm = policy_stream();

  EbArgs a;
  a.N = h.N;
  a.index = nullptr;
  a.accumulate = 0;
  a.reduce = SS_SUM;
  a.kahan = h.kahan;
  a.team_lanes = G;
  a.log2_team_lanes = h.log2G;
  a.colgroups = 1;
  a.log2_colgroups = 0;
  a.col_tile = h.col_tile;
  a.workers_per_block = h.workers_per_block;
  a.stage = h.stage;
  a.err = err;
  a.keep_frac = 1.0f;
  while (true) {
    int item = 0;
    if (lane == 0) item = atomicAdd(counter + blockIdx.y, 1);
    item = __shfl_sync(mask, item, 0, G);
    if (item >= h.total_items) break;
    const int m = item_mat[item];
    const BatchMat mt = mats[m];
    const int chunk = item - mt.item_begin;
    if (mt.nnz == 0) {  // zero-fill item
      a.M = mt.M;
      a.C = mt.C;
      zero_rows<TC, V, NV>(a, 0, mt.M - 1, col0, act, strm);
      continue;
    }
    a.M = mt.M;
    a.K = mt.K;
    a.nnz = mt.nnz;
    a.indptr = mt.indptr;
    a.cols = mt.indices;
    a.vals = mt.vals;
    a.B = mt.B;
    a.C = mt.C;
    a.chunk = mt.chunk;
    a.num_chunks = mt.num_chunks;
    a.use_tma = mt.use_tma;
    a.carry_rows = nullptr;
    a.carry_cnt = rows_all + (size_t)mt.item_begin * h.tiles;
    a.carry_vals = heads_all + (size_t)mt.item_begin * h.N;
    a.tail_vals = tails_all + (size_t)mt.item_begin * h.N;
    int cs, ce;
    if (mt.rows_per_item > 0) {  // a block of whole rows: each row summed by this group alone
      const int r0 = chunk * mt.rows_per_item;
      cs = __ldg(mt.indptr + r0);
      ce = __ldg(mt.indptr + min(mt.M, r0 + mt.rows_per_item));
      if (cs == ce) continue;  // empty rows only: the item holding the next nonzero zeroes them
    } else {
      cs = chunk * mt.chunk;
      ce = min(cs + mt.chunk, mt.nnz);
    }
    const bool done = sr_spmm_chunk<T, TC, V, NV>(a, chunk, cs, ce, lane, mask, st, L, col0, act, keep, strm);
    if (!done) break;  // a bounded wait expired
  }
}

template <typename T, typename TC>
inline void *batched_ptr(int V, int NV) {
  if (NV != 1) return nullptr;
  if (V == 1) return (void *)batched_kernel<T, TC, 1, 1>;
  if (V == 2) return (void *)batched_kernel<T, TC, 2, 1>;
  if (V == 4) return (void *)batched_kernel<T, TC, 4, 1>;
  if constexpr (sizeof(T) == 2) if (V == 8) return (void *)batched_kernel<T, TC, 8, 1>;
  return nullptr;
}

void *batched_kernel_f32(int V, int NV);
void *batched_kernel_bf16(int V, int NV, bool out_f32);
void *batched_kernel_f16(int V, int NV, bool out_f32);

}  // namespace ss
