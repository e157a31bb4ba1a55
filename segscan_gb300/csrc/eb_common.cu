// Carry fix-up for the element-balanced kernels (see eb_common.cuh).
//
// Chunk c's head slot holds the partial of its head row r (a row that
// started in an earlier chunk) or -1.  The first chunk of each run of
// consecutive chunks with the same head row is the run's leader; the chunk
// before it owns r and left r's partial in its tail slot.  The leader sums
// tail + heads in chunk order (compensated), adds the old output in
// accumulate mode, divides by the segment length for a mean, and stores the
// row once.  The order is fixed, so results are reproducible bit for bit.
#include "eb_common.cuh"
#include "internal.h"

#include <algorithm>

namespace ss {

size_t carry_rows_bytes(int num_chunks, int tiles) {
  return ((size_t)num_chunks * (size_t)std::max(1, tiles) * sizeof(int32_t) + 255) & ~(size_t)255;
}

size_t eb_workspace_bytes(const EbGeom &g, int N) {
  return carry_rows_bytes(g.num_chunks, g.cs.tiles) + 2 * (size_t)g.num_chunks * (size_t)N * sizeof(float);
}

size_t seg_sr_workspace_bytes(const EbGeom &g, int N) {
  return eb_workspace_bytes(g, N) + (((size_t)2 * g.num_chunks * sizeof(int32_t) + 255) & ~(size_t)255);
}

CarryView carry_view(void *ws, int num_chunks, int N, int tiles) {
  CarryView cv;
  size_t rows = carry_rows_bytes(num_chunks, tiles);
  cv.rows = (int32_t *)ws;
  cv.vals = (float *)((char *)ws + rows);
  cv.tails = cv.vals + (size_t)num_chunks * (size_t)N;
  return cv;
}

EbArgs eb_base_args(const EbGeom &g, void *ws, int N) {
  EbArgs a;
  a.N = N;
  a.team_lanes = g.team_lanes;
  a.log2_team_lanes = ilog2(g.team_lanes);
  a.colgroups = g.team_threads / g.team_lanes;
  a.log2_colgroups = ilog2(a.colgroups);
  a.col_tile = g.cs.col_tile;
  a.chunk = g.chunk;
  a.num_chunks = g.num_chunks;
  a.workers_per_block = g.workers_per_block;
  a.stage = g.stage;
  a.use_tma = 0;
  a.err = nullptr;
  a.keep_frac = 1.0f;
  CarryView cv = carry_view(ws, g.num_chunks, N, g.cs.tiles);
  a.carry_rows = cv.rows;
  a.carry_vals = cv.vals;
  a.tail_vals = cv.tails;
  a.carry_cnt = cv.rows;
  a.seg_cnt = nullptr;
  return a;
}

template <typename TC>
__global__ void __launch_bounds__(256) carry_fixup_kernel(const int32_t *__restrict__ rows,
                                                          const float *__restrict__ heads,
                                                          const float *__restrict__ tails, int num_chunks,
                                                          int N, int M, TC *C, int reduce, int accumulate,
                                                          const int32_t *__restrict__ index, int nnz) {
  // launched as a programmatic dependent of the walk kernel: wait until the
  // walk's writes (head/tail slots, owner rows) are complete and visible
  asm volatile("griddepcontrol.wait;" ::: "memory");
  // one warp per chunk, so the runs are assembled in parallel; most chunks
  // are not run leaders and return after two loads
  const int lane = threadIdx.x & 31;
  const int warps = (gridDim.x * blockDim.x) >> 5;
  for (int c = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; c < num_chunks; c += warps)
    fixup_chunk<TC>(rows, heads, tails, num_chunks, N, M, C, reduce, accumulate, index, nnz, c, lane);
}

ss_status launch_fixup(const CarryView &cv, int num_chunks, int N, int M, void *C, int c_dtype,
                       int reduce, int accumulate, const int32_t *index, int nnz, cudaStream_t s) {
  if (num_chunks <= 1 || N == 0 || M == 0) return SS_OK;  // chunk 0 never carries
  const int threads = 256;
  const int blocks = std::max(1, std::min((num_chunks + 7) / 8, sm_count() * 32));
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(blocks, 1, 1);
  cfg.blockDim = dim3(threads, 1, 1);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  cudaError_t e;
  if (c_dtype == SS_F32)
    e = cudaLaunchKernelEx(&cfg, carry_fixup_kernel<float>, (const int32_t *)cv.rows, (const float *)cv.vals,
                           (const float *)cv.tails, num_chunks, N, M, (float *)C, reduce, accumulate, index, nnz);
  else if (c_dtype == SS_BF16)
    e = cudaLaunchKernelEx(&cfg, carry_fixup_kernel<__nv_bfloat16>, (const int32_t *)cv.rows, (const float *)cv.vals,
                           (const float *)cv.tails, num_chunks, N, M, (__nv_bfloat16 *)C, reduce, accumulate, index,
                           nnz);
  else
    e = cudaLaunchKernelEx(&cfg, carry_fixup_kernel<__half>, (const int32_t *)cv.rows, (const float *)cv.vals,
                           (const float *)cv.tails, num_chunks, N, M, (__half *)C, reduce, accumulate, index, nnz);
  if (e != cudaSuccess) return cuda_fail(e, "carry fix-up launch");
  return SS_OK;
}

}  // namespace ss
