// Batched SpMM host side: plan building and the launch (kernels in
// batched.cuh, instantiated per storage type in batched_*.cu).
#include <algorithm>
#include <cstring>
#include <vector>

#include "batched.cuh"

namespace ss {

static size_t a256(size_t x) { return (x + 255) & ~(size_t)255; }

// Fills h (everything but the offsets' final sizes) and per-matrix chunk
// sizes; returns the number of items.
// strategies: per matrix SS_EBSR (element-balanced chunks) or SS_RBSR
// (blocks of whole rows), null = all SS_EBSR.
static ss_status batch_layout(int count, const ss_csr *mats, int N, const ss_knobs *per_mat, const int *strategies,
                              BatchHeader &h, std::vector<BatchMat> *out) {
  if (count < 1 || !mats || N < 1) return fail(SS_ERR_INVALID_ARG, "batch needs count >= 1, N >= 1 and matrices");
  const int dt = mats[0].value_dtype;
  ss_knobs k0;
  if (per_mat) k0 = per_mat[0];
  else ss_default_knobs(SS_EBSR, N, &k0);
  EbGeom g;
  ss_status st = geom_sr(1, 1, N, dt, dtype_size(dt), k0, g);
  if (st) return st;
  if (g.cs.NV != 1) return fail(SS_ERR_UNSUPPORTED_KNOBS, "batched walk needs one vector per lane (coarsen <= 16 B)");
  memset(&h, 0, sizeof(h));
  h.count = count;
  h.N = N;
  h.val_dtype = dt;
  h.V = g.cs.V;
  h.NV = g.cs.NV;
  h.G = g.team_lanes;
  h.log2G = ilog2(g.team_lanes);
  h.stage = g.stage;
  h.col_tile = g.cs.col_tile;
  h.tiles = g.cs.tiles;
  h.workers_per_block = g.workers_per_block;
  h.block = g.block;
  h.smem = g.smem;
  h.kahan = k0.kahan_threshold > 0 ? k0.kahan_threshold : 1024;
  long long items = 0;
  for (int m = 0; m < count; m++) {
    const ss_csr &A = mats[m];
    if (A.nrow < 0 || A.ncol < 0 || A.nnz < 0 || (A.nrow > 0 && !A.indptr) || (A.nnz > 0 && !A.indices))
      return fail(SS_ERR_INVALID_ARG, "matrix %d: bad descriptor", m);
    if (A.value_dtype != dt) return fail(SS_ERR_INVALID_ARG, "matrix %d: all matrices share one value dtype", m);
    const int tnz = per_mat ? per_mat[m].thread_nz : k0.thread_nz;
    if (tnz < 1 || tnz > 4096) return fail(SS_ERR_UNSUPPORTED_KNOBS, "matrix %d: thread_nz %d", m, tnz);
    BatchMat bm;
    memset(&bm, 0, sizeof(bm));
    bm.indptr = A.indptr;
    bm.indices = A.indices;
    bm.vals = A.values;
    bm.M = A.nrow;
    bm.K = A.ncol;
    bm.nnz = A.nnz;
    bm.chunk = tnz * h.G;
    bm.num_chunks = A.nnz > 0 ? ceil_div(A.nnz, bm.chunk) : (A.nrow > 0 ? 1 : 0);
    const int strategy = strategies ? strategies[m] : SS_EBSR;
    if (strategy != SS_EBSR && strategy != SS_RBSR)
      return fail(SS_ERR_UNSUPPORTED_KNOBS, "matrix %d: batched strategy %d is neither SS_EBSR nor SS_RBSR", m,
                  strategy);
    if (strategy == SS_RBSR && A.nnz > 0) {
      // whole rows per item, about one chunk of nonzeros at the mean row length
      const long long rows = ((long long)bm.chunk * A.nrow + A.nnz - 1) / A.nnz;
      bm.rows_per_item = (int)std::min<long long>(std::max(1LL, rows), (long long)A.nrow);
      bm.num_chunks = ceil_div(A.nrow, bm.rows_per_item);
    }
    bm.item_begin = (int)items;
    bm.use_tma = (((uintptr_t)A.indices & 15u) == 0) && (A.values == nullptr || ((uintptr_t)A.values & 15u) == 0) &&
                 (bm.chunk % 8) == 0;
    items += bm.num_chunks;
    if (items > 0x7fffffffLL) return fail(SS_ERR_CAPACITY, "too many work items");
    if (out) out->push_back(bm);
  }
  h.total_items = (int)items;
  size_t o = 0;
  h.mats_off = o; o += a256(sizeof(BatchMat) * (size_t)count);
  h.item_mat_off = o; o += a256(4 * (size_t)items);
  // arrival counts per (item, column tile), then the work counters: one
  // memset per step clears both
  h.rows_off = o; o += 4 * (size_t)items * (size_t)(h.tiles > 0 ? h.tiles : 1);
  h.counter_off = o; o = a256(o + 4 * (size_t)(h.tiles > 0 ? h.tiles : 1));
  h.heads_off = o; o += a256(4 * (size_t)items * N);
  h.tails_off = o; o += a256(4 * (size_t)items * N);
  h.dev_bytes = o;
  // the walk stores head/tail partials as vectors of up to 32 bytes
  if ((h.heads_off | h.tails_off | h.mats_off | h.item_mat_off | h.rows_off) & 255)
    return fail(SS_ERR_INVALID_ARG, "internal: misaligned batch plan layout");
  return SS_OK;
}

static size_t host_bytes_for(const BatchHeader &h) {
  return a256(sizeof(BatchHeader)) + a256(sizeof(BatchMat) * (size_t)h.count) + a256(4 * (size_t)h.total_items);
}

}  // namespace ss

using namespace ss;

extern "C" {

ss_status ss_batch_plan_size_ex(int count, const ss_csr *mats, int N, const ss_knobs *per_mat,
                                const int *per_mat_strategy, size_t *host_bytes, size_t *dev_bytes) {
  if (!host_bytes || !dev_bytes) return fail(SS_ERR_INVALID_ARG, "null size pointer");
  BatchHeader h;
  ss_status st = batch_layout(count, mats, N, per_mat, per_mat_strategy, h, nullptr);
  if (st) return st;
  *host_bytes = host_bytes_for(h);
  *dev_bytes = h.dev_bytes;
  return SS_OK;
}

ss_status ss_batch_plan_ex(int count, const ss_csr *mats, int N, const void *const *B, void *const *C,
                           int c_dtype, const ss_knobs *per_mat, const int *per_mat_strategy, void *host_buf,
                           size_t host_bytes, void *dev_buf, size_t dev_bytes, void *stream) {
  if (!B || !C || !host_buf || !dev_buf) return fail(SS_ERR_INVALID_ARG, "null pointer");
  BatchHeader h;
  std::vector<BatchMat> bm;
  ss_status st = batch_layout(count, mats, N, per_mat, per_mat_strategy, h, &bm);
  if (st) return st;
  if (c_dtype != SS_F32 && c_dtype != h.val_dtype) return fail(SS_ERR_INVALID_ARG, "c_dtype must be F32 or the value dtype");
  h.c_dtype = c_dtype;
  if (host_bytes < host_bytes_for(h) || dev_bytes < h.dev_bytes || ((uintptr_t)dev_buf % 256))
    return fail(SS_ERR_WORKSPACE, "plan needs %zu host bytes and %zu device bytes (256-byte aligned)",
                host_bytes_for(h), h.dev_bytes);
  const int es = dtype_size(h.val_dtype), cs = dtype_size(c_dtype);
  for (int m = 0; m < count; m++) {
    if ((mats[m].nnz > 0 && !B[m]) || (mats[m].nrow > 0 && !C[m]))
      return fail(SS_ERR_INVALID_ARG, "matrix %d: null B or C", m);
    if (((uintptr_t)B[m] % (size_t)(es * h.V)) || ((uintptr_t)C[m] % (size_t)(cs * h.V)))
      return fail(SS_ERR_ALIGNMENT, "matrix %d: B/C not aligned to the %d-element vector", m, h.V);
    bm[m].B = B[m];
    bm[m].C = C[m];
  }
  char *hb = (char *)host_buf;
  memcpy(hb, &h, sizeof(h));
  BatchMat *hm = (BatchMat *)(hb + a256(sizeof(BatchHeader)));
  memcpy(hm, bm.data(), sizeof(BatchMat) * (size_t)count);
  int32_t *him = (int32_t *)((char *)hm + a256(sizeof(BatchMat) * (size_t)count));
  for (int m = 0; m < count; m++)
    for (int c = 0; c < bm[m].num_chunks; c++) him[bm[m].item_begin + c] = m;
  cudaStream_t s = (cudaStream_t)stream;
  cudaError_t e = cudaMemcpyAsync((char *)dev_buf + h.mats_off, hm, sizeof(BatchMat) * (size_t)count,
                                  cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess && h.total_items > 0)
    e = cudaMemcpyAsync((char *)dev_buf + h.item_mat_off, him, 4 * (size_t)h.total_items, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);  // the host buffer may be reused after return
  return e == cudaSuccess ? SS_OK : cuda_fail(e, "batch plan upload");
}

ss_status ss_batch_plan_size(int count, const ss_csr *mats, int N, const ss_knobs *per_mat, size_t *host_bytes,
                             size_t *dev_bytes) {
  return ss_batch_plan_size_ex(count, mats, N, per_mat, nullptr, host_bytes, dev_bytes);
}

ss_status ss_batch_plan(int count, const ss_csr *mats, int N, const void *const *B, void *const *C, int c_dtype,
                        const ss_knobs *per_mat, void *host_buf, size_t host_bytes, void *dev_buf, size_t dev_bytes,
                        void *stream) {
  return ss_batch_plan_ex(count, mats, N, B, C, c_dtype, per_mat, nullptr, host_buf, host_bytes, dev_buf, dev_bytes,
                          stream);
}

ss_status ss_spmm_batched(const void *host_plan, void *dev_plan, void *stream) {
  ss::NvtxRange nvtx_range("ss_spmm_batched");
  if (!host_plan || !dev_plan) return fail(SS_ERR_INVALID_ARG, "null plan");
  BatchHeader h;
  memcpy(&h, host_plan, sizeof(h));
  if (h.total_items == 0) return SS_OK;
  cudaStream_t s = (cudaStream_t)stream;
  void *fn;
  if (h.val_dtype == SS_F32) fn = batched_kernel_f32(h.V, h.NV);
  else if (h.val_dtype == SS_BF16) fn = batched_kernel_bf16(h.V, h.NV, h.c_dtype == SS_F32);
  else fn = batched_kernel_f16(h.V, h.NV, h.c_dtype == SS_F32);
  if (!fn) return fail(SS_ERR_UNSUPPORTED_KNOBS, "no batched kernel for V=%d NV=%d", h.V, h.NV);
  cudaError_t e;
  if (h.smem > 48 * 1024) {
    e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)h.smem);
    if (e != cudaSuccess) return cuda_fail(e, "batched smem attribute");
  }
  int per_sm = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, h.block, h.smem);
  if (e != cudaSuccess || per_sm < 1) return fail(SS_ERR_UNSUPPORTED_KNOBS, "batched block does not fit an SM");
  long long grid = (long long)per_sm * sm_count();
  const long long need = ((long long)h.total_items + h.workers_per_block - 1) / h.workers_per_block;
  if (grid > need) grid = need;
  // arrival counts and work counters (adjacent in the plan)
  e = cudaMemsetAsync((char *)dev_plan + h.rows_off, 0, h.heads_off - h.rows_off, s);
  if (e != cudaSuccess) return cuda_fail(e, "batched counter reset");
  int *err_ptr = walk_error_ptr();
  const char *plan = (const char *)dev_plan;
  void *args[] = {&plan, &h, &err_ptr};
  e = cudaLaunchKernel(fn, dim3((unsigned)grid, (unsigned)h.tiles, 1), dim3(h.block, 1, 1), args, h.smem, s);
  return e == cudaSuccess ? SS_OK : cuda_fail(e, "batched launch");
}

}  // extern "C"
