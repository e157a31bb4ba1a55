// C ABI entry points: argument checks, knob -> launch geometry, dispatch.
//
// The geometry functions keep the formulas of the reference launchers
// (test-cg/include/spmm/spmm_cg.cuh:176-197, 333-353, 553-566, 664-677;
// new-cg/include/segscan/segscan.cuh:150-171, 817-829, 974-980) so a knob
// tuple means the same work decomposition here as there, with these
// deliberate differences (each fixes a reference hazard or maps it to
// GB300):
//  * lanes inside a team run along N, so a gathered B row is contiguous;
//  * an element-balanced worker owns one contiguous chunk of nonzeros
//    (ThreadNz * group for ebsr, steps * tile for ebpr) and the grid is cut
//    to the workers that own work, instead of launching nrow * block_factor
//    blocks that mostly exit;
//  * ebsr uses thread_per_block as the block size (the reference launches
//    256 threads whatever the knob says, spmm_cg.cuh:564);
//  * a coarsen factor that is not a power of two is rounded down and the
//    column grid recomputed (the reference falls back to CoarsenFactor 1 but
//    keeps the grid sized for the larger factor, dropping columns).
#include <atomic>
#include <cstdarg>
#include <cstdio>
#include <cstring>

#include "internal.h"

namespace ss {

static thread_local char g_last_error[512] = "";

ss_status fail(ss_status st, const char *fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_last_error, sizeof(g_last_error), fmt, ap);
  va_end(ap);
  return st;
}

ss_status cuda_fail(cudaError_t err, const char *what) {
  return fail(SS_ERR_CUDA, "%s: %s", what, cudaGetErrorString(err));
}

// L2 budget for the gathered operand; 0 = no budget (keep all of it, the
// measured best on the power-law SpMM at N = 16, 64, 128).
static std::atomic<long long> g_keep_bytes{0};

float l2_keep_fraction(size_t bytes) {
  const long long budget = g_keep_bytes.load(std::memory_order_relaxed);
  if (budget <= 0 || bytes == 0 || (long long)bytes <= budget) return 1.0f;
  float f = (float)((double)budget / (double)bytes);
  return f < 0.01f ? 0.01f : f;
}

// Largest power-of-two vector (<= 16 bytes, <= max_elems) dividing N.
static int pick_vec(int N, int dtype, int max_elems) {
  int v = 16 / dtype_size(dtype);
  if (max_elems < v) v = floor_pow2(max_elems < 1 ? 1 : max_elems);
  while (v > 1 && (N % v) != 0) v >>= 1;
  return v;
}

static ColSplit split_cols(int N, int dtype, int elems_req, int lanes_req) {
  ColSplit cs;
  int e = floor_pow2(elems_req < 1 ? 1 : (elems_req > 8 ? 8 : elems_req));
  cs.V = pick_vec(N, dtype, e);
  cs.NV = e / cs.V > 1 ? 2 : 1;
  int lanes = lanes_req < 1 ? 1 : lanes_req;
  lanes = ceil_pow2(lanes);
  if (lanes > 32) lanes = 32;
  cs.lanes = lanes;
  cs.col_tile = lanes * cs.V * cs.NV;
  cs.tiles = N > 0 ? ceil_div(N, cs.col_tile) : 0;
  return cs;
}

static long long workers_from_factor(long long units, const ss_knobs &k) {
  // (float)nrow * block_factor, truncated, as the reference launchers do
  float bf = (float)k.block_numer / (float)k.block_denom;
  long long w = (long long)((float)units * bf);
  return w < 1 ? 1 : w;
}

static ss_status check_common_knobs(const ss_knobs &k) {
  if (k.thread_per_block < 1 || k.thread_per_block > 1024)
    return fail(SS_ERR_UNSUPPORTED_KNOBS, "thread_per_block %d outside [1, 1024]", k.thread_per_block);
  if (k.block_numer < 1 || k.block_denom < 1 || k.block_numer > 1024 || k.block_denom > 1 << 20)
    return fail(SS_ERR_UNSUPPORTED_KNOBS, "block_factor %d/%d not positive", k.block_numer, k.block_denom);
  return SS_OK;
}

static int clamp_grid(long long g) {
  if (g < 1) g = 1;
  if (g > 0x7fffffffLL) g = 0x7fffffffLL;
  return (int)g;
}

// rbsr: csrspmm_seqreduce_rowbalance_cg (spmm_cg.cuh:664-677).
static ss_status geom_rbsr(int M, int N, int dtype, const ss_knobs &k, RbGeom &g) {
  ss_status st = check_common_knobs(k);
  if (st) return st;
  if (k.coarsen_factor < 1 || k.coarsen_factor > 8)
    return fail(SS_ERR_UNSUPPORTED_KNOBS, "rbsr coarsen_factor %d outside [1, 8]", k.coarsen_factor);
  if (k.tile_factor < 0 || k.tile_factor > 10)
    return fail(SS_ERR_UNSUPPORTED_KNOBS, "rbsr tile_factor %d outside [0, 10]", k.tile_factor);
  const int tile = 1 << k.tile_factor;
  ColSplit probe = split_cols(N, dtype, k.coarsen_factor, 1);
  const int E = probe.V * probe.NV;
  const int span = N < tile ? N : tile;
  g.cs = split_cols(N, dtype, k.coarsen_factor, ceil_div(span > 0 ? span : 1, E));
  g.slots = 1;
  g.team_threads = g.cs.lanes;
  g.teams_per_block = ceil_div(k.thread_per_block, g.cs.lanes);  // Mdim_thread_per_tb
  if (g.teams_per_block * g.cs.lanes > 1024) g.teams_per_block = 1024 / g.cs.lanes;
  g.block = g.teams_per_block * g.cs.lanes;
  long long rows_needed = ceil_div(M, g.teams_per_block);
  long long gx = ceil_div(workers_from_factor(M, k), g.teams_per_block);
  g.grid_x = clamp_grid(gx < rows_needed ? gx : rows_needed);
  return SS_OK;
}

// rbpr: csrspmm_parreduce_rowbalance_cg (spmm_cg.cuh:333-353).
static ss_status geom_rbpr(int M, int N, int dtype, const ss_knobs &k, RbGeom &g) {
  ss_status st = check_common_knobs(k);
  if (st) return st;
  if (k.tile_factor < 0 || k.tile_factor > 5)
    return fail(SS_ERR_UNSUPPORTED_KNOBS, "rbpr tile_factor %d outside [0, 5]", k.tile_factor);
  if (k.group_factor < 0 || k.group_factor > k.tile_factor)
    return fail(SS_ERR_UNSUPPORTED_KNOBS, "rbpr group_factor %d outside [0, tile_factor]", k.group_factor);
  const int tile = 1 << k.tile_factor;
  const int V = pick_vec(N, dtype, 16);
  const int span = N < tile ? N : tile;
  g.cs = split_cols(N, dtype, V, ceil_div(span > 0 ? span : 1, V));  // Ndim_warp_per_tb
  g.slots = tile;
  g.team_threads = tile * g.cs.lanes;
  if (g.team_threads > 1024)
    return fail(SS_ERR_UNSUPPORTED_KNOBS, "rbpr team of %d threads exceeds 1024", g.team_threads);
  int ref_warp_per_tb = k.thread_per_block / tile;
  if (ref_warp_per_tb < 1) ref_warp_per_tb = 1;
  g.teams_per_block = ceil_div(ref_warp_per_tb, g.cs.lanes);  // Mdim_warp_per_tb
  if (g.teams_per_block * g.team_threads > 1024) g.teams_per_block = 1024 / g.team_threads;
  g.block = g.teams_per_block * g.team_threads;
  long long rows_needed = ceil_div(M, g.teams_per_block);
  long long gx = ceil_div(workers_from_factor(M, k), g.teams_per_block);
  g.grid_x = clamp_grid(gx < rows_needed ? gx : rows_needed);
  return SS_OK;
}

static void finish_eb(long long worker_cap, EbGeom &g) {
  long long need = g.num_chunks > 0 ? ceil_div(g.num_chunks, g.workers_per_block) : 1;
  long long cap = ceil_div(worker_cap, g.workers_per_block);
  g.grid_x = clamp_grid(need < cap ? need : cap);
}

// ebsr: csrspmm_rowcaching_nnzbalance_cg (spmm_cg.cuh:553-566) and
// segment_coo_sr / _noshmem_sr / _noshmem_lessatom_sr (segscan.cuh:817-829).
ss_status geom_sr(long long worker_units, int nnz, int N, int dtype, int val_bytes, const ss_knobs &k,
                  EbGeom &g) {
  ss_status st = check_common_knobs(k);
  if (st) return st;
  if (k.group_factor < 0 || k.group_factor > 5)
    return fail(SS_ERR_UNSUPPORTED_KNOBS, "group_factor %d outside [0, 5]", k.group_factor);
  if (k.coarsen_factor < 1 || k.coarsen_factor > 8)
    return fail(SS_ERR_UNSUPPORTED_KNOBS, "CoarsenFactor %d outside [1, 8]", k.coarsen_factor);
  if (k.thread_nz < 1 || k.thread_nz > 4096)
    return fail(SS_ERR_UNSUPPORTED_KNOBS, "ThreadNz %d outside [1, 4096]", k.thread_nz);
  const int G = 1 << k.group_factor;
  if (k.thread_per_block > 512)
    return fail(SS_ERR_UNSUPPORTED_KNOBS, "sequential-walk blocks hold at most 512 threads (got %d)",
                k.thread_per_block);
  if (k.thread_per_block % G != 0)
    return fail(SS_ERR_UNSUPPORTED_KNOBS, "thread_per_block %d not a multiple of group size %d",
                k.thread_per_block, G);
  int coarsen = ceil_div(N > 0 ? N : 1, G);
  if (coarsen > k.coarsen_factor) coarsen = k.coarsen_factor;
  g.cs = split_cols(N, dtype, coarsen, G);
  g.team_lanes = G;
  g.team_threads = G;
  g.workers_per_block = k.thread_per_block / G;
  g.block = k.thread_per_block;
  g.chunk = k.thread_nz * G;
  // A group pays a chain of dependent loads to set up each chunk (first
  // row search, first staged tile, row window), so chunks much smaller than
  // the balanced share (nnz over the groups of one full wave on the
  // device's SMs at the walk's 1024 resident threads per SM) are merged up
  // to that share: small thread_nz tuples then run as fast as tuned ones.
  const long long wave_groups = (long long)sm_count() * 1024 / G;
  long long share = nnz > 0 ? ceil_div((long long)nnz, wave_groups) : 0;
  share = ceil_div(share, 32LL) * 32;  // a multiple of 8 keeps the bulk copies 16-byte aligned
  if (share > g.chunk && share <= (1LL << 30)) g.chunk = (int)share;
  g.num_chunks = nnz > 0 ? ceil_div(nnz, g.chunk) : 0;
  // staged tile: 64 nonzeros, smaller when the block's groups would need
  // more than 48 KB of shared memory (a multiple of 8 keeps bulk copies
  // 16-byte aligned)
  int stage = 64;
  while (stage > 8 && sr_smem_bytes(stage, g.workers_per_block, val_bytes) > 48 * 1024) stage >>= 1;
  g.stage = stage;
  g.smem = sr_smem_bytes(stage, g.workers_per_block, val_bytes);
  if (g.smem > 200 * 1024)
    return fail(SS_ERR_UNSUPPORTED_KNOBS, "%d groups per block need %zu B of shared memory",
                g.workers_per_block, g.smem);
  // reference grid: worker_units * block_factor blocks of thread_per_block
  finish_eb(workers_from_factor(worker_units, k) * g.workers_per_block, g);
  return SS_OK;
}

// ebpr: csrspmm_parreduce_nnzbalance_cg (spmm_cg.cuh:176-197) and
// segment_coo (segscan.cuh:150-171).
static ss_status geom_pr(long long worker_units, int nnz, int N, int dtype, const ss_knobs &k, EbGeom &g) {
  ss_status st = check_common_knobs(k);
  if (st) return st;
  if (k.tile_factor < 0 || k.tile_factor > 5)
    return fail(SS_ERR_UNSUPPORTED_KNOBS, "tile_factor %d outside [0, 5]", k.tile_factor);
  if (k.group_factor < 0 || k.group_factor > k.tile_factor)
    return fail(SS_ERR_UNSUPPORTED_KNOBS, "group_factor %d outside [0, tile_factor]", k.group_factor);
  const int tile = 1 << k.tile_factor;
  const int V = pick_vec(N, dtype, 16);
  const int span = N < tile ? N : tile;
  g.cs = split_cols(N, dtype, V, ceil_div(span > 0 ? span : 1, V));  // Ndim_warp_per_tb
  g.team_lanes = tile;
  g.team_threads = tile * g.cs.lanes;
  if (g.team_threads > 1024)
    return fail(SS_ERR_UNSUPPORTED_KNOBS, "worker of %d threads exceeds 1024", g.team_threads);
  int ref_warp_per_tb = k.thread_per_block / tile;
  if (ref_warp_per_tb < 1) ref_warp_per_tb = 1;
  g.workers_per_block = ceil_div(ref_warp_per_tb, g.cs.lanes);  // Nnzdim_warp_per_tb
  if (g.workers_per_block * g.team_threads > 1024) g.workers_per_block = 1024 / g.team_threads;
  g.block = g.workers_per_block * g.team_threads;
  long long gx_ref = ceil_div(workers_from_factor(worker_units, k), g.workers_per_block);
  long long workers = gx_ref * g.workers_per_block;
  long long steps_total = nnz > 0 ? ceil_div(nnz, tile) : 0;
  long long steps = workers > 0 ? (steps_total + workers - 1) / workers : 1;
  if (steps < 1) steps = 1;
  g.chunk = (int)(steps * tile);
  // chunks below the share of one full wave (1024 resident threads on each
  // of the device's SMs, shared by the column tiles) are merged up to it: each
  // chunk costs a chain of dependent loads to set up (cf. geom_sr)
  {
    long long blocks_per_sm = 1024 / g.block;
    if (blocks_per_sm < 1) blocks_per_sm = 1;
    long long wave = (long long)sm_count() * blocks_per_sm * g.workers_per_block / (g.cs.tiles > 0 ? g.cs.tiles : 1);
    if (wave < 1) wave = 1;
    long long share = nnz > 0 ? ceil_div((long long)nnz, wave) : 0;
    share = ceil_div(share, (long long)tile) * tile;
    if (share > g.chunk && share <= (1LL << 30)) g.chunk = (int)share;
  }
  g.num_chunks = nnz > 0 ? ceil_div(nnz, g.chunk) : 0;
  // per tile-lane set, a sliding shared-memory window of row starts, so the
  // row of each nonzero is searched on chip: up to chunk + 2 entries (a chunk
  // without empty rows fits), at most 256 + tile and 48 KB per block
  const long long sets = g.block / tile > 0 ? g.block / tile : 1;
  long long w = (long long)g.chunk + 2;
  if (w > 256 + tile) w = 256 + tile;
  const long long w_cap = (48LL * 1024 / 4) / sets;
  if (w > w_cap) w = w_cap;
  g.stage = w >= 4 ? (int)w : 0;
  g.smem = (size_t)sets * (size_t)g.stage * 4;
  finish_eb(workers, g);
  return SS_OK;
}

static ss_status check_csr(const ss_csr *A, int N) {
  if (!A) return fail(SS_ERR_INVALID_ARG, "A is null");
  if (A->nrow < 0 || A->ncol < 0 || A->nnz < 0 || N < 0)
    return fail(SS_ERR_INVALID_ARG, "negative size (nrow %d ncol %d nnz %d N %d)", A->nrow, A->ncol, A->nnz, N);
  if (A->nrow > 0 && !A->indptr) return fail(SS_ERR_INVALID_ARG, "indptr is null");
  if (A->nnz > 0 && !A->indices) return fail(SS_ERR_INVALID_ARG, "indices is null");
  if (A->value_dtype < SS_F32 || A->value_dtype > SS_F16)
    return fail(SS_ERR_INVALID_ARG, "value_dtype %d unknown", A->value_dtype);
  if ((long long)A->nrow * (long long)(N > 0 ? N : 1) > (1LL << 40))
    return fail(SS_ERR_INVALID_ARG, "output too large");
  return SS_OK;
}

// The caller's knobs, or the strategy's defaults; null (with the failure
// recorded) for an unknown strategy.
static const ss_knobs *knobs_or_default(int strategy, int N, const ss_knobs *k, ss_knobs &tmp) {
  if (k) return k;
  memset(&tmp, 0, sizeof(tmp));
  if (ss_default_knobs(strategy, N, &tmp) != SS_OK) return nullptr;
  return &tmp;
}

static ss_status make_spmm_call(int strategy, const ss_csr *A, int N, const void *B, void *C, int c_dtype,
                                int accumulate, const ss_knobs &k, SpmmCall &c) {
  ss_status st = check_csr(A, N);
  if (st) return st;
  if (A->nrow > 0 && N > 0 && !C) return fail(SS_ERR_INVALID_ARG, "C is null");
  if (A->nnz > 0 && N > 0 && !B) return fail(SS_ERR_INVALID_ARG, "B is null");
  // C is FP32 or the value type; ebsr with FP32 values also writes BF16/FP16
  // C directly (its stores round the FP32 sums)
  const bool c16_from_f32 = strategy == SS_EBSR && A->value_dtype == SS_F32 &&
                            (c_dtype == SS_BF16 || c_dtype == SS_F16);
  if (c_dtype != SS_F32 && c_dtype != A->value_dtype && !c16_from_f32)
    return fail(SS_ERR_INVALID_ARG, "c_dtype %d must be SS_F32 or the value dtype", c_dtype);
  if (accumulate != 0 && accumulate != 1) return fail(SS_ERR_INVALID_ARG, "accumulate must be 0 or 1");
  const int es = dtype_size(A->value_dtype);
  if (((uintptr_t)B % es) || ((uintptr_t)C % dtype_size(c_dtype)) || ((uintptr_t)A->values % es) ||
      ((uintptr_t)A->indices % 4) || ((uintptr_t)A->indptr % 4))
    return fail(SS_ERR_ALIGNMENT, "pointer not aligned to its element size");
  c.M = A->nrow; c.K = A->ncol; c.N = N; c.nnz = A->nnz;
  c.indptr = A->indptr; c.indices = A->indices; c.vals = A->values; c.val_dtype = A->value_dtype;
  c.B = B; c.C = C; c.c_dtype = c_dtype; c.accumulate = accumulate;
  c.kahan_threshold = k.kahan_threshold > 0 ? k.kahan_threshold : 1024;
  return SS_OK;
}

// Fewer than half as many nonzeros as output rows: at least half the rows
// are empty, and the element-balanced kernels would zero their runs one
// team per run.  Zeroing the output with a memset and accumulating is
// cheaper there; the sums are the same (0 + x = x).
static bool hypersparse(long long nnz, long long rows) { return 2 * nnz < rows; }

// Vector accesses need the B/C row starts aligned to V elements.
static ss_status check_vec_alignment(const void *B, const void *C, int es, int cs, int V) {
  if (((uintptr_t)B % (size_t)(es * V)) || ((uintptr_t)C % (size_t)(cs * V)))
    return fail(SS_ERR_ALIGNMENT, "B/C not aligned to the %d-element vector access", V);
  return SS_OK;
}

static ss_status spmm_geometry(int strategy, const SpmmCall &c, const ss_knobs &k, RbGeom &rg, EbGeom &eg) {
  switch (strategy) {
    case SS_RBSR: return geom_rbsr(c.M, c.N, c.val_dtype, k, rg);
    case SS_RBPR: return geom_rbpr(c.M, c.N, c.val_dtype, k, rg);
    case SS_EBSR: return geom_sr(c.M, c.nnz, c.N, c.val_dtype, dtype_size(c.val_dtype), k, eg);
    case SS_EBPR: return geom_pr(c.M, c.nnz, c.N, c.val_dtype, k, eg);
  }
  return fail(SS_ERR_INVALID_ARG, "unknown strategy %d", strategy);
}

}  // namespace ss

using namespace ss;

extern "C" {

int ss_version(void) { return SS_VERSION_MAJOR * 100 + SS_VERSION_MINOR; }

const char *ss_status_string(int status) {
  switch (status) {
    case SS_OK: return "ok";
    case SS_ERR_INVALID_ARG: return "invalid argument";
    case SS_ERR_UNSUPPORTED_KNOBS: return "unsupported knob tuple";
    case SS_ERR_WORKSPACE: return "workspace too small or misaligned";
    case SS_ERR_CUDA: return "CUDA runtime error";
    case SS_ERR_ALIGNMENT: return "misaligned pointer";
    case SS_ERR_BAD_DATA: return "malformed input data";
    case SS_ERR_TIMEOUT: return "device wait timed out";
    case SS_ERR_CAPACITY: return "size beyond fixed capacity";
  }
  return "unknown status";
}

const char *ss_last_error(void) { return g_last_error; }

ss_status ss_set_l2_keep_bytes(long long bytes) {
  if (bytes < 0) return fail(SS_ERR_INVALID_ARG, "negative L2 budget");
  g_keep_bytes.store(bytes, std::memory_order_relaxed);
  return SS_OK;
}

ss_status ss_default_knobs(int strategy, int N, ss_knobs *out) {
  if (!out) return fail(SS_ERR_INVALID_ARG, "out is null");
  ss_knobs k;
  memset(&k, 0, sizeof(k));
  k.thread_per_block = 256;
  k.block_numer = 1;
  k.block_denom = 1;
  k.coarsen_factor = 4;
  k.thread_nz = 1;
  k.kahan_threshold = 1024;
  switch (strategy) {
    case SS_EBPR:  // (5, 256, 5, 1, 8)  README.md:168-179
      k.group_factor = 5; k.tile_factor = 5; k.block_denom = 8;
      break;
    case SS_RBPR:  // (3, 256, 3, 1, 2)  README.md:185-196
      k.group_factor = 3; k.tile_factor = 3; k.block_denom = 2;
      break;
    case SS_EBSR:  // (4, 256, 4, 2, 1, 16) README.md:200-210
      k.group_factor = 4; k.coarsen_factor = 4; k.thread_nz = 2; k.block_denom = 16;
      break;
    case SS_RBSR:  // coarsen 4, tile 2^5 (test-cg/src/test.cu:59-82 sweeps these)
      k.coarsen_factor = 4; k.tile_factor = 5;
      break;
    default:
      return fail(SS_ERR_INVALID_ARG, "unknown strategy %d", strategy);
  }
  (void)N;
  *out = k;
  return SS_OK;
}

ss_status ss_spmm_workspace_size(int strategy, const ss_csr *A, int N, const ss_knobs *knobs, size_t *bytes) {
  if (!bytes) return fail(SS_ERR_INVALID_ARG, "bytes is null");
  ss_status st = check_csr(A, N);
  if (st) return st;
  ss_knobs tmp;
  const ss_knobs *k = knobs_or_default(strategy, N, knobs, tmp);
  if (!k) return SS_ERR_INVALID_ARG;
  SpmmCall c;
  c.M = A->nrow; c.K = A->ncol; c.N = N; c.nnz = A->nnz; c.val_dtype = A->value_dtype;
  RbGeom rg;
  EbGeom eg;
  st = spmm_geometry(strategy, c, *k, rg, eg);
  if (st) return st;
  *bytes = (strategy == SS_EBSR || strategy == SS_EBPR) ? eb_workspace_bytes(eg, N) : 0;
  return SS_OK;
}

ss_status ss_spmm(int strategy, const ss_csr *A, int N, const void *B, void *C, int c_dtype, int accumulate,
                  const ss_knobs *knobs, void *ws, size_t ws_bytes, void *stream) {
  ss::NvtxRange nvtx_range("ss_spmm");
  ss_knobs tmp;
  const ss_knobs *k = knobs_or_default(strategy, N, knobs, tmp);
  if (!k) return SS_ERR_INVALID_ARG;
  SpmmCall c;
  ss_status st = make_spmm_call(strategy, A, N, B, C, c_dtype, accumulate, *k, c);
  if (st) return st;
  RbGeom rg;
  EbGeom eg;
  st = spmm_geometry(strategy, c, *k, rg, eg);
  if (st) return st;
  cudaStream_t s = (cudaStream_t)stream;
  if (c.M == 0 || c.N == 0) return SS_OK;
  const bool eb = strategy == SS_EBSR || strategy == SS_EBPR;
  const ColSplit &cs = eb ? eg.cs : rg.cs;
  st = check_vec_alignment(B, C, dtype_size(c.val_dtype), dtype_size(c.c_dtype), cs.V);
  if (st) return st;
  if (eb) {
    if (c.nnz == 0) {
      if (accumulate) return SS_OK;
      cudaError_t e = cudaMemsetAsync(C, 0, (size_t)c.M * c.N * dtype_size(c.c_dtype), s);
      return e == cudaSuccess ? SS_OK : cuda_fail(e, "zero C");
    }
    const size_t need = eb_workspace_bytes(eg, N);
    if (ws_bytes < need || (need > 0 && (!ws || ((uintptr_t)ws % 256))))
      return fail(SS_ERR_WORKSPACE, "workspace needs %zu bytes (256-byte aligned), got %zu", need, ws_bytes);
    if (!accumulate && hypersparse(c.nnz, c.M)) {
      // at least half the rows are empty: zero C at copy bandwidth and add
      // into it, instead of chunks writing long runs of empty rows alone
      cudaError_t e = cudaMemsetAsync(C, 0, (size_t)c.M * c.N * dtype_size(c.c_dtype), s);
      if (e != cudaSuccess) return cuda_fail(e, "zero C");
      c.accumulate = 1;
    }
    return strategy == SS_EBSR ? launch_ebsr(c, eg, ws, s) : launch_ebpr(c, eg, ws, s);
  }
  return strategy == SS_RBSR ? launch_rbsr(c, rg, s) : launch_rbpr(c, rg, s);
}

ss_status ss_spmm_ebpr(const ss_csr *A, int N, const void *B, void *C, int c_dtype, int accumulate,
                       const ss_knobs *knobs, void *ws, size_t ws_bytes, void *stream) {
  return ss_spmm(SS_EBPR, A, N, B, C, c_dtype, accumulate, knobs, ws, ws_bytes, stream);
}
ss_status ss_spmm_rbpr(const ss_csr *A, int N, const void *B, void *C, int c_dtype, int accumulate,
                       const ss_knobs *knobs, void *ws, size_t ws_bytes, void *stream) {
  return ss_spmm(SS_RBPR, A, N, B, C, c_dtype, accumulate, knobs, ws, ws_bytes, stream);
}
ss_status ss_spmm_ebsr(const ss_csr *A, int N, const void *B, void *C, int c_dtype, int accumulate,
                       const ss_knobs *knobs, void *ws, size_t ws_bytes, void *stream) {
  return ss_spmm(SS_EBSR, A, N, B, C, c_dtype, accumulate, knobs, ws, ws_bytes, stream);
}
ss_status ss_spmm_rbsr(const ss_csr *A, int N, const void *B, void *C, int c_dtype, int accumulate,
                       const ss_knobs *knobs, void *ws, size_t ws_bytes, void *stream) {
  return ss_spmm(SS_RBSR, A, N, B, C, c_dtype, accumulate, knobs, ws, ws_bytes, stream);
}

// ---------------------------------------------------------------------
// segment_coo
// ---------------------------------------------------------------------
static ss_status seg_geometry(int seg_strategy, int nnz, int N, int dtype, const ss_knobs &k, EbGeom &g) {
  if (seg_strategy == SS_SEG_SR) return geom_sr(nnz, nnz, N, dtype, 0, k, g);
  if (seg_strategy == SS_SEG_PR) return geom_pr(nnz, nnz, N, dtype, k, g);
  return fail(SS_ERR_INVALID_ARG, "unknown segment strategy %d", seg_strategy);
}

static void seg_default_knobs(int seg_strategy, ss_knobs &k) {
  memset(&k, 0, sizeof(k));
  k.thread_per_block = 256;
  k.block_numer = 1;
  k.block_denom = 1;
  k.kahan_threshold = 1024;
  if (seg_strategy == SS_SEG_SR) {  // segment_coo_sr<4,256,4,1,1,16> (new-cg/src/main.cu:52)
    k.group_factor = 4; k.coarsen_factor = 4; k.thread_nz = 8; k.block_denom = 16;
  } else {                          // segment_coo<5,256,5,1,16> (new-cg/src/main.cu:50)
    k.group_factor = 5; k.tile_factor = 5; k.block_denom = 16; k.coarsen_factor = 4; k.thread_nz = 1;
  }
}

ss_status ss_segment_coo_workspace_size(int seg_strategy, int nnz, int N, const ss_knobs *knobs, size_t *bytes) {
  if (!bytes) return fail(SS_ERR_INVALID_ARG, "bytes is null");
  if (nnz < 0 || N < 0) return fail(SS_ERR_INVALID_ARG, "negative size");
  ss_knobs tmp;
  if (!knobs) { seg_default_knobs(seg_strategy, tmp); knobs = &tmp; }
  // the query has no source dtype: the chunking depends on it (16-bit
  // sources take wider vectors, so more, smaller chunks), so return the
  // largest need over the three
  size_t most = 0;
  for (int dt : {SS_F32, SS_BF16, SS_F16}) {
    EbGeom g;
    ss_status st = seg_geometry(seg_strategy, nnz, N, dt, *knobs, g);
    if (st) return st;
    const size_t need = seg_strategy == SS_SEG_SR ? seg_sr_workspace_bytes(g, N) : eb_workspace_bytes(g, N);
    if (need > most) most = need;
  }
  *bytes = most;
  return SS_OK;
}

ss_status ss_segment_coo(int seg_strategy, const void *src, int src_dtype, const int32_t *index, int nnz, int N,
                         int dst_len, float *dst, int reduce, int accumulate, const ss_knobs *knobs, void *ws,
                         size_t ws_bytes, void *stream) {
  ss::NvtxRange nvtx_range("ss_segment_coo");
  if (nnz < 0 || N < 0 || dst_len < 0) return fail(SS_ERR_INVALID_ARG, "negative size");
  if (src_dtype < SS_F32 || src_dtype > SS_F16) return fail(SS_ERR_INVALID_ARG, "src_dtype %d unknown", src_dtype);
  if (reduce < SS_SUM || reduce > SS_MEAN) return fail(SS_ERR_INVALID_ARG, "reduce %d unknown", reduce);
  if (accumulate != 0 && accumulate != 1) return fail(SS_ERR_INVALID_ARG, "accumulate must be 0 or 1");
  if (accumulate && reduce != SS_SUM) return fail(SS_ERR_INVALID_ARG, "accumulate is defined for SS_SUM only");
  if (nnz > 0 && N > 0 && (!src || !index)) return fail(SS_ERR_INVALID_ARG, "src/index is null");
  if (dst_len > 0 && N > 0 && !dst) return fail(SS_ERR_INVALID_ARG, "dst is null");
  ss_knobs tmp;
  if (!knobs) { seg_default_knobs(seg_strategy, tmp); knobs = &tmp; }
  EbGeom g;
  ss_status st = seg_geometry(seg_strategy, nnz, N, src_dtype, *knobs, g);
  if (st) return st;
  cudaStream_t s = (cudaStream_t)stream;
  if (dst_len == 0 || N == 0) return SS_OK;
  st = check_vec_alignment(src, dst, dtype_size(src_dtype), 4, g.cs.V);
  if (st) return st;
  if (nnz == 0) {
    if (accumulate) return SS_OK;
    cudaError_t e = cudaMemsetAsync(dst, 0, (size_t)dst_len * N * sizeof(float), s);
    return e == cudaSuccess ? SS_OK : cuda_fail(e, "zero dst");
  }
  const size_t need = seg_strategy == SS_SEG_SR ? seg_sr_workspace_bytes(g, N) : eb_workspace_bytes(g, N);
  if (ws_bytes < need || !ws || ((uintptr_t)ws % 256))
    return fail(SS_ERR_WORKSPACE, "workspace needs %zu bytes (256-byte aligned), got %zu", need, ws_bytes);
  SegCall c;
  c.nnz = nnz; c.N = N; c.dst_len = dst_len; c.src = src; c.src_dtype = src_dtype; c.index = index;
  c.dst = dst; c.reduce = reduce; c.accumulate = accumulate;
  if (!accumulate && reduce == SS_SUM && hypersparse(nnz, dst_len)) {
    cudaError_t e = cudaMemsetAsync(dst, 0, (size_t)dst_len * N * sizeof(float), s);
    if (e != cudaSuccess) return cuda_fail(e, "zero dst");
    c.accumulate = 1;
  }
  c.kahan_threshold = knobs->kahan_threshold > 0 ? knobs->kahan_threshold : 1024;
  return seg_strategy == SS_SEG_SR ? launch_seg_sr(c, g, ws, s) : launch_seg_pr(c, g, ws, s);
}

}  // extern "C"
