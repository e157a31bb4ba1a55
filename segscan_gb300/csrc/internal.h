// Host-side interface between the C ABI layer (abi.cu) and the kernel
// translation units.  Not installed; not part of the public ABI.
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include <nvtx3/nvToolsExt.h>

#include "../../include/segscan_gb300.h"

namespace ss {

// NVTX range around one library call (shows the entry point on a profiler
// timeline; a no-op unless a tool is attached).
struct NvtxRange {
  explicit NvtxRange(const char *name) { nvtxRangePushA(name); }
  ~NvtxRange() { nvtxRangePop(); }
  NvtxRange(const NvtxRange &) = delete;
  NvtxRange &operator=(const NvtxRange &) = delete;
};

// Records a failure message for ss_last_error() and returns `st`.
ss_status fail(ss_status st, const char *fmt, ...);
ss_status cuda_fail(cudaError_t err, const char *what);

// One SpMM problem after argument checks.
struct SpmmCall {
  int M, K, N, nnz;
  const int32_t *indptr, *indices;
  const void *vals;  // may be null (all ones)
  int val_dtype;     // ss_dtype of vals and B
  const void *B;
  void *C;
  int c_dtype;       // SS_F32 or val_dtype
  int accumulate;
  int kahan_threshold;
};

// One segment_coo problem after argument checks.
struct SegCall {
  int nnz, N, dst_len;
  const void *src;
  int src_dtype;
  const int32_t *index;
  float *dst;
  int reduce;  // ss_reduce
  int accumulate;
  int kahan_threshold;
};

// Column decomposition shared by every kernel: each lane owns E = V * NV
// consecutive elements of a row of B / C, loaded as NV vectors of V.
struct ColSplit {
  int V;         // elements per vector access (power of two, divides N)
  int NV;        // vectors per lane (1 or 2)
  int lanes;     // lanes covering one column tile (power of two <= 32)
  int col_tile;  // lanes * V * NV columns per blockIdx.y
  int tiles;     // gridDim.y
};

// Row-balanced launch (rbsr, rbpr).
struct RbGeom {
  ColSplit cs;
  int slots;          // lanes along a row's nonzeros (rbpr tile_size; 1 for rbsr)
  int team_threads;   // slots * cs.lanes
  int teams_per_block;
  int block;          // threads per block
  int grid_x;
};

// Element-balanced launch (ebpr, ebsr and both segment families).
struct EbGeom {
  ColSplit cs;
  int team_lanes;        // lanes per worker along nonzeros (pr) or along N (sr)
  int team_threads;      // threads per worker including column groups
  int workers_per_block;
  int block;             // threads per block
  int chunk;             // nonzeros per worker chunk
  int num_chunks;
  int grid_x;
  int stage;             // sr: elements staged in shared memory at a time
  size_t smem;           // dynamic shared memory per block
};

size_t eb_workspace_bytes(const EbGeom &g, int N);
// segment SR: the element-balanced workspace plus the straddling segments'
// element counts (2 ints per chunk, after eb_workspace_bytes)
size_t seg_sr_workspace_bytes(const EbGeom &g, int N);
// Sequential-walk geometry from knobs (abi.cu): worker_units scales
// block_factor (nrow for SpMM, nnz for segments); val_bytes 0 for segments.
ss_status geom_sr(long long worker_units, int nnz, int N, int dtype, int val_bytes, const ss_knobs &k, EbGeom &g);
// shared memory of the sequential-walk kernels (eb_walk.cu)
size_t sr_smem_bytes(int stage, int workers_per_block, int val_bytes);
// ebsr with one lane per group (eb_narrow.cu): the kernel for these value /
// output types and vector shape, or null
void *narrow_kernel(int val_dtype, int c_dtype, int V, int NV);
// device address of the bounded-wait status word (eb_walk.cu)
int *walk_error_ptr();
// streaming multiprocessors of the current device, looked up once per device
// (util.cu); 1 when the query fails
int sm_count();
// L2 size of the current device in bytes (cached per device).
long long l2_bytes();

// Launchers (kernels live in spmm_rb.cu, eb_walk.cu, eb_scan.cu).
ss_status launch_rbsr(const SpmmCall &c, const RbGeom &g, cudaStream_t s);
ss_status launch_rbpr(const SpmmCall &c, const RbGeom &g, cudaStream_t s);
ss_status launch_ebsr(const SpmmCall &c, const EbGeom &g, void *ws, cudaStream_t s);
ss_status launch_ebpr(const SpmmCall &c, const EbGeom &g, void *ws, cudaStream_t s);
ss_status launch_seg_sr(const SegCall &c, const EbGeom &g, void *ws, cudaStream_t s);
ss_status launch_seg_pr(const SegCall &c, const EbGeom &g, void *ws, cudaStream_t s);

// Carry fix-up shared by the element-balanced kernels (eb_common.cu).
struct CarryView {
  int32_t *rows;   // [num_chunks], -1 = no head row (fix-up kernel path);
                   // the same region is [num_chunks * tiles] arrival counts
                   // for the walks that assemble straddling rows in-kernel
  float *vals;     // [num_chunks * N] head-row partials
  float *tails;    // [num_chunks * N] partials of rows continuing past a chunk
};
CarryView carry_view(void *ws, int num_chunks, int N, int tiles);
size_t carry_rows_bytes(int num_chunks, int tiles);
ss_status launch_fixup(const CarryView &cv, int num_chunks, int N, int M, void *C, int c_dtype,
                       int reduce, int accumulate, const int32_t *index, int nnz, cudaStream_t s);

// Fraction of a gathered operand of `bytes` to mark evict_last: all of it
// when it fits the L2 budget, else the budget's share (abi.cu).
float l2_keep_fraction(size_t bytes);

inline int ceil_div(long long a, long long b) { return (int)((a + b - 1) / b); }
inline int floor_pow2(int x) {
  int p = 1;
  while (p * 2 <= x) p *= 2;
  return p;
}
inline int ceil_pow2(int x) {
  int p = 1;
  while (p < x) p *= 2;
  return p;
}
inline int ilog2(int x) {
  int l = 0;
  while ((1 << l) < x) l++;
  return l;
}
inline int dtype_size(int dt) { return dt == SS_F32 ? 4 : 2; }

}  // namespace ss
