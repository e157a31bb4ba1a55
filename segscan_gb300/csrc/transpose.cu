// Device CSR transpose (the backward pass's A^T) and value gather.
//
// Reference semantics: transpose + compressedRow
// (test-cg/include/dataloader/dataloader.hpp:109-144), a stable counting
// sort by column: entries of one column keep A's CSR order.  The device
// version gives the same result bit for bit:
//   1. column histogram (atomics)            -> counts
//   2. exclusive scan of counts (3 kernels; 5 when K > 4096^2, the tile
//      sums then scanned in two levels)      -> t_indptr
//   3. scatter nonzero ids by column (atomic cursors; order inside a column
//      is arbitrary here)                    -> perm
//   4. sort each column's ids ascending      -> the stable order
//      (thread insertion sort <= 32 entries, block bitonic sort in shared
//      memory <= 16384, block bitonic sort in global memory beyond)
//   5. t_indices[q] = row of perm[q]
// Every step is deterministic given the input, so repeated calls agree.
#include <algorithm>

#include "common.cuh"
#include "internal.h"

namespace ss {

constexpr int SCAN_TILE = 4096;  // elements per scan block (1024 threads x 4)
constexpr int SMEM_SORT_MAX = 16384;

struct TransposeWs {
  int32_t *counts;    // [K + 1]
  int32_t *cursor;    // [K]
  int32_t *bsum;      // [tiles]: per-tile sums, then (one level) their exclusive scan
  int32_t *bsum_scan; // [tiles]: the exclusive scan of bsum (two levels)
  int32_t *bsum2;     // [SCAN_TILE]: sums of bsum's tiles (two levels)
  int32_t *rowid;     // [nnz]
  int32_t *work;      // [1 + K]: count, then column ids with > 32 entries
};

static size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

static long long scan_tiles(long long n) { return (n + SCAN_TILE - 1) / SCAN_TILE; }

static size_t transpose_ws_bytes(int K, int nnz, TransposeWs *w, void *base) {
  const size_t tiles = (size_t)std::max(1LL, scan_tiles(K));
  size_t o = 0;
  const size_t counts = o; o += align256((size_t)(K + 1) * 4);
  const size_t cursor = o; o += align256((size_t)K * 4);
  const size_t bsum = o; o += align256(tiles * 4);
  const size_t bsum_scan = o; o += align256(tiles * 4);
  const size_t bsum2 = o; o += align256((size_t)SCAN_TILE * 4);
  const size_t rowid = o; o += align256((size_t)nnz * 4);
  const size_t work = o; o += align256((size_t)(K + 1) * 4);
  if (w) {
    char *b = (char *)base;
    w->counts = (int32_t *)(b + counts);
    w->cursor = (int32_t *)(b + cursor);
    w->bsum = (int32_t *)(b + bsum);
    w->bsum_scan = (int32_t *)(b + bsum_scan);
    w->bsum2 = (int32_t *)(b + bsum2);
    w->rowid = (int32_t *)(b + rowid);
    w->work = (int32_t *)(b + work);
  }
  return o;
}

static int grid_for(long long n, int threads) {
  long long b = (n + threads - 1) / threads;
  if (b > (long long)sm_count() * 32) b = (long long)sm_count() * 32;
  return b < 1 ? 1 : (int)b;
}

__global__ void hist_kernel(const int32_t *__restrict__ cols, int nnz, int K, int32_t *counts) {
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < nnz; p += (long long)gridDim.x * blockDim.x) {
    const int c = cols[p];
    if ((unsigned)c < (unsigned)K) atomicAdd(counts + c, 1);
  }
}

// Block-wide exclusive scan of SCAN_TILE ints: out = exclusive prefix, and
// the tile total to bsum[blockIdx.x].
__global__ void __launch_bounds__(1024) scan_tile_kernel(const int32_t *__restrict__ in, int n, int32_t *out,
                                                         int32_t *bsum) {
  __shared__ int32_t warp_tot[32];
  const int base = blockIdx.x * SCAN_TILE + threadIdx.x * 4;
  int v[4];
  #pragma unroll
  for (int i = 0; i < 4; i++) v[i] = base + i < n ? in[base + i] : 0;
  int t = v[0] + v[1] + v[2] + v[3];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  int incl = t;
  #pragma unroll
  for (int off = 1; off < 32; off <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, incl, off);
    if (lane >= off) incl += y;
  }
  if (lane == 31) warp_tot[wid] = incl;
  __syncthreads();
  if (wid == 0) {
    int w = lane < (int)(blockDim.x >> 5) ? warp_tot[lane] : 0;
    int wi = w;
    #pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, wi, off);
      if (lane >= off) wi += y;
    }
    warp_tot[lane] = wi - w;  // exclusive prefix of warp totals
    if (lane == 31) bsum[blockIdx.x] = wi;
  }
  __syncthreads();
  int run = warp_tot[wid] + incl - t;
  #pragma unroll
  for (int i = 0; i < 4; i++) {
    if (base + i < n) out[base + i] = run;
    run += v[i];
  }
}

// out[i] += prefix of bsum before i's tile; bsum is scanned in place by
// block 0 first (at most SCAN_TILE tiles).
__global__ void __launch_bounds__(1024) scan_bsum_kernel(int32_t *bsum, int nb, int32_t *total) {
  __shared__ int32_t warp_tot[32];
  const int base = threadIdx.x * 4;
  int v[4];
  #pragma unroll
  for (int i = 0; i < 4; i++) v[i] = base + i < nb ? bsum[base + i] : 0;
  const int t = v[0] + v[1] + v[2] + v[3];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  int incl = t;
  #pragma unroll
  for (int off = 1; off < 32; off <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, incl, off);
    if (lane >= off) incl += y;
  }
  if (lane == 31) warp_tot[wid] = incl;
  __syncthreads();
  if (wid == 0) {
    int w = warp_tot[lane];
    int wi = w;
    #pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, wi, off);
      if (lane >= off) wi += y;
    }
    warp_tot[lane] = wi - w;
    if (lane == 31) *total = wi;
  }
  __syncthreads();
  int run = warp_tot[wid] + incl - t;
  #pragma unroll
  for (int i = 0; i < 4; i++) {
    if (base + i < nb) bsum[base + i] = run;
    run += v[i];
  }
}

__global__ void scan_add_kernel(int32_t *out, int n, const int32_t *__restrict__ bsum) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    out[i] += bsum[i / SCAN_TILE];
}

__global__ void scatter_kernel(const int32_t *__restrict__ cols, int nnz, int K, int32_t *cursor, int32_t *perm) {
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < nnz; p += (long long)gridDim.x * blockDim.x) {
    const int c = cols[p];
    if ((unsigned)c < (unsigned)K) {
      const int q = atomicAdd(cursor + c, 1);
      perm[q] = (int32_t)p;
    }
  }
}

// Thread per column: insertion sort of short columns, queue the rest.
__global__ void sort_small_kernel(const int32_t *__restrict__ t_indptr, int K, int32_t *perm, int32_t *work) {
  for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < K; c += (long long)gridDim.x * blockDim.x) {
    const int s = t_indptr[c], e = t_indptr[c + 1];
    const int n = e - s;
    if (n <= 1) continue;
    if (n > 32) {
      const int slot = atomicAdd(work, 1);
      work[1 + slot] = (int32_t)c;
      continue;
    }
    int32_t *a = perm + s;
    for (int i = 1; i < n; i++) {
      const int32_t x = a[i];
      int j = i - 1;
      while (j >= 0 && a[j] > x) {
        a[j + 1] = a[j];
        j--;
      }
      a[j + 1] = x;
    }
  }
}

// Ascending bitonic sort of n keys at `a` (shared or global), padded to
// the next power of two with virtual +inf keys.  The first step of every
// merge stage compares mirrored positions, so all comparisons put the
// smaller key at the lower index and a padded (+inf) partner never moves.
__device__ __forceinline__ void bitonic_block(int32_t *a, int n) {
  int P = 1;
  while (P < n) P <<= 1;
  for (int k = 2; k <= P; k <<= 1) {
    for (int j = k >> 1; j > 0; j >>= 1) {
      for (int i = threadIdx.x; i < P; i += blockDim.x) {
        const int partner = (j == (k >> 1)) ? (i ^ (k - 1)) : (i ^ j);
        if (partner > i && partner < n) {
          const int32_t x = a[i], y = a[partner];
          if (x > y) {
            a[i] = y;
            a[partner] = x;
          }
        }
      }
      __syncthreads();
    }
  }
}

__global__ void __launch_bounds__(1024) sort_large_kernel(const int32_t *__restrict__ t_indptr, int32_t *perm,
                                                          const int32_t *__restrict__ work) {
  extern __shared__ int32_t keys[];
  const int count = work[0];
  for (int w = blockIdx.x; w < count; w += gridDim.x) {
    const int c = work[1 + w];
    const int s = t_indptr[c], n = t_indptr[c + 1] - s;
    if (n <= SMEM_SORT_MAX) {
      for (int i = threadIdx.x; i < n; i += blockDim.x) keys[i] = perm[s + i];
      __syncthreads();
      bitonic_block(keys, n);
      for (int i = threadIdx.x; i < n; i += blockDim.x) perm[s + i] = keys[i];
      __syncthreads();
    } else {
      bitonic_block(perm + s, n);  // in global memory; rare
      __syncthreads();
    }
  }
}

// rowid[p] = row of nonzero p (binary_search_segment_number semantics).
// A thread takes ROWID_RUN consecutive nonzeros: one row search for the
// first, then it walks indptr forward (rows only grow along p).
constexpr int ROWID_RUN = 16;
__global__ void rowid_kernel(const int32_t *__restrict__ indptr, int M, int nnz, int32_t *rowid) {
  const long long runs = ((long long)nnz + ROWID_RUN - 1) / ROWID_RUN;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < runs; t += (long long)gridDim.x * blockDim.x) {
    const int p0 = (int)(t * ROWID_RUN);
    const int p1 = min(p0 + ROWID_RUN, nnz);
    int r = row_search(indptr, 1, M, p0);
    int next = __ldg(indptr + min(r + 1, M));
    for (int p = p0; p < p1; p++) {
      while (p >= next && r < M - 1) {
        r++;
        next = __ldg(indptr + r + 1);
      }
      rowid[p] = r;
    }
  }
}

__global__ void gather_rows_kernel(const int32_t *__restrict__ perm, const int32_t *__restrict__ rowid, int nnz,
                                   int32_t *t_indices) {
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < nnz; q += (long long)gridDim.x * blockDim.x) {
    // entries past t_indptr[K] exist only when A has out-of-range columns
    const int p = perm[q];
    t_indices[q] = (unsigned)p < (unsigned)nnz ? rowid[p] : -1;
  }
}

// Steps 1-4: a stable counting sort of the positions [0, nnz) by key
// (keys outside [0, K) are left out): out_indptr [K + 1] gets each key's
// start, perm the positions grouped by key, ascending within a key.
static ss_status counting_sort(const int32_t *keys, int nnz, int K, int32_t *out_indptr, int32_t *perm,
                               const TransposeWs &w, cudaStream_t s) {
  const long long tiles = scan_tiles(K);
  cudaError_t e = cudaMemsetAsync(w.counts, 0, (size_t)(K + 1) * 4, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(w.work, 0, 4, s);
  if (e != cudaSuccess) return cuda_fail(e, "counting sort clear");
  if (K == 0) {  // no keys: out_indptr = [0]
    e = cudaMemsetAsync(out_indptr, 0, 4, s);
    return e == cudaSuccess ? SS_OK : cuda_fail(e, "counting sort clear");
  }
  if (nnz > 0) hist_kernel<<<grid_for(nnz, 256), 256, 0, s>>>(keys, nnz, K, w.counts);
  scan_tile_kernel<<<(int)tiles, 1024, 0, s>>>(w.counts, K, out_indptr, w.bsum);
  if (tiles <= SCAN_TILE) {
    scan_bsum_kernel<<<1, 1024, 0, s>>>(w.bsum, (int)tiles, out_indptr + K);
    scan_add_kernel<<<grid_for(K, 256), 256, 0, s>>>(out_indptr, K, w.bsum);
  } else {
    // the tile sums are themselves more than one tile: scan them the same
    // way (at most 4096 second-level tiles for any int32 K)
    const long long tiles2 = scan_tiles(tiles);
    scan_tile_kernel<<<(int)tiles2, 1024, 0, s>>>(w.bsum, (int)tiles, w.bsum_scan, w.bsum2);
    scan_bsum_kernel<<<1, 1024, 0, s>>>(w.bsum2, (int)tiles2, out_indptr + K);
    scan_add_kernel<<<grid_for(tiles, 256), 256, 0, s>>>(w.bsum_scan, (int)tiles, w.bsum2);
    scan_add_kernel<<<grid_for(K, 256), 256, 0, s>>>(out_indptr, K, w.bsum_scan);
  }
  e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "counting sort scan");
  if (nnz == 0) return SS_OK;
  e = cudaMemcpyAsync(w.cursor, out_indptr, (size_t)K * 4, cudaMemcpyDeviceToDevice, s);
  if (e != cudaSuccess) return cuda_fail(e, "counting sort cursor");
  scatter_kernel<<<grid_for(nnz, 256), 256, 0, s>>>(keys, nnz, K, w.cursor, perm);
  sort_small_kernel<<<grid_for(K, 256), 256, 0, s>>>(out_indptr, K, perm, w.work);
  e = cudaFuncSetAttribute(sort_large_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_SORT_MAX * 4);
  if (e != cudaSuccess) return cuda_fail(e, "counting sort attribute");
  sort_large_kernel<<<2 * sm_count(), 1024, SMEM_SORT_MAX * 4, s>>>(out_indptr, perm, w.work);
  e = cudaGetLastError();
  return e == cudaSuccess ? SS_OK : cuda_fail(e, "counting sort launch");
}

}  // namespace ss

using namespace ss;

extern "C" {

ss_status ss_csr_transpose_workspace_size(const ss_csr *A, size_t *bytes) {
  if (!A || !bytes || A->nrow < 0 || A->ncol < 0 || A->nnz < 0) return fail(SS_ERR_INVALID_ARG, "bad arguments");
  *bytes = transpose_ws_bytes(A->ncol, A->nnz, nullptr, nullptr);
  return SS_OK;
}

ss_status ss_csr_transpose(const ss_csr *A, int32_t *t_indptr, int32_t *t_indices, int32_t *perm, void *ws,
                           size_t ws_bytes, void *stream) {
  ss::NvtxRange nvtx_range("ss_csr_transpose");
  if (!A || A->nrow < 0 || A->ncol < 0 || A->nnz < 0) return fail(SS_ERR_INVALID_ARG, "bad CSR descriptor");
  const int M = A->nrow, K = A->ncol, nnz = A->nnz;
  if (!t_indptr || (nnz > 0 && (!t_indices || !perm || !A->indices || !A->indptr)))
    return fail(SS_ERR_INVALID_ARG, "null pointer");
  const size_t need = transpose_ws_bytes(K, nnz, nullptr, nullptr);
  if (ws_bytes < need || !ws || ((uintptr_t)ws % 256))
    return fail(SS_ERR_WORKSPACE, "workspace needs %zu bytes (256-byte aligned), got %zu", need, ws_bytes);
  TransposeWs w;
  transpose_ws_bytes(K, nnz, &w, ws);
  cudaStream_t s = (cudaStream_t)stream;
  ss_status st = counting_sort(A->indices, nnz, K, t_indptr, perm, w, s);
  if (st != SS_OK || nnz == 0 || K == 0) return st;
  rowid_kernel<<<grid_for((nnz + ROWID_RUN - 1) / ROWID_RUN, 256), 256, 0, s>>>(A->indptr, M, nnz, w.rowid);
  gather_rows_kernel<<<grid_for(nnz, 256), 256, 0, s>>>(perm, w.rowid, nnz, t_indices);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? SS_OK : cuda_fail(e, "transpose launch");
}

ss_status ss_coo_to_csr_workspace_size(int nrow, int nnz, size_t *bytes) {
  if (!bytes || nrow < 0 || nnz < 0) return fail(SS_ERR_INVALID_ARG, "bad arguments");
  *bytes = transpose_ws_bytes(nrow, nnz, nullptr, nullptr);
  return SS_OK;
}

ss_status ss_coo_to_csr(int nrow, int nnz, const int32_t *rows, const int32_t *cols, int32_t *indptr,
                        int32_t *out_cols, int32_t *perm, void *ws, size_t ws_bytes, void *stream) {
  ss::NvtxRange nvtx_range("ss_coo_to_csr");
  if (nrow < 0 || nnz < 0 || !indptr || (nnz > 0 && (!rows || !cols || !out_cols || !perm)))
    return fail(SS_ERR_INVALID_ARG, "bad arguments");
  const size_t need = transpose_ws_bytes(nrow, nnz, nullptr, nullptr);
  if (ws_bytes < need || !ws || ((uintptr_t)ws % 256))
    return fail(SS_ERR_WORKSPACE, "workspace needs %zu bytes (256-byte aligned), got %zu", need, ws_bytes);
  TransposeWs w;
  transpose_ws_bytes(nrow, nnz, &w, ws);
  cudaStream_t s = (cudaStream_t)stream;
  ss_status st = counting_sort(rows, nnz, nrow, indptr, perm, w, s);
  if (st != SS_OK || nnz == 0 || nrow == 0) return st;
  gather_rows_kernel<<<grid_for(nnz, 256), 256, 0, s>>>(perm, cols, nnz, out_cols);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? SS_OK : cuda_fail(e, "coo to csr launch");
}

}  // extern "C"
