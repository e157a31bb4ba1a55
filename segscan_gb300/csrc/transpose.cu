// Device CSR transpose (the backward pass's A^T), value gather and COO ->
// CSR.
//
// Reference semantics: transpose + compressedRow
// (test-cg/include/dataloader/dataloader.hpp:109-144), a stable counting
// sort by column: entries of one column keep A's CSR order.  The device
// versions give the same result bit for bit, as a sort of the nonzero
// positions p by column with p ascending inside a column.
//
// ss_csr_transpose: two-level bucket sort.  A bucket is F = 2^f consecutive
// columns, F chosen so that an average bucket fills at most half of one
// block's shared-memory record store.
//   1. bucket_count_kernel: per-block shared-memory histogram of col >> f,
//      one global add per bucket per block;
//   2. bucket_scan_kernel (one block): bucket starts, cursors, t_indptr[K];
//   3. bucket_partition_kernel: a tile of TB_E nonzeros finds the row of
//      each nonzero (the rows starting inside the tile are marked in shared
//      memory and a block max-scan spreads them), reserves one range per
//      bucket it touches, groups its (position, row, column) records by
//      bucket in shared memory and writes each group as one contiguous run;
//   4. bucket_sort_kernel: a block per bucket counts its columns in shared
//      memory (writing t_indptr), places the records by column and sorts
//      each column by position (insertion sort up to 32 entries, bitonic
//      beyond), then writes perm, t_indices and, optionally, the gathered
//      values.  Rows grow with positions, so a column's rows sorted on their
//      own equal the rows of its sorted positions.  A bucket larger than the
//      record store is placed and sorted in the output arrays instead.
// Order inside a column before step 4's sort depends on atomics; after it,
// only on the input, so repeated calls agree.
//
// ss_coo_to_csr (and ss_csr_transpose beyond TB_NB_MAX buckets of 8192
// columns): a one-level counting sort,
//   1. key histogram (atomics)               -> counts
//   2. exclusive scan of counts (3 kernels; 5 when K > 4096^2, the tile
//      sums then scanned in two levels)      -> t_indptr
//   3. scatter positions by key (atomic cursors)
//   4. sort each key's positions ascending (thread insertion sort <= 32
//      entries, block bitonic sort in shared memory <= 16384, in global
//      memory beyond)
//   5. for the transpose: t_indices[q] = row of perm[q].
#include <algorithm>
#include <climits>

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

// ---------------------------------------------------------------------
// Two-level bucket transpose (ss_csr_transpose)
// ---------------------------------------------------------------------
constexpr int TB_T = 1024;            // threads per block (count, scan)
#ifndef SS_TB_PT
#define SS_TB_PT 1024
#endif
#ifndef SS_TB_PER
#define SS_TB_PER 8
#endif
#ifndef SS_TB_PART_BLOCKS
#define SS_TB_PART_BLOCKS 1
#endif
constexpr int TB_PT = SS_TB_PT;                    // threads per block (partition)
constexpr int TB_PER = SS_TB_PER;                  // nonzeros per thread in a partition tile
constexpr int TB_PART_BLOCKS = SS_TB_PART_BLOCKS;  // partition blocks resident per SM
constexpr int TB_E = TB_PT * TB_PER;  // nonzeros per partition tile
#ifndef SS_TB_ST
#define SS_TB_ST 1024
#endif
#ifndef SS_TB_SORT_BLOCKS
#define SS_TB_SORT_BLOCKS 1
#endif
constexpr int TB_ST = SS_TB_ST;                  // threads per block (bucket sort)
constexpr int TB_SORT_BLOCKS = SS_TB_SORT_BLOCKS;  // bucket-sort blocks resident per SM
constexpr int TB_F_LOG2_MAX = 13;  // at most 8192 columns per bucket
constexpr int TB_NB_MAX = 8192;    // buckets
#ifndef SS_TB_SORT_SMEM_KB
#define SS_TB_SORT_SMEM_KB 220
#endif
constexpr int TB_SORT_SMEM = SS_TB_SORT_SMEM_KB * 1024;
constexpr int TB_LONG = 40;  // slot of the long-column count in the sort block's scratch

struct BucketPlan {
  bool ok;             // false: more than TB_NB_MAX buckets of 8192 columns
  int f, F, NB, cap;   // F = 2^f columns per bucket; cap = records a sort block holds
};

// Records a sort block holds (a multiple of 4): each takes five ints (the
// three staged record arrays, the two placed ones) beside the mbarrier (4
// ints), eight ints of alignment slack per staged array, 2F + 1 counters and
// 64 ints of scratch.
static int sort_bytes(int F, int cap) { return (4 + 3 * (cap + 8) + 2 * cap + 2 * F + 1 + 64) * 4; }
static int sort_cap(int F) { return ((TB_SORT_SMEM - sort_bytes(F, 0)) / 20) & ~3; }

static BucketPlan bucket_plan(int K, int nnz) {
  BucketPlan p;
  const double avg = K > 0 ? (double)nnz / K : 0.0;
  int f = TB_F_LOG2_MAX;
  while (f > 0 && (double)(1 << f) * avg > sort_cap(1 << f) / 2) f--;
  long long nb = ((long long)K + (1LL << f) - 1) >> f;
  while (nb > TB_NB_MAX && f < TB_F_LOG2_MAX) {
    f++;
    nb = ((long long)K + (1LL << f) - 1) >> f;
  }
  p.ok = nb <= TB_NB_MAX;
  p.f = f;
  p.F = 1 << f;
  p.NB = (int)nb;
  p.cap = sort_cap(p.F);
  return p;
}

struct BucketWs {
  int32_t *count;   // [NB]: nonzeros per bucket
  int32_t *start;   // [NB + 1]: bucket starts
  int32_t *cursor;  // [NB]: partition cursors
  int32_t *pos, *row, *col;  // [nnz] records, grouped by bucket
};

static size_t bucket_ws_bytes(const BucketPlan &p, int nnz, BucketWs *w, void *base) {
  size_t o = 0;
  const size_t count = o; o += align256((size_t)(p.NB + 1) * 4);
  const size_t start = o; o += align256((size_t)(p.NB + 1) * 4);
  const size_t cursor = o; o += align256((size_t)(p.NB + 1) * 4);
  // four spare entries each: a sort block reads whole 16-byte words
  const size_t pos = o; o += align256((size_t)(nnz + 4) * 4);
  const size_t row = o; o += align256((size_t)(nnz + 4) * 4);
  const size_t col = o; o += align256((size_t)(nnz + 4) * 4);
  if (w) {
    char *b = (char *)base;
    w->count = (int32_t *)(b + count);
    w->start = (int32_t *)(b + start);
    w->cursor = (int32_t *)(b + cursor);
    w->pos = (int32_t *)(b + pos);
    w->row = (int32_t *)(b + row);
    w->col = (int32_t *)(b + col);
  }
  return o;
}

// Scan of x[0, n) in place by the whole block: exclusive prefix sums (MAX
// false) or inclusive prefix maxima (MAX true).  Each warp owns a contiguous
// segment and scans it 32 consecutive entries at a time with shuffles (no
// shared-memory bank conflicts), then the warps' totals are scanned and
// applied.  Returns the sum / the maximum to every thread.  wbuf: 33 ints of
// shared memory.  Callers synchronise the block before the call: the scan
// writes x[] from its first step, and a warp's segment is not the range its
// own threads filled or read.
template <bool MAX>
__device__ int block_scan(int32_t *x, int n, int32_t *wbuf) {
  constexpr int ID = MAX ? INT_MIN : 0;
  auto op = [](int u, int v) { return MAX ? max(u, v) : u + v; };
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5, W = blockDim.x >> 5;
  const int seg = ((n + W - 1) / W + 31) & ~31;  // entries per warp, a multiple of 32
  const int lo = min(wid * seg, n), hi = min(lo + seg, n);
  int carry = ID;
  for (int base = lo; base < hi; base += 32) {
    const int i = base + lane;
    const int v0 = i < hi ? x[i] : ID;
    int v = v0;
    #pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, v, off);
      if (lane >= off) v = op(v, y);
    }
    v = op(carry, v);  // inclusive within the warp's segment
    if (i < hi) x[i] = MAX ? v : v - v0;
    carry = __shfl_sync(0xffffffffu, v, 31);
  }
  if (lane == 0) wbuf[wid] = carry;
  __syncthreads();
  if (wid == 0) {
    const int w = lane < W ? wbuf[lane] : ID;
    int wi = w;
    #pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, wi, off);
      if (lane >= off) wi = op(wi, y);
    }
    int we = __shfl_up_sync(0xffffffffu, wi, 1);
    if (lane == 0) we = ID;
    wbuf[lane] = we;  // what the warps before each one contribute
    if (lane == 31) wbuf[32] = wi;
  }
  __syncthreads();
  const int pre = wbuf[wid];
  if (wid > 0)
    for (int i = lo + lane; i < hi; i += 32) x[i] = op(pre, x[i]);
  const int total = wbuf[32];
  __syncthreads();
  return total;
}

// Largest r in [0, M) with indptr[r] <= key (indptr[0] = 0 <= key): the 32
// lanes of a warp probe 32 split points of the open range per round.
__device__ int warp_row_of(const int32_t *__restrict__ indptr, int M, int key, int lane) {
  int lo = 0, hi = M - 1;  // indptr[lo] <= key; the answer lies in [lo, hi]
  while (lo < hi) {
    const int probe = lo + 1 + (int)(((long long)(hi - lo) * lane) >> 5);  // in (lo, hi]
    const bool ok = __ldg(indptr + probe) <= key;
    const unsigned hits = __ballot_sync(0xffffffffu, ok);
    if (!hits) {
      hi = lo;
      break;
    }
    const int last = 31 - __clz(hits);  // probes are ordered, so hits are a prefix
    const int nlo = __shfl_sync(0xffffffffu, probe, last);
    const int nxt = __shfl_sync(0xffffffffu, probe, last < 31 ? last + 1 : 31);
    hi = last < 31 ? nxt - 1 : hi;
    lo = nlo;
  }
  return lo;
}

__global__ void __launch_bounds__(TB_T) bucket_count_kernel(const int32_t *__restrict__ cols, int nnz, int K, int f,
                                                            int NB, int32_t *count) {
  extern __shared__ int32_t hist[];
  for (int i = threadIdx.x; i < NB; i += TB_T) hist[i] = 0;
  __syncthreads();
  const long long step = (long long)gridDim.x * TB_T * 4;
  for (long long b = (long long)blockIdx.x * TB_T * 4 + threadIdx.x; b < nnz; b += step) {
    int c[4];
    #pragma unroll
    for (int u = 0; u < 4; u++) c[u] = b + u * TB_T < nnz ? __ldg(cols + b + u * TB_T) : -1;
    #pragma unroll
    for (int u = 0; u < 4; u++)
      if ((unsigned)c[u] < (unsigned)K) atomicAdd(hist + (c[u] >> f), 1);
  }
  __syncthreads();
  for (int i = threadIdx.x; i < NB; i += TB_T) {
    const int h = hist[i];
    if (h) atomicAdd(count + i, h);
  }
}

// Bucket starts and partition cursors; t_indptr[K] = nonzeros with a column
// in [0, K); the entries past it (nonzeros with other columns) get -1.
__global__ void __launch_bounds__(TB_T) bucket_scan_kernel(const int32_t *__restrict__ count, int NB, int nnz, int K,
                                                           int32_t *start, int32_t *cursor, int32_t *t_indptr,
                                                           int32_t *perm, int32_t *t_indices) {
  __shared__ int32_t x[TB_NB_MAX];
  __shared__ int32_t wbuf[33];
  for (int i = threadIdx.x; i < NB; i += TB_T) x[i] = count[i];
  __syncthreads();
  const int total = block_scan<false>(x, NB, wbuf);
  for (int i = threadIdx.x; i < NB; i += TB_T) {
    start[i] = x[i];
    cursor[i] = x[i];
  }
  if (threadIdx.x == 0) {
    start[NB] = total;
    t_indptr[K] = total;
  }
  for (int q = total + threadIdx.x; q < nnz; q += TB_T) {
    perm[q] = -1;
    t_indices[q] = -1;
  }
}

struct PartArgs {
  const int32_t *indptr, *cols;
  int M, K, nnz, f, NB;
  int32_t *cursor, *pos, *row, *col;
};

// One tile of TB_E nonzeros per round: the row of each nonzero, then the
// tile's (position, row, column) records grouped by bucket in shared memory
// (a counting sort of the tile) and written out as one contiguous run per
// bucket into the range the tile reserved there, so that consecutive
// threads store consecutive addresses.
__global__ void __launch_bounds__(TB_PT, TB_PART_BLOCKS) bucket_partition_kernel(PartArgs a) {
  extern __shared__ int32_t sm[];
  int32_t *lst = sm;               // [NB + 1]: the tile's count per bucket, then its start in the tile
  int32_t *cur = lst + a.NB + 1;   // [NB]: placement cursors
  int32_t *base = cur + a.NB;      // [NB]: the tile's range in each bucket
  int32_t *rows = base + a.NB;     // [TB_E]: rows (marks, running maximum); then the staged rows
  int32_t *s_pos = rows + TB_E;    // [TB_E]: staged positions
  int32_t *s_col = s_pos + TB_E;   // [TB_E]: staged columns
  __shared__ int32_t wbuf[33];
  __shared__ int32_t r01[2];
  const int tid = threadIdx.x;
  for (long long t = blockIdx.x; t * TB_E < a.nnz; t += gridDim.x) {
    const int b0 = (int)(t * TB_E);
    const int n = (int)min((long long)TB_E, (long long)a.nnz - b0);
    if (tid < 64) {  // warp 0: the row holding b0; warp 1: the row holding the tile's last nonzero
      const int r = warp_row_of(a.indptr, a.M, tid < 32 ? b0 : b0 + n - 1, tid & 31);
      if ((tid & 31) == 0) r01[tid >> 5] = r;
    }
    for (int i = tid; i < a.NB; i += TB_PT) lst[i] = 0;
    int c[TB_PER], rr[TB_PER];
    #pragma unroll
    for (int k = 0; k < TB_PER; k++) {
      const int e = tid + k * TB_PT;
      c[k] = e < n ? __ldg(a.cols + b0 + e) : -1;
    }
    __syncthreads();
    const int r0 = r01[0], r1 = r01[1];
    if ((long long)(r1 - r0) <= 4LL * TB_E) {
      // mark each row's first nonzero (the last of the rows that start
      // there: rows before it are empty), then a running maximum
      for (int e = tid; e < TB_E; e += TB_PT) rows[e] = e == 0 ? r0 : -1;
      __syncthreads();
      for (int r = r0 + 1 + tid; r <= r1; r += TB_PT) {
        const int e = __ldg(a.indptr + r) - b0;
        if ((unsigned)e < (unsigned)TB_E) atomicMax(rows + e, r);
      }
      __syncthreads();
      block_scan<true>(rows, n, wbuf);
      #pragma unroll
      for (int k = 0; k < TB_PER; k++) {
        const int e = tid + k * TB_PT;
        rr[k] = e < n ? rows[e] : -1;
      }
    } else {
      // long runs of empty rows: a binary search in [r0, r1] per nonzero
      #pragma unroll
      for (int k = 0; k < TB_PER; k++) {
        const int e = tid + k * TB_PT;
        int lo = r0, hi = r1;
        while (lo < hi) {
          const int mid = lo + ((hi - lo + 1) >> 1);
          if (__ldg(a.indptr + mid) <= b0 + e) lo = mid; else hi = mid - 1;
        }
        rr[k] = lo;
      }
    }
    #pragma unroll
    for (int k = 0; k < TB_PER; k++)
      if ((unsigned)c[k] < (unsigned)a.K) atomicAdd(lst + (c[k] >> a.f), 1);
    __syncthreads();  // counts complete; rows read into registers
    // the tile's range in each bucket it touches
    for (int i = tid; i < a.NB; i += TB_PT) {
      const int h = lst[i];
      base[i] = h ? atomicAdd(a.cursor + i, h) : 0;
    }
    // every count is read before the scan overwrites them: with more buckets
    // than threads a thread reads counts that another warp scans
    __syncthreads();
    const int valid = block_scan<false>(lst, a.NB, wbuf);  // lst: each bucket's start in the tile
    for (int i = tid; i < a.NB; i += TB_PT) cur[i] = lst[i];
    if (tid == 0) lst[a.NB] = valid;
    __syncthreads();
    #pragma unroll
    for (int k = 0; k < TB_PER; k++) {
      if ((unsigned)c[k] < (unsigned)a.K) {
        const int q = atomicAdd(cur + (c[k] >> a.f), 1);
        s_pos[q] = b0 + tid + k * TB_PT;
        rows[q] = rr[k];
        s_col[q] = c[k];
      }
    }
    __syncthreads();
    for (int i = tid; i < valid; i += TB_PT) {
      const int col = s_col[i];
      const int bk = col >> a.f;
      const int q = base[bk] + (i - lst[bk]);
      a.pos[q] = s_pos[i];
      a.row[q] = rows[i];
      a.col[q] = col;
    }
    __syncthreads();  // the next tile reuses the shared arrays
  }
}

// Sorts n keys ascending, the values moved along (n small).
__device__ __forceinline__ void insertion_sort2(int32_t *k, int32_t *v, int n) {
  for (int i = 1; i < n; i++) {
    const int32_t x = k[i], y = v[i];
    int j = i - 1;
    while (j >= 0 && k[j] > x) {
      k[j + 1] = k[j];
      v[j + 1] = v[j];
      j--;
    }
    k[j + 1] = x;
    v[j + 1] = y;
  }
}

// Sorts n <= 8 keys ascending in registers by a fixed network of 19
// compare-exchanges (Batcher's odd-even merge sort for eight inputs), the
// entries past n padded with INT_MAX.  The values are sorted by the same
// network on their own: a column's rows grow with its positions, so the
// sorted rows are the rows of the sorted positions.  All eight loads are
// independent, so a column costs one shared-memory round trip instead of a
// chain of them.
__device__ __forceinline__ void sort8(int32_t *k, int32_t *v, int n) {
  int32_t a[8], b[8];
  #pragma unroll
  for (int j = 0; j < 8; j++) {
    a[j] = j < n ? k[j] : INT_MAX;
    b[j] = j < n ? v[j] : INT_MAX;
  }
  constexpr int NET[19][2] = {{0, 1}, {2, 3}, {4, 5}, {6, 7}, {0, 2}, {1, 3}, {4, 6}, {5, 7}, {1, 2}, {5, 6},
                              {0, 4}, {1, 5}, {2, 6}, {3, 7}, {2, 4}, {3, 5}, {1, 2}, {3, 4}, {5, 6}};
  #pragma unroll
  for (int c = 0; c < 19; c++) {
    const int x = NET[c][0], y = NET[c][1];
    const int32_t alo = min(a[x], a[y]), ahi = max(a[x], a[y]);
    const int32_t blo = min(b[x], b[y]), bhi = max(b[x], b[y]);
    a[x] = alo; a[y] = ahi;
    b[x] = blo; b[y] = bhi;
  }
  #pragma unroll
  for (int j = 0; j < 8; j++)
    if (j < n) {
      k[j] = a[j];
      v[j] = b[j];
    }
}

// Block sort of n keys in global memory: staged through shared memory when
// they fit.
__device__ void sort_segment(int32_t *seg, int n, int32_t *stage, int cap) {
  if (n <= cap) {
    for (int i = threadIdx.x; i < n; i += blockDim.x) stage[i] = seg[i];
    __syncthreads();
    bitonic_block(stage, n);
    for (int i = threadIdx.x; i < n; i += blockDim.x) seg[i] = stage[i];
  } else {
    bitonic_block(seg, n);
  }
  __syncthreads();
}

struct SortArgs {
  const int32_t *start, *pos, *row, *col;
  int K, NB, f, F, cap;
  int32_t *t_indptr, *perm, *t_indices;
  const void *vals;  // A's values, or null: no value gather
  void *t_vals;
  int vsize;         // 4 or 2 bytes
  int *err;          // device status word for the bounded waits
};

constexpr uint32_t TB_SPIN_LIMIT = 1u << 22;  // mbarrier polls before giving up

// Sorts each of a bucket's columns (cnt: column starts, cnt[nf] the end)
// shorter than 33 entries by position, one thread per column, the rows
// moved along: up to eight entries in registers (sort8), more by insertion.
// Longer columns are listed in longs (count at *nlong) for the block to
// sort.  kp / vp are shared or global; the call site fixes which.
__device__ __forceinline__ void sort_short_columns(int32_t *kp, int32_t *vp, const int32_t *cnt, int32_t *longs,
                                                   int32_t *nlong, int nf) {
  for (int i = threadIdx.x; i < nf; i += blockDim.x) {
    const int s = cnt[i], len = cnt[i + 1] - s;
    if (len > 32) longs[atomicAdd(nlong, 1)] = i;
    else if (len > 8) insertion_sort2(kp + s, vp + s, len);
    else if (len > 1) sort8(kp + s, vp + s, len);
  }
}

// t_vals[s0 + i] = vals[src[i]] for the bucket's n entries, eight gathers
// in flight per thread; src is shared or global, the call site fixes which.
__device__ __forceinline__ void gather_bucket_values(const SortArgs &a, const int32_t *src, int s0, int n) {
  for (int i0 = 0; i0 < n; i0 += 8 * blockDim.x) {
    uint32_t v[8];
    #pragma unroll
    for (int u = 0; u < 8; u++) {
      const int i = i0 + threadIdx.x + u * blockDim.x;
      const int p = i < n ? src[i] : 0;
      v[u] = a.vsize == 4 ? __ldg((const uint32_t *)a.vals + p) : __ldg((const unsigned short *)a.vals + p);
    }
    #pragma unroll
    for (int u = 0; u < 8; u++) {
      const int i = i0 + threadIdx.x + u * blockDim.x;
      if (i >= n) break;
      if (a.vsize == 4) ((uint32_t *)a.t_vals)[s0 + i] = v[u];
      else ((uint16_t *)a.t_vals)[s0 + i] = (uint16_t)v[u];
    }
  }
}

// The records of bucket b into the staging arrays: one bulk copy per array
// from the 16-byte word holding its first record to the one holding its
// last, completing on bar.  Returns the offset of the first record in the
// staged arrays (0..3).  Thread 0 only.
__device__ __forceinline__ int stage_bucket(const SortArgs &a, int b, int32_t *rc, int32_t *rp, int32_t *rr,
                                            uint64_t *bar) {
  const int s0 = __ldg(a.start + b), n = __ldg(a.start + b + 1) - s0;
  const int w0 = s0 & ~3, w1 = (s0 + n + 3) & ~3;
  const uint32_t bytes = (uint32_t)(w1 - w0) * 4u;
  fence_async_smem();
  mbar_expect_tx(bar, 3u * bytes);
  bulk_g2s(rc, a.col + w0, bytes, bar);
  bulk_g2s(rp, a.pos + w0, bytes, bar);
  bulk_g2s(rr, a.row + w0, bytes, bar);
  return s0 - w0;
}

// A bucket per round, one block per SM.  A bucket that fits the record store
// arrives by bulk copies (the next one's issued as soon as this one's
// records are placed, so it lands while this one is sorted and written); its
// columns are counted, its records placed by column and sorted inside each
// column, all in shared memory.  A larger bucket is placed and sorted in
// the output arrays.
__global__ void __launch_bounds__(TB_ST, TB_SORT_BLOCKS) bucket_sort_kernel(SortArgs a) {
  extern __shared__ __align__(16) int32_t sm[];
  uint64_t *bar = reinterpret_cast<uint64_t *>(sm);  // [4 ints]
  const int stg = a.cap + 8;          // staged array length (alignment slack; a multiple of 4)
  int32_t *rc = sm + 4;               // [stg] staged columns
  int32_t *rp = rc + stg;             // [stg] staged positions
  int32_t *rr = rp + stg;             // [stg] staged rows
  int32_t *sp = rr + stg;             // [cap] placed positions
  int32_t *sr = sp + a.cap;           // [cap] placed rows
  int32_t *cnt = sr + a.cap;          // [F + 1]: counts, then column starts
  int32_t *cur = cnt + a.F + 1;       // [F]: placement cursors, then the long columns
  int32_t *wbuf = cur + a.F;          // [64]: scan scratch; [TB_LONG]: long-column count; [48]: staged offset
  const int tid = threadIdx.x;
  uint32_t phase = 0;
  // bucket b arrives by bulk copies: not empty, and it fits the record store
  auto fits_at = [&](int b) {
    if (b >= a.NB) return false;
    const int n = __ldg(a.start + b + 1) - __ldg(a.start + b);
    return n > 0 && n <= a.cap;
  };
  auto wait_staged = [&]() -> bool {
    for (uint32_t it = 0; it < TB_SPIN_LIMIT; it++)
      if (mbar_try_wait(bar, phase)) return true;
    return false;
  };
  if (tid == 0) {
    mbar_init(bar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    if (fits_at(blockIdx.x)) wbuf[48] = stage_bucket(a, blockIdx.x, rc, rp, rr, bar);
  }
  __syncthreads();
  for (int b = blockIdx.x; b < a.NB; b += gridDim.x) {
    const int c0 = b << a.f;
    const int nf = min(a.F, a.K - c0);
    const int s0 = __ldg(a.start + b), n = __ldg(a.start + b + 1) - s0;
    const bool fits = n <= a.cap;
    const bool staged = n > 0 && fits;
    for (int i = tid; i < nf; i += TB_ST) cnt[i] = 0;
    if (tid == 0) wbuf[TB_LONG] = 0;
    int d = 0;  // first staged record
    if (staged) {
      if (!__syncthreads_and(wait_staged())) {
        // the copies did not land: record it, wait (bounded) once more for
        // them, and stop; no other copy of this block is in flight
        if (tid == 0 && a.err) atomicExch(a.err, (int)SS_ERR_TIMEOUT);
        wait_staged();
        return;
      }
      phase ^= 1u;
      d = wbuf[48];
    } else {
      __syncthreads();
    }
    // count the bucket's columns
    if (fits) {
      #pragma unroll 4
      for (int i = tid; i < n; i += TB_ST) {
        const int c = rc[d + i] - c0;
        if ((unsigned)c < (unsigned)nf) atomicAdd(cnt + c, 1);
      }
    } else {
      for (int i0 = 0; i0 < n; i0 += 4 * TB_ST) {
        int c[4];
        #pragma unroll
        for (int u = 0; u < 4; u++) {
          const int i = i0 + tid + u * TB_ST;
          c[u] = i < n ? __ldg(a.col + s0 + i) - c0 : -1;
        }
        #pragma unroll
        for (int u = 0; u < 4; u++)
          if ((unsigned)c[u] < (unsigned)nf) atomicAdd(cnt + c[u], 1);
      }
    }
    __syncthreads();
    const int total = block_scan<false>(cnt, nf, wbuf);
    for (int i = tid; i < nf; i += TB_ST) {
      a.t_indptr[c0 + i] = s0 + cnt[i];
      cur[i] = cnt[i];
    }
    if (tid == 0) cnt[nf] = total;
    __syncthreads();
    // The shared-memory and the global-memory paths are written apart, so
    // every access has a known address space: through a pointer that may be
    // either, shared accesses become generic ones that queue with the global
    // loads and stores.
    if (fits) {
      for (int i = tid; i < n; i += TB_ST) {
        const int c = rc[d + i] - c0;
        if ((unsigned)c < (unsigned)nf) {
          const int q = atomicAdd(cur + c, 1);
          sp[q] = rp[d + i];
          sr[q] = rr[d + i];
        }
      }
      __syncthreads();
      // the staged arrays are free: the next bucket of this block streams in
      if (tid == 0 && fits_at(b + gridDim.x)) wbuf[48] = stage_bucket(a, b + gridDim.x, rc, rp, rr, bar);
    } else {
      for (int i0 = 0; i0 < n; i0 += 4 * TB_ST) {
        int c[4], p[4], r[4];
        #pragma unroll
        for (int u = 0; u < 4; u++) {
          const int i = i0 + tid + u * TB_ST;
          c[u] = i < n ? __ldg(a.col + s0 + i) - c0 : -1;
          p[u] = i < n ? __ldg(a.pos + s0 + i) : 0;
          r[u] = i < n ? __ldg(a.row + s0 + i) : 0;
        }
        #pragma unroll
        for (int u = 0; u < 4; u++) {
          if ((unsigned)c[u] < (unsigned)nf) {
            const int q = atomicAdd(cur + c[u], 1);
            a.perm[s0 + q] = p[u];
            a.t_indices[s0 + q] = r[u];
          }
        }
      }
      __syncthreads();
      // this bucket used no staging; the next one, if it fits, is staged now
      if (tid == 0 && fits_at(b + gridDim.x)) wbuf[48] = stage_bucket(a, b + gridDim.x, rc, rp, rr, bar);
    }
    // each column by position: short ones by a thread, long ones by the block
    if (fits) sort_short_columns(sp, sr, cnt, cur, wbuf + TB_LONG, nf);
    else sort_short_columns(a.perm + s0, a.t_indices + s0, cnt, cur, wbuf + TB_LONG, nf);
    __syncthreads();
    const int nl = wbuf[TB_LONG];
    for (int l = 0; l < nl; l++) {
      const int i = cur[l];
      const int s = cnt[i], len = cnt[i + 1] - s;
      if (fits) {
        bitonic_block(sp + s, len);
        bitonic_block(sr + s, len);
      } else {
        sort_segment(a.perm + s0 + s, len, sp, 2 * a.cap);
        sort_segment(a.t_indices + s0 + s, len, sp, 2 * a.cap);
      }
    }
    if (fits) {
      for (int i = tid; i < n; i += TB_ST) {
        a.perm[s0 + i] = sp[i];
        a.t_indices[s0 + i] = sr[i];
      }
    }
    if (a.t_vals) {  // the values, eight gathers in flight per thread
      if (fits) gather_bucket_values(a, sp, s0, n);
      else gather_bucket_values(a, a.perm + s0, s0, n);
    }
    __syncthreads();  // the next bucket reuses the shared memory
  }
}

static ss_status bucket_transpose(const ss_csr *A, const BucketPlan &pl, int32_t *t_indptr, int32_t *t_indices,
                                  int32_t *perm, void *t_vals, const BucketWs &w, cudaStream_t s) {
  const int M = A->nrow, K = A->ncol, nnz = A->nnz;
  const int sms = sm_count();
  cudaError_t e = cudaMemsetAsync(w.count, 0, (size_t)pl.NB * 4, s);
  if (e != cudaSuccess) return cuda_fail(e, "transpose clear");
  const size_t hist_smem = (size_t)pl.NB * 4;
  const size_t part_smem = (size_t)(3 * pl.NB + 1 + 3 * TB_E) * 4;
  const size_t sort_smem = (size_t)sort_bytes(pl.F, pl.cap);
  e = cudaFuncSetAttribute(bucket_count_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)hist_smem);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(bucket_partition_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)part_smem);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(bucket_sort_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sort_smem);
  if (e != cudaSuccess) return cuda_fail(e, "transpose attributes");
  const long long tiles = ((long long)nnz + TB_E - 1) / TB_E;
  const int count_blocks = (int)std::min<long long>(((long long)nnz + 4 * TB_T - 1) / (4 * TB_T), 2LL * sms);
  bucket_count_kernel<<<count_blocks, TB_T, hist_smem, s>>>(A->indices, nnz, K, pl.f, pl.NB, w.count);
  bucket_scan_kernel<<<1, TB_T, 0, s>>>(w.count, pl.NB, nnz, K, w.start, w.cursor, t_indptr, perm, t_indices);
  PartArgs pa;
  pa.indptr = A->indptr; pa.cols = A->indices;
  pa.M = M; pa.K = K; pa.nnz = nnz; pa.f = pl.f; pa.NB = pl.NB;
  pa.cursor = w.cursor; pa.pos = w.pos; pa.row = w.row; pa.col = w.col;
  bucket_partition_kernel<<<(int)std::min<long long>(tiles, (long long)sms * TB_PART_BLOCKS), TB_PT, part_smem, s>>>(pa);
  SortArgs sa;
  sa.start = w.start; sa.pos = w.pos; sa.row = w.row; sa.col = w.col;
  sa.K = K; sa.NB = pl.NB; sa.f = pl.f; sa.F = pl.F; sa.cap = pl.cap;
  sa.t_indptr = t_indptr; sa.perm = perm; sa.t_indices = t_indices;
  sa.vals = t_vals ? A->values : nullptr;
  sa.t_vals = t_vals;
  sa.vsize = dtype_size(A->value_dtype);
  sa.err = walk_error_ptr();
  bucket_sort_kernel<<<std::min(pl.NB, sms * TB_SORT_BLOCKS), TB_ST, sort_smem, s>>>(sa);
  e = cudaGetLastError();
  return e == cudaSuccess ? SS_OK : cuda_fail(e, "transpose launch");
}

}  // namespace ss

using namespace ss;

extern "C" {

ss_status ss_csr_transpose_workspace_size(const ss_csr *A, size_t *bytes) {
  if (!A || !bytes || A->nrow < 0 || A->ncol < 0 || A->nnz < 0) return fail(SS_ERR_INVALID_ARG, "bad arguments");
  const BucketPlan pl = bucket_plan(A->ncol, A->nnz);
  *bytes = pl.ok ? bucket_ws_bytes(pl, A->nnz, nullptr, nullptr) : transpose_ws_bytes(A->ncol, A->nnz, nullptr, nullptr);
  return SS_OK;
}

ss_status ss_csr_transpose_values(const ss_csr *A, int32_t *t_indptr, int32_t *t_indices, int32_t *perm,
                                  void *t_values, void *ws, size_t ws_bytes, void *stream) {
  ss::NvtxRange nvtx_range("ss_csr_transpose");
  if (!A || A->nrow < 0 || A->ncol < 0 || A->nnz < 0) return fail(SS_ERR_INVALID_ARG, "bad CSR descriptor");
  const int M = A->nrow, K = A->ncol, nnz = A->nnz;
  if (!t_indptr || (nnz > 0 && (!t_indices || !perm || !A->indices || !A->indptr)))
    return fail(SS_ERR_INVALID_ARG, "null pointer");
  if (t_values && nnz > 0 && !A->values) return fail(SS_ERR_INVALID_ARG, "t_values given but A has no values");
  if (t_values && (A->value_dtype < SS_F32 || A->value_dtype > SS_F16))
    return fail(SS_ERR_INVALID_ARG, "value_dtype %d unknown", A->value_dtype);
  const BucketPlan pl = bucket_plan(K, nnz);
  const size_t need = pl.ok ? bucket_ws_bytes(pl, nnz, nullptr, nullptr) : transpose_ws_bytes(K, nnz, nullptr, nullptr);
  if (ws_bytes < need || !ws || ((uintptr_t)ws % 256))
    return fail(SS_ERR_WORKSPACE, "workspace needs %zu bytes (256-byte aligned), got %zu", need, ws_bytes);
  cudaStream_t s = (cudaStream_t)stream;
  if (nnz == 0 || K == 0) {  // no entries: t_indptr = zeros; nonzeros with no valid column get -1
    cudaError_t e = cudaMemsetAsync(t_indptr, 0, (size_t)(K + 1) * 4, s);
    if (e == cudaSuccess && nnz > 0) e = cudaMemsetAsync(perm, 0xff, (size_t)nnz * 4, s);
    if (e == cudaSuccess && nnz > 0) e = cudaMemsetAsync(t_indices, 0xff, (size_t)nnz * 4, s);
    return e == cudaSuccess ? SS_OK : cuda_fail(e, "transpose clear");
  }
  if (pl.ok) {
    BucketWs w;
    bucket_ws_bytes(pl, nnz, &w, ws);
    return bucket_transpose(A, pl, t_indptr, t_indices, perm, t_values, w, s);
  }
  TransposeWs w;
  transpose_ws_bytes(K, nnz, &w, ws);
  ss_status st = counting_sort(A->indices, nnz, K, t_indptr, perm, w, s);
  if (st != SS_OK) return st;
  rowid_kernel<<<grid_for((nnz + ROWID_RUN - 1) / ROWID_RUN, 256), 256, 0, s>>>(A->indptr, M, nnz, w.rowid);
  gather_rows_kernel<<<grid_for(nnz, 256), 256, 0, s>>>(perm, w.rowid, nnz, t_indices);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "transpose launch");
  return t_values ? ss_gather_values(A->values, A->value_dtype, perm, nnz, t_values, stream) : SS_OK;
}

ss_status ss_csr_transpose(const ss_csr *A, int32_t *t_indptr, int32_t *t_indices, int32_t *perm, void *ws,
                           size_t ws_bytes, void *stream) {
  return ss_csr_transpose_values(A, t_indptr, t_indices, perm, nullptr, ws, ws_bytes, stream);
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
