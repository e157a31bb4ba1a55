// Element-balanced machinery shared by the sequential (ebsr, segment SR) and
// parallel (ebpr, segment PR) kernels.
//
// Work is cut into chunks of consecutive nonzeros.  A row is OWNED by the
// chunk that holds its first nonzero; the owner writes the row with plain
// stores when the row also ends in that chunk.  Only two rows of a chunk can
// straddle a chunk boundary: the HEAD row (started in an earlier chunk) and
// the last row (continues into the next chunk).  Their FP32 partials go to
// the chunk's head and tail slots, and each straddling row is assembled
// once as owner tail + following heads (by the last of its chunks to finish,
// carry_arrive / seg_carry_arrive, in the ebsr, segment SR and batched
// walks; by the fix-up kernel, fixup_chunk, after the ebpr and segment PR
// kernels) and stored once, so a
// 16-bit output is rounded once.  Empty rows (empty
// segments) are written as zero by the chunk holding the next nonzero, so in
// overwrite mode every output row is written exactly once, no zero fill and
// no atomics are needed, and the result is deterministic.  This replaces the
// reference's per-segment atomicAdd into a pre-zeroed C
// (test-cg/include/spmm/spmm_cg.cuh:80,104,466,474; new-cg/include/segscan/
// segscan.cuh:58,77,452,459).
#pragma once
#include <climits>

#include "common.cuh"

namespace ss {

struct EbArgs {
  int M;  // rows of C (SpMM) or dst_len (segment)
  int K, N, nnz;
  const int32_t *indptr;  // SpMM: A's row pointer
  const int32_t *cols;    // SpMM: A's column indices
  const int32_t *index;   // segment: sorted segment ids
  const void *vals;       // SpMM: A's values (null = ones)
  const void *B;          // SpMM: B; segment: src
  void *C;
  int accumulate, reduce, kahan;
  int team_lanes, log2_team_lanes;
  int colgroups, log2_colgroups;  // pr kernels: column groups per worker
  int col_tile;
  int chunk, num_chunks, workers_per_block, stage;
  int use_tma;          // sr kernels: stage the streams with bulk copies
  int *err;             // device status word for bounded waits (may be null)
  float keep_frac;      // fraction of B's lines kept in L2 (evict_last)
  int32_t *carry_rows;  // [num_chunks] head row of each chunk, -1 = none
  float *carry_vals;    // [num_chunks * N] head-row partials
  float *tail_vals;     // [num_chunks * N] partial of a last row that continues
  int *carry_cnt;       // [num_chunks * column tiles] arrivals per straddling row (zeroed per launch)
  int *seg_cnt;         // segment SR walk: [2 * num_chunks] elements of the owner's tail segment
                        // (k) and of the head segment (num_chunks + k) in chunk k, for means
};

struct ChunkInfo {
  int cs, ce;        // nonzero range [cs, ce)
  int r_first;       // row of nonzero cs
  int r_last;        // row of nonzero ce - 1
  int prev_row;      // row of nonzero cs - 1 (-1 when cs == 0)
  bool has_head;     // r_first started before cs
};

template <bool SEG>
__device__ __forceinline__ ChunkInfo chunk_info(const EbArgs &a, int chunk) {
  ChunkInfo ci;
  ci.cs = chunk * a.chunk;
  ci.ce = min(ci.cs + a.chunk, a.nnz);
  if (SEG) {
    ci.r_first = __ldg(a.index + ci.cs);
    ci.r_last = __ldg(a.index + ci.ce - 1);
    ci.prev_row = ci.cs > 0 ? __ldg(a.index + ci.cs - 1) : -1;
    ci.has_head = ci.cs > 0 && ci.prev_row == ci.r_first;
  } else {
    // binary_search_segment_number semantics (check.cuh:88-102)
    ci.r_first = row_search(a.indptr, 1, a.M, ci.cs);
    ci.r_last = row_search(a.indptr, 1, a.M, ci.ce - 1);
    ci.has_head = ci.cs > 0 && __ldg(a.indptr + ci.r_first) < ci.cs;
    ci.prev_row = ci.cs == 0 ? -1 : (ci.has_head ? ci.r_first : row_search(a.indptr, 1, a.M, ci.cs - 1));
  }
  return ci;
}

// Row (segment) of nonzero p inside a chunk whose rows span [r_first, r_last].
template <bool SEG>
__device__ __forceinline__ int chunk_row(const EbArgs &a, const ChunkInfo &ci, int p) {
  if (SEG) return __ldg(a.index + p);
  return row_search(a.indptr, ci.r_first + 1, ci.r_last + 1, p);
}

// Does the chunk's last row end inside the chunk?
template <bool SEG>
__device__ __forceinline__ bool row_ends_in_chunk(const EbArgs &a, const ChunkInfo &ci, int row) {
  if (ci.ce >= a.nnz) return true;
  if (SEG) return __ldg(a.index + ci.ce) != row;
  if ((unsigned)row >= (unsigned)a.M) return true;
  return __ldg(a.indptr + row + 1) <= ci.ce;
}

// Writes zeros to rows [lo, hi] (clamped to the output) for this lane's
// columns.  Used only in overwrite mode.
template <typename TC, int V, int NV>
__device__ __forceinline__ void zero_rows(const EbArgs &a, int lo, int hi, int col0,
                                          const bool (&act)[NV], uint64_t pol) {
  lo = max(lo, 0);
  hi = min(hi, a.M - 1);
  float z[V];
  #pragma unroll
  for (int i = 0; i < V; i++) z[i] = 0.f;
  TC *C = (TC *)a.C;
  for (int r = lo; r <= hi; r++)
    #pragma unroll
    for (int j = 0; j < NV; j++)
      if (act[j]) store_vec<TC, V>(C + (int64_t)r * a.N + col0 + j * V, z, pol);
}

// Writes one row partial: to the head slot when it is the chunk's head row,
// to the tail slot when the row continues past the chunk (`complete` false),
// else to C (the owner of a row that starts and ends in this chunk).
template <typename TC, int V, int NV>
__device__ __forceinline__ void flush_row(const EbArgs &a, const ChunkInfo &ci, int chunk, int row,
                                          float (&acc)[NV][V], int cnt, bool complete, int col0,
                                          const bool (&act)[NV], uint64_t pol) {
  if (ci.has_head && row == ci.r_first) {
    #pragma unroll
    for (int j = 0; j < NV; j++)
      if (act[j]) store_vec<float, V>(a.carry_vals + (int64_t)chunk * a.N + col0 + j * V, acc[j], pol);
    return;
  }
  if (!complete) {
    #pragma unroll
    for (int j = 0; j < NV; j++)
      if (act[j]) store_vec<float, V>(a.tail_vals + (int64_t)chunk * a.N + col0 + j * V, acc[j], pol);
    return;
  }
  if ((unsigned)row >= (unsigned)a.M) return;
  TC *C = (TC *)a.C;
  #pragma unroll
  for (int j = 0; j < NV; j++) {
    if (!act[j]) continue;
    float out[V];
    #pragma unroll
    for (int i = 0; i < V; i++) out[i] = acc[j][i];
    if (a.reduce == SS_MEAN) {
      #pragma unroll
      for (int i = 0; i < V; i++) out[i] = acc[j][i] / (float)cnt;
    }
    TC *dst = C + (int64_t)row * a.N + col0 + j * V;
    if (a.accumulate) {
      float prev[V];
      load_out<TC, V>(dst, prev);
      #pragma unroll
      for (int i = 0; i < V; i++) out[i] += prev[i];
    }
    store_vec<TC, V>(dst, out, pol);
  }
}

// V floats from a carry slot written by other blocks in this launch: read
// at L2 (ld.global.cg), never from a possibly stale L1 line.
template <int V>
__device__ __forceinline__ void load_slot(const float *p, float (&out)[V]) {
  if constexpr (V == 1) {
    out[0] = __ldcg(p);
  } else if constexpr (V == 2) {
    const float2 x = __ldcg(reinterpret_cast<const float2 *>(p));
    out[0] = x.x; out[1] = x.y;
  } else {
    #pragma unroll
    for (int i = 0; i < V; i += 4) {
      const float4 x = __ldcg(reinterpret_cast<const float4 *>(p + i));
      out[i] = x.x; out[i + 1] = x.y; out[i + 2] = x.z; out[i + 3] = x.w;
    }
  }
}

// In-kernel carry fix-up of the SpMM walks.  Row r straddles chunks o..l
// (o holds its first nonzero and left r's partial in its tail slot; o+1..l
// left theirs in their head slots).  Each of the l - o + 1 participants
// calls this after storing its slot; the last to arrive (atomic count per
// owner chunk and column tile) sums tail(o) + heads(o+1..l) in chunk order
// with compensation, adds the old output in accumulate mode and stores the
// row once - the same arithmetic, in the same order, as fixup_chunk, so the
// result does not depend on which participant finishes last.  Nothing
// waits: a participant that is not last returns at once.
template <typename TC, int V, int NV, int BATCH = 1>
__device__ __forceinline__ void carry_arrive(const EbArgs &a, int r, int lane, int G, unsigned mask, int col0,
                                          const bool (&act)[NV], uint64_t pol) {
  const int o = __ldg(a.indptr + r) / a.chunk;
  const int l = (__ldg(a.indptr + r + 1) - 1) / a.chunk;
  int *cnt = a.carry_cnt + (size_t)o * gridDim.y + blockIdx.y;
  __threadfence();  // this lane's slot stores are visible before the count moves
  __syncwarp(mask);
  int last = 0;
  if (lane == 0) last = atomicAdd(cnt, 1) == l - o;
  last = __shfl_sync(mask, last, 0, G);
  if (!last) return;
  __threadfence();  // every other participant's slot is visible now
  TC *C = (TC *)a.C;
  #pragma unroll
  for (int j = 0; j < NV; j++) {
    if (!act[j]) continue;
    const int64_t col = col0 + j * V;
    float acc[V], comp[V], x[V];
    load_slot<V>(a.tail_vals + (int64_t)o * a.N + col, acc);
    #pragma unroll
    for (int i = 0; i < V; i++) comp[i] = 0.f;
    if constexpr (BATCH == 1) {
      for (int k = o + 1; k <= l; k++) {
        load_slot<V>(a.carry_vals + (int64_t)k * a.N + col, x);
        #pragma unroll
        for (int i = 0; i < V; i++) kahan_add(acc[i], comp[i], x[i]);
      }
    } else {  // BATCH heads in flight, added in the same order
      for (int k0 = o + 1; k0 <= l; k0 += BATCH) {
        float xb[BATCH][V];
        #pragma unroll
        for (int u = 0; u < BATCH; u++) {
          if (k0 + u <= l) {
            load_slot<V>(a.carry_vals + (int64_t)(k0 + u) * a.N + col, xb[u]);
          } else {
            #pragma unroll
            for (int i = 0; i < V; i++) xb[u][i] = 0.f;
          }
        }
        #pragma unroll
        for (int u = 0; u < BATCH; u++) {
          if (k0 + u > l) break;
          #pragma unroll
          for (int i = 0; i < V; i++) kahan_add(acc[i], comp[i], xb[u][i]);
        }
      }
    }
    TC *dst = C + (int64_t)r * a.N + col;
    if (a.accumulate) {
      float prev[V];
      load_out<TC, V>(dst, prev);
      #pragma unroll
      for (int i = 0; i < V; i++) acc[i] += prev[i];
    }
    store_vec<TC, V>(dst, acc, pol);
  }
}

// ---------------------------------------------------------------------
// In-kernel carry assembly of the segment SR walk.  A segment has no
// row pointer, so the chunks it spans are found from chunk boundaries: a
// chunk j > o holds part of segment r iff index[j * chunk] == r, and the
// owner o is the last chunk before the participant whose first id is
// smaller than r (or 0).  Each lane of a group probes one boundary; the
// first round's probes are loaded when the chunk starts, so their latency
// overlaps the walk.
// ---------------------------------------------------------------------
__device__ __forceinline__ unsigned group_ballot(unsigned mask, bool pred, int G) {
  const unsigned bits = G >= 32 ? 0xffffffffu : ((1u << G) - 1u);
  const unsigned shift = (threadIdx.x & 31u) & ~(unsigned)(G - 1);
  return (__ballot_sync(mask, pred) >> shift) & bits;
}

// index[(chunk - 1 - lane) * a.chunk], INT_MIN before the array
__device__ __forceinline__ int seg_probe_back(const EbArgs &a, int chunk, int lane) {
  const long long j = (long long)chunk - 1 - lane;
  return j >= 0 ? __ldg(a.index + j * a.chunk) : INT_MIN;
}
// index[(chunk + 1 + lane) * a.chunk], INT_MAX past the array
__device__ __forceinline__ int seg_probe_fwd(const EbArgs &a, int chunk, int lane) {
  const long long e = ((long long)chunk + 1 + lane) * a.chunk;
  return e < a.nnz ? __ldg(a.index + e) : INT_MAX;
}

// Owner chunk of segment r, which continues into `chunk` from before it;
// `back` is this lane's seg_probe_back(chunk).  The nearest chunk j before
// `chunk` whose first id is below r holds r's start unless r starts exactly
// at chunk j + 1's first element (then j + 1 owns it): the last id of
// chunk j tells which.
__device__ __forceinline__ int seg_owner(const EbArgs &a, int r, int chunk, int back, int lane, int G,
                                         unsigned mask) {
  int base = chunk - 1;  // lane i holds the first id of chunk base - i
  int v = back;
  while (true) {
    const unsigned m = group_ballot(mask, v < r, G);
    if (m) {
      const int j = base - (__ffs(m) - 1);
      if (j < 0) return 0;  // a probe before the array: r starts at element 0
      return __ldg(a.index + (int64_t)(j + 1) * a.chunk - 1) == r ? j : j + 1;
    }
    base -= G;  // every probe was r: r started before all of them (base >= G here)
    v = seg_probe_back(a, base + 1, lane);
  }
}

// Last chunk holding part of segment r, which `chunk` holds and which
// continues past it; `fwd` is this lane's seg_probe_fwd(chunk).
__device__ __forceinline__ int seg_last(const EbArgs &a, int r, int chunk, int fwd, int lane, int G,
                                        unsigned mask) {
  int base = chunk + 1;  // lane i holds the first id of chunk base + i
  int v = fwd;
  while (true) {
    const unsigned m = group_ballot(mask, v != r, G);
    if (m) return base + (__ffs(m) - 1) - 1;
    base += G;
    v = seg_probe_fwd(a, base - 1, lane);
  }
}

// carry_arrive for segment r spanning chunks o..l: the last participant
// combines tail(o) and heads(o+1..l) in chunk order (Kahan sum, or max),
// divides a mean by the segment's length (owner's tail count + full middle
// chunks + the last chunk's head count) and stores dst once; the same
// arithmetic in the same order as fixup_chunk.
template <int V, int NV>
__device__ __forceinline__ void seg_carry_arrive(const EbArgs &a, int r, int o, int l, int lane, int G,
                                              unsigned mask, int col0, const bool (&act)[NV], uint64_t pol) {
  if ((unsigned)r >= (unsigned)a.M) return;  // every participant sees the same r: none counts
  int *cnt = a.carry_cnt + (size_t)o * gridDim.y + blockIdx.y;
  __threadfence();  // this lane's slot and count stores are visible before the count moves
  __syncwarp(mask);
  int last = 0;
  if (lane == 0) last = atomicAdd(cnt, 1) == l - o;
  last = __shfl_sync(mask, last, 0, G);
  if (!last) return;
  __threadfence();  // every other participant's stores are visible now
  const bool is_max = a.reduce == SS_MAX;
  float count = 1.f;
  if (a.reduce == SS_MEAN)
    count = (float)(__ldcg(a.seg_cnt + o) + (l - o - 1) * a.chunk + __ldcg(a.seg_cnt + a.num_chunks + l));
  float *C = (float *)a.C;
  #pragma unroll
  for (int j = 0; j < NV; j++) {
    if (!act[j]) continue;
    const int64_t col = col0 + j * V;
    float acc[V], comp[V], x[V];
    load_slot<V>(a.tail_vals + (int64_t)o * a.N + col, acc);
    #pragma unroll
    for (int i = 0; i < V; i++) comp[i] = 0.f;
    for (int k = o + 1; k <= l; k++) {
      load_slot<V>(a.carry_vals + (int64_t)k * a.N + col, x);
      #pragma unroll
      for (int i = 0; i < V; i++) {
        if (is_max) acc[i] = fmaxf(acc[i], x[i]);
        else kahan_add(acc[i], comp[i], x[i]);
      }
    }
    float *dst = C + (int64_t)r * a.N + col;
    if (a.accumulate) {
      float prev[V];
      load_out<float, V>(dst, prev);
      #pragma unroll
      for (int i = 0; i < V; i++) acc[i] += prev[i];
    }
    if (a.reduce == SS_MEAN) {
      #pragma unroll
      for (int i = 0; i < V; i++) acc[i] = acc[i] / count;
    }
    store_vec<float, V>(dst, acc, pol);
  }
}

// First r in [0, M] with indptr[r] >= key, found by all G lanes of the
// group: each round every lane probes one of G split points of [lo, hi].
__device__ __forceinline__ int group_lower_bound(const int32_t *indptr, int M, int key, int lane, int G,
                                                 unsigned mask) {
  int lo = 0, hi = M;  // answer in [lo, hi]
  const unsigned lanes_bits = G >= 32 ? 0xffffffffu : ((1u << G) - 1u);
  const unsigned shift = (threadIdx.x & 31u) & ~(unsigned)(G - 1);
  while (lo < hi) {
    const long long span = (long long)(hi - lo);
    const int probe = lo + (int)((span * (lane + 1)) / (G + 1));
    const bool ge = __ldg(indptr + probe) >= key;
    const unsigned hits = (__ballot_sync(mask, ge) >> shift) & lanes_bits;
    const int first = hits ? __ffs(hits) - 1 : G;  // first lane whose probe is >= key
    const int nhi = first < G ? __shfl_sync(mask, probe, first, G) : hi;
    const int nlo = first > 0 ? __shfl_sync(mask, probe, first - 1, G) + 1 : lo;
    lo = nlo;
    hi = nhi;
  }
  return lo;
}

// chunk_info for the SpMM path with the G lanes of a worker searching
// together (group_lower_bound); the same rows as chunk_info<false>:
// row_search(indptr, 1, M, e) is the first r >= 1 with indptr[r] > e, less
// one, capped at M - 1, i.e. min(lower_bound(e + 1), M) - 1.
__device__ __forceinline__ ChunkInfo chunk_info_group(const EbArgs &a, int chunk, int lane, int G, unsigned mask) {
  ChunkInfo ci;
  ci.cs = chunk * a.chunk;
  ci.ce = min(ci.cs + a.chunk, a.nnz);
  ci.r_first = min(group_lower_bound(a.indptr, a.M, ci.cs + 1, lane, G, mask), a.M) - 1;
  ci.r_last = min(group_lower_bound(a.indptr, a.M, ci.ce, lane, G, mask), a.M) - 1;
  ci.has_head = ci.cs > 0 && __ldg(a.indptr + ci.r_first) < ci.cs;
  if (ci.cs == 0) ci.prev_row = -1;
  else if (ci.has_head) ci.prev_row = ci.r_first;
  else ci.prev_row = min(group_lower_bound(a.indptr, a.M, ci.cs, lane, G, mask), a.M) - 1;
  return ci;
}

__device__ __forceinline__ int lower_bound_idx(const int32_t *index, int n, int key) {
  int lo = 0, hi = n;
  while (lo < hi) {
    int mid = (lo + hi) >> 1;
    if (__ldg(index + mid) < key) lo = mid + 1; else hi = mid;
  }
  return lo;
}

// Carry fix-up of chunk c (one warp): when c leads a run of chunks whose
// head is row r, row r = owner's tail (chunk c - 1) + the run's heads, summed
// in chunk order with compensation (max for SS_MAX), plus the old output in
// accumulate mode, divided by the segment length for a mean.
template <typename TC>
__device__ __forceinline__ void fixup_chunk(const int32_t *__restrict__ rows, const float *__restrict__ heads,
                                            const float *__restrict__ tails, int num_chunks, int N, int M, TC *C,
                                            int reduce, int accumulate, const int32_t *__restrict__ index, int nnz,
                                            int c, int lane) {
  const int r = rows[c];
  if (c == 0 || r < 0 || r >= M) return;
  if (rows[c - 1] == r) return;  // not the leader of this run
  // end of the run: the warp compares 32 head rows per step
  int cend = c + 1;
  while (true) {
    const int k = cend + lane;
    const bool same = k < num_chunks && rows[k] == r;
    const unsigned m = __ballot_sync(0xffffffffu, same);
    if (m == 0xffffffffu) {
      cend += 32;
    } else {
      cend += __ffs(~m) - 1;
      break;
    }
  }
  float count = 1.f;
  if (reduce == SS_MEAN && index != nullptr) {
    int lo = 0, hi = 0;
    if (lane == 0) {
      lo = lower_bound_idx(index, nnz, r);
      hi = lower_bound_idx(index, nnz, r + 1);
    }
    lo = __shfl_sync(0xffffffffu, lo, 0);
    hi = __shfl_sync(0xffffffffu, hi, 0);
    count = (float)max(hi - lo, 1);
  }
  TC *crow = C + (int64_t)r * N;
  for (int j = lane; j < N; j += 32) {
    float acc = tails[(int64_t)(c - 1) * N + j];  // the owner's partial
    float comp = 0.f;
    for (int k0 = c; k0 < cend; k0 += 8) {  // eight heads in flight, added in order
      float x[8];
      #pragma unroll
      for (int u = 0; u < 8; u++) x[u] = k0 + u < cend ? heads[(int64_t)(k0 + u) * N + j] : 0.f;
      #pragma unroll
      for (int u = 0; u < 8; u++) {
        if (k0 + u >= cend) break;
        if (reduce == SS_MAX) acc = fmaxf(acc, x[u]);
        else kahan_add(acc, comp, x[u]);
      }
    }
    if (accumulate) acc += Elem<TC>::to_f(crow[j]);
    if (reduce == SS_MEAN) acc = acc / count;
    crow[j] = Elem<TC>::from_f(acc);
  }
}

}  // namespace ss
