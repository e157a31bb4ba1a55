// Element-balanced, sequential reduction: ebsr SpMM and the sequential
// segment_coo family.
//
// Reference counterparts: csrspmm_rowcaching_nnzbalance_cg_kernel
// (test-cg/include/spmm/spmm_cg.cuh:376-551) and segscan_sr_kernel /
// segscan_sr_noshmem_kernel / segscan_sr_noshmem_lessatom_kernel /
// segscan_sr_sorted_kernel (new-cg/include/segscan/segscan.cuh:357-815).
//
// A worker is a group of G lanes laid along N: lane l owns E = V*NV
// consecutive columns, so one gathered B row is a single contiguous request
// across the group.  A worker walks its chunk of nonzeros in order:
//  * the chunk's column and value streams are staged in shared memory in
//    tiles of S nonzeros by TMA bulk copies (cp.async.bulk completed on an
//    mbarrier), double buffered so the next tile lands while this one is
//    walked; misaligned streams fall back to coalesced loads;
//  * the first row is found by a G-ary search of indptr (every lane probes
//    one split point per round), and rows are then tracked from a window of
//    indptr staged in shared memory - no per-nonzero search;
//  * four B rows are gathered ahead of the multiply-adds, with registers
//    capped at 64 so that 32+ warps per SM keep enough gathers in flight;
//  * rows longer than kahan_threshold accumulate with compensated
//    summation, every nonzero of them: the tile labelling marks their
//    nonzeros (one bit each), and the multiply-add of a marked nonzero is a
//    compensated step;
//  * a row is flushed when the walk passes its end (eb_common.cuh: owner
//    store, head/tail slots for the two rows that straddle the chunk,
//    zeros for empty rows).
// Every wait on an mbarrier is bounded; on expiry the kernel records
// SS_ERR_TIMEOUT in the device flag a.err (ss_device_error) and the group
// stops walking: it waits (bounded) for the copies it has in flight and
// issues no more.  This header holds the kernel templates; eb_walk_*.cu
// instantiate them per storage type and eb_walk.cu launches them.
#pragma once

#include "eb_common.cuh"
#include "internal.h"

namespace ss {

#ifndef SS_SR_GATHER
#define SS_SR_GATHER 4
#endif
#ifndef SS_SR_MIN_BLOCKS
#define SS_SR_MIN_BLOCKS 2
#endif
constexpr int SR_U = SS_SR_GATHER;            // B rows gathered ahead
constexpr uint32_t SR_SPIN_LIMIT = 1u << 22;  // try_wait polls before giving up

// Per-group shared memory: [bar0 bar1 | col[2][S] | val[2][S] | win[W]]
struct SrLayout {
  int S, W, vs;
  int col_off, val_off, info_off, win_off, bytes;
};

// Per-group shared memory: [bar0 bar1 | col[2][S] | val[2][S] | info[2][S] |
// win[W]].  info holds, per staged nonzero, its row and an end-of-row bit.
__host__ __device__ inline SrLayout sr_layout(int S, int vs) {
  SrLayout L;
  L.S = S;
  L.W = 2 * S + 8;
  L.vs = vs;
  int o = 16;  // two mbarriers
  L.col_off = o;
  o += 2 * S * 4;
  L.val_off = o;
  o += (2 * S * vs + 15) & ~15;
  L.info_off = o;
  o += 2 * S * 4;
  L.win_off = o;
  o += L.W * 4;
  L.bytes = (o + 15) & ~15;
  return L;
}

struct Stage {
  uint64_t *bar;    // [2]
  int32_t *col;     // [2][S]
  char *val;        // [2][S * vs]
  int32_t *info;    // [2][S]
  int32_t *win;     // [W]
  uint32_t phases;  // bit b: parity to wait for on bar[b]
  uint32_t tma;     // bit b: buffer b was filled by a bulk copy
};

// Starts loading nonzeros [sb, sb + n) into buffer b.
template <typename T, bool SEG>
__device__ __forceinline__ void stage_issue(const EbArgs &a, Stage &st, const SrLayout &L, int b, int sb, int n,
                                            int lane, int G, unsigned mask, uint64_t strm) {
  int32_t *dcol = st.col + b * L.S;
  T *dval = reinterpret_cast<T *>(st.val + b * L.S * L.vs);
  const int32_t *scol = SEG ? a.index : a.cols;
  const T *sval = SEG ? nullptr : (const T *)a.vals;
  __syncwarp(mask);  // every lane is done reading buffer b
  // bulk copies need 16-byte aligned sources and sizes: 8-element multiples
  // (row-aligned batch items start anywhere; their misaligned tiles load plainly)
  const bool tma = a.use_tma && (n % 8) == 0 && (sb % 8) == 0;
  st.tma = tma ? (st.tma | (1u << b)) : (st.tma & ~(1u << b));
  if (tma) {
    if (lane == 0) {
      fence_async_smem();
      const uint32_t bytes = (uint32_t)n * 4u + (sval ? (uint32_t)n * (uint32_t)sizeof(T) : 0u);
      mbar_expect_tx(st.bar + b, bytes);
      bulk_g2s(dcol, scol + sb, (uint32_t)n * 4u, st.bar + b);
      if (sval) bulk_g2s(dval, sval + sb, (uint32_t)n * (uint32_t)sizeof(T), st.bar + b);
    }
  } else {
    for (int i = lane; i < n; i += G) {
      dcol[i] = ld_idx(scol + sb + i, strm);
      if (sval) dval[i] = sval[sb + i];
    }
  }
}

// Waits for buffer b; false when the bounded wait expired.  The group
// agrees on the outcome; the phase advances only on success, so a buffer
// whose wait expired can be waited for again (stage_drain).
__device__ __forceinline__ bool stage_wait(Stage &st, int b, unsigned mask, int *err) {
  bool ok = true;
  if (st.tma & (1u << b)) {
    uint32_t it = 0;
    while (!mbar_try_wait(st.bar + b, (st.phases >> b) & 1u)) {
      if (++it > SR_SPIN_LIMIT) {
        ok = false;
        break;
      }
    }
    ok = __all_sync(mask, ok);
    if (ok) st.phases ^= 1u << b;
    else if (err) atomicExch(err, (int)SS_ERR_TIMEOUT);
  }
  __syncwarp(mask);
  return ok;
}

// After an expired wait: waits again, bounded, for the staged tiles
// [from, to) whose bulk copies may still be landing, so the group leaves no
// copy in flight into its buffers.
__device__ __forceinline__ void stage_drain(Stage &st, int from, int to, unsigned mask) {
  for (int t = from; t < to; t++) stage_wait(st, t & 1, mask, nullptr);
}

template <int V, int NV, bool KAHAN>
__device__ __forceinline__ void add_row(float (&acc)[NV][V], float (&comp)[NV][V], float v,
                                        const float (&b)[NV][V]) {
  #pragma unroll
  for (int j = 0; j < NV; j++)
    #pragma unroll
    for (int i = 0; i < V; i++) {
      if (KAHAN) kahan_fma(acc[j][i], comp[j][i], v, b[j][i]);
      else acc[j][i] = fmaf(v, b[j][i], acc[j][i]);
    }
}

// acc += v * b, compensated when the row is longer than the threshold.
template <int V, int NV>
__device__ __forceinline__ void add_row(float (&acc)[NV][V], float (&comp)[NV][V], float v,
                                        const float (&b)[NV][V], bool kahan) {
  if (kahan) add_row<V, NV, true>(acc, comp, v, b);
  else add_row<V, NV, false>(acc, comp, v, b);
}

// ---------------------------------------------------------------------
// SpMM chunk walk
//
// State carried from tile to tile: cur = row of the latest nonzero (or the
// chunk's first row), acc = partial of cur that is not yet written (open).
// Fast tile: the lanes first label every staged nonzero with its row and an
// end-of-row bit (binary search in the indptr window, in parallel) and zero
// the empty rows that follow a row end; the walk then only gathers,
// multiplies, and stores on the end bits.  A tile whose rows do not fit the
// window (long runs of empty rows) is walked element by element instead.
// ---------------------------------------------------------------------
template <typename TC, int V, int NV>
__device__ __forceinline__ void store_out(const EbArgs &a, int row, float (&acc)[NV][V], int col0,
                                          const bool (&act)[NV], uint64_t pol) {
  TC *C = (TC *)a.C;
  #pragma unroll
  for (int j = 0; j < NV; j++) {
    if (!act[j]) continue;
    TC *dst = C + (int64_t)row * a.N + col0 + j * V;
    if (a.accumulate) {
      float prev[V], out[V];
      load_out<TC, V>(dst, prev);
      #pragma unroll
      for (int i = 0; i < V; i++) out[i] = acc[j][i] + prev[i];
      store_vec<TC, V>(dst, out, pol);
    } else {
      store_vec<TC, V>(dst, acc[j], pol);
    }
  }
}

// Walks nonzeros [cs, ce) as work item `chunk` (its head / tail slots); the
// first two tiles are in flight, lb is the first row starting at or after
// cs and the window holds indptr from win_base on.  The tile labelling marks
// the nonzeros of rows longer than a.kahan (kmask), which are summed with
// compensation.  Returns false when a bounded wait expired (the caller then
// stops).
template <typename T, typename TC, int V, int NV>
__device__ __forceinline__ bool sr_spmm_walk(const EbArgs &a, int chunk, int cs, int ce, int nst, int lb,
                                             int win_base, int lane, unsigned mask, Stage &st, const SrLayout &L,
                                             int col0, const bool (&act)[NV], uint64_t keep, uint64_t strm) {
  const T *__restrict__ B = (const T *)a.B;
  const int G = a.team_lanes;
  const bool ones = a.vals == nullptr;
  // B rows gathered ahead: four, or two when a lane holds 8+ elements of a
  // row (the gathered values then need as many registers), except that the
  // full-tile loop keeps four 16-bit rows of eight elements packed
  constexpr int SR_FU = V * NV >= 8 ? 2 : 4;
  constexpr int SR_UP = V * NV >= 8 ? 2 : SR_U;
  constexpr bool PACKED = sizeof(T) == 2 && V == 8 && NV == 1;
  ChunkInfo ci;
  ci.cs = cs;
  ci.ce = ce;
  auto win_fill = [&](int base) {
    __syncwarp(mask);
    win_base = base;
    for (int i = lane; i < L.W; i += G) st.win[i] = __ldg(a.indptr + min(base + i, a.M));
    __syncwarp(mask);
  };
  auto wget = [&](int r) -> int {
    if (r - win_base >= L.W || r < win_base) win_fill(r);
    return st.win[r - win_base];
  };
  int cur;
  ci.has_head = lb > 0 && wget(lb) > ci.cs;  // cs lies inside row lb - 1
  if (ci.has_head) {
    cur = lb - 1;
  } else {
    cur = lb;
    // rows that start and end at cs are empty; this chunk owns them
    while (cur < a.M - 1 && wget(cur + 1) <= ci.cs) {
      if (!a.accumulate) zero_rows<TC, V, NV>(a, cur, cur, col0, act, strm);
      cur++;
    }
  }
  ci.r_first = cur;
  ci.r_last = cur;
  ci.prev_row = -1;
  const int head = ci.has_head ? cur : -1;

  bool open = false;
  float acc[NV][V], comp[NV][V];
  #pragma unroll
  for (int j = 0; j < NV; j++)
    #pragma unroll
    for (int i = 0; i < V; i++) { acc[j][i] = 0.f; comp[j][i] = 0.f; }

  // writes acc for row r (head slot, owner store) and clears it
  auto flush_done = [&](int r) {
    if (r == head) {
      #pragma unroll
      for (int j = 0; j < NV; j++)
        if (act[j]) store_vec<float, V>(a.carry_vals + (int64_t)chunk * a.N + col0 + j * V, acc[j], strm);
    } else if ((unsigned)r < (unsigned)a.M) {
      store_out<TC, V, NV>(a, r, acc, col0, act, strm);
    }
    #pragma unroll
    for (int j = 0; j < NV; j++)
      #pragma unroll
      for (int i = 0; i < V; i++) { acc[j][i] = 0.f; comp[j][i] = 0.f; }
  };

  for (int s = 0; s < nst; s++) {
    const int b = s & 1;
    const int sb = ci.cs + s * L.S;
    const int n = min(L.S, ci.ce - sb);
    const int last = sb + n - 1;
    if (!stage_wait(st, b, mask, a.err)) {
      stage_drain(st, s, min(nst, s + 2), mask);  // tiles s and s + 1 may still be landing
      return false;
    }
    const int32_t *scol = st.col + b * L.S;
    const T *sval = reinterpret_cast<const T *>(st.val + b * L.S * L.vs);
    int32_t *sinfo = st.info + b * L.S;

    // the window must hold the starts of every row this tile touches and of
    // the row after the last one
    if (cur < win_base || st.win[L.W - 1] <= last) win_fill(cur);
    const bool fast = st.win[L.W - 1] > last || win_base + L.W - 1 >= a.M;

    if (fast) {
      // ---- label the tile's nonzeros with row | end-of-row bit, and mark
      // those of long rows (kmask bit e); empty rows starting where a row's
      // first nonzero sits are zeroed by the whole group (each lane owns one
      // column slice)
      const int c0 = cur - win_base;
      const int rounds = (n + G - 1) / G;
      bool bad = false;  // a column outside [0, K) in this tile
      uint64_t kmask = 0;
      for (int k = 0; k < rounds; k++) {
        const int e = lane + k * G;
        int zlo = 0, zhi = -1;
        bool kah = false;
        if (e < n) {
          bad |= (unsigned)scol[e] >= (unsigned)a.K;
          const int p = sb + e;
          int lo = c0 + 1, hi = L.W - 1;
          while (lo < hi) {
            const int mid = (lo + hi) >> 1;
            if (st.win[mid] <= p) lo = mid + 1; else hi = mid;
          }
          const int rr = lo - 1;  // window slot of p's row
          const bool end = st.win[rr + 1] == p + 1;
          kah = st.win[rr + 1] - st.win[rr] > a.kahan;
          sinfo[e] = (win_base + rr) | (end ? (int)0x80000000 : 0);
          if (st.win[rr] == p && p != ci.cs) {  // p opens row rr: empties before it start at p too
            int q = rr - 1;
            while (q > c0 && st.win[q] == p) q--;
            zlo = win_base + q + 1;
            zhi = win_base + rr - 1;
          }
        }
        kmask |= (uint64_t)group_ballot(mask, kah, G) << (k * G);
        unsigned todo = __ballot_sync(mask, zlo <= zhi);
        while (todo) {
          const int src = __ffs(todo) - 1;
          const int lo_r = __shfl_sync(mask, zlo, src);
          const int hi_r = __shfl_sync(mask, zhi, src);
          if (!a.accumulate) zero_rows<TC, V, NV>(a, lo_r, hi_r, col0, act, strm);
          todo &= todo - 1;
        }
      }
      __syncwarp(mask);  // labels written by every lane are visible to the group
      // a full tile of valid columns takes the lean loop: four staged
      // columns, labels and values per shared-memory read, no bounds checks
      const bool full = n == L.S && !__any_sync(mask, bad);
      auto consume = [&](int info, float v, const float (&b)[NV][V], bool kah) {
        add_row<V, NV>(acc, comp, v, b, kah);
        cur = info & 0x7fffffff;
        open = true;
        if (info < 0) {
          flush_done(cur);
          open = false;
        }
      };
      if (full) {
        const int4 *col4 = reinterpret_cast<const int4 *>(scol);
        const int4 *info4 = reinterpret_cast<const int4 *>(sinfo);
        for (int q = 0; q < n; q += 4) {
          const int4 cc = col4[q >> 2];
          const int4 in4 = info4[q >> 2];
          const int cs4[4] = {cc.x, cc.y, cc.z, cc.w};
          const int is4[4] = {in4.x, in4.y, in4.z, in4.w};
          float v4[4];
          if (ones) {
            v4[0] = v4[1] = v4[2] = v4[3] = 1.f;
          } else if constexpr (sizeof(T) == 4) {
            const float4 x = *reinterpret_cast<const float4 *>(sval + q);
            v4[0] = x.x; v4[1] = x.y; v4[2] = x.z; v4[3] = x.w;
          } else {
            const uint2 x = *reinterpret_cast<const uint2 *>(sval + q);
            unpack2(x.x, v4[0], v4[1], (T *)nullptr);
            unpack2(x.y, v4[2], v4[3], (T *)nullptr);
          }
          const unsigned k4 = (unsigned)(kmask >> q) & 0xfu;  // compensated among these four
          if constexpr (PACKED) {
            // 16-bit rows of one 16-byte vector per lane: the four rows stay
            // packed (four registers each) until their multiply-adds
            uint4 raw[4];
            #pragma unroll
            for (int u = 0; u < 4; u++)
              raw[u] = act[0] ? ld_u128(B + (int64_t)cs4[u] * a.N + col0, keep) : make_uint4(0, 0, 0, 0);
            #pragma unroll
            for (int u = 0; u < 4; u++) {
              float bv[1][V];
              unpack2(raw[u].x, bv[0][0], bv[0][1], (T *)nullptr);
              unpack2(raw[u].y, bv[0][2], bv[0][3], (T *)nullptr);
              unpack2(raw[u].z, bv[0][4], bv[0][5], (T *)nullptr);
              unpack2(raw[u].w, bv[0][6], bv[0][7], (T *)nullptr);
              consume(is4[u], v4[u], reinterpret_cast<const float(&)[NV][V]>(bv), (k4 >> u) & 1u);
            }
          } else {
            #pragma unroll
            for (int h = 0; h < 4; h += SR_FU) {
              float bv[SR_FU][NV][V];
              #pragma unroll
              for (int u = 0; u < SR_FU; u++)
                #pragma unroll
                for (int j = 0; j < NV; j++) {
                  if (act[j]) {
                    load_vec<T, V>(B + (int64_t)cs4[h + u] * a.N + col0 + j * V, bv[u][j], keep);
                  } else {
                    #pragma unroll
                    for (int i = 0; i < V; i++) bv[u][j][i] = 0.f;
                  }
                }
              #pragma unroll
              for (int u = 0; u < SR_FU; u++) consume(is4[h + u], v4[h + u], bv[u], (k4 >> (h + u)) & 1u);
            }
          }
        }
      } else for (int q = 0; q < n; q += SR_UP) {  // ---- partial tile: gather, multiply, store at row ends
        float bv[SR_UP][NV][V];
        #pragma unroll
        for (int u = 0; u < SR_UP; u++) {
          const int c = q + u < n ? scol[q + u] : -1;
          const bool live = (unsigned)c < (unsigned)a.K;
          #pragma unroll
          for (int j = 0; j < NV; j++) {
            if (live && act[j]) {
              load_vec<T, V>(B + (int64_t)c * a.N + col0 + j * V, bv[u][j], keep);
            } else {
              #pragma unroll
              for (int i = 0; i < V; i++) bv[u][j][i] = 0.f;
            }
          }
        }
        #pragma unroll
        for (int u = 0; u < SR_UP; u++) {
          if (q + u >= n) break;
          consume(sinfo[q + u], ones ? 1.f : Elem<T>::to_f(sval[q + u]), bv[u], (kmask >> (q + u)) & 1u);
        }
      }
    } else {
      // ---- element by element (tiles crossing long runs of empty rows)
      int next_start = wget(cur + 1);
      if (!open) {
        // the previous row ended at sb: move to the row of the tile's first
        // nonzero, zeroing the empty rows on the way
        while (cur < a.M - 1 && next_start <= sb) {
          cur++;
          next_start = wget(cur + 1);
          if (next_start <= sb && !a.accumulate) zero_rows<TC, V, NV>(a, cur, cur, col0, act, strm);
        }
      }
      bool kah = next_start - wget(cur) > a.kahan;  // row cur is compensated
      for (int q = 0; q < n; q++) {
        const int p = sb + q;
        const int c = scol[q];
        float bq[NV][V];
        #pragma unroll
        for (int j = 0; j < NV; j++) {
          if ((unsigned)c < (unsigned)a.K && act[j]) {
            load_vec<T, V>(B + (int64_t)c * a.N + col0 + j * V, bq[j], keep);
          } else {
            #pragma unroll
            for (int i = 0; i < V; i++) bq[j][i] = 0.f;
          }
        }
        if (p >= next_start) {  // the walk left row cur
          if (open) flush_done(cur);
          int ns;
          do {
            cur++;
            ns = wget(cur + 1);
            if (ns <= p && !a.accumulate) zero_rows<TC, V, NV>(a, cur, cur, col0, act, strm);
          } while (ns <= p && cur < a.M - 1);
          next_start = ns;
          kah = next_start - wget(cur) > a.kahan;
        }
        const float v = ones ? 1.f : Elem<T>::to_f(sval[q]);
        add_row<V, NV>(acc, comp, v, bq, kah);
        open = true;
      }
      // close a row that ends exactly at the tile end; the next tile zeroes
      // any empty rows that follow it
      if (next_start == last + 1) {
        flush_done(cur);
        open = false;
      }
    }
    __syncwarp(mask);
    if (s + 2 < nst)
      stage_issue<T, false>(a, st, L, b, sb + 2 * L.S, min(L.S, ci.ce - sb - 2 * L.S), lane, G, mask, strm);
  }
  // the last row continues past the chunk: head slot or tail slot
  const bool tail = open && cur != head;
  if (open) {
    float *slot = (cur == head ? a.carry_vals : a.tail_vals) + (int64_t)chunk * a.N + col0;
    #pragma unroll
    for (int j = 0; j < NV; j++)
      if (act[j]) store_vec<float, V>(slot + j * V, acc[j], strm);
  }
  if (!a.accumulate && ci.ce >= a.nnz) zero_rows<TC, V, NV>(a, cur + 1, a.M - 1, col0, act, strm);
  // the head row's partial was stored (at its end, or just above): count
  // this chunk in for the head row and, when it has one, the tail row
  if (head >= 0) carry_arrive<TC, V, NV>(a, head, lane, G, mask, col0, act, strm);
  if (tail) carry_arrive<TC, V, NV>(a, cur, lane, G, mask, col0, act, strm);
  return true;
}

// Walks nonzeros [cs, ce) as work item `chunk`.  Element-balanced items are
// chunk * a.chunk onwards; a row-balanced item (batched) starts and ends on
// row boundaries, so no row straddles it.  The first two tiles are issued,
// the first row searched and the indptr window filled from the row before
// it (which holds cs when the chunk starts inside a row).  Returns false
// when a bounded wait expired.
template <typename T, typename TC, int V, int NV>
__device__ __forceinline__ bool sr_spmm_chunk(const EbArgs &a, int chunk, int cs, int ce, int lane, unsigned mask,
                                              Stage &st, const SrLayout &L, int col0, const bool (&act)[NV],
                                              uint64_t keep, uint64_t strm) {
  const int G = a.team_lanes;
  const int nst = (ce - cs + L.S - 1) / L.S;
  stage_issue<T, false>(a, st, L, 0, cs, min(L.S, ce - cs), lane, G, mask, strm);
  if (nst > 1) stage_issue<T, false>(a, st, L, 1, cs + L.S, min(L.S, ce - cs - L.S), lane, G, mask, strm);
  const int lb = group_lower_bound(a.indptr, a.M, cs, lane, G, mask);
  const int base = lb > 0 ? lb - 1 : 0;
  __syncwarp(mask);
  for (int i = lane; i < L.W; i += G) st.win[i] = __ldg(a.indptr + min(base + i, a.M));
  __syncwarp(mask);
  return sr_spmm_walk<T, TC, V, NV>(a, chunk, cs, ce, nst, lb, base, lane, mask, st, L, col0, act, keep, strm);
}

// ---------------------------------------------------------------------
// segment_coo chunk walk: segment ids come from the staged sorted index,
// src rows are streamed in order
// ---------------------------------------------------------------------
// Returns false when a bounded wait expired (the caller then stops).
template <typename T, int V, int NV, bool KAHAN>
__device__ __forceinline__ bool sr_seg_chunk(const EbArgs &a, int chunk, int lane, unsigned mask, Stage &st,
                                             const SrLayout &L, int col0, const bool (&act)[NV], uint64_t strm) {
  const T *__restrict__ src = (const T *)a.B;
  const int G = a.team_lanes;
  const bool is_max = a.reduce == SS_MAX;
  const float ident = is_max ? -INFINITY : 0.f;
  ChunkInfo ci;
  ci.cs = chunk * a.chunk;
  ci.ce = min(ci.cs + a.chunk, a.nnz);
  const int nst = (ci.ce - ci.cs + L.S - 1) / L.S;
  stage_issue<T, true>(a, st, L, 0, ci.cs, min(L.S, ci.ce - ci.cs), lane, G, mask, strm);
  if (nst > 1) stage_issue<T, true>(a, st, L, 1, ci.cs + L.S, min(L.S, ci.ce - ci.cs - L.S), lane, G, mask, strm);
  ci.r_first = __ldg(a.index + ci.cs);
  ci.r_last = ci.r_first;
  ci.prev_row = ci.cs > 0 ? __ldg(a.index + ci.cs - 1) : -1;
  ci.has_head = ci.cs > 0 && ci.prev_row == ci.r_first;
  const int head = ci.has_head ? ci.r_first : -1;
  // chunk-boundary probes for the carry assembly at the end, in flight now
  const int probe_back = head >= 0 ? seg_probe_back(a, chunk, lane) : INT_MIN;
  const int probe_fwd = seg_probe_fwd(a, chunk, lane);
  if (!a.accumulate && !ci.has_head)
    zero_rows<float, V, NV>(a, ci.prev_row + 1, ci.r_first - 1, col0, act, strm);

  int cur = ci.r_first;
  int cnt = 0;
  int head_n = 0;  // elements of the head segment in this chunk
  float acc[NV][V], comp[NV][V];
  #pragma unroll
  for (int j = 0; j < NV; j++)
    #pragma unroll
    for (int i = 0; i < V; i++) { acc[j][i] = ident; comp[j][i] = 0.f; }

  for (int s = 0; s < nst; s++) {
    const int b = s & 1;
    const int sb = ci.cs + s * L.S;
    const int n = min(L.S, ci.ce - sb);
    if (!stage_wait(st, b, mask, a.err)) {
      stage_drain(st, s, min(nst, s + 2), mask);  // tiles s and s + 1 may still be landing
      return false;
    }
    const int32_t *sidx = st.col + b * L.S;
    for (int q = 0; q < n; q += SR_U) {
      float bv[SR_U][NV][V];
      #pragma unroll
      for (int u = 0; u < SR_U; u++) {
        const bool live = q + u < n;
        #pragma unroll
        for (int j = 0; j < NV; j++) {
          if (live && act[j]) {
            load_vec<T, V>(src + (int64_t)(sb + q + u) * a.N + col0 + j * V, bv[u][j], strm);
          } else {
            #pragma unroll
            for (int i = 0; i < V; i++) bv[u][j][i] = 0.f;
          }
        }
      }
      #pragma unroll
      for (int u = 0; u < SR_U; u++) {
        if (q + u >= n) break;
        const int r = sidx[q + u];
        if (r != cur) {
          flush_row<float, V, NV>(a, ci, chunk, cur, acc, cnt, true, col0, act, strm);
          if (cur == head) head_n = cnt;
          if (!a.accumulate) zero_rows<float, V, NV>(a, cur + 1, r - 1, col0, act, strm);
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
            if (is_max) acc[j][i] = fmaxf(acc[j][i], bv[u][j][i]);
            else if (KAHAN) kahan_add(acc[j][i], comp[j][i], bv[u][j][i]);
            else acc[j][i] += bv[u][j][i];
          }
      }
    }
    if (s + 2 < nst)
      stage_issue<T, true>(a, st, L, b, sb + 2 * L.S, min(L.S, ci.ce - sb - 2 * L.S), lane, G, mask, strm);
  }
  const bool complete = ci.ce >= a.nnz || __ldg(a.index + ci.ce) != cur;
  flush_row<float, V, NV>(a, ci, chunk, cur, acc, cnt, complete, col0, act, strm);
  if (cur == head) head_n = cnt;
  if (!a.accumulate && ci.ce >= a.nnz) zero_rows<float, V, NV>(a, cur + 1, a.M - 1, col0, act, strm);
  // straddling segments: count this chunk in (head, then a tail that
  // continues), the last participant of each stores it
  const bool tail = !complete && cur != head;
  const bool mean = a.reduce == SS_MEAN;
  if (head >= 0 && (unsigned)head < (unsigned)a.M) {
    const int o = seg_owner(a, head, chunk, probe_back, lane, G, mask);
    const int l = seg_last(a, head, chunk, probe_fwd, lane, G, mask);
    // every column tile writes the count (the same value): the last arriver
    // of any tile may read it
    if (mean && l == chunk && lane == 0) a.seg_cnt[a.num_chunks + chunk] = head_n;
    seg_carry_arrive<V, NV>(a, head, o, l, lane, G, mask, col0, act, strm);
  }
  if (tail && (unsigned)cur < (unsigned)a.M) {
    const int l = seg_last(a, cur, chunk, probe_fwd, lane, G, mask);
    if (mean && lane == 0) a.seg_cnt[chunk] = cnt;
    seg_carry_arrive<V, NV>(a, cur, chunk, l, lane, G, mask, col0, act, strm);
  }
  return true;
}

template <typename T, typename TC, int V, int NV, bool SEG>
__global__ void __launch_bounds__(512, SS_SR_MIN_BLOCKS) eb_sr_kernel(EbArgs a) {
  extern __shared__ __align__(16) char smem_raw[];
  const int tid = threadIdx.x;
  const int G = a.team_lanes;
  const int lane = tid & (G - 1);
  const int wib = tid >> a.log2_team_lanes;
  const unsigned wl = tid & 31;
  const unsigned mask = G >= 32 ? 0xffffffffu : (((1u << G) - 1u) << (wl & ~(unsigned)(G - 1)));
  const SrLayout L = sr_layout(a.stage, SEG ? 0 : (int)sizeof(T));
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
  const int col0 = blockIdx.y * a.col_tile + lane * (V * NV);
  bool act[NV];
  #pragma unroll
  for (int j = 0; j < NV; j++) act[j] = col0 + j * V < a.N;
  const uint64_t keep = policy_keep(a.keep_frac), strm = policy_stream();
  const bool kahan = a.chunk > a.kahan;  // segments: compensated within a chunk longer than the threshold
  const int stride = gridDim.x * a.workers_per_block;
  for (int chunk = blockIdx.x * a.workers_per_block + wib; chunk < a.num_chunks; chunk += stride) {
    bool ok;
    if (SEG) {
      ok = kahan ? sr_seg_chunk<T, V, NV, true>(a, chunk, lane, mask, st, L, col0, act, strm)
                 : sr_seg_chunk<T, V, NV, false>(a, chunk, lane, mask, st, L, col0, act, strm);
    } else {
      const int cs = chunk * a.chunk;
      ok = sr_spmm_chunk<T, TC, V, NV>(a, chunk, cs, min(cs + a.chunk, a.nnz), lane, mask, st, L, col0, act,
                                       keep, strm);
    }
    // a bounded wait expired: the group waited again for its copies in
    // flight and issues nothing more into its buffers
    if (!ok) break;
  }
  // every issued stage was waited for: no bulk copy is in flight here
}

template <typename T, typename TC, bool SEG>
inline void *sr_ptr(int V, int NV) {
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

// Kernel tables, one translation unit per storage type (eb_walk_*.cu).
void *sr_kernel_f32(int V, int NV, bool seg);
void *sr_kernel_f32_c16(int V, int NV, int c_dtype);  // FP32 inputs, BF16/FP16 C (SpMM)
void *sr_kernel_bf16(int V, int NV, bool seg, bool out_f32);
void *sr_kernel_f16(int V, int NV, bool seg, bool out_f32);

}  // namespace ss
