// ebsr SpMM walk with B rows gathered by the tensor memory accelerator.
//
// The register walk (eb_walk.cuh) gathers four B rows per group into
// registers and then waits for them.  Loads into registers sustain fewer
// random rows per second on this GPU than copies into shared memory at the
// same depth (bench_gather_ceiling.cu: 18.7 against 33 G rows/s for 256-byte
// rows), and per-lane cp.async rings cost the walk more issue slots than
// they save.  Here one lane of a group issues a `cp.async.bulk.tensor`
// `tile::gather4`: four rows of B (the group's column slice of each, one
// tensor-map box {col_tile, 1} per row) land in a shared-memory ring slot and
// complete on that slot's mbarrier.  The ring has G4_R slots, so 4 * G4_R
// rows are in flight per group while the group walks the oldest slot.
//
// Everything else is the register walk: A's column and value streams staged
// by bulk copies, tiles labelled with rows and end bits, long rows
// compensated, owner stores, head/tail slots and the in-walk assembly of
// straddling rows.  A column outside [0, K) is a tensor coordinate out of
// range, which the copy fills with zeros, as the register walk zeroes it.
// Waits are bounded; on expiry the group records SS_ERR_TIMEOUT, waits
// (bounded) for its copies in flight and stops.
//
// Used for SpMM when a lane's share of a row is one or two 16-byte vectors
// (FP32 V = 4, 16-bit V = 8) and B's rows are 16-byte aligned; a one-lane
// group, segment_coo and batched launches keep the register walk.
#pragma once
#include <cuda.h>

#include "eb_walk.cuh"

namespace ss {

constexpr int G4_R = 4;  // ring slots (four rows each) per group

struct G4Args {
  CUtensorMap tmap;  // B as a 2-D tensor {N, K}, box {col_tile, 1}
  EbArgs a;
};

// Per-group shared memory: [ring slots | ring mbarriers (64 B) | staging (SrLayout)].
__host__ __device__ inline int g4_ring_bytes(int col_tile, int es) { return G4_R * 4 * col_tile * es; }
__host__ __device__ inline int g4_worker_bytes(int stage, int es, int col_tile) {
  return (g4_ring_bytes(col_tile, es) + 64 + sr_layout(stage, es).bytes + 127) & ~127;
}

struct G4Ring {
  char *slots;      // [G4_R][4 rows][col_tile elements]
  uint64_t *bar;    // [G4_R]
  uint32_t phases;  // bit r: parity to wait for on bar[r]
  int row_bytes;    // col_tile * sizeof(T)
};

// Four rows y0..y3 of the tensor map's box at column x, stored back to back
// at dst; one thread issues it, completion on bar.
__device__ __forceinline__ void tma_gather4(void *dst, const CUtensorMap *tmap, int x, int y0, int y1, int y2, int y3,
                                            uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile::gather4.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3, %4, %5, %6}], [%7];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(tmap)), "r"(x), "r"(y0), "r"(y1), "r"(y2), "r"(y3), "r"(smem_u32(bar))
      : "memory");
}

// This lane's NV x V elements of row u of a ring slot, widened to FP32.
template <typename T, int V, int NV>
__device__ __forceinline__ void ring_row(const char *slot, int row_bytes, int u, int lane, float (&out)[NV][V]) {
  const uint4 *p = reinterpret_cast<const uint4 *>(slot + u * row_bytes + lane * (V * NV * (int)sizeof(T)));
  #pragma unroll
  for (int j = 0; j < NV; j++) {
    const uint4 w = p[j];
    if constexpr (sizeof(T) == 4) {
      out[j][0] = __uint_as_float(w.x); out[j][1] = __uint_as_float(w.y);
      out[j][2] = __uint_as_float(w.z); out[j][3] = __uint_as_float(w.w);
    } else {
      unpack2(w.x, out[j][0], out[j][1], (T *)nullptr); unpack2(w.y, out[j][2], out[j][3], (T *)nullptr);
      unpack2(w.z, out[j][4], out[j][5], (T *)nullptr); unpack2(w.w, out[j][6], out[j][7], (T *)nullptr);
    }
  }
}

// Walks nonzeros [cs, ce) as work item `chunk`; see sr_spmm_walk for the
// row bookkeeping, which is the same.  Groups of four nonzeros (g = 0 ..
// ng - 1 from cs) are gathered in order into slot g % G4_R, G4_R groups
// ahead of the one being walked.
template <typename T, typename TC, int V, int NV>
__device__ __forceinline__ bool sr_spmm_walk_g4(const EbArgs &a, const CUtensorMap *tmap, int chunk, int cs, int ce,
                                                int lane, unsigned mask, Stage &st, const SrLayout &L, G4Ring &rg,
                                                int x0, int col0, const bool (&act)[NV], uint64_t strm) {
  const int G = a.team_lanes;
  const bool ones = a.vals == nullptr;
  const int nst = (ce - cs + L.S - 1) / L.S;
  const int ng = (ce - cs + 3) >> 2;
  const int gpt = L.S >> 2;  // groups per staged tile
  int waited = 0;            // staged tiles waited for
  int staged = min(nst, 2);  // staged tiles issued
  int issued = 0;            // groups whose gather is issued
  stage_issue<T, false>(a, st, L, 0, cs, min(L.S, ce - cs), lane, G, mask, strm);
  if (nst > 1) stage_issue<T, false>(a, st, L, 1, cs + L.S, min(L.S, ce - cs - L.S), lane, G, mask, strm);

  // tile t's column stream has landed (tiles are waited for in order)
  auto tile_ready = [&](int t) -> bool {
    while (waited <= t) {
      if (!stage_wait(st, waited & 1, mask, a.err)) return false;
      waited++;
    }
    return true;
  };
  // gather of group g into slot g % G4_R, issued by lane 0 once its columns landed
  auto issue = [&](int g) -> bool {
    const int t = (g * 4) / L.S;
    if (!tile_ready(t)) return false;
    if (lane == 0) {
      const int32_t *scol = st.col + (t & 1) * L.S + (g * 4) % L.S;
      const int p = cs + g * 4;
      int c[4];
      #pragma unroll
      for (int u = 0; u < 4; u++) c[u] = p + u < ce ? scol[u] : -1;  // past the chunk: filled with zeros
      const int slot = g % G4_R;
      fence_async_smem();
      mbar_expect_tx(rg.bar + slot, 4u * (uint32_t)rg.row_bytes);
      tma_gather4(rg.slots + slot * 4 * rg.row_bytes, tmap, x0, c[0], c[1], c[2], c[3], rg.bar + slot);
    }
    issued = g + 1;
    return true;
  };
  // group g's rows have landed (the group agrees)
  auto acquire = [&](int g) -> bool {
    const int slot = g % G4_R;
    bool ok = true;
    uint32_t it = 0;
    while (!mbar_try_wait(rg.bar + slot, (rg.phases >> slot) & 1u)) {
      if (++it > SR_SPIN_LIMIT) {
        ok = false;
        break;
      }
    }
    ok = __all_sync(mask, ok);
    if (ok) rg.phases ^= 1u << slot;
    else if (a.err) atomicExch(a.err, (int)SS_ERR_TIMEOUT);
    return ok;
  };
  // group g is walked: its slot takes group g + G4_R
  auto release = [&](int g) -> bool {
    __syncwarp(mask);
    return g + G4_R < ng ? issue(g + G4_R) : true;
  };
  // after an expired wait: wait again, bounded, for every copy in flight
  auto drain = [&](int from_g) {
    for (int g = from_g; g < issued; g++) acquire(g);
    stage_drain(st, waited, staged, mask);
  };

  // first row and the indptr window (from the row before it)
  const int lb = group_lower_bound(a.indptr, a.M, cs, lane, G, mask);
  int win_base = lb > 0 ? lb - 1 : 0;
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
  win_fill(win_base);
  for (int g = 0; g < min(G4_R, ng); g++) {
    if (!issue(g)) {
      drain(0);
      return false;
    }
  }

  ChunkInfo ci;
  ci.cs = cs;
  ci.ce = ce;
  int cur;
  ci.has_head = lb > 0 && wget(lb) > ci.cs;
  if (ci.has_head) {
    cur = lb - 1;
  } else {
    cur = lb;
    while (cur < a.M - 1 && wget(cur + 1) <= ci.cs) {
      if (!a.accumulate) zero_rows<TC, V, NV>(a, cur, cur, col0, act, strm);
      cur++;
    }
  }
  const int head = ci.has_head ? cur : -1;

  bool open = false;
  float acc[NV][V], comp[NV][V];
  #pragma unroll
  for (int j = 0; j < NV; j++)
    #pragma unroll
    for (int i = 0; i < V; i++) { acc[j][i] = 0.f; comp[j][i] = 0.f; }
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
    const int g0 = s * gpt;
    if (!tile_ready(s)) {
      drain(g0);
      return false;
    }
    const T *sval = reinterpret_cast<const T *>(st.val + b * L.S * L.vs);
    int32_t *sinfo = st.info + b * L.S;
    if (cur < win_base || st.win[L.W - 1] <= last) win_fill(cur);
    const bool fast = st.win[L.W - 1] > last || win_base + L.W - 1 >= a.M;

    if (fast) {
      // ---- labels: row | end-of-row bit; long rows' nonzeros in kmask;
      // empty rows opened at a row start zeroed by the group
      const int c0 = cur - win_base;
      const int rounds = (n + G - 1) / G;
      uint64_t kmask = 0;
      for (int k = 0; k < rounds; k++) {
        const int e = lane + k * G;
        int zlo = 0, zhi = -1;
        bool kah = false;
        if (e < n) {
          const int p = sb + e;
          int lo = c0 + 1, hi = L.W - 1;
          while (lo < hi) {
            const int mid = (lo + hi) >> 1;
            if (st.win[mid] <= p) lo = mid + 1; else hi = mid;
          }
          const int rr = lo - 1;
          const bool end = st.win[rr + 1] == p + 1;
          kah = st.win[rr + 1] - st.win[rr] > a.kahan;
          sinfo[e] = (win_base + rr) | (end ? (int)0x80000000 : 0);
          if (st.win[rr] == p && p != ci.cs) {
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
      __syncwarp(mask);
      const bool full = n == L.S;
      const int4 *info4 = reinterpret_cast<const int4 *>(sinfo);
      for (int q = 0; q < n; q += 4) {
        const int g = g0 + (q >> 2);
        if (!acquire(g)) {
          drain(g);
          return false;
        }
        int is4[4];
        float v4[4];
        if (full) {
          const int4 in4 = info4[q >> 2];
          is4[0] = in4.x; is4[1] = in4.y; is4[2] = in4.z; is4[3] = in4.w;
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
        } else {
          #pragma unroll
          for (int u = 0; u < 4; u++) {
            is4[u] = q + u < n ? sinfo[q + u] : 0;
            v4[u] = q + u < n ? (ones ? 1.f : Elem<T>::to_f(sval[q + u])) : 0.f;
          }
        }
        const unsigned k4 = (unsigned)(kmask >> q) & 0xfu;
        const char *slot = rg.slots + (g % G4_R) * 4 * rg.row_bytes;
        #pragma unroll
        for (int u = 0; u < 4; u++) {
          if (q + u >= n) break;
          float bv[NV][V];
          ring_row<T, V, NV>(slot, rg.row_bytes, u, lane, bv);
          add_row<V, NV>(acc, comp, v4[u], bv, (k4 >> u) & 1u);
          cur = is4[u] & 0x7fffffff;
          open = true;
          if (is4[u] < 0) {
            flush_done(cur);
            open = false;
          }
        }
        if (!release(g)) {
          drain(g + 1);
          return false;
        }
      }
    } else {
      // ---- element by element (tiles crossing long runs of empty rows)
      int next_start = wget(cur + 1);
      if (!open) {
        while (cur < a.M - 1 && next_start <= sb) {
          cur++;
          next_start = wget(cur + 1);
          if (next_start <= sb && !a.accumulate) zero_rows<TC, V, NV>(a, cur, cur, col0, act, strm);
        }
      }
      bool kah = next_start - wget(cur) > a.kahan;
      for (int q0 = 0; q0 < n; q0 += 4) {
        const int g = g0 + (q0 >> 2);
        if (!acquire(g)) {
          drain(g);
          return false;
        }
        const char *slot = rg.slots + (g % G4_R) * 4 * rg.row_bytes;
        for (int u = 0; u < 4 && q0 + u < n; u++) {
          const int q = q0 + u;
          const int p = sb + q;
          float bq[NV][V];
          ring_row<T, V, NV>(slot, rg.row_bytes, u, lane, bq);
          if (p >= next_start) {
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
        if (!release(g)) {
          drain(g + 1);
          return false;
        }
      }
      if (next_start == last + 1) {
        flush_done(cur);
        open = false;
      }
    }
    __syncwarp(mask);
    if (s + 2 < nst) {
      stage_issue<T, false>(a, st, L, b, sb + 2 * L.S, min(L.S, ci.ce - sb - 2 * L.S), lane, G, mask, strm);
      staged = s + 3;
    }
  }
  const bool tail = open && cur != head;
  if (open) {
    float *slotp = (cur == head ? a.carry_vals : a.tail_vals) + (int64_t)chunk * a.N + col0;
    #pragma unroll
    for (int j = 0; j < NV; j++)
      if (act[j]) store_vec<float, V>(slotp + j * V, acc[j], strm);
  }
  if (!a.accumulate && ci.ce >= a.nnz) zero_rows<TC, V, NV>(a, cur + 1, a.M - 1, col0, act, strm);
  if (head >= 0) carry_arrive<TC, V, NV>(a, head, lane, G, mask, col0, act, strm);
  if (tail) carry_arrive<TC, V, NV>(a, cur, lane, G, mask, col0, act, strm);
  return true;
}

template <typename T, typename TC, int V, int NV>
__global__ void __launch_bounds__(512, 1) eb_g4_kernel(const __grid_constant__ G4Args p) {
  const EbArgs &a = p.a;
  extern __shared__ __align__(128) char smem_g4[];
  const int tid = threadIdx.x;
  const int G = a.team_lanes;
  const int lane = tid & (G - 1);
  const int wib = tid >> a.log2_team_lanes;
  const unsigned wl = tid & 31;
  const unsigned mask = G >= 32 ? 0xffffffffu : (((1u << G) - 1u) << (wl & ~(unsigned)(G - 1)));
  const SrLayout L = sr_layout(a.stage, (int)sizeof(T));
  const int ring = g4_ring_bytes(a.col_tile, (int)sizeof(T));
  char *g = smem_g4 + (size_t)wib * g4_worker_bytes(a.stage, (int)sizeof(T), a.col_tile);
  G4Ring rg;
  rg.slots = g;
  rg.bar = reinterpret_cast<uint64_t *>(g + ring);
  rg.phases = 0;
  rg.row_bytes = a.col_tile * (int)sizeof(T);
  char *sg = g + ring + 64;
  Stage st;
  st.bar = reinterpret_cast<uint64_t *>(sg);
  st.col = reinterpret_cast<int32_t *>(sg + L.col_off);
  st.val = sg + L.val_off;
  st.info = reinterpret_cast<int32_t *>(sg + L.info_off);
  st.win = reinterpret_cast<int32_t *>(sg + L.win_off);
  st.phases = 0;
  st.tma = 0;
  if (lane == 0) {
    mbar_init(st.bar, 1);
    mbar_init(st.bar + 1, 1);
    #pragma unroll
    for (int r = 0; r < G4_R; r++) mbar_init(rg.bar + r, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncwarp(mask);
  const int x0 = blockIdx.y * a.col_tile;
  const int col0 = x0 + lane * (V * NV);
  bool act[NV];
  #pragma unroll
  for (int j = 0; j < NV; j++) act[j] = col0 + j * V < a.N;
  const uint64_t strm = policy_stream();
  const int stride = gridDim.x * a.workers_per_block;
  for (int chunk = blockIdx.x * a.workers_per_block + wib; chunk < a.num_chunks; chunk += stride) {
    const int cs = chunk * a.chunk;
    if (!sr_spmm_walk_g4<T, TC, V, NV>(a, &p.tmap, chunk, cs, min(cs + a.chunk, a.nnz), lane, mask, st, L, rg, x0,
                                        col0, act, strm))
      break;  // a bounded wait expired: nothing of this group is in flight any more
  }
}

template <typename T, typename TC>
inline void *g4_ptr(int V, int NV) {
  constexpr int VV = 16 / (int)sizeof(T);  // one 16-byte vector per lane per j
  if (V != VV) return nullptr;
  if (NV == 1) return (void *)eb_g4_kernel<T, TC, VV, 1>;
  if (NV == 2) return (void *)eb_g4_kernel<T, TC, VV, 2>;
  return nullptr;
}

// Kernel tables (eb_walk_*.cu).
void *g4_kernel_f32(int V, int NV, int c_dtype);
void *g4_kernel_f32_c16(int V, int NV, int c_dtype);
void *g4_kernel_bf16(int V, int NV, bool out_f32);
void *g4_kernel_f16(int V, int NV, bool out_f32);

}  // namespace ss
