// Row-balanced SpMM: rbsr (sequential reduction) and rbpr (parallel
// reduction).  C (=|+=) A * B with every row owned by exactly one team, so
// rows are written with plain vector stores, no atomics and no zero fill.
//
// Reference counterparts: csrspmm_seqreduce_rowbalance_cg_kernel and
// csrspmm_parreduce_rowbalance_cg_kernel (test-cg/include/spmm/
// spmm_cg.cuh:593-662 and :220-331).  The knob -> geometry formulas of their
// launchers are kept (abi.cu); inside a team the lanes run along N so each
// gathered B row is one contiguous, vectorised request.
#include <algorithm>

#include "common.cuh"
#include "internal.h"

namespace ss {

struct RbArgs {
  int M, K, N, nnz;
  const int32_t *indptr, *indices;
  const void *vals, *B;
  void *C;
  int accumulate, kahan;
  int lanes, log2_lanes;   // column lanes per slot
  int col_tile;
  int tiles;               // column tiles (rbpr: the fastest-varying part of blockIdx.x)
  int slots, log2_slots;   // nonzero slots per team (1 for rbsr)
  int team_threads, log2_team;
  int teams_per_block;
  float keep_frac;  // fraction of B's lines kept in L2 (evict_last)
};

// rbpr numbers its blocks row block major, column tile minor, so the column
// tiles of the same rows run at the same time and share the B rows they
// gather in L2; a 2-D grid (tiles on y) runs every row block of tile 0
// first and fetches each B row from DRAM once per tile.  At the reference's
// rbpr tuple (8 tiles of 8 columns) this is 9-12 % faster on the power-law
// and banded matrices.  rbsr keeps the 2-D grid: its tiles are wide (one
// or two for N <= 64) and the 1-D form measured 8-31 % slower there.
struct RbBlock {
  int tile, row0, stride;
};
__device__ __forceinline__ RbBlock rb_block(const RbArgs &a) {
  RbBlock b;
  const int rb = blockIdx.x / a.tiles;
  b.tile = blockIdx.x - rb * a.tiles;
  b.row0 = rb * a.teams_per_block;
  b.stride = (gridDim.x / a.tiles) * a.teams_per_block;
  return b;
}

template <int V, int NV> struct Acc {
  float v[NV][V];
  __device__ __forceinline__ void zero() {
    #pragma unroll
    for (int j = 0; j < NV; j++)
      #pragma unroll
      for (int i = 0; i < V; i++) v[j][i] = 0.f;
  }
};

__device__ __forceinline__ void clamp_row(const RbArgs &a, int row, int &s, int &e) {
  s = __ldg(a.indptr + row);
  e = __ldg(a.indptr + row + 1);
  s = max(0, min(s, a.nnz));
  e = max(s, min(e, a.nnz));
}

template <typename TC, int V, int NV>
__device__ __forceinline__ void store_row(const RbArgs &a, int row, int col0, const bool (&act)[NV],
                                          Acc<V, NV> &acc, uint64_t pol) {
  TC *C = (TC *)a.C;
  #pragma unroll
  for (int j = 0; j < NV; j++) {
    if (!act[j]) continue;
    TC *dst = C + (int64_t)row * a.N + col0 + j * V;
    if (a.accumulate) {
      float prev[V];
      load_out<TC, V>(dst, prev);
      #pragma unroll
      for (int i = 0; i < V; i++) acc.v[j][i] += prev[i];
    }
    store_vec<TC, V>(dst, acc.v[j], pol);
  }
}

// ---------------------------------------------------------------------
// rbsr: one team of `lanes` lanes per (row, column tile).  The team loads
// `lanes` (column, value) pairs of the row at once (coalesced), then walks
// them in order, broadcasting each pair by shuffle and gathering four B rows
// ahead of the multiply-adds.
// ---------------------------------------------------------------------
template <typename T, typename TC, int V, int NV, bool KAHAN>
__device__ __forceinline__ void rbsr_row(const RbArgs &a, int s, int e, int lane, unsigned mask, int col0,
                                         const bool (&act)[NV], Acc<V, NV> &acc, uint64_t keep,
                                         uint64_t strm) {
  const T *__restrict__ B = (const T *)a.B;
  const T *__restrict__ vals = (const T *)a.vals;
  const int L = a.lanes;
  Acc<V, NV> comp;
  comp.zero();
  for (int base = s; base < e; base += L) {
    const int p = base + lane;
    int mc = 0;
    float mv = 0.f;
    if (p < e) {
      mc = ld_idx(a.indices + p, strm);
      mv = load_val<T>(vals, p, strm);
      if ((unsigned)mc >= (unsigned)a.K) { mc = 0; mv = 0.f; }
    }
    const int cnt = min(L, e - base);
    for (int q = 0; q < cnt; q += 4) {
      int c[4];
      float v[4];
      float b[4][NV][V];
      #pragma unroll
      for (int u = 0; u < 4; u++) {
        c[u] = __shfl_sync(mask, mc, q + u, L);
        v[u] = __shfl_sync(mask, mv, q + u, L);
      }
      #pragma unroll
      for (int u = 0; u < 4; u++) {
        const bool live = q + u < cnt;
        #pragma unroll
        for (int j = 0; j < NV; j++) {
          if (live && act[j]) {
            load_vec<T, V>(B + (int64_t)c[u] * a.N + col0 + j * V, b[u][j], keep);
          } else {
            #pragma unroll
            for (int i = 0; i < V; i++) b[u][j][i] = 0.f;
          }
        }
        if (!live) v[u] = 0.f;
      }
      // a compensated step of a zero term is not a no-op (it can fold the
      // correction in early): slots past the row end are skipped there
      #pragma unroll
      for (int u = 0; u < 4; u++)
        #pragma unroll
        for (int j = 0; j < NV; j++)
          #pragma unroll
          for (int i = 0; i < V; i++) {
            if (KAHAN) {
              if (q + u < cnt) kahan_fma(acc.v[j][i], comp.v[j][i], v[u], b[u][j][i]);
            } else {
              acc.v[j][i] = fmaf(v[u], b[u][j][i], acc.v[j][i]);
            }
          }
    }
  }
}

template <typename T, typename TC, int V, int NV>
__global__ void __launch_bounds__(1024) rbsr_kernel(RbArgs a) {
  const int tid = threadIdx.x;
  const int lane = tid & (a.lanes - 1);
  const int team = tid >> a.log2_lanes;
  const unsigned wl = tid & 31;
  const unsigned mask = a.lanes >= 32 ? 0xffffffffu
                                      : (((1u << a.lanes) - 1u) << (wl & ~(unsigned)(a.lanes - 1)));
  const int col0 = blockIdx.y * a.col_tile + lane * (V * NV);
  bool act[NV];
  #pragma unroll
  for (int j = 0; j < NV; j++) act[j] = col0 + j * V < a.N;
  const uint64_t keep = policy_keep(a.keep_frac), strm = policy_stream();
  const int stride = gridDim.x * a.teams_per_block;
  for (int row = blockIdx.x * a.teams_per_block + team; row < a.M; row += stride) {
    int s, e;
    clamp_row(a, row, s, e);
    Acc<V, NV> acc;
    acc.zero();
    if (e - s > a.kahan) rbsr_row<T, TC, V, NV, true>(a, s, e, lane, mask, col0, act, acc, keep, strm);
    else rbsr_row<T, TC, V, NV, false>(a, s, e, lane, mask, col0, act, acc, keep, strm);
    store_row<TC, V, NV>(a, row, col0, act, acc, strm);
  }
}

// ---------------------------------------------------------------------
// rbpr: one team of slots x lanes threads per (row, column tile).  Slot s
// accumulates nonzeros s, s + slots, ... of the row; the slots are then
// reduced by a butterfly of shuffles (and, when the team spans several
// warps, through shared memory), and one slot stores the row.
// ---------------------------------------------------------------------
template <typename T, int V, int NV, bool KAHAN>
__device__ __forceinline__ void rbpr_slot(const RbArgs &a, int s, int e, int slot, int col0,
                                          const bool (&act)[NV], Acc<V, NV> &acc, uint64_t keep,
                                          uint64_t strm) {
  const T *__restrict__ B = (const T *)a.B;
  const T *__restrict__ vals = (const T *)a.vals;
  const int S = a.slots;
  Acc<V, NV> comp;
  comp.zero();
  // four nonzeros per slot per step: their indices and values are loaded
  // together, then their four B rows, so a long row costs two dependent
  // round trips per four of its nonzeros on each slot
  constexpr int U = 4;
  // the next step's columns and values are loaded while this step's B rows
  // are in flight: one dependent round trip per step on a long row
  int cn[U];
  float vn[U];
  #pragma unroll
  for (int u = 0; u < U; u++) {
    const int p = s + slot + u * S;
    cn[u] = -1;
    vn[u] = 0.f;
    if (p < e) {
      cn[u] = ld_idx(a.indices + p, strm);
      vn[u] = load_val<T>(vals, p, strm);
    }
  }
  for (int p0 = s + slot; p0 < e; p0 += U * S) {
    int c[U];
    float v[U];
    float b[U][NV][V];
    #pragma unroll
    for (int u = 0; u < U; u++) {
      c[u] = cn[u];
      v[u] = vn[u];
      if ((unsigned)c[u] >= (unsigned)a.K) { c[u] = -1; v[u] = 0.f; }  // past the row, or a bad column
      #pragma unroll
      for (int j = 0; j < NV; j++) {
        if (c[u] >= 0 && act[j]) {
          load_vec<T, V>(B + (int64_t)c[u] * a.N + col0 + j * V, b[u][j], keep);
        } else {
          #pragma unroll
          for (int i = 0; i < V; i++) b[u][j][i] = 0.f;
        }
      }
    }
    #pragma unroll
    for (int u = 0; u < U; u++) {
      const int p = p0 + U * S + u * S;
      cn[u] = -1;
      vn[u] = 0.f;
      if (p < e) {
        cn[u] = ld_idx(a.indices + p, strm);
        vn[u] = load_val<T>(vals, p, strm);
      }
    }
    #pragma unroll
    for (int u = 0; u < U; u++)
      #pragma unroll
      for (int j = 0; j < NV; j++)
        #pragma unroll
        for (int i = 0; i < V; i++) {
          if (KAHAN) {
            if (p0 + u * S < e) kahan_fma(acc.v[j][i], comp.v[j][i], v[u], b[u][j][i]);  // not past the row
          } else {
            acc.v[j][i] = fmaf(v[u], b[u][j][i], acc.v[j][i]);
          }
        }
  }
}

template <typename T, typename TC, int V, int NV>
__global__ void __launch_bounds__(1024) rbpr_kernel(RbArgs a) {
  extern __shared__ float red[];  // [warps per block][lanes][V*NV], multi-warp teams only
  const int tid = threadIdx.x;
  const int t_in_team = tid & (a.team_threads - 1);
  const int team = tid >> a.log2_team;
  const int lane = t_in_team & (a.lanes - 1);
  const int slot = t_in_team >> a.log2_lanes;
  const unsigned wl = tid & 31;
  const int warp_threads = min(a.team_threads, 32);
  const unsigned wmask = warp_threads >= 32
                             ? 0xffffffffu
                             : (((1u << warp_threads) - 1u) << (wl & ~(unsigned)(warp_threads - 1)));
  const RbBlock blk = rb_block(a);
  const int col0 = blk.tile * a.col_tile + lane * (V * NV);
  bool act[NV];
  #pragma unroll
  for (int j = 0; j < NV; j++) act[j] = col0 + j * V < a.N;
  const uint64_t keep = policy_keep(a.keep_frac), strm = policy_stream();
  // warps a team spans; 0 when the team fits in one warp (no shared memory then)
  const int warps_in_team = a.team_threads > 32 ? a.team_threads >> 5 : 0;
  for (int row = blk.row0 + team; row < a.M; row += blk.stride) {
    int s, e;
    clamp_row(a, row, s, e);
    Acc<V, NV> acc;
    acc.zero();
    if (e - s > a.kahan) rbpr_slot<T, V, NV, true>(a, s, e, slot, col0, act, acc, keep, strm);
    else rbpr_slot<T, V, NV, false>(a, s, e, slot, col0, act, acc, keep, strm);
    // butterfly over the slots held by this warp
    for (int off = a.lanes; off < warp_threads; off <<= 1)
      #pragma unroll
      for (int j = 0; j < NV; j++)
        #pragma unroll
        for (int i = 0; i < V; i++) acc.v[j][i] += __shfl_xor_sync(wmask, acc.v[j][i], off);
    if (warps_in_team == 0) {
      if (slot == 0) store_row<TC, V, NV>(a, row, col0, act, acc, strm);
    } else {
      // team spans several warps: warp partials through shared memory
      const int w_in_team = t_in_team >> 5;
      const int first_warp = (team * a.team_threads) >> 5;
      constexpr int E = V * NV;
      if ((t_in_team & 31) < a.lanes) {
        float *dst = red + ((size_t)(first_warp + w_in_team) * a.lanes + lane) * E;
        #pragma unroll
        for (int j = 0; j < NV; j++)
          #pragma unroll
          for (int i = 0; i < V; i++) dst[j * V + i] = acc.v[j][i];
      }
      asm volatile("bar.sync %0, %1;" ::"r"(team), "r"(a.team_threads) : "memory");
      if (t_in_team < a.lanes) {
        for (int w = 1; w < warps_in_team; w++) {
          const float *src = red + ((size_t)(first_warp + w) * a.lanes + lane) * E;
          #pragma unroll
          for (int j = 0; j < NV; j++)
            #pragma unroll
            for (int i = 0; i < V; i++) acc.v[j][i] += src[j * V + i];
        }
        store_row<TC, V, NV>(a, row, col0, act, acc, strm);
      }
      asm volatile("bar.sync %0, %1;" ::"r"(team), "r"(a.team_threads) : "memory");
    }
  }
}

// ---------------------------------------------------------------------
// Launchers
// ---------------------------------------------------------------------
static RbArgs make_args(const SpmmCall &c, const RbGeom &g) {
  RbArgs a;
  a.M = c.M; a.K = c.K; a.N = c.N; a.nnz = c.nnz;
  a.indptr = c.indptr; a.indices = c.indices; a.vals = c.vals; a.B = c.B; a.C = c.C;
  a.accumulate = c.accumulate; a.kahan = c.kahan_threshold;
  a.lanes = g.cs.lanes; a.log2_lanes = ilog2(g.cs.lanes);
  a.col_tile = g.cs.col_tile;
  a.tiles = g.cs.tiles;
  a.slots = g.slots; a.log2_slots = ilog2(g.slots);
  a.team_threads = g.team_threads; a.log2_team = ilog2(g.team_threads);
  a.teams_per_block = g.teams_per_block;
  a.keep_frac = l2_keep_fraction((size_t)c.K * c.N * dtype_size(c.val_dtype));
  return a;
}

#define SS_RB_KERNEL_TABLE(NAME)                                                        \
  template <typename T, typename TC>                                                    \
  static void *NAME##_ptr(int V, int NV) {                                              \
    if (NV == 1) {                                                                      \
      if (V == 1) return (void *)NAME##_kernel<T, TC, 1, 1>;                            \
      if (V == 2) return (void *)NAME##_kernel<T, TC, 2, 1>;                            \
      if (V == 4) return (void *)NAME##_kernel<T, TC, 4, 1>;                            \
      if constexpr (sizeof(T) == 2) if (V == 8) return (void *)NAME##_kernel<T, TC, 8, 1>; \
    } else {                                                                            \
      if (V == 1) return (void *)NAME##_kernel<T, TC, 1, 2>;                            \
      if (V == 2) return (void *)NAME##_kernel<T, TC, 2, 2>;                            \
      if (V == 4) return (void *)NAME##_kernel<T, TC, 4, 2>;                            \
      if constexpr (sizeof(T) == 2) if (V == 8) return (void *)NAME##_kernel<T, TC, 8, 2>; \
    }                                                                                   \
    return nullptr;                                                                     \
  }

SS_RB_KERNEL_TABLE(rbsr)
SS_RB_KERNEL_TABLE(rbpr)

static void *pick_rb(bool pr, int dt, int cdt, int V, int NV) {
  if (dt == SS_F32) return pr ? rbpr_ptr<float, float>(V, NV) : rbsr_ptr<float, float>(V, NV);
  if (dt == SS_BF16) {
    if (cdt == SS_F32) return pr ? rbpr_ptr<__nv_bfloat16, float>(V, NV) : rbsr_ptr<__nv_bfloat16, float>(V, NV);
    return pr ? rbpr_ptr<__nv_bfloat16, __nv_bfloat16>(V, NV) : rbsr_ptr<__nv_bfloat16, __nv_bfloat16>(V, NV);
  }
  if (cdt == SS_F32) return pr ? rbpr_ptr<__half, float>(V, NV) : rbsr_ptr<__half, float>(V, NV);
  return pr ? rbpr_ptr<__half, __half>(V, NV) : rbsr_ptr<__half, __half>(V, NV);
}

static ss_status launch_rb(bool pr, const SpmmCall &c, const RbGeom &g, cudaStream_t s) {
  if (c.M == 0 || c.N == 0) return SS_OK;
  void *fn = pick_rb(pr, c.val_dtype, c.c_dtype, g.cs.V, g.cs.NV);
  if (!fn) return fail(SS_ERR_UNSUPPORTED_KNOBS, "no %s kernel for V=%d NV=%d", pr ? "rbpr" : "rbsr", g.cs.V, g.cs.NV);
  RbArgs a = make_args(c, g);
  size_t smem = 0;
  if (pr && g.team_threads > 32) smem = (size_t)(g.block / 32) * g.cs.lanes * g.cs.V * g.cs.NV * sizeof(float);
  dim3 grid(g.grid_x, g.cs.tiles, 1), block(g.block, 1, 1);
  if (pr) {
    const long long row_blocks = std::min<long long>(g.grid_x, 0x7fffffffLL / g.cs.tiles);
    grid = dim3((unsigned)(row_blocks * g.cs.tiles), 1, 1);
  }
  void *args[] = {&a};
  cudaError_t err = cudaLaunchKernel(fn, grid, block, args, smem, s);
  if (err != cudaSuccess) return cuda_fail(err, pr ? "rbpr launch" : "rbsr launch");
  return SS_OK;
}

ss_status launch_rbsr(const SpmmCall &c, const RbGeom &g, cudaStream_t s) { return launch_rb(false, c, g, s); }
ss_status launch_rbpr(const SpmmCall &c, const RbGeom &g, cudaStream_t s) { return launch_rb(true, c, g, s); }

}  // namespace ss
