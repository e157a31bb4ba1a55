// ebsr with one lane per group (group_factor 0): the narrow-width walk.
//
// At small N a whole B row is one or two vectors of a single lane, so a
// group of lanes along N would idle; the reference's csrspmm_rowcaching_
// nnzbalance_cg (test-cg/include/spmm/spmm_cg.cuh:376-591) with group
// size 1 gives each thread its own run of nonzeros.  Here each lane walks
// its chunk alone, with no shared-memory staging: its columns and values
// are read eight at a time in 16-byte vectors (a lane's accesses are not
// coalesced with its neighbours', so fewer, wider ones keep the L1 off the
// critical path), their eight B rows are gathered together, and rows are
// followed along indptr from a single binary search at the chunk start.
// On the power-law 1e6 matrix this is 66 us at N = 4 (ebpr: 83 us, the
// group walk with one lane: 250 us) and 113 us at N = 8; from N = 16 the
// group walk is faster.  Rows that end in
// the chunk are stored once; the chunk's head and tail rows go to the slots
// and are assembled by carry_arrive as in the group walk, so the results
// have the same structure (owner stores, one rounding, no atomics on C).
// Empty rows are zeroed by the chunk in front of them (the rows after its
// last row, up to the next nonzero), and by chunk 0 before its first row.
#include "eb_common.cuh"
#include "internal.h"

namespace ss {

// Rows [lo, hi] of C zeroed by one lane (its V * NV columns).
template <typename TC, int V, int NV>
__device__ __forceinline__ void narrow_zero(const EbArgs &a, int lo, int hi, int col0, const bool (&act)[NV],
                                            uint64_t pol) {
  float z[V];
  #pragma unroll
  for (int i = 0; i < V; i++) z[i] = 0.f;
  TC *C = (TC *)a.C;
  for (int r = lo; r <= hi; r++)
    #pragma unroll
    for (int j = 0; j < NV; j++)
      if (act[j]) store_vec<TC, V>(C + (int64_t)r * a.N + col0 + j * V, z, pol);
}

// Row r, complete inside this chunk, stored by its owner.
template <typename TC, int V, int NV>
__device__ __forceinline__ void narrow_store(const EbArgs &a, int r, float (&acc)[NV][V], int col0,
                                             const bool (&act)[NV], uint64_t pol) {
  TC *C = (TC *)a.C;
  #pragma unroll
  for (int j = 0; j < NV; j++) {
    if (!act[j]) continue;
    TC *dst = C + (int64_t)r * a.N + col0 + j * V;
    if (a.accumulate) {
      float prev[V];
      load_out<TC, V>(dst, prev);
      #pragma unroll
      for (int i = 0; i < V; i++) acc[j][i] += prev[i];
    }
    store_vec<TC, V>(dst, acc[j], pol);
  }
}

__device__ __forceinline__ bool use_vec_streams(const EbArgs &a) {
  return (a.chunk % 8) == 0 && ((uintptr_t)a.cols & 15u) == 0 && ((uintptr_t)a.vals & 15u) == 0;
}

template <int V, int NV>
__device__ __forceinline__ void narrow_slot(float *slot, float (&acc)[NV][V], const bool (&act)[NV],
                                            uint64_t pol) {
  #pragma unroll
  for (int j = 0; j < NV; j++)
    if (act[j]) store_vec<float, V>(slot + j * V, acc[j], pol);
}

// Eight consecutive columns and values of A from p (16-byte vector loads
// when p and the arrays allow it; zero past `lim`).
template <typename T>
__device__ __forceinline__ void narrow_block(const EbArgs &a, int p, int lim, bool vec, int (&c)[8],
                                             float (&v)[8], uint64_t pol) {
  const T *vals = (const T *)a.vals;
  if (vec && p + 8 <= lim) {
    const uint4 c0 = ld_u128(a.cols + p, pol), c1 = ld_u128(a.cols + p + 4, pol);
    c[0] = (int)c0.x; c[1] = (int)c0.y; c[2] = (int)c0.z; c[3] = (int)c0.w;
    c[4] = (int)c1.x; c[5] = (int)c1.y; c[6] = (int)c1.z; c[7] = (int)c1.w;
    if (vals == nullptr) {
      #pragma unroll
      for (int u = 0; u < 8; u++) v[u] = 1.f;
    } else if constexpr (sizeof(T) == 4) {
      const uint4 v0 = ld_u128(vals + p, pol), v1 = ld_u128(vals + p + 4, pol);
      v[0] = __uint_as_float(v0.x); v[1] = __uint_as_float(v0.y);
      v[2] = __uint_as_float(v0.z); v[3] = __uint_as_float(v0.w);
      v[4] = __uint_as_float(v1.x); v[5] = __uint_as_float(v1.y);
      v[6] = __uint_as_float(v1.z); v[7] = __uint_as_float(v1.w);
    } else {
      load_vec<T, 8>(vals + p, v, pol);
    }
  } else {
    #pragma unroll
    for (int u = 0; u < 8; u++) {
      const bool live = p + u < lim;
      c[u] = live ? ld_idx(a.cols + p + u, pol) : 0;
      v[u] = live ? load_val<T>(vals, p + u, pol) : 0.f;
    }
  }
}

template <typename T, typename TC, int V, int NV>
__global__ void __launch_bounds__(512) eb_narrow_kernel(EbArgs a) {
  const T *__restrict__ B = (const T *)a.B;
  const int col0 = blockIdx.y * a.col_tile;
  bool act[NV];
  #pragma unroll
  for (int j = 0; j < NV; j++) act[j] = col0 + j * V < a.N;
  const uint64_t keep = policy_keep(a.keep_frac), strm = policy_stream();
  const unsigned self = 1u << (threadIdx.x & 31);
  // 16-byte loads of the column / value streams: chunks start on multiples
  // of 8 nonzeros, so every block of 8 is aligned when the arrays are
  const bool vec = use_vec_streams(a);
  const int stride = gridDim.x * blockDim.x;
  for (int chunk = blockIdx.x * blockDim.x + threadIdx.x; chunk < a.num_chunks; chunk += stride) {
    const int cs = chunk * a.chunk;
    const int ce = min(cs + a.chunk, a.nnz);
    int r = row_search(a.indptr, 1, a.M, cs);  // row of nonzero cs
    const int start = __ldg(a.indptr + r);
    const bool has_head = cs > 0 && start < cs;
    const int head = has_head ? r : -1;
    if (cs == 0 && !a.accumulate) narrow_zero<TC, V, NV>(a, 0, r - 1, col0, act, strm);
    int end = __ldg(a.indptr + r + 1);  // one past row r's last nonzero
    bool kahan = end - start > a.kahan;  // row r is compensated
    float acc[NV][V], comp[NV][V];
    #pragma unroll
    for (int j = 0; j < NV; j++)
      #pragma unroll
      for (int i = 0; i < V; i++) { acc[j][i] = 0.f; comp[j][i] = 0.f; }
    for (int pb = cs; pb < ce; pb += 8) {
      int c[8];
      float v[8];
      narrow_block<T>(a, pb, ce, vec, c, v, strm);
      float b[8][NV][V];
      #pragma unroll
      for (int u = 0; u < 8; u++) {
        const bool ok = pb + u < ce && (unsigned)c[u] < (unsigned)a.K;
        if (!ok) v[u] = 0.f;
        #pragma unroll
        for (int j = 0; j < NV; j++) {
          if (ok && act[j]) {
            load_vec<T, V>(B + (int64_t)c[u] * a.N + col0 + j * V, b[u][j], keep);
          } else {
            #pragma unroll
            for (int i = 0; i < V; i++) b[u][j][i] = 0.f;
          }
        }
      }
      #pragma unroll
      for (int u = 0; u < 8; u++) {
        const int p = pb + u;
        if (p >= ce) break;
        // rows that end before p: stored (an empty one as zero), then the
        // next row; the head row goes to the head slot
        while (p >= end) {
          if (r == head) narrow_slot<V, NV>(a.carry_vals + (int64_t)chunk * a.N + col0, acc, act, strm);
          else narrow_store<TC, V, NV>(a, r, acc, col0, act, strm);
          #pragma unroll
          for (int j = 0; j < NV; j++)
            #pragma unroll
            for (int i = 0; i < V; i++) { acc[j][i] = 0.f; comp[j][i] = 0.f; }
          r++;
          const int next = __ldg(a.indptr + r + 1);
          kahan = next - end > a.kahan;
          end = next;
        }
        #pragma unroll
        for (int j = 0; j < NV; j++)
          #pragma unroll
          for (int i = 0; i < V; i++) {
            if (kahan) kahan_fma(acc[j][i], comp[j][i], v[u], b[u][j][i]);
            else acc[j][i] = fmaf(v[u], b[u][j][i], acc[j][i]);
          }
      }
    }
    int tail = -1;
    if (end > ce) {  // row r continues past the chunk
      if (r == head) {
        narrow_slot<V, NV>(a.carry_vals + (int64_t)chunk * a.N + col0, acc, act, strm);
      } else {
        narrow_slot<V, NV>(a.tail_vals + (int64_t)chunk * a.N + col0, acc, act, strm);
        tail = r;
      }
    } else {  // row r ends with the chunk; the empty rows after it are zeroed here
      if (r == head) narrow_slot<V, NV>(a.carry_vals + (int64_t)chunk * a.N + col0, acc, act, strm);
      else narrow_store<TC, V, NV>(a, r, acc, col0, act, strm);
      while (r + 1 < a.M && __ldg(a.indptr + r + 2) == end) {
        r++;
        if (!a.accumulate) narrow_zero<TC, V, NV>(a, r, r, col0, act, strm);
      }
    }
    // straddling rows: count this chunk in; the last participant stores
    // (small chunks: a long row has hundreds of heads, so eight are loaded
    // at a time)
    if (head >= 0) carry_arrive<TC, V, NV, 8>(a, head, 0, 1, self, col0, act, strm);
    if (tail >= 0) carry_arrive<TC, V, NV, 8>(a, tail, 0, 1, self, col0, act, strm);
  }
}

template <typename T, typename TC>
static void *narrow_ptr(int V, int NV) {
  if (NV == 1) {
    if (V == 1) return (void *)eb_narrow_kernel<T, TC, 1, 1>;
    if (V == 2) return (void *)eb_narrow_kernel<T, TC, 2, 1>;
    if (V == 4) return (void *)eb_narrow_kernel<T, TC, 4, 1>;
    if constexpr (sizeof(T) == 2) if (V == 8) return (void *)eb_narrow_kernel<T, TC, 8, 1>;
  } else {
    if (V == 1) return (void *)eb_narrow_kernel<T, TC, 1, 2>;
    if (V == 2) return (void *)eb_narrow_kernel<T, TC, 2, 2>;
    if (V == 4) return (void *)eb_narrow_kernel<T, TC, 4, 2>;
    if constexpr (sizeof(T) == 2) if (V == 8) return (void *)eb_narrow_kernel<T, TC, 8, 2>;
  }
  return nullptr;
}

// The narrow kernel for the value / output types of an ebsr call, or null
// (then the group walk runs).
void *narrow_kernel(int val_dtype, int c_dtype, int V, int NV) {
  if (val_dtype == SS_F32) {
    if (c_dtype == SS_F32) return narrow_ptr<float, float>(V, NV);
    if (c_dtype == SS_BF16) return narrow_ptr<float, __nv_bfloat16>(V, NV);
    if (c_dtype == SS_F16) return narrow_ptr<float, __half>(V, NV);
    return nullptr;
  }
  if (val_dtype == SS_BF16)
    return c_dtype == SS_F32 ? narrow_ptr<__nv_bfloat16, float>(V, NV)
                             : narrow_ptr<__nv_bfloat16, __nv_bfloat16>(V, NV);
  return c_dtype == SS_F32 ? narrow_ptr<__half, float>(V, NV) : narrow_ptr<__half, __half>(V, NV);
}

}  // namespace ss
