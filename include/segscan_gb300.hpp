// segscan_gb300.hpp - C++ host interface with the reference's launcher
// templates, on top of the C ABI in segscan_gb300.h.
//
// zhang677/segScan's operator API is a set of templated host launchers that
// a driver instantiates per knob tuple (test-cg/include/spmm/spmm_cg.cuh,
// new-cg/include/segscan/segscan.cuh).  This header keeps their names,
// template parameters, argument order and output contract, so a reference
// caller switches by changing its include:
//
//   csrspmm_parreduce_nnzbalance_cg<Index, DType, group_factor,
//       thread_per_block, tile_factor, block_numer, block_denom>(A, N, B, C)
//
// Differences a caller sees:
//   * errors throw segscan_gb300::Error (the reference calls exit());
//   * an optional trailing cudaStream_t (the reference uses the legacy
//     default stream);
//   * scratch for the element-balanced strategies comes from a workspace
//     per (device, stream) that this header grows with cudaMalloc on first
//     use, outside the hot path: calls on one stream run in order and can
//     share it, calls on different streams never do; C callers pass their
//     own through the C ABI instead.
// The ebpr / rbpr / ebsr launchers ADD into C (the reference's callers zero
// C first, test-cg/include/util/check.cuh:71), rbsr overwrites C, and the
// segment_coo launchers ADD into dst, as in the reference.
#ifndef SEGSCAN_GB300_HPP
#define SEGSCAN_GB300_HPP

#include <cuda_runtime.h>

#include <cstdint>
#include <map>
#include <mutex>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <vector>

#include "segscan_gb300.h"

namespace segscan_gb300 {

struct Error : std::runtime_error {
  int status;
  Error(int st, const std::string &what) : std::runtime_error(what), status(st) {}
};

inline void check(ss_status st, const char *where) {
  if (st != SS_OK)
    throw Error(st, std::string(where) + ": " + ss_status_string(st) + " - " + ss_last_error());
}

template <class T> struct dtype_of;
template <> struct dtype_of<float> { static constexpr int value = SS_F32; };

// Device CSR handle, the reference's SpMatCsrDescr_t
// (test-cg/include/dataloader/dataloader.hpp:146-168) without the host
// mirror: the caller owns the three device arrays.  data == nullptr means
// every stored value is 1.
template <class Index, class DType> struct SpMatCsrDescr_t {
  static_assert(std::is_same<Index, int>::value || std::is_same<Index, int32_t>::value,
                "indices are int32");
  int nrow = 0, ncol = 0, nnz = 0;
  const Index *indptr = nullptr;
  const Index *indices = nullptr;
  const DType *data = nullptr;

  ss_csr descr() const {
    ss_csr d;
    d.nrow = nrow;
    d.ncol = ncol;
    d.nnz = nnz;
    d.indptr = reinterpret_cast<const int32_t *>(indptr);
    d.indices = reinterpret_cast<const int32_t *>(indices);
    d.values = data;
    d.value_dtype = dtype_of<DType>::value;
    return d;
  }
};

// Scratch per (device, stream), grown on demand and kept for the life of
// the process.  Work on one stream is ordered, so its calls share a buffer;
// a buffer is only replaced (to grow it) after its stream has drained.
// Host threads that launch on one shared stream must serialise their calls:
// a growth on one thread between another thread's get() and its launch
// would free the buffer that launch was given.
class Workspace {
 public:
  static void *get(size_t bytes, cudaStream_t stream) {
    static std::mutex mu;
    static std::map<std::pair<int, cudaStream_t>, std::pair<void *, size_t>> slots;
    int dev = 0;
    check(cudaGetDevice(&dev) == cudaSuccess ? SS_OK : SS_ERR_CUDA, "cudaGetDevice");
    std::lock_guard<std::mutex> lock(mu);
    auto &slot = slots[{dev, stream}];
    if (slot.second < bytes) {
      if (slot.first) {
        // earlier calls on this stream may still read the old buffer
        if (cudaStreamSynchronize(stream) != cudaSuccess) throw Error(SS_ERR_CUDA, "workspace stream sync failed");
        cudaFree(slot.first);
      }
      slot = {nullptr, 0};
      if (cudaMalloc(&slot.first, bytes) != cudaSuccess) throw Error(SS_ERR_CUDA, "workspace cudaMalloc failed");
      slot.second = bytes;
    }
    return slot.first;
  }
};

namespace detail {
inline ss_knobs knobs(int group_factor, int tile_factor, int thread_per_block, int block_numer, int block_denom,
                      int coarsen_factor = 4, int thread_nz = 1) {
  ss_knobs k;
  k.group_factor = group_factor;
  k.tile_factor = tile_factor;
  k.thread_per_block = thread_per_block;
  k.block_numer = block_numer;
  k.block_denom = block_denom;
  k.coarsen_factor = coarsen_factor;
  k.thread_nz = thread_nz;
  k.kahan_threshold = 0;
  return k;
}

template <class Index, class DType>
inline void spmm(int strategy, const SpMatCsrDescr_t<Index, DType> &A, int N, const DType *B, DType *C,
                 int accumulate, const ss_knobs &k, cudaStream_t s, const char *where) {
  ss_csr d = A.descr();
  size_t ws = 0;
  check(ss_spmm_workspace_size(strategy, &d, N, &k, &ws), where);
  void *w = ws ? Workspace::get(ws, s) : nullptr;
  check(ss_spmm(strategy, &d, N, B, C, dtype_of<DType>::value, accumulate, &k, w, ws, (void *)s), where);
}

template <class V, class I>
inline void segment(int strategy, const V *src, const I *index, int nnz, int N, V *dst, int dst_len,
                    const ss_knobs &k, cudaStream_t s, const char *where) {
  static_assert(std::is_same<V, float>::value, "segment_coo dst is float");
  size_t ws = 0;
  check(ss_segment_coo_workspace_size(strategy, nnz, N, &k, &ws), where);
  void *w = ws ? Workspace::get(ws, s) : nullptr;
  check(ss_segment_coo(strategy, src, dtype_of<V>::value, reinterpret_cast<const int32_t *>(index), nnz, N, dst_len,
                       dst, SS_SUM, 1, &k, w, ws, (void *)s),
        where);
}
}  // namespace detail

// ---------------------------------------------------------------------
// SpMM launchers (test-cg/include/spmm/spmm_cg.cuh)
// ---------------------------------------------------------------------

// spmm_cg.cuh:176-178: C += A * B, element-balanced, parallel reduction.
template <class Index, class DType, int group_factor, int thread_per_block, int tile_factor, int block_numer,
          int block_denom>
void csrspmm_parreduce_nnzbalance_cg(const SpMatCsrDescr_t<Index, DType> &A, const int N, const DType *B, DType *C,
                                     cudaStream_t s = 0) {
  detail::spmm(SS_EBPR, A, N, B, C, 1,
               detail::knobs(group_factor, tile_factor, thread_per_block, block_numer, block_denom), s,
               "csrspmm_parreduce_nnzbalance_cg");
}

// spmm_cg.cuh:333-335: C += A * B, row-balanced, parallel reduction.
template <class Index, class DType, int group_factor, int thread_per_block, int tile_factor, int block_numer,
          int block_denom>
void csrspmm_parreduce_rowbalance_cg(const SpMatCsrDescr_t<Index, DType> &A, const int N, const DType *B, DType *C,
                                     cudaStream_t s = 0) {
  detail::spmm(SS_RBPR, A, N, B, C, 1,
               detail::knobs(group_factor, tile_factor, thread_per_block, block_numer, block_denom), s,
               "csrspmm_parreduce_rowbalance_cg");
}

// spmm_cg.cuh:553-555: C += A * B, element-balanced, sequential reduction.
template <class Index, class DType, int group_factor, int thread_per_block, int CoarsenFactor, int ThreadNz,
          int block_numer, int block_denom>
void csrspmm_rowcaching_nnzbalance_cg(const SpMatCsrDescr_t<Index, DType> &A, const int N, const DType *B, DType *C,
                                      cudaStream_t s = 0) {
  detail::spmm(SS_EBSR, A, N, B, C, 1,
               detail::knobs(group_factor, 0, thread_per_block, block_numer, block_denom, CoarsenFactor, ThreadNz), s,
               "csrspmm_rowcaching_nnzbalance_cg");
}

// spmm_cg.cuh:664-666: C = A * B, row-balanced, sequential reduction.
template <class Index, class DType, int coarsen_factor, int thread_per_block, int tile_factor, int block_numer,
          int block_denom>
void csrspmm_seqreduce_rowbalance_cg(const SpMatCsrDescr_t<Index, DType> &A, const int N, const DType *B, DType *C,
                                     cudaStream_t s = 0) {
  detail::spmm(SS_RBSR, A, N, B, C, 0,
               detail::knobs(0, tile_factor, thread_per_block, block_numer, block_denom, coarsen_factor), s,
               "csrspmm_seqreduce_rowbalance_cg");
}

// ---------------------------------------------------------------------
// segment_coo launchers (new-cg/include/segscan/segscan.cuh): dst += sums.
// The reference signature has no output length; dst_len bounds the writes
// and defaults to "every index is in range" (the reference's assumption).
// ---------------------------------------------------------------------
constexpr int kUnboundedDst = 0x7fffffff;

// segscan.cuh:150-151
template <class V, class I, int group_factor, int thread_per_block, int tile_factor, int block_numer, int block_denom>
void segment_coo(const V *src, const I *index, const int nnz, const int N, V *dst, int dst_len = kUnboundedDst,
                 cudaStream_t s = 0) {
  detail::segment(SS_SEG_PR, src, index, nnz, N, dst, dst_len,
                  detail::knobs(group_factor, tile_factor, thread_per_block, block_numer, block_denom), s,
                  "segment_coo");
}

// segscan.cuh:327-328 (2-D split): the shuffle-scan family, one step per worker.
template <class V, class I, int group_factor, int thread_per_block, int tile_factor, int blockDimY>
void segment_coo_new(const V *src, const I *index, const int nnz, const int N, V *dst, int dst_len = kUnboundedDst,
                     cudaStream_t s = 0) {
  detail::segment(SS_SEG_PR, src, index, nnz, N, dst, dst_len,
                  detail::knobs(group_factor, tile_factor, thread_per_block, 1, 1 << tile_factor), s,
                  "segment_coo_new");
}

// segscan.cuh:817-818
template <class V, class I, int group_factor, int thread_per_block, int CoarsenFactor, int ThreadNz, int block_numer,
          int block_denom>
void segment_coo_sr(const V *src, const I *index, const int nnz, const int N, V *dst, int dst_len = kUnboundedDst,
                    cudaStream_t s = 0) {
  detail::segment(SS_SEG_SR, src, index, nnz, N, dst, dst_len,
                  detail::knobs(group_factor, 0, thread_per_block, block_numer, block_denom, CoarsenFactor, ThreadNz),
                  s, "segment_coo_sr");
}

// segscan.cuh:868-869
template <class V, class I, int group_factor, int thread_per_block, int CoarsenFactor, int ThreadNz, int block_numer,
          int block_denom>
void segment_coo_noshmem_sr(const V *src, const I *index, const int nnz, const int N, V *dst,
                            int dst_len = kUnboundedDst, cudaStream_t s = 0) {
  segment_coo_sr<V, I, group_factor, thread_per_block, CoarsenFactor, ThreadNz, block_numer, block_denom>(
      src, index, nnz, N, dst, dst_len, s);
}

// segscan.cuh:918-919
template <class V, class I, int group_factor, int thread_per_block, int CoarsenFactor, int ThreadNz, int block_numer,
          int block_denom>
void segment_coo_noshmem_lessatom_sr(const V *src, const I *index, const int nnz, const int N, V *dst,
                                     int dst_len = kUnboundedDst, cudaStream_t s = 0) {
  segment_coo_sr<V, I, group_factor, thread_per_block, CoarsenFactor, ThreadNz, block_numer, block_denom>(
      src, index, nnz, N, dst, dst_len, s);
}

// segscan.cuh:974-975: a worker of DtileSize lanes along N reduces runs of
// ThreadNz elements; DtileNum x BlockDimY workers per block.
template <class V, class I, int CoarsenFactor, int ThreadNz, int DtileSize, int DtileNum, int BlockDimY>
void segment_coo_sorted_sr(const V *src, const I *index, const int nnz, const int N, V *dst,
                           int dst_len = kUnboundedDst, cudaStream_t s = 0) {
  int gf = 0;
  while ((2 << gf) <= DtileSize && gf < 5) gf++;
  const int G = 1 << gf;
  int tpb = G * DtileNum * BlockDimY;
  if (tpb > 512) tpb = 512;
  if (tpb < G) tpb = G;
  tpb -= tpb % G;
  const int tnz = ThreadNz / G > 0 ? ThreadNz / G : 1;
  detail::segment(SS_SEG_SR, src, index, nnz, N, dst, dst_len, detail::knobs(gf, 0, tpb, 1, 1, CoarsenFactor, tnz),
                  s, "segment_coo_sorted_sr");
}

}  // namespace segscan_gb300

#endif  // SEGSCAN_GB300_HPP
