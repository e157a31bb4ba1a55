// ebsr SpMM for callers that cannot allocate device memory.
//
// Every other entry point of this library takes its scratch from the caller
// (ws, ws_bytes).  Some callers cannot provide that: a host in another
// language that only receives device buffers already allocated by someone
// else and has no device allocator of its own, or a latency-bound loop where
// calling cudaMalloc is not acceptable because it can block, synchronise the
// device or fail part-way through a run.  ss_spmm_ebsr_noalloc serves them:
// the element-balanced SpMM's scratch (the per-chunk carry slots) lives in
// the fixed array below, so the call allocates nothing.  The caller still
// passes A, B and C.
//
// Limits and sharing:
//  * the array holds kNoallocScratchBytes (16 MiB) on every GPU that loads
//    this library, for the life of the process;
//  * a call whose scratch need (ss_spmm_workspace_size for SS_EBSR with the
//    same A, N and knobs) is larger is rejected with SS_ERR_CAPACITY;
//  * all calls on a device share the one array.  Calls that overlap on the
//    GPU (different streams, or host threads that do not order them) race on
//    it; serialise them.  Nothing in the array needs clearing by the
//    caller: the call zeroes its arrival counts itself (stream-ordered) and
//    the walk writes every carry slot before it is read, so the previous
//    call's contents are never used;
//  * the first call on each device looks up the array's device address
//    (cudaGetSymbolAddress) with that device current; make that first call
//    before any stream capture.  The address is kept for the life of the
//    process: after cudaDeviceReset the array may live elsewhere, so a
//    process that resets a device does not call this entry point on it
//    again.
#include <mutex>

#include "internal.h"

namespace ss {

constexpr size_t kNoallocScratchBytes = (size_t)16 << 20;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoallocScratchBytes];

// Device address of g_noalloc_scratch on the current device, looked up once
// per device.  In host code the symbol itself is only a host-side stand-in.
static void *noalloc_scratch(ss_status *st) {
  static std::mutex mu;
  static void *addr[64] = {nullptr};
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) {
    *st = cuda_fail(e, "ss_spmm_ebsr_noalloc: cudaGetDevice");
    return nullptr;
  }
  if (dev < 0 || dev >= 64) {
    *st = fail(SS_ERR_CAPACITY, "ss_spmm_ebsr_noalloc: device %d beyond the 64 devices it tracks", dev);
    return nullptr;
  }
  std::lock_guard<std::mutex> lock(mu);
  if (addr[dev] == nullptr) {
    void *p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || p == nullptr) {
      *st = cuda_fail(e != cudaSuccess ? e : cudaErrorInvalidSymbol,
                      "ss_spmm_ebsr_noalloc: cudaGetSymbolAddress of the fixed scratch");
      return nullptr;
    }
    addr[dev] = p;
  }
  return addr[dev];
}

}  // namespace ss

using namespace ss;

extern "C" ss_status ss_spmm_ebsr_noalloc(const ss_csr *A, int N, const void *B, void *C, int c_dtype,
                                          int accumulate, const ss_knobs *knobs, void *stream) {
  size_t need = 0;
  ss_status st = ss_spmm_workspace_size(SS_EBSR, A, N, knobs, &need);
  if (st != SS_OK) return st;
  if (need > kNoallocScratchBytes)
    return fail(SS_ERR_CAPACITY,
                "ss_spmm_ebsr_noalloc: this call needs %zu bytes of scratch, above the fixed %zu bytes; "
                "raise thread_nz (fewer, longer chunks) or use ss_spmm_ebsr with a workspace",
                need, kNoallocScratchBytes);
  void *scratch = noalloc_scratch(&st);
  if (scratch == nullptr) return st;
  return ss_spmm(SS_EBSR, A, N, B, C, c_dtype, accumulate, knobs, scratch, kNoallocScratchBytes, stream);
}
