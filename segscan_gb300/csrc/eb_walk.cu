// Launchers of the sequential-walk kernels (templates in eb_walk.cuh).
#include <mutex>

#include "eb_walk.cuh"

namespace ss {

// Device status of the bounded waits; kernels get its address in EbArgs.
__device__ int g_walk_error;

int *walk_error_ptr() {
  static std::mutex mu;
  static int *p[64] = {nullptr};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return nullptr;
  std::lock_guard<std::mutex> lock(mu);
  if (!p[dev]) {
    int *q = nullptr;
    if (cudaGetSymbolAddress((void **)&q, g_walk_error) == cudaSuccess) p[dev] = q;
  }
  return p[dev];
}

// ---------------------------------------------------------------------
// Launch
// ---------------------------------------------------------------------
EbArgs eb_base_args(const EbGeom &g, void *ws, int N);

size_t sr_smem_bytes(int stage, int workers_per_block, int val_bytes) {
  return (size_t)workers_per_block * (size_t)sr_layout(stage, val_bytes).bytes;
}

static ss_status run_sr(void *fn, void *arg, const EbGeom &g, size_t smem, cudaStream_t s, const char *what) {
  if (!fn) return fail(SS_ERR_UNSUPPORTED_KNOBS, "no %s kernel for V=%d NV=%d", what, g.cs.V, g.cs.NV);
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return cuda_fail(e, what);
  }
  // at most one resident wave; workers stride over the chunks
  int per_sm = 0;
  cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, g.block, smem);
  if (e != cudaSuccess) return cuda_fail(e, what);
  if (per_sm < 1)
    return fail(SS_ERR_UNSUPPORTED_KNOBS, "%s: block of %d threads with %zu B shared memory does not fit", what,
                g.block, smem);
  int gx = g.grid_x;
  const long long wave = (long long)per_sm * sm_count();
  if (gx > wave) gx = (int)wave;
  dim3 grid(gx, g.cs.tiles, 1), block(g.block, 1, 1);
  void *args[] = {arg};
  cudaError_t err = cudaLaunchKernel(fn, grid, block, args, smem, s);
  if (err != cudaSuccess) return cuda_fail(err, what);
  return SS_OK;
}

static bool aligned16(const void *p) { return ((uintptr_t)p & 15u) == 0; }

ss_status launch_ebsr(const SpmmCall &c, const EbGeom &g, void *ws, cudaStream_t s) {
  EbArgs a = eb_base_args(g, ws, c.N);
  a.M = c.M; a.K = c.K; a.nnz = c.nnz;
  a.indptr = c.indptr; a.cols = c.indices; a.index = nullptr; a.vals = c.vals; a.B = c.B; a.C = c.C;
  a.accumulate = c.accumulate; a.reduce = SS_SUM; a.kahan = c.kahan_threshold;
  a.keep_frac = l2_keep_fraction((size_t)c.K * c.N * dtype_size(c.val_dtype));
  a.use_tma = aligned16(c.indices) && (c.vals == nullptr || aligned16(c.vals)) && (g.chunk % 8) == 0;
  a.err = walk_error_ptr();
  void *fn = nullptr;
  if (c.val_dtype == SS_F32)
    fn = c.c_dtype == SS_F32 ? sr_kernel_f32(g.cs.V, g.cs.NV, false) : sr_kernel_f32_c16(g.cs.V, g.cs.NV, c.c_dtype);
  else if (c.val_dtype == SS_BF16) fn = sr_kernel_bf16(g.cs.V, g.cs.NV, false, c.c_dtype == SS_F32);
  else fn = sr_kernel_f16(g.cs.V, g.cs.NV, false, c.c_dtype == SS_F32);
  // straddling rows are assembled inside the walk (carry_arrive): only the
  // arrival counts need zeroing, no fix-up launch follows
  if (g.num_chunks > 0) {
    cudaError_t e = cudaMemsetAsync(a.carry_cnt, 0, carry_rows_bytes(g.num_chunks, g.cs.tiles), s);
    if (e != cudaSuccess) return cuda_fail(e, "ebsr carry counts");
  }
  // one lane per group: the narrow walk (eb_narrow.cu), no staging
  if (g.cs.lanes == 1) {
    void *nf = narrow_kernel(c.val_dtype, c.c_dtype, g.cs.V, g.cs.NV);
    if (nf) return run_sr(nf, &a, g, 0, s, "ebsr narrow launch");
  }
  return run_sr(fn, &a, g, sr_smem_bytes(g.stage, g.workers_per_block, dtype_size(c.val_dtype)), s, "ebsr launch");
}

ss_status launch_seg_sr(const SegCall &c, const EbGeom &g, void *ws, cudaStream_t s) {
  EbArgs a = eb_base_args(g, ws, c.N);
  a.M = c.dst_len; a.K = c.nnz; a.nnz = c.nnz;
  a.indptr = nullptr; a.cols = nullptr; a.index = c.index; a.vals = nullptr; a.B = c.src; a.C = c.dst;
  a.accumulate = c.accumulate; a.reduce = c.reduce; a.kahan = c.kahan_threshold;
  a.use_tma = aligned16(c.index) && (g.chunk % 8) == 0;
  a.err = walk_error_ptr();
  a.seg_cnt = (int *)((char *)ws + eb_workspace_bytes(g, c.N));
  void *fn = nullptr;
  if (c.src_dtype == SS_F32) fn = sr_kernel_f32(g.cs.V, g.cs.NV, true);
  else if (c.src_dtype == SS_BF16) fn = sr_kernel_bf16(g.cs.V, g.cs.NV, true, true);
  else fn = sr_kernel_f16(g.cs.V, g.cs.NV, true, true);
  // straddling segments are assembled inside the walk (seg_carry_arrive):
  // arrival counts need zeroing, no fix-up launch follows
  if (g.num_chunks > 0) {
    cudaError_t e = cudaMemsetAsync(a.carry_cnt, 0, carry_rows_bytes(g.num_chunks, g.cs.tiles), s);
    if (e != cudaSuccess) return cuda_fail(e, "segment carry counts");
  }
  return run_sr(fn, &a, g, sr_smem_bytes(g.stage, g.workers_per_block, 0), s, "segment_coo sr launch");
}

}  // namespace ss

extern "C" ss_status ss_device_error(int *status, int clear) {
  if (!status) return ss::fail(SS_ERR_INVALID_ARG, "status is null");
  int v = 0;
  cudaError_t e = cudaMemcpyFromSymbol(&v, ss::g_walk_error, sizeof(int));
  if (e != cudaSuccess) return ss::cuda_fail(e, "read device error flag");
  if (clear && v != 0) {
    const int zero = 0;
    e = cudaMemcpyToSymbol(ss::g_walk_error, &zero, sizeof(int));
    if (e != cudaSuccess) return ss::cuda_fail(e, "clear device error flag");
  }
  *status = v;
  return SS_OK;
}

namespace ss {

// One bounded wait that can never complete: an mbarrier expecting 16 bytes
// of transaction that no copy will deliver.  The wait gives up after
// `polls` tries and records SS_ERR_TIMEOUT in the flag the walk kernels use,
// the path a lost bulk copy would take, without any fault.
__global__ void bounded_wait_selftest_kernel(int polls, int *err) {
  __shared__ __align__(8) uint64_t bar;
  if (threadIdx.x != 0) return;
  mbar_init(&bar, 1);
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  mbar_expect_tx(&bar, 16);
  for (int it = 0; !mbar_try_wait(&bar, 0); ) {
    if (++it >= polls) {
      if (err) atomicExch(err, (int)SS_ERR_TIMEOUT);
      break;
    }
  }
}

}  // namespace ss

extern "C" ss_status ss_selftest_bounded_wait(int polls, void *stream) {
  if (polls < 1 || polls > (1 << 22)) return ss::fail(SS_ERR_INVALID_ARG, "polls %d outside [1, 2^22]", polls);
  int *err = ss::walk_error_ptr();
  if (!err) return ss::fail(SS_ERR_CUDA, "device error flag unavailable");
  ss::bounded_wait_selftest_kernel<<<1, 32, 0, (cudaStream_t)stream>>>(polls, err);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? SS_OK : ss::cuda_fail(e, "bounded-wait self-test launch");
}

