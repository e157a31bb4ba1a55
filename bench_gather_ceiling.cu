// Random-row gather ceiling of this GPU (measurement program for bench.py's
// roofline notes; not part of the library).
//
// SpMM on a matrix with uniformly random columns is a stream of random B-row
// gathers plus a stream of C-row writes.  This program times that access
// pattern alone, with nothing else in the kernel, so the SpMM kernels can be
// judged against what the memory system delivers for it rather than against
// a streaming copy:
//   * 4.63 M gathers of 256-byte rows (FP32, N = 64) or 128-byte rows (BF16)
//     with uniform random row ids over a footprint of 1M ... 32K rows, so the
//     L2 hit rate runs from capacity misses to resident (ncu's L2 counters
//     on these launches give the hit-rate curve);
//   * a group of 16 (FP32) or 8 (BF16) lanes gathers one row, 16 bytes per
//     lane; the rows' ids are loaded a batch ahead into registers;
//   * "reg": the gathered rows land in registers, 4 rows in flight per
//     group; "ring": per-lane cp.async into a 4-slot shared-memory ring;
//   * "+w": one 256-byte output row written (streaming stores) per five
//     gathers, like the C rows of the power-law SpMM (4.6 nonzeros a row).
// L2 is flushed (a 1 GiB memset) before every timed launch; each line is the
// median of 9 launches (CUDA events).
//
//   nvcc -gencode arch=compute_103a,code=sm_103a -O3 -o _build/bench_gather_ceiling bench_gather_ceiling.cu
//   _build/bench_gather_ceiling [case]        (case: one table line, for ncu)
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <random>
#include <vector>

#define CK(x)                                                                              \
  do {                                                                                     \
    cudaError_t e_ = (x);                                                                  \
    if (e_ != cudaSuccess) {                                                               \
      std::printf("CUDA error %s at line %d: %s\n", #x, __LINE__, cudaGetErrorString(e_)); \
      std::exit(1);                                                                        \
    }                                                                                      \
  } while (0)

namespace {

constexpr int kRows = 4630000;   // gathers per launch (the power-law matrix's nonzeros)
constexpr int kK = 1000000;      // rows of the gathered operand
constexpr int kAhead = 4;        // rows in flight per group

struct Args {
  const int *ids;   // [kRows] row ids
  const char *B;    // [kK][row_bytes]
  float *out;       // [kRows / 5][64]
  int chunk;        // gathers per group
  int row_bytes;    // 256 or 128
  int write_every;  // 0: no output rows
};

__device__ __forceinline__ uint32_t smem_addr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ uint4 ld_row16(const void *p) {
  uint4 v;
  asm volatile("ld.global.nc.L1::no_allocate.v4.u32 {%0,%1,%2,%3}, [%4];"
               : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w)
               : "l"(p));
  return v;
}

__device__ __forceinline__ void add16(float (&acc)[4], uint4 v) {
  acc[0] += __uint_as_float(v.x);
  acc[1] += __uint_as_float(v.y);
  acc[2] += __uint_as_float(v.z);
  acc[3] += __uint_as_float(v.w);
}

__device__ __forceinline__ int load_id(const Args &a, long long e, int e1) { return e < e1 ? __ldg(a.ids + e) : 0; }

// G lanes x 16 bytes per row; RING: cp.async into shared memory, else registers.
template <int G, bool RING>
__global__ void __launch_bounds__(256, 4) gather_kernel(Args a) {
  extern __shared__ __align__(16) uint4 ring[];
  const int lane = threadIdx.x % G;
  const int grp = threadIdx.x / G;
  const unsigned wl = threadIdx.x & 31;
  const unsigned mask = G >= 32 ? 0xffffffffu : (((1u << G) - 1u) << (wl & ~(unsigned)(G - 1)));
  const long long e0 = ((long long)blockIdx.x * blockDim.x + threadIdx.x) / G * a.chunk;
  const int e1 = (int)min(e0 + (long long)a.chunk, (long long)kRows);
  float acc[4] = {0.f, 0.f, 0.f, 0.f};
  if (e0 >= e1) return;
  uint4 *slots = ring + (size_t)grp * kAhead * G + lane;
  uint4 regs[kAhead];
  auto issue = [&](int slot, int id) {
    const char *src = a.B + (long long)id * a.row_bytes + lane * 16;
    if (RING)
      asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_addr(slots + slot * G)), "l"(src)
                   : "memory");
    else
      regs[slot] = ld_row16(src);
  };
  int cur = load_id(a, e0 + lane, e1), next = load_id(a, e0 + G + lane, e1);
#pragma unroll
  for (int u = 0; u < kAhead; u++) {
    const int id = __shfl_sync(mask, cur, u, G);
    if (e0 + u < e1) issue(u, id);
    if (RING) asm volatile("cp.async.commit_group;" ::: "memory");
  }
  long long written = 0;
  for (long long base = e0; base < e1; base += G) {
    const int after = load_id(a, base + 2 * G + lane, e1);
#pragma unroll
    for (int i = 0; i < G; i++) {
      const long long e = base + i;
      const int j = i + kAhead;  // < 2G
      const int id = j < G ? __shfl_sync(mask, cur, j % G, G) : __shfl_sync(mask, next, (j - G) % G, G);
      const int slot = i % kAhead;
      if (RING) asm volatile("cp.async.wait_group %0;" ::"n"(kAhead - 1) : "memory");
      if (e < e1) {
        add16(acc, RING ? slots[slot * G] : regs[slot]);
        if (a.write_every > 0 && e % a.write_every == 0) {
          float *o = a.out + (e / a.write_every) * 64 + lane * (64 / G);
          for (int k = 0; k < 64 / G; k += 4)
            asm volatile("st.global.cs.v4.f32 [%0], {%1,%2,%3,%4};" ::"l"(o + k), "f"(acc[0]), "f"(acc[1]),
                         "f"(acc[2]), "f"(acc[3])
                         : "memory");
          written++;
        }
        if (e + kAhead < e1) issue(slot, id);
      }
      if (RING) asm volatile("cp.async.commit_group;" ::: "memory");
    }
    cur = next;
    next = after;
  }
  if (RING) asm volatile("cp.async.wait_all;" ::: "memory");
  if (acc[0] + acc[1] + acc[2] + acc[3] == 12345.678f) a.out[0] = (float)written;  // keeps the sums live
}

struct Case {
  const char *name;
  int row_bytes;
  bool ring;
  int footprint_rows;
  int write_every;
};

}  // namespace

int main(int argc, char **argv) {
  const int only = argc > 1 ? std::atoi(argv[1]) : -1;
  int sms = 0;
  CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, 0));
  std::vector<Case> cases;
  for (int rb : {256, 128}) {
    for (int fp : {1000000, 500000, 250000, 125000, 32000}) cases.push_back({"reg", rb, false, fp, 0});
    cases.push_back({"ring", rb, true, 1000000, 0});
    cases.push_back({"reg+w", rb, false, 1000000, 5});
    cases.push_back({"ring+w", rb, true, 1000000, 5});
  }
  char *B = nullptr, *flush = nullptr;
  int *ids = nullptr;
  float *out = nullptr;
  const size_t flush_bytes = (size_t)1 << 30;
  CK(cudaMalloc(&B, (size_t)kK * 256));
  CK(cudaMalloc(&ids, (size_t)kRows * 4));
  CK(cudaMalloc(&out, ((size_t)kRows / 5 + 1) * 256));
  CK(cudaMalloc(&flush, flush_bytes));
  CK(cudaMemset(B, 0, (size_t)kK * 256));
  std::vector<int> h(kRows);
  int loaded_fp = -1;
  std::printf("%-4s %-7s %5s %10s %9s %10s %11s\n", "case", "kind", "row_B", "footprint", "ms", "G_rows/s",
              "gather_GB/s");
  for (int c = 0; c < (int)cases.size(); c++) {
    if (only >= 0 && c != only) continue;
    const Case &k = cases[c];
    if (k.footprint_rows != loaded_fp) {
      std::mt19937_64 rng(1234);
      for (int i = 0; i < kRows; i++) h[i] = (int)(rng() % (uint64_t)k.footprint_rows);
      CK(cudaMemcpy(ids, h.data(), (size_t)kRows * 4, cudaMemcpyHostToDevice));
      loaded_fp = k.footprint_rows;
    }
    const int G = k.row_bytes / 16;
    void *fn = G == 16 ? (k.ring ? (void *)gather_kernel<16, true> : (void *)gather_kernel<16, false>)
                       : (k.ring ? (void *)gather_kernel<8, true> : (void *)gather_kernel<8, false>);
    const size_t smem = k.ring ? (size_t)(256 / G) * kAhead * G * 16 : 0;
    int per_sm = 0;
    CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, 256, smem));
    const int grid = per_sm * sms;
    const long long groups = (long long)grid * (256 / G);
    Args a{ids, B, out, (int)((kRows + groups - 1) / groups), k.row_bytes, k.write_every};
    void *args[] = {&a};
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    std::vector<float> ms;
    for (int it = 0; it < 12; it++) {
      CK(cudaMemsetAsync(flush, it & 0xff, flush_bytes));
      CK(cudaEventRecord(e0));
      CK(cudaLaunchKernel(fn, dim3(grid), dim3(256), args, smem, 0));
      CK(cudaEventRecord(e1));
      CK(cudaEventSynchronize(e1));
      float t = 0.f;
      CK(cudaEventElapsedTime(&t, e0, e1));
      if (it >= 3) ms.push_back(t);
    }
    CK(cudaGetLastError());
    std::sort(ms.begin(), ms.end());
    const double t = ms[ms.size() / 2];
    std::printf("%-4d %-7s %5d %8.0fMB %9.4f %10.2f %11.1f\n", c, k.name, k.row_bytes,
                (double)k.footprint_rows * k.row_bytes / 1e6, t, kRows / t / 1e6, (double)kRows * k.row_bytes / t / 1e6);
    std::fflush(stdout);
  }
  return 0;
}
