// C++ check driver over include/segscan_gb300.hpp, in the shape of the
// reference's check mode (test-cg/src/test.cu:50-82): build A and B, compute
// the CPU SpMM, call launcher instantiations one after another, download,
// compare, print Passed!/Not Passed!, reset C.  Inputs are a seeded
// Poisson(16) 4096 x 4096 matrix with U[-1,1] values and B (the reference
// uses all-ones); the comparison is against an FP64 CPU product with
// tolerance 1e-5 * sum|a*b| per element (the reference uses 1e-2).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <random>
#include <vector>

#include "segscan_gb300.hpp"

using namespace segscan_gb300;
typedef int Index;
typedef float DType;

static int failures = 0;

static void check_result(const char *name, int M, int N, const std::vector<float> &got,
                         const std::vector<double> &ref, const std::vector<double> &absref) {
  bool pass = true;
  for (long long i = 0; i < (long long)M * N && pass; i++)
    if (std::fabs((double)got[i] - ref[i]) > 1e-5 * absref[i] + 1e-30) {
      printf("Wrong result: i = %lld, j = %lld, result = %f, reference = %f.\n", i / N, i % N, got[i], ref[i]);
      pass = false;
    }
  printf("%-40s %s\n", name, pass ? "Passed!" : "Not Passed!");
  if (!pass) failures++;
}

int main() {
  const int M = 4096, K = 4096;
  std::mt19937 gen(0);
  std::poisson_distribution<int> len(16.0);
  std::uniform_int_distribution<int> col(0, K - 1);
  std::uniform_real_distribution<float> val(-1.f, 1.f);
  std::vector<Index> indptr(M + 1, 0), indices;
  std::vector<DType> data;
  for (int i = 0; i < M; i++) {
    std::vector<int> cols;
    int l = len(gen);
    for (int t = 0; t < l; t++) cols.push_back(col(gen));
    std::sort(cols.begin(), cols.end());
    cols.erase(std::unique(cols.begin(), cols.end()), cols.end());
    for (int c : cols) { indices.push_back(c); data.push_back(val(gen)); }
    indptr[i + 1] = (Index)indices.size();
  }
  const int nnz = (int)indices.size();
  for (int N : {4, 16, 64}) {
    std::vector<DType> B((size_t)K * N);
    for (auto &x : B) x = val(gen);
    std::vector<double> ref((size_t)M * N, 0.0), absref((size_t)M * N, 0.0);
    for (int i = 0; i < M; i++)
      for (int p = indptr[i]; p < indptr[i + 1]; p++)
        for (int j = 0; j < N; j++) {
          double prod = (double)data[p] * B[(size_t)indices[p] * N + j];
          ref[(size_t)i * N + j] += prod;
          absref[(size_t)i * N + j] += std::fabs(prod);
        }
    Index *d_indptr, *d_indices;
    DType *d_data, *d_B, *d_C;
    cudaMalloc(&d_indptr, sizeof(Index) * (M + 1));
    cudaMalloc(&d_indices, sizeof(Index) * nnz);
    cudaMalloc(&d_data, sizeof(DType) * nnz);
    cudaMalloc(&d_B, sizeof(DType) * K * N);
    cudaMalloc(&d_C, sizeof(DType) * M * N);
    cudaMemcpy(d_indptr, indptr.data(), sizeof(Index) * (M + 1), cudaMemcpyHostToDevice);
    cudaMemcpy(d_indices, indices.data(), sizeof(Index) * nnz, cudaMemcpyHostToDevice);
    cudaMemcpy(d_data, data.data(), sizeof(DType) * nnz, cudaMemcpyHostToDevice);
    cudaMemcpy(d_B, B.data(), sizeof(DType) * K * N, cudaMemcpyHostToDevice);
    SpMatCsrDescr_t<Index, DType> H;
    H.nrow = M; H.ncol = K; H.nnz = nnz;
    H.indptr = d_indptr; H.indices = d_indices; H.data = d_data;
    std::vector<float> got((size_t)M * N);
    char name[96];
#define RUN(CALL, LABEL)                                                        \
    do {                                                                        \
      cudaMemset(d_C, 0, sizeof(DType) * M * N); /* out_feature.reset() */      \
      CALL;                                                                     \
      cudaMemcpy(got.data(), d_C, sizeof(DType) * M * N, cudaMemcpyDeviceToHost); \
      snprintf(name, sizeof(name), "N=%d %s", N, LABEL);                        \
      check_result(name, M, N, got, ref, absref);                               \
    } while (0)
    RUN((csrspmm_parreduce_nnzbalance_cg<Index, DType, 5, 256, 5, 1, 8>(H, N, d_B, d_C)), "ebpr<5,256,5,1,8>");
    RUN((csrspmm_parreduce_nnzbalance_cg<Index, DType, 2, 128, 3, 1, 1>(H, N, d_B, d_C)), "ebpr<2,128,3,1,1>");
    RUN((csrspmm_parreduce_rowbalance_cg<Index, DType, 3, 256, 3, 1, 2>(H, N, d_B, d_C)), "rbpr<3,256,3,1,2>");
    RUN((csrspmm_parreduce_rowbalance_cg<Index, DType, 5, 256, 5, 2, 1>(H, N, d_B, d_C)), "rbpr<5,256,5,2,1>");
    RUN((csrspmm_rowcaching_nnzbalance_cg<Index, DType, 4, 256, 4, 1, 1, 16>(H, N, d_B, d_C)),
        "ebsr<4,256,4,1,1,16>");
    RUN((csrspmm_rowcaching_nnzbalance_cg<Index, DType, 2, 256, 2, 8, 1, 1>(H, N, d_B, d_C)),
        "ebsr<2,256,2,8,1,1>");
    RUN((csrspmm_seqreduce_rowbalance_cg<Index, DType, 4, 256, 5, 1, 1>(H, N, d_B, d_C)), "rbsr<4,256,5,1,1>");
    RUN((csrspmm_seqreduce_rowbalance_cg<Index, DType, 1, 256, 2, 1, 4>(H, N, d_B, d_C)), "rbsr<1,256,2,1,4>");
    // segment_coo over the same nonzeros: dst[row(p)] += B-row slice p (src = first nnz rows of a dense matrix)
    {
      std::vector<DType> src((size_t)nnz * N);
      for (auto &x : src) x = val(gen);
      std::vector<Index> index(nnz);
      for (int i = 0; i < M; i++)
        for (int p = indptr[i]; p < indptr[i + 1]; p++) index[p] = i;
      std::vector<double> sref((size_t)M * N, 0.0), sabs((size_t)M * N, 0.0);
      for (int p = 0; p < nnz; p++)
        for (int j = 0; j < N; j++) {
          sref[(size_t)index[p] * N + j] += src[(size_t)p * N + j];
          sabs[(size_t)index[p] * N + j] += std::fabs(src[(size_t)p * N + j]);
        }
      DType *d_src;
      Index *d_index;
      cudaMalloc(&d_src, sizeof(DType) * nnz * N);
      cudaMalloc(&d_index, sizeof(Index) * nnz);
      cudaMemcpy(d_src, src.data(), sizeof(DType) * nnz * N, cudaMemcpyHostToDevice);
      cudaMemcpy(d_index, index.data(), sizeof(Index) * nnz, cudaMemcpyHostToDevice);
#define SEG(CALL, LABEL)                                                        \
      do {                                                                      \
        cudaMemset(d_C, 0, sizeof(DType) * M * N);                              \
        CALL;                                                                   \
        cudaMemcpy(got.data(), d_C, sizeof(DType) * M * N, cudaMemcpyDeviceToHost); \
        snprintf(name, sizeof(name), "N=%d %s", N, LABEL);                      \
        check_result(name, M, N, got, sref, sabs);                              \
      } while (0)
      SEG((segment_coo<DType, Index, 5, 256, 5, 1, 16>(d_src, d_index, nnz, N, d_C, M)), "segment_coo<5,256,5,1,16>");
      SEG((segment_coo_new<DType, Index, 5, 256, 5, 2>(d_src, d_index, nnz, N, d_C, M)), "segment_coo_new<5,256,5,2>");
      SEG((segment_coo_sr<DType, Index, 4, 256, 4, 1, 1, 16>(d_src, d_index, nnz, N, d_C, M)),
          "segment_coo_sr<4,256,4,1,1,16>");
      SEG((segment_coo_noshmem_lessatom_sr<DType, Index, 4, 256, 4, 2, 1, 16>(d_src, d_index, nnz, N, d_C, M)),
          "segment_coo_noshmem_lessatom_sr");
      SEG((segment_coo_sorted_sr<DType, Index, 2, 4, 8, 2, 16>(d_src, d_index, nnz, N, d_C, M)),
          "segment_coo_sorted_sr<2,4,8,2,16>");
      cudaFree(d_src);
      cudaFree(d_index);
    }
    // two streams at once: each gets its own workspace from the header, so
    // interleaved ebsr / ebpr calls on them do not share scratch
    {
      cudaStream_t s1, s2;
      cudaStreamCreateWithFlags(&s1, cudaStreamNonBlocking);
      cudaStreamCreateWithFlags(&s2, cudaStreamNonBlocking);
      DType *d_C2;
      cudaMalloc(&d_C2, sizeof(DType) * M * N);
      std::vector<float> got2((size_t)M * N);
      for (int rep = 0; rep < 8; rep++) {
        cudaMemsetAsync(d_C, 0, sizeof(DType) * M * N, s1);
        cudaMemsetAsync(d_C2, 0, sizeof(DType) * M * N, s2);
        csrspmm_rowcaching_nnzbalance_cg<Index, DType, 4, 256, 4, 1, 1, 16>(H, N, d_B, d_C, s1);
        csrspmm_parreduce_nnzbalance_cg<Index, DType, 5, 256, 5, 1, 8>(H, N, d_B, d_C2, s2);
      }
      cudaStreamSynchronize(s1);
      cudaStreamSynchronize(s2);
      cudaMemcpy(got.data(), d_C, sizeof(DType) * M * N, cudaMemcpyDeviceToHost);
      cudaMemcpy(got2.data(), d_C2, sizeof(DType) * M * N, cudaMemcpyDeviceToHost);
      snprintf(name, sizeof(name), "N=%d ebsr on stream 1", N);
      check_result(name, M, N, got, ref, absref);
      snprintf(name, sizeof(name), "N=%d ebpr on stream 2", N);
      check_result(name, M, N, got2, ref, absref);
      cudaFree(d_C2);
      cudaStreamDestroy(s1);
      cudaStreamDestroy(s2);
    }
    cudaFree(d_indptr); cudaFree(d_indices); cudaFree(d_data); cudaFree(d_B); cudaFree(d_C);
  }
  printf("%s\n", failures ? "FAILED" : "ALL PASSED");
  return failures ? 1 : 0;
}
