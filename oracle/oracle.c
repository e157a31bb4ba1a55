/*
 * CPU oracle for the segScan hot path.  TEST INFRASTRUCTURE ONLY.
 *
 * Only the tests, the smoke check and the CPU-baseline leg of bench.py load
 * this library, and only as the checker or as the timed CPU baseline.  The
 * product path (the CUDA library under segscan_gb300/) never calls it.
 *
 * Every function restates one piece of zhang677/segScan in plain C:
 *
 *   oracle_spmm_check_f32     test-cg/include/util/check.cuh:139-158  (spmm_reference_host)
 *   oracle_row_of_nz          test-cg/include/util/check.cuh:88-102   (binary_search_segment_number)
 *   oracle_segment_coo_f32    new-cg/include/utils/check.cuh:44-52    (segment_coo_sequencial)
 *   oracle_csr_transpose      test-cg/include/dataloader/dataloader.hpp:109-144
 *                             (compressedRow + transpose, a stable counting sort)
 *
 * and adds FP64 versions of the same loops (the accuracy reference), the
 * absolute-value products used to scale tolerances, segment max/mean (absent
 * from the reference; FP64 only) and the SDDMM used by the backward pass
 * (absent from the reference; FP64 only).
 *
 * Parity pin: tests/golden/ holds outputs of the reference's own host code
 * (compiled from its sources by oracle/Makefile, target `ref`), and the
 * tests check these restatements against them bit for bit.
 */
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define EXPORT __attribute__((visibility("default")))

/* ------------------------------------------------------------------ */
/* SpMM: the reference's CPU check path, FP32, accumulation order     */
/* i (rows) -> p (row's nonzeros, CSR order) -> j (columns).           */
/* C += A*B exactly as check.cuh:139-158 (the caller zero-fills C).   */
/* ------------------------------------------------------------------ */
static void spmm_check_rows(int64_t r0, int64_t r1, int N, const int32_t *indptr,
                            const int32_t *indices, const float *vals,
                            const float *B, float *C) {
  for (int64_t i = r0; i < r1; i++) {
    int32_t begin = indptr[i];
    int32_t end = indptr[i + 1];
    for (int32_t p = begin; p < end; p++) {
      int64_t k = indices[p];
      float val = vals[p];
      const float *brow = B + k * (int64_t)N;
      float *crow = C + i * (int64_t)N;
      for (int64_t j = 0; j < N; j++) crow[j] += val * brow[j];
    }
  }
}

EXPORT void oracle_spmm_check_f32(int M, int N, const int32_t *indptr,
                                  const int32_t *indices, const float *vals,
                                  const float *B, float *C) {
  spmm_check_rows(0, M, N, indptr, indices, vals, B, C);
}

/* Row-parallel form of the same loop.  Rows are independent and each row
 * keeps the sequential order above, so the result is bit-identical to
 * oracle_spmm_check_f32 for any thread count. */
typedef struct {
  int64_t r0, r1;
  int N;
  int zero;
  const int32_t *indptr, *indices;
  const float *vals, *B;
  float *C;
} spmm_job;

static void *spmm_job_run(void *arg) {
  spmm_job *j = (spmm_job *)arg;
  if (j->zero)  /* out_ref.fill_zero_h() for this thread's rows */
    memset(j->C + j->r0 * (int64_t)j->N, 0, (size_t)(j->r1 - j->r0) * (size_t)j->N * sizeof(float));
  spmm_check_rows(j->r0, j->r1, j->N, j->indptr, j->indices, j->vals, j->B, j->C);
  return NULL;
}

static void spmm_check_mt(int M, int N, const int32_t *indptr, const int32_t *indices, const float *vals,
                          const float *B, float *C, int nthreads, int zero);

EXPORT void oracle_spmm_check_f32_mt(int M, int N, const int32_t *indptr,
                                     const int32_t *indices, const float *vals,
                                     const float *B, float *C, int nthreads) {
  spmm_check_mt(M, N, indptr, indices, vals, B, C, nthreads, 0);
}

/* C = 0; C += A*B with every thread zeroing and then filling its own row
 * block (the timed CPU baseline: zero fill and loop, as the reference's
 * check mode does them). */
EXPORT void oracle_spmm_f32_zero_mt(int M, int N, const int32_t *indptr,
                                    const int32_t *indices, const float *vals,
                                    const float *B, float *C, int nthreads) {
  spmm_check_mt(M, N, indptr, indices, vals, B, C, nthreads, 1);
}

static void spmm_check_mt(int M, int N, const int32_t *indptr, const int32_t *indices, const float *vals,
                          const float *B, float *C, int nthreads, int zero) {
  if (nthreads <= 1 || M < 2 * nthreads) {
    if (zero) memset(C, 0, (size_t)M * (size_t)N * sizeof(float));
    oracle_spmm_check_f32(M, N, indptr, indices, vals, B, C);
    return;
  }
  if (nthreads > 256) nthreads = 256;
  pthread_t th[256];
  spmm_job jobs[256];
  /* split by nonzeros so power-law rows do not serialise one thread */
  int64_t nnz = indptr[M];
  int64_t r = 0;
  for (int t = 0; t < nthreads; t++) {
    int64_t target = (nnz * (t + 1)) / nthreads;
    int64_t r1 = r;
    if (t == nthreads - 1) {
      r1 = M;
    } else {
      /* first row whose end passes the target, at least one row */
      int64_t lo = r, hi = M;
      while (lo < hi) {
        int64_t mid = (lo + hi) >> 1;
        if (indptr[mid + 1] <= target) lo = mid + 1; else hi = mid;
      }
      r1 = lo + 1 > M ? M : lo + 1;
      if (r1 < r) r1 = r;
    }
    jobs[t].r0 = r; jobs[t].r1 = r1; jobs[t].N = N; jobs[t].zero = zero;
    jobs[t].indptr = indptr; jobs[t].indices = indices; jobs[t].vals = vals;
    jobs[t].B = B; jobs[t].C = C;
    r = r1;
  }
  int started = 0;
  for (int t = 0; t < nthreads; t++) {
    if (pthread_create(&th[t], NULL, spmm_job_run, &jobs[t]) != 0) {
      spmm_job_run(&jobs[t]);
      th[t] = 0;
    } else {
      started++;
    }
  }
  for (int t = 0; t < nthreads; t++)
    if (th[t]) pthread_join(th[t], NULL);
  (void)started;
}

/* FP64 accuracy reference: C64 = A*B and Cabs = |A|*|B| (the scale of the
 * rounding error bound of any FP32 summation order).  vals == NULL means
 * every stored value is 1 (check.cuh:104-111, __guard_load_default_one). */
EXPORT void oracle_spmm_f64(int M, int N, const int32_t *indptr,
                            const int32_t *indices, const float *vals,
                            const float *B, double *C, double *Cabs) {
  for (int64_t i = 0; i < M; i++) {
    double *crow = C + i * (int64_t)N;
    double *arow = Cabs ? Cabs + i * (int64_t)N : NULL;
    for (int64_t j = 0; j < N; j++) {
      crow[j] = 0.0;
      if (arow) arow[j] = 0.0;
    }
    for (int32_t p = indptr[i]; p < indptr[i + 1]; p++) {
      int64_t k = indices[p];
      double v = vals ? (double)vals[p] : 1.0;
      const float *brow = B + k * (int64_t)N;
      for (int64_t j = 0; j < N; j++) {
        double prod = v * (double)brow[j];
        crow[j] += prod;
        if (arow) arow[j] += fabs(prod);
      }
    }
  }
}

/* Row-parallel form of oracle_spmm_f64 for the full-size parity checks.
 * Rows are independent and keep the sequential order, so the result is
 * bit-identical for any thread count. */
typedef struct {
  int64_t r0, r1;
  int N;
  const int32_t *indptr, *indices;
  const float *vals, *B;
  double *C, *Cabs;
} spmm64_job;

static void *spmm64_job_run(void *arg) {
  spmm64_job *j = (spmm64_job *)arg;
  const int64_t N = j->N;
  /* indptr holds absolute positions into indices, so the row block only
   * shifts indptr and the outputs */
  oracle_spmm_f64((int)(j->r1 - j->r0), j->N, j->indptr + j->r0, j->indices, j->vals, j->B,
                  j->C + j->r0 * N, j->Cabs ? j->Cabs + j->r0 * N : NULL);
  return NULL;
}

EXPORT void oracle_spmm_f64_mt(int M, int N, const int32_t *indptr, const int32_t *indices,
                               const float *vals, const float *B, double *C, double *Cabs,
                               int nthreads) {
  if (nthreads <= 1 || M < 2 * nthreads) {
    oracle_spmm_f64(M, N, indptr, indices, vals, B, C, Cabs);
    return;
  }
  if (nthreads > 256) nthreads = 256;
  pthread_t th[256];
  int started[256];
  spmm64_job jobs[256];
  int64_t nnz = indptr[M];
  int64_t r = 0;
  for (int t = 0; t < nthreads; t++) {
    int64_t target = (nnz * (t + 1)) / nthreads;
    int64_t r1;
    if (t == nthreads - 1) {
      r1 = M;
    } else {
      int64_t lo = r, hi = M;
      while (lo < hi) {
        int64_t mid = (lo + hi) >> 1;
        if (indptr[mid + 1] <= target) lo = mid + 1; else hi = mid;
      }
      r1 = lo + 1 > M ? M : lo + 1;
      if (r1 < r) r1 = r;
    }
    jobs[t].r0 = r; jobs[t].r1 = r1; jobs[t].N = N;
    jobs[t].indptr = indptr; jobs[t].indices = indices; jobs[t].vals = vals; jobs[t].B = B;
    jobs[t].C = C; jobs[t].Cabs = Cabs;
    r = r1;
  }
  for (int t = 0; t < nthreads; t++) {
    started[t] = pthread_create(&th[t], NULL, spmm64_job_run, &jobs[t]) == 0;
    if (!started[t]) spmm64_job_run(&jobs[t]);
  }
  for (int t = 0; t < nthreads; t++)
    if (started[t]) pthread_join(th[t], NULL);
}

/* ------------------------------------------------------------------ */
/* Row of a nonzero: upper_bound(indptr[1..M-1], e) - 1.               */
/* Empty rows are skipped; e >= nnz gives M-1 (check.cuh:88-102).      */
/* ------------------------------------------------------------------ */
EXPORT int32_t oracle_row_of_nz(const int32_t *indptr, int32_t M, int32_t nnz,
                                int32_t e) {
  (void)nnz;
  int32_t lo = 1, hi = M;
  while (lo < hi) {
    int32_t mid = (lo + hi) >> 1;
    if (indptr[mid] <= e) lo = mid + 1; else hi = mid;
  }
  return hi - 1;
}

EXPORT void oracle_row_ids(const int32_t *indptr, int32_t M, int32_t nnz,
                           const int32_t *elems, int64_t count, int32_t *rows) {
  for (int64_t i = 0; i < count; i++)
    rows[i] = oracle_row_of_nz(indptr, M, nnz, elems[i]);
}

/* ------------------------------------------------------------------ */
/* segment_coo                                                          */
/* ------------------------------------------------------------------ */
/* dst[index[i], :] += src[i, :], FP32, i ascending (new-cg check.cuh:44-52). */
EXPORT void oracle_segment_coo_f32(const float *src, const int32_t *index,
                                   int nnz, int N, float *dst) {
  for (int64_t i = 0; i < nnz; i++) {
    const float *s = src + i * (int64_t)N;
    float *d = dst + (int64_t)index[i] * N;
    for (int64_t j = 0; j < N; j++) d[j] += s[j];
  }
}

/* FP64 segment reduction over a sorted index.  reduce: 0 sum, 1 max,
 * 2 mean.  Empty segments give 0 for every reduction.  dabs (optional)
 * receives sum |src| per segment (the tolerance scale for sum/mean). */
EXPORT void oracle_segment_coo_f64(const float *src, const int32_t *index,
                                   int nnz, int N, int dst_len, int reduce,
                                   double *dst, double *dabs) {
  int64_t total = (int64_t)dst_len * N;
  int64_t *count = (int64_t *)calloc((size_t)(dst_len > 0 ? dst_len : 1), sizeof(int64_t));
  for (int64_t t = 0; t < total; t++) {
    dst[t] = reduce == 1 ? -INFINITY : 0.0;
    if (dabs) dabs[t] = 0.0;
  }
  for (int64_t i = 0; i < nnz; i++) {
    int64_t r = index[i];
    if (r < 0 || r >= dst_len) continue;
    count[r]++;
    const float *s = src + i * (int64_t)N;
    double *d = dst + r * N;
    double *a = dabs ? dabs + r * N : NULL;
    for (int64_t j = 0; j < N; j++) {
      double x = (double)s[j];
      if (reduce == 1) {
        if (x > d[j]) d[j] = x;
      } else {
        d[j] += x;
      }
      if (a) a[j] += fabs(x);
    }
  }
  for (int64_t r = 0; r < dst_len; r++) {
    double *d = dst + r * N;
    for (int64_t j = 0; j < N; j++) {
      if (count[r] == 0) d[j] = 0.0;
      else if (reduce == 2) d[j] /= (double)count[r];
    }
    if (dabs && reduce == 2 && count[r] > 0)
      for (int64_t j = 0; j < N; j++) dabs[r * N + j] /= (double)count[r];
  }
  free(count);
}

/* ------------------------------------------------------------------ */
/* CSR transpose (dataloader.hpp:123-144 then compressedRow :109-121). */
/* A stable counting sort by column: within a column, entries keep     */
/* their CSR order.  perm[q] = source nonzero of transposed entry q.   */
/* ------------------------------------------------------------------ */
EXPORT void oracle_csr_transpose(int M, int K, const int32_t *indptr,
                                 const int32_t *indices, int32_t *t_indptr,
                                 int32_t *t_indices, int32_t *perm) {
  int64_t nnz = indptr[M];
  int64_t *next = (int64_t *)calloc((size_t)K + 1, sizeof(int64_t));
  for (int64_t p = 0; p < nnz; p++) next[indices[p] + 1]++;
  for (int64_t c = 0; c < K; c++) next[c + 1] += next[c];
  for (int64_t c = 0; c <= K; c++) t_indptr[c] = (int32_t)next[c];
  for (int64_t i = 0; i < M; i++) {
    for (int32_t p = indptr[i]; p < indptr[i + 1]; p++) {
      int64_t q = next[indices[p]]++;
      t_indices[q] = (int32_t)i;
      if (perm) perm[q] = p;
    }
  }
  free(next);
}

/* ------------------------------------------------------------------ */
/* SDDMM for the backward pass: out[p] = dot(dC[i,:], B[k,:]) for the  */
/* stored nonzero p = (i, k).  FP64.  No counterpart in the reference. */
/* ------------------------------------------------------------------ */
EXPORT void oracle_sddmm_f64(int M, int N, const int32_t *indptr,
                             const int32_t *indices, const float *dC,
                             const float *B, double *out, double *outabs) {
  for (int64_t i = 0; i < M; i++) {
    const float *g = dC + i * (int64_t)N;
    for (int32_t p = indptr[i]; p < indptr[i + 1]; p++) {
      const float *b = B + (int64_t)indices[p] * N;
      double s = 0.0, a = 0.0;
      for (int64_t j = 0; j < N; j++) {
        double prod = (double)g[j] * (double)b[j];
        s += prod;
        a += fabs(prod);
      }
      out[p] = s;
      if (outabs) outabs[p] = a;
    }
  }
}
