/*
 * segscan_gb300 - C ABI of the GB300 (sm_103a) SpMM / segment_coo library.
 *
 * The reference (zhang677/segScan) has no library boundary: its operator API
 * is header-only C++ templates that a driver instantiates per knob tuple.
 * This header is the drop-in replacement for those templates: the same four
 * SpMM strategies and the segment_coo family, with the same tuning knobs
 * passed at run time instead of as template arguments.  Every entry point
 * cites the reference interface it replaces.  include/segscan_gb300.hpp
 * re-creates the reference's template signatures on top of this ABI.
 *
 * Conventions
 *  - All array arguments are DEVICE pointers owned by the caller.  Nothing
 *    here allocates device memory; scratch space comes from the caller
 *    through (ws, ws_bytes), sized by the matching *_workspace_size query.
 *  - `stream` is a cudaStream_t passed as void* (NULL = legacy default
 *    stream).  Every call is stream-ordered and asynchronous; calls that
 *    share no buffers may run concurrently on different streams.
 *  - Errors come back as ss_status.  Nothing calls exit().  Argument and
 *    knob errors are detected on the host before any launch.  Malformed
 *    device data (column out of range, indptr not monotone, unsorted
 *    segment index) never makes a kernel access memory out of bounds; the
 *    ss_*_validate calls report it.
 *  - Outputs: with accumulate = 0 the output is overwritten (C = A*B), every
 *    row including empty rows is written, and the caller need not zero it.
 *    With accumulate = 1 the result is added (C += A*B), matching the
 *    reference launchers whose callers pre-zero C.
 *  - Values and B share one storage type (SS_F32, SS_BF16 or SS_F16);
 *    arithmetic is FP32 in every kernel; C is FP32 or the storage type
 *    (ebsr with FP32 storage also writes a BF16/FP16 C, rounding in its
 *    stores).
 */
#ifndef SEGSCAN_GB300_H
#define SEGSCAN_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SS_VERSION_MAJOR 0
#define SS_VERSION_MINOR 1

typedef enum {
  SS_OK = 0,
  SS_ERR_INVALID_ARG = 1,       /* null pointer, negative size, bad enum */
  SS_ERR_UNSUPPORTED_KNOBS = 2, /* knob tuple outside the compiled table */
  SS_ERR_WORKSPACE = 3,         /* ws too small or misaligned */
  SS_ERR_CUDA = 4,              /* a CUDA runtime call failed */
  SS_ERR_ALIGNMENT = 5,         /* a pointer is not aligned to its element */
  SS_ERR_BAD_DATA = 6,          /* reported by the *_validate calls */
  SS_ERR_TIMEOUT = 7,           /* a bounded device wait gave up */
  SS_ERR_CAPACITY = 8           /* size beyond a fixed capacity */
} ss_status;

typedef enum { SS_F32 = 0, SS_BF16 = 1, SS_F16 = 2 } ss_dtype;

typedef enum {
  SS_EBPR = 0, /* element-balanced, parallel reduction  */
  SS_RBPR = 1, /* row-balanced, parallel reduction      */
  SS_EBSR = 2, /* element-balanced, sequential reduction */
  SS_RBSR = 3  /* row-balanced, sequential reduction    */
} ss_strategy;

typedef enum { SS_SUM = 0, SS_MAX = 1, SS_MEAN = 2 } ss_reduce;

typedef enum {
  SS_SEG_PR = 0, /* shuffle-scan family: segment_coo, segment_coo_new            */
  SS_SEG_SR = 1  /* sequential family: segment_coo_sr, _noshmem_sr,
                    _noshmem_lessatom_sr, _sorted_sr                               */
} ss_seg_strategy;

/* CSR matrix A [nrow x ncol] (SpMatCsrDescr_t, test-cg/include/dataloader/
 * dataloader.hpp:146-168).  values == NULL means every stored value is 1
 * (__guard_load_default_one, test-cg/include/util/check.cuh:104-111). */
typedef struct {
  int32_t nrow, ncol, nnz;
  const int32_t *indptr;  /* [nrow + 1], indptr[0] = 0, indptr[nrow] = nnz */
  const int32_t *indices; /* [nnz], column of each nonzero, in [0, ncol)   */
  const void *values;     /* [nnz] of value_dtype, or NULL                 */
  int32_t value_dtype;    /* ss_dtype                                       */
} ss_csr;

/* Tuning knobs, the reference's template parameters at run time.
 *   group_factor     group_size = 1 << group_factor lanes that reduce together
 *                    (ebpr, rbpr) or that share one staged nonzero tile (ebsr)
 *   tile_factor      tile_size  = 1 << tile_factor (the README's tail_factor):
 *                    lanes per row (rbpr), nonzeros per step (ebpr), column
 *                    tile width (ebpr, rbpr, rbsr)
 *   thread_per_block threads per CTA
 *   block_numer/block_denom  block_factor: workers = nrow * numer / denom
 *   coarsen_factor   elements of N per lane (ebsr CoarsenFactor, rbsr
 *                    coarsen_factor; ebpr/rbpr derive it from N as the
 *                    reference does)
 *   thread_nz        staged tiles per worker step (ebsr ThreadNz)
 *   kahan_threshold  SpMM: the nonzeros of a row longer than this are
 *                    accumulated with compensated (Kahan) summation by the
 *                    sequential strategies (ebsr, rbsr, and rbpr within each
 *                    slot); ebpr adds in a shuffle-scan tree.  segment_coo
 *                    (sequential family): a chunk longer than this is
 *                    summed with compensation.  Partials of rows or
 *                    segments that straddle chunks are always combined with
 *                    compensation.  <= 0 selects the default (1024),
 *                    INT32_MAX disables the per-row compensation. */
typedef struct {
  int32_t group_factor;
  int32_t tile_factor;
  int32_t thread_per_block;
  int32_t block_numer;
  int32_t block_denom;
  int32_t coarsen_factor;
  int32_t thread_nz;
  int32_t kahan_threshold;
} ss_knobs;

/* ---------------------------------------------------------------- */
/* Library                                                            */
/* ---------------------------------------------------------------- */
int ss_version(void);                      /* major * 100 + minor */
const char *ss_status_string(int status);  /* static string */
/* Text of the last failure on the calling host thread ("" if none). */
const char *ss_last_error(void);
/* Device-side status of the bounded waits in the kernels: *status gets 0 or
 * SS_ERR_TIMEOUT (a wait gave up and the group that waited stopped, leaving
 * its outputs unwritten).  clear = 1 resets it.  Synchronous with respect to
 * the device.  The flag is one word per device, shared by every launch on
 * every stream and host thread of the process: a timeout on one stream is
 * seen by whichever caller reads next, and a clear by one thread can erase a
 * timeout another thread has not read yet, so callers that share a device
 * read and clear it at a point where they have ordered their launches.  No
 * counterpart in the reference (its kernels never wait). */
ss_status ss_device_error(int *status, int clear);
/* Diagnostic: one bounded mbarrier wait that can never complete (an
 * expected transaction no copy delivers) gives up after `polls` tries and
 * sets the device flag above to SS_ERR_TIMEOUT, the path a lost bulk copy
 * takes in the walk kernels; the context stays usable.  No counterpart in
 * the reference. */
ss_status ss_selftest_bounded_wait(int polls, void *stream);
/* L2 budget (bytes) for the gathered dense operand B: when B is larger,
 * only a fixed address subset of that size is marked evict_last and the
 * rest evict_first, so the kept subset stays resident.  0 (the default)
 * marks all of B evict_last.  Process-wide.  No counterpart in the
 * reference. */
ss_status ss_set_l2_keep_bytes(long long bytes);
/* Knob tuple the reference's README reports as best static choice for a
 * strategy (test-cg README.md:168-210), used when knobs == NULL. */
ss_status ss_default_knobs(int strategy, int N, ss_knobs *out);

/* ---------------------------------------------------------------- */
/* SpMM: C[nrow x N] (=|+=) A[nrow x ncol] * B[ncol x N], row-major.  */
/* ---------------------------------------------------------------- */

/* Scratch bytes a strategy needs for (A, N, knobs); 0 for rbpr/rbsr. */
ss_status ss_spmm_workspace_size(int strategy, const ss_csr *A, int N,
                                 const ss_knobs *knobs, size_t *bytes);

/* Replaces csrspmm_parreduce_nnzbalance_cg<Index, DType, group_factor,
 * thread_per_block, tile_factor, block_numer, block_denom>
 * (test-cg/include/spmm/spmm_cg.cuh:176-178). */
ss_status ss_spmm_ebpr(const ss_csr *A, int N, const void *B, void *C,
                       int c_dtype, int accumulate, const ss_knobs *knobs,
                       void *ws, size_t ws_bytes, void *stream);

/* Replaces csrspmm_parreduce_rowbalance_cg<...same knobs...>
 * (spmm_cg.cuh:333-335). */
ss_status ss_spmm_rbpr(const ss_csr *A, int N, const void *B, void *C,
                       int c_dtype, int accumulate, const ss_knobs *knobs,
                       void *ws, size_t ws_bytes, void *stream);

/* Replaces csrspmm_rowcaching_nnzbalance_cg<Index, DType, group_factor,
 * thread_per_block, CoarsenFactor, ThreadNz, block_numer, block_denom>
 * (spmm_cg.cuh:553-555).  Chunks (ThreadNz * 2^group_factor nonzeros)
 * smaller than the nonzeros' share per resident group of one full wave are
 * merged up to that share (also for ebpr); the result is the same up to
 * FP32 rounding order, deterministic for given inputs and knobs. */
ss_status ss_spmm_ebsr(const ss_csr *A, int N, const void *B, void *C,
                       int c_dtype, int accumulate, const ss_knobs *knobs,
                       void *ws, size_t ws_bytes, void *stream);

/* The ebsr SpMM without a workspace argument, for callers that cannot
 * allocate device memory: a host that only holds buffers handed to it by
 * another allocator, or a loop where cudaMalloc's blocking, device
 * synchronisation or failure is not acceptable.  Its scratch is a fixed
 * 16 MiB array inside the library (held on every GPU that loads it); calls
 * needing more get SS_ERR_CAPACITY.  All calls on a device share that array,
 * so calls that overlap on the GPU race.  The first call on a device looks
 * up the array's address and keeps it; make it before any stream capture,
 * and do not call this again on a device after cudaDeviceReset.  No
 * counterpart in the reference. */
ss_status ss_spmm_ebsr_noalloc(const ss_csr *A, int N, const void *B, void *C,
                               int c_dtype, int accumulate,
                               const ss_knobs *knobs, void *stream);

/* Replaces csrspmm_seqreduce_rowbalance_cg<Index, DType, coarsen_factor,
 * thread_per_block, tile_factor, block_numer, block_denom>
 * (spmm_cg.cuh:664-666). */
ss_status ss_spmm_rbsr(const ss_csr *A, int N, const void *B, void *C,
                       int c_dtype, int accumulate, const ss_knobs *knobs,
                       void *ws, size_t ws_bytes, void *stream);

/* One entry for any strategy (the four calls above dispatch here). */
ss_status ss_spmm(int strategy, const ss_csr *A, int N, const void *B,
                  void *C, int c_dtype, int accumulate, const ss_knobs *knobs,
                  void *ws, size_t ws_bytes, void *stream);

/* ---------------------------------------------------------------- */
/* segment_coo: dst[index[i], :] (op)= src[i, :] over sorted index.    */
/* ---------------------------------------------------------------- */

/* Workspace bytes ss_segment_coo needs for nnz x N with these knobs, for
 * any source dtype (the largest of the three). */
ss_status ss_segment_coo_workspace_size(int seg_strategy, int nnz, int N,
                                        const ss_knobs *knobs, size_t *bytes);

/* Replaces segment_coo / segment_coo_new (SS_SEG_PR) and segment_coo_sr,
 * segment_coo_noshmem_sr, segment_coo_noshmem_lessatom_sr,
 * segment_coo_sorted_sr (SS_SEG_SR)
 * (new-cg/include/segscan/segscan.cuh:150-151, 327-328, 817-818, 868-869,
 * 918-919, 974-975), which compute the sum only; max and mean are added.
 * src [nnz x N] of src_dtype, index [nnz] sorted ascending, dst
 * [dst_len x N] FP32.  Empty segments get 0.  accumulate = 1 is allowed for
 * SS_SUM only (the reference's dst += contract). */
ss_status ss_segment_coo(int seg_strategy, const void *src, int src_dtype,
                         const int32_t *index, int nnz, int N, int dst_len,
                         float *dst, int reduce, int accumulate,
                         const ss_knobs *knobs, void *ws, size_t ws_bytes,
                         void *stream);

/* ---------------------------------------------------------------- */
/* Row assignment, transpose, SDDMM, validation                        */
/* ---------------------------------------------------------------- */

/* rows[i] = row owning nonzero elems[i]: upper_bound(indptr[1..M-1], e) - 1,
 * empty rows skipped, e >= nnz gives M-1.  Replaces
 * binary_search_segment_number (test-cg/include/util/check.cuh:88-102). When
 * elems == NULL, rows[e] is written for every e in [0, count). */
ss_status ss_row_ids(const int32_t *indptr, int M, int nnz,
                     const int32_t *elems, int64_t count, int32_t *rows,
                     void *stream);

/* Transposed pattern of A: t_indptr [ncol + 1], t_indices [nnz] (row ids),
 * perm [nnz] (source nonzero of each transposed entry).  Stable: within a
 * column the entries keep A's CSR order, so the result is bit-identical to
 * the host counting sort transpose + compressedRow
 * (test-cg/include/dataloader/dataloader.hpp:109-144). */
ss_status ss_csr_transpose_workspace_size(const ss_csr *A, size_t *bytes);
ss_status ss_csr_transpose(const ss_csr *A, int32_t *t_indptr,
                           int32_t *t_indices, int32_t *perm, void *ws,
                           size_t ws_bytes, void *stream);
/* As ss_csr_transpose, and t_values [nnz] = A's values in transposed order
 * (A->value_dtype; the same as ss_gather_values on perm, in the same pass).
 * t_values NULL: the pattern only.  Same workspace.  Entries past
 * t_indptr[ncol] (nonzeros whose column is outside [0, ncol)) get perm and
 * t_indices -1. */
ss_status ss_csr_transpose_values(const ss_csr *A, int32_t *t_indptr,
                                  int32_t *t_indices, int32_t *perm,
                                  void *t_values, void *ws, size_t ws_bytes,
                                  void *stream);

/* COO -> CSR on the device, the counterpart of compressedRow
 * (test-cg/include/dataloader/dataloader.hpp:109-121), which assumes its
 * input sorted by row: here any order is accepted and the result is the
 * stable counting sort by row (entries of a row keep their input order).
 * indptr [nrow + 1], out_cols [nnz], perm [nnz] (perm[q] = input position
 * of entry q; pass it to ss_gather_values for the values).  Rows outside
 * [0, nrow) are left out (they land past indptr[nrow]).  Workspace from
 * ss_coo_to_csr_workspace_size. */
ss_status ss_coo_to_csr_workspace_size(int nrow, int nnz, size_t *bytes);
ss_status ss_coo_to_csr(int nrow, int nnz, const int32_t *rows,
                        const int32_t *cols, int32_t *indptr,
                        int32_t *out_cols, int32_t *perm, void *ws,
                        size_t ws_bytes, void *stream);

/* out[p] = perm-gathered values: out[q] = values[perm[q]] (any dtype). */
ss_status ss_gather_values(const void *values, int dtype, const int32_t *perm,
                           int nnz, void *out, void *stream);

/* SDDMM for the backward of C = A*B: dvals[p] = dot(dC[i, :], B[k, :]) for
 * every stored nonzero p = (i, k).  dC is FP32 [nrow x N]; B is A's value
 * dtype [ncol x N]; dvals is FP32 [nnz].  No counterpart in the reference. */
ss_status ss_sddmm(const ss_csr *A, int N, const float *dC, const void *B,
                   float *dvals, void *stream);

/* Fused backward of C = A*B, walked over the rows of A^T: dB = A^T * dC and
 * dvals[p] = dot(dC[i, :], B[k, :]) at every stored nonzero p = (i, k), one
 * gather of each dC row serving both (ss_sddmm followed by an SpMM on A^T
 * gathers a B row and then a dC row per nonzero).  AT is the pattern of A^T
 * as ss_csr_transpose builds it (nrow = A's ncol, ncol = A's nrow; its
 * values are not read; value_dtype = the storage type of `values` and B);
 * perm [nnz] maps an A^T position to its A position.  values: A's values in
 * A's order (NULL = ones).  dC [A.nrow x N] FP32; B [A.ncol x N] of
 * value_dtype; dB [A.ncol x N] SS_F32 or value_dtype, overwritten, each row
 * summed in position order (compensated above kahan_threshold, <= 0 = 1024)
 * as rbsr sums A^T's rows; dvals [nnz] FP32 in A's order.  A group of lanes
 * owns a row of A^T, so a very long row of A^T (a dense column of A) is one
 * group's work.  N up to 64 x the widest vector of <= 4 FP32 dividing N
 * (256 for N divisible by 4); beyond that SS_ERR_UNSUPPORTED_KNOBS (use
 * ss_sddmm and ss_spmm on A^T).  No counterpart in the reference. */
ss_status ss_spmm_backward(const ss_csr *AT, const int32_t *perm,
                           const void *values, int N, const float *dC,
                           const void *B, void *dB, int dB_dtype,
                           float *dvals, int kahan_threshold, void *stream);

/* Checks indptr (0 first, nnz last, monotone) and column range; writes 0 to
 * *d_flag (device int) when A is well formed, else a nonzero code. */
ss_status ss_csr_validate(const ss_csr *A, int32_t *d_flag, void *stream);
/* Checks index sorted and inside [0, dst_len); same flag convention. */
ss_status ss_index_validate(const int32_t *index, int nnz, int dst_len,
                            int32_t *d_flag, void *stream);

/* ---------------------------------------------------------------- */
/* Matrix Market input (host side).                                   */
/* ---------------------------------------------------------------- */

/* Replaces read_mtx_file (test-cg/include/dataloader/dataloader.hpp:22-107):
 * a coordinate file's pattern as CSR (values dropped; pass values = NULL to
 * the SpMM calls for ones, as the reference's descriptor does), symmetric
 * files expanded and de-duplicated, entries sorted by (row, column).
 * SS_MTX_REFERENCE gives the reference's result exactly, including its CSR
 * build stopping after the file's declared entry count (an expanded
 * symmetric file loses its last rows' entries there); SS_MTX_FULL keeps every
 * entry and also expands skew-symmetric and hermitian files.  Errors are
 * status codes (the reference exit()s): SS_ERR_BAD_DATA for a malformed file,
 * SS_ERR_CAPACITY when host memory runs out or a full-mode expansion passes
 * 2^31 - 1 entries.  ss_mtx_shape then ss_mtx_csr copy
 * the result into caller buffers of nrow + 1 and nnz int32. */
typedef struct ss_mtx ss_mtx;
enum { SS_MTX_REFERENCE = 0, SS_MTX_FULL = 1 };
ss_status ss_mtx_read(const char *path, int mode, ss_mtx **out);
ss_status ss_mtx_shape(const ss_mtx *m, int *nrow, int *ncol, int *nnz);
ss_status ss_mtx_csr(const ss_mtx *m, int32_t *indptr, int32_t *indices);
void ss_mtx_free(ss_mtx *m);

/* ---------------------------------------------------------------- */
/* Batched SpMM: many independent CSR matrices in one persistent launch */
/* ---------------------------------------------------------------- */

/* A batch plan lives in caller memory: host_bytes of host memory (kept by
 * the caller and passed to every launch) and dev_bytes of device memory
 * (256-byte aligned), both sized by ss_batch_plan_size.  mats, B and C are
 * host arrays of `count` entries (B/C holding device pointers; all
 * matrices share N and the value dtype).  per_mat[m].thread_nz sets matrix
 * m's chunk (thread_nz * 2^group_factor nonzeros); group_factor,
 * coarsen_factor and thread_per_block come from per_mat[0] (NULL = ebsr
 * defaults).  ss_batch_plan uploads the plan and synchronises the stream.
 * ss_spmm_batched then computes C[m] = A[m] * B[m] for every m in one
 * persistent launch (after one memset of its counters; rows that straddle
 * work items are assembled inside that launch), stream-ordered (it can be
 * replayed from a captured CUDA graph).  Not in the reference. */
ss_status ss_batch_plan_size(int count, const ss_csr *mats, int N,
                             const ss_knobs *per_mat, size_t *host_bytes,
                             size_t *dev_bytes);
ss_status ss_batch_plan(int count, const ss_csr *mats, int N,
                        const void *const *B, void *const *C, int c_dtype,
                        const ss_knobs *per_mat, void *host_buf,
                        size_t host_bytes, void *dev_buf, size_t dev_bytes,
                        void *stream);
/* The same with a strategy per matrix: per_mat_strategy[m] is SS_EBSR
 * (element-balanced chunks, as above) or SS_RBSR (row-balanced: items are
 * blocks of whole rows holding about one chunk of nonzeros, so every row is
 * summed in order by one worker with no straddling rows, rbsr's arithmetic);
 * NULL = all SS_EBSR.  The reference has no batched mode; its four
 * strategies are separate launchers (spmm_cg.cuh:553-555, 664-666). */
ss_status ss_batch_plan_size_ex(int count, const ss_csr *mats, int N,
                                const ss_knobs *per_mat,
                                const int *per_mat_strategy,
                                size_t *host_bytes, size_t *dev_bytes);
ss_status ss_batch_plan_ex(int count, const ss_csr *mats, int N,
                           const void *const *B, void *const *C, int c_dtype,
                           const ss_knobs *per_mat, const int *per_mat_strategy,
                           void *host_buf, size_t host_bytes, void *dev_buf,
                           size_t dev_bytes, void *stream);
ss_status ss_spmm_batched(const void *host_plan, void *dev_plan, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* SEGSCAN_GB300_H */
