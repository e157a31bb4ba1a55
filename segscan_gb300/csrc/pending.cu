// Entry points declared in the ABI whose kernels land in later commits.
#include "internal.h"
using namespace ss;
extern "C" {
ss_status ss_batch_plan_size(int, const ss_csr *, int, size_t *, size_t *) { return fail(SS_ERR_INVALID_ARG, "batched not built"); }
ss_status ss_batch_plan(int, const ss_csr *, int, const void *const *, void *const *, int, const ss_knobs *, void *, size_t, void *, size_t, void *) { return fail(SS_ERR_INVALID_ARG, "batched not built"); }
ss_status ss_spmm_batched(const void *, size_t, void *) { return fail(SS_ERR_INVALID_ARG, "batched not built"); }
}
