"""Seeded random cases at the workload configurations' scale (1e5 to 2.5e6
rows and columns, up to about 1e7 nonzeros), where size thresholds of the
kernels come into play: more column buckets than a transpose block has
threads, grids capped at the resident wave with workers striding over the
chunks, rows longer than the compensation threshold, two column slices per
lane group.  Each case checks, against the oracle:
  * SpMM with the autotuner's pick and with each strategy's default knobs,
    FP32 C within 1e-5 of the sum of |terms| elementwise and normwise
    (16-bit storage: against FP64 on the rounded inputs, the same bar);
  * the device transpose bit for bit (stable counting sort);
  * SDDMM and the fused backward (dB = A^T dC, dA.values) within 1e-5.

Every case is generated on the host from its seed, so a failure names a
case that reproduces."""
import os

import numpy as np
import pytest
import torch

import oracle_lib
from gpu_util import check_close, rounded
from segscan_gb300 import api, autotune, synth

pytestmark = pytest.mark.gpu
THREADS = max(1, os.cpu_count() or 1)


def case(seed):
    rng = np.random.default_rng(9100 + seed)
    M = int(np.exp(rng.uniform(np.log(1e5), np.log(2.5e6))))
    K = int(np.exp(rng.uniform(np.log(1e5), np.log(2.5e6))))
    kind = seed % 4
    if kind == 0:  # power-law rows with long ones past the compensation threshold
        L = np.clip(rng.zipf(rng.uniform(1.9, 2.4), size=M), 1, int(rng.integers(2000, 30000)))
    elif kind == 1:  # Poisson rows, dense enough for many column buckets
        L = rng.poisson(rng.uniform(2.0, 6.0), size=M)
    elif kind == 2:  # mostly empty rows
        L = np.where(rng.random(M) < 0.7, 0, rng.integers(1, 30, size=M))
    else:  # constant rows
        L = np.full(M, int(rng.integers(1, 9)))
    L = np.minimum(L, K)
    scale = max(1.0, L.sum() / 1.0e7)  # at most about 1e7 nonzeros
    if scale > 1.0:
        L = np.floor(L / scale).astype(np.int64)
    A = synth.csr_from_lengths(M, K, L, rng)
    N = [64, 16, 128, 33, 160, 4, 64, 1][seed % 8]
    dt = [torch.float32, torch.bfloat16, torch.float32, torch.float16][seed % 4 if seed % 3 else 0]
    return A, N, dt, rng


@pytest.mark.parametrize("seed", range(8))
def test_scale_fuzz(cuda, seed):
    A, N, dt, rng = case(seed)
    what = f"seed {seed}: {A.nrow}x{A.ncol} nnz {A.nnz} N {N} {dt}"
    vals_h = A.values if dt == torch.float32 else rounded(A.values, dt)
    B = synth.dense(A.ncol, N, seed=seed)
    B_h = B if dt == torch.float32 else rounded(B, dt)
    Ad = api.CsrMatrix.from_host(A, torch.device("cuda"), dt)
    Bd = torch.from_numpy(B).cuda().to(dt)

    # SpMM: the autotuner's pick and every strategy at its defaults
    C64, absC = oracle_lib.spmm_f64(A.indptr, A.indices, vals_h, B_h, threads=THREADS)
    runs = [autotune.best(Ad, N, Bd)] + [(s, None) for s in ("ebsr", "ebpr", "rbsr", "rbpr")]
    for strategy, knobs in runs:
        C = api.spmm(Ad, Bd, strategy, knobs=knobs)
        torch.cuda.synchronize()
        got = C.float().cpu().numpy()
        del C
        check_close(got, C64, absC, 1e-5, 1e-5, f"{what} spmm {strategy}")
    del C64, absC

    # transpose, bit for bit
    AT, perm = api.transpose(Ad)
    torch.cuda.synchronize()
    t_indptr, t_indices, operm = oracle_lib.csr_transpose(A.indptr, A.indices, A.ncol)
    assert np.array_equal(AT.indptr.cpu().numpy(), t_indptr), f"{what}: t_indptr"
    assert np.array_equal(AT.indices.cpu().numpy(), t_indices), f"{what}: t_indices"
    assert np.array_equal(perm.cpu().numpy(), operm), f"{what}: perm"

    # SDDMM and the fused backward
    dC = rng.standard_normal((A.nrow, N)).astype(np.float32)
    dCd = torch.from_numpy(dC).cuda()
    dv64, dvabs = oracle_lib.sddmm_f64(A.indptr, A.indices, dC, B_h)
    sd = api.sddmm(Ad, dCd, Bd)
    torch.cuda.synchronize()
    check_close(sd.cpu().numpy(), dv64, dvabs, 1e-5, 1e-5, f"{what} sddmm")
    if N <= api.spmm_backward_limit(N):
        dvals, dB = api.spmm_backward(AT, perm, Ad.values, dCd, Bd)
        torch.cuda.synchronize()
        check_close(dvals.cpu().numpy(), dv64, dvabs, 1e-5, 1e-5, f"{what} fused dvals")
        dB64, absdB = oracle_lib.spmm_f64(t_indptr, t_indices, vals_h[operm], dC, threads=THREADS)
        check_close(dB.float().cpu().numpy(), dB64, absdB, 1e-5, 1e-5, f"{what} fused dB")
