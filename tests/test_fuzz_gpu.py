"""Seeded random cases across shapes, row-length distributions, widths,
storage types, strategies and knob tuples, each checked against the FP64
oracle: SpMM within 1e-5 of the sum of |terms| elementwise (FP32 and, on
the rounded inputs, BF16 storage), segment_coo the same (max exactly).

Every case is generated on the host from its seed, so a failure names a
case that reproduces."""
import numpy as np
import pytest
import torch

import oracle_lib
from gpu_util import check_close, rounded
from segscan_gb300 import api, synth, sweep

pytestmark = pytest.mark.gpu

WIDTHS = [1, 2, 3, 4, 5, 8, 12, 16, 17, 32, 33, 48, 64, 96, 128, 130]


def lengths_for(rng, M, K):
    kind = rng.integers(0, 5)
    if kind == 0:  # Poisson rows
        L = rng.poisson(rng.uniform(0.5, 40.0), size=M)
    elif kind == 1:  # power law, up to a few thousand per row
        L = np.clip(rng.zipf(rng.uniform(1.6, 3.0), size=M), 1, int(rng.integers(10, 4000)))
    elif kind == 2:  # mostly empty rows
        L = np.where(rng.random(M) < 0.8, 0, rng.integers(1, 60, size=M))
    elif kind == 3:  # one very long row among short ones
        L = rng.integers(0, 6, size=M)
        L[rng.integers(0, M)] = int(rng.integers(2000, 9000))
    else:  # constant rows
        L = np.full(M, int(rng.integers(1, 33)))
    return np.minimum(L, K), int(kind)


def spmm_case(seed):
    rng = np.random.default_rng(7000 + seed)
    M, K = int(rng.integers(1, 6000)), int(rng.integers(1, 6000))
    L, kind = lengths_for(rng, M, K)
    A = synth.csr_from_lengths(M, K, L, rng)
    N = int(rng.choice(WIDTHS))
    bf16 = bool(rng.random() < 0.25)
    strategy = ["ebsr", "ebpr", "rbsr", "rbpr"][int(rng.integers(0, 4))]
    acts = [k for s, k in sweep.library_actions(N, torch.bfloat16 if bf16 else torch.float32) if s == strategy]
    knobs = acts[int(rng.integers(0, len(acts)))]
    accumulate = bool(rng.random() < 0.2)
    return A, N, bf16, strategy, knobs, accumulate, kind, rng


@pytest.mark.parametrize("seed", range(64))
def test_spmm_fuzz(cuda, seed):
    A, N, bf16, strategy, knobs, accumulate, kind, rng = spmm_case(seed)
    B = synth.dense(A.ncol, N, seed=seed)
    dt = torch.bfloat16 if bf16 else torch.float32
    vals = rounded(A.values, dt) if bf16 else A.values
    Bc = rounded(B, dt) if bf16 else B
    Ad = api.CsrMatrix.from_host(A, "cuda", dt)
    Bd = torch.from_numpy(B).cuda().to(dt)
    C0 = synth.dense(A.nrow, N, seed=seed + 1) if accumulate else None
    out = torch.from_numpy(C0).cuda() if accumulate else torch.full((A.nrow, N), float("nan"), device="cuda")
    try:
        api.spmm(Ad, Bd, strategy, knobs=knobs, out=out, accumulate=accumulate)
    except api._lib.SegscanError as exc:  # a tuple the geometry rejects is refused, not computed
        assert exc.status == api._lib.Status.UNSUPPORTED_KNOBS, exc
        return
    torch.cuda.synchronize()
    C64, absC = oracle_lib.spmm_f64(A.indptr, A.indices, vals, Bc)
    if accumulate:
        C64 = C64 + C0
        absC = absC + np.abs(C0)
    what = (f"seed {seed}: M={A.nrow} K={A.ncol} nnz={A.nnz} kind={kind} N={N} bf16={bf16} "
            f"{sweep.label(strategy, knobs)} accumulate={accumulate}")
    check_close(out.cpu().numpy(), C64, absC, 1e-5, None, what)


@pytest.mark.parametrize("seed", range(48))
def test_segment_fuzz(cuda, seed):
    rng = np.random.default_rng(9000 + seed)
    segs = int(rng.integers(1, 5000))
    L, kind = lengths_for(rng, segs, 1 << 30)
    index = np.repeat(np.arange(segs, dtype=np.int32), L)
    dst_len = segs + int(rng.integers(0, 20))
    N = int(rng.choice(WIDTHS))
    reduce = ["sum", "max", "mean"][int(rng.integers(0, 3))]
    strategy = ["sr", "pr"][int(rng.integers(0, 2))]
    bf16 = bool(rng.random() < 0.25)
    src = synth.dense(index.size, N, seed=seed)
    dt = torch.bfloat16 if bf16 else torch.float32
    srcd = torch.from_numpy(src).cuda().to(dt)
    out = api.segment(srcd, torch.from_numpy(index).cuda(), dst_len, reduce, strategy)
    torch.cuda.synchronize()
    ref, dabs = oracle_lib.segment_coo_f64(rounded(src, dt) if bf16 else src, index, dst_len,
                                           {"sum": 0, "max": 1, "mean": 2}[reduce])
    what = f"seed {seed}: segments={segs} nnz={index.size} kind={kind} N={N} {reduce} {strategy} bf16={bf16}"
    got = out.cpu().numpy()
    if reduce == "max":
        assert np.array_equal(got.astype(np.float64), ref), what
    else:
        check_close(got, ref, dabs, 1e-5, None, what)
