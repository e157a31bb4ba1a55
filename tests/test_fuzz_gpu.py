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
    dt = [torch.float32, torch.float32, torch.float32, torch.bfloat16, torch.float16][int(rng.integers(0, 5))]
    strategy = ["ebsr", "ebpr", "rbsr", "rbpr"][int(rng.integers(0, 4))]
    acts = [k for s, k in sweep.library_actions(N, dt) if s == strategy]
    knobs = acts[int(rng.integers(0, len(acts)))]
    accumulate = bool(rng.random() < 0.2)
    # C: FP32, or the 16-bit storage type, or (ebsr only) 16-bit from FP32 inputs
    c16 = [torch.bfloat16, torch.float16][int(rng.integers(0, 2))] if dt == torch.float32 else dt
    cdt = c16 if (rng.random() < 0.3 and (dt != torch.float32 or strategy == "ebsr")) else torch.float32
    return A, N, dt, cdt, strategy, knobs, accumulate, kind, rng


# one output rounding: half an ulp of the 16-bit type, relative (FP16 also
# absolute for its subnormals)
C_ROUND = {torch.float32: (0.0, 0.0), torch.bfloat16: (2.0 ** -8, 0.0), torch.float16: (2.0 ** -11, 2.0 ** -24)}


@pytest.mark.parametrize("seed", range(64))
def test_spmm_fuzz(cuda, seed):
    A, N, dt, cdt, strategy, knobs, accumulate, kind, rng = spmm_case(seed)
    B = synth.dense(A.ncol, N, seed=seed)
    vals = rounded(A.values, dt) if dt != torch.float32 else A.values
    Bc = rounded(B, dt) if dt != torch.float32 else B
    Ad = api.CsrMatrix.from_host(A, "cuda", dt)
    Bd = torch.from_numpy(B).cuda().to(dt)
    C0 = rounded(synth.dense(A.nrow, N, seed=seed + 1), cdt) if accumulate else None
    out = torch.from_numpy(C0).cuda().to(cdt) if accumulate else torch.full((A.nrow, N), float("nan"),
                                                                             dtype=cdt, device="cuda")
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
    what = (f"seed {seed}: M={A.nrow} K={A.ncol} nnz={A.nnz} kind={kind} N={N} storage={dt} C={cdt} "
            f"{sweep.label(strategy, knobs)} accumulate={accumulate}")
    rel, ab = C_ROUND[cdt]
    check_close(out.float().cpu().numpy(), C64, absC + rel * np.abs(C64) / 1e-5, 1e-5, None, what, atol=ab)


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
    out = torch.full((dst_len, N), float("nan"), device="cuda")  # a row nobody stores shows up
    api.segment(srcd, torch.from_numpy(index).cuda(), dst_len, reduce, strategy, out=out)
    torch.cuda.synchronize()
    ref, dabs = oracle_lib.segment_coo_f64(rounded(src, dt) if bf16 else src, index, dst_len,
                                           {"sum": 0, "max": 1, "mean": 2}[reduce])
    what = f"seed {seed}: segments={segs} nnz={index.size} kind={kind} N={N} {reduce} {strategy} bf16={bf16}"
    got = out.cpu().numpy()
    if reduce == "max":
        assert np.array_equal(got.astype(np.float64), ref), what
    else:
        check_close(got, ref, dabs, 1e-5, None, what)


@pytest.mark.parametrize("seed", range(24))
def test_transpose_and_sddmm_fuzz(cuda, seed):
    """Random matrices: the device transpose is bit-exact against a stable
    argsort by column (pattern, permutation, gathered values), and SDDMM is
    within 1e-5 of FP64 dot products."""
    rng = np.random.default_rng(11000 + seed)
    M, K = int(rng.integers(1, 5000)), int(rng.integers(1, 5000))
    L, kind = lengths_for(rng, M, K)
    A = synth.csr_from_lengths(M, K, L, rng)
    Ad = api.CsrMatrix.from_host(A, "cuda")
    AT, perm = api.transpose(Ad)
    order = np.argsort(A.indices, kind="stable")
    rows_of = np.repeat(np.arange(M, dtype=np.int32), np.diff(A.indptr))
    exp_indptr = np.zeros(K + 1, np.int64)
    np.cumsum(np.bincount(A.indices, minlength=K), out=exp_indptr[1:])
    what = f"seed {seed}: M={M} K={K} nnz={A.nnz} kind={kind}"
    assert np.array_equal(AT.indptr.cpu().numpy(), exp_indptr.astype(np.int32)), what
    assert np.array_equal(AT.indices.cpu().numpy(), rows_of[order]), what
    assert np.array_equal(perm.cpu().numpy(), order.astype(np.int32)), what
    assert np.array_equal(AT.values.cpu().numpy(), A.values[order]), what
    N = int(rng.choice(WIDTHS))
    dC = synth.dense(M, N, seed=seed + 3)
    B = synth.dense(K, N, seed=seed + 4)
    got = api.sddmm(Ad, torch.from_numpy(dC).cuda(), torch.from_numpy(B).cuda()).cpu().numpy()
    x = dC[rows_of].astype(np.float64) * B[A.indices].astype(np.float64)
    check_close(got, x.sum(axis=1), np.abs(x).sum(axis=1), 1e-5, None, f"SDDMM {what} N={N}")


@pytest.mark.parametrize("seed", range(12))
def test_batched_fuzz(cuda, seed):
    """Random batches (2-40 matrices of random shapes, widths and chunk
    targets) in one persistent launch, each matrix against FP64."""
    from segscan_gb300 import autotune, batched
    rng = np.random.default_rng(13000 + seed)
    count = int(rng.integers(2, 41))
    N = int(rng.choice([1, 4, 8, 16, 32, 33, 64, 128]))
    mats_h = []
    for _ in range(count):
        M, K = int(rng.integers(1, 3000)), int(rng.integers(1, 3000))
        L, _ = lengths_for(rng, M, K)
        mats_h.append(synth.csr_from_lengths(M, K, L, rng))
    mats = [api.CsrMatrix.from_host(A, "cuda") for A in mats_h]
    Bs_h = [synth.dense(A.ncol, N, seed=seed * 100 + i) for i, A in enumerate(mats_h)]
    Bs = [torch.from_numpy(B).cuda() for B in Bs_h]
    target = int(rng.choice([128, 256, 512, 1024]))
    plan = batched.BatchedSpMM(mats, Bs, knobs=autotune.batch_knobs(mats, N, target))
    plan.run()
    torch.cuda.synchronize()
    for i, (A, B) in enumerate(zip(mats_h, Bs_h)):
        C64, absC = oracle_lib.spmm_f64(A.indptr, A.indices, A.values, B)
        check_close(plan.out[i].cpu().numpy(), C64, absC, 1e-5, None,
                    f"seed {seed}: matrix {i} of {count} ({A.nrow}x{A.ncol}, nnz {A.nnz}) N={N} target={target}")


@pytest.mark.parametrize("seed", range(12))
def test_coo_to_csr_fuzz(cuda, seed):
    """Random COO (shuffled, skewed, some rows out of range) to CSR, bit for
    bit against a stable argsort by row."""
    rng = np.random.default_rng(15000 + seed)
    nrow = int(rng.integers(1, 40000))
    nnz = int(rng.integers(0, 300000))
    rows = rng.integers(0, nrow, size=nnz).astype(np.int32)
    if nnz and rng.random() < 0.5:  # one heavy row
        rows[rng.random(nnz) < rng.uniform(0.05, 0.6)] = int(rng.integers(0, nrow))
    if nnz and rng.random() < 0.3:  # entries outside [0, nrow) are left out
        bad = rng.random(nnz) < 0.02
        rows[bad] = np.where(rng.random(int(bad.sum())) < 0.5, -1, nrow + 5)
    ncol = int(rng.integers(1, 50000))
    cols = rng.integers(0, ncol, size=nnz).astype(np.int32)
    vals = rng.standard_normal(nnz).astype(np.float32)
    A, perm = api.coo_to_csr(nrow, torch.from_numpy(rows).cuda(), torch.from_numpy(cols).cuda(), ncol=ncol,
                             values=torch.from_numpy(vals).cuda())
    torch.cuda.synchronize()
    valid = (rows >= 0) & (rows < nrow)
    order = np.nonzero(valid)[0][np.argsort(rows[valid], kind="stable")].astype(np.int32)
    indptr = np.concatenate([[0], np.cumsum(np.bincount(rows[valid], minlength=nrow))]).astype(np.int32)
    m = int(valid.sum())
    what = f"seed {seed}: nrow={nrow} nnz={nnz} valid={m}"
    assert np.array_equal(A.indptr.cpu().numpy(), indptr), what
    assert np.array_equal(perm.cpu().numpy()[:m], order), what
    assert np.array_equal(A.indices.cpu().numpy()[:m], cols[order]), what
    assert np.array_equal(A.values.cpu().numpy()[:m], vals[order]), what
