"""Operands past 2^31 elements.

The reference computes every dense offset in `int` (row * ldC, k * ldB in
spmm_cg.cuh and dst offsets in segscan.cuh), so its kernels cannot address
a C, B or src of more than 2^31 elements.  This library's offsets are
64-bit: here M = K = 34,000,000 rows at N = 64 (2.18e9 elements, 8.7 GB per
dense operand), with nonzeros in rows and columns on both sides of
2^31 / N = 33,554,432.  Every written row is checked against the FP64
oracle and every other row must read exactly zero (C starts as NaN, so a
row the kernel never wrote shows up)."""
import numpy as np
import pytest
import torch

import oracle_lib
from gpu_util import check_close
from segscan_gb300 import api, synth

pytestmark = pytest.mark.gpu

M = K = 34_000_000
N = 64
EDGE = (1 << 31) // N  # first row whose offset row * N exceeds 2^31


@pytest.fixture(scope="module")
def big(cuda):
    rng = np.random.default_rng(40)
    rows = np.array([0, 1, 5_000_000, EDGE - 2, EDGE - 1, EDGE, EDGE + 1, M - 3, M - 2, M - 1])
    lengths = np.zeros(M, np.int64)
    lengths[rows] = rng.integers(1, 40, size=rows.size)
    lengths[M - 3] = 3000  # a long row: chunks straddle it
    lengths[EDGE - 1] = 1500
    indptr = np.zeros(M + 1, np.int64)
    np.cumsum(lengths, out=indptr[1:])
    nnz = int(indptr[-1])
    cols = np.empty(nnz, np.int64)
    half = nnz // 2
    cols[:half] = rng.integers(EDGE - 1000, K, size=half)  # columns whose B offset exceeds 2^31
    cols[half:] = rng.integers(0, K, size=nnz - half)
    rng.shuffle(cols)
    for r in rows:  # distinct sorted columns per row
        s, e = indptr[r], indptr[r + 1]
        u = np.unique(cols[s:e])
        while u.size < e - s:
            u = np.unique(np.concatenate([u, rng.integers(0, K, size=e - s - u.size)]))
        cols[s:e] = u
    vals = rng.uniform(-1, 1, size=nnz).astype(np.float32)
    A = synth.Csr(M, K, indptr.astype(np.int32), cols.astype(np.int32), vals)
    Ad = api.CsrMatrix.from_host(A, "cuda")
    g = torch.Generator(device="cuda")
    g.manual_seed(41)
    B = torch.empty((K, N), device="cuda")
    B.uniform_(-1, 1, generator=g)
    # the oracle's problem: the nonempty rows, over the B rows they touch
    ucols, inv = np.unique(cols, return_inverse=True)
    Bg = B[torch.from_numpy(ucols).cuda()].cpu().numpy()
    small = synth.Csr(rows.size, ucols.size, np.concatenate([[0], np.cumsum(lengths[rows])]).astype(np.int32),
                      inv.astype(np.int32), vals)
    C64, absC = oracle_lib.spmm_f64(small.indptr, small.indices, small.values, Bg)
    return dict(A=A, Ad=Ad, B=B, rows=rows, C64=C64, absC=absC, ucols=ucols, inv=inv, Bg=Bg)


@pytest.mark.parametrize("strategy", ["ebsr", "ebpr", "rbsr", "rbpr"])
def test_spmm_past_2_31_elements(big, strategy):
    C = torch.full((M, N), float("nan"), device="cuda")
    api.spmm(big["Ad"], big["B"], strategy, out=C)
    torch.cuda.synchronize()
    idx = torch.from_numpy(big["rows"]).cuda()
    got = C[idx].cpu().numpy()
    check_close(got, big["C64"], big["absC"], 1e-5, None, f"{strategy} rows on both sides of 2^31/N")
    C[idx] = 0
    assert int(torch.count_nonzero(C)) == 0, f"{strategy}: rows without nonzeros are not all zero"
    del C
    torch.cuda.empty_cache()


def test_sddmm_past_2_31_elements(big):
    """dA.vals = rowwise dot(dC[row], B[col]); dC is B itself (M = K)."""
    A, B = big["A"], big["B"]
    out = api.sddmm(big["Ad"], B, B).cpu().numpy()
    rows_of = np.repeat(big["rows"], np.diff(A.indptr)[big["rows"]])
    dC = B[torch.from_numpy(rows_of).cuda()].cpu().numpy().astype(np.float64)
    Bc = big["Bg"][big["inv"]].astype(np.float64)
    ref = (dC * Bc).sum(axis=1)
    absref = (np.abs(dC) * np.abs(Bc)).sum(axis=1)
    check_close(out, ref, absref, 1e-5, None, "SDDMM past 2^31 elements")


def test_transpose_of_a_34m_row_matrix(big):
    """The transposed pattern, bit-exact against a stable argsort of the
    nonzeros by column."""
    A = big["A"]
    AT, perm = api.transpose(big["Ad"])
    rows_of = np.repeat(np.arange(M, dtype=np.int64), np.diff(A.indptr))
    order = np.argsort(A.indices, kind="stable")
    exp_indptr = np.zeros(K + 1, np.int64)
    np.cumsum(np.bincount(A.indices, minlength=K), out=exp_indptr[1:])
    assert np.array_equal(AT.indptr.cpu().numpy(), exp_indptr.astype(np.int32))
    assert np.array_equal(AT.indices.cpu().numpy(), rows_of[order].astype(np.int32))
    assert np.array_equal(perm.cpu().numpy(), order.astype(np.int32))


@pytest.mark.parametrize("strategy", ["sr", "pr"])
def test_segment_sum_past_2_31_elements(cuda, strategy):
    """src of 34,000,000 x 64 (2.18e9 elements) into 40,000 segments; the
    first and the last three segments are checked against FP64."""
    nnz, dst_len = M, 40_000
    g = torch.Generator(device="cuda")
    g.manual_seed(42)
    src = torch.empty((nnz, N), device="cuda")
    src.uniform_(-1, 1, generator=g)
    index = (torch.arange(nnz, device="cuda", dtype=torch.int64) * dst_len // nnz).to(torch.int32)
    out = api.segment(src, index, dst_len, "sum", strategy)
    torch.cuda.synchronize()
    bounds = np.searchsorted(np.arange(nnz, dtype=np.int64) * dst_len // nnz, np.arange(dst_len + 1))
    for seg in (0, dst_len - 3, dst_len - 2, dst_len - 1):
        s, e = int(bounds[seg]), int(bounds[seg + 1])
        x = src[s:e].cpu().numpy().astype(np.float64)
        check_close(out[seg].cpu().numpy()[None], x.sum(axis=0)[None], np.abs(x).sum(axis=0)[None], 1e-5, None,
                    f"segment {seg} ({strategy})")
    del src, index, out
    torch.cuda.empty_cache()
