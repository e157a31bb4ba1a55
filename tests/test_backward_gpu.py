"""Backward pass: device transpose (bit-exact vs the reference's stable
counting sort), SDDMM (vs FP64) and the autograd binding (vs FP64 central
finite differences and a dense FP64 gradient).  FP32 tolerance: 1e-6 of
sum|terms| for gradients, 1e-5 for SDDMM."""
from pathlib import Path

import numpy as np
import pytest
import torch

import oracle_lib
from gpu_util import check_close, dev_csr, powerlaw_medium, rounded
from segscan_gb300 import synth

pytestmark = pytest.mark.gpu
GOLD = Path(__file__).resolve().parent / "golden"


def test_transpose_golden(cuda):
    from segscan_gb300 import api
    g = np.load(GOLD / "transpose_edge.npz")
    csr = synth.Csr(g["indptr"].size - 1, int(g["ncol"]), g["indptr"], g["indices"],
                    np.arange(g["indices"].size, dtype=np.float32))
    AT, perm = api.transpose(dev_csr(csr))
    torch.cuda.synchronize()
    assert np.array_equal(AT.indptr.cpu().numpy(), g["t_indptr"])
    assert np.array_equal(AT.indices.cpu().numpy(), g["t_indices"])
    _, _, operm = oracle_lib.csr_transpose(g["indptr"], g["indices"], int(g["ncol"]))
    assert np.array_equal(perm.cpu().numpy(), operm)
    assert np.array_equal(AT.values.cpu().numpy(), operm.astype(np.float32))  # values follow perm


def long_column_matrix():
    """Column 0 in 20000 rows (global-memory sort), columns 1..40 in ~2000
    rows each (shared-memory sort), the rest short."""
    rng = np.random.default_rng(9)
    M, K = 30000, 5000
    rows, cols = [], []
    r0 = rng.choice(M, 20000, replace=False)
    rows.append(r0); cols.append(np.zeros(r0.size, np.int64))
    for c in range(1, 41):
        r = rng.choice(M, int(rng.integers(33, 4000)), replace=False)
        rows.append(r); cols.append(np.full(r.size, c))
    r = rng.integers(0, M, 60000); rows.append(r); cols.append(rng.integers(41, K, r.size))
    return synth._build(M, K, np.concatenate(rows), np.concatenate(cols), rng)


@pytest.mark.parametrize("which", ["powerlaw", "long_columns", "many_buckets"])
def test_transpose_matches_oracle(cuda, which):
    """many_buckets: 1.1 M columns with about five nonzeros each go to more
    column buckets (1075) than a partition block has threads (1024), so
    each thread reserves ranges for two buckets."""
    from segscan_gb300 import api
    if which == "powerlaw":
        csr = powerlaw_medium()
    elif which == "long_columns":
        csr = long_column_matrix()
    else:
        csr = synth.poisson(1_100_000, 1_100_000, 5.0, seed=12)
    A = dev_csr(csr)
    AT, perm = api.transpose(A)
    AT2, perm2 = api.transpose(A)
    torch.cuda.synchronize()
    t_indptr, t_indices, operm = oracle_lib.csr_transpose(csr.indptr, csr.indices, csr.ncol)
    assert np.array_equal(AT.indptr.cpu().numpy(), t_indptr)
    assert np.array_equal(AT.indices.cpu().numpy(), t_indices)
    assert np.array_equal(perm.cpu().numpy(), operm)
    assert torch.equal(perm, perm2) and torch.equal(AT.indices, AT2.indices)
    assert np.array_equal(AT.values.cpu().numpy(), csr.values[operm])


@pytest.mark.parametrize("N", [1, 3, 8, 64, 128, 160, 256])
@pytest.mark.parametrize("dtype", [torch.float32, torch.bfloat16])
def test_sddmm(cuda, N, dtype):
    """N of 128 and more take the whole-warp kernel; 160 and 256 walk two
    column slices (160: the second one partly idle)."""
    from segscan_gb300 import api
    csr = powerlaw_medium(M=20000, lmax=3000)
    rng = np.random.default_rng(N)
    dC = rng.standard_normal((csr.nrow, N)).astype(np.float32)
    B = synth.dense(csr.ncol, N, seed=N)
    out = api.sddmm(dev_csr(csr, dtype), torch.from_numpy(dC).cuda(), torch.from_numpy(B).cuda().to(dtype))
    torch.cuda.synchronize()
    ref, absref = oracle_lib.sddmm_f64(csr.indptr, csr.indices, dC, rounded(B, dtype))
    check_close(out.cpu().numpy(), ref, absref, 1e-5, 1e-5, f"sddmm N={N} {dtype}")


def row_submatrix(csr, rows):
    """The rows [0, rows) of csr with all their nonzeros (a row-induced submatrix)."""
    end = int(csr.indptr[rows])
    return synth.Csr(rows, csr.ncol, csr.indptr[:rows + 1].copy(), csr.indices[:end].copy(),
                     csr.values[:end].copy())


def loss64(csr, vals, B, W):
    C, _ = oracle_lib.spmm_f64(csr.indptr, csr.indices, vals, B)
    return float((C * W).sum())


def test_autograd_finite_differences(cuda):
    """2,000-row submatrix of a power-law matrix (Zipf 2.1, clip 50000), N = 8:
    the analytic gradients of L = sum(W * (A @ B)) match FP64 central finite
    differences on sampled parameters to 1e-6 of the summed |terms|."""
    from segscan_gb300 import autograd
    big = synth.powerlaw(200_000, 200_000, 2.1, 1, 50000, seed=4)
    csr = row_submatrix(big, 2000)
    N = 8
    rng = np.random.default_rng(4)
    B = synth.dense(csr.ncol, N, seed=44)
    W = rng.standard_normal((csr.nrow, N)).astype(np.float32)
    A = dev_csr(csr, values=False)
    vals = torch.from_numpy(csr.values.copy()).cuda().requires_grad_(True)
    Bd = torch.from_numpy(B).cuda().requires_grad_(True)
    C = autograd.spmm(A, vals, Bd)
    (C * torch.from_numpy(W).cuda()).sum().backward()
    gv = vals.grad.cpu().numpy().astype(np.float64)
    gB = Bd.grad.cpu().numpy().astype(np.float64)
    h = 1e-3
    rows = np.repeat(np.arange(csr.nrow), csr.row_lengths())
    for p in rng.choice(csr.nnz, 150, replace=False):
        vp, vm = csr.values.astype(np.float64).copy(), csr.values.astype(np.float64).copy()
        vp[p] += h; vm[p] -= h
        fd = (loss64(csr, vp.astype(np.float32), B, W) - loss64(csr, vm.astype(np.float32), B, W)) / (2 * h)
        # linear in the value: the FD of the FP64 loss is exact up to rounding of vals +- h in FP32
        exact = float(np.dot(W[rows[p]].astype(np.float64), B[csr.indices[p]].astype(np.float64)))
        scale = float(np.abs(W[rows[p]] * B[csr.indices[p]]).sum())
        assert abs(gv[p] - exact) <= 1e-6 * scale + 1e-12, p
        assert abs(fd - exact) <= 1e-3 * scale + 1e-9  # h rounding in FP32 inputs
    cols_used = np.unique(csr.indices)
    AT_rows = {}
    for k in rng.choice(cols_used, 100, replace=False):
        for j in rng.choice(N, 2, replace=False):
            sel = csr.indices == k
            exact = float((csr.values[sel].astype(np.float64) * W[rows[sel], j].astype(np.float64)).sum())
            scale = float(np.abs(csr.values[sel] * W[rows[sel], j]).sum())
            Bp, Bm = B.astype(np.float64).copy(), B.astype(np.float64).copy()
            Bp[k, j] += h; Bm[k, j] -= h
            fd = (loss64(csr, csr.values, Bp.astype(np.float32), W) - loss64(csr, csr.values, Bm.astype(np.float32), W)) / (2 * h)
            assert abs(gB[k, j] - exact) <= 1e-6 * scale + 1e-12, (k, j)
            assert abs(fd - exact) <= 1e-3 * scale + 1e-9
    # columns of B that A never touches get exactly zero gradient
    unused = np.setdiff1d(np.arange(min(csr.ncol, 50000)), cols_used)[:1000]
    assert not gB[unused].any()


@pytest.mark.parametrize("dtype", [torch.float32, torch.bfloat16])
def test_autograd_dense_reference(cuda, dtype):
    from segscan_gb300 import autograd
    csr = synth.poisson(300, 500, 7.0, seed=12)
    N = 16
    rng = np.random.default_rng(12)
    B = synth.dense(500, N, seed=13)
    W = rng.standard_normal((300, N)).astype(np.float32)
    A = dev_csr(csr, values=False)
    vals = torch.from_numpy(csr.values.copy()).cuda().to(dtype).requires_grad_(True)
    Bd = torch.from_numpy(B).cuda().to(dtype).requires_grad_(True)
    C = autograd.spmm(A, vals, Bd)
    (C.float() * torch.from_numpy(W).cuda()).sum().backward()
    # dense FP64 reference on the stored (rounded) inputs
    v64 = rounded(csr.values, dtype).astype(np.float64)
    B64 = rounded(B, dtype).astype(np.float64)
    Ad = np.zeros((300, 500))
    rows = np.repeat(np.arange(300), csr.row_lengths())
    Ad[rows, csr.indices] = v64
    W64 = W.astype(np.float64)
    gB_ref = Ad.T @ W64
    gv_ref = (W64 @ B64.T)[rows, csr.indices]
    tol = 1e-6 if dtype == torch.float32 else 2.0 ** -8
    sB = np.abs(Ad.T) @ np.abs(W64)
    sv = (np.abs(W64) @ np.abs(B64.T))[rows, csr.indices]
    assert np.all(np.abs(Bd.grad.float().cpu().numpy() - gB_ref) <= tol * (sB + np.abs(gB_ref)) + 1e-12)
    assert np.all(np.abs(vals.grad.float().cpu().numpy() - gv_ref) <= tol * (sv + np.abs(gv_ref)) + 1e-12)


@pytest.mark.parametrize("case", ["sorted", "shuffled", "skewed", "out_of_range", "empty"])
def test_coo_to_csr(cuda, case):
    """Device COO -> CSR: the stable counting sort by row (compressedRow,
    dataloader.hpp:109-121, on sorted input), bit for bit against numpy's
    stable argsort; rows outside [0, nrow) are left out."""
    from segscan_gb300 import api
    rng = np.random.default_rng(7)
    nrow, nnz = 5000, 60000
    rows = rng.integers(0, nrow, size=nnz).astype(np.int32)
    if case == "sorted":
        rows = np.sort(rows)
    elif case == "skewed":
        rows[: nnz // 2] = 17  # one row with half the entries (global-memory sort path)
        rng.shuffle(rows)
    elif case == "out_of_range":
        rows[::97] = nrow + 3
        rows[::89] = -1
    elif case == "empty":
        rows = rows[:0]
    cols = rng.integers(0, 4000, size=rows.size).astype(np.int32)
    vals = rng.standard_normal(rows.size).astype(np.float32)
    A, perm = api.coo_to_csr(nrow, torch.from_numpy(rows).cuda(), torch.from_numpy(cols).cuda(), ncol=4000,
                             values=torch.from_numpy(vals).cuda())
    torch.cuda.synchronize()
    valid = (rows >= 0) & (rows < nrow)
    order = np.nonzero(valid)[0][np.argsort(rows[valid], kind="stable")].astype(np.int32)
    indptr = np.concatenate([[0], np.cumsum(np.bincount(rows[valid], minlength=nrow))]).astype(np.int32)
    m = int(valid.sum())
    assert np.array_equal(A.indptr.cpu().numpy(), indptr)
    assert np.array_equal(perm.cpu().numpy()[:m], order)
    assert np.array_equal(A.indices.cpu().numpy()[:m], cols[order])
    assert np.array_equal(A.values.cpu().numpy()[:m], vals[order])


@pytest.mark.parametrize("N", [1, 3, 8, 64, 128, 256])
@pytest.mark.parametrize("dtype", [torch.float32, torch.bfloat16])
@pytest.mark.parametrize("which", ["powerlaw", "long_columns"])
def test_fused_backward(cuda, N, dtype, which):
    """ss_spmm_backward against FP64: dB = A^T dC and dvals = SDDMM(dC, B)
    within 1e-5 of sum|terms| (on the values and B the kernel reads); for
    FP32, dB bit-identical to rbsr on A^T with the gathered values (both sum
    each row of A^T in position order)."""
    from segscan_gb300 import api
    csr = powerlaw_medium() if which == "powerlaw" else long_column_matrix()
    A = dev_csr(csr, dtype)
    B = synth.dense(csr.ncol, N, seed=N + 3)
    dC = synth.dense(csr.nrow, N, seed=N + 4)
    Bd = torch.from_numpy(B).cuda().to(dtype)
    dCd = torch.from_numpy(dC).cuda()
    AT, perm = api.transpose(A)
    dvals, dB = api.spmm_backward(AT, perm, A.values, dCd, Bd)
    torch.cuda.synchronize()
    vals = rounded(csr.values, dtype) if dtype != torch.float32 else csr.values
    Bh = rounded(B, dtype) if dtype != torch.float32 else B
    t_indptr, t_indices, operm = oracle_lib.csr_transpose(csr.indptr, csr.indices, csr.ncol)
    dB64, dBabs = oracle_lib.spmm_f64(t_indptr, t_indices, vals[operm], dC)
    dv64, dvabs = oracle_lib.sddmm_f64(csr.indptr, csr.indices, dC, Bh)
    check_close(dB.cpu().numpy(), dB64, dBabs, 1e-5, 1e-5, f"fused dB {which} N={N} {dtype}")
    check_close(dvals.cpu().numpy(), dv64, dvabs, 1e-5, 1e-5, f"fused dvals {which} N={N} {dtype}")
    if dtype == torch.float32:
        AT_v = AT.with_values(api.gather_values(A.values, perm))
        ref = api.spmm(AT_v, dCd, "rbsr", knobs=api.make_knobs("rbsr", N, coarsen_factor=4, tile_factor=7))
        torch.cuda.synchronize()
        assert torch.equal(dB, ref), f"fused dB differs from rbsr on A^T ({which}, N={N})"


def test_fused_backward_wide_refused(cuda):
    """N above the fused walk's width is refused before any launch."""
    from segscan_gb300 import api
    from segscan_gb300._lib import SegscanError
    csr = synth.poisson(100, 80, 3.0, seed=1)
    A = dev_csr(csr)
    AT, perm = api.transpose(A)
    N = 260
    with pytest.raises(SegscanError):
        api.spmm_backward(AT, perm, A.values, torch.zeros((100, N), device="cuda"),
                          torch.zeros((80, N), device="cuda"))
