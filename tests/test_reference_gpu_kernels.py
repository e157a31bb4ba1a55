"""This library against the reference's own CUDA kernels on the same GPU.

The reference's four SpMM kernels (test-cg/include/spmm/spmm_cg.cuh),
compiled for sm_103a from its sources (oracle/ref_gpu_kernels.cu, `make -C
oracle ref`), run through the driver API with the reference launchers'
geometry and README-best knobs at N = 64.  Both sides must land within the
SpMM tolerance of the FP64 oracle on the same inputs; the values of A are
small integers so rbsr's `int v` (spmm_cg.cuh:608) does not change its
result.  The timing test prints the reference kernels' times beside this
library's for the power-law 1e6 x 1e6 workload (C zeroing included for the
reference's atomic strategies, as its driver does at test.cu:58-82)."""
import json

import numpy as np
import pytest
import torch

from gpu_util import check_close, dev_csr, oracle64
from ref_kernels import RefKernels
from segscan_gb300 import api, synth

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(not RefKernels.available(), reason="reference kernels not built (needs the "
                                                                   "reference checkout at build time)")]

N = 64


def integer_valued(csr, seed):
    rng = np.random.default_rng(seed)
    vals = rng.integers(1, 4, size=csr.nnz).astype(np.float32)
    return synth.Csr(csr.nrow, csr.ncol, csr.indptr, csr.indices, vals)


@pytest.fixture(scope="module")
def ref(cuda):
    return RefKernels()


@pytest.mark.parametrize("strategy", ["ebpr", "rbpr", "ebsr", "rbsr"])
def test_reference_kernels_match_ours(ref, strategy):
    A = integer_valued(synth.powerlaw(30000, 30000, 2.1, 1, 3000, seed=21), 22)
    B = synth.dense(A.ncol, N, seed=23)
    Ad = dev_csr(A)
    Bd = torch.from_numpy(B).cuda()
    C_ref = torch.zeros((A.nrow, N), device="cuda")
    ref.launch(strategy, A.nrow, A.ncol, A.nnz, Ad.indptr, Ad.indices, Ad.values, Bd, C_ref)
    C_ours = api.spmm(Ad, Bd, strategy)
    torch.cuda.synchronize()
    C64, absC = oracle64(A, B)
    check_close(C_ref.cpu().numpy(), C64, absC, 1e-5, None, f"reference {strategy} kernel vs FP64")
    check_close(C_ours.cpu().numpy(), C64, absC, 1e-5, None, f"segscan_gb300 {strategy} vs FP64")


def _ms(fn, iters=10):
    fn()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(iters):
        fn()
    e1.record()
    e1.synchronize()
    return e0.elapsed_time(e1) / iters


def test_reference_kernel_timings(ref, capsys):
    """Power-law 1e6 x 1e6 (Zipf 2.1 clipped to [1, 20000], seed 1), N = 64, FP32."""
    from segscan_gb300 import autotune
    A = synth.powerlaw(1_000_000, 1_000_000, 2.1, 1, 20000, seed=1)
    Ad = dev_csr(A)
    Bd = torch.from_numpy(synth.dense(A.ncol, N, seed=2)).cuda()
    C = torch.empty((A.nrow, N), device="cuda")
    nbytes = synth.spmm_bytes(A, N)
    rows = {}
    for strategy in ("ebpr", "rbpr", "ebsr", "rbsr"):
        def run_ref():
            if strategy != "rbsr":
                C.zero_()
            ref.launch(strategy, A.nrow, A.ncol, A.nnz, Ad.indptr, Ad.indices, Ad.values, Bd, C)
        k = api.default_knobs(strategy, N)
        n = api.spmm_workspace_size(Ad, N, strategy, k)
        ws = torch.empty(n + 256, dtype=torch.uint8, device="cuda") if n else None
        t_ref = _ms(run_ref, 5 if strategy in ("rbpr", "rbsr") else 10)
        t_ours = _ms(lambda: api.spmm(Ad, Bd, strategy, knobs=k, out=C, workspace=ws))
        rows[strategy] = {"reference_ms": t_ref, "ours_same_knobs_ms": t_ours, "speedup": t_ref / t_ours,
                          "reference_GB/s": nbytes / t_ref / 1e6, "ours_GB/s": nbytes / t_ours / 1e6}
    s, k = autotune.best(Ad, N, Bd)
    n = api.spmm_workspace_size(Ad, N, s, k)
    ws = torch.empty(n + 256, dtype=torch.uint8, device="cuda") if n else None
    t_best = _ms(lambda: api.spmm(Ad, Bd, s, knobs=k, out=C, workspace=ws))
    best_ref = min(r["reference_ms"] for r in rows.values())
    rows["ours_tuned"] = {"strategy": s, "knobs": k.as_dict(), "ms": t_best, "GB/s": nbytes / t_best / 1e6,
                          "speedup_vs_best_reference_kernel": best_ref / t_best}
    with capsys.disabled():
        print("\nreference_kernels_sm103a " + json.dumps(rows))
    assert all(r["reference_ms"] > 0 for k_, r in rows.items() if k_ != "ours_tuned")


# ---------------------------------------------------------------------------
# segment_coo: the reference's segment_coo_sr and segment_coo_sorted_sr
# ---------------------------------------------------------------------------
from ref_kernels import RefSegmentKernels  # noqa: E402

seg_available = pytest.mark.skipif(not RefSegmentKernels.available(),
                                   reason="reference segment kernels not built (needs the reference checkout)")


@pytest.fixture(scope="module")
def ref_seg(cuda):
    return RefSegmentKernels()


def padded_index(index: np.ndarray) -> torch.Tensor:
    """The index on the device with RefSegmentKernels.PAD copies of its last
    id after it, so the reference kernel's reads past nnz stay in bounds."""
    pad = np.full(RefSegmentKernels.PAD, index[-1], dtype=np.int32)
    return torch.from_numpy(np.concatenate([index, pad])).cuda()


@seg_available
@pytest.mark.parametrize("which", ["sr", "sorted"])
def test_reference_segment_kernels_match_ours(ref_seg, which):
    import oracle_lib
    csr = synth.powerlaw(30000, 30000, 2.1, 1, 3000, seed=24)
    index = csr.coo_rows()
    src = synth.dense(csr.nnz, 64, seed=25)
    srcd = torch.from_numpy(src).cuda()
    dst_ref = torch.zeros((csr.nrow, 64), device="cuda")
    ref_seg.launch(which, srcd, padded_index(index), csr.nnz, dst_ref)
    dst_ours = api.segment(srcd, torch.from_numpy(index).cuda(), csr.nrow, "sum")
    torch.cuda.synchronize()
    d64, dabs = oracle_lib.segment_coo_f64(src, index, csr.nrow, 0)
    check_close(dst_ref.cpu().numpy(), d64, dabs, 1e-5, None, f"reference segment_coo {which} vs FP64")
    check_close(dst_ours.cpu().numpy(), d64, dabs, 1e-5, None, "segscan_gb300 segment sum vs FP64")


@seg_available
def test_reference_segment_timings(ref_seg, capsys):
    """segment sum over the power-law matrix's first 4,000,000 nonzeros
    (segment_coo_sorted_sr's grid.y cannot hold the whole 4.63 M), N = 64,
    dst zeroing included for the reference's atomic kernels."""
    csr = synth.powerlaw(1_000_000, 1_000_000, 2.1, 1, 20000, seed=1)
    nnz = 4_000_000
    index = csr.coo_rows()[:nnz]
    dst_len = int(index[-1]) + 1
    srcd = torch.rand((nnz, 64), device="cuda")
    idx_pad = padded_index(index)
    idx = idx_pad[:nnz]
    dst = torch.empty((dst_len, 64), device="cuda")
    nbytes = synth.segment_bytes(nnz, 64, dst_len)
    rows = {}
    for which in ("sr", "sorted"):
        def run():
            dst.zero_()
            ref_seg.launch(which, srcd, idx_pad, nnz, dst)
        t = _ms(run)
        rows[f"reference_{which}"] = {"ms": t, "GB/s": nbytes / t / 1e6}
    ws_n = api.segment_workspace_size(nnz, 64, "sr")
    t_ours = _ms(lambda: api.segment(srcd, idx, dst_len, "sum", "sr", out=dst))
    best_ref = min(r["ms"] for r in rows.values())
    rows["ours_sr"] = {"ms": t_ours, "GB/s": nbytes / t_ours / 1e6, "speedup_vs_best_reference": best_ref / t_ours,
                       "workspace_bytes": ws_n}
    with capsys.disabled():
        print("\nreference_segment_kernels_sm103a " + json.dumps(rows))
    assert all(r["ms"] > 0 for r in rows.values())
