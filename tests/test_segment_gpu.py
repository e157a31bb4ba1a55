"""segment_coo parity (sum / max / mean, both strategy families) against the
reference's host loop (golden fixture) and the FP64 oracle."""
from pathlib import Path

import numpy as np
import pytest
import torch

import oracle_lib
from gpu_util import check_close, rounded
from segscan_gb300 import synth

pytestmark = pytest.mark.gpu
GOLD = Path(__file__).resolve().parent / "golden"
REDUCE = {"sum": 0, "max": 1, "mean": 2}


def seg(src, index, dst_len, reduce, strategy, **kw):
    from segscan_gb300 import api
    if "out" not in kw:  # NaN first: a row the kernel never stores shows up
        kw["out"] = torch.full((dst_len, src.shape[1]), float("nan"), device=src.device)
    out = api.segment(src, index, dst_len, reduce, strategy, **kw)
    torch.cuda.synchronize()
    return out.cpu().numpy()


def oracle(src, index, dst_len, reduce):
    return oracle_lib.segment_coo_f64(src, index, dst_len, REDUCE[reduce])


def check(got, ref, dabs, reduce, tol, what):
    if reduce == "max":
        assert np.array_equal(got.astype(np.float64), ref), what
    else:
        check_close(got, ref, dabs, tol, None, what)


@pytest.mark.parametrize("strategy", ["pr", "sr"])
def test_golden_sum(cuda, strategy):
    g = np.load(GOLD / "segment_edge_n5.npz")
    src = torch.from_numpy(g["src"]).cuda()
    idx = torch.from_numpy(g["index"]).cuda()
    got = seg(src, idx, int(g["dst_len"]), "sum", strategy)
    ref, dabs = oracle(g["src"], g["index"], int(g["dst_len"]), "sum")
    check_close(got, ref, dabs, 1e-5, 1e-5, "vs FP64")
    check_close(got, g["dst"].astype(np.float64), dabs, 2e-5, None, "vs reference loop")


@pytest.mark.parametrize("strategy", ["pr", "sr"])
@pytest.mark.parametrize("reduce", ["sum", "max", "mean"])
@pytest.mark.parametrize("N", [1, 5, 32, 64])
def test_reductions(cuda, strategy, reduce, N):
    csr = synth.powerlaw(30000, 10, 2.1, 1, 4000, seed=N)  # long segments cross many chunks
    index = csr.coo_rows()
    L = csr.nrow + 3
    src = synth.dense(csr.nnz, N, seed=N + 7)
    got = seg(torch.from_numpy(src).cuda(), torch.from_numpy(index).cuda(), L, reduce, strategy)
    ref, dabs = oracle(src, index, L, reduce)
    check(got, ref, dabs, reduce, 1e-5, f"{strategy} {reduce} N={N}")


@pytest.mark.parametrize("reduce", ["sum", "max", "mean"])
def test_sr_many_tiles_and_long_runs(cuda, reduce):
    """SR with 4-lane groups and 16-column tiles (4 tiles at N = 64) and
    32-element chunks: segments of up to 4000 elements span over a hundred
    chunks, so the walk's straddling-segment probes take many rounds and
    every column tile assembles its own part of each segment.  Two runs
    give the same bits whichever chunk finishes a segment last."""
    from segscan_gb300 import api
    csr = synth.powerlaw(20000, 10, 2.1, 1, 4000, seed=31)
    index = csr.coo_rows()
    src = synth.dense(csr.nnz, 64, seed=32)
    k = api.make_knobs("ebsr", 64, group_factor=2, coarsen_factor=4, thread_nz=8, block_denom=1)
    srcd, idxd = torch.from_numpy(src).cuda(), torch.from_numpy(index).cuda()
    got = seg(srcd, idxd, csr.nrow, reduce, "sr", knobs=k)
    again = seg(srcd, idxd, csr.nrow, reduce, "sr", knobs=k)
    ref, dabs = oracle(src, index, csr.nrow, reduce)
    check(got, ref, dabs, reduce, 1e-5, f"sr 4 tiles {reduce}")
    assert np.array_equal(got, again)


@pytest.mark.parametrize("strategy", ["pr", "sr"])
@pytest.mark.parametrize("reduce", ["sum", "max", "mean"])
def test_bf16_src(cuda, strategy, reduce):
    csr = synth.poisson(3000, 10, 12.0, seed=3)
    index = csr.coo_rows()
    src = synth.dense(csr.nnz, 32, seed=8)
    got = seg(torch.from_numpy(src).cuda().to(torch.bfloat16), torch.from_numpy(index).cuda(), 3000, reduce,
              strategy)
    ref, dabs = oracle(rounded(src, torch.bfloat16), index, 3000, reduce)
    check(got, ref, dabs, reduce, 1e-5, f"bf16 {strategy} {reduce}")


@pytest.mark.parametrize("strategy", ["pr", "sr"])
def test_empty_and_accumulate(cuda, strategy):
    from segscan_gb300 import api
    out = torch.full((7, 4), 5.0, device="cuda")
    api.segment(torch.zeros(0, 4, device="cuda"), torch.zeros(0, dtype=torch.int32, device="cuda"), 7,
                out=out, strategy=strategy)
    torch.cuda.synchronize()
    assert not out.any()
    index = np.array([0, 0, 3, 3, 3, 6], np.int32)
    src = synth.dense(6, 4, seed=1)
    out = torch.ones(7, 4, device="cuda")
    api.segment(torch.from_numpy(src).cuda(), torch.from_numpy(index).cuda(), 7, out=out, accumulate=True,
                strategy=strategy)
    ref, dabs = oracle(src, index, 7, "sum")
    check_close(out.cpu().numpy(), ref + 1.0, dabs + 1.0, 1e-6, None, "accumulate")


def test_reference_named_wrappers(cuda):
    from segscan_gb300 import api
    g = np.load(GOLD / "segment_edge_n5.npz")
    src = torch.from_numpy(g["src"]).cuda()
    idx = torch.from_numpy(g["index"]).cuda()
    nnz, N, L = src.shape[0], src.shape[1], int(g["dst_len"])
    ref, dabs = oracle(g["src"], g["index"], L, "sum")
    calls = [
        (api.segment_coo, dict(group_factor=5, thread_per_block=256, tile_factor=5, block_numer=1, block_denom=16)),
        (api.segment_coo_new, dict(group_factor=5, thread_per_block=256, tile_factor=5, blockDimY=2)),
        (api.segment_coo_sr, dict(group_factor=4, thread_per_block=256, CoarsenFactor=4, ThreadNz=1,
                                  block_numer=1, block_denom=16)),
        (api.segment_coo_noshmem_sr, dict(group_factor=4, thread_per_block=256, CoarsenFactor=4, ThreadNz=2,
                                          block_numer=1, block_denom=16)),
        (api.segment_coo_noshmem_lessatom_sr, dict(group_factor=4, thread_per_block=256, CoarsenFactor=4,
                                                   ThreadNz=1, block_numer=1, block_denom=16)),
        (api.segment_coo_sorted_sr, dict(CoarsenFactor=2, ThreadNz=4, DtileSize=8, DtileNum=2, BlockDimY=16)),
    ]
    for fn, kw in calls:
        dst = torch.zeros(L, N, device="cuda")
        fn(src, idx, nnz, N, dst, **kw)
        torch.cuda.synchronize()
        check_close(dst.cpu().numpy(), ref, dabs, 1e-5, 1e-5, fn.__name__)


def test_index_validate(cuda):
    from segscan_gb300 import api
    idx = torch.tensor([0, 1, 1, 4], dtype=torch.int32, device="cuda")
    assert api.validate_index(idx, 5) == 0
    assert api.validate_index(idx, 4) & 32
    assert api.validate_index(torch.tensor([2, 1], dtype=torch.int32, device="cuda"), 5) & 16


@pytest.mark.parametrize("strategy", ["sr", "pr"])
@pytest.mark.parametrize("reduce", ["sum", "mean"])
def test_segment_plan_and_graph_match(cuda, strategy, reduce):
    """SegmentPlan.run and its CUDA graph give the same bits as api.segment."""
    from segscan_gb300 import api
    csr = synth.powerlaw(8000, 10, 2.1, 1, 500, seed=41)
    index = torch.from_numpy(csr.coo_rows()).cuda()
    src = torch.from_numpy(synth.dense(csr.nnz, 32, seed=42)).cuda()
    ref = api.segment(src, index, csr.nrow, reduce, strategy)
    plan = api.SegmentPlan(index, csr.nrow, 32, reduce, strategy)
    out = torch.full_like(ref, float("nan"))
    plan.run(src, out)
    torch.cuda.synchronize()
    assert torch.equal(out, ref)
    g = plan.capture(src, out)
    out.fill_(float("nan"))
    g.replay()
    torch.cuda.synchronize()
    assert torch.equal(out, ref)
    with pytest.raises(ValueError):
        plan.run(src[:, :16].contiguous(), out)


@pytest.mark.parametrize("reduce", ["sum", "max", "mean"])
@pytest.mark.parametrize("knobs_kw,chunk", [(dict(group_factor=2, thread_nz=8), 32),
                                            (dict(group_factor=4, thread_nz=8), 128)])
def test_sr_segments_starting_on_chunk_boundaries(cuda, reduce, knobs_kw, chunk):
    """Every segment starts exactly at a chunk boundary and most span several
    chunks: the owner of such a segment is the chunk it starts in, not the
    one before.  dst starts as NaN, so a segment nobody stores shows up."""
    from segscan_gb300 import api
    rng = np.random.default_rng(91 + chunk)
    lengths = chunk * rng.integers(1, 41, size=300)
    index = np.repeat(np.arange(lengths.size, dtype=np.int32), lengths)
    dst_len = lengths.size + 2
    src = synth.dense(index.size, 64, seed=92)
    k = api.make_knobs("ebsr", 64, coarsen_factor=4, block_denom=1, **knobs_kw)
    out = torch.full((dst_len, 64), float("nan"), device="cuda")
    api.segment(torch.from_numpy(src).cuda(), torch.from_numpy(index).cuda(), dst_len, reduce, "sr", knobs=k,
                out=out)
    torch.cuda.synchronize()
    ref, dabs = oracle(src, index, dst_len, reduce)
    check(out.cpu().numpy(), ref, dabs, reduce, 1e-5, f"segments on {chunk}-element boundaries, {reduce}")
