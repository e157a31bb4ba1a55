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
import os

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
@pytest.mark.parametrize("which", ["sr", "sorted", "pr", "new", "noshmem", "lessatom"])
def test_reference_segment_kernels_match_ours(ref_seg, which):
    import oracle_lib
    csr = synth.powerlaw(30000, 30000, 2.1, 1, 3000, seed=24)
    index = csr.coo_rows()
    src = synth.dense(csr.nnz, 64, seed=25)
    srcd = torch.from_numpy(src).cuda()
    dst_ref = torch.zeros((csr.nrow, 64), device="cuda")
    ref_seg.launch(which, srcd, padded_index(index), csr.nnz, dst_ref)
    dst_ours = api.segment(srcd, torch.from_numpy(index).cuda(), csr.nrow, "sum",
                           "pr" if which in ("pr", "new") else "sr")
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
    for which in ("sr", "sorted", "pr", "new", "noshmem", "lessatom"):
        def run():
            dst.zero_()
            ref_seg.launch(which, srcd, idx_pad, nnz, dst)
        t = _ms(run)
        rows[f"reference_{which}"] = {"ms": t, "GB/s": nbytes / t / 1e6}
    ws_n = api.segment_workspace_size(nnz, 64, "sr")
    t_ours = _ms(lambda: api.segment(srcd, idx, dst_len, "sum", "sr", out=dst))
    t_pr = _ms(lambda: api.segment(srcd, idx, dst_len, "sum", "pr", out=dst))
    best_ref = min(r["ms"] for r in rows.values())
    rows["ours_sr"] = {"ms": t_ours, "GB/s": nbytes / t_ours / 1e6, "speedup_vs_best_reference": best_ref / t_ours,
                       "workspace_bytes": ws_n}
    # this library's PR family at the reference's segment_coo tuple (5,256,5,1,16)
    rows["ours_pr"] = {"ms": t_pr, "GB/s": nbytes / t_pr / 1e6,
                       "speedup_vs_reference_pr": rows["reference_pr"]["ms"] / t_pr}
    with capsys.disabled():
        print("\nreference_segment_kernels_sm103a " + json.dumps(rows))
    assert all(r["ms"] > 0 for r in rows.values())


# ---------------------------------------------------------------------------
# dgSPARSE baseline kernels (spmm.cuh) and the README's "static vs dgSPARSE"
# ---------------------------------------------------------------------------
from ref_kernels import DgKernels  # noqa: E402


@pytest.fixture(scope="module")
def dg(ref):
    return DgKernels(ref)


@pytest.mark.parametrize("strategy,N", [("ebpr", 64), ("rbpr", 64), ("ebsr", 64), ("rbsr", 64), ("ebsr", 128),
                                        ("ebpr", 128), ("rbpr", 20)])
def test_dgsparse_kernels_match_fp64(dg, strategy, N):
    A = integer_valued(synth.powerlaw(30000, 30000, 2.1, 1, 3000, seed=26), 27)
    B = synth.dense(A.ncol, N, seed=28)
    Ad = dev_csr(A)
    Bd = torch.from_numpy(B).cuda()
    C = torch.zeros((A.nrow, N), device="cuda")
    dg.launch(strategy, A.nrow, A.ncol, A.nnz, Ad.indptr, Ad.indices, Ad.values, Bd, C)
    torch.cuda.synchronize()
    C64, absC = oracle64(A, B)
    check_close(C.cpu().numpy(), C64, absC, 1e-5, None, f"dgSPARSE {strategy} N={N} vs FP64")


# README.md:212-260 quotes, per strategy, dgSPARSE time / best static tuple
# time (geomean over SuiteSparse).  Seeded synthetic matrices of the
# configurations' shapes and a few more row-length distributions stand in for
# the SuiteSparse set, which is not available.
SWEEP_DATASETS = ["poisson:4096:16:0", "poisson:200000:16:0", "banded:120000:20:500:1", "banded:400000:48:2000:1",
                  "powerlaw:1000000:2.1:20000:1", "powerlaw:300000:1.8:50000:5", "powerlaw:600000:2.6:2000:6"]
REF_TUPLES = {"ebpr": dict(group_factor=5, thread_per_block=256, tile_factor=5, block_numer=1, block_denom=16),
              "rbpr": dict(group_factor=3, thread_per_block=256, tile_factor=3, block_numer=1, block_denom=2),
              "ebsr": dict(group_factor=4, thread_per_block=256, coarsen_factor=4, thread_nz=1, block_numer=1,
                           block_denom=16),
              "rbsr": dict(coarsen_factor=4, thread_per_block=256, tile_factor=5, block_numer=1, block_denom=1)}


def test_static_vs_dgsparse_sweep(ref, dg, capsys, tmp_path):
    from segscan_gb300 import ratios, sweep
    from segscan_gb300.ratios import Row

    same = {s: sweep.label(s, api.make_knobs(s, N, **kw)) for s, kw in REF_TUPLES.items()}
    swept = {sweep.label(s, k) for s, k in sweep.library_actions(N)}

    def extra(spec, Ah, A, B, timer):
        C = torch.empty((Ah.nrow, N), device="cuda")
        rows = []
        for s, kw in REF_TUPLES.items():  # this library at the reference's tuples, where the sweep lacks them
            if same[s] not in swept:
                k = api.make_knobs(s, N, **kw)
                n = api.spmm_workspace_size(A, N, s, k)
                ws = torch.empty(n + 256, dtype=torch.uint8, device="cuda") if n else None
                rows.append(Row(spec, N, same[s], "library",
                                timer(lambda: api.spmm(A, B, s, knobs=k, out=C, workspace=ws))))
        for s in ("ebpr", "rbpr", "ebsr", "rbsr"):
            zero = s != "rbsr"

            def run_ref():
                if zero:
                    C.zero_()
                ref.launch(s, Ah.nrow, Ah.ncol, Ah.nnz, A.indptr, A.indices, A.values, B, C)

            def run_dg():
                if zero:
                    C.zero_()
                dg.launch(s, Ah.nrow, Ah.ncol, Ah.nnz, A.indptr, A.indices, A.values, B, C)
            rows.append(Row(spec, N, f"reference_{s}", "external", timer(run_ref)))
            rows.append(Row(spec, N, f"dgsparse_{s}", "external", timer(run_dg)))
        return rows

    rows = sweep.run(SWEEP_DATASETS, N, iters=11, extra=extra)
    ratios.write_csv(os.environ.get("SEGSCAN_SWEEP_CSV") or tmp_path / "sweep.csv", rows)
    out = {"datasets": SWEEP_DATASETS, "N": N, "timing": "median of 11 CUDA-event launches, L2 flushed before each"}
    for s in ("ebpr", "rbpr", "ebsr", "rbsr"):
        out[s] = {"reference_static_vs_dgsparse": ratios.compare(rows, f"dgsparse_{s}", f"reference_{s}"),
                  "ours_same_tuple_vs_dgsparse": ratios.compare(rows, f"dgsparse_{s}", same[s]),
                  "ours_same_tuple_vs_reference": ratios.compare(rows, f"reference_{s}", same[s]),
                  "same_tuple": same[s]}
    lib_actions = [r.action for r in rows if r.kind == "library" and r.dataset == SWEEP_DATASETS[0]]
    out["tuning"] = ratios.tuning(rows, sweep.label("ebsr", api.default_knobs("ebsr", N)), lib_actions)
    st = ratios.static_ranking(rows, lib_actions)
    out["best_static"] = st["best_static"]
    best_lib, best_ref, best_act = {}, {}, {}
    table = ratios.pivot(rows)
    for key, t in table.items():
        best_act[key] = min((a for a in lib_actions if a in t), key=lambda a: t[a])
        best_lib[key] = t[best_act[key]]
        best_ref[key] = min(t[f"reference_{s}"] for s in ("ebpr", "rbpr", "ebsr", "rbsr"))
    r = [best_ref[k] / best_lib[k] for k in table]
    out["best_ours_vs_best_reference_kernel"] = ratios.stats(r)
    out["per_dataset_us"] = {k[0]: {"best_ours": best_lib[k], "best_ours_action": best_act[k],
                                    "best_reference": best_ref[k],
                                    "cusparse": table[k].get("cusparse"),
                                    **{f"dgsparse_{s}": table[k][f"dgsparse_{s}"] for s in REF_TUPLES}}
                             for k in table}
    with capsys.disabled():
        print("\nstatic_vs_dgsparse_sm103a " + json.dumps(out))
    assert len(table) == len(SWEEP_DATASETS)
