"""SpMM parity: every strategy against the reference's check path (golden
fixtures) and the FP64 oracle.  FP32 tolerance: |C - C64| <= 1e-5 * (|A||B|)
per element and 1e-5 normwise; BF16/FP16 storage: 2e-2 normwise against FP64
on the FP32 inputs."""
from pathlib import Path

import numpy as np
import pytest
import torch

import oracle_lib
from gpu_util import check_close, dev_csr, oracle64, powerlaw_medium, rounded
from segscan_gb300 import synth

pytestmark = pytest.mark.gpu
GOLD = Path(__file__).resolve().parent / "golden"
STRATS = ["ebpr", "rbpr", "ebsr", "rbsr"]


def spmm(A, B, strategy, **kw):
    from segscan_gb300 import api
    out = api.spmm(A, B, strategy, **kw)
    torch.cuda.synchronize()
    return out


@pytest.mark.parametrize("strategy", STRATS)
@pytest.mark.parametrize("name", ["spmm_poisson512_n4.npz", "spmm_poisson512_n16.npz", "spmm_edge_n3.npz"])
def test_golden(cuda, strategy, name):
    g = np.load(GOLD / name)
    csr = synth.Csr(g["indptr"].size - 1, int(g["ncol"]), g["indptr"], g["indices"], g["values"])
    A = dev_csr(csr)
    C = spmm(A, torch.from_numpy(g["B"]).cuda(), strategy).cpu().numpy()
    C64, absC = oracle64(csr, g["B"])
    check_close(C, C64, absC, 1e-5, 1e-5, f"{strategy} vs FP64")
    check_close(C, g["C"].astype(np.float64), absC, 2e-5, None, f"{strategy} vs reference check path")


@pytest.mark.parametrize("strategy", STRATS)
def test_ones_known_answer_exact(cuda, strategy):
    g = np.load(GOLD / "spmm_ones_kat_n8.npz")
    csr = synth.Csr(g["indptr"].size - 1, int(g["ncol"]), g["indptr"], g["indices"], g["values"])
    for values in (True, False):  # values=None is the reference's all-ones default
        A = dev_csr(csr, values=values)
        C = spmm(A, torch.from_numpy(g["B"]).cuda(), strategy).cpu().numpy()
        assert np.array_equal(C, g["C"]), strategy


@pytest.mark.parametrize("strategy", STRATS)
@pytest.mark.parametrize("N", [1, 2, 3, 4, 16, 33, 64, 128])
def test_widths(cuda, strategy, N):
    csr = synth.poisson(700, 900, 9.0, seed=N)
    B = synth.dense(900, N, seed=N + 1)
    C = spmm(dev_csr(csr), torch.from_numpy(B).cuda(), strategy).cpu().numpy()
    C64, absC = oracle64(csr, B)
    check_close(C, C64, absC, 1e-5, 1e-5, f"{strategy} N={N}")


@pytest.mark.parametrize("strategy", STRATS)
@pytest.mark.parametrize("N", [3, 64])
def test_powerlaw_long_rows(cuda, strategy, N):
    csr = powerlaw_medium()
    B = synth.dense(csr.ncol, N, seed=5)
    C = spmm(dev_csr(csr), torch.from_numpy(B).cuda(), strategy).cpu().numpy()
    C64, absC = oracle64(csr, B)
    check_close(C, C64, absC, 1e-5, 1e-5, f"{strategy} powerlaw N={N}")


KNOB_SWEEP = {
    # README.md:168-210 best static tuples and test-cg/src/params.md grids
    "ebpr": [dict(group_factor=5, tile_factor=5, block_denom=8), dict(group_factor=4, tile_factor=5, block_denom=4),
             dict(group_factor=2, tile_factor=2, block_numer=2), dict(group_factor=0, tile_factor=0, block_denom=32)],
    "rbpr": [dict(group_factor=3, tile_factor=3, block_denom=2), dict(group_factor=2, tile_factor=2, block_denom=1),
             dict(group_factor=5, tile_factor=5, block_denom=16), dict(group_factor=0, tile_factor=4)],
    "ebsr": [dict(group_factor=4, coarsen_factor=4, thread_nz=2, block_denom=16),
             dict(group_factor=3, coarsen_factor=2, thread_nz=1, block_denom=8),
             dict(group_factor=5, coarsen_factor=1, thread_nz=32, thread_per_block=128),
             dict(group_factor=0, coarsen_factor=8, thread_nz=64, thread_per_block=64),
             dict(group_factor=2, coarsen_factor=3, thread_nz=300, thread_per_block=512)],
    "rbsr": [dict(coarsen_factor=4, tile_factor=5), dict(coarsen_factor=2, tile_factor=1, block_denom=4),
             dict(coarsen_factor=1, tile_factor=0), dict(coarsen_factor=8, tile_factor=7, thread_per_block=1024)],
}


@pytest.mark.parametrize("strategy", STRATS)
@pytest.mark.parametrize("N", [5, 48])
def test_knob_sweep(cuda, strategy, N):
    from segscan_gb300 import api
    g = np.load(GOLD / "spmm_edge_n3.npz")
    csr = synth.Csr(g["indptr"].size - 1, int(g["ncol"]), g["indptr"], g["indices"], g["values"])
    B = synth.dense(csr.ncol, N, seed=9)
    C64, absC = oracle64(csr, B)
    A = dev_csr(csr)
    for kw in KNOB_SWEEP[strategy]:
        k = api.make_knobs(strategy, N, **kw)
        C = spmm(A, torch.from_numpy(B).cuda(), strategy, knobs=k).cpu().numpy()
        check_close(C, C64, absC, 1e-5, 1e-5, f"{strategy} {kw}")


# FP16 has subnormals below 2**-14: a 16-bit input or output there carries an
# absolute error up to 2**-25, so FP16 bounds add that absolute term.
F16_ATOL = 2.0 ** -24


@pytest.mark.parametrize("strategy", STRATS)
@pytest.mark.parametrize("dtype", [torch.bfloat16, torch.float16])
@pytest.mark.parametrize("out_f32", [True, False])
def test_half_storage(cuda, strategy, dtype, out_f32):
    csr = powerlaw_medium(M=20000, lmax=3000)
    N = 64
    B = synth.dense(csr.ncol, N, seed=2)
    A = dev_csr(csr, dtype)
    Bd = torch.from_numpy(B).cuda().to(dtype)
    C = spmm(A, Bd, strategy, out_dtype=torch.float32 if out_f32 else dtype).float().cpu().numpy()
    atol = F16_ATOL if dtype == torch.float16 else 1e-30
    C64, absC = oracle64(csr, B)
    # inputs rounded to 16 bits (u = 2**-8 bf16, 2**-11 fp16), FP32 sums, one output rounding
    check_close(C, C64, absC, 2e-2 if dtype == torch.bfloat16 else 5e-3, 2e-2,
                f"{strategy} {dtype} vs FP64(fp32 in)", atol=atol)
    # against FP64 on the stored (rounded) inputs only accumulation and the
    # single output rounding remain
    Cr64, absCr = oracle64(csr, rounded(B, dtype), rounded(csr.values, dtype))
    out_tol = 1e-5 if out_f32 else (2.0 ** -8 if dtype == torch.bfloat16 else 2.0 ** -11)
    bound = np.abs(Cr64) * out_tol + 1e-5 * absCr + atol
    err = np.abs(C - Cr64)
    assert np.all(err <= bound), f"{strategy} {dtype}: worst {np.max(err - bound):.3e} over the bound"


@pytest.mark.parametrize("out_dtype", [torch.bfloat16, torch.float16])
@pytest.mark.parametrize("accumulate", [False, True])
def test_f32_inputs_16bit_output(cuda, out_dtype, accumulate):
    """ebsr with FP32 values and B writes a BF16/FP16 C directly: FP32 sums
    (and, accumulating, the old C added in FP32), rounded once to the output
    type; other strategies refuse the combination."""
    from segscan_gb300 import api
    csr = powerlaw_medium(M=20000, lmax=3000)
    B = synth.dense(csr.ncol, 64, seed=12)
    A = dev_csr(csr)
    Bd = torch.from_numpy(B).cuda()
    old = torch.from_numpy(synth.dense(csr.nrow, 64, seed=13)).cuda().to(out_dtype)
    C = old.clone()
    api.spmm(A, Bd, "ebsr", out=C, accumulate=accumulate)
    torch.cuda.synchronize()
    C64, absC = oracle64(csr, B)
    if accumulate:
        prev = old.double().cpu().numpy()
        C64, absC = C64 + prev, absC + np.abs(prev)
    u = 2.0 ** -8 if out_dtype == torch.bfloat16 else 2.0 ** -11
    atol = F16_ATOL if out_dtype == torch.float16 else 1e-30
    err = np.abs(C.double().cpu().numpy() - C64)
    bound = np.abs(C64) * u + 1e-5 * absC + atol
    assert np.all(err <= bound), f"{out_dtype}: worst {np.max(err - bound):.3e} over the bound"
    for strategy in ("ebpr", "rbpr", "rbsr"):
        with pytest.raises(Exception):
            api.spmm(A, Bd, strategy, out_dtype=out_dtype)


@pytest.mark.parametrize("strategy", STRATS)
def test_accumulate(cuda, strategy):
    csr = synth.poisson(300, 300, 5.0, seed=4)
    B = synth.dense(300, 16, seed=4)
    C0 = synth.dense(300, 16, seed=44)
    out = torch.from_numpy(C0.copy()).cuda()
    spmm(dev_csr(csr), torch.from_numpy(B).cuda(), strategy, out=out, accumulate=True)
    C64, absC = oracle64(csr, B)
    check_close(out.cpu().numpy(), C64 + C0, absC + np.abs(C0), 1e-5, None, strategy)


@pytest.mark.parametrize("strategy", STRATS)
def test_degenerate_shapes(cuda, strategy):
    from segscan_gb300 import api
    # nnz = 0: overwrite mode writes zeros
    empty = synth.Csr(50, 40, np.zeros(51, np.int32), np.zeros(0, np.int32), np.zeros(0, np.float32))
    out = torch.full((50, 8), 7.0, device="cuda")
    spmm(dev_csr(empty), torch.ones(40, 8, device="cuda"), strategy, out=out)
    assert not out.any()
    # one row
    one = synth.poisson(1, 5000, 3000.0, seed=1)
    B = synth.dense(5000, 4, seed=1)
    C = spmm(dev_csr(one), torch.from_numpy(B).cuda(), strategy).cpu().numpy()
    C64, absC = oracle64(one, B)
    check_close(C, C64, absC, 1e-5, None, "M=1")
    # all rows empty but the last
    lengths = np.zeros(64, np.int64)
    lengths[-1] = 10
    last = synth.csr_from_lengths(64, 64, lengths, np.random.default_rng(0))
    B = synth.dense(64, 8, seed=2)
    out = torch.full((64, 8), 3.0, device="cuda")
    spmm(dev_csr(last), torch.from_numpy(B).cuda(), strategy, out=out)
    C64, absC = oracle64(last, B)
    check_close(out.cpu().numpy(), C64, absC, 1e-5, None, "trailing row")


def test_reference_named_wrappers(cuda):
    from segscan_gb300 import api
    g = np.load(GOLD / "spmm_poisson512_n16.npz")
    csr = synth.Csr(g["indptr"].size - 1, int(g["ncol"]), g["indptr"], g["indices"], g["values"])
    A = dev_csr(csr)
    B = torch.from_numpy(g["B"]).cuda()
    C64, absC = oracle64(csr, g["B"])
    calls = [
        (api.csrspmm_parreduce_nnzbalance_cg, dict(group_factor=5, thread_per_block=256, tile_factor=5,
                                                    block_numer=1, block_denom=8)),
        (api.csrspmm_parreduce_rowbalance_cg, dict(group_factor=3, thread_per_block=256, tile_factor=3,
                                                    block_numer=1, block_denom=2)),
        (api.csrspmm_rowcaching_nnzbalance_cg, dict(group_factor=4, thread_per_block=256, CoarsenFactor=4,
                                                     ThreadNz=1, block_numer=1, block_denom=16)),
        (api.csrspmm_seqreduce_rowbalance_cg, dict(coarsen_factor=4, thread_per_block=256, tile_factor=5,
                                                    block_numer=1, block_denom=1)),
    ]
    for fn, kw in calls:
        C = torch.zeros(A.nrow, 16, device="cuda")  # the reference's out_feature.reset()
        fn(A, 16, B, C, **kw)
        torch.cuda.synchronize()
        check_close(C.cpu().numpy(), C64, absC, 1e-5, 1e-5, fn.__name__)


def test_deterministic(cuda):
    csr = powerlaw_medium()
    B = torch.from_numpy(synth.dense(csr.ncol, 32, seed=3)).cuda()
    A = dev_csr(csr)
    for strategy in STRATS:
        c1 = spmm(A, B, strategy)
        c2 = spmm(A, B, strategy)
        assert torch.equal(c1, c2), strategy


def test_small_chunks_merge_to_the_wave_share(cuda):
    """Element-balanced chunks below the one-wave share are merged up to it:
    a tiny thread_nz and a thread_nz of exactly that share give the same
    chunking, hence the same bits; a larger thread_nz is kept (different
    chunking, same result within the FP32 tolerance)."""
    from segscan_gb300 import api
    csr = synth.powerlaw(200_000, 200_000, 2.1, 1, 20000, seed=31)
    B = torch.from_numpy(synth.dense(csr.ncol, 64, seed=32)).cuda()
    A = dev_csr(csr)
    G = 16
    sms = torch.cuda.get_device_properties(0).multi_processor_count  # the device's wave, as the library reads it
    share = -(-csr.nnz // (sms * 1024 // G))
    share = -(-share // 32) * 32
    assert share % G == 0
    tiny = spmm(A, B, "ebsr", knobs=api.make_knobs("ebsr", 64, group_factor=4, thread_nz=1, block_denom=1))
    exact = spmm(A, B, "ebsr", knobs=api.make_knobs("ebsr", 64, group_factor=4, thread_nz=share // G, block_denom=1))
    assert torch.equal(tiny, exact)
    big = spmm(A, B, "ebsr", knobs=api.make_knobs("ebsr", 64, group_factor=4, thread_nz=4 * share // G,
                                                     block_denom=1))
    C64, absC = oracle64(csr, B.cpu().numpy())
    for C in (tiny, big):
        check_close(C.cpu().numpy(), C64, absC, 1e-5, 1e-5, "merged chunks")
    n_tiny = api.spmm_workspace_size(A, 64, "ebsr", api.make_knobs("ebsr", 64, group_factor=4, thread_nz=1))
    n_exact = api.spmm_workspace_size(A, 64, "ebsr", api.make_knobs("ebsr", 64, group_factor=4,
                                                                     thread_nz=share // G))
    assert n_tiny == n_exact


def test_row_ids_bit_exact(cuda):
    from segscan_gb300 import api
    g = np.load(GOLD / "row_ids_edge.npz")
    ip = torch.from_numpy(g["indptr"]).cuda()
    rows = api.row_ids(ip, int(g["nnz"]), torch.from_numpy(g["elems"]).cuda()).cpu().numpy()
    assert np.array_equal(rows, g["rows"])
    big = powerlaw_medium()
    rows = api.row_ids(torch.from_numpy(big.indptr).cuda(), big.nnz).cpu().numpy()
    assert np.array_equal(rows, big.coo_rows())


def test_validate(cuda):
    from segscan_gb300 import api
    csr = synth.poisson(100, 100, 4.0, seed=1)
    A = dev_csr(csr)
    assert api.validate(A) == 0
    bad = A.indices.clone()
    bad[3] = 1000
    assert api.validate(api.CsrMatrix(A.nrow, A.ncol, A.indptr, bad, A.values)) & 8


def empty_runs_matrix(seed=5, M=20000, K=3000):
    """Short rows separated by runs of up to 400 empty rows (longer than any
    shared-memory row window), plus long rows, so chunk and tile boundaries
    land inside, before and after empty runs."""
    rng = np.random.default_rng(seed)
    lengths = np.zeros(M, np.int64)
    r = 0
    while r < M:
        run = int(rng.integers(0, 400)) if rng.random() < 0.08 else 0
        r += run
        if r >= M:
            break
        lengths[r] = int(rng.integers(1, 9)) if rng.random() < 0.95 else int(rng.integers(200, 1500))
        r += 1
    return synth.csr_from_lengths(M, K, lengths, rng)


@pytest.mark.parametrize("strategy", STRATS)
@pytest.mark.parametrize("accumulate", [False, True])
def test_empty_row_runs(cuda, strategy, accumulate):
    from segscan_gb300 import api
    csr = empty_runs_matrix()
    N = 16
    B = synth.dense(csr.ncol, N, seed=6)
    C0 = synth.dense(csr.nrow, N, seed=7)
    C64, absC = oracle64(csr, B)
    A = dev_csr(csr)
    sweeps = {"ebsr": [dict(group_factor=2, thread_nz=t) for t in (1, 2, 8, 16, 32, 64)],
              "ebpr": [dict(group_factor=5, tile_factor=5, block_denom=d) for d in (1, 16, 256)],
              "rbpr": [dict(group_factor=3, tile_factor=3)], "rbsr": [dict(coarsen_factor=4, tile_factor=4)]}
    for kw in sweeps[strategy]:
        out = torch.from_numpy(C0.copy()).cuda() if accumulate else torch.full((csr.nrow, N), 9.0, device="cuda")
        spmm(A, torch.from_numpy(B).cuda(), strategy, knobs=api.make_knobs(strategy, N, **kw), out=out,
             accumulate=accumulate)
        ref = C64 + C0 if accumulate else C64
        check_close(out.cpu().numpy(), ref, absC + (np.abs(C0) if accumulate else 0), 1e-5, None,
                    f"{strategy} {kw} acc={accumulate}")


@pytest.mark.parametrize("strategy", ["ebsr", "ebpr", "rbsr", "rbpr"])
def test_plan_run_and_graph_match_spmm(cuda, strategy):
    """SpmmPlan.run and its captured CUDA graph give the same bits as
    api.spmm; a wrong shape or dtype is refused."""
    from segscan_gb300 import api
    A = synth.poisson(4096, 4096, 16.0, seed=5)
    Ad = api.CsrMatrix.from_host(A, "cuda")
    B = torch.from_numpy(synth.dense(A.ncol, 16, seed=6)).cuda()
    ref = api.spmm(Ad, B, strategy)
    plan = api.SpmmPlan(Ad, 16, strategy)
    out = torch.full_like(ref, float("nan"))
    plan.run(B, out)
    torch.cuda.synchronize()
    assert torch.equal(out, ref)
    out2 = torch.full_like(ref, float("nan"))
    g = plan.capture(B, out2)
    out2.fill_(float("nan"))
    g.replay()
    torch.cuda.synchronize()
    assert torch.equal(out2, ref)
    with pytest.raises(ValueError):
        plan.run(B[:, :8].contiguous(), out)
    with pytest.raises(ValueError):
        plan.run(B.to(torch.bfloat16), out)


def test_plan_auto_strategy(cuda):
    """SpmmPlan(strategy="auto") runs the autotuner's pick, within 1e-5 of FP64."""
    from segscan_gb300 import api
    A = synth.powerlaw(20000, 20000, 2.1, 1, 2000, seed=7)
    Ad = api.CsrMatrix.from_host(A, "cuda")
    B = synth.dense(A.ncol, 16, seed=8)
    plan = api.SpmmPlan(Ad, 16, "auto")
    assert plan.strategy in ("ebpr", "rbpr", "ebsr", "rbsr")
    out = torch.full((A.nrow, 16), float("nan"), device="cuda")
    plan.run(torch.from_numpy(B).cuda(), out)
    torch.cuda.synchronize()
    C64, absC = oracle64(A, B)
    check_close(out.cpu().numpy(), C64, absC, 1e-5, None, f"auto plan ({plan.strategy})")


def test_concurrent_streams_and_threads(cuda):
    """The C ABI is stream-ordered and reentrant: four host threads, each
    with its own stream, matrix and workspace, call SpMM and segment_coo
    concurrently (ctypes releases the GIL during the calls); every result
    matches FP64, and the per-thread last-error message stays per thread."""
    import threading
    from segscan_gb300 import api
    jobs = []
    for t in range(4):
        A = synth.powerlaw(20000 + 1000 * t, 20000, 2.1, 1, 2000, seed=60 + t)
        B = synth.dense(A.ncol, 32, seed=70 + t)
        jobs.append((A, B, ["ebsr", "ebpr", "rbsr", "rbpr"][t]))
    results, errors = [None] * 4, []

    def work(t):
        try:
            A, B, strategy = jobs[t]
            s = torch.cuda.Stream()
            with torch.cuda.stream(s):
                Ad = api.CsrMatrix.from_host(A, "cuda")
                Bd = torch.from_numpy(B).cuda()
                idx = torch.from_numpy(A.coo_rows()).cuda()
                src = torch.from_numpy(synth.dense(A.nnz, 8, seed=80 + t)).cuda()
                for _ in range(20):
                    C = api.spmm(Ad, Bd, strategy, stream=s)
                    seg = api.segment(src, idx, A.nrow, "sum", stream=s)
                try:  # an invalid call on this thread: its message is this thread's
                    api.spmm(Ad, Bd[:, :7].contiguous(), strategy, knobs=api.make_knobs(strategy, 7, thread_per_block=4096))
                except api._lib.SegscanError as exc:
                    msg = str(exc)
                s.synchronize()
                results[t] = (C.cpu().numpy(), seg.cpu().numpy(), src.cpu().numpy(), msg)
        except Exception as exc:  # surfaced in the main thread
            errors.append(exc)

    # two more threads at the same time: the narrow walk at N = 4 and the
    # device transpose, each on its own stream
    extra = {}

    def narrow():
        try:
            A = synth.powerlaw(30000, 30000, 2.1, 1, 3000, seed=64)
            s = torch.cuda.Stream()
            with torch.cuda.stream(s):
                Ad = api.CsrMatrix.from_host(A, "cuda")
                B = torch.from_numpy(synth.dense(A.ncol, 4, seed=65)).cuda()
                k = api.make_knobs("ebsr", 4, group_factor=0, coarsen_factor=4, thread_nz=64, block_denom=1)
                for _ in range(20):
                    C = api.spmm(Ad, B, "ebsr", knobs=k, stream=s)
                s.synchronize()
                extra["narrow"] = (A, B.cpu().numpy(), C.cpu().numpy())
        except Exception as exc:
            errors.append(exc)

    def transpose():
        try:
            A = synth.powerlaw(25000, 18000, 2.1, 1, 3000, seed=66)
            s = torch.cuda.Stream()
            with torch.cuda.stream(s):
                Ad = api.CsrMatrix.from_host(A, "cuda")
                for _ in range(10):
                    AT, perm = api.transpose(Ad, stream=s)
                s.synchronize()
                extra["transpose"] = (A, AT.indptr.cpu().numpy(), AT.indices.cpu().numpy(), perm.cpu().numpy())
        except Exception as exc:
            errors.append(exc)

    threads = [threading.Thread(target=work, args=(t,)) for t in range(4)]
    threads += [threading.Thread(target=narrow), threading.Thread(target=transpose)]
    for th in threads:
        th.start()
    for th in threads:
        th.join()
    assert not errors, errors
    A, B, C = extra["narrow"]
    C64, absC = oracle64(A, B)
    check_close(C, C64, absC, 1e-5, None, "narrow walk thread")
    A, t_indptr, t_indices, perm = extra["transpose"]
    order = np.argsort(A.indices, kind="stable")
    assert np.array_equal(perm, order.astype(np.int32))
    assert np.array_equal(t_indices, np.repeat(np.arange(A.nrow, dtype=np.int32), np.diff(A.indptr))[order])
    assert np.array_equal(t_indptr, np.concatenate([[0], np.cumsum(np.bincount(A.indices, minlength=A.ncol))]))
    for t, (A, B, strategy) in enumerate(jobs):
        C, seg, src, msg = results[t]
        C64, absC = oracle64(A, B)
        check_close(C, C64, absC, 1e-5, None, f"thread {t} {strategy}")
        d64, dabs = oracle_lib.segment_coo_f64(src, A.coo_rows(), A.nrow, 0)
        check_close(seg, d64, dabs, 1e-5, None, f"thread {t} segment")
        assert "thread_per_block" in msg, msg


def test_one_workspace_reused_across_matrices_and_calls(cuda):
    """One caller-owned workspace, sized for the largest need, serves ebsr,
    ebpr and segment_coo calls on different matrices back to back: the
    arrival counts and slots are reset by each call, so nothing carries
    over from the call before."""
    from segscan_gb300 import api
    mats = [synth.powerlaw(9000 + 700 * i, 8000, 2.1, 1, 1500, seed=100 + i) for i in range(3)]
    N = 48
    devs = [api.CsrMatrix.from_host(A, "cuda") for A in mats]
    Bs = [torch.from_numpy(synth.dense(A.ncol, N, seed=110 + i)).cuda() for i, A in enumerate(mats)]
    need = max(api.spmm_workspace_size(Ad, N, s) for Ad in devs for s in ("ebsr", "ebpr"))
    need = max(need, max(api.segment_workspace_size(A.nnz, N, "sr") for A in mats))
    ws = torch.empty(need + 256, dtype=torch.uint8, device="cuda")
    for rep in range(2):
        for i, (A, Ad, B) in enumerate(zip(mats, devs, Bs)):
            C64, absC = oracle64(A, B.cpu().numpy())
            for s in ("ebsr", "ebpr"):
                C = torch.full((A.nrow, N), float("nan"), device="cuda")
                api.spmm(Ad, B, s, out=C, workspace=ws)
                torch.cuda.synchronize()
                check_close(C.cpu().numpy(), C64, absC, 1e-5, None, f"rep {rep} matrix {i} {s}")
            idx = torch.from_numpy(A.coo_rows()).cuda()
            src = torch.from_numpy(synth.dense(A.nnz, N, seed=120 + i)).cuda()
            out = torch.full((A.nrow, N), float("nan"), device="cuda")
            api.segment(src, idx, A.nrow, "sum", "sr", out=out, workspace=ws)
            torch.cuda.synchronize()
            d64, dabs = oracle_lib.segment_coo_f64(src.cpu().numpy(), A.coo_rows(), A.nrow, 0)
            check_close(out.cpu().numpy(), d64, dabs, 1e-5, None, f"rep {rep} matrix {i} segment")


def test_stream_argument_without_entering_the_stream(cuda):
    """spmm and segment given stream=s while another stream is current
    allocate their workspace and outputs on s.  Memory allocated and
    overwritten on the current stream right after each call therefore never
    lands on a block the launch on s still uses; every result matches
    FP64."""
    from segscan_gb300 import api
    A = synth.powerlaw(60000, 60000, 2.1, 1, 6000, seed=130)
    N = 64
    B = synth.dense(A.ncol, N, seed=131)
    Ad = api.CsrMatrix.from_host(A, "cuda")
    Bd = torch.from_numpy(B).cuda()
    idx = torch.from_numpy(A.coo_rows()).cuda()
    src_h = synth.dense(A.nnz, 16, seed=132)
    src = torch.from_numpy(src_h).cuda()
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    outs = []
    for strategy in ("ebsr", "ebpr", "ebsr"):
        C = api.spmm(Ad, Bd, strategy, stream=s)
        seg = api.segment(src, idx, A.nrow, "sum", stream=s)
        junk = torch.empty(64 << 20, dtype=torch.uint8, device="cuda").fill_(0xFF)  # on the current stream
        del junk
        outs.append((strategy, C, seg))
    torch.cuda.current_stream().wait_stream(s)
    torch.cuda.synchronize()
    C64, absC = oracle64(A, B)
    d64, dabs = oracle_lib.segment_coo_f64(src_h, A.coo_rows(), A.nrow, 0)
    for i, (strategy, C, seg) in enumerate(outs):
        check_close(C.cpu().numpy(), C64, absC, 1e-5, None, f"call {i} {strategy} on a side stream")
        check_close(seg.cpu().numpy(), d64, dabs, 1e-5, None, f"call {i} segment on a side stream")
