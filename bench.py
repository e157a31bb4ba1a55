#!/usr/bin/env python
"""SpMM benchmark: algorithmic HBM GB/s of C = A*B on the power-law matrix.

Workload (the configuration the headline metric is quoted on): A is
1,000,000 x 1,000,000 CSR with row lengths Zipf(2.1) clipped to [1, 20000]
and uniform columns (~4.6 M nonzeros), B is 1,000,000 x 64 FP32, seed 1;
synthetic data from segscan_gb300.synth.  One step = one SpMM
(C overwritten) through the C ABI.  Bytes per step are algorithmic:
nnz*(4+4) + (M+1)*4 + U*N*4 + M*N*4 with U = distinct columns of A.  B and C
(256 MB each) are larger than L2, so no flush is needed between steps.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

--impl reference times the reference's own CPU SpMM (its check path,
test-cg/include/util/check.cuh:139-158, restated in oracle/oracle.c and run
row-parallel on every host core) on the same workload.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "SpMM HBM GB/s (algorithmic bytes), power-law 1e6x1e6 Zipf2.1 N=64 FP32"
UNIT = "GB/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--N", type=int, default=64)
    ap.add_argument("--strategy", default="auto")
    ap.add_argument("--knobs", default=None,
                    help="knob overrides for --strategy: JSON or name=value:name=value")
    ap.add_argument("--e2e-steps", type=int, default=20)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--extras", dest="extras", action="store_true", default=True,
                    help="also measure BF16/FP16 precision, the 512-matrix batch and fwd+bwd (default)")
    ap.add_argument("--no-extras", dest="extras", action="store_false")
    return ap.parse_args()


def workload(N: int):
    from segscan_gb300 import synth
    A = synth.powerlaw(1_000_000, 1_000_000, 2.1, 1, 20000, seed=1)
    B = synth.dense(A.ncol, N, seed=2)
    return A, B


def config(A, N, extra=None):
    cfg = {"workload": "spmm_powerlaw_1e6_zipf2.1_clip20000_n%d_fp32" % N, "nrow": A.nrow, "ncol": A.ncol,
           "nnz": A.nnz, "N": N, "distinct_cols": A.distinct_columns(), "dtype_values": "f32",
           "dtype_B": "f32", "dtype_C": "f32", "seed": 1,
           "l2": "no flush: B and C (256 MB each) exceed the 126 MB L2"}
    if extra:
        cfg.update(extra)
    return cfg


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def traffic_from_profiles(kernel_file: str):
    """Per-launch DRAM bytes of the dominant kernel from the committed ncu summary, if any."""
    p = ROOT / "profiles" / kernel_file
    if not p.exists():
        return None
    for line in p.read_text().splitlines():
        if line.startswith("traffic_bytes_per_launch_full_workload:"):
            try:
                return int(float(line.split(":", 1)[1].strip()))
            except ValueError:
                return None
    return None


class ClockSampler:
    """nvidia-smi clocks and throttle reasons while the GPU is under load."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.file = None

    def start(self):
        try:
            self.file = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=self.file, stderr=subprocess.DEVNULL)
            time.sleep(0.3)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"], "samples": 0}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.file.flush()
        rows = []
        with open(self.file.name) as f:
            for line in f:
                parts = [x.strip() for x in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        os.unlink(self.file.name)
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        sm = []
        smax = None
        for r in rows:
            try:
                sm.append(float(r[1]))
                smax = float(r[2])
            except ValueError:
                continue
            for i, n in enumerate(names):
                if r[5 + i].lower() == "active":
                    reasons.add(n)
        loaded = [x for x in sm if smax and x > 0.5 * smax] or sm
        return {"sm_mhz": statistics.median(loaded) if loaded else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(rows)}


def dist_setup(args):
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def cpu_spmm_time(A, B, threads: int, budget_s: float, min_iters: int = 2, max_iters: int = 50):
    """Times the reference's CPU SpMM (oracle port: zero C, then the check-path
    loop, a row block per thread) on A, B: seconds per pass."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import numpy as np
    import oracle_lib
    out = np.empty((A.nrow, B.shape[1]), dtype=np.float32)
    times = []
    start = time.perf_counter()
    while len(times) < max_iters:
        t0 = time.perf_counter()
        oracle_lib.spmm_check_f32(A.indptr, A.indices, A.values, B, threads=threads, out=out)
        times.append(time.perf_counter() - t0)
        if len(times) >= min_iters and time.perf_counter() - start > budget_s:
            break
    return statistics.median(times), len(times)


def cpu_sample(A, B, target_s: float, threads: int):
    """Row block of A whose CPU pass takes about target_s (the whole matrix if faster)."""
    from segscan_gb300 import synth
    t, _ = cpu_spmm_time(A, B, threads, 0.0, 1, 1)
    if t <= target_s:
        return A, "whole matrix", t
    frac = target_s / t
    rows = max(1, int(A.nrow * frac))
    sub = synth.Csr(rows, A.ncol, A.indptr[:rows + 1].copy(), A.indices[:A.indptr[rows]].copy(),
                    A.values[:A.indptr[rows]].copy())
    return sub, f"first {rows} rows", None


def run_reference(args):
    ws, rank, _ = dist_setup(args)
    if rank != 0:
        return
    from segscan_gb300 import synth
    A, B = workload(args.N)
    threads = os.cpu_count() or 1
    sample, desc, _ = cpu_sample(A, B, 2.0, threads)
    nbytes = synth.spmm_bytes(sample, args.N)
    sys.path.insert(0, str(ROOT / "oracle"))
    import numpy as np
    import oracle_lib
    out = np.empty((sample.nrow, args.N), dtype=np.float32)
    for _ in range(max(0, args.warmup)):
        oracle_lib.spmm_check_f32(sample.indptr, sample.indices, sample.values, B, threads=threads, out=out)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        oracle_lib.spmm_check_f32(sample.indptr, sample.indices, sample.values, B, threads=threads, out=out)
    dt = (time.perf_counter() - t0) / args.steps
    gbs = nbytes / dt / 1e9
    line = {"metric": METRIC, "value": gbs, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": dt * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": config(A, args.N, {"sample": desc}), "impl": "reference",
            "cpu_baseline": {"value": gbs, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": f"{desc} of the workload, row-parallel restatement of "
                                       "spmm_reference_host (check.cuh:139-158)"},
            "e2e": {"value": gbs, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def choose(args, A_dev, N):
    from segscan_gb300 import api, autotune
    if args.strategy != "auto":
        kw = {}
        if args.knobs:
            if args.knobs.lstrip().startswith("{"):
                kw = json.loads(args.knobs)
            else:
                kw = {k: int(v) for k, v in (item.split("=") for item in args.knobs.split(":") if item)}
        return args.strategy, api.make_knobs(args.strategy, N, **kw)
    return autotune.best(A_dev, N)


def _event_ms(fn, iters, stream, warm=2):
    import torch
    for _ in range(warm):
        fn()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(iters):
        fn()
    e1.record(stream)
    e1.synchronize()
    return e0.elapsed_time(e1) / iters


def _errors(C, C64, absC):
    import numpy as np
    err = np.abs(C.astype(np.float64) - C64)
    return {"normwise_rel": float(np.linalg.norm(err) / max(np.linalg.norm(C64), 1e-300)),
            "max_rel_to_sum_abs": float((err / np.maximum(absC, 1e-300)).max()),
            "max_abs_over_max_ref": float(err.max() / max(np.abs(C64).max(), 1e-300))}


def _f64_product(A, B):
    """C = A @ B and |A| @ |B| in FP64 on the host (scipy's CSR product),
    the exact-enough reference the precision errors are measured against."""
    import numpy as np
    import scipy.sparse as sp
    M = sp.csr_matrix((A.values.astype(np.float64), A.indices, A.indptr), shape=(A.nrow, A.ncol))
    B64 = B.astype(np.float64)
    return np.asarray(M @ B64), np.asarray(abs(M) @ np.abs(B64))


def _check_output(A, B, C):
    """The timed C against FP64 (scipy): max |C - C64| / (|A||B|) per element
    and the normwise error, with the FP32 bar of the parity tests (1e-5)."""
    import numpy as np
    C64, absC = _f64_product(A, B)
    e = _errors(C.cpu().numpy(), C64, absC)
    return {"max_err": e["max_rel_to_sum_abs"], "normwise_err": e["normwise_rel"], "bar": 1e-5,
            "pass": bool(e["max_rel_to_sum_abs"] <= 1e-5 and e["normwise_rel"] <= 1e-5
                         and np.isfinite(e["normwise_rel"])),
            "against": "FP64 product on the host (scipy), per element relative to sum|a*b|"}


def extra_precision(A, B, N, fp32_ms, dev):
    """BF16 / FP16 storage of A.vals and B, FP32 accumulation (Kahan on rows
    above 1024 nonzeros), on the power-law matrix: throughput beside plain
    FP32, and error against FP64 on the FP32 inputs."""
    import torch
    from segscan_gb300 import api, autotune, synth
    C64, absC = _f64_product(A, B)
    out = {}
    stream = torch.cuda.current_stream(dev)
    for name, dt, cdt in (("bf16_c_f32", torch.bfloat16, torch.float32), ("bf16_c_bf16", torch.bfloat16, torch.bfloat16),
                          ("f16_c_f32", torch.float16, torch.float32)):
        Ad = api.CsrMatrix.from_host(A, dev, dt)
        Bd = torch.from_numpy(B).to(dev).to(dt)
        strategy, k = autotune.best(Ad, N, Bd)
        Cd = torch.empty((A.nrow, N), dtype=cdt, device=dev)
        wsz = api.spmm_workspace_size(Ad, N, strategy, k)
        ws = torch.empty(wsz + 256, dtype=torch.uint8, device=dev) if wsz else None
        ms = _event_ms(lambda: api.spmm(Ad, Bd, strategy, knobs=k, out=Cd, workspace=ws), 20, stream)
        nb = synth.spmm_bytes(A, N, val_bytes=2, b_bytes=2, c_bytes=2 if cdt != torch.float32 else 4)
        out[name] = {"ms": ms, "GB/s": nb / ms / 1e6, "speedup_vs_fp32": fp32_ms / ms, "strategy": strategy,
                     "knobs": k.as_dict(), **_errors(Cd.float().cpu().numpy(), C64, absC)}
    # the same at N = 128 (B and C twice as wide), against the FP32 time there
    B128 = synth.dense(A.ncol, 128, seed=2)
    C64, absC = _f64_product(A, B128)
    A32 = api.CsrMatrix.from_host(A, dev)
    B32 = torch.from_numpy(B128).to(dev)
    s32, k32 = autotune.best(A32, 128, B32)
    C32 = torch.empty((A.nrow, 128), device=dev)
    w32 = api.spmm_workspace_size(A32, 128, s32, k32)
    ws32 = torch.empty(w32 + 256, dtype=torch.uint8, device=dev) if w32 else None
    ms32 = _event_ms(lambda: api.spmm(A32, B32, s32, knobs=k32, out=C32, workspace=ws32), 20, stream)
    del A32, B32, C32, ws32
    Ad = api.CsrMatrix.from_host(A, dev, torch.bfloat16)
    Bd = torch.from_numpy(B128).to(dev).to(torch.bfloat16)
    strategy, k = autotune.best(Ad, 128, Bd)
    Cd = torch.empty((A.nrow, 128), device=dev)
    wsz = api.spmm_workspace_size(Ad, 128, strategy, k)
    ws = torch.empty(wsz + 256, dtype=torch.uint8, device=dev) if wsz else None
    ms = _event_ms(lambda: api.spmm(Ad, Bd, strategy, knobs=k, out=Cd, workspace=ws), 20, stream)
    nb = synth.spmm_bytes(A, 128, val_bytes=2, b_bytes=2)
    out["bf16_c_f32_n128"] = {"ms": ms, "GB/s": nb / ms / 1e6, "fp32_ms": ms32, "speedup_vs_fp32": ms32 / ms,
                              "strategy": strategy, "knobs": k.as_dict(), **_errors(Cd.cpu().numpy(), C64, absC)}
    out["tolerance"] = "normwise <= 2e-2 vs FP64 on FP32 inputs"
    return out


def extra_batched(dev, N=64, count=512, headline=None):
    """512 CSR matrices (rows log-uniform in [100, 50000], row length Zipf 2.3
    clipped to [1, 2000], seed 3): one persistent launch replayed from a CUDA
    graph (BF16 storage, FP32 accumulation) against one plain FP32 launch per
    matrix, and like for like: batched BF16 against batched FP32 on the same
    matrices, and batched BF16 against the plain FP32 headline SpMM per
    nonzero (headline = (nnz, ms) of the timed FP32 step)."""
    import numpy as np
    import torch
    from segscan_gb300 import api, autotune, batched, synth
    mats_h = synth.batch(count, 100, 50_000, 2.3, 2000, seed=3)
    rng = np.random.default_rng(33)
    Bh = [(rng.random((A.ncol, N), dtype=np.float32) * 2 - 1) for A in mats_h]
    stream = torch.cuda.current_stream(dev)
    res = {"matrices": count, "rows": int(sum(A.nrow for A in mats_h)), "nnz": int(sum(A.nnz for A in mats_h))}
    mats32 = [api.CsrMatrix.from_host(A, dev) for A in mats_h]
    B32 = [torch.from_numpy(b).to(dev) for b in Bh]
    outs = [torch.empty((A.nrow, N), device=dev) for A in mats_h]
    # the comparison: one ordinary launch per matrix, at the chunk size
    # (128, 256 or 512 nonzeros) that makes those launches fastest; a small
    # matrix is one short chain of dependent loads per chunk, so smaller
    # chunks finish sooner
    best = None
    for target in (128, 256, 512):
        knobs32 = autotune.batch_knobs(mats32, N, target)
        wss = []
        for A, k in zip(mats32, knobs32):
            n = api.spmm_workspace_size(A, N, "ebsr", k)
            wss.append(torch.empty(n + 256, dtype=torch.uint8, device=dev) if n else None)
        plain = (lambda kk, ww: lambda: batched.plain_per_matrix(mats32, B32, outs, [("ebsr", k) for k in kk], ww))(
            knobs32, wss)
        ms = _event_ms(plain, 3, stream, warm=1)
        if best is None or ms < best[0]:
            best = (ms, target, plain)
    plain_ms, plain_target, plain = best
    res["plain_fp32_per_matrix_ms"] = plain_ms
    res["plain_chunk_target"] = plain_target
    # the same per-matrix launches replayed from one CUDA graph (no host
    # overhead left: what remains is one memset and one walk per matrix)
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        plain()
    plain_graph_ms = _event_ms(g.replay, 5, stream)
    res["plain_fp32_per_matrix_graph_ms"] = plain_graph_ms
    del g
    for name, dt, cdt in (("batched_fp32_graph", torch.float32, torch.float32),
                          ("batched_bf16_graph", torch.bfloat16, torch.bfloat16),
                          ("batched_bf16_c_f32_graph", torch.bfloat16, torch.float32)):
        mats = [api.CsrMatrix.from_host(A, dev, dt) for A in mats_h]
        Bs = [b.to(dt) for b in B32]
        target, tried = autotune.tune_batch(mats, Bs, N)
        strategies, knobs = autotune.batch_plan(mats, N, target)  # strategy and chunk per matrix
        plan = batched.BatchedSpMM(mats, Bs, out_dtype=cdt, knobs=knobs, strategies=strategies)
        plan.capture()
        ms = _event_ms(plan.replay, 10, stream)
        err = []
        for i in range(0, count, 64):  # spot-check a few matrices against FP32 per-matrix results
            ref = outs[i].double()
            err.append(float((plan.out[i].double() - ref).norm() / max(float(ref.norm()), 1e-300)))
        res[name] = {"ms": ms, "rbsr_matrices": strategies.count("rbsr"), "speedup_vs_plain_fp32": plain_ms / ms,
                     "speedup_vs_plain_fp32_graph": plain_graph_ms / ms, "chunk_target": target,
                     "max_normwise_rel_vs_fp32": max(err), "gnnz_per_s": res["nnz"] / ms / 1e6}
    # like for like: the same batch in FP32 and BF16, and BF16 per nonzero
    # against the plain FP32 headline SpMM
    res["bf16_over_fp32_batched"] = res["batched_fp32_graph"]["ms"] / res["batched_bf16_c_f32_graph"]["ms"]
    if headline is not None:
        h_nnz, h_ms = headline
        res["plain_fp32_headline_gnnz_per_s"] = h_nnz / h_ms / 1e6
        res["batched_bf16_over_plain_fp32_per_nnz"] = (res["batched_bf16_c_f32_graph"]["gnnz_per_s"]
                                                       / res["plain_fp32_headline_gnnz_per_s"])
    return res


def _cusparse_ms(A, B, stream):
    """cuSPARSE CSR SpMM through torch.sparse.mm on the same matrix (comparison line)."""
    import torch
    At = torch.sparse_csr_tensor(A.indptr.long(), A.indices.long(), A.values, (A.nrow, A.ncol))
    return _event_ms(lambda: torch.sparse.mm(At, B), 10, stream)


CUSPARSE_LINE = ROOT / "_build" / "bench_cusparse.so"


def _cusparse_direct_ms(A, B, stream, C_ours=None):
    """cusparseSpMM (CSR, CUSPARSE_SPMM_ALG_DEFAULT) with its handle,
    descriptors and workspace made once (bench_cusparse.cu, the reference's
    cuSPARSE call): ms per call, and its normwise difference from C_ours."""
    import ctypes
    import torch
    lib = ctypes.CDLL(str(CUSPARSE_LINE))
    vp = ctypes.c_void_p
    lib.csp_create.argtypes = [ctypes.POINTER(vp), ctypes.c_int, ctypes.c_int, ctypes.c_int, vp, vp, vp,
                               ctypes.c_int, vp, vp]
    lib.csp_run.argtypes = [vp, vp]
    lib.csp_destroy.argtypes = [vp]
    N = int(B.shape[1])
    C = torch.empty((A.nrow, N), device=B.device)
    h = vp()
    st = lib.csp_create(ctypes.byref(h), A.nrow, A.ncol, A.nnz, A.indptr.data_ptr(), A.indices.data_ptr(),
                        A.values.data_ptr(), N, B.data_ptr(), C.data_ptr())
    if st:
        raise RuntimeError(f"cuSPARSE setup failed with status {st}")
    try:
        s = vp(stream.cuda_stream)
        ms = _event_ms(lambda: lib.csp_run(h, s), 10, stream)
        diff = None
        if C_ours is not None:
            diff = float((C.double() - C_ours.double()).norm() / max(float(C_ours.double().norm()), 1e-300))
        return ms, diff
    finally:
        lib.csp_destroy(h)


def extra_sweep(A_pl, dev):
    """Every configuration's shape through the tuned strategy, with cuSPARSE
    beside it (cusparseSpMM with handle and descriptors made once, and
    torch.sparse.mm): power-law 1e6 at N = 4, 16, 64, 128; banded 120k x 120k
    (20 per row, half-width 500) at N = 64; Poisson(16) 4096 x 4096 at
    N = 4, 16 (L2-resident and launch bound: no roofline meaning)."""
    import torch
    from segscan_gb300 import api, autotune, synth
    stream = torch.cuda.current_stream(dev)
    res = {}
    cases = [("powerlaw_1e6", A_pl, N) for N in (4, 16, 64, 128)]
    cases.append(("banded_120k", synth.banded(120_000, 120_000, 20, 500, seed=1), 64))
    P = synth.poisson(4096, 4096, 16.0, seed=0)
    cases += [("poisson_4096", P, 4), ("poisson_4096", P, 16)]
    for name, A, N in cases:
        Ad = api.CsrMatrix.from_host(A, dev)
        B = torch.from_numpy(synth.dense(A.ncol, N, seed=2)).to(dev)
        strategy, k = autotune.best(Ad, N, B)
        C = torch.empty((A.nrow, N), device=dev)
        # through an SpmmPlan: the small matrices' kernels are shorter than
        # api.spmm's per-call host work
        plan = api.SpmmPlan(Ad, N, strategy, k)
        ms = _event_ms(lambda: plan.run(B, C), 20, stream)
        nb = synth.spmm_bytes(A, N)
        entry = {"nnz": A.nnz, "ms": ms, "GB/s": nb / ms / 1e6, "strategy": strategy, "knobs": k.as_dict(),
                 "api": "SpmmPlan.run"}
        try:
            cs = _cusparse_ms(Ad, B, stream)
            entry.update({"cusparse_torch_ms": cs, "speedup_vs_cusparse_torch": cs / ms})
        except Exception as exc:
            entry["cusparse_torch_error"] = f"{type(exc).__name__}: {exc}"
        try:
            cd, diff = _cusparse_direct_ms(Ad, B, stream, C_ours=C)
            entry.update({"cusparse_ms": cd, "speedup_vs_cusparse": cd / ms, "cusparse_normwise_diff": diff})
        except Exception as exc:
            entry["cusparse_error"] = f"{type(exc).__name__}: {exc}"
        res[f"{name}_n{N}"] = entry
        del Ad, B, C, plan
        torch.cuda.empty_cache()
    return res


def extra_fwd_bwd(dev, N=128):
    """Differentiated SpMM layer: power-law 2e6 x 2e6 (Zipf 2.1 clipped to
    [1, 50000], seed 4), B 2e6 x 128, dC ~ N(0, 1).  Forward C = A B;
    backward dA.vals and dB = A^T dC from one fused walk over the
    device-built transpose (built once per pattern; its time is reported
    apart), with the separate SDDMM and A^T dC times beside it."""
    import numpy as np
    import torch
    from segscan_gb300 import api, autograd, synth
    A = synth.powerlaw(2_000_000, 2_000_000, 2.1, 1, 50_000, seed=4)
    stream = torch.cuda.current_stream(dev)
    rng = np.random.default_rng(4)
    dC = torch.from_numpy(rng.standard_normal((A.nrow, N), dtype=np.float32)).to(dev)
    B32 = torch.from_numpy(synth.dense(A.ncol, N, seed=44)).to(dev)
    res = {"nrow": A.nrow, "nnz": A.nnz, "N": N}
    # one B row per group: 32 lanes x 4 FP32, or 16 lanes x 8 BF16 (16 bytes per lane either way)
    knobs32 = api.make_knobs("ebsr", N, group_factor=5, thread_nz=32, thread_per_block=512, block_denom=1)
    knobs16 = api.make_knobs("ebsr", N, group_factor=4, coarsen_factor=8, thread_nz=32, thread_per_block=512,
                             block_denom=1)
    def one(dt):
        knobs = knobs32 if dt == torch.float32 else knobs16
        Ad = api.CsrMatrix.from_host(A, dev, dt, values=False)
        vals = torch.from_numpy(A.values).to(dev).to(dt).requires_grad_(True)
        Bd = B32.detach().to(dt, copy=True).requires_grad_(True)  # a fresh leaf for each precision
        pat = autograd.pattern(Ad)
        t_ms = _event_ms(lambda: api.transpose(Ad), 3, stream, warm=1)
        pat.transposed()

        def step():
            vals.grad = None
            Bd.grad = None
            C = autograd.spmm(Ad, vals, Bd, "ebsr", knobs, "ebsr", pattern=pat, bw_knobs=knobs32)
            C.backward(dC)

        def fwd():
            autograd.spmm(Ad, vals.detach(), Bd.detach(), "ebsr", knobs, pattern=pat)

        total = _event_ms(step, 5, stream, warm=3)
        f = _event_ms(fwd, 5, stream, warm=3)
        # the backward's pieces, timed alone
        A_v = Ad.with_values(vals.detach())
        sd = _event_ms(lambda: api.sddmm(A_v, dC, Bd.detach()), 5, stream)
        AT, perm = pat.transposed()
        AT_v = AT.with_values(api.gather_values(vals.detach().float(), perm))
        dB = torch.empty((A.ncol, N), device=dev)
        db = _event_ms(lambda: api.spmm(AT_v, dC, "ebsr", knobs=knobs32, out=dB), 5, stream)
        # the backward the autograd binding runs: both gradients from one walk over A^T
        out16 = dt if dt != torch.float32 else None
        fb = _event_ms(lambda: api.spmm_backward(AT, perm, vals.detach(), dC, Bd.detach(), out16), 5, stream)
        return {"fwd_bwd_ms": total, "fwd_ms": f, "bwd_ms": total - f, "fused_bwd_ms": fb,
                "separate_sddmm_ms": sd, "separate_dB_spmm_ms": db, "transpose_build_ms": t_ms,
                "knobs_fwd": knobs.as_dict()}

    # each precision in its own scope, the allocator's cache emptied between,
    # so one run's gigabyte-sized temporaries do not crowd the next
    for name, dt in (("fp32", torch.float32), ("bf16", torch.bfloat16)):
        torch.cuda.empty_cache()
        res[name] = one(dt)
    return res


def run_ours(args):
    import torch
    from segscan_gb300 import api, synth

    ws_, rank, local = dist_setup(args)
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if ws_ > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=dev)
    from segscan_gb300 import partition
    A, B = workload(args.N)
    N = args.N
    nbytes = synth.spmm_bytes(A, N)  # the whole job's algorithmic bytes, over every rank's rows
    # each rank holds its nnz-balanced row block of A (all of A on one GPU)
    # and a replicated B, and computes its rows of C with no collective: the
    # one matrix split over the ranks (strong scaling)
    S = partition.ShardedSpMM(A, rank, ws_, partition.DeviceKernels(dev))
    Ah, Ad = S.part, S.A
    Bd = torch.from_numpy(B).to(dev)
    strategy, knobs = choose(args, Ad, N)
    S.kernels.strategy, S.kernels.knobs = strategy, knobs
    C = torch.empty((Ah.nrow, N), dtype=torch.float32, device=dev)
    work = S.kernels.workspace(Ad, N)
    stream = torch.cuda.current_stream(dev)
    # ebsr: one walk launch (straddling rows assembled inside it, after a
    # memset of the arrival counts); ebpr: scan + fix-up; row-balanced: one
    kernels_per_step = 2 if strategy == "ebpr" else 1

    def step():
        S.forward(Bd, out=C, workspace=work, stream=stream)

    sampler = ClockSampler(local)
    sampler.start()
    for _ in range(max(3, args.warmup)):
        step()
    torch.cuda.synchronize(dev)

    def barrier():
        if ws_ > 1:
            import torch.distributed as dist
            dist.barrier()

    barrier()
    torch.cuda.synchronize(dev)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        step()
    e1.record(stream)
    torch.cuda.synchronize(dev)
    barrier()
    t = e0.elapsed_time(e1) / 1e3 / args.steps
    if ws_ > 1:
        import torch.distributed as dist
        tt = torch.tensor([t], device=dev, dtype=torch.float64)
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        t = float(tt.item())
    # the C the timed steps wrote, checked once (outside the timed region)
    # against an FP64 product on the host, at the FP32 parity bar
    check = _check_output(Ah, B, C)

    # end to end through the public API: host inputs in pinned memory,
    # H2D of A and B, the SpMM, D2H of C, every step.  Copies in, the SpMM
    # and the copy out run on three streams, and consecutive steps alternate
    # between two device buffer sets, ordered by events: step i's inputs go
    # up while step i-1 computes and step i-2's C comes down, so both link
    # directions stay busy (each step still moves all of its own bytes)
    h_indptr = torch.from_numpy(Ah.indptr).pin_memory()
    h_indices = torch.from_numpy(Ah.indices).pin_memory()
    h_values = torch.from_numpy(Ah.values).pin_memory()
    h_B = torch.from_numpy(B).pin_memory()
    e2e_streams = [torch.cuda.Stream(dev), torch.cuda.Stream(dev), torch.cuda.Stream(dev)]  # in, compute, out
    ev_in = [torch.cuda.Event() for _ in range(2)]     # set k's inputs are on the device
    ev_done = [torch.cuda.Event() for _ in range(2)]   # set k's SpMM finished (its inputs are free)
    ev_out = [torch.cuda.Event() for _ in range(2)]    # set k's C is on the host (its C is free)
    sets = []
    for _ in range(2):
        d = dict(indptr=torch.empty_like(Ad.indptr), indices=torch.empty_like(Ad.indices),
                 values=torch.empty_like(Ad.values), B=torch.empty_like(Bd), C=torch.empty_like(C),
                 hC=torch.empty((Ah.nrow, N), dtype=torch.float32).pin_memory(),
                 ws=torch.empty_like(work) if work is not None else None)
        d["A"] = api.CsrMatrix(Ah.nrow, Ah.ncol, d["indptr"], d["indices"], d["values"])
        sets.append(d)
    h2d = sum(x.numel() * x.element_size() for x in (h_indptr, h_indices, h_values, h_B))
    d2h = sets[0]["hC"].numel() * sets[0]["hC"].element_size()

    def e2e_step(i):
        k = i % 2
        d = sets[k]
        s_in, s_cmp, s_out = e2e_streams
        with torch.cuda.stream(s_in):
            if i >= 2:
                s_in.wait_event(ev_done[k])  # the SpMM of step i-2 no longer reads set k's inputs
            d["indptr"].copy_(h_indptr, non_blocking=True)
            d["indices"].copy_(h_indices, non_blocking=True)
            d["values"].copy_(h_values, non_blocking=True)
            d["B"].copy_(h_B, non_blocking=True)
            ev_in[k].record(s_in)
        with torch.cuda.stream(s_cmp):
            s_cmp.wait_event(ev_in[k])
            if i >= 2:
                s_cmp.wait_event(ev_out[k])  # step i-2's C has left set k
            api.spmm(d["A"], d["B"], strategy, knobs=knobs, out=d["C"], workspace=d["ws"], stream=s_cmp)
            ev_done[k].record(s_cmp)
        with torch.cuda.stream(s_out):
            s_out.wait_event(ev_done[k])
            d["hC"].copy_(d["C"], non_blocking=True)
            ev_out[k].record(s_out)

    def e2e_run(k):
        for s_ in e2e_streams:
            s_.wait_stream(stream)
        for i in range(k):
            e2e_step(i)
        for s_ in e2e_streams:
            stream.wait_stream(s_)

    t_e2e = float("nan")
    if args.e2e_steps > 0:
        e2e_run(2)
        torch.cuda.synchronize(dev)
        barrier()
        e0.record(stream)
        e2e_run(args.e2e_steps)
        e1.record(stream)
        torch.cuda.synchronize(dev)
        t_e2e = e0.elapsed_time(e1) / 1e3 / args.e2e_steps
    # link diagnostics for the e2e number: pinned-copy GB/s one way, and both
    # ways at once on two streams
    copy_gbs = {}
    if args.e2e_steps > 0:
        d0, d1 = sets[0], sets[1]

        def timed(fn, nbytes_, reps=5):
            fn()
            torch.cuda.synchronize(dev)
            e0.record(stream)
            for _ in range(reps):
                fn()
            e1.record(stream)
            torch.cuda.synchronize(dev)
            return nbytes_ * reps / (e0.elapsed_time(e1) / 1e3) / 1e9

        def both():
            for s_ in e2e_streams:
                s_.wait_stream(stream)
            with torch.cuda.stream(e2e_streams[0]):
                d0["B"].copy_(h_B, non_blocking=True)
            with torch.cuda.stream(e2e_streams[1]):
                d1["hC"].copy_(d1["C"], non_blocking=True)
            for s_ in e2e_streams:
                stream.wait_stream(s_)

        nb_B, nb_C = h_B.numel() * 4, d2h
        copy_gbs = {"h2d": timed(lambda: d0["B"].copy_(h_B, non_blocking=True), nb_B),
                    "d2h": timed(lambda: d0["hC"].copy_(d0["C"], non_blocking=True), nb_C),
                    "h2d_plus_d2h_concurrent": timed(both, nb_B + nb_C)}
    if ws_ > 1:
        import torch.distributed as dist
        tt = torch.tensor([t_e2e], device=dev, dtype=torch.float64)
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        t_e2e = float(tt.item())
    clocks = sampler.stop()

    if rank != 0:
        return
    peak, peak_kind = peaks()
    achieved = nbytes / t / 1e9  # the whole job: every rank's rows in the slowest rank's time
    per_gpu = achieved / ws_
    kernel_file = f"spmm_{strategy}_powerlaw_n{N}.md"
    line = {
        "metric": METRIC, "value": achieved, "unit": UNIT, "n_gpus": ws_, "steps": args.steps,
        "warmup": max(3, args.warmup), "ms_per_step": t * 1e3, "higher_is_better": True, "scaling": "strong",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": config(A, N, {"strategy": strategy, "knobs": knobs.as_dict(), "parallelism": f"row blocks x{ws_}, B replicated"}),
        "gflops": 2.0 * A.nnz * N / t / 1e9,
        "roofline": {"bound": "hbm", "achieved": per_gpu, "peak": peak, "unit": "GB/s",
                     "frac": per_gpu / peak, "peak_kind": peak_kind,
                     "traffic": traffic_from_profiles(kernel_file),
                     "gather_upper_bound_bytes": A.nnz * N * 4 + A.nnz * 8 + (A.nrow + 1) * 4 + A.nrow * N * 4,
                     "kernel": (f"{strategy} SpMM step (walk with in-kernel carry assembly)" if strategy == "ebsr"
                                else f"{strategy} SpMM step"),
                     "bytes_per_launch": nbytes},
        "e2e": {"value": nbytes / t_e2e / 1e9, "unit": UNIT, "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h, "ms_per_step": t_e2e * 1e3, "pinned_copy_gbs": copy_gbs},
        "check": check,
        "gpu_launches": kernels_per_step * args.steps,
        "clocks": clocks,
    }
    if ws_ == 1 and args.extras:
        configs = {}
        for key, fn in (("sweep_vs_cusparse", lambda: extra_sweep(A, dev)),
                        ("precision_powerlaw_n64", lambda: extra_precision(A, B, N, t * 1e3, dev)),
                        ("batched_512", lambda: extra_batched(dev, headline=(A.nnz, t * 1e3))),
                        ("fwd_bwd_powerlaw_2e6_n128", lambda: extra_fwd_bwd(dev))):
            try:
                configs[key] = fn()
            except Exception as exc:  # report, never hide, a failing extra measurement
                configs[key] = {"error": f"{type(exc).__name__}: {exc}"}
            torch.cuda.empty_cache()
        line["configs"] = configs
    if ws_ == 1 and not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        sample, desc, _ = cpu_sample(A, B, 2.0, threads)
        sec, iters = cpu_spmm_time(sample, B, threads, 10.0)
        line["cpu_baseline"] = {"value": synth.spmm_bytes(sample, N) / sec / 1e9, "unit": UNIT, "cores": threads,
                                "kind": "port", "sample": f"{desc}, {iters} passes, row-parallel restatement of "
                                                          "spmm_reference_host (check.cuh:139-158)"}
        # the reference's check loop as written runs on one thread: a separate line
        sample1, desc1, _ = cpu_sample(A, B, 2.0, 1)
        sec1, iters1 = cpu_spmm_time(sample1, B, 1, 4.0)
        line["cpu_baseline_single_thread"] = {"value": synth.spmm_bytes(sample1, N) / sec1 / 1e9, "unit": UNIT,
                                              "cores": 1, "kind": "port", "sample": f"{desc1}, {iters1} passes"}
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
