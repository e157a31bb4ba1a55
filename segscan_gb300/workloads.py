"""Profiling reproducer (measurement infrastructure, not part of the
library's API and not imported by the package): named single-kernel
workloads that run one case a few times and print its device time and
algorithmic throughput (GB/s of the bytes the operation must move).  The
commands of the ncu summaries under profiles/ run it, so each summary can be
reproduced on the synthetic matrices the benchmark configurations name.

    python -m segscan_gb300.workloads <case> [--iters K] [--scale S]

Cases: spmm-<strategy>-n<N> (strategy ebpr|rbpr|ebsr|rbsr, power-law
1e6 x 1e6), spmm-ebsr-banded-n64, spmm-ebsr-bf16-n64, segment-<sr|pr>-<sum|max|mean>-n<N>
(segments = the power-law matrix's rows), transpose, sddmm-n64,
backward-<f32|bf16>-n<N> (the fused backward of the 2e6 power-law layer), batched-bf16-n64,
batched-plain-n64 (the same 512 matrices, one launch each).
--scale shrinks the matrices (rows / scale) for small profiling runs.
"""
from __future__ import annotations

import argparse
import json
import sys

import torch

from . import api, autotune, synth


def _time(fn, iters):
    fn()
    torch.cuda.synchronize()
    s = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(s)
    for _ in range(iters):
        fn()
    e1.record(s)
    e1.synchronize()
    return e0.elapsed_time(e1) / iters


def _powerlaw(scale):
    M = max(1000, 1_000_000 // scale)
    return synth.powerlaw(M, M, 2.1, 1, max(10, 20000 // scale), seed=1)


# knobs the power-law N = 64 benchmark runs with (measured best of the ebsr sweep)
BEST = {("ebsr", 64): dict(group_factor=4, thread_nz=32, thread_per_block=256, block_denom=1)}


def parse_knobs(text: str | None) -> dict:
    """'k=v:k=v' or a JSON object."""
    if not text:
        return {}
    if text.lstrip().startswith("{"):
        return json.loads(text)
    return {k: int(v) for k, v in (item.split("=") for item in text.split(":") if item)}


def run(case: str, iters: int, scale: int, knobs: dict | None = None) -> dict:
    dev = torch.device("cuda")
    parts = case.split("-")
    if parts[0] == "spmm":
        strategy = parts[1]
        N = int(parts[-1][1:])
        dtype = torch.bfloat16 if "bf16" in parts else torch.float32
        A = synth.banded(max(1000, 120_000 // scale), max(1000, 120_000 // scale), 20, 500, seed=1) \
            if "banded" in parts else _powerlaw(scale)
        B = synth.dense(A.ncol, N, seed=2)
        Ad = api.CsrMatrix.from_host(A, dev, dtype)
        Bd = torch.from_numpy(B).to(dev).to(dtype)
        k = api.make_knobs(strategy, N, **(knobs or BEST.get((strategy, N), {})))
        C = torch.empty((A.nrow, N), device=dev)
        n = api.spmm_workspace_size(Ad, N, strategy, k)
        ws = torch.empty(n + 256, dtype=torch.uint8, device=dev) if n else None
        ms = _time(lambda: api.spmm(Ad, Bd, strategy, knobs=k, out=C, workspace=ws), iters)
        vb = 2 if dtype != torch.float32 else 4
        nb = synth.spmm_bytes(A, N, val_bytes=vb, b_bytes=vb)
    elif parts[0] == "segment":
        strategy, reduce, N = parts[1], parts[2], int(parts[3][1:])
        A = _powerlaw(scale)
        index = torch.from_numpy(A.coo_rows()).to(dev)
        src = torch.rand((A.nnz, N), device=dev)
        out = torch.empty((A.nrow, N), device=dev)
        k = api.make_knobs("ebsr" if strategy == "sr" else "ebpr", N, **knobs) if knobs else None
        ms = _time(lambda: api.segment(src, index, A.nrow, reduce, strategy, knobs=k, out=out), iters)
        nb = synth.segment_bytes(A.nnz, N, A.nrow)
    elif parts[0] == "transpose":
        A = _powerlaw(scale)
        Ad = api.CsrMatrix.from_host(A, dev)
        ms = _time(lambda: api.transpose(Ad), iters)
        nb = A.nnz * 4 * 6 + (A.ncol + 1) * 4 * 3  # read cols, write/sort perm, rows, gather values
    elif parts[0] == "backward":
        # fused backward (dA.values and dB = A^T dC in one walk over A^T) of
        # the 2e6 x 2e6 power-law layer (Zipf 2.1 clipped to 50000, seed 4);
        # backward-<f32|bf16>-n<N>
        dtype = torch.bfloat16 if parts[1] == "bf16" else torch.float32
        N = int(parts[2][1:])
        M = max(1000, 2_000_000 // scale)
        A = synth.powerlaw(M, M, 2.1, 1, max(10, 50_000 // scale), seed=4)
        Ad = api.CsrMatrix.from_host(A, dev, dtype)
        AT, perm = api.transpose(Ad)
        dC = torch.randn((A.nrow, N), device=dev)
        Bd = torch.rand((A.ncol, N), device=dev).to(dtype)
        out16 = dtype if dtype != torch.float32 else None
        ms = _time(lambda: api.spmm_backward(AT, perm, Ad.values, dC, Bd, out16), iters)
        vb = 2 if dtype != torch.float32 else 4
        # A^T's pattern and perm, the values, dC rows once, B and dB once, dvals
        nb = A.nnz * (4 + 4 + vb + 4) + (A.ncol + 1) * 4 + A.nrow * N * 4 + 2 * A.ncol * N * vb
    elif parts[0] == "sddmm":
        N = int(parts[1][1:])
        A = _powerlaw(scale)
        Ad = api.CsrMatrix.from_host(A, dev)
        dC = torch.rand((A.nrow, N), device=dev)
        Bd = torch.rand((A.ncol, N), device=dev)
        ms = _time(lambda: api.sddmm(Ad, dC, Bd), iters)
        nb = A.nnz * 12 + (A.nrow + 1) * 4 + A.nrow * N * 4 + A.distinct_columns() * N * 4
    elif parts[0] == "batched" and parts[1] == "plain":
        # the comparison for the batched launch: one ordinary launch per matrix
        from . import batched
        N = int(parts[-1][1:])
        mats_h = synth.batch(max(8, 512 // scale), 100, 50_000, 2.3, 2000, seed=3)
        mats = [api.CsrMatrix.from_host(A, dev) for A in mats_h]
        Bs = [torch.rand((A.ncol, N), device=dev) for A in mats_h]
        outs = [torch.empty((A.nrow, N), device=dev) for A in mats_h]
        kn = autotune.batch_knobs(mats, N)
        wss = []
        for A, k in zip(mats, kn):
            n = api.spmm_workspace_size(A, N, "ebsr", k)
            wss.append(torch.empty(n + 256, dtype=torch.uint8, device=dev) if n else None)
        ms = _time(lambda: batched.plain_per_matrix(mats, Bs, outs, [("ebsr", k) for k in kn], wss), iters)
        nb = sum(synth.spmm_bytes(A, N) for A in mats_h)
    elif parts[0] == "batched":
        from . import batched
        N = int(parts[-1][1:])
        dtype = torch.bfloat16 if "bf16" in parts else torch.float32
        mats_h = synth.batch(max(8, 512 // scale), 100, 50_000, 2.3, 2000, seed=3)
        mats = [api.CsrMatrix.from_host(A, dev, dtype) for A in mats_h]
        Bs = [torch.rand((A.ncol, N), device=dev).to(dtype) for A in mats_h]
        plan = batched.BatchedSpMM(mats, Bs, out_dtype=dtype, knobs=autotune.batch_knobs(mats, N))
        plan.capture()
        ms = _time(plan.replay, iters)
        vb = 2 if dtype != torch.float32 else 4
        nb = sum(synth.spmm_bytes(A, N, val_bytes=vb, b_bytes=vb, c_bytes=vb) for A in mats_h)
    else:
        raise SystemExit(f"unknown case {case}")
    return {"case": case, "ms": ms, "GB/s": nb / ms / 1e6, "bytes": nb}


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("case")
    ap.add_argument("--iters", type=int, default=5)
    ap.add_argument("--scale", type=int, default=1)
    ap.add_argument("--knobs", default=None, help="k=v:k=v or JSON; default: the library's defaults")
    a = ap.parse_args(argv)
    print(json.dumps(run(a.case, a.iters, a.scale, parse_knobs(a.knobs))), flush=True)


if __name__ == "__main__":
    sys.exit(main())
