"""Autotuner: picks the SpMM strategy and knob tuple for a matrix.

The reference tunes by hand: a driver instantiates every knob tuple of a
grid (test-cg/src/test.cu:58-330, grids in test-cg/src/params.md) and an
Nsight Compute sweep ranks them offline (test-cg/src/test.py:49-59,
count.py).  Here the candidates (the README's best static tuples,
README.md:168-210, and params.md-style grids, plus the chunk sizes this
implementation favours) are timed once on the device with CUDA events and the
winner is cached by a shape signature built from row-length statistics, so
matrices of the same shape class reuse it without measuring again.
"""
from __future__ import annotations

import json
import math
import os
import threading
from pathlib import Path
from typing import Optional

import numpy as np
import torch

from . import api
from ._lib import SsKnobs

_LOCK = threading.Lock()
_MEM: dict = {}


def cache_path() -> Path:
    p = os.environ.get("SEGSCAN_TUNE_CACHE")
    if p:
        return Path(p)
    return Path(os.path.expanduser("~")) / ".cache" / "segscan_gb300" / "tune.json"


def features(A: api.CsrMatrix) -> dict:
    lengths = torch.diff(A.indptr).to(torch.float64)
    M = max(1, A.nrow)
    mean = float(lengths.mean()) if A.nrow else 0.0
    std = float(lengths.std()) if A.nrow > 1 else 0.0
    return {"M": A.nrow, "K": A.ncol, "nnz": A.nnz, "mean": mean, "cv": std / mean if mean > 0 else 0.0,
            "max": int(lengths.max()) if A.nrow else 0,
            "frac_long": float((lengths > 32).sum()) / M}


# bumped whenever the candidate list or the way candidates are timed
# changes, so cached picks made the old way are measured again
CANDIDATES_REV = 4


def signature(A: api.CsrMatrix, N: int, f: Optional[dict] = None) -> str:
    f = f or features(A)
    lg = lambda x: int(round(math.log2(max(1, x))))
    cvb = 0 if f["cv"] < 0.5 else 1 if f["cv"] < 2 else 2 if f["cv"] < 8 else 3
    return f"M{lg(f['M'])}_nnz{lg(f['nnz'])}_mean{lg(f['mean'] + 1)}_max{lg(f['max'] + 1)}_cv{cvb}_N{N}_{A.dtype}_c{CANDIDATES_REV}"


def candidates(N: int, dtype: torch.dtype = torch.float32) -> list[tuple[str, dict]]:
    """Strategy / knob candidates (README best static tuples, params.md grids,
    and longer ebsr chunks, which suit the carry design).  16-bit storage also
    tries 8-element vectors (16 bytes per lane, half the lanes per B row)."""
    c: list[tuple[str, dict]] = []
    for gf, denom in ((5, 8), (5, 16), (4, 4)):
        c.append(("ebpr", dict(group_factor=gf, tile_factor=5, block_denom=denom)))
    for gf, tf, denom in ((3, 3, 2), (2, 2, 1), (4, 4, 2)):
        c.append(("rbpr", dict(group_factor=gf, tile_factor=tf, block_denom=denom)))
    vecs = (8, 4) if dtype in (torch.bfloat16, torch.float16) else (4,)
    for vec in vecs:
        lanes_gf = max(0, min(5, int(math.log2(max(1, N // vec)))))
        for gf in sorted({lanes_gf, max(0, lanes_gf - 1)}):
            for tnz in (2, 4, 8, 16, 32, 64):
                for tpb in (128, 256, 512):
                    c.append(("ebsr", dict(group_factor=gf, coarsen_factor=vec, thread_nz=tnz, block_denom=1,
                                           thread_per_block=tpb)))
    # one lane per group (the narrow walk) holding eight elements of a row
    # each: the fastest layout at N = 8 (the group walk wins from N = 16 up)
    if 8 <= N <= 16:
        for tnz in (32, 64):
            for tpb in (128, 256, 512):
                c.append(("ebsr", dict(group_factor=0, coarsen_factor=8, thread_nz=tnz, block_denom=1,
                                       thread_per_block=tpb)))
    # small blocks spread a small matrix's rows over more SMs
    for cf, tf in ((4, 5), (4, 6), (2, 5), (2, 6)):
        for tpb in (128, 256):
            c.append(("rbsr", dict(coarsen_factor=cf, tile_factor=tf, thread_per_block=tpb)))
    return c


def heuristic(f: dict, N: int, dtype: torch.dtype = torch.float32) -> tuple[str, dict]:
    """Choice without measuring: element-balanced sequential for skewed rows,
    row-balanced sequential for short regular rows."""
    vec = 8 if dtype in (torch.bfloat16, torch.float16) and N % 8 == 0 else 4
    lanes_gf = max(0, min(5, int(math.log2(max(1, N // vec)))))
    if f["cv"] > 1.0 or f["max"] > 256:
        return "ebsr", dict(group_factor=lanes_gf, coarsen_factor=vec, thread_nz=8, block_denom=1)
    return "rbsr", dict(coarsen_factor=4, tile_factor=max(0, min(7, int(math.log2(max(1, N))))),
                        thread_per_block=128)


def _load_disk() -> dict:
    p = cache_path()
    try:
        return json.loads(p.read_text())
    except (OSError, ValueError):
        return {}


def _store_disk(key: str, val: dict) -> None:
    p = cache_path()
    try:
        p.parent.mkdir(parents=True, exist_ok=True)
        d = _load_disk()
        d[key] = val
        tmp = p.with_suffix(".tmp")
        tmp.write_text(json.dumps(d, indent=1, sort_keys=True))
        os.replace(tmp, p)
    except OSError:
        pass


def time_candidate(A: api.CsrMatrix, B: torch.Tensor, strategy: str, knobs: SsKnobs, iters: int = 5) -> float:
    """Device ms per call, timed through an SpmmPlan: api.spmm's ~15 us of
    host work per call would hide the kernels of small matrices and make
    every candidate look alike."""
    out = torch.empty((A.nrow, B.shape[1]), dtype=torch.float32, device=B.device)
    plan = api.SpmmPlan(A, int(B.shape[1]), strategy, knobs)
    plan.run(B, out)
    s = torch.cuda.current_stream(B.device)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(s)
    for _ in range(iters):
        plan.run(B, out)
    e1.record(s)
    e1.synchronize()
    return e0.elapsed_time(e1) / iters


def tune(A: api.CsrMatrix, N: int, B: Optional[torch.Tensor] = None, iters: int = 5) -> list[tuple[float, str, dict]]:
    """Times every candidate; returns [(ms, strategy, knob dict)] sorted."""
    if B is None:
        B = torch.rand((A.ncol, N), device=A.indptr.device, dtype=torch.float32).to(A.dtype)
    res = []
    for strategy, kw in candidates(N, A.dtype):
        try:
            k = api.make_knobs(strategy, N, **kw)
            ms = time_candidate(A, B, strategy, k, iters)
        except Exception:  # a tuple the geometry rejects for this shape
            continue
        res.append((ms, strategy, k.as_dict()))
    res.sort(key=lambda r: r[0])
    return res


def best(A: api.CsrMatrix, N: int, B: Optional[torch.Tensor] = None, measure: bool = True) -> tuple[str, SsKnobs]:
    """(strategy, knobs) for A at width N: cached, else measured (or heuristic)."""
    f = features(A)
    key = signature(A, N, f)
    with _LOCK:
        hit = _MEM.get(key) or _load_disk().get(key)
    if hit is None:
        if measure:
            ranked = tune(A, N, B)
            strategy, kw = ranked[0][1], ranked[0][2]
            hit = {"strategy": strategy, "knobs": kw, "ms": ranked[0][0]}
        else:
            strategy, kw = heuristic(f, N, A.dtype)
            hit = {"strategy": strategy, "knobs": api.make_knobs(strategy, N, **kw).as_dict()}
        with _LOCK:
            _MEM[key] = hit
        if measure:
            _store_disk(key, hit)
    k = SsKnobs()
    for name, v in hit["knobs"].items():
        setattr(k, name, int(v))
    return hit["strategy"], k


# ---------------------------------------------------------------------------
# Batched SpMM: per-matrix chunk sizes
# ---------------------------------------------------------------------------
def _lanes_gf(N: int, dtype: torch.dtype) -> int:
    per_vec = 8 if dtype in (torch.bfloat16, torch.float16) else 4
    return max(0, min(5, int(math.log2(max(1, N // per_vec)))))


def batch_knobs(mats, N: int, target_chunk: int = 512) -> list[SsKnobs]:
    """Knobs for each matrix of a batch: the walk geometry is shared (group
    size from N), the chunk (thread_nz * group) is per matrix: at most
    target_chunk nonzeros, and small enough that a matrix splits into at
    least four items, so small and skewed matrices still spread over SMs."""
    out = []
    for A in mats:
        dtype = A.dtype
        gf = _lanes_gf(N, dtype)
        G = 1 << gf
        vec = 8 if dtype in (torch.bfloat16, torch.float16) else 4
        while vec > 1 and N % vec:
            vec //= 2  # one vector per lane: the widest that divides N
        nnz = max(1, A.nnz)
        chunk = min(target_chunk, max(8 * G, 1 << int(math.ceil(math.log2(max(1, nnz // 4))))))
        tnz = max(1, chunk // G)
        out.append(api.make_knobs("ebsr", N, group_factor=gf, coarsen_factor=vec, thread_nz=tnz, block_denom=1,
                                  thread_per_block=256))
    return out


def batch_plan(mats, N: int, target_chunk: int = 512) -> tuple[list[str], list[SsKnobs]]:
    """(strategy, knobs) of each matrix of a batch: the knobs of batch_knobs,
    and the strategy the single-matrix heuristic gives for its row-length
    statistics: "rbsr" (blocks of whole rows) for short regular rows, else
    "ebsr" (element-balanced chunks)."""
    knobs = batch_knobs(mats, N, target_chunk)
    strategies = []
    for A in mats:
        f = features(A) if A.nrow > 0 else {"cv": 0.0, "max": 0}
        strategies.append("rbsr" if A.nnz > 0 and heuristic(f, N, A.dtype)[0] == "rbsr" else "ebsr")
    return strategies, knobs


def tune_batch(mats, Bs, N: int, candidates=(256, 512, 1024, 2048), iters: int = 5):
    """Measures the batched launch for each target chunk; returns
    (best target, {target: ms})."""
    from . import batched
    times = {}
    for t in candidates:
        strategies, knobs = batch_plan(mats, N, t)
        plan = batched.BatchedSpMM(mats, Bs, knobs=knobs, strategies=strategies)
        plan.run()
        s = torch.cuda.current_stream()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(s)
        for _ in range(iters):
            plan.run()
        e1.record(s)
        e1.synchronize()
        times[t] = e0.elapsed_time(e1) / iters
    best = min(times, key=times.get)
    return best, times
