"""Kernel sweep: every strategy / knob tuple and cuSPARSE on a set of
matrices, written as a ratio table (`segscan_gb300.ratios`).

The counterpart of the reference's test mode (test-cg/src/test.py:50-62
profiles test.cu's action list on each matrix under ncu; test.cu:58-140
runs cuSPARSE, the dgSPARSE kernel and the static tuples in turn).  Here
each action is timed with CUDA events: `iters` single launches, each after
an L2 flush (ncu's default cache control also starts every profiled kernel
cold), median taken.  C zeroing is inside the library call, so every
strategy's time includes what its output contract needs.

    python -m segscan_gb300.sweep --datasets powerlaw:1000000 banded:120000 \\
        --N 64 --out table.csv
    python -m segscan_gb300.ratios table.csv --default "ebsr(4,256,4,2,1,16)"

(the default tuples of the width swept are printed as "defaults").

Datasets are synthetic specs or Matrix Market files:
  powerlaw:M[:alpha[:max_len[:seed]]]   Zipf row lengths, uniform columns
  poisson:M[:mean[:seed]]               Poisson row lengths
  banded:M[:per_row[:halfwidth[:seed]]] columns within halfwidth of the diagonal
  <path>.mtx                            pattern of a coordinate file (values 1)
"""
from __future__ import annotations

import argparse
import json
import statistics
import sys
from typing import Callable, Optional, Sequence

import torch

from . import api, autotune, synth
from ._lib import SegscanError
from .ratios import Row, write_csv

# the reference's tuple order per strategy (README.md:160-260, test.cu:58-140)
_TUPLE_FIELDS = {
    "ebpr": ("group_factor", "thread_per_block", "tile_factor", "block_numer", "block_denom"),
    "rbpr": ("group_factor", "thread_per_block", "tile_factor", "block_numer", "block_denom"),
    "ebsr": ("group_factor", "thread_per_block", "coarsen_factor", "thread_nz", "block_numer", "block_denom"),
    "rbsr": ("coarsen_factor", "thread_per_block", "tile_factor", "block_numer", "block_denom"),
}


def label(strategy: str, knobs) -> str:
    """`strategy(k1,k2,...)` in the reference's tuple order."""
    d = knobs.as_dict() if hasattr(knobs, "as_dict") else dict(knobs)
    return f"{strategy}({','.join(str(d[f]) for f in _TUPLE_FIELDS[strategy])})"


def dataset(spec: str) -> synth.Csr:
    """A matrix from a dataset spec (see the module docstring)."""
    if spec.endswith(".mtx"):
        from . import mtx
        return mtx.read(spec)
    kind, *args = spec.split(":")
    num = [float(a) for a in args]
    if kind == "powerlaw":
        M = int(num[0])
        alpha = num[1] if len(num) > 1 else 2.1
        lmax = int(num[2]) if len(num) > 2 else 20000
        seed = int(num[3]) if len(num) > 3 else 1
        return synth.powerlaw(M, M, alpha, 1, lmax, seed=seed)
    if kind == "poisson":
        M = int(num[0])
        return synth.poisson(M, M, num[1] if len(num) > 1 else 16.0, seed=int(num[2]) if len(num) > 2 else 0)
    if kind == "banded":
        M = int(num[0])
        return synth.banded(M, M, int(num[1]) if len(num) > 1 else 20, int(num[2]) if len(num) > 2 else 500,
                            seed=int(num[3]) if len(num) > 3 else 1)
    raise ValueError(f"unknown dataset spec {spec!r}")


class Timer:
    """Median of single-launch CUDA-event times, each after an L2 flush."""

    def __init__(self, device, iters: int = 20, flush_bytes: int = 256 << 20):
        self.iters = iters
        self.flush = torch.empty(flush_bytes // 4, dtype=torch.float32, device=device) if flush_bytes else None
        self.stream = torch.cuda.current_stream(device)

    def __call__(self, fn: Callable[[], None]) -> float:
        """Median time of fn in microseconds."""
        fn()
        self.stream.synchronize()
        times = []
        for _ in range(self.iters):
            if self.flush is not None:
                self.flush.fill_(1.0)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(self.stream)
            fn()
            e1.record(self.stream)
            e1.synchronize()
            times.append(e0.elapsed_time(e1) * 1e3)
        return statistics.median(times)


def library_actions(N: int, dtype=torch.float32, tuples: str = "candidates") -> list[tuple[str, object]]:
    """(strategy, knobs) list: each strategy's default tuple, then (for
    tuples='candidates') the autotuner's candidate tuples."""
    acts = [(s, api.default_knobs(s, N)) for s in ("ebpr", "rbpr", "ebsr", "rbsr")]
    if tuples == "candidates":
        seen = {label(s, k) for s, k in acts}
        for s, kw in autotune.candidates(N, dtype):
            k = api.make_knobs(s, N, **kw)
            if label(s, k) not in seen:
                seen.add(label(s, k))
                acts.append((s, k))
    return acts


def cusparse_fn(A: api.CsrMatrix, B: torch.Tensor) -> Callable[[], None]:
    """cuSPARSE CSR SpMM through torch.sparse.mm on the same matrix."""
    At = torch.sparse_csr_tensor(A.indptr.long(), A.indices.long(), A.values, (A.nrow, A.ncol))
    return lambda: torch.sparse.mm(At, B)


def run(specs: Sequence[str], N: int, device="cuda", iters: int = 20, tuples: str = "candidates",
        extra: Optional[Callable] = None, cusparse: bool = True, log=None) -> list[Row]:
    """The sweep table.  `extra(name, A_host, A_dev, B, timer)` may return
    more rows for a dataset (comparison kernels outside the library)."""
    dev = torch.device(device)
    timer = Timer(dev, iters)
    rows: list[Row] = []
    for spec in specs:
        Ah = dataset(spec)
        A = api.CsrMatrix.from_host(Ah, dev)
        B = torch.from_numpy(synth.dense(Ah.ncol, N, seed=2)).to(dev)
        C = torch.empty((Ah.nrow, N), device=dev)
        if cusparse:
            try:
                rows.append(Row(spec, N, "cusparse", "cusparse", timer(cusparse_fn(A, B))))
            except RuntimeError as exc:  # report and go on: cuSPARSE is a comparison line
                if log:
                    print(f"{spec}: cusparse failed: {exc}", file=log)
        for strategy, k in library_actions(N, tuples=tuples):
            try:
                n = api.spmm_workspace_size(A, N, strategy, k)
            except SegscanError:
                continue  # a tuple the geometry rejects for this width
            ws = torch.empty(n + 256, dtype=torch.uint8, device=dev) if n else None
            t = timer(lambda: api.spmm(A, B, strategy, knobs=k, out=C, workspace=ws))
            rows.append(Row(spec, N, label(strategy, k), "library", t))
        if extra is not None:
            rows.extend(extra(spec, Ah, A, B, timer))
        if log:
            print(f"{spec}: {Ah.nnz} nonzeros, {sum(1 for r in rows if r.dataset == spec)} actions", file=log)
        del A, B, C
        torch.cuda.empty_cache()
    return rows


def main(argv=None):
    ap = argparse.ArgumentParser(description="time every strategy / knob tuple and cuSPARSE on each dataset")
    ap.add_argument("--datasets", nargs="+", required=True)
    ap.add_argument("--N", type=int, nargs="+", default=[64])
    ap.add_argument("--iters", type=int, default=20)
    ap.add_argument("--tuples", choices=("defaults", "candidates"), default="candidates")
    ap.add_argument("--no-cusparse", action="store_true")
    ap.add_argument("--out", required=True, help="CSV table")
    a = ap.parse_args(argv)
    rows = []
    for N in a.N:
        rows += run(a.datasets, N, iters=a.iters, tuples=a.tuples, cusparse=not a.no_cusparse, log=sys.stderr)
    write_csv(a.out, rows)
    defaults = {N: {s: label(s, api.default_knobs(s, N)) for s in _TUPLE_FIELDS} for N in a.N}
    print(json.dumps({"rows": len(rows), "out": a.out, "defaults": defaults}))


if __name__ == "__main__":
    sys.exit(main())
