"""Batched SpMM: many independent CSR matrices in one persistent launch.

The C ABI builds a device plan of (matrix, item) work items
(ss_batch_plan_ex) and runs it in one persistent walk launch, which also
assembles the rows that straddle work items (ss_spmm_batched).  A matrix's
items are element-balanced chunks ("ebsr") or blocks of whole rows
("rbsr").  This module holds the plan, the outputs and an optional CUDA graph
of the step; autotune.batch_plan chooses each matrix's strategy and chunk
size from its row-length statistics.  The reference has no
batched mode; its drivers launch one matrix at a time.
"""
from __future__ import annotations

import ctypes
from typing import Optional, Sequence

import torch

from . import _lib, api
from ._lib import SsKnobs


class BatchedSpMM:
    """C[m] = A[m] @ B[m] for every m, one persistent launch per step."""

    @api._allocates_on_launch_stream
    def __init__(self, mats: Sequence[api.CsrMatrix], Bs: Sequence[torch.Tensor],
                 out_dtype: torch.dtype = torch.float32, knobs: Optional[Sequence[SsKnobs]] = None,
                 stream=None, strategies: Optional[Sequence[str]] = None):
        """strategies: per matrix "ebsr" (element-balanced chunks) or "rbsr"
        (blocks of whole rows); None = all "ebsr"."""
        if len(mats) != len(Bs) or not mats:
            raise ValueError("one B per matrix, at least one matrix")
        N = int(Bs[0].shape[1])
        dev = Bs[0].device
        for A, B in zip(mats, Bs):
            if B.shape != (A.ncol, N):
                raise ValueError("every B must be [ncol, N] with one common N")
            api._need_cuda("B", B, A.dtype)
        self.mats = list(mats)
        self.Bs = list(Bs)
        self.N = N
        self.out = [api._output((A.nrow, N), out_dtype, dev) for A in mats]
        count = len(mats)
        self._descr = (_lib.SsCsr * count)(*[A.descr() for A in mats])
        self._knobs = None
        if knobs is not None:
            self._knobs = (SsKnobs * count)(*knobs)
        self._strategies = None
        if strategies is not None:
            if len(strategies) != count:
                raise ValueError("one strategy per matrix")
            self._strategies = (ctypes.c_int * count)(*[int(api.STRATEGIES[s]) for s in strategies])
        hb, db = ctypes.c_size_t(), ctypes.c_size_t()
        _lib.call("ss_batch_plan_size_ex", count, self._descr, N, self._knobs, self._strategies, ctypes.byref(hb),
                  ctypes.byref(db))
        self._host = ctypes.create_string_buffer(int(hb.value))
        self._dev = torch.empty(int(db.value) + 256, dtype=torch.uint8, device=dev)
        dp = self._dev.data_ptr()
        self._dev_ptr = dp + ((-dp) % 256)
        B_ptrs = (ctypes.c_void_p * count)(*[B.data_ptr() for B in Bs])
        C_ptrs = (ctypes.c_void_p * count)(*[C.data_ptr() for C in self.out])
        _lib.call("ss_batch_plan_ex", count, self._descr, N, B_ptrs, C_ptrs, int(api.dtype_code(out_dtype)),
                  self._knobs, self._strategies, self._host, hb.value, self._dev_ptr, db.value,
                  api._stream(stream))
        self._graph: Optional[torch.cuda.CUDAGraph] = None

    def run(self, stream=None) -> list[torch.Tensor]:
        _lib.call("ss_spmm_batched", self._host, self._dev_ptr, api._stream(stream))
        return self.out

    def capture(self) -> None:
        """Captures one step into a CUDA graph (replayed by replay())."""
        s = torch.cuda.Stream()
        s.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(s):
            self.run(s)  # first call outside capture: kernel attributes, symbol lookups
        torch.cuda.current_stream().wait_stream(s)
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            self.run()
        self._graph = g

    def replay(self) -> list[torch.Tensor]:
        if self._graph is None:
            self.capture()
        self._graph.replay()
        return self.out


def plain_per_matrix(mats: Sequence[api.CsrMatrix], Bs: Sequence[torch.Tensor], outs: Sequence[torch.Tensor],
                     strategy_knobs: Sequence[tuple[str, SsKnobs]], workspaces=None) -> None:
    """The comparison: one ordinary SpMM launch per matrix."""
    for i, (A, B, C) in enumerate(zip(mats, Bs, outs)):
        strategy, k = strategy_knobs[i]
        ws = workspaces[i] if workspaces is not None else None
        api.spmm(A, B, strategy, knobs=k, out=C, workspace=ws)
