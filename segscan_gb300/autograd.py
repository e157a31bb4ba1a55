"""Differentiable SpMM: a thin torch.autograd.Function over the C ABI.

Forward: C = A @ B with one of the four strategies.  It saves only the
sparse pattern, A's values and B; nothing is recomputed in backward.
Backward:
  both gradients wanted: one fused walk over A^T's rows
  (ss_spmm_backward), each dC row gathered once for dB[k] += a * dC[i]
  and dA.vals[p] = dot(dC[i], B[k]); A^T's pattern is built on the device
  by the stable counting-sort transpose once per pattern and cached;
  one of them, or N above the fused walk's width:
  dA.vals = SDDMM(dC, B)            (ss_sddmm: dot of dC row i with B row k)
  dB      = A^T @ dC                (the forward kernels on A^T)
Values stored in BF16/FP16 get FP32 gradients cast back to their dtype;
dB is computed in FP32 (A^T values widened to FP32) and rounded to B's dtype
by the ebsr walk's own stores (other strategies: a cast after).
This module is the training / test binding only; the library is the C ABI.
"""
from __future__ import annotations

from typing import Optional

import torch

from . import api


class _Pattern:
    """A's pattern plus its lazily built transpose (cached across calls)."""

    def __init__(self, A: api.CsrMatrix):
        self.A = A.with_values(None)
        self._t: Optional[tuple[api.CsrMatrix, torch.Tensor]] = None

    def transposed(self) -> tuple[api.CsrMatrix, torch.Tensor]:
        if self._t is None:
            self._t = api.transpose(self.A)
        return self._t


class SpMMFunction(torch.autograd.Function):
    @staticmethod
    def forward(ctx, values, B, pattern: _Pattern, strategy: str, knobs, bw_strategy: str, bw_knobs):
        A = pattern.A.with_values(values.contiguous())
        C = api.spmm(A, B.contiguous(), strategy, knobs=knobs)
        ctx.save_for_backward(values, B)
        ctx.pattern = pattern
        ctx.bw_strategy = bw_strategy
        ctx.bw_knobs = bw_knobs
        return C

    @staticmethod
    def backward(ctx, dC):
        values, B = ctx.saved_tensors
        pattern: _Pattern = ctx.pattern
        dC = dC.contiguous().float()
        d_values = d_B = None
        if ctx.needs_input_grad[0] and ctx.needs_input_grad[1] and B.shape[1] <= api.spmm_backward_limit(
                int(B.shape[1])):
            # both gradients from one walk over A^T: each dC row gathered once
            AT, perm = pattern.transposed()
            out_dtype = B.dtype if B.dtype != torch.float32 else None
            knobs = ctx.bw_knobs
            d_values, d_B = api.spmm_backward(AT, perm, values.contiguous(), dC, B.contiguous(), out_dtype,
                                              knobs.kahan_threshold if knobs is not None else 0)
            return d_values.to(values.dtype), d_B.to(B.dtype), None, None, None, None, None
        if ctx.needs_input_grad[0]:
            A = pattern.A.with_values(values)
            d_values = api.sddmm(A, dC, B.contiguous()).to(values.dtype)
        if ctx.needs_input_grad[1]:
            AT, perm = pattern.transposed()
            t_vals = api.gather_values(values.float().contiguous(), perm)
            AT_v = AT.with_values(t_vals)
            if ctx.bw_strategy == "ebsr" and B.dtype != torch.float32:
                # the walk rounds its FP32 sums straight into B's 16-bit type
                d_B = api.spmm(AT_v, dC, "ebsr", knobs=ctx.bw_knobs, out_dtype=B.dtype)
            else:
                d_B = api.spmm(AT_v, dC, ctx.bw_strategy, knobs=ctx.bw_knobs).to(B.dtype)
        return d_values, d_B, None, None, None, None, None


def spmm(A: api.CsrMatrix, values: torch.Tensor, B: torch.Tensor, strategy: str = "ebsr", knobs=None,
         bw_strategy: str = "ebsr", pattern: Optional[_Pattern] = None, bw_knobs=None) -> torch.Tensor:
    """C = A(values) @ B, differentiable in values and B (bw_* choose the
    strategy and knobs of the backward's A^T @ dC)."""
    pattern = pattern or _Pattern(A)
    return SpMMFunction.apply(values, B, pattern, strategy, knobs, bw_strategy, bw_knobs)


def pattern(A: api.CsrMatrix) -> _Pattern:
    return _Pattern(A)
