"""Host API over the C ABI, for Python callers holding torch CUDA tensors.

The reference's operator API is a set of C++ launcher templates
(test-cg/include/spmm/spmm_cg.cuh:176-178, 333-335, 553-555, 664-666;
new-cg/include/segscan/segscan.cuh:150-151, 327-328, 817-818, 868-869,
918-919, 974-975).  The functions named after them here take the same
arguments in the same order (the template knobs become keyword arguments)
and keep their output contract: the three atomic-based strategies and the
segment_coo family ADD into a caller-zeroed output, rbsr overwrites.  The
generic ``spmm`` / ``segment`` calls overwrite by default.

torch supplies device memory and the current stream only; every computation
is a call into libsegscan_gb300.so.  Nothing here falls back to PyTorch.
"""
from __future__ import annotations

import contextlib
import ctypes
import dataclasses
import functools
import inspect
from typing import Optional

import numpy as np
import torch

from . import _lib
from ._lib import Dtype, Reduce, SegStrategy, SsCsr, SsKnobs, Strategy

_TORCH_DTYPE = {Dtype.F32: torch.float32, Dtype.BF16: torch.bfloat16, Dtype.F16: torch.float16}
_DTYPE_OF = {v: k for k, v in _TORCH_DTYPE.items()}

STRATEGIES = {"ebpr": Strategy.EBPR, "rbpr": Strategy.RBPR, "ebsr": Strategy.EBSR, "rbsr": Strategy.RBSR}
SEG_STRATEGIES = {"pr": SegStrategy.PR, "sr": SegStrategy.SR}
REDUCES = {"sum": Reduce.SUM, "max": Reduce.MAX, "mean": Reduce.MEAN}


def dtype_code(t: torch.dtype) -> Dtype:
    try:
        return _DTYPE_OF[t]
    except KeyError:
        raise TypeError(f"unsupported dtype {t}; use float32, bfloat16 or float16") from None


def _ptr(t: Optional[torch.Tensor]) -> Optional[int]:
    return None if t is None else t.data_ptr()


def _stream(stream) -> int:
    if stream is None:
        stream = torch.cuda.current_stream()
    return stream.cuda_stream if hasattr(stream, "cuda_stream") else int(stream)


def _on(stream):
    """Context in which the launch stream is the current stream (nothing to
    do when the caller passed none, so the current stream is the launch
    stream already)."""
    if stream is None:
        return contextlib.nullcontext()
    if not isinstance(stream, torch.cuda.Stream):
        handle = stream.cuda_stream if hasattr(stream, "cuda_stream") else int(stream)
        if handle == torch.cuda.current_stream().cuda_stream:
            return contextlib.nullcontext()
        stream = torch.cuda.ExternalStream(handle)
    return torch.cuda.stream(stream)


def _allocates_on_launch_stream(fn):
    """Runs fn with its ``stream`` argument as the current stream.

    torch's caching allocator ties each block to the stream current when it
    was allocated and, once the block is freed, hands it out again in that
    stream's order only.  A call that allocated its workspace and outputs on
    the current stream but launched on another could otherwise have its
    freed workspace handed out while the kernel still uses it, or write an
    output block that earlier work on the current stream still reads.
    Allocating on the launch stream, as torch's own operators do, closes
    both."""
    pos = list(inspect.signature(fn).parameters).index("stream")

    @functools.wraps(fn)
    def wrapper(*args, **kw):
        stream = kw.get("stream", args[pos] if len(args) > pos else None)
        with _on(stream):
            return fn(*args, **kw)
    return wrapper


def _need_cuda(name: str, t: torch.Tensor, dtype: Optional[torch.dtype] = None) -> None:
    if not t.is_cuda:
        raise ValueError(f"{name} must be a CUDA tensor")
    if not t.is_contiguous():
        raise ValueError(f"{name} must be contiguous")
    if dtype is not None and t.dtype != dtype:
        raise TypeError(f"{name} must be {dtype}, got {t.dtype}")


@dataclasses.dataclass
class CsrMatrix:
    """Device CSR matrix (the reference's SpMatCsrDescr_t, test-cg/include/
    dataloader/dataloader.hpp:146-168).  values=None means all ones."""

    nrow: int
    ncol: int
    indptr: torch.Tensor
    indices: torch.Tensor
    values: Optional[torch.Tensor]

    @property
    def nnz(self) -> int:
        return int(self.indices.numel())

    @property
    def dtype(self) -> torch.dtype:
        return self.values.dtype if self.values is not None else torch.float32

    @classmethod
    def from_host(cls, csr, device="cuda", dtype: torch.dtype = torch.float32, values: bool = True):
        ip = torch.from_numpy(np.ascontiguousarray(csr.indptr, dtype=np.int32)).to(device)
        ix = torch.from_numpy(np.ascontiguousarray(csr.indices, dtype=np.int32)).to(device)
        v = None
        if values:
            v = torch.from_numpy(np.ascontiguousarray(csr.values, dtype=np.float32)).to(device).to(dtype)
        return cls(int(csr.nrow), int(csr.ncol), ip, ix, v)

    def with_values(self, values: Optional[torch.Tensor]) -> "CsrMatrix":
        return CsrMatrix(self.nrow, self.ncol, self.indptr, self.indices, values)

    def descr(self) -> SsCsr:
        # the C ABI sees only pointers and sizes: tensors shorter than the
        # sizes claim would be read past their ends on the device
        if self.indptr.numel() != self.nrow + 1:
            raise ValueError(f"indptr must hold nrow + 1 = {self.nrow + 1} entries, got {self.indptr.numel()}")
        if self.values is not None and self.values.numel() != self.nnz:
            raise ValueError(f"values must hold nnz = {self.nnz} entries (as indices), got {self.values.numel()}")
        _need_cuda("indptr", self.indptr, torch.int32)
        _need_cuda("indices", self.indices, torch.int32)
        if self.values is not None:
            _need_cuda("values", self.values)
        return SsCsr(self.nrow, self.ncol, self.nnz, _ptr(self.indptr), _ptr(self.indices),
                     _ptr(self.values), int(dtype_code(self.dtype)))


def default_knobs(strategy: str, N: int = 64) -> SsKnobs:
    k = SsKnobs()
    _lib.call("ss_default_knobs", int(STRATEGIES[strategy]), N, ctypes.byref(k))
    return k


def make_knobs(strategy: str, N: int = 64, **kw) -> SsKnobs:
    """Default knobs of a strategy with the given fields replaced."""
    k = default_knobs(strategy, N)
    for name, val in kw.items():
        if val is None:
            continue
        if not hasattr(k, name):
            raise TypeError(f"unknown knob {name}")
        setattr(k, name, int(val))
    return k


def _output(shape, dtype: torch.dtype, device) -> torch.Tensor:
    """A result tensor the library's kernels fill (every allocation of an
    output goes through here; the tests poison it to catch unwritten
    elements)."""
    return torch.empty(shape, dtype=dtype, device=device)


def _workspace(nbytes: int, device) -> Optional[torch.Tensor]:
    if nbytes == 0:
        return None
    return torch.empty(nbytes + 256, dtype=torch.uint8, device=device)


def _aligned(ws: Optional[torch.Tensor]) -> tuple[Optional[int], int]:
    if ws is None:
        return None, 0
    p = ws.data_ptr()
    off = (-p) % 256
    return p + off, ws.numel() - off


def spmm_workspace_size(A: CsrMatrix, N: int, strategy: str, knobs: Optional[SsKnobs] = None) -> int:
    n = ctypes.c_size_t()
    d = A.descr()
    _lib.call("ss_spmm_workspace_size", int(STRATEGIES[strategy]), ctypes.byref(d), N,
              ctypes.byref(knobs) if knobs is not None else None, ctypes.byref(n))
    return int(n.value)


@_allocates_on_launch_stream
def spmm(A: CsrMatrix, B: torch.Tensor, strategy: str = "ebsr", knobs: Optional[SsKnobs] = None,
         out: Optional[torch.Tensor] = None, accumulate: bool = False,
         out_dtype: Optional[torch.dtype] = None, workspace: Optional[torch.Tensor] = None,
         stream=None) -> torch.Tensor:
    """C = A @ B (or C += A @ B with accumulate=True) with one of the four strategies."""
    if B.dim() != 2 or B.shape[0] != A.ncol:
        raise ValueError(f"B must be [{A.ncol}, N], got {tuple(B.shape)}")
    _need_cuda("B", B, A.dtype)
    N = int(B.shape[1])
    cdt = out_dtype or (out.dtype if out is not None else torch.float32)
    if out is None:
        out = _output((A.nrow, N), cdt, B.device)
    _need_cuda("out", out, cdt)
    if tuple(out.shape) != (A.nrow, N):
        raise ValueError(f"out must be [{A.nrow}, {N}]")
    d = A.descr()
    kp = ctypes.byref(knobs) if knobs is not None else None
    if workspace is None:
        workspace = _workspace(spmm_workspace_size(A, N, strategy, knobs), B.device)
    wp, wn = _aligned(workspace)
    _lib.call("ss_spmm", int(STRATEGIES[strategy]), ctypes.byref(d), N, _ptr(B), _ptr(out),
              int(dtype_code(cdt)), int(bool(accumulate)), kp, wp, wn, _stream(stream))
    return out


class _Plan:
    """A bound call: run() validates and makes one C call whose last argument
    is the stream handle; capture() records it into a CUDA graph."""

    _tail: tuple

    def run(self, *tensors):  # pragma: no cover - defined by subclasses
        raise NotImplementedError

    def capture(self, *tensors) -> "torch.cuda.CUDAGraph":
        """Records run(*tensors) into a CUDA graph (replay with .replay())."""
        self.run(*tensors)  # validates the arguments outside the capture
        dev = tensors[-1].device
        s = torch.cuda.Stream(device=dev)
        s.wait_stream(torch.cuda.current_stream(dev))
        g = torch.cuda.CUDAGraph()
        saved = self._tail
        self._tail = saved[:-1] + (s.cuda_stream,)
        try:
            with torch.cuda.graph(g, stream=s):
                self.run(*tensors)
        finally:
            self._tail = saved
        torch.cuda.current_stream(dev).wait_stream(s)
        self.graph = g
        return g


class SpmmPlan(_Plan):
    """One SpMM shape bound once, for launch-bound loops (small matrices
    called many times, as in a serving or training step).

    The descriptor, knobs, workspace and stream are resolved here, so run()
    is one C call (ss_spmm) after a shape and dtype check.  spmm() redoes
    that work on every call: measured on GB300 with a 4096-row matrix, a
    loop of spmm() costs 15 us of host time per call, of run() 3.8 us, and
    of replays of the graph capture() records 2.0 us, against kernels of
    6-12 us.  The plan keeps A's tensors and its workspace alive; the caller
    keeps B and out alive across replays of a captured graph."""

    @_allocates_on_launch_stream
    def __init__(self, A: CsrMatrix, N: int, strategy: str = "ebsr", knobs: Optional[SsKnobs] = None,
                 out_dtype: torch.dtype = torch.float32, accumulate: bool = False, stream=None):
        """strategy="auto" takes the autotuner's strategy and knobs for A at
        width N (measured once per shape signature, then cached)."""
        self.A = A
        self.N = int(N)
        if strategy == "auto":
            from . import autotune
            strategy, knobs = autotune.best(A, self.N)
        self.strategy = strategy
        self.knobs = knobs if knobs is not None else default_knobs(strategy, self.N)
        self.out_dtype = out_dtype
        self.B_dtype = A.dtype
        self._descr = A.descr()
        self.workspace = _workspace(spmm_workspace_size(A, self.N, strategy, self.knobs), A.indptr.device)
        wp, wn = _aligned(self.workspace)
        self._fn = _lib.load().ss_spmm
        self._head = (int(STRATEGIES[strategy]), ctypes.byref(self._descr), self.N)
        self._tail = (int(dtype_code(out_dtype)), int(bool(accumulate)), ctypes.byref(self.knobs), wp, wn,
                      _stream(stream))
        self._bshape = (A.ncol, self.N)
        self._cshape = (A.nrow, self.N)
        self.graph = None

    def run(self, B: torch.Tensor, out: torch.Tensor) -> torch.Tensor:
        """out = A @ B (or += with accumulate) on the plan's stream."""
        if B.shape != self._bshape or out.shape != self._cshape or B.dtype != self.B_dtype \
                or out.dtype != self.out_dtype or not (B.is_cuda and out.is_cuda):
            raise ValueError(f"plan is for B {self._bshape} {self.B_dtype} and out {self._cshape} "
                             f"{self.out_dtype} on the device")
        rc = self._fn(*self._head, B.data_ptr(), out.data_ptr(), *self._tail)
        if rc:
            _lib.check(rc)
        return out


class SegmentPlan(_Plan):
    """segment_coo over one sorted index bound once (a GNN layer's
    aggregation, called every step): the index, sizes, knobs, workspace and
    stream are resolved here, run(src, out) is one C call and capture()
    records it into a CUDA graph, as for SpmmPlan.  The plan keeps the
    index and its workspace alive."""

    @_allocates_on_launch_stream
    def __init__(self, index: torch.Tensor, dst_len: int, N: int, reduce: str = "sum", strategy: str = "sr",
                 src_dtype: torch.dtype = torch.float32, knobs: Optional[SsKnobs] = None, accumulate: bool = False,
                 stream=None):
        _need_cuda("index", index, torch.int32)
        if index.dim() != 1:
            raise ValueError("index must be 1-D")
        self.index = index
        self.nnz, self.N, self.dst_len = int(index.numel()), int(N), int(dst_len)
        self.src_dtype = src_dtype
        self.knobs = knobs
        self.workspace = _workspace(segment_workspace_size(self.nnz, self.N, strategy, knobs), index.device)
        wp, wn = _aligned(self.workspace)
        self._fn = _lib.load().ss_segment_coo
        self._seg = int(SEG_STRATEGIES[strategy])
        self._mid = (int(dtype_code(src_dtype)), index.data_ptr(), self.nnz, self.N, self.dst_len)
        self._tail = (int(REDUCES[reduce]), int(bool(accumulate)), ctypes.byref(knobs) if knobs is not None else None,
                      wp, wn, _stream(stream))
        self._sshape = (self.nnz, self.N)
        self._dshape = (self.dst_len, self.N)
        self.graph = None

    def run(self, src: torch.Tensor, out: torch.Tensor) -> torch.Tensor:
        """out[index[i], :] (op)= src[i, :] on the plan's stream."""
        if src.shape != self._sshape or out.shape != self._dshape or src.dtype != self.src_dtype \
                or out.dtype != torch.float32 or not (src.is_cuda and out.is_cuda):
            raise ValueError(f"plan is for src {self._sshape} {self.src_dtype} and out {self._dshape} float32 "
                             f"on the device")
        rc = self._fn(self._seg, src.data_ptr(), *self._mid, out.data_ptr(), *self._tail)
        if rc:
            _lib.check(rc)
        return out


def segment_workspace_size(nnz: int, N: int, strategy: str = "sr", knobs: Optional[SsKnobs] = None) -> int:
    n = ctypes.c_size_t()
    _lib.call("ss_segment_coo_workspace_size", int(SEG_STRATEGIES[strategy]), nnz, N,
              ctypes.byref(knobs) if knobs is not None else None, ctypes.byref(n))
    return int(n.value)


@_allocates_on_launch_stream
def segment(src: torch.Tensor, index: torch.Tensor, dst_len: int, reduce: str = "sum",
            strategy: str = "sr", knobs: Optional[SsKnobs] = None, out: Optional[torch.Tensor] = None,
            accumulate: bool = False, stream=None, workspace: Optional[torch.Tensor] = None) -> torch.Tensor:
    """dst[index[i], :] (op)= src[i, :] over a sorted index; op in sum / max / mean.
    workspace: a uint8 device tensor of at least segment_workspace_size()
    + 256 bytes, else one is allocated per call."""
    if src.dim() != 2 or index.dim() != 1 or index.shape[0] != src.shape[0]:
        raise ValueError("src must be [nnz, N] and index [nnz]")
    nnz, N = int(src.shape[0]), int(src.shape[1])
    if out is not None and tuple(out.shape) != (int(dst_len), N):
        raise ValueError(f"out must be [{int(dst_len)}, {N}], got {tuple(out.shape)}")
    _need_cuda("src", src)
    _need_cuda("index", index, torch.int32)
    if out is None:
        out = _output((dst_len, N), torch.float32, src.device)
    _need_cuda("out", out, torch.float32)
    ws = workspace if workspace is not None else _workspace(segment_workspace_size(nnz, N, strategy, knobs),
                                                             src.device)
    wp, wn = _aligned(ws)
    _lib.call("ss_segment_coo", int(SEG_STRATEGIES[strategy]), _ptr(src), int(dtype_code(src.dtype)),
              _ptr(index), nnz, N, int(dst_len), _ptr(out), int(REDUCES[reduce]), int(bool(accumulate)),
              ctypes.byref(knobs) if knobs is not None else None, wp, wn, _stream(stream))
    return out


@_allocates_on_launch_stream
def row_ids(indptr: torch.Tensor, nnz: int, elems: Optional[torch.Tensor] = None, stream=None) -> torch.Tensor:
    """Row of each nonzero (binary_search_segment_number, check.cuh:88-102)."""
    _need_cuda("indptr", indptr, torch.int32)
    M = int(indptr.numel()) - 1
    count = nnz if elems is None else int(elems.numel())
    rows = _output(count, torch.int32, indptr.device)
    if elems is not None:
        _need_cuda("elems", elems, torch.int32)
    _lib.call("ss_row_ids", _ptr(indptr), M, nnz, _ptr(elems), count, _ptr(rows), _stream(stream))
    return rows


@_allocates_on_launch_stream
def validate(A: CsrMatrix, stream=None) -> int:
    """0 when A is well formed, else the flag bits of ss_csr_validate (synchronises)."""
    flag = torch.zeros(1, dtype=torch.int32, device=A.indptr.device)
    d = A.descr()
    _lib.call("ss_csr_validate", ctypes.byref(d), _ptr(flag), _stream(stream))
    return int(flag.item())


@_allocates_on_launch_stream
def validate_index(index: torch.Tensor, dst_len: int, stream=None) -> int:
    flag = torch.zeros(1, dtype=torch.int32, device=index.device)
    _lib.call("ss_index_validate", _ptr(index), int(index.numel()), int(dst_len), _ptr(flag), _stream(stream))
    return int(flag.item())


# ---------------------------------------------------------------------------
# Reference-named operators (same argument order; knobs as keywords)
# ---------------------------------------------------------------------------
def _ref_spmm(strategy: str, A: CsrMatrix, N: int, B: torch.Tensor, C: torch.Tensor, accumulate: int,
              **kw) -> None:
    if B.shape[1] != N or C.shape[1] != N:
        raise ValueError("N does not match B / C")
    spmm(A, B, strategy, knobs=make_knobs(strategy, N, **kw), out=C, accumulate=bool(accumulate))


def csrspmm_parreduce_nnzbalance_cg(A, N, B, C, *, group_factor, thread_per_block, tile_factor,
                                    block_numer, block_denom):
    """ebpr: C += A*B (spmm_cg.cuh:176-178)."""
    _ref_spmm("ebpr", A, N, B, C, 1, group_factor=group_factor, thread_per_block=thread_per_block,
              tile_factor=tile_factor, block_numer=block_numer, block_denom=block_denom)


def csrspmm_parreduce_rowbalance_cg(A, N, B, C, *, group_factor, thread_per_block, tile_factor,
                                    block_numer, block_denom):
    """rbpr: C += A*B (spmm_cg.cuh:333-335)."""
    _ref_spmm("rbpr", A, N, B, C, 1, group_factor=group_factor, thread_per_block=thread_per_block,
              tile_factor=tile_factor, block_numer=block_numer, block_denom=block_denom)


def csrspmm_rowcaching_nnzbalance_cg(A, N, B, C, *, group_factor, thread_per_block, CoarsenFactor,
                                     ThreadNz, block_numer, block_denom):
    """ebsr: C += A*B (spmm_cg.cuh:553-555)."""
    _ref_spmm("ebsr", A, N, B, C, 1, group_factor=group_factor, thread_per_block=thread_per_block,
              coarsen_factor=CoarsenFactor, thread_nz=ThreadNz, block_numer=block_numer,
              block_denom=block_denom)


def csrspmm_seqreduce_rowbalance_cg(A, N, B, C, *, coarsen_factor, thread_per_block, tile_factor,
                                    block_numer, block_denom):
    """rbsr: C = A*B (spmm_cg.cuh:664-666)."""
    _ref_spmm("rbsr", A, N, B, C, 0, coarsen_factor=coarsen_factor, thread_per_block=thread_per_block,
              tile_factor=tile_factor, block_numer=block_numer, block_denom=block_denom)


def _seg_knobs(strategy: str, **kw) -> SsKnobs:
    k = SsKnobs()
    base = dict(group_factor=5 if strategy == "pr" else 4, tile_factor=5, thread_per_block=256,
                block_numer=1, block_denom=1, coarsen_factor=4, thread_nz=8, kahan_threshold=1024)
    base.update({k_: v for k_, v in kw.items() if v is not None})
    for name, val in base.items():
        setattr(k, name, int(val))
    return k


def _ref_segment(strategy, src, index, nnz, N, dst, **kw) -> None:
    if src.shape != (nnz, N) or dst.shape[1] != N:
        raise ValueError("shape mismatch")
    segment(src, index, int(dst.shape[0]), "sum", strategy, knobs=_seg_knobs(strategy, **kw), out=dst,
            accumulate=True)


def segment_coo(src, index, nnz, N, dst, *, group_factor, thread_per_block, tile_factor, block_numer,
                block_denom):
    """segscan.cuh:150-151: dst[index[i]] += src[i] (shuffle-scan family)."""
    _ref_segment("pr", src, index, nnz, N, dst, group_factor=group_factor, thread_per_block=thread_per_block,
                 tile_factor=tile_factor, block_numer=block_numer, block_denom=block_denom)


def segment_coo_new(src, index, nnz, N, dst, *, group_factor, thread_per_block, tile_factor, blockDimY):
    """segscan.cuh:327-328.  The reference's 2-D (nnz x column) split maps to
    the shuffle-scan family with one nonzero step per worker."""
    _ref_segment("pr", src, index, nnz, N, dst, group_factor=group_factor, thread_per_block=thread_per_block,
                 tile_factor=tile_factor, block_numer=1, block_denom=max(1, 1 << tile_factor))


def segment_coo_sr(src, index, nnz, N, dst, *, group_factor, thread_per_block, CoarsenFactor, ThreadNz,
                   block_numer, block_denom):
    """segscan.cuh:817-818 (smem-staged sequential)."""
    _ref_segment("sr", src, index, nnz, N, dst, group_factor=group_factor, thread_per_block=thread_per_block,
                 coarsen_factor=CoarsenFactor, thread_nz=ThreadNz, block_numer=block_numer,
                 block_denom=block_denom)


segment_coo_noshmem_sr = segment_coo_sr            # segscan.cuh:868-869
segment_coo_noshmem_lessatom_sr = segment_coo_sr   # segscan.cuh:918-919


def segment_coo_sorted_sr(src, index, nnz, N, dst, *, CoarsenFactor, ThreadNz, DtileSize, DtileNum, BlockDimY):
    """segscan.cuh:974-975: a worker of DtileSize lanes along N reduces a run
    of ThreadNz consecutive elements; DtileNum x BlockDimY workers per block."""
    gf = max(0, min(5, int(DtileSize).bit_length() - 1))
    G = 1 << gf
    tpb = max(G, min(512, G * int(DtileNum) * int(BlockDimY)))
    tpb -= tpb % G
    _ref_segment("sr", src, index, nnz, N, dst, group_factor=gf, thread_per_block=tpb,
                 coarsen_factor=CoarsenFactor, thread_nz=max(1, int(ThreadNz) // G),
                 block_numer=1, block_denom=1)


# ---------------------------------------------------------------------------
# Transpose, value gather, SDDMM (backward pass building blocks)
# ---------------------------------------------------------------------------
@_allocates_on_launch_stream
def transpose(A: CsrMatrix, stream=None) -> tuple[CsrMatrix, torch.Tensor]:
    """(A^T pattern with values gathered, perm): stable counting-sort transpose
    on the device (dataloader.hpp:109-144); perm[q] = source nonzero of entry q.
    The values are gathered in the same pass (ss_csr_transpose_values)."""
    d = A.descr()
    dev = A.indptr.device
    n = ctypes.c_size_t()
    _lib.call("ss_csr_transpose_workspace_size", ctypes.byref(d), ctypes.byref(n))
    ws = _workspace(int(n.value), dev)
    wp, wn = _aligned(ws)
    t_indptr = _output(A.ncol + 1, torch.int32, dev)
    t_indices = _output(A.nnz, torch.int32, dev)
    perm = _output(A.nnz, torch.int32, dev)
    vals = _output(A.values.shape, A.values.dtype, dev) if A.values is not None else None
    _lib.call("ss_csr_transpose_values", ctypes.byref(d), _ptr(t_indptr), _ptr(t_indices), _ptr(perm),
              _ptr(vals), wp, wn, _stream(stream))
    return CsrMatrix(A.ncol, A.nrow, t_indptr, t_indices, vals), perm


@_allocates_on_launch_stream
def coo_to_csr(nrow: int, rows: torch.Tensor, cols: torch.Tensor, ncol: Optional[int] = None,
               values: Optional[torch.Tensor] = None, stream=None) -> tuple[CsrMatrix, torch.Tensor]:
    """(CSR matrix, perm) from COO rows/cols on the device: a stable counting
    sort by row (compressedRow, dataloader.hpp:109-121, for sorted input);
    values, if given, are gathered along."""
    _need_cuda("rows", rows, torch.int32)
    _need_cuda("cols", cols, torch.int32)
    nnz = int(rows.numel())
    if cols.numel() != nnz:
        raise ValueError("rows and cols differ in length")
    dev = rows.device
    n = ctypes.c_size_t()
    _lib.call("ss_coo_to_csr_workspace_size", nrow, nnz, ctypes.byref(n))
    ws = _workspace(int(n.value), dev)  # held until the launches are queued: the
    wp, wn = _aligned(ws)                # allocator must not hand it to the outputs below
    indptr = _output(nrow + 1, torch.int32, dev)
    out_cols = _output(nnz, torch.int32, dev)
    perm = _output(nnz, torch.int32, dev)
    _lib.call("ss_coo_to_csr", nrow, nnz, _ptr(rows), _ptr(cols), _ptr(indptr), _ptr(out_cols), _ptr(perm), wp, wn,
              _stream(stream))
    vals = gather_values(values, perm, stream) if values is not None else None
    K = int(ncol) if ncol is not None else (int(cols.max()) + 1 if nnz else 0)
    return CsrMatrix(nrow, K, indptr, out_cols, vals), perm


@_allocates_on_launch_stream
def gather_values(values: torch.Tensor, perm: torch.Tensor, stream=None) -> torch.Tensor:
    if perm.numel() != values.numel():  # out has values' length and takes one entry per perm entry
        raise ValueError(f"perm ({perm.numel()}) and values ({values.numel()}) differ in length")
    _need_cuda("values", values)
    _need_cuda("perm", perm, torch.int32)
    out = _output(values.shape, values.dtype, values.device)
    _lib.call("ss_gather_values", _ptr(values), int(dtype_code(values.dtype)), _ptr(perm), int(perm.numel()),
              _ptr(out), _stream(stream))
    return out


@_allocates_on_launch_stream
def sddmm(A: CsrMatrix, dC: torch.Tensor, B: torch.Tensor, stream=None) -> torch.Tensor:
    """dvals[p] = dot(dC[i, :], B[k, :]) at every stored nonzero p = (i, k); FP32."""
    _need_cuda("dC", dC, torch.float32)
    _need_cuda("B", B, A.dtype)
    if dC.shape != (A.nrow, B.shape[1]) or B.shape[0] != A.ncol:
        raise ValueError("dC must be [nrow, N] and B [ncol, N]")
    out = _output(A.nnz, torch.float32, dC.device)
    d = A.descr()
    _lib.call("ss_sddmm", ctypes.byref(d), int(B.shape[1]), _ptr(dC), _ptr(B), _ptr(out), _stream(stream))
    return out


def spmm_backward_limit(N: int) -> int:
    """Largest N the fused backward covers at this width's vector size."""
    V = 4
    while V > 1 and N % V:
        V //= 2
    return 64 * V


@_allocates_on_launch_stream
def spmm_backward(AT: CsrMatrix, perm: torch.Tensor, values: Optional[torch.Tensor], dC: torch.Tensor,
                  B: torch.Tensor, out_dtype: Optional[torch.dtype] = None, kahan_threshold: int = 0,
                  stream=None) -> tuple[torch.Tensor, torch.Tensor]:
    """(dvals, dB) of C = A @ B from one walk over A^T's rows (AT, perm from
    transpose(A)): dvals[p] = dot(dC[i, :], B[k, :]) in A's order, FP32, and
    dB = A^T @ dC in out_dtype (FP32 by default, or B's dtype)."""
    _need_cuda("dC", dC, torch.float32)
    _need_cuda("B", B)
    _need_cuda("perm", perm, torch.int32)
    if values is not None:
        _need_cuda("values", values, B.dtype)
        if values.numel() != AT.nnz:
            raise ValueError(f"values ({values.numel()}) and A^T ({AT.nnz}) differ in nonzeros")
    N = int(B.shape[1])
    if dC.shape != (AT.ncol, N) or B.shape[0] != AT.nrow:
        raise ValueError(f"dC must be [{AT.ncol}, N] and B [{AT.nrow}, N]")
    if perm.numel() != AT.nnz:
        raise ValueError(f"perm ({perm.numel()}) and A^T ({AT.nnz}) differ in nonzeros")
    cdt = out_dtype or torch.float32
    dB = _output((AT.nrow, N), cdt, dC.device)
    dvals = _output(AT.nnz, torch.float32, dC.device)
    d = AT.with_values(None).descr()
    d.value_dtype = int(dtype_code(B.dtype))
    _lib.call("ss_spmm_backward", ctypes.byref(d), _ptr(perm), _ptr(values), N, _ptr(dC), _ptr(B), _ptr(dB),
              int(dtype_code(cdt)), _ptr(dvals), int(kahan_threshold), _stream(stream))
    return dvals, dB
