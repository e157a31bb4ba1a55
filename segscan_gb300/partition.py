"""Row-block sharding of the SpMM path across ranks (one GPU per rank).

SpMM shards by rows with no data-path collective: rank r owns a contiguous
block of A's rows chosen so every rank holds about nnz / world nonzeros (the
element balance the ebpr/ebsr strategies use inside a GPU, applied across
GPUs), reads the whole B (replicated, or only the B rows its block
references) and writes its rows of C.  Gathering C is only needed when one
rank wants all of it.  The backward's dB = A^T dC is a sum over row blocks,
so it needs one all-reduce; dA.vals (SDDMM) stays local.  ShardedSpMM is the
entry point; the functions above it are its pieces.  The reference has no
multi-GPU code; this module is host logic over torch.distributed.
"""
from __future__ import annotations

from typing import Optional

import numpy as np
import torch
import torch.distributed as dist

from .synth import Csr


def row_blocks(indptr: np.ndarray, parts: int) -> list[tuple[int, int]]:
    """Contiguous row ranges [r0, r1), one per part, with about nnz / parts
    nonzeros each (a row is never split; empty parts are possible only when
    there are fewer rows than parts)."""
    indptr = np.asarray(indptr, dtype=np.int64)
    M = indptr.size - 1
    nnz = int(indptr[-1])
    bounds = [0]
    for p in range(1, parts):
        target = nnz * p // parts
        r = int(np.searchsorted(indptr, target, side="left"))
        r = min(max(r, bounds[-1]), M)
        bounds.append(r)
    bounds.append(M)
    return [(bounds[i], bounds[i + 1]) for i in range(parts)]


def shard(csr: Csr, r0: int, r1: int) -> Csr:
    """Rows [r0, r1) of csr with every column (indptr rebased to 0)."""
    p0, p1 = int(csr.indptr[r0]), int(csr.indptr[r1])
    return Csr(r1 - r0, csr.ncol, (csr.indptr[r0:r1 + 1] - p0).astype(np.int32), csr.indices[p0:p1].copy(),
               csr.values[p0:p1].copy())


def local_shard(csr: Csr, rank: int, world: int) -> tuple[Csr, tuple[int, int]]:
    r0, r1 = row_blocks(csr.indptr, world)[rank]
    return shard(csr, r0, r1), (r0, r1)


def gather_rows(C_local: torch.Tensor, blocks: list[tuple[int, int]], group=None) -> torch.Tensor:
    """Concatenates every rank's rows of C (all_gather of padded blocks)."""
    world = len(blocks)
    rows = max(r1 - r0 for r0, r1 in blocks)
    N = C_local.shape[1]
    pad = torch.zeros((rows, N), dtype=C_local.dtype, device=C_local.device)
    pad[:C_local.shape[0]] = C_local
    parts = [torch.empty_like(pad) for _ in range(world)]
    dist.all_gather(parts, pad, group=group)
    return torch.cat([parts[i][:r1 - r0] for i, (r0, r1) in enumerate(blocks)], dim=0)


def reduce_dB(dB_partial: torch.Tensor, group=None) -> torch.Tensor:
    """dB = sum over ranks of (A_block^T dC_block): one all-reduce."""
    dist.all_reduce(dB_partial, op=dist.ReduceOp.SUM, group=group)
    return dB_partial


def referenced_rows(csr: Csr) -> np.ndarray:
    """Distinct columns of A (the B rows a rank must hold when B is not
    replicated)."""
    return np.unique(csr.indices)


def compact_columns(csr: Csr) -> tuple[Csr, np.ndarray]:
    """csr with its columns renumbered to the distinct columns it references
    (ncol = their count), and those columns: the B rows a rank holds when B
    is not replicated (B_local = B[cols])."""
    cols = referenced_rows(csr)
    idx = np.searchsorted(cols, csr.indices).astype(np.int32)
    return Csr(csr.nrow, int(cols.size), csr.indptr.copy(), idx, csr.values.copy()), cols


class DeviceKernels:
    """The per-rank compute of a ShardedSpMM: this library on the rank's GPU.
    strategy / knobs choose the forward SpMM (None: the autotuner's pick for
    the rank's shard), bw_strategy / bw_knobs the backward's A^T dC."""

    def __init__(self, device, strategy: Optional[str] = None, knobs=None, bw_strategy: str = "ebsr",
                 bw_knobs=None, dtype: torch.dtype = torch.float32):
        self.device = torch.device(device)
        self.strategy, self.knobs = strategy, knobs
        self.bw_strategy, self.bw_knobs = bw_strategy, bw_knobs
        self.dtype = dtype

    def upload(self, csr: Csr):
        from . import api
        return api.CsrMatrix.from_host(csr, self.device, self.dtype)

    def choose(self, A, N: int, B=None):
        from . import autotune
        if self.strategy is None:
            self.strategy, self.knobs = autotune.best(A, N, B)
        return self.strategy, self.knobs

    def workspace(self, A, N: int):
        """A reusable workspace for spmm(A, ., out=., workspace=.)."""
        from . import api
        self.choose(A, N)
        n = api.spmm_workspace_size(A, N, self.strategy, self.knobs)
        return torch.empty(n + 256, dtype=torch.uint8, device=self.device) if n else None

    def spmm(self, A, B: torch.Tensor, out: Optional[torch.Tensor] = None, workspace=None, stream=None):
        from . import api
        self.choose(A, int(B.shape[1]), B)
        return api.spmm(A, B, self.strategy, knobs=self.knobs, out=out, workspace=workspace, stream=stream)

    def backward(self, A, B: torch.Tensor, dC: torch.Tensor) -> tuple[torch.Tensor, torch.Tensor]:
        """(dA.values, A^T dC) for the rank's block: SDDMM and the forward
        kernels on the device-built transpose."""
        from . import api
        dvals = api.sddmm(A, dC, B)
        AT, perm = api.transpose(A)
        AT_v = AT.with_values(api.gather_values(A.values.float().contiguous(), perm))
        return dvals, api.spmm(AT_v, dC, self.bw_strategy, knobs=self.bw_knobs)


class ShardedSpMM:
    """C = A @ B with A's rows sharded over the ranks of a process group.

    Rank r holds its nnz-balanced row block (row_blocks) on its device and
    computes its rows of C with no collective.  With compact_B the block's
    columns are renumbered to the distinct columns it references and the rank
    needs only those rows of B (local_B); otherwise B is replicated.  gather
    all-gathers C when one rank wants all of it; backward returns the block's
    dA.values (local) and dB = A^T dC, summed over the ranks by one
    all-reduce.  `kernels` does the per-rank compute (DeviceKernels: this
    library on the rank's GPU)."""

    def __init__(self, csr: Csr, rank: int, world: int, kernels, compact_B: bool = False, group=None):
        self.rank, self.world, self.group = rank, world, group
        self.ncol = csr.ncol
        self.blocks = row_blocks(csr.indptr, world)
        self.r0, self.r1 = self.blocks[rank]
        part = shard(csr, self.r0, self.r1)
        self.cols = None
        if compact_B:
            part, self.cols = compact_columns(part)
        self.part = part
        self.kernels = kernels
        self.A = kernels.upload(part)

    def local_B(self, B):
        """The rows of B this rank's block needs (all of B when replicated)."""
        if self.cols is None:
            return B
        if isinstance(B, torch.Tensor):
            return B[torch.from_numpy(self.cols.astype(np.int64)).to(B.device)].contiguous()
        return np.ascontiguousarray(B[self.cols])

    def forward(self, B_local, **kw):
        """This rank's rows of C from local_B(B)."""
        return self.kernels.spmm(self.A, B_local, **kw)

    def gather(self, C_local: torch.Tensor) -> torch.Tensor:
        return gather_rows(C_local, self.blocks, self.group)

    def backward(self, dC_local, B_local):
        """(dA.values of this block, dB [ncol, N] summed over all ranks)."""
        dvals, dB_part = self.kernels.backward(self.A, B_local, dC_local)
        dB_part = torch.as_tensor(dB_part)
        if self.cols is not None:  # scatter the referenced rows into a full-size dB
            full = torch.zeros((self.ncol, dB_part.shape[1]), dtype=dB_part.dtype, device=dB_part.device)
            full[torch.from_numpy(self.cols.astype(np.int64)).to(dB_part.device)] = dB_part
            dB_part = full
        return dvals, reduce_dB(dB_part.contiguous(), self.group)


def init_from_env(backend: Optional[str] = None) -> tuple[int, int]:
    """(rank, world) from torchrun's environment; initialises the group once."""
    if not dist.is_initialized():
        dist.init_process_group(backend or ("nccl" if torch.cuda.is_available() else "gloo"))
    return dist.get_rank(), dist.get_world_size()
