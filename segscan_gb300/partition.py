"""Row-block sharding of the SpMM path across ranks (one GPU per rank).

SpMM shards by rows with no data-path collective: rank r owns a contiguous
block of A's rows chosen so every rank holds about nnz / world nonzeros (the
element balance the ebpr/ebsr strategies use inside a GPU, applied across
GPUs), reads the whole B (replicated, or only the B rows its block
references) and writes its rows of C.  Gathering C is only needed when one
rank wants all of it.  The backward's dB = A^T dC is a sum over row blocks,
so it needs one all-reduce; dA.vals (SDDMM) stays local.  The reference has
no multi-GPU code; this module is host logic over torch.distributed.
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


def init_from_env(backend: Optional[str] = None) -> tuple[int, int]:
    """(rank, world) from torchrun's environment; initialises the group once."""
    if not dist.is_initialized():
        dist.init_process_group(backend or ("nccl" if torch.cuda.is_available() else "gloo"))
    return dist.get_rank(), dist.get_world_size()
