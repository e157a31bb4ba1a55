"""Rank body for the gloo tests of segscan_gb300.partition (spawned
processes; CPU only)."""
import os

import numpy as np
import torch
import torch.distributed as dist


def matrix(case: str):
    """The sharded matrix: a power-law one, or two rows (with more ranks
    than rows, some ranks hold an empty shard)."""
    from segscan_gb300 import synth
    if case == "two_rows":
        return synth.Csr(2, 5, np.array([0, 3, 5], np.int32), np.array([0, 2, 4, 1, 4], np.int32),
                         np.array([0.5, -1.0, 2.0, 1.5, -0.25], np.float32))
    return synth.powerlaw(3000, 2500, 2.1, 1, 400, seed=17)


def run(rank: int, world: int, port: int, out_dir: str, case: str = "powerlaw") -> None:
    import oracle_lib
    from segscan_gb300 import partition, synth
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        csr = matrix(case)
        N = 8
        B = synth.dense(csr.ncol, N, seed=18)
        dC = synth.dense(csr.nrow, N, seed=19)
        blocks = partition.row_blocks(csr.indptr, world)
        part, (r0, r1) = partition.local_shard(csr, rank, world)
        # forward: this rank's rows with the reference's check-path loop
        C_local = oracle_lib.spmm_check_f32(part.indptr, part.indices, part.values, B)
        C = partition.gather_rows(torch.from_numpy(C_local), blocks)
        # backward: partial dB = A_block^T dC_block in FP64, then one all-reduce
        t_indptr, t_indices, perm = oracle_lib.csr_transpose(part.indptr, part.indices, part.ncol)
        dB_part, _ = oracle_lib.spmm_f64(t_indptr, t_indices, part.values[perm], dC[r0:r1])
        dB = partition.reduce_dB(torch.from_numpy(dB_part))
        if rank == 0:
            np.save(os.path.join(out_dir, "C.npy"), C.numpy())
            np.save(os.path.join(out_dir, "dB.npy"), dB.numpy())
    finally:
        dist.destroy_process_group()


class HostKernels:
    """ShardedSpMM's per-rank compute on the host with the oracle (the CPU
    tests have no CUDA kernels): the reference's check-path SpMM forward,
    FP64 SDDMM and A^T dC backward."""

    def upload(self, csr):
        return csr

    def spmm(self, A, B, **kw):
        import oracle_lib
        return torch.from_numpy(oracle_lib.spmm_check_f32(A.indptr, A.indices, A.values, B))

    def backward(self, A, B, dC):
        import oracle_lib
        t_indptr, t_indices, perm = oracle_lib.csr_transpose(A.indptr, A.indices, A.ncol)
        dB, _ = oracle_lib.spmm_f64(t_indptr, t_indices, A.values[perm], dC)
        dvals, _ = oracle_lib.sddmm_f64(A.indptr, A.indices, dC, B)
        return torch.from_numpy(dvals), torch.from_numpy(dB)


def run_sharded(rank: int, world: int, port: int, out_dir: str, case: str, compact: bool) -> None:
    """The same forward and backward through partition.ShardedSpMM."""
    from segscan_gb300 import partition, synth
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        csr = matrix(case)
        N = 8
        B = synth.dense(csr.ncol, N, seed=18)
        dC = synth.dense(csr.nrow, N, seed=19)
        S = partition.ShardedSpMM(csr, rank, world, HostKernels(), compact_B=compact)
        B_local = S.local_B(B)
        C = S.gather(S.forward(B_local))
        dvals, dB = S.backward(np.ascontiguousarray(dC[S.r0:S.r1]), B_local)
        np.save(os.path.join(out_dir, f"dvals_{rank}.npy"), dvals.numpy())
        if rank == 0:
            np.save(os.path.join(out_dir, "C.npy"), C.numpy())
            np.save(os.path.join(out_dir, "dB.npy"), dB.numpy())
    finally:
        dist.destroy_process_group()
