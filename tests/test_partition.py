"""Row-block sharding (segscan_gb300.partition): balance and coverage, and a
world-size-2 gloo run (CPU) whose gathered C and all-reduced dB equal the
unsharded results."""
import socket

import numpy as np
import pytest
import torch

import oracle_lib
from segscan_gb300 import partition, synth


def test_row_blocks_cover_and_balance():
    csr = synth.powerlaw(50000, 50000, 2.1, 1, 5000, seed=2)
    L = csr.row_lengths()
    for parts in (1, 2, 3, 8, 17):
        blocks = partition.row_blocks(csr.indptr, parts)
        assert blocks[0][0] == 0 and blocks[-1][1] == csr.nrow
        assert all(b[1] == c[0] for b, c in zip(blocks, blocks[1:]))
        sizes = [int(csr.indptr[r1] - csr.indptr[r0]) for r0, r1 in blocks]
        assert sum(sizes) == csr.nnz
        assert max(sizes) - csr.nnz / parts <= L.max()  # off by less than one row


def test_row_blocks_edge_cases():
    empty = np.zeros(11, np.int32)  # 10 rows, no nonzeros
    assert sum(r1 - r0 for r0, r1 in partition.row_blocks(empty, 3)) == 10
    one_row = np.array([0, 1000], np.int32)
    blocks = partition.row_blocks(one_row, 4)
    assert sum(r1 - r0 for r0, r1 in blocks) == 1
    few = np.array([0, 1, 2], np.int32)
    assert sum(r1 - r0 for r0, r1 in partition.row_blocks(few, 5)) == 2


def test_shards_reassemble_on_cpu():
    csr = synth.poisson(2000, 1500, 6.0, seed=3)
    B = synth.dense(1500, 4, seed=4)
    full = oracle_lib.spmm_check_f32(csr.indptr, csr.indices, csr.values, B)
    parts = [partition.shard(csr, r0, r1) for r0, r1 in partition.row_blocks(csr.indptr, 3)]
    got = np.concatenate([oracle_lib.spmm_check_f32(p.indptr, p.indices, p.values, B) for p in parts])
    assert np.array_equal(got.view(np.uint32), full.view(np.uint32))  # rows are independent: same bits


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


@pytest.mark.parametrize("world, case", [(2, "powerlaw"), (3, "two_rows")])
def test_gloo_forward_and_backward(tmp_path, world, case):
    """Ranks as gloo processes: the gathered C equals the unsharded one bit
    for bit and the all-reduced dB equals the unsharded FP64 product, also
    with more ranks than rows (a rank with an empty shard)."""
    import dist_worker
    torch.multiprocessing.start_processes(dist_worker.run, args=(world, free_port(), str(tmp_path), case),
                                          nprocs=world, join=True, start_method="spawn")
    csr = dist_worker.matrix(case)
    B = synth.dense(csr.ncol, 8, seed=18)
    dC = synth.dense(csr.nrow, 8, seed=19)
    full = oracle_lib.spmm_check_f32(csr.indptr, csr.indices, csr.values, B)
    C = np.load(tmp_path / "C.npy")
    assert np.array_equal(C.view(np.uint32), full.view(np.uint32))
    t_indptr, t_indices, perm = oracle_lib.csr_transpose(csr.indptr, csr.indices, csr.ncol)
    dB_full, dB_abs = oracle_lib.spmm_f64(t_indptr, t_indices, csr.values[perm], dC)
    dB = np.load(tmp_path / "dB.npy")
    assert np.all(np.abs(dB - dB_full) <= 1e-12 * dB_abs + 1e-300)


@pytest.mark.parametrize("world, case", [(2, "powerlaw"), (3, "two_rows")])
@pytest.mark.parametrize("compact", [False, True])
def test_gloo_sharded_entry_point(tmp_path, world, case, compact):
    """The same through partition.ShardedSpMM, with B replicated or only the
    referenced B rows on each rank: C bit for bit, dB and the concatenated
    dA.values within 1e-12 of the unsharded FP64 results."""
    import dist_worker
    torch.multiprocessing.start_processes(dist_worker.run_sharded,
                                          args=(world, free_port(), str(tmp_path), case, compact),
                                          nprocs=world, join=True, start_method="spawn")
    csr = dist_worker.matrix(case)
    B = synth.dense(csr.ncol, 8, seed=18)
    dC = synth.dense(csr.nrow, 8, seed=19)
    full = oracle_lib.spmm_check_f32(csr.indptr, csr.indices, csr.values, B)
    assert np.array_equal(np.load(tmp_path / "C.npy").view(np.uint32), full.view(np.uint32))
    t_indptr, t_indices, perm = oracle_lib.csr_transpose(csr.indptr, csr.indices, csr.ncol)
    dB_full, dB_abs = oracle_lib.spmm_f64(t_indptr, t_indices, csr.values[perm], dC)
    assert np.all(np.abs(np.load(tmp_path / "dB.npy") - dB_full) <= 1e-12 * dB_abs + 1e-300)
    dv_full, dv_abs = oracle_lib.sddmm_f64(csr.indptr, csr.indices, dC, B)
    dv = np.concatenate([np.load(tmp_path / f"dvals_{r}.npy") for r in range(world)])
    assert np.all(np.abs(dv - dv_full) <= 1e-12 * dv_abs + 1e-300)


def test_compact_columns_renumber():
    csr = synth.poisson(300, 5000, 4.0, seed=5)
    part, cols = partition.compact_columns(csr)
    assert np.array_equal(cols[part.indices], csr.indices)
    assert part.ncol == cols.size and np.all(np.diff(cols) > 0)


@pytest.mark.gpu
def test_gpu_sharded_entry_point(cuda):
    """ShardedSpMM on the GPU for every rank of a 4-way split (one process;
    no collective): the stacked rows match FP64 with B replicated and with
    compact B; the backward's dA.values match FP64 SDDMM."""
    from gpu_util import check_close, oracle64
    csr = synth.powerlaw(40000, 40000, 2.1, 1, 5000, seed=23)
    N = 64
    B = synth.dense(csr.ncol, N, seed=24)
    Bd = torch.from_numpy(B).cuda()
    C64, absC = oracle64(csr, B)
    for compact in (False, True):
        parts = []
        for rank in range(4):
            S = partition.ShardedSpMM(csr, rank, 4, partition.DeviceKernels("cuda", "ebsr"), compact_B=compact)
            parts.append(S.forward(S.local_B(Bd)).cpu().numpy())
        check_close(np.concatenate(parts), C64, absC, 1e-5, 1e-5, f"sharded, compact={compact}")


@pytest.mark.gpu
def test_gpu_shards_reassemble(cuda):
    from gpu_util import check_close, dev_csr, oracle64
    from segscan_gb300 import api
    csr = synth.powerlaw(40000, 40000, 2.1, 1, 5000, seed=21)
    N = 64
    B = synth.dense(csr.ncol, N, seed=22)
    Bd = torch.from_numpy(B).cuda()
    C64, absC = oracle64(csr, B)
    for strategy in ("ebsr", "rbsr"):
        full = api.spmm(dev_csr(csr), Bd, strategy).cpu().numpy()
        parts = [api.spmm(dev_csr(partition.shard(csr, r0, r1)), Bd, strategy).cpu().numpy()
                 for r0, r1 in partition.row_blocks(csr.indptr, 4)]
        got = np.concatenate(parts)
        check_close(got, C64, absC, 1e-5, 1e-5, f"{strategy} shards")
        if strategy == "rbsr":  # a row's arithmetic does not depend on the sharding
            assert np.array_equal(got.view(np.uint32), full.view(np.uint32))
