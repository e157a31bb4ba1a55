"""ss_spmm_ebsr_noalloc: the ebsr SpMM for callers that cannot allocate device
memory (a host that only holds buffers handed to it by another allocator, or
a loop where cudaMalloc cannot be called), whose scratch is a fixed array
inside the library.  This file is collected last on purpose."""
import ctypes

import numpy as np
import pytest
import torch

from gpu_util import check_close, dev_csr, oracle64
from segscan_gb300 import synth
from segscan_gb300._lib import SsCsr, SsKnobs, Status


def call_noalloc(lib, A, N, B, C, knobs, accumulate=0):
    d = A.descr()
    return lib.ss_spmm_ebsr_noalloc(ctypes.byref(d), N, B.data_ptr(), C.data_ptr(), 0, accumulate,
                                    ctypes.byref(knobs), torch.cuda.current_stream().cuda_stream)


@pytest.mark.gpu
def test_noalloc_matches_workspace_entry_point(cuda, lib):
    """Two calls in a row on different matrices (the second sees the first's
    leftovers in the shared array); each must agree with ss_spmm_ebsr run
    with a caller workspace, at the SpMM tolerance (1e-5 of sum|a*b|)."""
    from segscan_gb300 import api
    N = 64
    for seed in (21, 22):
        csr = synth.powerlaw(30000, 30000, 2.1, 1, 3000, seed=seed)
        B = synth.dense(csr.ncol, N, seed=seed + 100)
        A = dev_csr(csr)
        Bd = torch.from_numpy(B).cuda()
        knobs = api.make_knobs("ebsr", N, group_factor=4, thread_nz=8, block_denom=1)
        ref = api.spmm(A, Bd, "ebsr", knobs=knobs)
        out = torch.full_like(ref, float("nan"))
        st = call_noalloc(lib, A, N, Bd, out, knobs)
        assert st == Status.OK, lib.ss_last_error()
        torch.cuda.synchronize()
        C64, absC = oracle64(csr, B)
        got, want = out.cpu().numpy(), ref.cpu().numpy()
        check_close(got, want.astype(np.float64), absC, 1e-5, None, f"noalloc vs workspace entry, seed {seed}")
        check_close(got, C64, absC, 1e-5, 1e-5, f"noalloc vs FP64, seed {seed}")


# The other paths through the fixed scratch: the narrow walk (one lane per
# group), accumulate mode, and the hypersparse path (output zeroed by a
# memset, then accumulated into).  Each runs twice in a row on different
# matrices, so the second call sees the first call's leftovers.
OTHER_PATHS = {
    "narrow": dict(N=8, knobs=dict(group_factor=0, coarsen_factor=8, thread_nz=64, block_denom=1),
                   rows=30000, hyper=False, accumulate=0),
    "accumulate": dict(N=64, knobs=dict(group_factor=4, thread_nz=8, block_denom=1), rows=30000, hyper=False,
                       accumulate=1),
    "hypersparse": dict(N=32, knobs=dict(group_factor=3, thread_nz=8, block_denom=1), rows=60000, hyper=True,
                        accumulate=0),
}


@pytest.mark.gpu
@pytest.mark.parametrize("path", list(OTHER_PATHS))
def test_noalloc_other_paths_match_workspace_entry_point(cuda, lib, path):
    from segscan_gb300 import api
    cfg = OTHER_PATHS[path]
    N = cfg["N"]
    for seed in (31, 32):
        rows = cfg["rows"]
        if cfg["hyper"]:  # fewer than half as many nonzeros as rows
            lengths = np.zeros(rows, dtype=np.int64)
            rng = np.random.default_rng(seed)
            lengths[rng.choice(rows, rows // 8, replace=False)] = rng.integers(1, 4, size=rows // 8)
            csr = synth.csr_from_lengths(rows, rows, lengths, rng)
            assert 2 * csr.nnz < rows
        else:
            csr = synth.powerlaw(rows, rows, 2.1, 1, 3000, seed=seed)
        B = synth.dense(csr.ncol, N, seed=seed + 100)
        A = dev_csr(csr)
        Bd = torch.from_numpy(B).cuda()
        knobs = api.make_knobs("ebsr", N, **cfg["knobs"])
        start = torch.from_numpy(synth.dense(csr.nrow, N, seed=seed + 200)).cuda()
        ref = start.clone() if cfg["accumulate"] else None
        ref = api.spmm(A, Bd, "ebsr", knobs=knobs, out=ref, accumulate=bool(cfg["accumulate"]))
        out = start.clone() if cfg["accumulate"] else torch.full_like(ref, float("nan"))
        st = call_noalloc(lib, A, N, Bd, out, knobs, cfg["accumulate"])
        assert st == Status.OK, lib.ss_last_error()
        torch.cuda.synchronize()
        C64, absC = oracle64(csr, B)
        if cfg["accumulate"]:
            C64 = C64 + start.cpu().numpy().astype(np.float64)
            absC = absC + np.abs(start.cpu().numpy().astype(np.float64))
        got, want = out.cpu().numpy(), ref.cpu().numpy()
        check_close(got, want.astype(np.float64), absC, 1e-5, None, f"{path}: noalloc vs workspace, seed {seed}")
        check_close(got, C64, absC, 1e-5, 1e-5, f"{path}: noalloc vs FP64, seed {seed}")


def test_noalloc_rejects_oversize_scratch(lib):
    """A call whose scratch would exceed the fixed array is refused before any
    device work (the pointers here are never dereferenced)."""
    big = SsCsr(4_000_000, 4_000_000, 400_000_000, 256, 512, 1024, 0)
    knobs = SsKnobs(0, 0, 256, 1, 1, 4, 1, 0)
    # one-lane groups: at least 1024 chunks (one wave's share each, 1024
    # groups per SM on any SM count) of 4096-wide head and tail partials,
    # 32 KB per chunk: 32 MB of carries or more
    st = lib.ss_spmm_ebsr_noalloc(ctypes.byref(big), 4096, 4096, 8192, 0, 0, ctypes.byref(knobs), None)
    assert st == Status.CAPACITY
    assert b"fixed" in lib.ss_last_error()
