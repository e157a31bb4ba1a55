"""Parity at the workload configurations' real sizes, as the reference's
check mode runs it: every kernel instantiation on the whole input against a
CPU product (test-cg/src/test.cu:51-82, checkSpMMsuffix at
test-cg/include/util/check.cuh:62-72), here against the FP64 oracle.

Configurations (seeded synthetic matrices with the stated distributions):
  1. Poisson(16) 4096 x 4096, seed 0, N in {4, 16}, and segment_coo sum over
     its sorted row ids;
  2. (i) power law 1e6 x 1e6, Zipf 2.1 clipped to [1, 20000], seed 1,
     N in {4, 16, 64, 128}; (ii) banded 120k x 120k, 20 per row within
     +-500 of the diagonal, seed 1, N = 64; segment_coo sum / max / mean over
     both matrices' sorted row ids;
  3. both matrices with values and B stored in BF16 and FP16, FP32
     accumulation, N in {64, 128}, B seed 2;
  5. the differentiated layer: power law 2e6 x 2e6, Zipf 2.1 clipped to
     [1, 50000], seed 4, N = 128: the device transpose bit-exact, the fused
     backward's dB = A^T dC and dA.values against FP64.

Bars: FP32 |C - C64| <= 1e-5 * sum|a*b| per element and 1e-5 normwise;
segment max bit-exact; 16-bit storage 2e-2 normwise against FP64 on the FP32
inputs.  Each strategy runs with the reference README's best static tuple
(README.md:168-210) and the autotuner's pick."""
import os

import numpy as np
import pytest
import torch

import oracle_lib
from gpu_util import check_close, dev_csr
from segscan_gb300 import synth

pytestmark = pytest.mark.gpu
THREADS = max(1, os.cpu_count() or 1)
STRATS = ["ebpr", "rbpr", "ebsr", "rbsr"]
README_TUPLES = {
    "ebpr": dict(group_factor=5, tile_factor=5, block_denom=8),                      # (5,256,5,1,8)
    "rbpr": dict(group_factor=3, tile_factor=3, block_denom=2),                      # (3,256,3,1,2)
    "ebsr": dict(group_factor=4, coarsen_factor=4, thread_nz=1, block_denom=16),     # (4,256,4,1,1,16)
    "rbsr": dict(coarsen_factor=4, tile_factor=5),
}
REDUCE = {"sum": 0, "max": 1, "mean": 2}
_MATS = {}


def matrix(name):
    if name not in _MATS:
        if name == "poisson4096":
            _MATS[name] = synth.poisson(4096, 4096, 16.0, seed=0)
        elif name == "powerlaw1e6":
            _MATS[name] = synth.powerlaw(1_000_000, 1_000_000, 2.1, 1, 20000, seed=1)
        else:
            _MATS[name] = synth.banded(120_000, 120_000, 20, 500, seed=1)
    return _MATS[name]


def oracle(csr, B):
    return oracle_lib.spmm_f64(csr.indptr, csr.indices, csr.values, B, threads=THREADS)


def run_all(csr, B, C64, absC, what, dtype=torch.float32, tol=1e-5, normwise=1e-5):
    """Every strategy at its README tuple, then the autotuned pick."""
    from segscan_gb300 import api, autotune
    A = dev_csr(csr, dtype)
    Bd = torch.from_numpy(B).cuda().to(dtype)
    runs = [(s, api.make_knobs(s, B.shape[1], **README_TUPLES[s])) for s in STRATS]
    runs.append(autotune.best(A, B.shape[1], Bd))
    for strategy, knobs in runs:
        C = api.spmm(A, Bd, strategy, knobs=knobs)
        torch.cuda.synchronize()
        got = C.float().cpu().numpy()
        del C
        if dtype == torch.float32:
            check_close(got, C64, absC, tol, normwise, f"{what} {strategy} {knobs.as_dict()}")
        else:
            assert np.isfinite(got).all(), f"{what} {strategy}: non-finite output"
            err = np.linalg.norm(got.astype(np.float64) - C64) / np.linalg.norm(C64)
            assert err <= normwise, f"{what} {strategy}: normwise {err:.3e} > {normwise}"
    del A, Bd
    torch.cuda.empty_cache()


@pytest.mark.parametrize("N", [4, 16])
def test_config1_poisson_spmm(cuda, N):
    csr = matrix("poisson4096")
    B = synth.dense(csr.ncol, N, seed=0)
    C64, absC = oracle(csr, B)
    run_all(csr, B, C64, absC, f"poisson4096 N={N}")


@pytest.mark.parametrize("strategy", ["sr", "pr"])
@pytest.mark.parametrize("N", [4, 16])
def test_config1_poisson_segment_sum(cuda, strategy, N):
    from segscan_gb300 import api
    csr = matrix("poisson4096")
    index = csr.coo_rows()
    src = synth.dense(csr.nnz, N, seed=1)
    out = api.segment(torch.from_numpy(src).cuda(), torch.from_numpy(index).cuda(), csr.nrow, "sum", strategy)
    ref, dabs = oracle_lib.segment_coo_f64(src, index, csr.nrow, 0)
    check_close(out.cpu().numpy(), ref, dabs, 1e-5, 1e-5, f"segment sum {strategy} N={N}")


@pytest.mark.parametrize("N", [4, 16, 64, 128])
def test_config2_powerlaw_spmm(cuda, N):
    csr = matrix("powerlaw1e6")
    B = synth.dense(csr.ncol, N, seed=2)
    C64, absC = oracle(csr, B)
    run_all(csr, B, C64, absC, f"powerlaw1e6 N={N}")


def test_config2_banded_spmm(cuda):
    csr = matrix("banded120k")
    B = synth.dense(csr.ncol, 64, seed=2)
    C64, absC = oracle(csr, B)
    run_all(csr, B, C64, absC, "banded120k N=64")


@pytest.mark.parametrize("name", ["powerlaw1e6", "banded120k"])
@pytest.mark.parametrize("N", [16, 64])
def test_config2_segments(cuda, name, N):
    """segment_coo sum / max / mean over the matrix's sorted row ids, both
    strategy families, src [nnz x N] U[-1, 1]."""
    from segscan_gb300 import api
    csr = matrix(name)
    index = csr.coo_rows()
    src = synth.dense(csr.nnz, N, seed=3)
    src_d = torch.from_numpy(src).cuda()
    idx_d = torch.from_numpy(index).cuda()
    for reduce in ("sum", "max", "mean"):
        ref, dabs = oracle_lib.segment_coo_f64(src, index, csr.nrow, REDUCE[reduce])
        for strategy in ("sr", "pr"):
            out = api.segment(src_d, idx_d, csr.nrow, reduce, strategy)
            torch.cuda.synchronize()
            got = out.cpu().numpy()
            del out
            what = f"{name} segment {reduce} {strategy} N={N}"
            if reduce == "max":
                assert np.array_equal(got.astype(np.float64), ref), what
            else:
                check_close(got, ref, dabs, 1e-5, 1e-5, what)
        del ref, dabs
    del src_d, idx_d
    torch.cuda.empty_cache()


@pytest.mark.parametrize("name", ["powerlaw1e6", "banded120k"])
@pytest.mark.parametrize("dtype", [torch.bfloat16, torch.float16])
@pytest.mark.parametrize("N", [64, 128])
def test_config3_precision(cuda, name, dtype, N):
    """16-bit storage of values and B, FP32 accumulation and C: within 2e-2
    normwise of FP64 on the FP32 inputs."""
    csr = matrix(name)
    B = synth.dense(csr.ncol, N, seed=2)
    C64, _ = oracle(csr, B)
    run_all(csr, B, C64, None, f"{name} {dtype} N={N}", dtype=dtype, normwise=2e-2)


def test_config5_transpose_and_backward(cuda):
    """Config 5 at its size.  The transpose sorts into 1954 column buckets,
    more than the 1024 threads of a partition block; the fused backward
    walks the result."""
    from segscan_gb300 import api
    csr = synth.powerlaw(2_000_000, 2_000_000, 2.1, 1, 50_000, seed=4)
    A = dev_csr(csr)
    AT, perm = api.transpose(A)
    torch.cuda.synchronize()
    t_indptr, t_indices, operm = oracle_lib.csr_transpose(csr.indptr, csr.indices, csr.ncol)
    assert np.array_equal(AT.indptr.cpu().numpy(), t_indptr)
    assert np.array_equal(AT.indices.cpu().numpy(), t_indices)
    assert np.array_equal(perm.cpu().numpy(), operm)
    assert np.array_equal(AT.values.cpu().numpy(), csr.values[operm])
    N = 128
    dC = np.random.default_rng(4).standard_normal((csr.nrow, N), dtype=np.float32)
    B = synth.dense(csr.ncol, N, seed=44)
    dvals, dB = api.spmm_backward(AT, perm, A.values, torch.from_numpy(dC).cuda(), torch.from_numpy(B).cuda())
    torch.cuda.synchronize()
    dB64, absdB = oracle_lib.spmm_f64(t_indptr, t_indices, csr.values[operm], dC, threads=THREADS)
    check_close(dB.cpu().numpy(), dB64, absdB, 1e-5, 1e-5, "config 5 dB = A^T dC")
    del dB64, absdB
    dv64, dvabs = oracle_lib.sddmm_f64(csr.indptr, csr.indices, dC, B)
    check_close(dvals.cpu().numpy(), dv64, dvabs, 1e-5, 1e-5, "config 5 dA.values")
