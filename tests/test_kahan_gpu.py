"""Per-row compensated summation (kahan_threshold).

A row of 20,000 nonzeros whose first product is 1.0 and whose other 19,999
products are 2^-27 (below half an ulp of 1.0 in FP32): summed in order
without compensation, every small term after the 1.0 is lost within the
sequential run that holds it, so the row misses the library's parity bar
(|C - C64| <= 1e-5 * sum|a*b|) by a wide margin; with the row above the
threshold, each run is compensated and the row lands within the bar.
Knobs put the 1.0 in a sequential run of 2,500-4,096 terms for every
sequential strategy (ebsr group walk, ebsr narrow walk, rbsr, rbpr slots).
The short rows around it stay within the bar either way."""
import numpy as np
import pytest
import torch

from gpu_util import check_close, dev_csr, oracle64
from segscan_gb300 import synth

pytestmark = pytest.mark.gpu
LONG = 20000
DELTA = 2.0 ** -27
N = 64
CASES = {
    "ebsr": dict(group_factor=4, coarsen_factor=4, thread_nz=256, thread_per_block=256, block_denom=1),
    "ebsr_narrow": dict(group_factor=0, coarsen_factor=8, thread_nz=4096, thread_per_block=256, block_denom=1),
    "rbsr": dict(coarsen_factor=4, tile_factor=6),
    "rbpr": dict(group_factor=3, tile_factor=3, block_denom=2),  # 8 slots: 2,500 terms each
}


def cancelling_matrix():
    lengths = np.array([5, LONG, 7], dtype=np.int64)
    K = LONG + 16
    rng = np.random.default_rng(9)
    indptr = np.concatenate([[0], np.cumsum(lengths)]).astype(np.int32)
    cols = [np.sort(rng.choice(K, 5, replace=False)), np.arange(LONG), np.sort(rng.choice(K, 7, replace=False))]
    indices = np.concatenate(cols).astype(np.int32)
    values = np.ones(indices.size, dtype=np.float32)
    B = np.full((K, N), DELTA, dtype=np.float32)
    B[0, :] = 1.0  # the long row's first product
    return synth.Csr(3, K, indptr, indices, values), B


@pytest.mark.parametrize("name", list(CASES))
def test_long_row_compensated(cuda, name):
    from segscan_gb300 import api
    csr, B = cancelling_matrix()
    strategy = name.split("_")[0]
    A = dev_csr(csr)
    Bd = torch.from_numpy(B).cuda()
    C64, absC = oracle64(csr, B)
    errs = {}
    for thr in (0, 2**31 - 1):  # 0 selects the default threshold (1024); INT32_MAX turns it off
        knobs = api.make_knobs(strategy, N, kahan_threshold=thr, **CASES[name])
        C = api.spmm(A, Bd, strategy, knobs=knobs).cpu().numpy().astype(np.float64)
        errs[thr] = np.abs(C[1] - C64[1]).max()
        # the short rows pass the bar either way
        check_close(C[[0, 2]], C64[[0, 2]], absC[[0, 2]], 1e-5, None, f"{name} short rows, threshold {thr}")
    bar = 1e-5 * absC[1].max()
    assert errs[0] <= bar, f"{name}: compensated long row off by {errs[0]:.3e} > {bar:.3e}"
    assert errs[2**31 - 1] > bar, (f"{name}: the uncompensated long row met the bar ({errs[2**31 - 1]:.3e}), "
                                   "so this case does not show compensation at work")
