import numpy as np

from segscan_gb300 import synth


def check_csr(a):
    assert a.indptr[0] == 0 and a.indptr[-1] == a.nnz
    assert np.all(np.diff(a.indptr) >= 0)
    for r in range(min(a.nrow, 2000)):
        cols = a.indices[a.indptr[r]:a.indptr[r + 1]]
        assert np.all(np.diff(cols) > 0)  # sorted, distinct
    assert a.indices.min(initial=0) >= 0 and a.indices.max(initial=0) < a.ncol


def test_poisson_deterministic():
    a, b = synth.poisson(seed=0), synth.poisson(seed=0)
    assert np.array_equal(a.indices, b.indices) and np.array_equal(a.values, b.values)
    check_csr(a)
    assert abs(a.nnz / a.nrow - 16) < 0.5


def test_powerlaw_small():
    a = synth.powerlaw(20000, 20000, 2.1, 1, 2000, seed=1)
    check_csr(a)
    lengths = a.row_lengths()
    assert lengths.min() >= 1 and lengths.max() <= 2000
    assert (lengths == 1).mean() > 0.5


def test_banded():
    a = synth.banded(2000, 2000, 20, 50, seed=1)
    check_csr(a)
    rows = a.coo_rows()
    assert np.all(np.abs(a.indices - rows) <= 50)


def test_batch_and_bytes():
    mats = synth.batch(8, 100, 1000, seed=3)
    assert len(mats) == 8
    for m in mats:
        check_csr(m)
    a = mats[0]
    assert synth.spmm_bytes(a, 64) == a.nnz * 8 + (a.nrow + 1) * 4 + a.distinct_columns() * 256 + a.nrow * 256
