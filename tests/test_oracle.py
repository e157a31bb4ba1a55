"""The CPU oracle pinned against the reference's own host code (golden
fixtures made by tests/golden/make_golden.py from zhang677/segScan sources)."""
from pathlib import Path

import numpy as np
import pytest

import oracle_lib

GOLD = Path(__file__).resolve().parent / "golden"


def gold(name):
    return np.load(GOLD / name)


@pytest.mark.parametrize("name", ["spmm_poisson512_n4.npz", "spmm_poisson512_n16.npz", "spmm_edge_n3.npz",
                                  "spmm_ones_kat_n8.npz"])
@pytest.mark.parametrize("threads", [1, 4])
def test_spmm_check_path_bit_exact(name, threads):
    g = gold(name)
    C = oracle_lib.spmm_check_f32(g["indptr"], g["indices"], g["values"], g["B"], threads=threads)
    assert np.array_equal(C.view(np.uint32), g["C"].view(np.uint32))


def test_ones_known_answer():
    g = gold("spmm_ones_kat_n8.npz")
    lengths = np.diff(g["indptr"]).astype(np.float32)
    assert np.array_equal(g["C"], np.repeat(lengths[:, None], 8, axis=1))


def test_spmm_f64_close_to_check_path():
    g = gold("spmm_edge_n3.npz")
    C64, absC = oracle_lib.spmm_f64(g["indptr"], g["indices"], g["values"], g["B"])
    err = np.abs(g["C"].astype(np.float64) - C64)
    assert np.all(err <= 1e-5 * absC + 1e-30)


def test_row_ids_bit_exact():
    g = gold("row_ids_edge.npz")
    rows = oracle_lib.row_ids(g["indptr"], int(g["nnz"]), g["elems"])
    assert np.array_equal(rows, g["rows"])
    # past-the-end elements map to the last row (check.cuh:88-102)
    assert rows[-1] == g["indptr"].size - 2


def test_transpose_bit_exact():
    g = gold("transpose_edge.npz")
    t_indptr, t_indices, perm = oracle_lib.csr_transpose(g["indptr"], g["indices"], int(g["ncol"]))
    assert np.array_equal(t_indptr, g["t_indptr"])
    assert np.array_equal(t_indices, g["t_indices"])
    # perm maps each transposed entry back to its source nonzero
    coo = np.repeat(np.arange(g["indptr"].size - 1), np.diff(g["indptr"]))
    assert np.array_equal(coo[perm], t_indices)
    assert np.array_equal(g["indices"][perm], np.repeat(np.arange(int(g["ncol"])), np.diff(t_indptr)))


def test_segment_sum_bit_exact():
    g = gold("segment_edge_n5.npz")
    dst = oracle_lib.segment_coo_f32(g["src"], g["index"], int(g["dst_len"]))
    assert np.array_equal(dst.view(np.uint32), g["dst"].view(np.uint32))


def test_segment_f64_reductions():
    g = gold("segment_edge_n5.npz")
    src, index, L = g["src"], g["index"], int(g["dst_len"])
    s, _ = oracle_lib.segment_coo_f64(src, index, L, 0)
    mx, _ = oracle_lib.segment_coo_f64(src, index, L, 1)
    mean, _ = oracle_lib.segment_coo_f64(src, index, L, 2)
    counts = np.bincount(index, minlength=L)
    for r in range(L):
        rows = src[index == r].astype(np.float64)
        if counts[r] == 0:
            assert not s[r].any() and not mx[r].any() and not mean[r].any()
        else:
            assert np.allclose(s[r], rows.sum(0), rtol=1e-12, atol=1e-12)
            assert np.array_equal(mx[r], rows.max(0))
            assert np.allclose(mean[r], rows.mean(0), rtol=1e-12, atol=1e-12)


def test_sddmm_f64():
    rng = np.random.default_rng(3)
    g = gold("spmm_edge_n3.npz")
    M = g["indptr"].size - 1
    dC = rng.standard_normal((M, 3)).astype(np.float32)
    out, _ = oracle_lib.sddmm_f64(g["indptr"], g["indices"], dC, g["B"])
    rows = np.repeat(np.arange(M), np.diff(g["indptr"]))
    ref = np.einsum("ij,ij->i", dC[rows].astype(np.float64), g["B"][g["indices"]].astype(np.float64))
    assert np.allclose(out, ref, rtol=1e-12, atol=1e-12)


def test_spmm_f64_threads_same_bits():
    """The row-parallel FP64 product used by the full-size parity tests gives
    the single-thread bits."""
    from segscan_gb300 import synth
    A = synth.powerlaw(50000, 40000, 2.1, 1, 3000, seed=12)
    B = synth.dense(A.ncol, 9, seed=13)
    c1, a1 = oracle_lib.spmm_f64(A.indptr, A.indices, A.values, B)
    c8, a8 = oracle_lib.spmm_f64(A.indptr, A.indices, A.values, B, threads=8)
    assert np.array_equal(c1, c8) and np.array_equal(a1, a8)
