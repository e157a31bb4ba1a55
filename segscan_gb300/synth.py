"""Seeded synthetic CSR matrices and dense operands for the SpMM / segment_coo
workloads.

The reference sweeps SuiteSparse matrices read from Matrix Market files
(test-cg/include/dataloader/dataloader.hpp:22-107) with every value set to 1
(dataloader.hpp:155) and B set to 1 (test-cg/src/test.cu:42).  Those files are
not available, so the workloads here are seeded synthetic matrices with the
row-length distributions the benchmark configurations name:

* ``poisson``  - row length ~ Poisson(mean), columns uniform (4096 x 4096, mean 16)
* ``powerlaw`` - row length ~ Zipf(alpha) clipped to [lmin, lmax], columns uniform
                 (1e6 x 1e6, alpha 2.1, clip [1, 20000])
* ``banded``   - ~per_row columns drawn within +-halfwidth of the diagonal
                 (120000 x 120000, 20 per row, +-500)

Columns within a row are sorted and distinct: they are drawn with replacement
and duplicates inside a row are dropped, so a row can come out slightly
shorter than its drawn length (expected loss < 0.1 % for these configs).
Values and B are U[-1, 1] in FP32.  Draw order from one
``numpy.random.default_rng(seed)``: row lengths, columns, values, then B.
"""
from __future__ import annotations

import dataclasses

import numpy as np


@dataclasses.dataclass
class Csr:
    """Host CSR matrix: int32 indptr[M+1], int32 indices[nnz], float32 values[nnz]."""

    nrow: int
    ncol: int
    indptr: np.ndarray
    indices: np.ndarray
    values: np.ndarray

    @property
    def nnz(self) -> int:
        return int(self.indices.shape[0])

    def row_lengths(self) -> np.ndarray:
        return np.diff(self.indptr)

    def distinct_columns(self) -> int:
        """Number of distinct columns referenced (B rows that must be read at least once)."""
        if self.nnz == 0:
            return 0
        return int(np.count_nonzero(np.bincount(self.indices, minlength=self.ncol)))

    def coo_rows(self) -> np.ndarray:
        return np.repeat(np.arange(self.nrow, dtype=np.int32), self.row_lengths())


def _build(nrow: int, ncol: int, rows: np.ndarray, cols: np.ndarray,
           rng: np.random.Generator) -> Csr:
    key = rows.astype(np.int64) * ncol + cols.astype(np.int64)
    key.sort(kind="stable")
    if key.size:
        keep = np.empty(key.size, dtype=bool)
        keep[0] = True
        np.not_equal(key[1:], key[:-1], out=keep[1:])
        key = key[keep]
    r = (key // ncol).astype(np.int32)
    c = (key % ncol).astype(np.int32)
    counts = np.bincount(r, minlength=nrow).astype(np.int64)
    indptr = np.zeros(nrow + 1, dtype=np.int64)
    np.cumsum(counts, out=indptr[1:])
    if indptr[-1] >= 2**31:
        raise ValueError("nnz exceeds int32 indexing")
    vals = rng.random(c.size, dtype=np.float32) * np.float32(2.0) - np.float32(1.0)
    return Csr(nrow, ncol, indptr.astype(np.int32), c, vals)


def csr_from_lengths(nrow: int, ncol: int, lengths: np.ndarray,
                     rng: np.random.Generator) -> Csr:
    lengths = np.clip(lengths.astype(np.int64), 0, ncol)
    rows = np.repeat(np.arange(nrow, dtype=np.int64), lengths)
    cols = rng.integers(0, ncol, size=rows.size, dtype=np.int64)
    return _build(nrow, ncol, rows, cols, rng)


def poisson(nrow: int = 4096, ncol: int = 4096, mean: float = 16.0, seed: int = 0) -> Csr:
    rng = np.random.default_rng(seed)
    lengths = rng.poisson(mean, size=nrow)
    return csr_from_lengths(nrow, ncol, lengths, rng)


def powerlaw(nrow: int = 1_000_000, ncol: int = 1_000_000, alpha: float = 2.1,
             lmin: int = 1, lmax: int = 20000, seed: int = 1) -> Csr:
    rng = np.random.default_rng(seed)
    lengths = np.clip(rng.zipf(alpha, size=nrow), lmin, lmax)
    return csr_from_lengths(nrow, ncol, lengths, rng)


def banded(nrow: int = 120_000, ncol: int = 120_000, per_row: int = 20,
           halfwidth: int = 500, seed: int = 1) -> Csr:
    rng = np.random.default_rng(seed)
    lengths = np.full(nrow, per_row, dtype=np.int64)
    rows = np.repeat(np.arange(nrow, dtype=np.int64), lengths)
    off = rng.integers(-halfwidth, halfwidth + 1, size=rows.size, dtype=np.int64)
    cols = np.clip(rows + off, 0, ncol - 1)
    return _build(nrow, ncol, rows, cols, rng)


def dense(nrow: int, ncol: int, seed: int, low: float = -1.0, high: float = 1.0) -> np.ndarray:
    """Row-major FP32 U[low, high] matrix."""
    rng = np.random.default_rng(seed)
    out = rng.random((nrow, ncol), dtype=np.float32)
    out *= np.float32(high - low)
    out += np.float32(low)
    return out


def sorted_index(csr: Csr) -> np.ndarray:
    """Sorted segment ids for segment_coo over the same nonzeros: the COO row of each nonzero."""
    return csr.coo_rows()


def batch(count: int = 512, rows_lo: int = 100, rows_hi: int = 50_000,
          alpha: float = 2.3, lmax: int = 2000, seed: int = 3) -> list[Csr]:
    """Independent square matrices: rows log-uniform in [rows_lo, rows_hi],
    row length ~ Zipf(alpha) clipped to [1, lmax], columns uniform per matrix."""
    rng = np.random.default_rng(seed)
    sizes = np.exp(rng.uniform(np.log(rows_lo), np.log(rows_hi), size=count)).astype(np.int64)
    mats = []
    for m in sizes:
        m = int(m)
        lengths = np.clip(rng.zipf(alpha, size=m), 1, min(lmax, m))
        mats.append(csr_from_lengths(m, m, lengths, rng))
    return mats


def spmm_bytes(csr: Csr, N: int, val_bytes: int = 4, b_bytes: int = 4, c_bytes: int = 4,
               distinct: int | None = None) -> int:
    """Algorithmic bytes of one SpMM: nnz*(4+val) + rowptr + U*N*b + M*N*c, where
    U = distinct columns referenced (each needed B row read once)."""
    U = csr.distinct_columns() if distinct is None else distinct
    return (csr.nnz * (4 + val_bytes) + (csr.nrow + 1) * 4 + U * N * b_bytes
            + csr.nrow * N * c_bytes)


def segment_bytes(nnz: int, N: int, dst_len: int, src_bytes: int = 4, dst_bytes: int = 4) -> int:
    """Algorithmic bytes of one segment_coo: nnz*(N*src + 4) + dst_len*N*dst."""
    return nnz * (N * src_bytes + 4) + dst_len * N * dst_bytes
