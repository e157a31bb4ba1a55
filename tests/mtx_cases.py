"""Seeded Matrix Market coordinate files for the loader tests: every field
(real, integer, complex, pattern) and symmetry the reference reads,
duplicates, diagonal entries, comments, CRLF line ends and odd spacing."""
from __future__ import annotations

import numpy as np

CASES = ["general_real", "general_dups", "symmetric", "symmetric_dups", "pattern", "integer_crlf", "complex",
         "skew", "empty_rows", "single"]


def _entries(rng, M, K, nnz, sym=False, diag_frac=0.2):
    rows = rng.integers(1, M + 1, size=nnz)
    cols = rng.integers(1, K + 1, size=nnz)
    if sym:  # lower triangle (j <= i) plus some diagonal
        lo, hi = np.minimum(rows, cols), np.maximum(rows, cols)
        rows, cols = hi, lo
        d = rng.random(nnz) < diag_frac
        cols[d] = rows[d]
    return rows, cols


def text(case: str, seed: int = 0) -> str:
    rng = np.random.default_rng(seed * 101 + CASES.index(case))
    field, symmetry, nl = "real", "general", "\n"
    M, K, nnz = 37, 29, 150
    dups = False
    if case == "general_dups":
        dups = True
    elif case in ("symmetric", "symmetric_dups", "skew"):
        symmetry = "skew-symmetric" if case == "skew" else "symmetric"
        K = M
        dups = case == "symmetric_dups"
    elif case == "pattern":
        field = "pattern"
    elif case == "integer_crlf":
        field, nl = "integer", "\r\n"
    elif case == "complex":
        field = "complex"
    elif case == "empty_rows":
        M = 60
    elif case == "single":
        M, K, nnz = 1, 1, 1
    rows, cols = _entries(rng, M, K, nnz, sym=symmetry != "general")
    if case == "empty_rows":
        rows = rows % 20 + 1  # rows 21.. stay empty
    if dups:
        k = nnz // 5
        rows[-k:], cols[-k:] = rows[:k], cols[:k]
    if case == "skew":
        keep = rows != cols  # no diagonal in a skew-symmetric file
        rows, cols = rows[keep], cols[keep]
    lines = [f"%%MatrixMarket matrix coordinate {field} {symmetry}", "% seeded test file",
             "%   with two comment lines", f"{M} {K} {rows.size}"]
    for i, (r, c) in enumerate(zip(rows, cols)):
        sep = "  " if i % 7 == 0 else " "
        if field == "pattern":
            lines.append(f"{r}{sep}{c}")
        elif field == "integer":
            lines.append(f"{r}{sep}{c} {int(rng.integers(-9, 10))}")
        elif field == "complex":
            lines.append(f"{r} {c} {rng.standard_normal():.6g} {rng.standard_normal():.6g}")
        else:
            lines.append(f"{r} {c}{sep}{rng.standard_normal():.8e}")
    return nl.join(lines) + nl


def write(path, case: str, seed: int = 0) -> None:
    with open(path, "w", newline="") as f:
        f.write(text(case, seed))
