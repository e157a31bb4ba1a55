"""Generates the golden fixtures in this directory from the REFERENCE'S OWN
host code (zhang677/segScan), compiled by `make -C oracle ref` from the
reference sources into oracle/_ref/libsegscan_ref.so:

  util::spmm_reference_host        test-cg/include/util/check.cuh:139-158
  binary_search_segment_number     test-cg/include/util/check.cuh:88-102
  transpose + compressedRow        test-cg/include/dataloader/dataloader.hpp:109-144
  segment_coo_sequencial           new-cg/include/utils/check.cuh:44-52
  read_mtx_file                    test-cg/include/dataloader/dataloader.hpp:22-107

Run it where the reference checkout exists:
    python tests/golden/make_golden.py [--ref /path/to/segScan]
The inputs are seeded synthetic matrices (segscan_gb300.synth); each .npz
holds the inputs and the reference's outputs.
"""
from __future__ import annotations

import argparse
import os
import ctypes
import subprocess
import sys
from ctypes import c_int, c_longlong, c_void_p
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))

from segscan_gb300 import synth  # noqa: E402

REF_LIB = ROOT / "oracle" / "_ref" / "libsegscan_ref.so"


def _p(a):
    return a.ctypes.data_as(c_void_p)


def load_ref(ref_root: str) -> ctypes.CDLL:
    subprocess.run(["make", "-s", "-C", str(ROOT / "oracle"), "ref", f"REF={ref_root}"], check=True)
    return ctypes.CDLL(str(REF_LIB))


def ref_spmm(lib, csr, B):
    M, N = csr.nrow, B.shape[1]
    C = np.zeros((M, N), dtype=np.float32)  # out_ref.fill_zero_h() (test-cg/src/test.cu:44)
    lib.ref_spmm_reference_host(c_int(M), c_int(N), _p(csr.indptr), _p(csr.indices), _p(csr.values),
                                _p(np.ascontiguousarray(B)), _p(C))
    return C


def ref_row_ids(lib, csr, elems):
    out = np.empty(elems.size, dtype=np.int32)
    lib.ref_row_ids(_p(csr.indptr), c_int(csr.nrow), c_int(csr.nnz), _p(elems), c_longlong(elems.size), _p(out))
    return out


def ref_transpose(lib, csr):
    t_indptr = np.empty(csr.ncol + 1, dtype=np.int32)
    t_indices = np.empty(csr.nnz, dtype=np.int32)
    coo = csr.coo_rows()
    lib.ref_transpose(c_int(csr.nrow), c_int(csr.ncol), c_int(csr.nnz), _p(coo), _p(csr.indices),
                      _p(t_indptr), _p(t_indices))
    return t_indptr, t_indices


def ref_segment(lib, src, index, dst_len):
    dst = np.zeros((dst_len, src.shape[1]), dtype=np.float32)
    lib.ref_segment_coo_sequencial(_p(src), _p(index), c_int(index.size), c_int(src.shape[1]), c_int(dst_len),
                                   _p(dst))
    return dst


def edge_matrix(seed: int = 7) -> synth.Csr:
    """Rows with leading, interior and trailing empty rows, many length-1
    rows, and one 1500-nonzero row (longer than the 1024 compensation
    threshold); 300 x 2048."""
    rng = np.random.default_rng(seed)
    M, K = 300, 2048
    lengths = rng.poisson(3.0, size=M)
    lengths[:3] = 0
    lengths[100:105] = 0
    lengths[-4:] = 0
    lengths[150:170] = 1
    lengths[42] = 1500
    return synth.csr_from_lengths(M, K, lengths, rng)


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.environ.get("SEGSCAN_REF"),
                    help="the reference checkout (default: $SEGSCAN_REF)")
    args = ap.parse_args()
    lib = load_ref(args.ref)

    # 1. SpMM on a Poisson(16) matrix (the CPU-runnable configuration's
    #    structure at 512 x 512), N = 16 and N = 4.
    A = synth.poisson(512, 512, 16.0, seed=0)
    for N in (4, 16):
        B = synth.dense(512, N, seed=100 + N)
        np.savez_compressed(HERE / f"spmm_poisson512_n{N}.npz", indptr=A.indptr, indices=A.indices,
                            values=A.values, B=B, C=ref_spmm(lib, A, B), ncol=A.ncol)

    # 2. SpMM on the edge-case matrix, odd N = 3 (residue columns).
    E = edge_matrix()
    B = synth.dense(E.ncol, 3, seed=103)
    np.savez_compressed(HERE / "spmm_edge_n3.npz", indptr=E.indptr, indices=E.indices, values=E.values, B=B,
                        C=ref_spmm(lib, E, B), ncol=E.ncol)

    # 3. The reference's own known-answer test: A and B all ones, so
    #    C[i, :] = row length (dataloader.hpp:155, test.cu:42).
    ones = synth.Csr(A.nrow, A.ncol, A.indptr, A.indices, np.ones(A.nnz, dtype=np.float32))
    B1 = np.ones((A.ncol, 8), dtype=np.float32)
    np.savez_compressed(HERE / "spmm_ones_kat_n8.npz", indptr=A.indptr, indices=A.indices, values=ones.values,
                        B=B1, C=ref_spmm(lib, ones, B1), ncol=A.ncol)

    # 4. Row of every nonzero, past-the-end elements included.
    elems = np.arange(E.nnz + 8, dtype=np.int32)
    np.savez_compressed(HERE / "row_ids_edge.npz", indptr=E.indptr, nnz=E.nnz, elems=elems,
                        rows=ref_row_ids(lib, E, elems))

    # 5. Transposed pattern (stable counting sort).
    t_indptr, t_indices = ref_transpose(lib, E)
    np.savez_compressed(HERE / "transpose_edge.npz", indptr=E.indptr, indices=E.indices, ncol=E.ncol,
                        t_indptr=t_indptr, t_indices=t_indices)

    # 6. segment_coo sum over sorted ids with empty segments inside and at
    #    both ends, N = 5.
    index = E.coo_rows()
    src = synth.dense(E.nnz, 5, seed=105)
    dst_len = E.nrow + 2
    np.savez_compressed(HERE / "segment_edge_n5.npz", index=index, src=src, dst_len=dst_len,
                        dst=ref_segment(lib, src, index, dst_len))
    # 7. Matrix Market files (tests/mtx_cases.py) read by the reference's
    #    loader; the .mtx texts are committed beside the expected CSR.
    sys.path.insert(0, str(HERE.parent))
    import mtx_cases
    expect = {}
    for case in mtx_cases.CASES:
        path = HERE / f"mtx_{case}.mtx"
        mtx_cases.write(path, case)
        M, K, Z = c_int(), c_int(), c_int()
        lib.ref_read_mtx(str(path).encode(), ctypes.byref(M), ctypes.byref(K), ctypes.byref(Z), None, None)
        ip = np.empty(M.value + 1, np.int32)
        ix = np.empty(max(Z.value, 1), np.int32)
        lib.ref_read_mtx(str(path).encode(), ctypes.byref(M), ctypes.byref(K), ctypes.byref(Z), _p(ip), _p(ix))
        expect[f"{case}_shape"] = np.array([M.value, K.value, Z.value], np.int64)
        expect[f"{case}_indptr"] = ip
        expect[f"{case}_indices"] = ix[:Z.value]
    np.savez_compressed(HERE / "mtx_reference.npz", **expect)
    for f in sorted(HERE.glob("*.npz")):
        print(f"{f.name}: {f.stat().st_size} bytes")


if __name__ == "__main__":
    main()
