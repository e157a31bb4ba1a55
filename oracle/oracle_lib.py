"""ctypes binding of the CPU oracle (oracle/oracle.c).

Test infrastructure only: the tests, the smoke check and bench.py's CPU
baseline leg use it, as the checker or as the timed CPU baseline; the
product never calls it.  Builds _build/liboracle.so with make when missing.
"""
from __future__ import annotations

import ctypes
import subprocess
from ctypes import POINTER, c_double, c_float, c_int, c_int32, c_int64, c_void_p
from pathlib import Path

import numpy as np

ORACLE_DIR = Path(__file__).resolve().parent
LIB = ORACLE_DIR / "_build" / "liboracle.so"
REF_LIB = ORACLE_DIR / "_ref" / "libsegscan_ref.so"

_lib = None


def build() -> None:
    subprocess.run(["make", "-s", "-C", str(ORACLE_DIR), "oracle"], check=True)


def load():
    global _lib
    if _lib is None:
        if not LIB.exists():
            build()
        _lib = ctypes.CDLL(str(LIB))
        _lib.oracle_row_of_nz.restype = c_int32
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data_as(c_void_p)


def spmm_check_f32(indptr, indices, vals, B, threads: int = 1, out=None):
    """The reference's CPU check path (check.cuh:139-158): C = 0; C += A*B in FP32.
    With `out` the result goes there (zeroed inside, row block per thread)."""
    M = indptr.size - 1
    N = B.shape[1]
    lib = load()
    if out is None:
        C = np.zeros((M, N), dtype=np.float32)
        args = (c_int(M), c_int(N), _p(np.ascontiguousarray(indptr, np.int32)),
                _p(np.ascontiguousarray(indices, np.int32)), _p(np.ascontiguousarray(vals, np.float32)),
                _p(np.ascontiguousarray(B, np.float32)), _p(C))
        if threads > 1:
            lib.oracle_spmm_check_f32_mt(*args, c_int(threads))
        else:
            lib.oracle_spmm_check_f32(*args)
        return C
    assert out.dtype == np.float32 and out.shape == (M, N) and out.flags.c_contiguous
    lib.oracle_spmm_f32_zero_mt(c_int(M), c_int(N), _p(np.ascontiguousarray(indptr, np.int32)),
                                _p(np.ascontiguousarray(indices, np.int32)),
                                _p(np.ascontiguousarray(vals, np.float32)), _p(np.ascontiguousarray(B, np.float32)),
                                _p(out), c_int(threads))
    return out


def spmm_f64(indptr, indices, vals, B, threads: int = 1):
    """(C64, |A||B|) in FP64; vals None means ones.  threads > 1 splits the
    rows over host threads (the same bits: rows are independent)."""
    M = indptr.size - 1
    N = B.shape[1]
    C = np.empty((M, N), dtype=np.float64)
    A = np.empty((M, N), dtype=np.float64)
    args = (c_int(M), c_int(N), _p(np.ascontiguousarray(indptr, np.int32)),
            _p(np.ascontiguousarray(indices, np.int32)),
            None if vals is None else _p(np.ascontiguousarray(vals, np.float32)),
            _p(np.ascontiguousarray(B, np.float32)), _p(C), _p(A))
    if threads > 1:
        load().oracle_spmm_f64_mt(*args, c_int(threads))
    else:
        load().oracle_spmm_f64(*args)
    return C, A


def row_ids(indptr, nnz, elems):
    elems = np.ascontiguousarray(elems, np.int32)
    out = np.empty(elems.size, dtype=np.int32)
    load().oracle_row_ids(_p(np.ascontiguousarray(indptr, np.int32)), c_int32(indptr.size - 1),
                          c_int32(nnz), _p(elems), c_int64(elems.size), _p(out))
    return out


def segment_coo_f32(src, index, dst_len):
    N = src.shape[1]
    dst = np.zeros((dst_len, N), dtype=np.float32)
    load().oracle_segment_coo_f32(_p(np.ascontiguousarray(src, np.float32)),
                                  _p(np.ascontiguousarray(index, np.int32)), c_int(index.size), c_int(N),
                                  _p(dst))
    return dst


def segment_coo_f64(src, index, dst_len, reduce: int):
    N = src.shape[1]
    dst = np.empty((dst_len, N), dtype=np.float64)
    dabs = np.empty((dst_len, N), dtype=np.float64)
    load().oracle_segment_coo_f64(_p(np.ascontiguousarray(src, np.float32)),
                                  _p(np.ascontiguousarray(index, np.int32)), c_int(index.size), c_int(N),
                                  c_int(dst_len), c_int(reduce), _p(dst), _p(dabs))
    return dst, dabs


def csr_transpose(indptr, indices, ncol):
    M = indptr.size - 1
    nnz = indices.size
    t_indptr = np.empty(ncol + 1, dtype=np.int32)
    t_indices = np.empty(nnz, dtype=np.int32)
    perm = np.empty(nnz, dtype=np.int32)
    load().oracle_csr_transpose(c_int(M), c_int(ncol), _p(np.ascontiguousarray(indptr, np.int32)),
                                _p(np.ascontiguousarray(indices, np.int32)), _p(t_indptr), _p(t_indices),
                                _p(perm))
    return t_indptr, t_indices, perm


def sddmm_f64(indptr, indices, dC, B):
    M, N = dC.shape
    out = np.empty(indices.size, dtype=np.float64)
    outabs = np.empty(indices.size, dtype=np.float64)
    load().oracle_sddmm_f64(c_int(M), c_int(N), _p(np.ascontiguousarray(indptr, np.int32)),
                            _p(np.ascontiguousarray(indices, np.int32)), _p(np.ascontiguousarray(dC, np.float32)),
                            _p(np.ascontiguousarray(B, np.float32)), _p(out), _p(outabs))
    return out, outabs
