"""Matrix Market input: the reference's loader path, read natively.

`read` parses a coordinate file into a CSR pattern with ss_mtx_read (C++,
segscan_gb300/csrc/mtx.cu), the counterpart of read_mtx_file
(test-cg/include/dataloader/dataloader.hpp:22-107).  `data_loader` is the
counterpart of DataLoader (dataloader.hpp:170-183): the matrix and its
transpose, here with the transpose built on the device (ss_csr_transpose,
the same order as the reference's host counting sort).  Values are ones, as
the reference's SpMatCsrDescr_t fills them (dataloader.hpp:155).
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from .synth import Csr

MODES = {"reference": 0, "full": 1}


def read(path: str, mode: str = "reference") -> Csr:
    """CSR pattern of a Matrix Market coordinate file (values set to 1).
    mode='reference' reproduces the reference's result exactly; 'full'
    keeps every entry of an expanded symmetric file and expands
    skew-symmetric and hermitian files too."""
    lib = _lib.load()
    h = ctypes.c_void_p()
    _lib.check(lib.ss_mtx_read(str(path).encode(), MODES[mode], ctypes.byref(h)))
    try:
        M, K, Z = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        _lib.check(lib.ss_mtx_shape(h, ctypes.byref(M), ctypes.byref(K), ctypes.byref(Z)))
        indptr = np.empty(M.value + 1, dtype=np.int32)
        indices = np.empty(max(Z.value, 1), dtype=np.int32)
        _lib.check(lib.ss_mtx_csr(h, indptr.ctypes.data, indices.ctypes.data))
    finally:
        lib.ss_mtx_free(h)
    return Csr(M.value, K.value, indptr, indices[:Z.value].copy(), np.ones(Z.value, dtype=np.float32))


def data_loader(path: str, device="cuda", mode: str = "reference"):
    """(A, A^T) as device CsrMatrix objects with unit values."""
    from . import api
    A = api.CsrMatrix.from_host(read(path, mode), device)
    AT, _ = api.transpose(A)
    return A, AT
