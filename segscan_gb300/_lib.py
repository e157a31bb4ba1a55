"""ctypes binding of the C ABI declared in include/segscan_gb300.h.

Only plain pointers, sizes and the two POD structs cross the boundary.  The
library is the in-tree ``libsegscan_gb300.so``; importing this module fails
loudly if it has not been built (there is no fallback path).
"""
from __future__ import annotations

import ctypes
import enum
from ctypes import POINTER, c_char_p, c_int, c_int32, c_int64, c_size_t, c_void_p
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "libsegscan_gb300.so"


class Status(enum.IntEnum):
    OK = 0
    INVALID_ARG = 1
    UNSUPPORTED_KNOBS = 2
    WORKSPACE = 3
    CUDA = 4
    ALIGNMENT = 5
    BAD_DATA = 6
    TIMEOUT = 7
    CAPACITY = 8


class Dtype(enum.IntEnum):
    F32 = 0
    BF16 = 1
    F16 = 2


class Strategy(enum.IntEnum):
    EBPR = 0
    RBPR = 1
    EBSR = 2
    RBSR = 3


class Reduce(enum.IntEnum):
    SUM = 0
    MAX = 1
    MEAN = 2


class SegStrategy(enum.IntEnum):
    PR = 0
    SR = 1


class SsCsr(ctypes.Structure):
    _fields_ = [("nrow", c_int32), ("ncol", c_int32), ("nnz", c_int32),
                ("indptr", c_void_p), ("indices", c_void_p), ("values", c_void_p),
                ("value_dtype", c_int32)]


class SsKnobs(ctypes.Structure):
    _fields_ = [("group_factor", c_int32), ("tile_factor", c_int32),
                ("thread_per_block", c_int32), ("block_numer", c_int32),
                ("block_denom", c_int32), ("coarsen_factor", c_int32),
                ("thread_nz", c_int32), ("kahan_threshold", c_int32)]

    def as_dict(self) -> dict:
        return {f: int(getattr(self, f)) for f, _ in self._fields_}


class SegscanError(RuntimeError):
    def __init__(self, status: int, message: str):
        self.status = Status(status) if status in Status._value2member_map_ else status
        super().__init__(f"{self.status!s}: {message}")


# Every symbol the header declares, with its signature.
_SIGNATURES = {
    "ss_version": (c_int, []),
    "ss_status_string": (c_char_p, [c_int]),
    "ss_last_error": (c_char_p, []),
    "ss_default_knobs": (c_int, [c_int, c_int, POINTER(SsKnobs)]),
    "ss_device_error": (c_int, [POINTER(c_int), c_int]),
    "ss_selftest_bounded_wait": (c_int, [c_int, c_void_p]),
    "ss_coo_to_csr_workspace_size": (c_int, [c_int, c_int, POINTER(c_size_t)]),
    "ss_coo_to_csr": (c_int, [c_int, c_int, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_size_t,
                              c_void_p]),
    "ss_mtx_read": (c_int, [c_char_p, c_int, POINTER(c_void_p)]),
    "ss_mtx_shape": (c_int, [c_void_p, POINTER(c_int), POINTER(c_int), POINTER(c_int)]),
    "ss_mtx_csr": (c_int, [c_void_p, c_void_p, c_void_p]),
    "ss_mtx_free": (None, [c_void_p]),
    "ss_set_l2_keep_bytes": (c_int, [ctypes.c_longlong]),
    "ss_spmm_workspace_size": (c_int, [c_int, POINTER(SsCsr), c_int, POINTER(SsKnobs), POINTER(c_size_t)]),
    "ss_spmm_ebpr": (c_int, [POINTER(SsCsr), c_int, c_void_p, c_void_p, c_int, c_int, POINTER(SsKnobs),
                             c_void_p, c_size_t, c_void_p]),
    "ss_spmm_rbpr": (c_int, [POINTER(SsCsr), c_int, c_void_p, c_void_p, c_int, c_int, POINTER(SsKnobs),
                             c_void_p, c_size_t, c_void_p]),
    "ss_spmm_ebsr": (c_int, [POINTER(SsCsr), c_int, c_void_p, c_void_p, c_int, c_int, POINTER(SsKnobs),
                             c_void_p, c_size_t, c_void_p]),
    "ss_spmm_rbsr": (c_int, [POINTER(SsCsr), c_int, c_void_p, c_void_p, c_int, c_int, POINTER(SsKnobs),
                             c_void_p, c_size_t, c_void_p]),
    "ss_spmm": (c_int, [c_int, POINTER(SsCsr), c_int, c_void_p, c_void_p, c_int, c_int, POINTER(SsKnobs),
                        c_void_p, c_size_t, c_void_p]),
    "ss_spmm_ebsr_noalloc": (c_int, [POINTER(SsCsr), c_int, c_void_p, c_void_p, c_int, c_int,
                                     POINTER(SsKnobs), c_void_p]),
    "ss_segment_coo_workspace_size": (c_int, [c_int, c_int, c_int, POINTER(SsKnobs), POINTER(c_size_t)]),
    "ss_segment_coo": (c_int, [c_int, c_void_p, c_int, c_void_p, c_int, c_int, c_int, c_void_p, c_int,
                               c_int, POINTER(SsKnobs), c_void_p, c_size_t, c_void_p]),
    "ss_row_ids": (c_int, [c_void_p, c_int, c_int, c_void_p, c_int64, c_void_p, c_void_p]),
    "ss_csr_transpose_workspace_size": (c_int, [POINTER(SsCsr), POINTER(c_size_t)]),
    "ss_csr_transpose": (c_int, [POINTER(SsCsr), c_void_p, c_void_p, c_void_p, c_void_p, c_size_t,
                                 c_void_p]),
    "ss_csr_transpose_values": (c_int, [POINTER(SsCsr), c_void_p, c_void_p, c_void_p, c_void_p, c_void_p,
                                        c_size_t, c_void_p]),
    "ss_gather_values": (c_int, [c_void_p, c_int, c_void_p, c_int, c_void_p, c_void_p]),
    "ss_sddmm": (c_int, [POINTER(SsCsr), c_int, c_void_p, c_void_p, c_void_p, c_void_p]),
    "ss_spmm_backward": (c_int, [POINTER(SsCsr), c_void_p, c_void_p, c_int, c_void_p, c_void_p, c_void_p, c_int,
                                 c_void_p, c_int, c_void_p]),
    "ss_csr_validate": (c_int, [POINTER(SsCsr), c_void_p, c_void_p]),
    "ss_index_validate": (c_int, [c_void_p, c_int, c_int, c_void_p, c_void_p]),
    "ss_batch_plan_size": (c_int, [c_int, POINTER(SsCsr), c_int, POINTER(SsKnobs), POINTER(c_size_t),
                                   POINTER(c_size_t)]),
    "ss_batch_plan": (c_int, [c_int, POINTER(SsCsr), c_int, POINTER(c_void_p), POINTER(c_void_p), c_int,
                              POINTER(SsKnobs), c_void_p, c_size_t, c_void_p, c_size_t, c_void_p]),
    "ss_batch_plan_size_ex": (c_int, [c_int, POINTER(SsCsr), c_int, POINTER(SsKnobs), POINTER(c_int),
                                      POINTER(c_size_t), POINTER(c_size_t)]),
    "ss_batch_plan_ex": (c_int, [c_int, POINTER(SsCsr), c_int, POINTER(c_void_p), POINTER(c_void_p), c_int,
                                 POINTER(SsKnobs), POINTER(c_int), c_void_p, c_size_t, c_void_p, c_size_t,
                                 c_void_p]),
    "ss_spmm_batched": (c_int, [c_void_p, c_void_p, c_void_p]),
}

_lib: ctypes.CDLL | None = None


def load(path: Path | str | None = None) -> ctypes.CDLL:
    """Loads the library once and binds every ABI symbol (raises if any is missing)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise ImportError(
            f"{p} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'` "
            "(there is no CPU fallback)")
    lib = ctypes.CDLL(str(p))
    for name, (res, args) in _SIGNATURES.items():
        fn = getattr(lib, name)  # AttributeError if the symbol is not exported
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib


def symbols() -> list[str]:
    return list(_SIGNATURES)


def check(status: int) -> None:
    if status != Status.OK:
        msg = load().ss_last_error().decode(errors="replace")
        raise SegscanError(status, msg)


def call(name: str, *args) -> None:
    check(getattr(load(), name)(*args))
