"""segscan_gb300: CSR x dense SpMM and sorted segment reduction for GB300 (sm_103a).

The compute lives in the in-tree CUDA library libsegscan_gb300.so, called
through its C ABI (include/segscan_gb300.h).  This package is the Python
host side: the ctypes binding, a host API that mirrors the reference's
operator names, seeded synthetic workloads, the autotuner, the batched
planner and the autograd binding.
"""
from . import _lib, synth
from ._lib import Dtype, Reduce, SegscanError, SegStrategy, SsCsr, SsKnobs, Status, Strategy

__all__ = ["_lib", "synth", "Dtype", "Reduce", "SegscanError", "SegStrategy", "SsCsr", "SsKnobs",
           "Status", "Strategy", "api", "load"]


def load():
    """Loads libsegscan_gb300.so (raises ImportError when it is not built)."""
    return _lib.load()


def __getattr__(name):
    # torch-dependent modules load lazily so C-ABI checks work without CUDA
    if name in ("api", "autograd", "autotune", "batched", "partition", "mtx"):
        import importlib
        return importlib.import_module(f".{name}", __name__)
    raise AttributeError(name)
