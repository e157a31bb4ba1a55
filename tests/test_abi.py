"""The C-ABI library loads, exports every symbol include/*.h declares, and
rejects bad arguments on the host (no GPU needed)."""
import ctypes
import re
from pathlib import Path

import pytest

import segscan_gb300
from segscan_gb300 import _lib
from segscan_gb300._lib import SsCsr, SsKnobs, Status

HEADERS = sorted((Path(__file__).resolve().parent.parent / "include").glob("*.h"))


def declared_symbols():
    names = set()
    for h in HEADERS:
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        names |= set(re.findall(r"\b(ss_[a-z0-9_]+)\s*\(", text))
    return names


def test_every_declared_symbol_is_exported(lib):
    names = declared_symbols()
    assert len(names) >= 20
    for n in sorted(names):
        assert hasattr(lib, n), n
    assert names <= set(_lib.symbols())


def test_version_and_status_strings(lib):
    assert lib.ss_version() >= 1
    assert lib.ss_status_string(0) == b"ok"
    assert lib.ss_status_string(Status.UNSUPPORTED_KNOBS) == b"unsupported knob tuple"


@pytest.mark.parametrize("strategy", range(4))
def test_default_knobs(lib, strategy):
    k = SsKnobs()
    assert lib.ss_default_knobs(strategy, 64, ctypes.byref(k)) == 0
    assert k.thread_per_block == 256 and k.block_numer >= 1 and k.block_denom >= 1


def fake_csr(nrow=100, ncol=100, nnz=1000):
    # device pointers are never dereferenced by the size/argument checks
    return SsCsr(nrow, ncol, nnz, 256, 512, 1024, 0)


def test_workspace_size_queries(lib):
    A = fake_csr()
    n = ctypes.c_size_t()
    for strategy in (1, 3):  # row-balanced strategies need no scratch
        assert lib.ss_spmm_workspace_size(strategy, ctypes.byref(A), 64, None, ctypes.byref(n)) == 0
        assert n.value == 0
    for strategy in (0, 2):
        assert lib.ss_spmm_workspace_size(strategy, ctypes.byref(A), 64, None, ctypes.byref(n)) == 0
        assert n.value > 0
    assert lib.ss_segment_coo_workspace_size(1, 1000, 16, None, ctypes.byref(n)) == 0
    assert n.value > 0


@pytest.mark.parametrize("N", [1, 3, 16, 33, 64, 100, 128, 256])
def test_batch_plan_layout_sizes(lib, N):
    """ss_batch_plan_size lays the plan out on the host (the layout checks
    its own vector alignment) for item counts and column tilings of every
    residue; the device buffer grows with the items."""
    vec = 4 if N % 4 == 0 else 2 if N % 2 == 0 else 1  # one vector per lane, as batch_knobs picks
    gf = min(5, max(0, (N // vec).bit_length() - 1))
    sizes = []
    for count in (1, 2, 3, 5, 7, 13):
        mats = (SsCsr * count)(*[SsCsr(50 + 7 * i, 40 + 3 * i, 97 * (i + 1) + i * i, 256, 512, 1024, 0)
                                  for i in range(count)])
        knobs = (SsKnobs * count)()
        for i in range(count):
            assert lib.ss_default_knobs(2, N, ctypes.byref(knobs[i])) == 0
            knobs[i].group_factor, knobs[i].coarsen_factor = gf, vec
            knobs[i].thread_nz, knobs[i].block_denom = 1 + i % 5, 1
        hb, db = ctypes.c_size_t(), ctypes.c_size_t()
        assert lib.ss_batch_plan_size(count, mats, N, knobs, ctypes.byref(hb), ctypes.byref(db)) == 0, \
            lib.ss_last_error()
        assert db.value % 256 == 0 and hb.value > 0
        sizes.append(db.value)
    assert sizes == sorted(sizes)


def test_bad_arguments_rejected_without_launch(lib):
    A = fake_csr()
    n = ctypes.c_size_t()
    assert lib.ss_spmm(0, None, 4, 1, 1, 0, 0, None, None, 0, None) == Status.INVALID_ARG
    bad = SsKnobs(9, 9, 256, 1, 1, 4, 1, 0)
    assert lib.ss_spmm_workspace_size(0, ctypes.byref(A), 64, ctypes.byref(bad), ctypes.byref(n)) == \
        Status.UNSUPPORTED_KNOBS
    assert b"tile_factor" in lib.ss_last_error()
    assert lib.ss_spmm(3, ctypes.byref(A), 64, 4096, 8192, 5, 0, None, None, 0, None) == Status.INVALID_ARG
    # segment: accumulate only for sums
    assert lib.ss_segment_coo(1, 4096, 0, 8192, 10, 4, 10, 4096, 1, 1, None, None, 0, None) == \
        Status.INVALID_ARG
    # workspace too small for an element-balanced strategy
    assert lib.ss_spmm(2, ctypes.byref(A), 64, 4096, 8192, 0, 0, None, 4096, 16, None) in \
        (Status.WORKSPACE, Status.CUDA)


@pytest.mark.parametrize("N", [1, 3, 4, 8, 16, 33, 64, 128, 130])
def test_autotuner_candidates_pass_knob_validation(lib, N):
    """Every tuple the autotuner may time, and its no-measurement pick, is a
    tuple the library accepts (so tuning never spends a trial on a refused
    launch), for FP32 and 16-bit storage at widths of every residue."""
    import torch
    from segscan_gb300 import api, autotune
    n = ctypes.c_size_t()
    features = {"cv": 3.0, "max": 20000}, {"cv": 0.2, "max": 30}
    for code, dtype in ((0, torch.float32), (1, torch.bfloat16), (2, torch.float16)):
        A = SsCsr(1000, 1000, 5000, 256, 512, 1024, code)
        picks = autotune.candidates(N, dtype) + [autotune.heuristic(f, N, dtype) for f in features]
        for strategy, kw in picks:
            k = api.make_knobs(strategy, N, **kw)
            st = lib.ss_spmm_workspace_size(int(api.STRATEGIES[strategy]), ctypes.byref(A), N, ctypes.byref(k),
                                            ctypes.byref(n))
            assert st == Status.OK, (strategy, kw, dtype, lib.ss_last_error())


def test_launch_stream_argument_found_by_position_and_keyword(monkeypatch):
    """The Python calls make their stream argument current while they
    allocate and launch; the wrapper finds it passed by keyword, by
    position, or not at all."""
    import contextlib
    from segscan_gb300 import api
    seen = []
    monkeypatch.setattr(api, "_on", lambda s: (seen.append(s), contextlib.nullcontext())[1])

    @api._allocates_on_launch_stream
    def call(a, b=None, stream=None):
        return a

    assert call(1) == 1 and call(1, 2, "s1") == 1 and call(1, stream="s2") == 1
    assert seen == [None, "s1", "s2"]


C_CALLER = r"""
#include <string.h>
#include "segscan_gb300.h"
int main(void) {
  ss_knobs k;
  if (ss_default_knobs(SS_EBSR, 64, &k) != SS_OK) return 1;
  if (strcmp(ss_status_string(SS_ERR_CAPACITY), "ok") == 0) return 2;
  return ss_version() >= 1 ? 0 : 3;
}
"""


def test_headers_compile_for_plain_c_and_cpp_callers(lib, tmp_path):
    """include/segscan_gb300.h is plain C: a C99 program that includes it
    (pedantic, warnings as errors, no CUDA headers) links against the library
    and runs on a machine without a GPU; the C++ header compiles with the
    host C++ compiler alone."""
    import shutil
    import subprocess
    from segscan_gb300 import _lib
    if shutil.which("gcc") is None or shutil.which("g++") is None:
        pytest.skip("no host C/C++ compiler")
    inc = str(Path(__file__).resolve().parent.parent / "include")
    src, exe = tmp_path / "caller.c", tmp_path / "caller"
    src.write_text(C_CALLER)
    libdir = str(_lib.LIB_PATH.parent)
    subprocess.run(["gcc", "-std=c99", "-Wall", "-Wextra", "-pedantic", "-Werror", "-I", inc, str(src), "-o", str(exe),
                    "-L", libdir, "-lsegscan_gb300", f"-Wl,-rpath,{libdir}"], check=True)
    assert subprocess.run([str(exe)]).returncode == 0
    cpp = tmp_path / "caller.cpp"
    cpp.write_text('#include "segscan_gb300.hpp"\nint main() { return 0; }\n')
    cuda_inc = Path(shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc").resolve().parent.parent / "include"
    subprocess.run(["g++", "-std=c++17", "-Wall", "-Wextra", "-Werror", "-fsyntax-only", "-I", inc, "-I", str(cuda_inc),
                    str(cpp)], check=True)


def test_missing_library_fails_loudly(tmp_path):
    with pytest.raises(ImportError):
        _lib.load(tmp_path / "nope.so")


def test_python_api_refuses_host_tensors_and_bad_shapes(lib):
    """The Python entry points check their arguments before any launch: host
    tensors, mismatched shapes and unknown strategies are refused on a
    machine without a GPU as on one with it."""
    import torch
    from segscan_gb300 import api
    indptr = torch.tensor([0, 1, 2], dtype=torch.int32)
    indices = torch.tensor([0, 1], dtype=torch.int32)
    A = api.CsrMatrix(2, 2, indptr, indices, torch.ones(2))
    with pytest.raises(ValueError, match="CUDA"):
        A.descr()
    with pytest.raises(ValueError, match="nrow \\+ 1"):
        api.CsrMatrix(3, 2, indptr, indices, torch.ones(2)).descr()
    with pytest.raises(ValueError, match="values must hold nnz"):
        api.CsrMatrix(2, 2, indptr, indices, torch.ones(3)).descr()
    with pytest.raises(ValueError, match="differ in length"):
        api.gather_values(torch.ones(2), torch.zeros(3, dtype=torch.int32))
    with pytest.raises(ValueError, match="out must be"):
        api.segment(torch.ones(2, 4), torch.zeros(2, dtype=torch.int32), 3, out=torch.zeros(2, 4))
    with pytest.raises(ValueError, match="B must be"):
        api.spmm(A, torch.ones(3, 4), "ebsr")
    with pytest.raises(ValueError, match="CUDA"):
        api.spmm(A, torch.ones(2, 4), "ebsr")
    with pytest.raises(ValueError, match="src must be"):
        api.segment(torch.ones(3, 4), torch.zeros(2, dtype=torch.int32), 2)
    with pytest.raises(KeyError):
        api.default_knobs("csr_magic", 4)
    with pytest.raises(TypeError, match="unknown knob"):
        api.make_knobs("ebsr", 4, warp_count=2)
