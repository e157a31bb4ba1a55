"""The C++ host interface (include/segscan_gb300.hpp): a check driver shaped
like the reference's check mode, compiled against the library and run."""
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
SRC = Path(__file__).resolve().parent / "cpp" / "spmm_check.cu"


def build(out: Path) -> None:
    lib_dir = ROOT / "segscan_gb300"
    subprocess.run(["nvcc", "-std=c++17", "-O2", "-gencode", "arch=compute_103a,code=sm_103a",
                    "-I", str(ROOT / "include"), str(SRC), "-o", str(out), "-L", str(lib_dir),
                    "-lsegscan_gb300", f"-Xlinker=-rpath,{lib_dir}"], check=True)


def test_cpp_driver_compiles(tmp_path, lib):
    build(tmp_path / "spmm_check")


@pytest.mark.gpu
def test_cpp_driver_passes(tmp_path, cuda):
    exe = tmp_path / "spmm_check"
    build(exe)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "ALL PASSED" in r.stdout
    assert r.stdout.count("Passed!") >= 39
