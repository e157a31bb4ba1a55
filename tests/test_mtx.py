"""Matrix Market input (ss_mtx_read): the reference's loader
(read_mtx_file, test-cg/include/dataloader/dataloader.hpp:22-107) on the
committed seeded files, bit for bit in reference mode; the full mode against
a restatement here; malformed files refused with status codes."""
import ctypes
from pathlib import Path

import numpy as np
import pytest

import mtx_cases
from segscan_gb300 import SegscanError, Status, mtx

GOLD = Path(__file__).resolve().parent / "golden"
REF_LIB = Path(__file__).resolve().parent.parent / "oracle" / "_ref" / "libsegscan_ref.so"


@pytest.mark.parametrize("case", mtx_cases.CASES)
def test_reference_mode_matches_reference_loader(lib, case):
    g = np.load(GOLD / "mtx_reference.npz")
    A = mtx.read(GOLD / f"mtx_{case}.mtx", "reference")
    M, K, Z = g[f"{case}_shape"]
    assert (A.nrow, A.ncol, A.nnz) == (M, K, Z)
    assert np.array_equal(A.indptr, g[f"{case}_indptr"])
    assert np.array_equal(A.indices, g[f"{case}_indices"])
    assert np.all(A.values == 1.0)


def full_restated(text: str):
    """Every entry, mirrored ones added for symmetric, skew-symmetric and
    hermitian files, de-duplicated for those, sorted by (row, column)."""
    lines = [l for l in text.splitlines() if l.strip() and not l.lstrip().startswith("%")]
    banner = text.splitlines()[0].lower().split()
    sym = banner[4] != "general"
    M, K, Z = map(int, lines[0].split())
    pairs = []
    for l in lines[1:1 + Z]:
        i, j = (int(t) - 1 for t in l.split()[:2])
        pairs.append((i, j))
        if sym and i != j:
            pairs.append((j, i))
    pairs = sorted(set(pairs)) if sym else sorted(pairs)
    indptr = np.zeros(M + 1, np.int32)
    for i, _ in pairs:
        indptr[i + 1] += 1
    return M, K, np.cumsum(indptr).astype(np.int32), np.array([j for _, j in pairs], np.int32)


@pytest.mark.parametrize("case", mtx_cases.CASES)
def test_full_mode(lib, case):
    path = GOLD / f"mtx_{case}.mtx"
    M, K, indptr, indices = full_restated(path.read_text())
    A = mtx.read(path, "full")
    assert (A.nrow, A.ncol) == (M, K)
    assert np.array_equal(A.indptr, indptr)
    assert np.array_equal(A.indices, indices)


@pytest.mark.skipif(not REF_LIB.exists(), reason="reference loader not built (needs the reference checkout)")
@pytest.mark.parametrize("seed", range(6))
def test_random_files_against_reference_loader(lib, tmp_path, seed):
    ref = ctypes.CDLL(str(REF_LIB))
    for case in mtx_cases.CASES:
        p = tmp_path / f"{case}_{seed}.mtx"
        mtx_cases.write(p, case, seed=seed + 10)
        M, K, Z = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        ref.ref_read_mtx(str(p).encode(), ctypes.byref(M), ctypes.byref(K), ctypes.byref(Z), None, None)
        ip = np.empty(M.value + 1, np.int32)
        ix = np.empty(max(1, Z.value), np.int32)
        ref.ref_read_mtx(str(p).encode(), ctypes.byref(M), ctypes.byref(K), ctypes.byref(Z),
                         ip.ctypes.data_as(ctypes.c_void_p), ix.ctypes.data_as(ctypes.c_void_p))
        A = mtx.read(p, "reference")
        assert np.array_equal(A.indptr, ip), case
        assert np.array_equal(A.indices, ix[:Z.value]), case


@pytest.mark.parametrize("body, status", [
    ("%%MatrixMarket matrix array real general\n2 2\n1\n2\n3\n4\n", Status.BAD_DATA),
    ("%%NotMatrixMarket matrix coordinate real general\n1 1 1\n1 1 1\n", Status.BAD_DATA),
    ("%%MatrixMarket matrix coordinate real general\n2 2 1\n3 1 1.0\n", Status.BAD_DATA),
    ("%%MatrixMarket matrix coordinate real general\n2 2 2\n1 1 1.0\n", Status.BAD_DATA),
    ("%%MatrixMarket matrix coordinate real general\n2 2 1\n1 1\n", Status.BAD_DATA),
    ("%%MatrixMarket matrix coordinate real unknown\n2 2 1\n1 1 1\n", Status.BAD_DATA),
])
def test_malformed_files_refused(lib, tmp_path, body, status):
    p = tmp_path / "bad.mtx"
    p.write_text(body)
    with pytest.raises(SegscanError) as e:
        mtx.read(p)
    assert e.value.status == status


_CAPPED_READ = r"""
import ctypes, resource, sys
resource.setrlimit(resource.RLIMIT_AS, (2 << 30, 2 << 30))
lib = ctypes.CDLL(sys.argv[1])
h = ctypes.c_void_p()
print(*(lib.ss_mtx_read(sys.argv[2].encode(), mode, ctypes.byref(h)) for mode in (0, 1)))
"""


@pytest.mark.parametrize("size_line, status", [
    ("3 3 2100000000", Status.BAD_DATA),   # declared count far beyond what the file holds
    ("2147483647 2147483647 1", Status.CAPACITY),  # row pointers beyond the host memory allowed
])
def test_huge_declared_sizes_return_a_status(lib, tmp_path, size_line, status):
    """A short file whose size line declares a huge matrix gets a status code
    in both modes, in a process limited to 2 GB of address space: no
    reservation sized by the declared count alone, and an allocation failure
    is reported instead of ending the process (no exception crosses the C
    boundary)."""
    import subprocess
    import sys
    from segscan_gb300 import _lib
    p = tmp_path / "huge.mtx"
    p.write_text(f"%%MatrixMarket matrix coordinate pattern symmetric\n{size_line}\n1 2\n")
    r = subprocess.run([sys.executable, "-c", _CAPPED_READ, str(_lib.LIB_PATH), str(p)], capture_output=True,
                       text=True, timeout=120)
    assert r.returncode == 0, r.stderr[-500:]
    assert r.stdout.split() == [str(int(status))] * 2


def test_mutated_files_parse_or_are_refused(lib, tmp_path):
    """Seeded byte-level mutations of the committed files (deletions,
    insertions of banner and digit characters, random bytes, truncation):
    each read either gives a well-formed CSR (row pointers from 0 to nnz,
    non-decreasing, columns inside the matrix) or is refused with
    SS_ERR_BAD_DATA, in both modes."""
    import random
    bases = [p.read_bytes() for p in sorted(GOLD.glob("mtx_*.mtx"))]
    alphabet = b"0123456789 \t\r\n%-+.eE%%MatrixMarketcoordinatepatternsymmetricgeneralrealinteger"
    rng = random.Random(7)
    p = tmp_path / "mutated.mtx"
    parsed = 0
    for _ in range(400):
        b = bytearray(rng.choice(bases))
        for _ in range(rng.randint(1, 8)):
            op, pos = rng.random(), rng.randint(0, len(b))
            if op < 0.3 and b:
                del b[pos:pos + rng.randint(1, 12)]
            elif op < 0.6:
                b[pos:pos] = bytes(rng.choice(alphabet) for _ in range(rng.randint(1, 12)))
            elif op < 0.8 and b:
                b[min(pos, len(b) - 1)] = rng.randrange(256)
            else:
                del b[pos:]
        p.write_bytes(bytes(b))
        for mode in ("reference", "full"):
            try:
                A = mtx.read(p, mode)
            except SegscanError as e:
                assert e.status == Status.BAD_DATA, str(e)
                continue
            parsed += 1
            assert A.indptr[0] == 0 and A.indptr[-1] == A.nnz and np.all(np.diff(A.indptr) >= 0)
            assert A.indices.size == A.nnz and np.all((A.indices >= 0) & (A.indices < max(A.ncol, 1)))
    assert parsed > 0


def test_missing_file(lib, tmp_path):
    with pytest.raises(SegscanError) as e:
        mtx.read(tmp_path / "absent.mtx")
    assert e.value.status == Status.INVALID_ARG


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["general_real", "symmetric", "empty_rows"])
def test_data_loader_pair(cuda, case):
    """DataLoader counterpart: A and its transpose built on the device equal
    the stable host transpose (dataloader.hpp:109-144 restated in the
    oracle)."""
    import oracle_lib
    path = GOLD / f"mtx_{case}.mtx"
    host = mtx.read(path)
    A, AT = mtx.data_loader(path)
    assert np.array_equal(A.indptr.cpu().numpy(), host.indptr)
    t_indptr, t_indices, _ = oracle_lib.csr_transpose(host.indptr, host.indices, host.ncol)
    assert np.array_equal(AT.indptr.cpu().numpy(), t_indptr)
    assert np.array_equal(AT.indices.cpu().numpy(), t_indices)
    assert (AT.nrow, AT.ncol) == (host.ncol, host.nrow)
