"""Launches the reference's own SpMM kernels (test-cg/include/spmm/
spmm_cg.cuh, compiled for sm_103a into oracle/_ref/ref_kernels.cubin by
`make -C oracle ref`) through the CUDA driver API, with the launch geometry
of the reference's launchers (spmm_cg.cuh:176-197, 333-353, 553-566,
664-677) at its README-best static knobs for N = 64.  Test and measurement
infrastructure only: the comparison line for this library's kernels."""
from __future__ import annotations

import ctypes
from pathlib import Path

import torch

CUBIN = Path(__file__).resolve().parent.parent / "oracle" / "_ref" / "ref_kernels.cubin"
SEG_CUBIN = Path(__file__).resolve().parent.parent / "oracle" / "_ref" / "ref_segment_kernels.cubin"


def ceil_div(a, b):
    return (a + b - 1) // b


class RefKernels:
    """The four reference kernels for N = 64 (float4 accesses)."""

    N = 64

    def __init__(self):
        torch.cuda.init()
        torch.empty(1, device="cuda")  # the primary context is current on this thread
        self.cu = ctypes.CDLL("libcuda.so.1")
        self.mod = ctypes.c_void_p()
        self._check(self.cu.cuModuleLoad(ctypes.byref(self.mod), str(CUBIN).encode()), "cuModuleLoad")
        self.fn = {}
        for name in ("ebpr", "rbpr", "ebsr", "rbsr"):
            f = ctypes.c_void_p()
            self._check(self.cu.cuModuleGetFunction(ctypes.byref(f), self.mod, f"ref_{name}_n64".encode()),
                        f"cuModuleGetFunction ref_{name}_n64")
            self.fn[name] = f

    @staticmethod
    def available() -> bool:
        return CUBIN.exists()

    @staticmethod
    def _check(rc, what):
        if rc != 0:
            raise RuntimeError(f"{what} failed with CUresult {rc}")

    def geometry(self, strategy: str, M: int, N: int):
        """(grid, block, smem) the reference's launcher computes."""
        assert N == self.N
        if strategy == "ebpr":  # (5,256,5,1,16): group 32, tile 32
            tile, tpb, factor = 32, 256, 1 / 16
            cf = 4
            ndim_tb = ceil_div(N, tile)
            ndim_warp = min(N, tile) // cf
            nnz_warp_per_tb = ceil_div(tpb // tile, ndim_warp)
            return (ceil_div(int(M * factor), nnz_warp_per_tb), ndim_tb, 1), (ndim_warp * tile, nnz_warp_per_tb, 1), 0
        if strategy == "rbpr":  # (3,256,3,1,2): group 8, tile 8
            tile, tpb, factor = 8, 256, 1 / 2
            cf = 4
            ndim_tb = ceil_div(N, tile)
            ndim_warp = min(N, tile) // cf
            m_warp_per_tb = ceil_div(tpb // tile, ndim_warp)
            return (ceil_div(int(M * factor), m_warp_per_tb), ndim_tb, 1), (ndim_warp * tile, m_warp_per_tb, 1), 0
        if strategy == "ebsr":  # (4,256,4,1,1,16): group 16, CoarsenFactor 4, ThreadNz 1
            group, tpb, factor = 16, 256, 1 / 16
            coarsen = min(ceil_div(N, group), 4)
            return (int(M * factor), ceil_div(N, group * coarsen), 1), (256, 1, 1), 12 * tpb
        if strategy == "rbsr":  # coarsen 4, tile 2^5, 256 threads
            tile, tpb, cf = 32, 256, 4
            ndim_tb = ceil_div(N, tile)
            nthr = min(N, tile) // cf
            mthr = ceil_div(tpb, nthr)
            return (ceil_div(M, mthr), ndim_tb, 1), (mthr, nthr, 1), 0
        raise ValueError(strategy)

    def launch(self, strategy: str, M: int, K: int, nnz: int, indptr, indices, data, B, C, stream=None):
        """One launch (C must be zeroed first for all but rbsr, as the reference requires)."""
        N = int(B.shape[1])
        grid, block, smem = self.geometry(strategy, M, N)
        ints = [ctypes.c_int(M), ctypes.c_int(N), ctypes.c_int(K)]
        if strategy in ("ebpr", "ebsr"):
            ints.append(ctypes.c_int(nnz))
        ptrs = [ctypes.c_void_p(t.data_ptr()) for t in (indptr, indices, data, B, C)]
        vals = ints + ptrs
        params = (ctypes.c_void_p * len(vals))(*[ctypes.cast(ctypes.pointer(v), ctypes.c_void_p) for v in vals])
        s = (stream or torch.cuda.current_stream()).cuda_stream
        self._check(self.cu.cuLaunchKernel(self.fn[strategy], grid[0], grid[1], grid[2], block[0], block[1], block[2],
                                           smem, ctypes.c_void_p(s), params, None), f"launch {strategy}")


class DgKernels:
    """The dgSPARSE baseline kernels (test-cg/include/spmm/spmm.cuh:17-637)
    from the same cubin, with their launchers' geometry (spmm.cuh:167-200,
    310-343, 522-590, 621-637; RefThreadPerBlock 256, check.cuh:13), for N a
    multiple of 4 up to 256: the widths the launchers would pick there
    (float4 for ebpr/rbpr, ebsr CoarsenFactor 1 below N = 128 and 2 from
    128), and rbsr's one thread per (row, column) stays inside N."""

    TPB = 256

    def __init__(self, ref: RefKernels):
        self.cu, self.mod = ref.cu, ref.mod
        self.fn = {}
        for name in ("dg_ebpr_f4", "dg_rbpr_f4", "dg_ebsr_c1", "dg_ebsr_c2", "dg_rbsr"):
            f = ctypes.c_void_p()
            RefKernels._check(self.cu.cuModuleGetFunction(ctypes.byref(f), self.mod, name.encode()), name)
            self.fn[name] = f

    def geometry(self, strategy: str, M: int, N: int):
        """(kernel, grid, block, smem) as the dgSPARSE launcher computes them."""
        assert N % 4 == 0 and 0 < N <= 256, N
        if strategy in ("ebpr", "rbpr"):
            cf = 4
            ndim_tb = ceil_div(N, 32)
            ndim_warp = min(N, 32) // cf
            warp_per_tb = ceil_div(self.TPB // 32, ndim_warp)
            return (f"dg_{strategy}_f4", (ceil_div(M, warp_per_tb), ndim_tb, 1), (ndim_warp * 32, warp_per_tb, 1), 0)
        if strategy == "ebsr":
            cf = 2 if N >= 128 else 1
            return (f"dg_ebsr_c{cf}", (ceil_div(M, self.TPB // 32), ceil_div(N, 32 * cf), 1), (self.TPB, 1, 1),
                    12 * self.TPB)
        if strategy == "rbsr":
            nthr = min(N, self.TPB)
            mthr = ceil_div(self.TPB, nthr)
            return "dg_rbsr", (ceil_div(M, mthr), ceil_div(N, self.TPB), 1), (nthr, mthr, 1), 0
        raise ValueError(strategy)

    def launch(self, strategy: str, M: int, K: int, nnz: int, indptr, indices, data, B, C, stream=None):
        """One launch; C must be zeroed first for all but rbsr."""
        N = int(B.shape[1])
        fn, grid, block, smem = self.geometry(strategy, M, N)
        ints = [ctypes.c_int(M), ctypes.c_int(N), ctypes.c_int(K)]
        if strategy in ("ebpr", "ebsr"):
            ints.append(ctypes.c_int(nnz))
        ptrs = [ctypes.c_void_p(t.data_ptr()) for t in (indptr, indices, data, B, C)]
        vals = ints + ptrs
        params = (ctypes.c_void_p * len(vals))(*[ctypes.cast(ctypes.pointer(v), ctypes.c_void_p) for v in vals])
        s = (stream or torch.cuda.current_stream()).cuda_stream
        RefKernels._check(self.cu.cuLaunchKernel(self.fn[fn], grid[0], grid[1], grid[2], block[0], block[1], block[2],
                                                 smem, ctypes.c_void_p(s), params, None), f"launch {fn}")


class RefSegmentKernels:
    """Four of the reference's segment_coo kernels (new-cg/include/segscan/
    segscan.cuh), each with its launcher's geometry:
      sr      segment_coo_sr<float, int, 4, 256, 4, 1, 1, 16> (:817-829)
      sorted  segment_coo_sorted_sr<float, int, 2, 4, 8, 2, 16> (:974-981), the one
              new-cg/src/main.cu runs
      pr      segment_coo<float, int, 5, 256, 5, 1, 16> (:150-171)
      new     segment_coo_new<float, int, 5, 256, 5, 2> (:327-342)
      noshmem segment_coo_noshmem_sr<float, int, 4, 256, 4, 2, 1, 16> (:868-880)
      lessatom segment_coo_noshmem_lessatom_sr<float, int, 4, 256, 4, 1, 1, 16> (:918-930)
    All add into dst, which the caller zeroes.  They read index[] past nnz
    (up to 15, 31 and blockDim.x - 1 = 127 entries: :402, :31, :209):
    `launch` requires an index buffer padded by at least PAD entries."""

    PAD = 256

    def __init__(self):
        torch.cuda.init()
        torch.empty(1, device="cuda")
        self.cu = ctypes.CDLL("libcuda.so.1")
        self.mod = ctypes.c_void_p()
        RefKernels._check(self.cu.cuModuleLoad(ctypes.byref(self.mod), str(SEG_CUBIN).encode()), "cuModuleLoad")
        self.fn = {}
        for name in ("ref_seg_sr_n64", "ref_seg_sorted_sr", "ref_seg_pr_f4", "ref_seg_new_f4", "ref_seg_noshmem_n64",
                     "ref_seg_lessatom_n64"):
            f = ctypes.c_void_p()
            RefKernels._check(self.cu.cuModuleGetFunction(ctypes.byref(f), self.mod, name.encode()), name)
            self.fn[name] = f

    @staticmethod
    def available() -> bool:
        return SEG_CUBIN.exists()

    def launch(self, which: str, src, index_padded, nnz: int, dst, stream=None):
        N = int(src.shape[1])
        assert index_padded.numel() >= nnz + self.PAD
        if which == "sr":  # group 16, 256 threads, CoarsenFactor min(CEIL(N, 16), 4), block_factor 1/16
            assert N == 64
            grid, block, smem, fn = (int(nnz / 16), ceil_div(N, 16 * 4), 1), (256, 1, 1), 12 * 256, "ref_seg_sr_n64"
        elif which == "sorted":  # CoarsenFactor 2, ThreadNz 4, DtileSize 8, DtileNum 2, BlockDimY 16
            bx = min(2, ceil_div(N, 8 * 2)) * 8
            by = min(16, ceil_div(nnz, 4))
            grid, block, smem, fn = (ceil_div(N, bx * 2), ceil_div(nnz, by * 4), 1), (bx, by, 1), 0, "ref_seg_sorted_sr"
            if grid[1] > 65535:
                raise ValueError(f"segment_coo_sorted_sr's grid.y {grid[1]} exceeds 65535 (nnz {nnz})")
        elif which == "pr":  # float4, tile 32, 256 threads, block_factor 1/16
            assert N % 4 == 0
            ndim_warp = min(N, 32) // 4
            nnz_warp_per_tb = ceil_div(256 // 32, ndim_warp)
            workers = int(nnz * (1.0 / 16.0))
            grid = (max(1, ceil_div(workers, nnz_warp_per_tb)), ceil_div(N, 32), 1)
            block, smem, fn = (ndim_warp * 32, nnz_warp_per_tb, 1), 0, "ref_seg_pr_f4"
        elif which in ("noshmem", "lessatom"):  # group 16, 256 threads, CoarsenFactor 4, block_factor 1/16
            assert N == 64
            grid, block, smem, fn = (int(nnz / 16), ceil_div(N, 16 * 4), 1), (256, 1, 1), 0, f"ref_seg_{which}_n64"
        elif which == "new":  # float4, tile 32, 256 threads, blockDimY 2
            assert N % 4 == 0
            tiles_y = ceil_div(N, 4)
            by = min(tiles_y, 2)  # blockDimY 2 is below 256 / tile = 8
            bx = ceil_div(256, by)
            grid, block, smem, fn = (ceil_div(nnz, bx), ceil_div(tiles_y, by), 1), (bx, by, 1), 0, "ref_seg_new_f4"
            assert bx <= self.PAD
        else:
            raise ValueError(which)
        vals = [ctypes.c_void_p(src.data_ptr()), ctypes.c_void_p(index_padded.data_ptr()), ctypes.c_int(nnz),
                ctypes.c_int(N), ctypes.c_void_p(dst.data_ptr())]
        params = (ctypes.c_void_p * len(vals))(*[ctypes.cast(ctypes.pointer(v), ctypes.c_void_p) for v in vals])
        s = (stream or torch.cuda.current_stream()).cuda_stream
        RefKernels._check(self.cu.cuLaunchKernel(self.fn[fn], grid[0], grid[1], grid[2], block[0], block[1], block[2],
                                                 smem, ctypes.c_void_p(s), params, None), f"launch {fn}")
