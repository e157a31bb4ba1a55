"""Shared helpers for the GPU parity tests (checker side)."""
import numpy as np
import torch

import oracle_lib
from segscan_gb300 import synth


def dev_csr(csr, dtype=torch.float32, values=True):
    from segscan_gb300 import api
    return api.CsrMatrix.from_host(csr, "cuda", dtype, values)


def rounded(x, dtype):
    """FP32 array rounded through a 16-bit storage type (what the GPU reads)."""
    return torch.from_numpy(np.ascontiguousarray(x)).to(dtype).float().numpy()


def check_close(C, C64, absC, rtol, normwise=None, what="", atol=1e-30):
    C = np.asarray(C, dtype=np.float64)
    err = np.abs(C - C64)
    bound = rtol * absC + atol
    bad = ~(err <= bound)  # NaN (an element never written, or computed as NaN) counts as off
    assert not bad.any(), (f"{what}: {bad.sum()} elements off; worst err {err.max():.3e} "
                           f"at {np.unravel_index(np.argmax(err - bound), err.shape)}")
    if normwise is not None:
        den = np.linalg.norm(C64)
        if den > 0:
            rel = np.linalg.norm(C - C64) / den
            assert rel <= normwise, f"{what}: normwise {rel:.3e} > {normwise}"


def powerlaw_medium(seed=11, M=40000, lmax=6000):
    return synth.powerlaw(M, M, 2.1, 1, lmax, seed=seed)


def oracle64(csr, B, vals=None):
    return oracle_lib.spmm_f64(csr.indptr, csr.indices, csr.values if vals is None else vals, B)
