"""Failure detection on the GPU without a fault: a bounded wait that runs
out sets the device status word (SS_ERR_TIMEOUT), the host reads and clears
it, and the same context keeps computing correct results."""
import ctypes

import pytest
import torch

from gpu_util import check_close, dev_csr, oracle64
from segscan_gb300 import _lib, api, synth
from segscan_gb300._lib import Status

pytestmark = pytest.mark.gpu


def device_status(lib, clear=0):
    st = ctypes.c_int(-1)
    assert lib.ss_device_error(ctypes.byref(st), clear) == 0
    return st.value


def test_bounded_wait_times_out_and_context_survives(cuda, lib):
    device_status(lib, clear=1)
    assert device_status(lib) == 0
    s = torch.cuda.current_stream().cuda_stream
    assert lib.ss_selftest_bounded_wait(2000, s) == 0
    torch.cuda.synchronize()
    assert device_status(lib) == Status.TIMEOUT
    assert device_status(lib, clear=1) == Status.TIMEOUT
    assert device_status(lib) == 0
    # the context is healthy: a full SpMM runs and is right, with no new timeout
    csr = synth.powerlaw(20000, 20000, 2.1, 1, 2000, seed=41)
    B = synth.dense(csr.ncol, 32, seed=42)
    C = api.spmm(dev_csr(csr), torch.from_numpy(B).cuda(), "ebsr")
    torch.cuda.synchronize()
    C64, absC = oracle64(csr, B)
    check_close(C.cpu().numpy(), C64, absC, 1e-5, 1e-5, "after the timeout")
    assert device_status(lib) == 0


def test_selftest_rejects_bad_poll_counts(cuda, lib):
    assert lib.ss_selftest_bounded_wait(0, None) == Status.INVALID_ARG
    assert lib.ss_selftest_bounded_wait(1 << 23, None) == Status.INVALID_ARG
