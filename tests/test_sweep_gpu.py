"""The kernel sweep (segscan_gb300/sweep.py) on the GPU: every action of a
small sweep runs, lands in the table, and reduces through the ratio
summaries; each library action's result is checked against FP64 on one
matrix, so a tuple the sweep times is a tuple that computes SpMM."""
import numpy as np
import pytest
import torch

from gpu_util import check_close, oracle64
from segscan_gb300 import api, ratios, synth, sweep

pytestmark = pytest.mark.gpu


def test_sweep_table_and_ratios(cuda, tmp_path):
    specs = ["poisson:3000:12:0", "powerlaw:20000:2.1:2000:7"]
    rows = sweep.run(specs, 32, iters=3, tuples="defaults")
    p = tmp_path / "t.csv"
    ratios.write_csv(p, rows)
    back = ratios.read_csv(p)
    assert back == rows
    table = ratios.pivot(back)
    assert set(table) == {(s, 32) for s in specs}
    for t in table.values():
        assert "cusparse" in t and len(t) == 5 and all(v > 0 for v in t.values())
    out = ratios.tuning(back, sweep.label("ebsr", api.default_knobs("ebsr", 32)))
    assert out["datasets"] == 2 and sum(out["best_histogram"].values()) == 2


def test_every_swept_tuple_computes_spmm(cuda):
    A = synth.powerlaw(8000, 8000, 2.1, 1, 1500, seed=8)
    N = 64
    B = synth.dense(A.ncol, N, seed=9)
    Ad = api.CsrMatrix.from_host(A, "cuda")
    Bd = torch.from_numpy(B).cuda()
    C64, absC = oracle64(A, B)
    n = 0
    for s, k in sweep.library_actions(N):
        C = api.spmm(Ad, Bd, s, knobs=k)
        torch.cuda.synchronize()
        check_close(C.cpu().numpy(), C64, absC, 1e-5, None, f"{sweep.label(s, k)}")
        n += 1
    assert n == len(sweep.library_actions(N))
