"""L2 ceiling model for the SpMM row gathers of the power-law workload.

Replays the column stream of A (the order the walk reads B rows: CSR order;
columns are uniform, so the interleaving of concurrent chunks does not
change the reuse statistics) through an ideal LRU cache of B rows, for the
whole L2 and for the share one die's SMs can use, and turns the miss counts
into DRAM bytes and a lower bound on the launch time at a given DRAM rate:

    python bench_l2_model.py --N 64 --l2-mb 126 63 --dram-gbs 5100

DRAM bytes per launch = misses * row bytes + A's streams (indptr, indices,
values) + C's writes.  The algorithmic bytes count each distinct B row once,
so the ratio of the two is the traffic the cache capacity forces, and
algorithmic bytes / (DRAM bytes / rate) is the highest algorithmic fraction
a kernel can reach at that rate.  CPU only; takes about ten seconds per
capacity.

With --backward it replays instead the dC row stream of the fused backward
on the 2e6 x 2e6 layer (Zipf 2.1 clipped to 50000, seed 4): A^T's entries
(k, i) in A^T order, each reading dC row i, with the kernel's groups
advancing through their contiguous blocks in lockstep.  Rows of A-rows
shorter than --hot-min bypass the cache (1: every row is cached):

    python bench_l2_model.py --backward --N 128 --l2-mb 63 126 --hot-min 1 8
"""
from __future__ import annotations

import argparse
import json
from collections import OrderedDict

import numpy as np

from segscan_gb300 import synth


def lru_misses(stream: np.ndarray, lines: int) -> int:
    """Misses of a fully associative LRU cache of `lines` entries."""
    cache: OrderedDict = OrderedDict()
    misses = 0
    for x in stream.tolist():
        if x in cache:
            cache.move_to_end(x)
        else:
            misses += 1
            cache[x] = None
            if len(cache) > lines:
                cache.popitem(last=False)
    return misses


def model(A: synth.Csr, N: int, l2_mb: list[float], dram_gbs: float, value_bytes: int = 4) -> dict:
    row = N * 4
    distinct = int(np.unique(A.indices).size)
    streams = A.nnz * (4 + value_bytes) + (A.nrow + 1) * 4
    c_bytes = A.nrow * N * 4
    alg = streams + distinct * row + c_bytes
    out = {"nnz": A.nnz, "distinct_columns": distinct, "row_bytes": row, "algorithmic_mb": round(alg / 1e6, 1),
           "compulsory_hit_ceiling": round(1 - distinct / A.nnz, 4), "capacities": []}
    for mb in l2_mb:
        lines = int(mb * 1e6 / row)
        miss = lru_misses(A.indices, lines)
        dram = streams + miss * row + c_bytes
        t_us = dram / (dram_gbs * 1e3)
        out["capacities"].append({
            "l2_mb": mb, "lines": lines, "hit_rate": round(1 - miss / A.nnz, 4),
            "dram_mb": round(dram / 1e6, 1), "traffic_over_alg": round(dram / alg, 3),
            "time_us_at_rate": round(t_us, 1), "alg_gbs_ceiling": round(alg / t_us / 1e3, 1)})
    return out


def lru_hits_hot(stream: np.ndarray, lens: np.ndarray, lines: int, hot_min: int) -> int:
    """Hits of an LRU of `lines` rows that only rows with lens >= hot_min enter."""
    cache: OrderedDict = OrderedDict()
    hits = 0
    for x, n in zip(stream.tolist(), lens.tolist()):
        if n < hot_min:
            continue
        if x in cache:
            hits += 1
            cache.move_to_end(x)
        else:
            cache[x] = None
            if len(cache) > lines:
                cache.popitem(last=False)
    return hits


def backward_model(N: int, l2_mb: list[float], hot_mins: list[int], groups: int) -> dict:
    A = synth.powerlaw(2_000_000, 2_000_000, 2.1, 1, 50_000, seed=4)
    rowlen = np.diff(A.indptr)
    rows = np.repeat(np.arange(A.nrow, dtype=np.int64), rowlen)  # A's row of each nonzero
    seq = rows[np.argsort(A.indices, kind="stable")]               # the dC row of each A^T entry
    blk = -(-seq.size // groups)
    q = np.arange(seq.size)
    stream = seq[np.lexsort((q // blk, q % blk))]                  # groups in lockstep
    lens = rowlen[stream]
    out = {"nnz": int(seq.size), "row_bytes": N * 4, "groups": groups, "capacities": []}
    for mb in l2_mb:
        lines = int(mb * 2 ** 20 / (N * 4))
        for h in hot_mins:
            hits = lru_hits_hot(stream, lens, lines, h)
            out["capacities"].append({"l2_mb": mb, "hot_min": h, "hit_rate": round(hits / seq.size, 4)})
    return out


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--N", type=int, default=64)
    ap.add_argument("--l2-mb", type=float, nargs="+", default=[126.0, 63.0])
    ap.add_argument("--dram-gbs", type=float, default=5100.0,
                    help="DRAM rate of random row reads mixed with C writes")
    ap.add_argument("--peak-gbs", type=float, default=None, help="adds alg_gbs_ceiling / peak")
    ap.add_argument("--backward", action="store_true", help="the fused backward's dC stream instead")
    ap.add_argument("--hot-min", type=int, nargs="+", default=[1])
    ap.add_argument("--groups", type=int, default=152 * 4 * 8 * 2,
                    help="backward: groups walking A^T (about the resident ones)")
    a = ap.parse_args(argv)
    if a.backward:
        print(json.dumps(backward_model(a.N, a.l2_mb, a.hot_min, a.groups), indent=1))
        return
    A = synth.powerlaw(1_000_000, 1_000_000, 2.1, 1, 20000, seed=1)
    out = model(A, a.N, a.l2_mb, a.dram_gbs)
    if a.peak_gbs:
        for c in out["capacities"]:
            c["frac_ceiling"] = round(c["alg_gbs_ceiling"] / a.peak_gbs, 3)
    print(json.dumps(out, indent=1))


if __name__ == "__main__":
    main()
