"""Ratio summaries of a kernel sweep: the reference's analysis methodology.

The reference profiles every kernel variant ("action") on every matrix
("dataset") and reduces the kernel times to a few ratios
(test-cg/src/count.py, static.py, dgcmp.py, fed by clean.py's table):

* tuning speed-up (count.py:33): time of one fixed action / time of the
  dataset's best action, with the histogram of which action was best;
* vs cuSPARSE (count.py:25-34): cuSPARSE's time (the sum of its kernels) /
  the best action's time; above 1 means the tuned kernel is faster;
* static ranking (static.py:17-34): for each action, the mean, standard
  deviation and geometric mean over datasets of its time / the best time,
  and the actions within `epsilon` of the smallest geometric mean;
* one action against another (dgcmp.py:18-30): time(base) / time(action),
  e.g. the dgSPARSE kernel against a static tuple.

A table here is a list of `Row`s (dataset, N, action, kind, time_us), kind
one of "cusparse" (summed per dataset), "library" or "external" (a
comparison kernel that is not cuSPARSE); it is written and read as CSV.
Times come from `segscan_gb300.sweep` (CUDA events) or from an ncu launch
list (`from_ncu_csv`), which is what the reference's tables hold.

    python -m segscan_gb300.ratios table.csv --default "ebsr(4,256,4,2,1,16)"
"""
from __future__ import annotations

import argparse
import csv
import json
import math
import sys
from dataclasses import dataclass
from typing import Iterable, Optional, Sequence

FIELDS = ("dataset", "N", "action", "kind", "time_us")


@dataclass(frozen=True)
class Row:
    dataset: str
    N: int
    action: str
    kind: str  # "cusparse" | "library" | "external"
    time_us: float


def write_csv(path, rows: Iterable[Row]) -> None:
    with open(path, "w", newline="") as f:
        w = csv.writer(f)
        w.writerow(FIELDS)
        for r in rows:
            w.writerow([r.dataset, r.N, r.action, r.kind, repr(float(r.time_us))])


def read_csv(path) -> list[Row]:
    with open(path, newline="") as f:
        rd = csv.DictReader(f)
        missing = set(FIELDS) - set(rd.fieldnames or ())
        if missing:
            raise ValueError(f"{path}: columns {sorted(missing)} missing")
        return [Row(d["dataset"], int(d["N"]), d["action"], d["kind"], float(d["time_us"])) for d in rd]


def _number(text: str) -> float:
    return float(text.replace(",", ""))


def ncu_launches(path) -> list[tuple[str, float]]:
    """(kernel name, duration in us) per launch, in launch order, from an
    `ncu --csv --metrics gpu__time_duration.sum` log (the reference's Time
    column, clean.py:19).  Lines before the CSV header (==PROF== notes) are
    skipped."""
    scale = {"ns": 1e-3, "nsecond": 1e-3, "usecond": 1.0, "us": 1.0, "msecond": 1e3, "ms": 1e3, "second": 1e6,
             "s": 1e6}
    with open(path, newline="") as f:
        lines = f.read().splitlines()
    start = next((i for i, l in enumerate(lines) if l.startswith('"ID"')), None)
    if start is None:
        raise ValueError(f"{path}: no ncu CSV header")
    out = []
    for d in csv.DictReader(lines[start:]):
        if d.get("Metric Name") != "gpu__time_duration.sum":
            continue
        unit = d.get("Metric Unit", "ns")
        if unit not in scale:
            raise ValueError(f"{path}: unknown time unit {unit!r}")
        out.append((d["Kernel Name"], _number(d["Metric Value"]) * scale[unit]))
    return out


def from_ncu_csv(path, dataset: str, N: int, actions: Sequence[tuple[str, str, int]]) -> list[Row]:
    """Rows for one dataset from an ncu launch list: `actions` gives, in
    launch order, (action, kind, number of kernel launches it makes); each
    action's time is the sum of its launches (as count.py sums cuSPARSE's
    records).  The launch count must match exactly."""
    launches = ncu_launches(path)
    need = sum(n for _, _, n in actions)
    if need != len(launches):
        raise ValueError(f"{path}: {len(launches)} launches, the actions account for {need}")
    rows, i = [], 0
    for action, kind, n in actions:
        rows.append(Row(dataset, N, action, kind, sum(t for _, t in launches[i:i + n])))
        i += n
    return rows


def pivot(rows: Iterable[Row]) -> dict[tuple[str, int], dict[str, float]]:
    """{(dataset, N): {action: time}}; cuSPARSE rows are summed under
    "cusparse"."""
    out: dict[tuple[str, int], dict[str, float]] = {}
    for r in rows:
        d = out.setdefault((r.dataset, r.N), {})
        if r.kind == "cusparse":
            d["cusparse"] = d.get("cusparse", 0.0) + r.time_us
        else:
            d[r.action] = r.time_us
    return out


def gmean(xs: Sequence[float]) -> float:
    return math.exp(sum(math.log(x) for x in xs) / len(xs))


def stats(xs: Sequence[float]) -> dict:
    """max, mean, population std (numpy's default) and geometric mean."""
    n = len(xs)
    mean = sum(xs) / n
    return {"n": n, "max": max(xs), "mean": mean, "std": math.sqrt(sum((x - mean) ** 2 for x in xs) / n),
            "gmean": gmean(xs)}


def _candidates(rows: Sequence[Row], candidates: Optional[Sequence[str]]) -> list[str]:
    if candidates is not None:
        return list(candidates)
    seen = []
    for r in rows:
        if r.kind == "library" and r.action not in seen:
            seen.append(r.action)
    return seen


def tuning(rows: Sequence[Row], default: str, candidates: Optional[Sequence[str]] = None) -> dict:
    """count.py's summary: over datasets, which candidate was best, the
    speed-up of the best over `default`, and cuSPARSE / best."""
    cands = _candidates(rows, candidates)
    table = pivot(rows)
    hist = {a: 0 for a in cands}
    speedups, vs_cu, names, names_cu = [], [], [], []
    for key, t in sorted(table.items()):
        have = [a for a in cands if a in t]
        if not have or default not in t:
            continue
        best = min(have, key=lambda a: t[a])
        hist[best] += 1
        speedups.append(t[default] / t[best])
        names.append(key)
        if "cusparse" in t:
            vs_cu.append(t["cusparse"] / t[best])
            names_cu.append(key)
    if not speedups:
        raise ValueError("no dataset has the default action and a candidate")
    out = {"datasets": len(speedups), "best_histogram": hist, "default": default,
           "tuning_speedup": dict(stats(speedups), argmax=_name(names[speedups.index(max(speedups))]))}
    if vs_cu:
        faster = [(_name(n), r) for n, r in zip(names_cu, vs_cu) if r > 1]
        out["vs_cusparse"] = dict(stats(vs_cu), argmax=_name(names_cu[vs_cu.index(max(vs_cu))]),
                                  faster=len(faster), faster_datasets=[n for n, _ in faster])
    return out


def static_ranking(rows: Sequence[Row], candidates: Optional[Sequence[str]] = None,
                   epsilon: float = 0.01) -> dict:
    """static.py's summary: each candidate's time / the best candidate's
    time over datasets; the candidates whose geometric mean is within
    epsilon of the smallest are the best static choices."""
    cands = _candidates(rows, candidates)
    table = pivot(rows)
    per: dict[str, list[float]] = {a: [] for a in cands}
    for t in table.values():
        have = [a for a in cands if a in t]
        if len(have) != len(cands):
            continue  # a dataset every candidate ran on, as the reference's fixed action list
        best = min(t[a] for a in cands)
        for a in cands:
            per[a].append(t[a] / best)
    if not per[cands[0]]:
        raise ValueError("no dataset has every candidate")
    ranked = {a: stats(v) for a, v in per.items()}
    low = min(s["gmean"] for s in ranked.values())
    return {"datasets": len(per[cands[0]]), "epsilon": epsilon,
            "best_static": [dict(action=a, **ranked[a]) for a in cands if abs(ranked[a]["gmean"] - low) < epsilon],
            "all": ranked}


def compare(rows: Sequence[Row], base: str, action: str) -> dict:
    """dgcmp.py's summary of time(base) / time(action) over the datasets
    that ran both; above 1 means `action` is faster."""
    r, names = [], []
    for key, t in sorted(pivot(rows).items()):
        if base in t and action in t:
            r.append(t[base] / t[action])
            names.append(key)
    if not r:
        raise ValueError(f"no dataset ran both {base} and {action}")
    return dict(stats(r), base=base, action=action, argmax=_name(names[r.index(max(r))]),
                faster=sum(1 for x in r if x > 1))


def per_strategy(rows: Sequence[Row], defaults: dict) -> dict:
    """README.md's tables 4 and 5 per strategy and width: over the datasets,
    the speed-up of the strategy's best tuple over its default tuple
    (table 4) and cuSPARSE time / the strategy's best time (table 5).
    defaults[N][strategy] is the default tuple's label."""
    out: dict = {}
    widths = sorted({r.N for r in rows})
    for N in widths:
        sub = [r for r in rows if r.N == N]
        for strategy, default in sorted(defaults.get(N, {}).items()):
            cands = sorted({r.action for r in sub if r.kind == "library" and r.action.startswith(strategy + "(")})
            if default not in cands:
                continue
            t = tuning(sub, default, cands)
            out[f"{strategy}@N={N}"] = {"datasets": t["datasets"], "tuning_speedup": t["tuning_speedup"],
                                        "vs_cusparse": t.get("vs_cusparse")}
    return out


def _name(key: tuple[str, int]) -> str:
    return f"{key[0]}@N={key[1]}"


def main(argv=None):
    ap = argparse.ArgumentParser(description="ratio summaries of a sweep table")
    ap.add_argument("table")
    ap.add_argument("--default", help="the fixed action the tuning speed-up is measured against")
    ap.add_argument("--compare", nargs=2, action="append", default=[], metavar=("BASE", "ACTION"))
    ap.add_argument("--epsilon", type=float, default=0.01)
    ap.add_argument("--per-strategy", metavar="DEFAULTS_JSON",
                    help="the JSON line `segscan_gb300.sweep` printed: adds the per-strategy tables")
    a = ap.parse_args(argv)
    rows = read_csv(a.table)
    out = {}
    if a.default:
        out = {"tuning": tuning(rows, a.default), "static": static_ranking(rows, epsilon=a.epsilon)}
        out["static"].pop("all")
    out["compare"] = [compare(rows, b, x) for b, x in a.compare]
    if a.per_strategy:
        with open(a.per_strategy) as f:
            line = [ln for ln in f if ln.strip().startswith("{")][-1]
        defaults = {int(n): d for n, d in json.loads(line)["defaults"].items()}
        out["per_strategy"] = per_strategy(rows, defaults)
    print(json.dumps(out, indent=1))


if __name__ == "__main__":
    sys.exit(main())
