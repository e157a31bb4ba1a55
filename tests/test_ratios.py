"""The sweep's ratio summaries (segscan_gb300/ratios.py) against values
worked out by hand, the ncu launch-list reader, and the sweep's dataset
specs and tuple labels (CPU only)."""
import math

import pytest

from segscan_gb300 import ratios
from segscan_gb300.ratios import Row


def table():
    # two datasets; cuSPARSE in two kernels on the first, one on the second
    return [
        Row("a", 64, "cusparse", "cusparse", 30.0), Row("a", 64, "cusparse", "cusparse", 10.0),
        Row("a", 64, "dg", "external", 50.0),
        Row("a", 64, "t0", "library", 20.0), Row("a", 64, "t1", "library", 10.0), Row("a", 64, "t2", "library", 40.0),
        Row("b", 64, "cusparse", "cusparse", 12.0),
        Row("b", 64, "dg", "external", 30.0),
        Row("b", 64, "t0", "library", 15.0), Row("b", 64, "t1", "library", 30.0), Row("b", 64, "t2", "library", 15.0),
    ]


def test_pivot_sums_cusparse_kernels():
    p = ratios.pivot(table())
    assert p[("a", 64)]["cusparse"] == 40.0 and p[("b", 64)]["cusparse"] == 12.0
    assert p[("a", 64)]["t1"] == 10.0


def test_tuning_summary():
    out = ratios.tuning(table(), default="t0")
    # best: a -> t1 (10), b -> t0 (15; first of the tie, as list.index picks)
    assert out["best_histogram"] == {"t0": 1, "t1": 1, "t2": 0}
    sp = out["tuning_speedup"]
    assert sp["max"] == 2.0 and sp["argmax"] == "a@N=64"
    assert math.isclose(sp["mean"], 1.5) and math.isclose(sp["gmean"], math.sqrt(2.0))
    assert math.isclose(sp["std"], 0.5)
    cu = out["vs_cusparse"]  # 40/10 = 4 and 12/15 = 0.8
    assert cu["faster"] == 1 and cu["faster_datasets"] == ["a@N=64"]
    assert math.isclose(cu["gmean"], math.sqrt(4 * 0.8)) and cu["max"] == 4.0


def test_static_ranking():
    out = ratios.static_ranking(table(), epsilon=0.01)
    # t0: 2, 1 -> gmean sqrt 2; t1: 1, 2 -> sqrt 2; t2: 4, 1 -> 2
    assert math.isclose(out["all"]["t0"]["gmean"], math.sqrt(2))
    assert math.isclose(out["all"]["t2"]["gmean"], 2.0)
    assert [b["action"] for b in out["best_static"]] == ["t0", "t1"]


def test_compare_base_over_action():
    out = ratios.compare(table(), "dg", "t0")  # 50/20 = 2.5, 30/15 = 2
    assert math.isclose(out["gmean"], math.sqrt(5.0)) and out["faster"] == 2 and out["argmax"] == "a@N=64"
    with pytest.raises(ValueError):
        ratios.compare(table(), "dg", "missing")


def test_per_strategy_tables():
    rows = [
        Row("a", 4, "cusparse", "cusparse", 40.0), Row("b", 4, "cusparse", "cusparse", 12.0),
        Row("a", 4, "ebsr(1,2)", "library", 20.0), Row("a", 4, "ebsr(3,4)", "library", 10.0),
        Row("b", 4, "ebsr(1,2)", "library", 15.0), Row("b", 4, "ebsr(3,4)", "library", 30.0),
        Row("a", 4, "rbsr(5)", "library", 8.0), Row("b", 4, "rbsr(5)", "library", 24.0),
    ]
    out = ratios.per_strategy(rows, {4: {"ebsr": "ebsr(1,2)", "rbsr": "rbsr(5)", "ebpr": "ebpr(9)"}})
    assert set(out) == {"ebsr@N=4", "rbsr@N=4"}  # no ebpr rows: left out
    e = out["ebsr@N=4"]  # best a: 10 (2x over the default), b: the default 15 (1x)
    assert math.isclose(e["tuning_speedup"]["gmean"], math.sqrt(2.0)) and e["tuning_speedup"]["max"] == 2.0
    assert math.isclose(e["vs_cusparse"]["gmean"], math.sqrt(4.0 * 0.8))  # 40/10, 12/15
    r = out["rbsr@N=4"]  # one tuple: no tuning gain; cuSPARSE 40/8 and 12/24
    assert r["tuning_speedup"]["max"] == 1.0 and math.isclose(r["vs_cusparse"]["gmean"], math.sqrt(5.0 * 0.5))


def test_csv_round_trip(tmp_path):
    p = tmp_path / "t.csv"
    ratios.write_csv(p, table())
    assert ratios.read_csv(p) == table()


NCU_LOG = '''==WARNING== Note: Running with unmodified GPU clocks.
==PROF== Connected to process 1 (/usr/bin/python3)
"ID","Process ID","Process Name","Host Name","Kernel Name","Context","Stream","Block Size","Grid Size","Device","CC","Section Name","Metric Name","Metric Unit","Metric Value"
"0","1","python3","h","csrmm_kernel_a","1","7","(256, 1, 1)","(10, 1, 1)","0","10.3","Command line profiler metrics","gpu__time_duration.sum","ns","1,500"
"1","1","python3","h","csrmm_kernel_b","1","7","(256, 1, 1)","(10, 1, 1)","0","10.3","Command line profiler metrics","gpu__time_duration.sum","ns","500"
"2","1","python3","h","void eb_sr_kernel<float, float, 4, 1, 0>(EbArgs)","1","7","(256, 1, 1)","(565, 1, 1)","0","10.3","Command line profiler metrics","gpu__time_duration.sum","usecond","3.25"
"3","1","python3","h","void eb_pr_kernel(EbArgs)","1","7","(256, 1, 1)","(565, 1, 1)","0","10.3","Command line profiler metrics","gpu__time_duration.sum","ns","4000"
"4","1","python3","h","void fixup_kernel(EbArgs)","1","7","(256, 1, 1)","(565, 1, 1)","0","10.3","Command line profiler metrics","gpu__time_duration.sum","ns","250"
'''


def test_ncu_launch_list(tmp_path):
    p = tmp_path / "launches.csv"
    p.write_text(NCU_LOG)
    launches = ratios.ncu_launches(p)
    assert [round(t, 6) for _, t in launches] == [1.5, 0.5, 3.25, 4.0, 0.25]
    rows = ratios.from_ncu_csv(p, "m", 64, [("cusparse", "cusparse", 2), ("ebsr(x)", "library", 1),
                                            ("ebpr(y)", "library", 2)])
    assert [(r.action, round(r.time_us, 6)) for r in rows] == [("cusparse", 2.0), ("ebsr(x)", 3.25),
                                                               ("ebpr(y)", 4.25)]
    with pytest.raises(ValueError):
        ratios.from_ncu_csv(p, "m", 64, [("cusparse", "cusparse", 2)])


def test_sweep_specs_and_labels():
    from segscan_gb300 import api, sweep
    A = sweep.dataset("powerlaw:2000:2.1:100:3")
    assert A.nrow == 2000 and A.indptr[-1] == A.nnz
    assert sweep.dataset("poisson:1000:8").nrow == 1000
    assert sweep.dataset("banded:1000:5:20").nnz <= 5000
    with pytest.raises(ValueError):
        sweep.dataset("uniform:10")
    k = api.make_knobs("ebsr", 64, group_factor=4, thread_per_block=256, coarsen_factor=4, thread_nz=1,
                       block_numer=1, block_denom=16)
    assert sweep.label("ebsr", k) == "ebsr(4,256,4,1,1,16)"
    acts = sweep.library_actions(64)
    labels = [sweep.label(s, k) for s, k in acts]
    assert len(labels) == len(set(labels)) and labels[:4] == [sweep.label(s, api.default_knobs(s, 64))
                                                              for s in ("ebpr", "rbpr", "ebsr", "rbsr")]


def test_ratios_cli(tmp_path, capsys):
    p = tmp_path / "t.csv"
    ratios.write_csv(p, table())
    ratios.main([str(p), "--default", "t0", "--compare", "dg", "t1"])
    out = capsys.readouterr().out
    assert '"tuning"' in out and '"best_static"' in out and '"base": "dg"' in out
