"""Autotuner of the speed-only knobs (t-fsm_gb300/autotune.py).

CPU: the per-level coordinate descent picks, for every level, the value with the lowest time
(the default on ties) on a synthetic cost table; the signature buckets graph statistics.
GPU: tuning a real graph keeps the mined pattern set, and a cached table is applied to a new handle.
"""
from __future__ import annotations

import importlib.util
import sys

import pytest

from conftest import CASES, PKG, golden_pattern_set
from golden_io import read_results

spec = importlib.util.spec_from_file_location("autotune", PKG / "autotune.py")
autotune = importlib.util.module_from_spec(spec)
sys.modules["autotune"] = autotune
spec.loader.exec_module(autotune)


def test_per_level_choice_on_synthetic_costs():
    # level 1 prefers chunk_words 2, level 2 prefers step_budget 64; everything else is flat
    def run(per_level):
        t = [0.0] * 4
        for lv, o in per_level.items():
            t[lv] = 10.0
            if lv == 1 and o.get("chunk_words") == 2:
                t[lv] -= 3
            if lv == 2 and o.get("step_budget") == 64:
                t[lv] -= 2
            if lv == 3 and o.get("split_slice") == 128:
                t[lv] += 5
        return t

    best, log = autotune.tune_levels(run, 3, repeats=1)
    assert best[1]["chunk_words"] == 2 and best[2]["chunk_words"] == 1
    assert best[2]["step_budget"] == 64 and best[1]["step_budget"] == 16
    assert best[3]["split_slice"] == 64  # default kept on ties and where others are worse
    assert log["runs"] == sum(len(v) for _, v in autotune.SPACE)


def test_signature_buckets_statistics():
    info = dict(n_vertices=47039, n_edges=255090, n_frequent_vertex_labels=9, n_frequent_edge_labels=1,
                max_degree=1400)
    s1 = autotune.signature(info, 9000, 5)
    s2 = autotune.signature(dict(info, n_vertices=50000, n_edges=260000), 9000, 5)
    assert s1 == s2
    assert autotune.signature(info, 9000, 6) != s1


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["cfg1", "el3"])
def test_tuned_options_keep_results(tfsm, case_graph, case, tmp_path):
    c = CASES[case]
    cache = tmp_path / "tuning.json"
    with tfsm.Graph.load(case_graph(case), c["tau"]) as g:
        best = autotune.tune(g, c["max_nodes"], repeats=1, cache=cache)
        assert best
        out = tmp_path / "r.txt"
        g.mine(max_nodes=c["max_nodes"], results_path=out)
        assert set(read_results(out)) == golden_pattern_set(case)
    with tfsm.Graph.load(case_graph(case), c["tau"]) as g:
        assert autotune.apply(g, c["max_nodes"], cache)
        out = tmp_path / "r2.txt"
        st = g.mine(max_nodes=c["max_nodes"], results_path=out)
        assert set(read_results(out)) == golden_pattern_set(case)
        assert sum(st["level_ms"]) > 0
