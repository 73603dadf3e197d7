"""Autotuner of the engine's speed-only knobs, per growth level, keyed on the graph's label and
degree statistics.

The knobs (lanes per search, work-item size, merge/galloping switch ratio, teams per hub
search, sharing budget and slice, refinement rounds) never
change a result, only the work's shape; the best values depend on the pattern size (the growth
level) and on the graph's degree and label distribution.  `tune()` runs complete mining runs of
the caller's workload, one knob at a time (coordinate descent), and keeps for every level the
value with the lowest engine time of that level (best of `repeats` runs).  The table is cached
in a JSON file under a signature of the graph (vertex and edge counts, label count, mean and
maximum degree, each bucketed by powers of two) plus tau and maxNodes, so a similar graph reuses
it; `apply()` loads it onto a graph handle (tfsm_set_level_options).
"""
from __future__ import annotations

import json
import math
from pathlib import Path
from typing import Callable

# candidate values per knob, in the order they are tuned; the first is the engine default
SPACE = [
    ("search_lanes", [8, 32]),
    ("chunk_words", [1, 2]),
    ("isect_ratio", [16, 4, 64]),
    ("hub_parts", [4, 1, 2, 8]),  # teams that search one hub candidate's first depth together
    ("step_budget", [16, 8, 32, 64]),
    ("split_slice", [64, 32, 128]),
    ("refine_rounds", [1, 2, 0]),
    ("refine_scope", [1, 0]),
]


def signature(info: dict, tau: int, max_nodes: int) -> str:
    """Graph key: counts and degree statistics bucketed by powers of two."""
    n, m = info["n_vertices"], info["n_edges"]
    mean = 2.0 * m / max(1, n)

    def b(x):
        return int(math.floor(math.log2(max(1.0, float(x)))))

    return (f"n{b(n)}-m{b(m)}-l{info['n_frequent_vertex_labels']}-el{info['n_frequent_edge_labels']}"
            f"-d{b(mean)}-D{b(info['max_degree'])}-t{b(tau)}-k{max_nodes}")


def tune_levels(run: Callable[[dict], list[float]], levels: int, repeats: int = 2,
                space=SPACE) -> tuple[dict[int, dict], dict]:
    """Coordinate descent with a per-level choice.

    run(per_level_options) mines once with {level: {knob: value}} applied and returns the engine
    time of every level (index = level).  Returns ({level: options}, log)."""
    best = {lv: {} for lv in range(1, levels + 1)}
    log = {"runs": 0, "knobs": {}}
    for knob, values in space:
        times = {}  # value -> per-level best time
        for v in values:
            trial = {lv: dict(best[lv], **{knob: v}) for lv in best}
            t = None
            for _ in range(repeats):
                r = run(trial)
                log["runs"] += 1
                t = r if t is None else [min(a, c) for a, c in zip(t, r)]
            times[v] = t
        choice = {}
        for lv in best:
            vals = [(times[v][lv] if lv < len(times[v]) else math.inf, i, v) for i, v in enumerate(values)]
            _, _, v = min(vals)  # ties: the earlier (default) value
            best[lv][knob] = v
            choice[lv] = v
        log["knobs"][knob] = {"choice": choice, "times": {str(v): t for v, t in times.items()}}
    return best, log


def tune(graph, max_nodes: int, flags: int = 0, repeats: int = 2, cache: str | Path | None = None) -> dict[int, dict]:
    """Tunes `graph` (a tfsm.Graph) for mining with `max_nodes` and returns {level: options};
    the result is applied to the handle and, with `cache`, stored under the graph's signature."""
    base = graph.mine(max_nodes=max_nodes, flags=flags)
    levels = int(base["levels"])

    def run(per_level):
        for lv, o in per_level.items():
            graph.set_level_options(lv, o)
        st = graph.mine(max_nodes=max_nodes, flags=flags)
        return list(st["level_ms"])

    best, log = tune_levels(run, levels, repeats)
    graph.set_level_options(0, None)
    for lv, o in best.items():
        graph.set_level_options(lv, o)
    if cache:
        p = Path(cache)
        table = json.loads(p.read_text()) if p.exists() else {}
        table[signature(graph.info(), graph.tau, max_nodes)] = {str(k): v for k, v in best.items()}
        p.write_text(json.dumps(table, indent=1, sort_keys=True))
    return best


def apply(graph, max_nodes: int, cache: str | Path) -> bool:
    """Applies a cached table for this graph's signature; False when there is none."""
    p = Path(cache)
    if not p.exists():
        return False
    table = json.loads(p.read_text()).get(signature(graph.info(), graph.tau, max_nodes))
    if not table:
        return False
    graph.set_level_options(0, None)
    for lv, o in table.items():
        graph.set_level_options(int(lv), o)
    return True
