"""Benchmark: frequent subgraph mining (MNI support) on GB300 — batched vs plain GPU paths.

One step = one complete mining run of the workload graph (every support evaluation of every
growth level).  Metric: support evaluations per second (whole job), with the wall clock of a
mining run, the graph load time and intersections per second beside it; the batched path is the
headline, and the plain one-pattern-per-launch path, the batched path without sub-pattern pruning
and the batched path with learned matching orders are timed on the same graph with their outputs
checked equal.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gpu|reference] [--workload NAME]
                    [--tuned] [--no-cpu-baseline]

N > 1 runs N independent replicas (one per GPU, launched by torchrun): the path has no data
exchange, so `value` sums all ranks' evaluations over the slowest rank's time ("scaling": "weak").
`--impl reference` times the CPU restatement of the reference algorithm (oracle/tfsm_port, all
host threads) on the same workload, one time-bounded mining run per step; under torchrun only rank
0 runs it.
"""
from __future__ import annotations

import argparse
import json
import os
import re
import statistics
import subprocess
import sys
import tempfile
import threading
import time
from pathlib import Path

if "LOCAL_RANK" in os.environ:  # one replica per GPU: the library reads TFSM_DEVICE
    os.environ.setdefault("TFSM_DEVICE", os.environ["LOCAL_RANK"])

ROOT = Path(__file__).resolve().parent
PKG = ROOT / "t-fsm_gb300"
METRIC = "FSM wall-clock & pattern-support evals/s: batched vs plain GPU, identical output"

CFG2_GEN = dict(n=100000, mean=22, gamma=2.2, max_degree=1400, labels=29, zipf=1.2, elabels=1, seed=1)
CFG4_GEN = dict(n=2000000, mean=20, gamma=2.05, max_degree=50000, labels=50, zipf=1.1, elabels=3, seed=2)
WORKLOADS = {
    "cfg1": dict(gen=dict(n=5000, mean=8, gamma=2.5, max_degree=500, labels=10, zipf=1.0, elabels=1, seed=0),
                 tau=200, max_nodes=4, desc="Chung-Lu 5k vertices / 20k edges, tau=200, maxNodes=4"),
    "cfg2_t9000": dict(gen=CFG2_GEN, tau=9000, max_nodes=5,
                       desc="Chung-Lu 100k vertices / 1.1M edges (gamma 2.2), 29 Zipf(1.2) labels, tau=9000, "
                            "maxNodes=5"),
    "cfg2_t7000": dict(gen=CFG2_GEN, tau=7000, max_nodes=5,
                       desc="Chung-Lu 100k vertices / 1.1M edges, tau=7000, maxNodes=5"),
    "cfg3": dict(gen=CFG2_GEN, tau=5000, max_nodes=6,
                 desc="Chung-Lu 100k vertices / 1.1M edges, tau=5000, maxNodes=6 (batched form)"),
    "cfg4_m4": dict(gen=CFG4_GEN, tau=20000, max_nodes=4,
                    desc="Chung-Lu 2M vertices / 20M edges (gamma 2.05, hubs), 50 Zipf(1.1) labels, 3 edge labels, "
                         "tau=20000, maxNodes=4"),
    "cfg4": dict(gen=CFG4_GEN, tau=20000, max_nodes=5,
                 desc="Chung-Lu 2M vertices / 20M edges (gamma 2.05, hubs), 50 Zipf(1.1) labels, 3 edge labels, "
                      "tau=20000, maxNodes=5"),
}
DEFAULT_WORKLOAD = "cfg4_m4"
L2_NOTE = "flushed between steps (256 MiB write); graph resident in HBM"


def binding():
    import importlib.util

    if "tfsm" in sys.modules:
        return sys.modules["tfsm"]
    spec = importlib.util.spec_from_file_location("tfsm", PKG / "tfsm.py")
    mod = importlib.util.module_from_spec(spec)
    sys.modules["tfsm"] = mod
    spec.loader.exec_module(mod)
    return mod


def ensure_built() -> None:
    sys.path.insert(0, str(PKG))
    import build as pkg_build

    pkg_build.build()


def make_graph(w: dict) -> Path:
    """The workload's .lg file (and its raw host arrays, same prefix), generated once per machine."""
    g = w["gen"]
    tag = "_".join(f"{k}{v}" for k, v in sorted(g.items()))
    path = Path(tempfile.gettempdir()) / f"tfsm_bench_{tag}.lg"
    if not path.exists() or not path.with_suffix(".src").exists():
        tmp = path.with_suffix(".tmp")
        cmd = [str(PKG / "bin" / "gen_lg"), "--out", str(tmp), "--arrays", str(path.with_suffix("")), "--n",
               str(g["n"]), "--mean", str(g["mean"]), "--gamma", str(g["gamma"]), "--max-degree",
               str(g["max_degree"]), "--labels", str(g["labels"]), "--zipf", str(g["zipf"]), "--elabels",
               str(g["elabels"]), "--seed", str(g["seed"])]
        subprocess.run(cmd, check=True, capture_output=True)
        tmp.rename(path)
    return path


def read_arrays(path: Path):
    import numpy as np

    p = path.with_suffix("")
    return (np.fromfile(f"{p}.vlabel", dtype=np.int32), np.fromfile(f"{p}.src", dtype=np.uint32),
            np.fromfile(f"{p}.dst", dtype=np.uint32), np.fromfile(f"{p}.elabel", dtype=np.int32))


def config_of(args, w: dict) -> dict:
    """The workload as both arms report it (the same dict, so the two lines compare directly)."""
    return {"workload": args.workload, "graph": w["desc"], "tau": w["tau"], "max_nodes": w["max_nodes"],
            "l2": L2_NOTE}


class ClockSampler:
    """Samples nvidia-smi clocks and throttle reasons during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.rows: list[list[str]] = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except FileNotFoundError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self) -> dict:
        sm = [float(r[0]) for r in self.rows if len(r) >= 6 and r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in self.rows if len(r) >= 6 and r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows if len(r) >= 6 for i in range(4) if r[2 + i] == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(sm)}


def measured_peak_hbm() -> tuple[float, str]:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        return float(json.loads(p.read_text())["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def profiled_traffic(workload: str) -> float | None:
    """Per-launch DRAM traffic of the search kernel for this workload from the committed ncu summary."""
    p = ROOT / "profiles" / f"k_search_{workload}.md"
    if not p.exists():
        return None
    m = re.search(r"traffic_bytes_per_launch:\s*([0-9.eE+]+)", p.read_text())
    return float(m.group(1)) if m else None


def run_port(graph: Path, w: dict, threads: int, time_limit: float = 0.0, repeat: int = 1) -> list[dict]:
    """The CPU restatement (oracle/tfsm_port): `repeat` mining runs after one load, each stopped
    after `time_limit` seconds of mining when set; per run its mining time and evaluations."""
    port = ROOT / "oracle" / "tfsm_port"
    if not port.exists():
        subprocess.run(["make", "-s", "-C", str(ROOT / "oracle"), "port"], check=True, capture_output=True)
    cmd = [str(port), "-file", str(graph), "-freq", str(w["tau"]), "-maxNodes", str(w["max_nodes"]), "-thread",
           str(threads), "-repeat", str(repeat)]
    if time_limit > 0:
        cmd += ["-time-limit", str(time_limit)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode not in (0, 3):  # 3: the time limit stopped the (last) run
        raise RuntimeError(f"tfsm_port failed: {r.stderr[-2000:]}")
    load_s = float(re.search(r"Loading Graph Time: ([0-9.]+)", r.stdout).group(1))
    if repeat > 1:
        runs = [{"mine_s": float(a), "evals": int(b)}
                for a, b in re.findall(r"\[SAMPLE\] \d+ mine_s ([0-9.]+) evaluations (\d+)", r.stdout)]
    else:
        runs = [{"mine_s": float(re.search(r"Mining Time: ([0-9.]+)", r.stdout).group(1)),
                 "evals": int(re.search(r"# Support Evaluations: (\d+)", r.stdout).group(1))}]
    for x in runs:
        x["load_s"] = load_s
        x["complete"] = time_limit <= 0 or x["mine_s"] < time_limit
    return runs


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("gloo", init_method="env://")
    return world, rank


def barrier(world):
    if world > 1:
        import torch.distributed as dist

        dist.barrier()


def max_over_ranks(world, x: float) -> float:
    if world == 1:
        return x
    import torch
    import torch.distributed as dist

    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(world, x: float) -> float:
    if world == 1:
        return x
    import torch
    import torch.distributed as dist

    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


# Bounded CPU samples: a reference step is one mining run of the workload stopped after this many
# seconds of mining (a complete run on the 2M-vertex graph takes the reference far longer).
REFERENCE_SAMPLE_S = 10.0


def reference_arm(args, w, world, rank):
    if rank != 0:
        return 0
    graph = make_graph(w)
    threads = os.cpu_count() or 1
    runs = run_port(graph, w, threads, REFERENCE_SAMPLE_S, args.warmup + args.steps)[args.warmup:]
    mine_s = sum(r["mine_s"] for r in runs)
    evals = sum(r["evals"] for r in runs)
    value = evals / mine_s
    sample = (f"{args.steps} mining runs of the workload by the CPU restatement of the reference's evaluation on "
              f"{threads} threads, each stopped after {REFERENCE_SAMPLE_S:.0f} s of mining "
              f"({'complete' if all(r['complete'] for r in runs) else 'partial: the early, cheaper levels'}; "
              f"{runs[0]['evals']} support evaluations in the first)")
    line = {
        "metric": METRIC, "impl": "reference", "value": value, "unit": "evals/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * mine_s / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32", "data": "synthetic",
        "config": config_of(args, w),
        "cpu_baseline": {"value": value, "unit": "evals/s", "cores": threads, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": "evals/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "load_s": runs[0]["load_s"],
    }
    print(json.dumps(line), flush=True)
    return 0


# Training graphs of the learned matching order: the shapes of the two smaller configurations,
# seeds 10..12 (never the benchmarked graph), mined by the plain miner with random orders.
TRAINING = [(dict(WORKLOADS["cfg1"]["gen"], seed=s), 200, 4) for s in (10, 11, 12)] + \
           [(dict(CFG2_GEN, seed=s), 9000, 5) for s in (10, 11, 12)]


def training_set(w: dict) -> list:
    """Graphs the cost model learns from: configuration 1 and 2 shapes (seeds 10-12) and, for a
    hub-graph workload (several edge labels or hubs past 10k neighbours), two graphs of the
    workload's own shape at a quarter of its size (seeds 10, 11; tau / 4, at most 4 vertices):
    never the timed graph."""
    g = w["gen"]
    extra = []
    if g["elabels"] > 1 or g["max_degree"] >= 10000:
        small = dict(g, n=g["n"] // 4, max_degree=max(1, g["max_degree"] // 4))
        extra = [(dict(small, seed=s), max(1, w["tau"] // 4), min(4, w["max_nodes"])) for s in (10, 11)]
    return TRAINING + extra


def train_cost_model(tfsm, w: dict):
    import numpy as np

    feats, costs = [], []
    train = training_set(w)
    for k, (gen, tau, mn) in enumerate(train):
        with tfsm.Graph.load(make_graph(dict(gen=gen)), tau) as gt:
            gt.set_order_policy(tfsm.ORDER_RANDOM, seed=k + 1)
            gt.record_orders(True)
            gt.mine(max_nodes=mn, flags=tfsm.FLAG_PLAIN)
            f, c = gt.take_records()
            feats.append(f)
            costs.append(c)
    x, t = np.concatenate(feats), np.concatenate(costs)
    model = tfsm.CostModel(seed=1)
    t0 = time.perf_counter()
    mse = model.train(x, t, epochs=60, batch=64, lr=2e-3, seed=2)
    what = "configuration 1 and 2 shapes, seeds 10-12"
    if len(train) > len(TRAINING):
        what += "; the workload's shape at a quarter of its size, seeds 10-11, tau / 4"
    return model, {"training_records": int(len(x)), "train_mse": mse, "train_s": time.perf_counter() - t0,
                   "training_graphs": what + "; plain miner, random orders"}


def gpu_arm(args, w, world, rank):
    import torch

    tfsm = binding()
    # the plain path is the reference's miner loop around the drop-in evaluation: one engine call
    # per candidate, fixed (GQL) matching order, no sub-pattern pruning (the reference searches
    # every candidate)
    PLAIN = tfsm.FLAG_PLAIN | tfsm.FLAG_NO_SUBPATTERN_PRUNING
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    graph = make_graph(w)
    g = tfsm.Graph.load(graph, w["tau"])
    info = g.info()
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")  # > 129 MB L2
    mn = w["max_nodes"]

    def one_step(flags):
        flush.fill_(1)  # evict the graph and level memory from L2 between timed steps
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        t0 = time.perf_counter()
        e0.record()
        st = g.mine(max_nodes=mn, flags=flags)
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1), time.perf_counter() - t0, st

    def outputs(flags) -> set:
        out = Path(tempfile.mktemp(suffix=".txt"))
        g.mine(max_nodes=mn, flags=flags, results_path=out)
        got = set(tfsm.read_results(out))
        out.unlink()
        return got

    def timed(flags, warm, steps):
        for _ in range(warm):
            one_step(flags)
        runs = [one_step(flags) for _ in range(steps)]
        return sum(r[0] for r in runs) / len(runs), runs

    batched_set = outputs(0)
    identical = outputs(PLAIN) == batched_set
    identical_no_pruning = outputs(tfsm.FLAG_NO_SUBPATTERN_PRUNING) == batched_set

    # ---- the headline: batched path, W warm-up steps, K timed steps ----
    for _ in range(args.warmup):
        one_step(0)
    barrier(world)
    torch.cuda.synchronize()
    ms, wall, stats = [], [], []
    with ClockSampler(local) as clk:
        for _ in range(args.steps):
            a, b, st = one_step(0)
            ms.append(a)
            wall.append(b)
            stats.append(st)
    torch.cuda.synchronize()
    barrier(world)
    step_ms = max_over_ranks(world, sum(ms) / len(ms))
    evals = stats[0]["evaluations"]
    value = sum_over_ranks(world, evals) * 1e3 / step_ms
    isects = stats[0]["intersections"]

    few = max(1, args.steps // 4)
    plain_ms, pruns = timed(PLAIN, 1, few)
    plain_ms = max_over_ranks(world, plain_ms)
    nop_ms, nruns = timed(tfsm.FLAG_NO_SUBPATTERN_PRUNING, 1, few)

    # ---- learned matching orders: a cost model trained on records of other graphs ----
    model, mlp_info = train_cost_model(tfsm, w)
    tuned = None
    try:
        g.set_order_policy(tfsm.ORDER_MODEL, model=model)
        identical_mlp = outputs(0) == batched_set
        mlp_ms, mruns = timed(0, 1, max(1, args.steps // 2))
        g.set_order_policy(tfsm.ORDER_GQL)
        if args.tuned:
            tuned = tuned_arm(args, w, g, tfsm, timed, outputs, batched_set, model)
    finally:
        g.set_order_policy(tfsm.ORDER_GQL)
        model.close()

    # ---- roofline of the dominant kernel (the search): algorithmic bytes / device time ----
    s_ms = sum(st["search_ms"] for st in stats)
    s_bytes = sum(st["search_bytes"] for st in stats)
    s_launch = sum(st["search_launches"] for st in stats)
    achieved = s_bytes / (s_ms * 1e-3) / 1e9 if s_ms > 0 else 0.0
    peak, peak_kind = measured_peak_hbm()

    # ---- end to end through the C ABI from host arrays: prune + upload + mine + read results ----
    vl, src, dst, el = read_arrays(graph)
    e2e_ms, e2e_h2d, e2e_d2h = [], 0, 0
    for i in range(1 + max(1, args.steps // 2)):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        with tfsm.Graph.from_edges(vl, src, dst, el, w["tau"]) as g2:
            st = g2.mine(max_nodes=mn)
            load_h2d = g2.info()["load_h2d_bytes"]
        dt = time.perf_counter() - t0
        if i >= 1:
            e2e_ms.append(dt * 1e3)
            e2e_h2d, e2e_d2h = load_h2d + st["h2d_bytes"], st["d2h_bytes"]
    e2e_step = max_over_ranks(world, sum(e2e_ms) / len(e2e_ms))
    e2e_value = sum_over_ranks(world, evals) * 1e3 / e2e_step

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        r = run_port(graph, w, threads, REFERENCE_SAMPLE_S)[0]
        cpu = {"value": r["evals"] / r["mine_s"], "unit": "evals/s", "cores": threads, "kind": "port",
               "sample": f"one mining run of the workload by the CPU restatement of the reference's evaluation, "
                         f"stopped after {REFERENCE_SAMPLE_S:.0f} s of mining ({r['evals']} support evaluations, "
                         f"{'complete' if r['complete'] else 'the early, cheaper levels only'})"}

    launches = sum(st["init_launches"] + st["refine_launches"] + st["search_launches"] for st in stats)
    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "evals/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": step_ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "u32", "data": "synthetic", "config": config_of(args, w),
            "path": "batched (one engine call per growth level while calls take under 2 ms, smaller calls after a "
                    f"slower one); searches split into tasks after {g.options()['step_budget']} chunk steps",
            "parallelism": "replicas" if world > 1 else "single GPU",
            "graph_vertices": info["n_vertices"], "graph_edges": info["n_edges"],
            "load_s": info["load_ms"] / 1e3, "wall_clock_mine_s": step_ms / 1e3,
            "intersections_per_s": isects * 1e3 / step_ms,
            "frequent_patterns": stats[0]["frequent"], "support_evaluations": evals,
            "decided_by_subpattern": stats[0]["pruned"], "decided_by_filters": stats[0]["by_filter"],
            "searches": stats[0]["searches"], "split_searches": stats[0]["split_searches"],
            "plain": {"value": evals * 1e3 / plain_ms, "ms_per_step": plain_ms,
                      "engine_calls": pruns[0][2]["engine_calls"],
                      "path": "reference miner loop + drop-in evaluation: one engine call per candidate, GQL order, "
                              "no sub-pattern pruning"},
            "batched_over_plain": plain_ms / step_ms, "identical_output": identical,
            "batched_no_subpattern_pruning": {"value": evals * 1e3 / nop_ms, "ms_per_step": nop_ms,
                                              "over_plain": plain_ms / nop_ms,
                                              "identical_output": identical_no_pruning},
            "batched_mlp": dict(mlp_info, value=evals * 1e3 / mlp_ms, ms_per_step=mlp_ms,
                                over_batched=step_ms / mlp_ms, identical_output=identical_mlp,
                                search_ms_per_step=sum(r[2]["search_ms"] for r in mruns) / len(mruns),
                                steps_per_run=mruns[0][2]["steps"]),
            "batched_autotuned": tuned,
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": profiled_traffic(args.workload),
                         "kernel": "k_search (+k_split)", "peak_kind": peak_kind,
                         "algorithmic_bytes_per_launch": s_bytes / max(1, s_launch),
                         "avg_launch_ms": s_ms / max(1, s_launch)},
            "kernel_ms_per_step": {k: sum(st[k] for st in stats) / len(stats) for k in
                                   ("init_ms", "refine_ms", "search_ms")},
            "host_extend_ms_per_step": sum(st["extend_ms"] for st in stats) / len(stats),
            "cpu_baseline": cpu,
            "e2e": {"value": e2e_value, "unit": "evals/s", "h2d_bytes_per_step": e2e_h2d,
                    "d2h_bytes_per_step": e2e_d2h, "ms_per_step": e2e_step},
            "gpu_launches": launches,
            "clocks": clk.summary(),
            "wall_ms_per_step": 1e3 * sum(wall) / len(wall),
        }
        print(json.dumps(line), flush=True)
    g.close()
    same = identical and identical_no_pruning and identical_mlp and (tuned is None or tuned["identical_output"])
    return 0 if same else 1


def tuned_arm(args, w, g, tfsm, timed, outputs, batched_set, model) -> dict:
    """Batched path with the knobs the autotuner picks per level on a held-out graph of the same
    shape (seed + 10), then applied to the benchmarked graph; alone and with the learned orders."""
    import importlib.util

    spec = importlib.util.spec_from_file_location("autotune", PKG / "autotune.py")
    at = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(at)
    held_out = dict(w, gen=dict(w["gen"], seed=w["gen"]["seed"] + 10))
    t0 = time.perf_counter()
    with tfsm.Graph.load(make_graph(held_out), w["tau"]) as gt:
        best = at.tune(gt, w["max_nodes"], repeats=2)
    tune_s = time.perf_counter() - t0
    try:
        for lv, o in best.items():
            g.set_level_options(int(lv), o)
        identical = outputs(0) == batched_set
        ms, _ = timed(0, 1, max(1, args.steps // 2))
        g.set_order_policy(tfsm.ORDER_MODEL, model=model)
        identical_mlp = outputs(0) == batched_set
        ms_mlp, _ = timed(0, 1, max(1, args.steps // 2))
    finally:
        g.set_order_policy(tfsm.ORDER_GQL)
        g.set_level_options(0, None)
    evals = g.mine(max_nodes=w["max_nodes"])["evaluations"]
    return {"value": evals * 1e3 / ms, "ms_per_step": ms, "identical_output": identical, "tune_s": tune_s,
            "tuned_on": "held-out graph of the same shape (seed + 10)",
            "with_learned_orders": {"value": evals * 1e3 / ms_mlp, "ms_per_step": ms_mlp,
                                    "identical_output": identical_mlp, "over_tuned": ms / ms_mlp},
            "levels": {str(k): v for k, v in best.items()}}


def main() -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["gpu", "reference"], default="gpu")
    ap.add_argument("--workload", choices=sorted(WORKLOADS), default=DEFAULT_WORKLOAD)
    ap.add_argument("--tuned", action="store_true", help="also time the autotuned path (tuned on a held-out graph)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    args = ap.parse_args()
    args.warmup = max(3, args.warmup)
    ensure_built()
    world, rank = dist_setup()
    w = WORKLOADS[args.workload]
    if args.impl == "reference":
        return reference_arm(args, w, world, rank)
    return gpu_arm(args, w, world, rank)


if __name__ == "__main__":
    sys.exit(main())
