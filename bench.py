"""Benchmark: frequent subgraph mining (MNI support) on GB300 — batched vs plain GPU paths.

One step = one complete mining run of the workload graph (every support evaluation of every
growth level).  Metric: support evaluations per second (whole job), with wall-clock per mining
run; the batched path is the headline, the plain one-pattern-per-launch path and the equality of
their outputs are reported beside it.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gpu|reference] [--workload NAME]

N > 1 runs N independent replicas (one per GPU, launched by torchrun): the path has no data
exchange, so `value` sums all ranks' evaluations over the slowest rank's time ("scaling": "weak").
`--impl reference` times the CPU restatement of the reference algorithm (oracle/tfsm_port, all
host threads) on the same workload; under torchrun only rank 0 runs it.
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

WORKLOADS = {
    # plain GPU drop-in at medium scale (the headline workload)
    "cfg2_t9000": dict(gen=dict(n=100000, mean=22, gamma=2.2, max_degree=1400, labels=29, zipf=1.2, elabels=1,
                                seed=1), tau=9000, max_nodes=5,
                       desc="Chung-Lu 100k vertices / 1.1M edges (gamma 2.2), 29 Zipf(1.2) labels, tau=9000, "
                            "maxNodes=5"),
    "cfg2_t7000": dict(gen=dict(n=100000, mean=22, gamma=2.2, max_degree=1400, labels=29, zipf=1.2, elabels=1,
                                seed=1), tau=7000, max_nodes=5,
                       desc="Chung-Lu 100k vertices / 1.1M edges, tau=7000, maxNodes=5"),
    "cfg3": dict(gen=dict(n=100000, mean=22, gamma=2.2, max_degree=1400, labels=29, zipf=1.2, elabels=1,
                          seed=1), tau=5000, max_nodes=6,
                 desc="Chung-Lu 100k vertices / 1.1M edges, tau=5000, maxNodes=6 (batched form)"),
    "cfg1": dict(gen=dict(n=5000, mean=8, gamma=2.5, max_degree=500, labels=10, zipf=1.0, elabels=1, seed=0),
                 tau=200, max_nodes=4, desc="Chung-Lu 5k vertices / 20k edges, tau=200, maxNodes=4"),
    "cfg4": dict(gen=dict(n=2000000, mean=20, gamma=2.05, max_degree=50000, labels=50, zipf=1.1, elabels=3,
                          seed=2), tau=20000, max_nodes=5,
                 desc="Chung-Lu 2M vertices / 20M edges (gamma 2.05, hubs), 50 labels, 3 edge labels, "
                      "tau=20000, maxNodes=5"),
}


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
    g = w["gen"]
    tag = "_".join(f"{k}{v}" for k, v in sorted(g.items()))
    path = Path(tempfile.gettempdir()) / f"tfsm_bench_{tag}.lg"
    if not path.exists():
        tmp = path.with_suffix(".tmp")
        cmd = [str(PKG / "bin" / "gen_lg"), "--out", str(tmp), "--n", str(g["n"]), "--mean", str(g["mean"]),
               "--gamma", str(g["gamma"]), "--max-degree", str(g["max_degree"]), "--labels", str(g["labels"]),
               "--zipf", str(g["zipf"]), "--elabels", str(g["elabels"]), "--seed", str(g["seed"])]
        subprocess.run(cmd, check=True, capture_output=True)
        tmp.rename(path)
    return path


def read_arrays(path: Path):
    import numpy as np

    vl, es = [], []
    with open(path) as f:
        for line in f:
            if line[0] == "v":
                vl.append(int(line.split()[2]))
            elif line[0] == "e":
                es.append(line)
    e = np.array([list(map(int, l.split()[1:4])) for l in es], dtype=np.int64).reshape(-1, 3)
    return (np.array(vl, dtype=np.int32), e[:, 0].astype(np.uint32), e[:, 1].astype(np.uint32),
            e[:, 2].astype(np.int32))


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


def profiled_traffic() -> float | None:
    """Per-launch DRAM traffic of k_search from the committed ncu summary, if present."""
    p = ROOT / "profiles" / "k_search_cfg2_t9000.md"
    if not p.exists():
        return None
    m = re.search(r"traffic_bytes_per_launch:\s*([0-9.eE+]+)", p.read_text())
    return float(m.group(1)) if m else None


def run_port(graph: Path, w: dict, threads: int) -> dict:
    port = ROOT / "oracle" / "tfsm_port"
    if not port.exists():
        subprocess.run(["make", "-s", "-C", str(ROOT / "oracle"), "port"], check=True, capture_output=True)
    r = subprocess.run([str(port), "-file", str(graph), "-freq", str(w["tau"]), "-maxNodes", str(w["max_nodes"]),
                        "-thread", str(threads)], capture_output=True, text=True, check=True)
    mine_s = float(re.search(r"Mining Time: ([0-9.]+)", r.stdout).group(1))
    total_s = float(re.search(r"Total Elapsed Time: ([0-9.]+)", r.stdout).group(1))
    evals = int(re.search(r"# Support Evaluations: (\d+)", r.stdout).group(1))
    freq = int(re.search(r"# Frequent Patterns: (\d+)", r.stdout).group(1))
    return {"mine_s": mine_s, "total_s": total_s, "evals": evals, "frequent": freq}


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


def reference_arm(args, w, world, rank):
    if rank != 0:
        return 0
    graph = make_graph(w)
    threads = os.cpu_count() or 1
    for _ in range(args.warmup):
        run_port(graph, w, threads)
    runs = [run_port(graph, w, threads) for _ in range(args.steps)]
    mine_s = sum(r["mine_s"] for r in runs)
    value = sum(r["evals"] for r in runs) / mine_s
    line = {
        "metric": METRIC, "impl": "reference", "value": value, "unit": "evals/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * mine_s / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32", "data": "synthetic",
        "config": {"workload": args.workload, "graph": w["desc"], "tau": w["tau"], "max_nodes": w["max_nodes"]},
        "cpu_baseline": {"value": value, "unit": "evals/s", "cores": threads, "kind": "port",
                         "sample": f"{args.steps} complete mining runs of the workload ({runs[0]['evals']} support "
                                   f"evaluations, {runs[0]['frequent']} frequent patterns each)"},
        "e2e": {"value": value, "unit": "evals/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "wall_clock_mine_s": mine_s / args.steps,
    }
    print(json.dumps(line), flush=True)
    return 0


def mlp_arm(args, w, g, tfsm, one_step, batched_results: Path) -> dict:
    import numpy as np

    feats, costs = [], []
    for k in range(3):
        wk = dict(w, gen=dict(w["gen"], seed=w["gen"]["seed"] + 10 + k))
        with tfsm.Graph.load(make_graph(wk), w["tau"]) as gt:
            gt.set_order_policy(tfsm.ORDER_RANDOM, seed=k + 1)
            gt.record_orders(True)
            gt.mine(max_nodes=w["max_nodes"], flags=tfsm.FLAG_PLAIN)
            f, c = gt.take_records()
            feats.append(f)
            costs.append(c)
    x, t = np.concatenate(feats), np.concatenate(costs)
    model = tfsm.CostModel(seed=1)
    t0 = time.perf_counter()
    mse = model.train(x, t, epochs=60, batch=64, lr=2e-3, seed=2)
    train_s = time.perf_counter() - t0
    g.set_order_policy(tfsm.ORDER_MODEL, model=model)
    try:
        outm = Path(tempfile.mktemp(suffix=".m.txt"))
        g.mine(max_nodes=w["max_nodes"], results_path=outm)
        identical = set(tfsm.read_results(outm)) == set(tfsm.read_results(batched_results))
        for _ in range(args.warmup):
            one_step(0)
        runs = [one_step(0) for _ in range(args.steps)]
    finally:
        g.set_order_policy(tfsm.ORDER_GQL)
    ms = sum(r[0] for r in runs) / len(runs)
    st = runs[0][2]
    return model, {"value": st["evaluations"] * 1e3 / ms, "ms_per_step": ms, "identical_output": identical,
            "search_ms_per_step": sum(r[2]["search_ms"] for r in runs) / len(runs),
            "steps_per_run": st["steps"], "training_records": int(len(x)), "train_mse": mse,
            "train_s": train_s, "training_graphs": "workload shape, seeds +10..+12, plain miner, random orders"}


def tuned_arm(args, w, g, tfsm, one_step, batched_results: Path, model) -> dict:
    """Batched path with the knobs the autotuner picks per level for this workload; then the
    same with the learned matching orders as well."""
    import importlib.util

    spec = importlib.util.spec_from_file_location("autotune", PKG / "autotune.py")
    at = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(at)
    t0 = time.perf_counter()
    best = at.tune(g, w["max_nodes"], repeats=2)
    tune_s = time.perf_counter() - t0
    try:
        outt = Path(tempfile.mktemp(suffix=".t.txt"))
        g.mine(max_nodes=w["max_nodes"], results_path=outt)
        identical = set(tfsm.read_results(outt)) == set(tfsm.read_results(batched_results))
        for _ in range(args.warmup):
            one_step(0)
        runs = [one_step(0) for _ in range(args.steps)]
        g.set_order_policy(tfsm.ORDER_MODEL, model=model)
        outb = Path(tempfile.mktemp(suffix=".tm.txt"))
        g.mine(max_nodes=w["max_nodes"], results_path=outb)
        identical_both = set(tfsm.read_results(outb)) == set(tfsm.read_results(batched_results))
        for _ in range(args.warmup):
            one_step(0)
        runs_both = [one_step(0) for _ in range(args.steps)]
    finally:
        g.set_level_options(0, None)
        g.set_order_policy(tfsm.ORDER_GQL)
    ms = sum(r[0] for r in runs) / len(runs)
    ms_both = sum(r[0] for r in runs_both) / len(runs_both)
    evals = runs[0][2]["evaluations"]
    return {"value": evals * 1e3 / ms, "ms_per_step": ms, "identical_output": identical,
            "tune_s": tune_s, "levels": {str(k): v for k, v in best.items()},
            "with_learned_orders": {"value": evals * 1e3 / ms_both, "ms_per_step": ms_both,
                                    "identical_output": identical_both}}


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

    def one_step(flags):
        flush.fill_(1)  # evict the graph and level memory from L2 between timed steps
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        t0 = time.perf_counter()
        e0.record()
        st = g.mine(max_nodes=w["max_nodes"], flags=flags)
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1), time.perf_counter() - t0, st

    # identical output of the batched and plain paths
    outb, outp = Path(tempfile.mktemp(suffix=".b.txt")), Path(tempfile.mktemp(suffix=".p.txt"))
    g.mine(max_nodes=w["max_nodes"], results_path=outb)
    g.mine(max_nodes=w["max_nodes"], flags=PLAIN, results_path=outp)
    identical = set(tfsm.read_results(outb)) == set(tfsm.read_results(outp))

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

    # plain path, same workload
    for _ in range(max(1, args.warmup // 2)):
        one_step(PLAIN)
    pruns = [one_step(PLAIN) for _ in range(max(1, args.steps // 2))]
    pms = [r[0] for r in pruns]
    plain_ms = max_over_ranks(world, sum(pms) / len(pms))

    # batched + learned matching orders: a cost model trained on records that the plain miner logs
    # (random connected orders) on three training graphs of the workload's shape (other seeds)
    model, mlp = mlp_arm(args, w, g, tfsm, one_step, outb)
    try:
        tuned = tuned_arm(args, w, g, tfsm, one_step, outb, model)
    finally:
        model.close()

    # roofline of the dominant kernel (the search): algorithmic bytes / device time
    s_ms = sum(st["search_ms"] for st in stats)
    s_bytes = sum(st["search_bytes"] for st in stats)
    s_launch = sum(st["search_launches"] for st in stats)
    achieved = s_bytes / (s_ms * 1e-3) / 1e9 if s_ms > 0 else 0.0
    peak, peak_kind = measured_peak_hbm()
    traffic = profiled_traffic()

    # end to end through the C ABI with host buffers: prune + upload + mine + read results
    vl, src, dst, el = read_arrays(graph)
    e2e_ms, e2e_h2d, e2e_d2h = [], 0, 0
    for i in range(args.warmup + args.steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        with tfsm.Graph.from_edges(vl, src, dst, el, w["tau"]) as g2:
            st = g2.mine(max_nodes=w["max_nodes"])
            dev_bytes = g2.info()["device_bytes"]
        dt = time.perf_counter() - t0
        if i >= args.warmup:
            e2e_ms.append(dt * 1e3)
            e2e_h2d, e2e_d2h = dev_bytes + st["h2d_bytes"], st["d2h_bytes"]
    e2e_step = max_over_ranks(world, sum(e2e_ms) / len(e2e_ms))
    e2e_value = sum_over_ranks(world, evals) * 1e3 / e2e_step

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        r = run_port(graph, w, threads)
        cpu = {"value": r["evals"] / r["mine_s"], "unit": "evals/s", "cores": threads, "kind": "port",
               "sample": f"one complete mining run of the workload ({r['evals']} support evaluations, "
                         f"{r['mine_s']:.2f} s)"}

    launches = sum(st["init_launches"] + st["refine_launches"] + st["search_launches"] for st in stats)
    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "evals/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": step_ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "u32", "data": "synthetic",
            "config": {"workload": args.workload, "graph": w["desc"], "tau": w["tau"], "max_nodes": w["max_nodes"],
                       "path": "batched (one engine call per growth level while calls take under 2 ms, smaller calls after a slower one)",
                       "l2": "flushed between steps (256 MiB write); graph resident in HBM",
                       "parallelism": "replicas" if world > 1 else "single GPU",
                       "graph_vertices": info["n_vertices"], "graph_edges": info["n_edges"]},
            "wall_clock_mine_s": step_ms / 1e3,
            "frequent_patterns": stats[0]["frequent"], "support_evaluations": evals,
            "decided_by_subpattern": stats[0]["pruned"], "decided_by_filters": stats[0]["by_filter"],
            "plain": {"value": evals * 1e3 / plain_ms, "ms_per_step": plain_ms,
                      "engine_calls": pruns[0][2]["engine_calls"],
                      "path": "reference miner loop + drop-in evaluation: one engine call per candidate, GQL order, "
                              "no sub-pattern pruning"},
            "batched_over_plain": plain_ms / step_ms, "identical_output": identical,
            "batched_mlp": mlp,
            "batched_autotuned": tuned,
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic, "kernel": "k_search (+k_split)",
                         "peak_kind": peak_kind,
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
    same = (identical and mlp["identical_output"] and tuned["identical_output"]
            and tuned["with_learned_orders"]["identical_output"])
    return 0 if same else 1


def main() -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["gpu", "reference"], default="gpu")
    ap.add_argument("--workload", choices=sorted(WORKLOADS), default="cfg2_t9000")
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
