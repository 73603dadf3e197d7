"""Generate the golden fixtures of the parity tests from the reference T-FSM itself.

Runs only where the reference sources exist (oracle/Makefile reads them from the tree its REF
variable names): `make -C oracle ref harness port brute REF=<tree>` builds
  oracle/_ref/serial_run    the reference serial miner   (serial/Makefile flags)
  oracle/_ref/parallel_run  the reference parallel miner (parallel/Makefile flags)
  oracle/_ref/mni_harness   exact MNI domains from the reference's GMatchEngine
  oracle/tfsm_port          the CPU restatement (used here only to list candidate patterns)
  oracle/mni_brute          exact MNI domains from the definition by plain backtracking

For every case it writes, next to this script:
  <case>.patterns.txt  frequent patterns (DFS-code keys, sorted) from the serial build; the
                       parallel build must agree, else the script stops
  <case>.mni.txt       "<key> | c0 c1 ..." exact per-vertex MNI domain sizes from the harness, for
                       frequent and infrequent candidates alike
and cases.json with the graph recipe (generator arguments or a committed graph file), tau,
maxNodes and the graph checksum.  For the pattern samples of MNI_SAMPLES it writes
<sample>.brute.txt (oracle/mni_brute) and, where the sample asks for it, <sample>.mni.txt (the
harness) for the patterns that <sample>.keys.txt lists.

usage: python tests/golden/make_golden.py [case or sample ...]
"""
from __future__ import annotations

import json
import os
import random
import re
import subprocess
import sys
import tempfile
from pathlib import Path

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
REF = ROOT / "oracle" / "_ref"
GEN = ROOT / "t-fsm_gb300" / "bin" / "gen_lg"
PORT = ROOT / "oracle" / "tfsm_port"
BRUTE = ROOT / "oracle" / "mni_brute"
sys.path.insert(0, str(ROOT / "tests"))
from golden_io import read_parallel_stdout, read_results, graph_checksum  # noqa: E402

# Synthetic graphs of the benchmark configurations (Chung-Lu degrees, Zipf labels).
GEN_CASES = {
    "cfg1": dict(gen=dict(n=5000, mean=8, gamma=2.5, max_degree=500, labels=10, zipf=1.0, elabels=1, seed=0),
                 tau=200, max_nodes=4, mni="all"),
    "el3": dict(gen=dict(n=3000, mean=8, gamma=2.3, max_degree=300, labels=5, zipf=1.0, elabels=3, seed=7),
                tau=60, max_nodes=4, mni="every5"),
    "cfg2_t9000": dict(gen=dict(n=100000, mean=22, gamma=2.2, max_degree=1400, labels=29, zipf=1.2, elabels=1,
                                seed=1), tau=9000, max_nodes=5, mni="all"),
    "cfg2_t7000": dict(gen=dict(n=100000, mean=22, gamma=2.2, max_degree=1400, labels=29, zipf=1.2, elabels=1,
                                seed=1), tau=7000, max_nodes=5, mni="all", serial=False),
    # the batched workload: the config-2 graph at tau 5000 with up to 6 pattern vertices (the
    # 5,000-vertex graph has no label frequent at tau 5000)
    "cfg3": dict(gen=dict(n=100000, mean=22, gamma=2.2, max_degree=1400, labels=29, zipf=1.2, elabels=1,
                          seed=1), tau=5000, max_nodes=6, mni="none", serial=False, threads=0),
    # the held-out graph of the learned-order evaluation: config-2 shape, seed 99, tau 20000
    "cfg5_seed99": dict(gen=dict(n=100000, mean=22, gamma=2.2, max_degree=1400, labels=29, zipf=1.2, elabels=1,
                                 seed=99), tau=20000, max_nodes=5, mni="all"),
    # the hub-heavy 2M-vertex graph (3 edge labels) with up to 3 pattern vertices: the largest
    # maxNodes the reference's parallel build completes here in about an hour on all cores
    "cfg4_m3": dict(gen=dict(n=2000000, mean=20, gamma=2.05, max_degree=50000, labels=50, zipf=1.1, elabels=3,
                             seed=2), tau=20000, max_nodes=3, mni="none", serial=False, threads=0),
}

# Exact MNI of listed patterns on a case's graph, without a mining run: <name>.keys.txt holds the
# patterns (DFS-code keys), the harness writes <name>.mni.txt.  cfg4_sample: 4- and 5-vertex
# patterns of the 2M-vertex hub graph, beyond what the reference's miners finish here (maxNodes 4
# and 5); its keys are every 190th frequent 4-vertex tree, every 90th 4-vertex cycle and every
# 8000th 5-vertex pattern of the GPU miner's maxNodes-5 output on that graph (output order), plus
# every 400th 4-vertex tree from the 8th with its last vertex relabelled to the rarest frequent
# label (infrequent candidates).  The reference's engine decides every one of them.
# cfg4_wide: 392 more patterns of the same graph, for the definition checker only (the reference's
# engine needs minutes per pattern there): every 10th frequent 4-vertex pattern from the 4th and
# every 1500th 5-vertex pattern from the 6th of the same outputs, and every 50th 4-vertex pattern
# from the 12th whose last code is a forward edge, its new vertex relabelled to label 8, 7 or 6
# (the first that gives no frequent pattern's code), none of them in cfg4_sample.
# cfg4_m4: every pattern the GPU miner reports on that graph at maxNodes 4 (3 412; its
# grami_results.txt keys, sorted; oracle/tfsm_port reports the same set in about 33 minutes on 8
# cores), for the definition checker: each must have support >= tau.
MNI_SAMPLES = {"cfg4_sample": dict(graph_case="cfg4_m3", reference=True),
               "cfg4_wide": dict(graph_case="cfg4_m3", reference=False),
               "cfg4_m4": dict(graph_case="cfg4_m3", reference=False),
               # every 100th (from the first) of the sorted 5-vertex keys the GPU miner reports
               # there at maxNodes 5 (423 of 42 277)
               "cfg4_m5_sample": dict(graph_case="cfg4_m3", reference=False),
               # the 358 patterns of at most 4 vertices frequent there by the definition
               # (oracle/enumerate_frequent.py) that the reference's growth never produces (the
               # cfg4_m4 set lacks them), in oracle/enumerate_frequent.py's key order
               "cfg4_unreached": dict(graph_case="cfg4_m3", reference=False)}

# Small hand-made graphs for edge cases, written by make_small_graphs().
FILE_CASES = {
    "clique": dict(file="graphs/clique.lg", tau=3, max_nodes=5, mni="all"),
    "star_hub": dict(file="graphs/star_hub.lg", tau=4, max_nodes=4, mni="all"),
    "quirk_elabels": dict(file="graphs/quirk_elabels.lg", tau=3, max_nodes=5, mni="all"),
    "no_edges": dict(file="graphs/no_edges.lg", tau=1, max_nodes=4, mni="all"),
    "no_frequent": dict(file="graphs/no_frequent.lg", tau=50, max_nodes=4, mni="all"),
    "tau1_small": dict(file="graphs/tau1_small.lg", tau=1, max_nodes=4, mni="all"),
    # patterns of up to 23 vertices (maxNodes unbounded): three copies of a 22-vertex path with
    # alternating labels and a chord closing a 4-cycle
    "long_paths": dict(file="graphs/long_paths.lg", tau=3, max_nodes=-1, mni="all"),
}


def write_lg(path: Path, labels: list[int], edges: list[tuple[int, int, int]]) -> None:
    lines = [f"t {len(labels)} {len(edges)}"]
    deg = [0] * len(labels)
    for a, b, _ in edges:
        deg[a] += 1
        deg[b] += 1
    lines += [f"v {i} {l} {deg[i]}" for i, l in enumerate(labels)]
    lines += [f"e {a} {b} {l}" for a, b, l in edges]
    path.write_text("\n".join(lines) + "\n")


def make_small_graphs() -> None:
    g = HERE / "graphs"
    g.mkdir(exist_ok=True)
    rnd = random.Random(20240611)
    # clique: four disjoint K5's with labels 0/1 -> many automorphisms and backward edges
    labels, edges = [], []
    for c in range(4):
        base = len(labels)
        labels += [0, 0, 1, 1, 0]
        edges += [(base + i, base + j, 1) for i in range(5) for j in range(i + 1, 5)]
    write_lg(g / "clique.lg", labels, edges)
    # star_hub: two hubs joined to many leaves, leaves form a sparse ring -> hub-rooted searches
    labels = [0, 0] + [1 + (i % 2) for i in range(200)]
    edges = []
    for i in range(200):
        edges.append((0, 2 + i, 1))
        if i % 3 == 0:
            edges.append((1, 2 + i, 1))
        if i + 1 < 200 and i % 4 != 3:
            edges.append((2 + i, 3 + i, 1))
    edges.append((0, 1, 1))
    write_lg(g / "star_hub.lg", labels, edges)
    # quirk_elabels: small random graph with 3 edge labels and 3 vertex labels, dense enough for
    # 4-5 vertex patterns with mixed edge labels (exercises the canonical-check ordering)
    n = 40
    labels = [rnd.randrange(3) for _ in range(n)]
    es = set()
    while len(es) < 110:
        a, b = rnd.randrange(n), rnd.randrange(n)
        if a != b:
            es.add((min(a, b), max(a, b)))
    edges = [(a, b, 1 + rnd.randrange(3)) for a, b in sorted(es)]
    write_lg(g / "quirk_elabels.lg", labels, edges)
    # no_edges: labelled vertices only
    write_lg(g / "no_edges.lg", [i % 3 for i in range(30)], [])
    # no_frequent: every label rarer than tau=50
    n = 60
    labels = [i % 6 for i in range(n)]
    edges = [(i, (i * 7 + 3) % n, 1) for i in range(n) if i < (i * 7 + 3) % n]
    write_lg(g / "no_frequent.lg", labels, edges)
    # tau1_small: tau = 1, every pattern present at least once is frequent
    labels = [0, 1, 0, 1, 2, 0, 2]
    edges = [(0, 1, 1), (1, 2, 1), (2, 3, 1), (3, 0, 1), (0, 4, 1), (4, 5, 1), (5, 6, 1), (2, 6, 1)]
    write_lg(g / "tau1_small.lg", labels, edges)


def gen_args(p: dict) -> list[str]:
    return ["--n", str(p["n"]), "--mean", str(p["mean"]), "--gamma", str(p["gamma"]), "--max-degree",
            str(p["max_degree"]), "--labels", str(p["labels"]), "--zipf", str(p["zipf"]), "--elabels",
            str(p["elabels"]), "--seed", str(p["seed"])]


def run(cmd, cwd=None, timeout=None) -> subprocess.CompletedProcess:
    r = subprocess.run([str(c) for c in cmd], cwd=cwd, capture_output=True, text=True, timeout=timeout)
    if r.returncode != 0:
        raise RuntimeError(f"{cmd} failed: {r.stdout[-2000:]} {r.stderr[-2000:]}")
    return r


def make_mni_sample(name: str) -> None:
    """<name>.mni.txt (samples marked `reference`): the harness on every pattern of
    <name>.keys.txt, the keys split over all cores (one harness process each, every process loads
    the graph); <name>.brute.txt: the definition checker on the same patterns."""
    spec = GEN_CASES[MNI_SAMPLES[name]["graph_case"]]
    keys = [k for k in (HERE / f"{name}.keys.txt").read_text().splitlines() if k.strip()]
    with tempfile.TemporaryDirectory() as tmp:
        tmp = Path(tmp)
        graph = tmp / "g.lg"
        run([GEN, "--out", graph, *gen_args(spec["gen"])])
        parts = min(len(keys), os.cpu_count() or 4) if MNI_SAMPLES[name]["reference"] else 0
        procs = []
        for i in range(parts):
            plist = tmp / f"pats{i}.txt"
            plist.write_text("".join(k + "\n" for k in keys[i::parts]))
            procs.append(subprocess.Popen([str(REF / "mni_harness"), "-file", str(graph), "-freq", str(spec["tau"]),
                                           "-patterns", str(plist)], stdout=subprocess.PIPE, text=True))
        got = {}
        for p in procs:
            out, _ = p.communicate(timeout=7200)
            if p.returncode != 0:
                sys.exit(f"{name}: mni_harness failed")
            for ln in out.splitlines():
                if " | " in ln:
                    got[ln.split(" | ")[0]] = ln
        missing = [k for k in keys if k not in got]
        if parts and missing:
            sys.exit(f"{name}: no result for {len(missing)} patterns, e.g. {missing[0]}")
        if parts:
            (HERE / f"{name}.mni.txt").write_text("".join(got[k] + "\n" for k in keys))
        # the same patterns through the definition checker (oracle/mni_brute.cpp)
        plist = tmp / "all.txt"
        plist.write_text("".join(k + "\n" for k in keys))
        b = run([BRUTE, "-file", graph, "-freq", spec["tau"], "-patterns", plist], timeout=7200)
        brute = {ln.split(" | ")[0]: ln for ln in b.stdout.splitlines() if " | " in ln}
        if [k for k in keys if k not in brute]:
            sys.exit(f"{name}: the definition checker skipped patterns")
        (HERE / f"{name}.brute.txt").write_text("".join(brute[k] + "\n" for k in keys))
    differ = [k for k in keys if k in got and got[k] != brute[k]]
    print(name, len(keys), "patterns;", len(differ), "where the reference engine differs from the definition",
          flush=True)


def main(names: list[str]) -> None:
    for tool in (REF / "serial_run", REF / "parallel_run", REF / "mni_harness", PORT, BRUTE, GEN):
        if not tool.exists():
            sys.exit(f"missing {tool}: run `make -C oracle ref harness port brute REF=<tree>` and "
                     "t-fsm_gb300/build.py first")
    make_small_graphs()
    cases_path = HERE / "cases.json"
    cases = json.loads(cases_path.read_text()) if cases_path.exists() else {}
    todo = {**GEN_CASES, **FILE_CASES}
    for name in [n for n in names or list(MNI_SAMPLES) if n in MNI_SAMPLES]:
        make_mni_sample(name)
    for name in [n for n in names if n not in MNI_SAMPLES] if names else list(todo):
        spec = todo[name]
        with tempfile.TemporaryDirectory() as tmp:
            tmp = Path(tmp)
            if "gen" in spec:
                graph = tmp / "g.lg"
                run([GEN, "--out", graph, *gen_args(spec["gen"])])
            else:
                graph = HERE / spec["file"]
            tau, mn = spec["tau"], spec["max_nodes"]
            ser = None
            if spec.get("serial", True):
                sdir = tmp / "serial"
                sdir.mkdir()
                run([REF / "serial_run", "-file", graph, "-freq", tau, "-maxNodes", mn], cwd=sdir)
                ser = sorted(read_results(sdir / "grami_results.txt"))
            # one thread by default: the parallel build prints patterns from several threads without
            # a lock, which can garble its stdout; the task-based code path is the same.  Long cases
            # use every core (threads=0) and must then reproduce the build's own pattern count.
            threads = spec.get("threads", 1) or (os.cpu_count() or 4)
            pr = run([REF / "parallel_run", "-file", graph, "-freq", tau, "-thread", threads, "-maxNodes", mn],
                     cwd=tmp)
            par = sorted(read_parallel_stdout(pr.stdout))
            m = re.search(r"# Frequent Patterns: (\d+)", pr.stdout)
            n_one_edge = None
            if ser is not None:
                multi = sorted(k for k in ser if " " in k)
                if multi != par:
                    sys.exit(f"{name}: serial and parallel reference builds disagree")
                pats = ser
            else:
                pats = par  # parallel prints multi-edge patterns only: add 1-edge ones from the port
                port_out = tmp / "port.txt"  # (mined to 2 vertices: the 1-edge patterns are all it gives)
                run([PORT, "-file", graph, "-freq", tau, "-maxNodes", 2 if int(mn) < 0 else min(int(mn), 2), "-thread",
                     os.cpu_count() or 4, "-out", port_out])
                one_edge = sorted(k for k in read_results(port_out) if " " not in k)
                pats = sorted(one_edge + par)
                n_one_edge = len(one_edge)
            if m and n_one_edge is not None and int(m.group(1)) != len(pats):
                sys.exit(f"{name}: parsed {len(pats)} patterns, the parallel build counted {m.group(1)}")
            (HERE / f"{name}.patterns.txt").write_text("".join(k + "\n" for k in pats))
            mni_lines = 0
            if spec["mni"] != "none":
                sup = tmp / "port.sup"
                run([PORT, "-file", graph, "-freq", tau, "-maxNodes", mn, "-thread", os.cpu_count() or 4,
                     "-supports", sup])
                keys = [line.split(" | ")[0][2:] for line in sup.read_text().splitlines()]
                if spec["mni"] == "every5":
                    keys = keys[::5]
                plist = tmp / "pats.txt"
                plist.write_text("".join(k + "\n" for k in keys))
                if keys:
                    h = run([REF / "mni_harness", "-file", graph, "-freq", tau, "-patterns", plist], timeout=7200)
                    lines = [ln for ln in h.stdout.splitlines() if " | " in ln]
                else:
                    lines = []
                (HERE / f"{name}.mni.txt").write_text("".join(ln + "\n" for ln in lines))
                mni_lines = len(lines)
            rec = {"tau": tau, "max_nodes": mn, "n_patterns": len(pats), "n_mni": mni_lines,
                   "checksum": graph_checksum(graph), "serial_checked": ser is not None,
                   "parallel_threads": threads}
            rec.update({"gen": spec["gen"]} if "gen" in spec else {"file": spec["file"]})
            cases[name] = rec
            print(name, rec, flush=True)
        cases_path.write_text(json.dumps(cases, indent=1, sort_keys=True) + "\n")


if __name__ == "__main__":
    main(sys.argv[1:])
