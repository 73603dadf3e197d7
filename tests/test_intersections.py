"""Set intersections of the search step: merge and probe forms against the oracle.

A search step intersects the anchor's adjacency slice with the label range of every other
backward neighbour.  The kernel merges a range that is at most `isect_ratio` times the anchor's
(streamed with 128-bit loads through a shared-memory tile, the cursor moving chunk by chunk) and
probes a longer one by binary search from a moving start (the galloping form); the reference
switches between merge and galloping at a size ratio of 50 (intersection/computesetintersection.cpp:
9-44).  The gadget graphs below make those ranges long and skewed on purpose: every gadget is two
adjacent hubs a (label 0) and b (label 1) whose leaves (label 2) are na and nb vertices with
`shared` of them adjacent to both, so triangle and 4-cycle searches intersect lists whose size
ratio is just below, at and above 50, far above, equal, and disjoint.  Exact MNI of every candidate
pattern of the gadget graph must equal the oracle's (the CPU restatement of the reference's
engine) for every merge/probe switch ratio and team size.

CPU: the oracle's own hybrid intersection equals std::set_intersection; the emulated kernels (ASan)
on a lighter gadget graph.  GPU: the full gadget graph through the C ABI.
"""
from __future__ import annotations

import os
import random
import subprocess
import sys

import pytest

from conftest import ROOT
from golden_io import read_mni

GADGETS = [  # (na, nb, shared)
    (1, 50, 1), (2, 99, 2), (2, 100, 1), (2, 101, 2), (10, 490, 7), (10, 500, 10), (10, 510, 3), (20, 1000, 13),
    (40, 40, 17), (64, 64, 64), (5, 3000, 4), (3, 3, 0), (30, 60, 0), (1, 1, 1), (7, 350, 5),
]
# the emulated kernels run every collective as a thread rendezvous: a lighter set, 3-vertex patterns
SMALL_GADGETS = [(1, 50, 1), (2, 101, 2), (4, 200, 3), (3, 3, 0), (30, 60, 0), (40, 40, 17), (9, 9, 9)]
TAU = 1


def write_gadget_graph(path, gadgets=GADGETS, seed: int = 5) -> None:
    """Gadgets, leaf ids shuffled so that ranges start at every alignment."""
    rnd = random.Random(seed)
    labels, edges = [], []
    for na, nb, shared in gadgets:
        a, b = len(labels), len(labels) + 1
        labels += [0, 1]
        edges.append((a, b))
        leaves = list(range(len(labels), len(labels) + na + nb - shared))
        labels += [2] * len(leaves)
        for i, v in enumerate(leaves):
            if i < na:
                edges.append((a, v))
            if i < shared or i >= na:
                edges.append((b, v))
    # a few label-3 vertices tie gadget leaves together (longer patterns with several backward
    # neighbours at the last depth)
    for _ in range(40):
        c = len(labels)
        labels.append(3)
        for v in rnd.sample([i for i, l in enumerate(labels[:-1]) if l == 2], 3):
            edges.append((c, v))
    perm = list(range(len(labels)))
    rnd.shuffle(perm)
    inv = [0] * len(perm)
    for new, old in enumerate(perm):
        inv[old] = new
    nl = [labels[perm[i]] for i in range(len(labels))]
    ne = sorted({(min(inv[x], inv[y]), max(inv[x], inv[y])) for x, y in edges})
    deg = [0] * len(nl)
    for x, y in ne:
        deg[x] += 1
        deg[y] += 1
    lines = [f"t {len(nl)} {len(ne)}"] + [f"v {i} {l} {deg[i]}" for i, l in enumerate(nl)]
    lines += [f"e {x} {y} 1" for x, y in ne]
    path.write_text("\n".join(lines) + "\n")


def oracle_mni(graph, max_nodes, d):
    """{pattern key: exact MNI} from the oracle for every candidate of the mining run, and the same
    as a golden-format file."""
    port = ROOT / "oracle" / "tfsm_port"
    if not port.exists():
        subprocess.run(["make", "-s", "-C", str(ROOT / "oracle"), "port"], check=True)
    sup = d / "port.sup"
    subprocess.run([str(port), "-file", str(graph), "-freq", str(TAU), "-maxNodes", str(max_nodes), "-exact", "1",
                    "-thread", str(os.cpu_count() or 4), "-supports", str(sup)], check=True, capture_output=True)
    mni = d / "gadget.mni.txt"
    mni.write_text("".join(line[2:] + "\n" for line in sup.read_text().splitlines()))
    return mni, read_mni(mni)


@pytest.fixture(scope="module")
def gadget(tmp_path_factory):
    d = tmp_path_factory.mktemp("gadget")
    graph = d / "gadget.lg"
    write_gadget_graph(graph)
    mni, want = oracle_mni(graph, 4, d)
    assert len(want) > 50 and any(len(k.split()) >= 4 for k in want)
    return graph, mni, want


@pytest.fixture(scope="module")
def small_gadget(tmp_path_factory):
    d = tmp_path_factory.mktemp("small_gadget")
    graph = d / "gadget.lg"
    write_gadget_graph(graph, SMALL_GADGETS)
    mni, want = oracle_mni(graph, 3, d)
    assert any(len(k.split()) >= 3 for k in want)  # triangles: two backward neighbours
    return graph, mni, want


def test_oracle_intersection_equals_set_intersection(tmp_path):
    exe = tmp_path / "isect_check"
    subprocess.run(["g++", "-std=c++17", "-O2", "-pthread", "-I", str(ROOT / "t-fsm_gb300" / "csrc"),
                    str(ROOT / "tests" / "native" / "isect_check.cpp"), "-o", str(exe)], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and r.stdout.startswith("ok"), r.stdout


@pytest.fixture(scope="module")
def abi_emu():
    sys.path.insert(0, str(ROOT / "tests" / "simt"))
    import build_emu

    return build_emu.build("asan", "abi")


@pytest.mark.parametrize("ratio,lanes", [(1, 32), (50, 32), (1000000, 32), (4, 8), (1000000, 8)])
def test_emulated_intersections_match_oracle(abi_emu, small_gadget, ratio, lanes):
    """The kernels' exact sources under the SIMT emulation (ASan/UBSan): every count equals the
    oracle's, with the merge form for every range (huge ratio), for almost none (ratio 1), and the
    reference's switch (50)."""
    graph, mni, _ = small_gadget
    env = dict(os.environ, ASAN_OPTIONS="detect_leaks=1:abort_on_error=1", UBSAN_OPTIONS="halt_on_error=1",
               ISECT_RATIO=str(ratio), SEARCH_LANES=str(lanes))
    r = subprocess.run([str(abi_emu), str(graph), str(TAU), str(mni)], capture_output=True, text=True, timeout=900,
                       env=env)
    assert r.returncode == 0, r.stdout[-3000:] + r.stderr[-3000:]
    assert r.stdout.strip().splitlines()[-1].startswith("ok")


@pytest.mark.gpu
@pytest.mark.parametrize("lanes", [8, 32])
@pytest.mark.parametrize("ratio", [1, 4, 16, 50, 64, 1000000])
def test_gpu_intersections_match_oracle(tfsm, gadget, ratio, lanes):
    graph, _, want = gadget
    keys = list(want)
    with tfsm.Graph.load(graph, TAU) as g:
        g.set_options(isect_ratio=ratio, search_lanes=lanes)
        res = g.evaluate([tfsm.parse_key(k) for k in keys], flags=tfsm.FLAG_EXACT)
        assert [r.mni for r in res] == [want[k] for k in keys]
        st = g.mine(max_nodes=4)
        assert st["intersections"] > 0
