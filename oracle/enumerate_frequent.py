"""ORACLE — test infrastructure only.  The frequent-pattern set of a graph up to `max_nodes` vertices
from the definition alone: every connected labelled pattern whose MNI support reaches tau, found
level by level (patterns of k + 1 edges grown from the frequent patterns of k edges by one edge,
kept when every connected sub-pattern with one edge fewer is frequent: MNI support is
anti-monotone) and decided by oracle/mni_brute (-decide 1).  No DFS codes and no gSpan rules: the
output is the set of isomorphism classes, so it checks the completeness of a miner's output as
well as its soundness.  Patterns are simple graphs (one edge per vertex pair), as the reference's.

usage: python oracle/enumerate_frequent.py -file G.lg -freq TAU -maxNodes N [-out keys.txt]
                                           [-compare results.txt | -compare-keys keys.txt]
  prints the number of frequent patterns per edge count; with -compare (a grami_results.txt-format
  file) or -compare-keys (DFS-code keys, one pattern per line), also whether that file holds
  exactly the same isomorphism classes (exit status 1 when not).
"""
from __future__ import annotations

import argparse
import itertools
import subprocess
import sys
import tempfile
from collections import Counter
from pathlib import Path

HERE = Path(__file__).resolve().parent
BRUTE = HERE / "mni_brute"


def canon(labels: tuple, edges: frozenset) -> tuple:
    """Smallest (labels, sorted edges) over all vertex orders: an isomorphism-class key."""
    n = len(labels)
    best = None
    for perm in itertools.permutations(range(n)):  # new vertex i is old vertex perm[i]
        lab = tuple(labels[perm[i]] for i in range(n))
        pos = {old: new for new, old in enumerate(perm)}
        es = tuple(sorted((min(pos[a], pos[b]), max(pos[a], pos[b]), el) for a, b, el in edges))
        key = (lab, es)
        if best is None or key < best:
            best = key
    return best


def to_codes(key: tuple) -> str:
    """The pattern as a valid DFS code sequence "a,b,la,el,lb ..." (not necessarily the minimal one):
    the first code is (0,1), every later one either adds the next vertex id (forward) or joins two
    vertices already numbered (backward), as tfsm_evaluate_support and the checkers accept."""
    labels, edges = key
    a0, b0, el0 = edges[0]
    num = {a0: 0, b0: 1}
    codes = [(0, 1, labels[a0], el0, labels[b0])]
    rest = list(edges[1:])
    while rest:
        for e in rest:
            x, y, el = e
            if x in num and y in num:
                codes.append((num[x], num[y], labels[x], el, labels[y]))
            elif x in num or y in num:
                old, new = (x, y) if x in num else (y, x)
                num[new] = len(num)
                codes.append((num[old], num[new], labels[old], el, labels[new]))
            else:
                continue
            rest.remove(e)
            break
    return " ".join(f"{a},{b},{la},{el},{lb}" for a, b, la, el, lb in codes)


def from_results(path: Path) -> set:
    """Isomorphism-class keys of a grami_results.txt file."""
    out, v, e = set(), [], []
    for line in path.read_text().splitlines() + ["====="]:
        t = line.split()
        if not t:
            continue
        if t[0].startswith("=====") or t[0] == "t":
            if v:
                out.add(canon(tuple(v), frozenset((int(a), int(b), int(l)) for a, b, l in e)))
            v, e = [], []
        elif t[0] == "v":
            v.append(int(t[2]))
        elif t[0] == "e":
            e.append((t[1], t[2], t[3]))
    return out


def from_keys(path: Path) -> set:
    """Isomorphism-class keys of a file of DFS-code keys ("a,b,la,el,lb ..." per line)."""
    out = set()
    for line in path.read_text().splitlines():
        codes = [tuple(int(x) for x in c.split(",")) for c in line.split()]
        if not codes:
            continue
        lab = {}
        for a, b, la, el, lb in codes:
            lab[a], lab[b] = la, lb
        out.add(canon(tuple(lab[i] for i in range(len(lab))), frozenset((a, b, el) for a, b, _, el, _ in codes)))
    return out


def sub_patterns(labels: tuple, edges: tuple):
    """The connected components with an edge left after removing one edge (each must be frequent)."""
    for drop in edges:
        rest = [e for e in edges if e != drop]
        n = len(labels)
        adj = {i: set() for i in range(n)}
        for a, b, _ in rest:
            adj[a].add(b)
            adj[b].add(a)
        seen_all = set()
        for s in range(n):
            if s in seen_all:
                continue
            comp, stack = {s}, [s]
            while stack:
                for y in adj[stack.pop()]:
                    if y not in comp:
                        comp.add(y)
                        stack.append(y)
            seen_all |= comp
            ce = [e for e in rest if e[0] in comp]
            if not ce:
                continue
            idx = {old: new for new, old in enumerate(sorted(comp))}
            yield canon(tuple(labels[i] for i in sorted(comp)),
                        frozenset((idx[a], idx[b], el) for a, b, el in ce))


def decide(graph: Path, tau: int, keys: list) -> set:
    """The keys whose MNI support reaches tau (one checker run for the whole list)."""
    if not keys:
        return set()
    with tempfile.TemporaryDirectory() as tmp:
        plist = Path(tmp) / "p.txt"
        codes = [to_codes(k) for k in keys]
        plist.write_text("".join(c + "\n" for c in codes))
        r = subprocess.run([str(BRUTE), "-file", str(graph), "-freq", str(tau), "-patterns", str(plist), "-decide",
                            "1"], capture_output=True, text=True, check=True)
    got = {}
    for line in r.stdout.splitlines():
        if " | " in line:
            c, counts = line.split(" | ")
            got[c] = min(int(x) for x in counts.split()) >= tau
    return {k for k, c in zip(keys, codes) if got[c]}


def frequent_set(graph: Path, tau: int, max_nodes: int, log=print) -> set:
    """Isomorphism-class keys of every connected pattern of at most max_nodes vertices whose MNI
    support on `graph` reaches tau."""
    if not BRUTE.exists():
        subprocess.run(["make", "-s", "-C", str(HERE), "brute"], check=True)
    vcount, elabels = Counter(), set()
    with open(graph) as f:
        for line in f:
            t = line.split()
            if len(t) >= 3 and t[0] == "v":
                vcount[int(t[2])] += 1
            elif len(t) >= 4 and t[0] == "e":
                elabels.add(int(t[3]))
    vlabels = sorted(x for x, c in vcount.items() if c >= tau)
    elabels = sorted(elabels)
    level = sorted({canon((la, lb), frozenset({(0, 1, el)})) for la in vlabels for lb in vlabels for el in elabels})
    frequent = set()
    k = 1
    while level:
        freq_k = decide(graph, tau, level)
        log(f"{k} edges: {len(level)} candidates, {len(freq_k)} frequent")
        frequent |= freq_k
        cands = set()
        for labels, edges in freq_k:
            n = len(labels)
            present = {(x, y) for x, y, _ in edges}
            ext = []
            if n < max_nodes:
                ext += [(labels + (L,), edges + ((i, n, el),)) for i in range(n) for L in vlabels for el in elabels]
            ext += [(labels, edges + ((i, j, el),)) for i in range(n) for j in range(i + 1, n)
                    if (i, j) not in present for el in elabels]
            for lab2, ed2 in ext:
                c = canon(lab2, frozenset(ed2))
                if c in cands or c in frequent:
                    continue
                if all(s in frequent for s in sub_patterns(*c)):
                    cands.add(c)
        level = sorted(cands)
        k += 1
    return frequent


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("-file", required=True)
    ap.add_argument("-freq", type=int, required=True)
    ap.add_argument("-maxNodes", type=int, required=True)
    ap.add_argument("-compare", help="grami_results.txt-format file")
    ap.add_argument("-compare-keys", dest="compare_keys", help="file of DFS-code keys, one pattern per line")
    ap.add_argument("-out", help="write the frequent patterns here, one key per line")
    a = ap.parse_args()
    frequent = frequent_set(Path(a.file), a.freq, a.maxNodes, log=lambda m: print(m, flush=True))
    print("frequent patterns:", len(frequent), flush=True)
    if a.out:
        Path(a.out).write_text("".join(to_codes(k) + "\n" for k in sorted(frequent)))
    if a.compare or a.compare_keys:
        mined = from_results(Path(a.compare)) if a.compare else from_keys(Path(a.compare_keys))
        print("compare:", "identical" if mined == frequent else
              f"differ: {len(mined - frequent)} reported but not frequent, {len(frequent - mined)} frequent but "
              "not reported")
        sys.exit(0 if mined == frequent else 1)


if __name__ == "__main__":
    main()
