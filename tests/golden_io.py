"""Readers for the reference miners' outputs and the golden fixtures (test infrastructure)."""
from __future__ import annotations

import hashlib
from pathlib import Path


def _key(vlabels: list[int], edges: list[tuple[int, int, int]]) -> str:
    return " ".join(f"{a},{b},{vlabels[a]},{l},{vlabels[b]}" for a, b, l in edges)


def read_results(path) -> list[str]:
    """Pattern keys of a grami_results.txt file (serial/grami.h:622-635 format), in file order."""
    pats, v, e = [], [], []
    for line in Path(path).read_text().splitlines():
        t = line.split()
        if not t:
            continue
        if t[0].startswith("====="):
            if v:
                pats.append(_key(v, e))
            v, e = [], []
        elif t[0] == "v":
            v.append(int(t[2]))
        elif t[0] == "e":
            e.append((int(t[1]), int(t[2]), int(t[3])))
    if v:
        pats.append(_key(v, e))
    return pats


def read_parallel_stdout(text: str) -> set[str]:
    """Patterns printed by the parallel reference build (parallel/comper.h:1027-1031, 1095-1101).

    Its threads print without a lock, so marker lines may interleave; each pattern's `v`/`e`
    lines come from one string and stay together: a block is a run of v lines then e lines.
    """
    pats: set[str] = set()
    v: list[int] = []
    e: list[tuple[int, int, int]] = []
    for line in text.splitlines():
        t = line.split()
        if t and t[0] == "v" and len(t) == 3:
            if e:
                pats.add(_key(v, e))
                v, e = [], []
            v.append(int(t[2]))
        elif t and t[0] == "e" and len(t) == 4:
            e.append((int(t[1]), int(t[2]), int(t[3])))
        else:
            if v and e:
                pats.add(_key(v, e))
            v, e = [], []
    if v and e:
        pats.add(_key(v, e))
    return pats


def read_mni(path) -> dict[str, list[int]]:
    out = {}
    for line in Path(path).read_text().splitlines():
        if " | " not in line:
            continue
        k, c = line.split(" | ")
        out[k.strip()] = [int(x) for x in c.split()]
    return out


def graph_checksum(path) -> str:
    return hashlib.sha256(Path(path).read_bytes()).hexdigest()[:16]
