"""The multi-threaded loader used by the C ABI (host/lg_fast.hpp) builds exactly the graph of the
plain restatement of the reference loader (host/lg_graph.hpp): pruned vertices and edges, sorted
adjacency, frequent labels and the 1-edge pattern table, and the same errors for malformed input.
CPU only."""
from __future__ import annotations

import subprocess

import pytest

from conftest import CASES, GOLDEN, ROOT


@pytest.fixture(scope="module")
def checker(tmp_path_factory):
    out = tmp_path_factory.mktemp("loader") / "loader_check"
    subprocess.run(["g++", "-std=c++17", "-O2", "-pthread", "-I", str(ROOT / "t-fsm_gb300" / "csrc"),
                    str(ROOT / "tests" / "native" / "loader_check.cpp"), "-o", str(out)], check=True)
    return out


FILE_CASES = [n for n, c in CASES.items() if "file" in c]


@pytest.mark.parametrize("case", FILE_CASES)
@pytest.mark.parametrize("threads", [1, 7])
def test_fast_loader_equals_reference_loader_on_golden_graphs(checker, case, threads):
    c = CASES[case]
    r = subprocess.run([str(checker), str(GOLDEN / c["file"]), str(c["tau"]), str(threads)], capture_output=True,
                       text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr


@pytest.mark.parametrize("seed", range(6))
@pytest.mark.parametrize("tau", [1, 40, 400])
def test_fast_loader_equals_reference_loader_on_random_multigraphs(checker, seed, tau):
    r = subprocess.run([str(checker), "--random", str(seed), str(tau)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr


@pytest.mark.parametrize("text", [
    "t # 0\nv 0 1\nv 1 2\ne 0 1 3\n",
    "t # 0\nv 0 1\nv 2 2\n",             # ids out of order
    "t # 0\nv 0 1\nx 1 2\n",             # unknown line kind
    "t # 0\nv 0 1\nv 1 1\ne 0 1\n",      # malformed edge line
    "t # 0\nv 0 1\ne 0 5 1\n",           # endpoint out of range
    "v 0 1\n\nv 1 1\n  e 0 1 2\r\n",
])
def test_fast_parser_same_result_and_errors(checker, tmp_path, text):
    f = tmp_path / "g.lg"
    f.write_text(text)
    r = subprocess.run([str(checker), str(f), "1", "4"], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0, r.stdout + r.stderr


def test_fast_parser_multi_chunk_file(checker, tmp_path):
    """A file of several MB is parsed in chunks by several threads; same graph, same errors."""
    import random

    rnd = random.Random(5)
    n = 60000
    lines = ["t # 0"] + [f"v {i} {rnd.randrange(6)}" for i in range(n)]
    lines += [f"e {rnd.randrange(n)} {rnd.randrange(n)} {rnd.randrange(3)}" for _ in range(300000)]
    f = tmp_path / "big.lg"
    f.write_text("\n".join(lines) + "\n")
    assert f.stat().st_size > 3 << 20
    for threads in ("1", "5", "16"):
        r = subprocess.run([str(checker), str(f), "50", threads], capture_output=True, text=True, timeout=120)
        assert r.returncode == 0 and "same" in r.stdout, r.stdout + r.stderr
    # a malformed line deep inside a later chunk: same message (with its line number) from both
    lines[250000] = "e 1 2"
    f.write_text("\n".join(lines) + "\n")
    r = subprocess.run([str(checker), str(f), "50", "16"], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and "line 250001" in r.stdout, r.stdout + r.stderr


def test_subpattern_key_is_an_isomorphism_invariant(tmp_path):
    """canonical_key (sub-pattern pruning): equal for relabelled copies, one key per class."""
    exe = tmp_path / "subpattern_check"
    subprocess.run(["g++", "-std=c++17", "-O2", "-I", str(ROOT / "t-fsm_gb300" / "csrc"),
                    str(ROOT / "tests" / "native" / "subpattern_check.cpp"), "-o", str(exe)], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
