"""Host pattern growth under AddressSanitizer / UndefinedBehaviorSanitizer (CPU).

The canonical check keeps the reference's forward-extension ordering, which is not a strict weak
ordering with several edge labels (parallel/canonical.h:40-44).  With it, std::map::operator[] can
hand out the map's end(); the check must drop that projection instead of writing into the map's
header (on the 2M-vertex graph with three edge labels, the level with 5-edge patterns hit this
and the host process died).  Every canonical pattern over two vertex labels and three edge labels
is extended up to six edges, checked again and decomposed into sub-patterns, on several threads
(the unfixed check overflows its stack frame on this enumeration within seconds).
"""
from __future__ import annotations

import subprocess

from conftest import ROOT


def test_canonical_check_stays_in_bounds_with_three_edge_labels(tmp_path):
    exe = tmp_path / "canonical_enum"
    subprocess.run(["g++", "-std=c++17", "-O1", "-g", "-fsanitize=address,undefined", "-fno-sanitize-recover=undefined",
                    "-pthread", "-I", str(ROOT / "t-fsm_gb300" / "csrc"),
                    str(ROOT / "tests" / "native" / "canonical_enum.cpp"), "-o", str(exe)], check=True)
    r = subprocess.run([str(exe), "8", "2", "6"], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0 and r.stdout.startswith("ok"), r.stdout[-2000:] + r.stderr[-4000:]
