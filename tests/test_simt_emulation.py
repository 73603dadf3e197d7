"""The CUDA kernels' exact sources run on the CPU under a SIMT emulation (tests/simt/) with
AddressSanitizer + UndefinedBehaviorSanitizer: every global/shared access in bounds, no UB, warp
collectives executed uniformly (a divergent collective deadlocks the emulated warp and is reported
with each lane's source line), and results equal to the reference on small graphs — including the
hub-splitting path forced on every search.  Test infrastructure only; the product has no CPU path.
"""
from __future__ import annotations

import os
import subprocess
import sys

import pytest

from conftest import CASES, GOLDEN, ROOT, golden_pattern_set
from golden_io import read_results

sys.path.insert(0, str(ROOT / "tests" / "simt"))

SMALL = ["tau1_small", "clique", "star_hub", "quirk_elabels"]


@pytest.fixture(scope="module")
def emu():
    import build_emu

    return build_emu.build("asan")


OPTS = {"default": [],
        # every search splits at its first chunk step; split tasks of one position each
        "split": ["-step-budget", "1", "-split-slice", "1", "-chunk-words", "1"],
        # every search's first depth is split at once into four tasks
        "hub": ["-hub-span", "0", "-hub-parts", "4", "-split-slice", "1"],
        "no_split": ["-no-split"],
        "merge_all": ["-isect-ratio", "1000000", "-step-budget", "2"],
        "probe_all": ["-isect-ratio", "1"],
        "no_refine": ["-refine-rounds", "0"],
        "refine_all": ["-refine-scope", "0", "-refine-rounds", "2"],
        "plain": ["-plain", "-refine-rounds", "1"], "exact": ["-exact"], "batch3": ["-max-batch", "3"],
        "random_orders": ["-random-orders", "7", "-step-budget", "2"],
        "lanes8": ["-search-lanes", "8"],
        "lanes4": ["-search-lanes", "4"],
        "lanes4_split": ["-search-lanes", "4", "-step-budget", "1", "-split-slice", "1"],
        "lanes8_split": ["-search-lanes", "8", "-step-budget", "1", "-split-slice", "1"],
        "lanes8_exact": ["-search-lanes", "8", "-exact", "-step-budget", "1", "-split-slice", "1"],
        "rank_window2": ["-rank-window", "2", "-step-budget", "2"],
        # every emulated call is slower than 1 us: calls shrink to 4 patterns after the first
        "adaptive_calls": ["-call-ms", "0.001"]}
# (the quirk case's many-call variants are the slowest to emulate; its other variants cover it)
RUNS = [(c, o) for c in SMALL for o in OPTS if not (o in ("plain", "batch3") and c == "quirk_elabels")]
RUNS += [(c, "tiny_buffers") for c in ("clique", "star_hub", "quirk_elabels")]
# patterns of up to 23 vertices: the whole-warp search with 32-vertex state (the emulated split
# rounds of the smaller levels are slow, so these runs do not split)
OPTS["no_split_exact"] = ["-no-split", "-exact"]
RUNS += [("long_paths", o) for o in ("no_split", "no_split_exact")]
# with TFSM_SPLIT_CAPACITY=5: claims straddle the end, searches are set aside and retried by later
# passes, the last pass finishes them in place
OPTS["tiny_buffers"] = OPTS["split"]


@pytest.mark.parametrize("case,opt", RUNS)
def test_emulated_kernels_match_reference(emu, case, opt, tmp_path):
    opts = OPTS[opt]
    c = CASES[case]
    out = tmp_path / "res.txt"
    # emulated kernels run on the host cores: keep the host growth (which overlaps them) small
    env = dict(os.environ, ASAN_OPTIONS="detect_leaks=1:abort_on_error=1", UBSAN_OPTIONS="halt_on_error=1",
               TFSM_HOST_THREADS="3")
    if opt == "tiny_buffers":
        env["TFSM_SPLIT_CAPACITY"] = "5"
    r = subprocess.run([str(emu), "-file", str(GOLDEN / c["file"]), "-freq", str(c["tau"]), "-maxNodes",
                        str(c["max_nodes"]), "-out", str(out), *opts, "-call-ms", "0"], capture_output=True,
                       text=True, timeout=600,
                       env=env)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-4000:]
    assert set(read_results(out)) == golden_pattern_set(case)


@pytest.fixture(scope="module")
def abi_emu():
    import build_emu

    return build_emu.build("asan", "abi")


@pytest.mark.parametrize("case", SMALL)
def test_emulated_level_calls_with_parent_domains_match_golden_mni(abi_emu, case):
    """tfsm_evaluate_level, level by level with exact MNI: every pattern whose DFS-code prefix was
    evaluated by the previous call starts from the prefix's kept domains, and every count equals the
    reference's; bad parents (not a sub-pattern, index out of range, another graph) are rejected."""
    c = CASES[case]
    env = dict(os.environ, ASAN_OPTIONS="detect_leaks=1:abort_on_error=1", UBSAN_OPTIONS="halt_on_error=1")
    r = subprocess.run([str(abi_emu), str(GOLDEN / c["file"]), str(c["tau"]), str(GOLDEN / f"{case}.mni.txt")],
                       capture_output=True, text=True, timeout=600, env=env)
    assert r.returncode == 0, r.stdout[-3000:] + r.stderr[-3000:]
    last = r.stdout.strip().splitlines()[-1]
    assert last.startswith("ok"), last
    assert int(last.split("with_parent=")[1].split()[0]) > 0


def test_emulated_mining_is_race_free_under_thread_sanitizer(tmp_path):
    """Host growth runs on a helper thread and the host workers while the engine calls run; under
    ThreadSanitizer (emulated kernels included) no race is reported and the result is the
    reference's.  Calls shrink to 4 patterns after the first, so growth overlaps many calls."""
    import build_emu

    exe = build_emu.build("tsan")
    c = CASES["clique"]
    out = tmp_path / "res.txt"
    env = dict(os.environ, TSAN_OPTIONS="halt_on_error=1")
    r = subprocess.run([str(exe), "-file", str(GOLDEN / c["file"]), "-freq", str(c["tau"]), "-maxNodes",
                        str(c["max_nodes"]), "-out", str(out), "-call-ms", "0.001"], capture_output=True, text=True,
                       timeout=900, env=env)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-4000:]
    assert "ThreadSanitizer" not in r.stderr
    assert set(read_results(out)) == golden_pattern_set("clique")


@pytest.mark.parametrize("case", ["clique", "quirk_elabels"])
@pytest.mark.parametrize("limit", ["0.000001", "0.2"])  # before the first call; after some calls
def test_emulated_time_limit_stops_cleanly(emu, case, limit, tmp_path):
    """The time limit drops a level's remaining candidates while their growth runs on the helper
    thread: the run ends cleanly (sanitizers on) and reports a subset of the reference's patterns."""
    c = CASES[case]
    out = tmp_path / "res.txt"
    env = dict(os.environ, ASAN_OPTIONS="detect_leaks=1:abort_on_error=1", UBSAN_OPTIONS="halt_on_error=1",
               TFSM_HOST_THREADS="3")
    r = subprocess.run([str(emu), "-file", str(GOLDEN / c["file"]), "-freq", str(c["tau"]), "-maxNodes",
                        str(c["max_nodes"]), "-out", str(out), "-max-batch", "2", "-time-limit", limit],
                       capture_output=True, text=True, timeout=600, env=env)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-4000:]
    assert set(read_results(out)) <= golden_pattern_set(case)
