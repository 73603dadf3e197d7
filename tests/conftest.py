"""Shared fixtures: build products, the CPU oracle, fixture graphs and golden data.

Marker `gpu`: tests that need a CUDA device (run on the GB300 host with `-m gpu`).
"""
from __future__ import annotations

import importlib.util
import json
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
PKG = ROOT / "t-fsm_gb300"
GOLDEN = ROOT / "tests" / "golden"
sys.path.insert(0, str(ROOT / "tests"))

from golden_io import graph_checksum, read_mni  # noqa: E402


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); run with -m gpu")


def load_binding():
    """Import t-fsm_gb300/tfsm.py (the directory name is not a Python identifier)."""
    if "tfsm" in sys.modules:
        return sys.modules["tfsm"]
    spec = importlib.util.spec_from_file_location("tfsm", PKG / "tfsm.py")
    mod = importlib.util.module_from_spec(spec)
    sys.modules["tfsm"] = mod
    spec.loader.exec_module(mod)
    return mod


@pytest.fixture(scope="session")
def built():
    """Builds the library, CLI and generator when missing or stale."""
    sys.path.insert(0, str(PKG))
    import build as pkg_build  # t-fsm_gb300/build.py

    pkg_build.build()
    return PKG


@pytest.fixture(scope="session")
def tfsm(built):
    return load_binding()


@pytest.fixture(scope="session")
def port(built):
    """The CPU oracle binary (oracle/tfsm_port), built from source."""
    r = subprocess.run(["make", "-s", "-C", str(ROOT / "oracle"), "port"], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    return ROOT / "oracle" / "tfsm_port"


@pytest.fixture(scope="session")
def brute():
    """The definition checker (oracle/mni_brute), built from source."""
    r = subprocess.run(["make", "-s", "-C", str(ROOT / "oracle"), "brute"], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    return ROOT / "oracle" / "mni_brute"


CASES = json.loads((GOLDEN / "cases.json").read_text())


def gen_cmd(out: Path, g: dict) -> list[str]:
    return [str(PKG / "bin" / "gen_lg"), "--out", str(out), "--n", str(g["n"]), "--mean", str(g["mean"]), "--gamma",
            str(g["gamma"]), "--max-degree", str(g["max_degree"]), "--labels", str(g["labels"]), "--zipf",
            str(g["zipf"]), "--elabels", str(g["elabels"]), "--seed", str(g["seed"])]


@pytest.fixture(scope="session")
def graph_dir(tmp_path_factory):
    return tmp_path_factory.mktemp("graphs")


@pytest.fixture(scope="session")
def case_graph(built, graph_dir):
    """case name -> path of its .lg graph (generated or committed), checksum-verified."""
    cache: dict[str, Path] = {}

    def get(name: str) -> Path:
        if name in cache:
            return cache[name]
        c = CASES[name]
        if "file" in c:
            path = GOLDEN / c["file"]
        else:
            key = "_".join(f"{k}{v}" for k, v in sorted(c["gen"].items()))
            path = graph_dir / f"g_{key}.lg"
            if not path.exists():
                r = subprocess.run(gen_cmd(path, c["gen"]), capture_output=True, text=True)
                assert r.returncode == 0, r.stderr
        assert graph_checksum(path) == c["checksum"], f"{name}: generated graph differs from the golden graph"
        cache[name] = path
        return path

    return get


def golden_pattern_set(name: str) -> set[str]:
    p = GOLDEN / f"{name}.patterns.txt"
    return {l for l in p.read_text().splitlines() if l.strip()} if p.exists() else set()


def golden_mni(name: str) -> dict[str, list[int]]:
    p = GOLDEN / f"{name}.mni.txt"
    return read_mni(p) if p.exists() else {}


def has_gpu() -> bool:
    try:
        import torch

        return torch.cuda.is_available()
    except Exception:
        return False
