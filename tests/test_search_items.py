"""The search kernel's work items are decoded on the device from per-call item groups
(dev::item_at in t-fsm_gb300/csrc/cuda/dev_common.cuh): every group's runs of bitmap words come
round by round, and every (pattern vertex, run) is claimed exactly once.  CPU only (the same
function compiled for the host)."""
from __future__ import annotations

import subprocess

import pytest

from conftest import ROOT


@pytest.fixture(scope="module")
def checker(tmp_path_factory):
    out = tmp_path_factory.mktemp("items") / "items_check"
    subprocess.run(["g++", "-std=c++17", "-O2", "-I", str(ROOT / "t-fsm_gb300" / "csrc"),
                    str(ROOT / "tests" / "native" / "items_check.cpp"), "-o", str(out)], check=True)
    return out


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_item_decoding_enumerates_every_run_once(checker, seed):
    r = subprocess.run([str(checker), str(seed)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
