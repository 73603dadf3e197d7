"""GPU ingestion of the data graph (t-fsm_gb300/csrc/cuda/ingest.cu) builds the device graph the
host loader builds (host/lg_fast.hpp + the GpuEngine constructor), from `.lg` files and from edge
arrays: the same row offsets, neighbour lists, edge labels, label starts, label-offset table,
frequent labels, 1-edge pattern table and statistics, and the same error (code and message) for
malformed input.

CPU: the rules the kernels share with the host loader (the `.lg` line parser with C's strtol
semantics, the column-major id fill) against the host code, on random texts.
GPU: device ingestion == host ingestion (TFSM_INGEST=host) on every golden graph, random
multigraphs (self-loops, parallel edges, negative and wide-range labels, 40 edge labels), both
forms of the adjacency sort, and malformed files.
"""
from __future__ import annotations

import os
import subprocess

import numpy as np
import pytest

from conftest import CASES, GOLDEN, ROOT

FIELDS = ("row_off", "col", "elab", "label_start", "lab_off", "vlabels", "elabels", "label_mean_degree")


@pytest.fixture(scope="module")
def rules_check(tmp_path_factory):
    out = tmp_path_factory.mktemp("ingest") / "ingest_rules_check"
    subprocess.run(["g++", "-std=c++17", "-O2", "-pthread", "-I", str(ROOT / "t-fsm_gb300" / "csrc"),
                    str(ROOT / "tests" / "native" / "ingest_rules_check.cpp"), "-o", str(out)], check=True)
    return out


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_line_rules_equal_host_parsers(rules_check, seed):
    r = subprocess.run([str(rules_check), "parse", str(seed), "4000"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr


def test_id_fill_rule_equals_engine_loop(rules_check):
    r = subprocess.run([str(rules_check), "rank"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr


# ---- GPU: device ingestion against host ingestion ----------------------------------------------


class _Ingest:
    """Sets TFSM_INGEST (read by the library at each load) for the duration of a block."""

    def __init__(self, mode: str | None, wide: bool = False):
        self.mode, self.wide = mode, wide

    def __enter__(self):
        self.saved = {k: os.environ.get(k) for k in ("TFSM_INGEST", "TFSM_INGEST_WIDE_IDS")}
        if self.mode is None:
            os.environ.pop("TFSM_INGEST", None)
        else:
            os.environ["TFSM_INGEST"] = self.mode
        if self.wide:
            os.environ["TFSM_INGEST_WIDE_IDS"] = "1"
        else:
            os.environ.pop("TFSM_INGEST_WIDE_IDS", None)

    def __exit__(self, *a):
        for k, v in self.saved.items():
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v


def _snapshot(tfsm, load):
    with load() as g:
        info = g.info()
        ex = g.export()
    info.pop("load_ms")
    info.pop("load_h2d_bytes")  # input bytes (device ingestion) vs the built graph (host loader)
    return info, ex


def _assert_same(a, b):
    info_a, ex_a = a
    info_b, ex_b = b
    assert info_a == info_b
    for f in FIELDS:
        assert np.array_equal(ex_a[f], ex_b[f]), f
    assert ex_a["edge_patterns"] == ex_b["edge_patterns"]


def _both(tfsm, load, wide=False):
    with _Ingest("host"):
        host = _snapshot(tfsm, load)
    with _Ingest(None, wide):
        device = _snapshot(tfsm, load)
    return host, device


def _error_of(tfsm, load):
    try:
        with load():
            return None
    except tfsm.TfsmError as e:
        return (e.code, str(e))


FILE_CASES = [n for n, c in CASES.items() if "file" in c]


@pytest.mark.gpu
@pytest.mark.parametrize("case", FILE_CASES + ["cfg1", "el3", "cfg2_t9000"])
def test_device_ingestion_equals_host_on_golden_graphs(tfsm, case_graph, case):
    path, tau = case_graph(case), CASES[case]["tau"]
    host, device = _both(tfsm, lambda: tfsm.Graph.load(path, tau))
    _assert_same(host, device)


def _random_graph(seed, n, m, labels, elabels, label_spread):
    rng = np.random.default_rng(seed)
    vl = (rng.zipf(1.3, n) % labels).astype(np.int32) * label_spread - 7
    src = rng.integers(0, n, m, dtype=np.uint32)
    dst = np.where(rng.random(m) < 0.05, src, rng.integers(0, n, m, dtype=np.uint32)).astype(np.uint32)
    dup = rng.random(m) < 0.05  # parallel edges: repeat an earlier edge
    idx = rng.integers(0, max(1, m), m)
    src[dup], dst[dup] = src[idx[dup]], dst[idx[dup]]
    el = (rng.integers(0, elabels, m).astype(np.int32) * 3 - 5).astype(np.int32)
    return vl, src, dst, el


@pytest.mark.gpu
@pytest.mark.parametrize("seed,n,m,labels,elabels,tau", [
    (0, 2000, 9000, 6, 1, 50), (1, 5000, 30000, 12, 3, 1), (2, 3000, 12000, 40, 40, 2),
    (3, 1000, 500, 3, 2, 0), (4, 4000, 20000, 250, 1, 1), (5, 50, 0, 4, 1, 1), (6, 0, 0, 1, 1, 1)])
def test_device_ingestion_equals_host_on_edge_arrays(tfsm, seed, n, m, labels, elabels, tau):
    vl, src, dst, el = _random_graph(seed, n, m, labels, elabels, 1_000_003)
    host, device = _both(tfsm, lambda: tfsm.Graph.from_edges(vl, src, dst, el, tau))
    _assert_same(host, device)


@pytest.mark.gpu
@pytest.mark.parametrize("seed", [7, 8])
def test_wide_id_sort_equals_packed_sort(tfsm, seed):
    vl, src, dst, el = _random_graph(seed, 6000, 40000, 10, 4, 1)
    host, device = _both(tfsm, lambda: tfsm.Graph.from_edges(vl, src, dst, el, 2), wide=True)
    _assert_same(host, device)


def _write_lg(path, vl, src, dst, el):
    lines = ["t # 0"] + [f"v {i} {int(x)}" for i, x in enumerate(vl)] + [
        f"e {int(a)} {int(b)} {int(c)}" for a, b, c in zip(src, dst, el)]
    path.write_text("\n".join(lines) + "\n")
    return path


@pytest.mark.gpu
@pytest.mark.parametrize("seed", [10, 11, 12])
def test_device_ingestion_equals_host_on_random_files(tfsm, tmp_path, seed):
    vl, src, dst, el = _random_graph(seed, 3000, 15000, 8, 3, 1)
    path = _write_lg(tmp_path / "g.lg", vl, src, dst, el)
    host, device = _both(tfsm, lambda: tfsm.Graph.load(path, 20))
    _assert_same(host, device)
    # the file and the arrays it holds give the same graph
    with _Ingest(None):
        arrays = _snapshot(tfsm, lambda: tfsm.Graph.from_edges(vl, src, dst, el, 20))
    _assert_same(device, arrays)


MALFORMED = {
    "bad_kind": "t # 0\nv 0 1\nx 1 2\n",
    "vertex_missing_label": "v 0 1\nv 1\n",
    "vertex_negative": "v -1 3\n",
    "edge_negative": "v 0 1\nv 1 1\ne 0 -1 2\n",
    "edge_short": "v 0 1\nv 1 1\ne 0 1\n",
    "vertex_order": "v 0 1\nv 2 1\nv 1 1\n",
    "vertex_order_last_line_no_newline": "v 0 1\nv 5 1",
    "endpoint": "v 0 1\nv 1 1\ne 0 2 0\n",
    "endpoint_wraps": "v 0 1\nv 1 1\ne 4294967296 1 0\n",
    "overflow_label": "v 0 99999999999999999999\nv 1 -99999999999999999999\ne 0 1 9223372036854775807\n",
    "tabs_and_cr": "v\t0 1\r\nv 1 \t 1\r\ne 0 1 0 \r\n",
    "first_error_wins": "v 0 1\nq\nv 3 1\n",
    "empty": "",
    "comments_only": "# x\nt # 0\n\n   \n",
}


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(MALFORMED))
def test_device_ingestion_errors_equal_host(tfsm, tmp_path, name):
    path = tmp_path / f"{name}.lg"
    path.write_bytes(MALFORMED[name].encode())
    with _Ingest("host"):
        want = _error_of(tfsm, lambda: tfsm.Graph.load(path, 1))
    with _Ingest(None):
        got = _error_of(tfsm, lambda: tfsm.Graph.load(path, 1))
    assert got == want
    if want is None:
        host, device = _both(tfsm, lambda: tfsm.Graph.load(path, 1))
        _assert_same(host, device)


@pytest.mark.gpu
def test_device_ingestion_errors_on_edge_arrays(tfsm):
    vl = np.array([1, 1, 2], np.int32)
    src, dst, el = np.array([0, 1], np.uint32), np.array([1, 3], np.uint32), np.array([0, 0], np.int32)
    with _Ingest("host"):
        want = _error_of(tfsm, lambda: tfsm.Graph.from_edges(vl, src, dst, el, 1))
    with _Ingest(None):
        got = _error_of(tfsm, lambda: tfsm.Graph.from_edges(vl, src, dst, el, 1))
    assert want is not None and got == want
