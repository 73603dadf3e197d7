"""The allocation-free entry point, tfsm_evaluate_support_noalloc (marker: gpu).

Some callers cannot allocate device memory while they evaluate a pattern (their framework's
allocator owns the device, or cudaMalloc's device-wide synchronisation is not acceptable to them).
For them the library keeps one fixed 16 MiB device array per GPU and evaluates the pattern with all
per-call buffers carved out of it.  These tests call that entry point through the C ABI and require
the same results as tfsm_evaluate_support — bit-exact MNI per vertex and the same frequent decision —
on two calls in a row (the array keeps the previous call's contents), and a clear TFSM_ERR_LIMIT for
a pattern whose buffers exceed the array.  This file sorts last so that a failure here comes after
every other test has run; it also passes on its own in a fresh process.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from conftest import CASES, golden_mni

pytestmark = pytest.mark.gpu


def as_pattern(tfsm, codes):
    arr = (tfsm.DfsCode * len(codes))(*[tfsm.DfsCode(*c) for c in codes])
    p = tfsm.PatternC()
    p.n_codes = len(codes)
    p.codes = C.cast(arr, C.POINTER(tfsm.DfsCode))
    return p, arr


def call(tfsm, fn, graph, codes, tau, flags):
    p, keep = as_pattern(tfsm, codes)
    r = tfsm.ResultC()
    rc = fn(graph._h, C.byref(p), tau, flags, C.byref(r))
    return rc, r


@pytest.fixture(scope="module")
def cfg1_graph(tfsm, case_graph):
    g = tfsm.Graph.load(case_graph("cfg1"), CASES["cfg1"]["tau"])
    yield g
    g.close()


@pytest.mark.parametrize("flags", [1, 0])  # exact MNI, then the lazy decision
def test_noalloc_matches_evaluate_support_twice(tfsm, cfg1_graph, flags):
    lib = tfsm.lib()
    tau = CASES["cfg1"]["tau"]
    keys = list(golden_mni("cfg1"))
    patterns = [tfsm.parse_key(k) for k in keys]
    for _ in range(2):  # a second call must not see stale state from the first
        for codes in patterns:
            rc_a, a = call(tfsm, lib.tfsm_evaluate_support, cfg1_graph, codes, tau, flags)
            rc_b, b = call(tfsm, lib.tfsm_evaluate_support_noalloc, cfg1_graph, codes, tau, flags)
            assert rc_a == 0 and rc_b == 0, lib.tfsm_last_error()
            assert b.status == 0 and b.n_vertices == a.n_vertices
            assert bool(b.frequent) == bool(a.frequent), codes
            if flags & 1:
                assert list(b.mni[: b.n_vertices]) == list(a.mni[: a.n_vertices]), codes
                assert b.support == a.support


def test_noalloc_exact_equals_reference_engine(tfsm, cfg1_graph):
    lib = tfsm.lib()
    want = golden_mni("cfg1")
    for k, v in list(want.items())[::7]:
        rc, r = call(tfsm, lib.tfsm_evaluate_support_noalloc, cfg1_graph, tfsm.parse_key(k), CASES["cfg1"]["tau"], 1)
        assert rc == 0 and list(r.mni[: r.n_vertices]) == v, k


def test_noalloc_rejects_patterns_beyond_its_scratch(tfsm):
    lib = tfsm.lib()
    n = 3_000_000  # one label: a 16-vertex pattern needs 16 bitmaps of 93,750 words x 3 > 16 MiB
    src = np.arange(n - 1, dtype=np.uint32)
    with tfsm.Graph.from_edges(np.zeros(n, np.int32), src, src + 1, np.ones(n - 1, np.int32), 1) as g:
        path16 = [(i, i + 1, 0, 1, 0) for i in range(15)]
        rc, r = call(tfsm, lib.tfsm_evaluate_support_noalloc, g, path16, 1, 1)
        assert rc == tfsm.TFSM_ERR_LIMIT and r.status == tfsm.TFSM_ERR_LIMIT
        assert b"16 MiB" in lib.tfsm_last_error()
        # the allocating entry point handles it, and a small pattern still works afterwards
        rc2, r2 = call(tfsm, lib.tfsm_evaluate_support, g, path16[:2], 1, 1)
        rc3, r3 = call(tfsm, lib.tfsm_evaluate_support_noalloc, g, path16[:2], 1, 1)
        assert rc2 == 0 and rc3 == 0
        assert list(r3.mni[:3]) == list(r2.mni[:3])
