"""The C-ABI library: it loads, exports what include/tfsm.h declares, and reports host-side errors
(I/O, malformed input, bad arguments) with status codes before any device work."""
from __future__ import annotations

import ctypes as C
import re

import pytest

from conftest import ROOT, has_gpu


def declared_functions() -> list[str]:
    text = (ROOT / "include" / "tfsm.h").read_text()
    return sorted(set(re.findall(r"\b(tfsm_[a-z_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol(tfsm):
    lib = tfsm.lib()
    names = declared_functions()
    assert "tfsm_evaluate_support" in names and "tfsm_mine" in names
    for n in names:
        assert hasattr(lib, n), f"{n} declared in include/tfsm.h but not exported"
    assert sorted(tfsm.EXPORTED) == names


def test_missing_file_is_an_io_error(tfsm, tmp_path):
    with pytest.raises(tfsm.TfsmError) as e:
        tfsm.Graph.load(tmp_path / "nope.lg", 5)
    assert e.value.code == tfsm.TFSM_ERR_IO


@pytest.mark.parametrize("text", [
    "t 2 1\nv 0 1 1\nv 1 1 1\ne 0 5 1\n",        # endpoint out of range
    "t 2 1\nv 0 1 1\nv 2 1 1\n",                 # ids not 0..N-1 in order
    "t 1 0\nv 0\n",                              # missing label
    "t 2 1\nv 0 1 1\nv 1 1 1\nx 0 1 1\n",        # unknown line kind
    "t 2 1\nv 0 1 1\nv 1 1 1\ne 0 1\n",          # missing edge label
])
def test_malformed_lg_is_a_format_error(tfsm, tmp_path, text):
    p = tmp_path / "bad.lg"
    p.write_text(text)
    with pytest.raises(tfsm.TfsmError) as e:
        tfsm.Graph.load(p, 1)
    assert e.value.code == tfsm.TFSM_ERR_FORMAT


def test_null_arguments(tfsm):
    lib = tfsm.lib()
    h = C.c_void_p()
    assert lib.tfsm_graph_load(None, 1, C.byref(h)) == tfsm.TFSM_ERR_ARG
    assert lib.tfsm_mine(None, 1, 3, 0, None, None) == tfsm.TFSM_ERR_ARG
    assert lib.tfsm_evaluate_batch(None, None, 0, 1, 0, None) == tfsm.TFSM_ERR_ARG
    assert lib.tfsm_graph_info(None, None) == tfsm.TFSM_ERR_ARG
    assert lib.tfsm_last_error()  # a message is set


@pytest.mark.skipif(has_gpu(), reason="checks the no-device error path")
def test_no_device_is_reported(tfsm):
    p = ROOT / "tests" / "golden" / "graphs" / "clique.lg"
    with pytest.raises(tfsm.TfsmError) as e:
        tfsm.Graph.load(p, 3)
    assert e.value.code == tfsm.TFSM_ERR_NO_DEVICE


def test_cli_usage_error(built):
    import subprocess

    r = subprocess.run([str(built / "bin" / "run")], capture_output=True, text=True)
    assert r.returncode == 2 and "usage" in r.stderr


def test_ctypes_structs_match_the_header_layout(tfsm, tmp_path):
    """Every struct of the binding has the size and field offsets the C compiler gives the header's
    (the option and statistics structs grow at their ends; a mismatch would shift fields)."""
    import shutil
    import subprocess

    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    structs = {"tfsm_dfs_code": tfsm.DfsCode, "tfsm_pattern": tfsm.PatternC, "tfsm_result": tfsm.ResultC,
               "tfsm_graph_info_t": tfsm.GraphInfoC, "tfsm_mine_stats": tfsm.MineStatsC,
               "tfsm_options": tfsm.OptionsC, "tfsm_parent": tfsm.ParentC}
    lines = ["#include <stddef.h>", "#include <stdio.h>", '#include "tfsm.h"', "int main(void) {"]
    for cname, cls in structs.items():
        lines.append(f'    printf("{cname} %zu\\n", sizeof({cname}));')
        for fname, _ in cls._fields_:
            cfield = fname.rstrip("_")  # ctypes name from_ is the C field from
            lines.append(f'    printf("{cname}.{fname} %zu\\n", offsetof({cname}, {cfield}));')
    lines += ["    return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run([cc, "-std=c11", "-I", str(ROOT / "include"), str(src), "-o", str(exe)], check=True)
    got = dict(line.rsplit(" ", 1) for line in subprocess.run([str(exe)], capture_output=True, text=True,
                                                              check=True).stdout.splitlines())
    for cname, cls in structs.items():
        assert int(got[cname]) == C.sizeof(cls), cname
        for fname, _ in cls._fields_:
            assert int(got[f"{cname}.{fname}"]) == getattr(cls, fname).offset, f"{cname}.{fname}"
