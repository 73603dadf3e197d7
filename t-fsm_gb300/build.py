"""Build recipe of the GB300 T-FSM engine (no cmake; a handful of translation units in parallel).

Produces, inside this package directory:
  libtfsm_gb300.so   C-ABI library (include/tfsm.h): CUDA kernels for sm_103a + host engine
  bin/run            command-line drop-in for the reference miners
  bin/gen_lg         seeded synthetic .lg generator
Objects go to _build/.  Run `python t-fsm_gb300/build.py` or call build().
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
# TFSM_BOUNDS_CHECK=1 builds the self-checking variant (every global access of the search kernels
# bounds-checked, first violation reported as an error) into its own object directory.
CHECKED = os.environ.get("TFSM_BOUNDS_CHECK") == "1"
BUILD = PKG / ("_build_checked" if CHECKED else "_build")
BIN = PKG / "bin"
LIB = PKG / "libtfsm_gb300.so"
ROOT = PKG.parent

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CXXFLAGS = ["-std=c++17", "-O3", "-fPIC", "-Wall", "-Wno-unused-function"]
# TFSM_HOST_DEBUG=1: host code keeps frame pointers and debug information (crash reports with
# symbolised stacks); device code is unchanged.
HOST_DEBUG = ["-g", "-fno-omit-frame-pointer"] if os.environ.get("TFSM_HOST_DEBUG") == "1" else []
# TFSM_SEARCH_MIN_BLOCKS=N: resident blocks per SM the search kernels are compiled for (register budget)
DEVICE_DEFS = ([f"-DTFSM_SEARCH_MIN_BLOCKS={int(os.environ['TFSM_SEARCH_MIN_BLOCKS'])}"]
               if os.environ.get("TFSM_SEARCH_MIN_BLOCKS") else [])


def _cuda_home() -> Path:
    for c in (os.environ.get("CUDA_HOME"), os.environ.get("CUDA_PATH"), "/usr/local/cuda"):
        if c and (Path(c) / "bin" / "nvcc").exists():
            return Path(c)
    nvcc = shutil.which("nvcc")
    if nvcc:
        return Path(nvcc).resolve().parent.parent
    raise RuntimeError("nvcc not found: set CUDA_HOME")


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + r.stdout)


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def _lib_is_checked() -> bool:
    marker = PKG / "_build_checked" / "linked"
    return LIB.exists() and marker.exists() and marker.stat().st_mtime >= LIB.stat().st_mtime - 1


def build(verbose: bool = False) -> Path:
    cuda = _cuda_home()
    nvcc = str(cuda / "bin" / "nvcc")
    BUILD.mkdir(exist_ok=True)
    BIN.mkdir(exist_ok=True)
    headers = list(CSRC.rglob("*.h")) + list(CSRC.rglob("*.hpp")) + list(CSRC.rglob("*.cuh")) + [ROOT / "include" / "tfsm.h"]
    cu = [CSRC / "cuda" / "kernels.cu", CSRC / "cuda" / "ingest.cu", CSRC / "engine.cu", CSRC / "noalloc.cu",
          CSRC / "costmodel" / "mlp.cu"]
    cpp = [CSRC / "miner.cpp", CSRC / "capi.cpp"]
    jobs = []
    objs = []
    for src in cu:
        obj = BUILD / (src.stem + ".o")
        objs.append(obj)
        if _stale(obj, [src] + headers):
            jobs.append([nvcc, *ARCH, "-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC",
                         *(["-Xcompiler", ",".join(HOST_DEBUG)] if HOST_DEBUG else []), "-I", str(CSRC),
                         *(["-DTFSM_BOUNDS_CHECK"] if CHECKED else []), *DEVICE_DEFS, "-c", str(src), "-o", str(obj)])
    for src in cpp:
        obj = BUILD / (src.stem + ".o")
        objs.append(obj)
        if _stale(obj, [src] + headers):
            jobs.append(["g++", *CXXFLAGS, *HOST_DEBUG, "-pthread", "-I", str(CSRC), "-I", str(cuda / "include"),
                         "-c", str(src),
                         "-o", str(obj)])
    gen = BIN / "gen_lg"
    gen_src = CSRC / "tools" / "gen_lg.cpp"
    if _stale(gen, [gen_src]):
        jobs.append(["g++", "-std=c++17", "-O2", "-ffp-contract=off", str(gen_src), "-o", str(gen)])
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for cmd in jobs:
            if verbose:
                print(" ".join(cmd), flush=True)
        list(ex.map(_run, jobs))
    if _stale(LIB, objs) or CHECKED != _lib_is_checked():
        cmd = [nvcc, *ARCH, "-shared", "-o", str(LIB), *map(str, objs), "-Xcompiler", "-pthread"]
        if verbose:
            print(" ".join(cmd), flush=True)
        _run(cmd)
        marker = PKG / "_build_checked" / "linked"
        if CHECKED:
            marker.write_text("checked build\n")
        elif marker.exists():
            marker.unlink()
    run_bin = BIN / "run"
    run_src = CSRC / "run_main.cpp"
    if _stale(run_bin, [run_src, LIB]):
        cmd = ["g++", "-std=c++17", "-O2", *HOST_DEBUG, str(run_src), "-o", str(run_bin), "-L", str(PKG), "-ltfsm_gb300",
               "-Wl,-rpath,$ORIGIN/.."]
        if verbose:
            print(" ".join(cmd), flush=True)
        _run(cmd)
    return LIB


if __name__ == "__main__":
    build(verbose="-v" in sys.argv)
    print(LIB)
