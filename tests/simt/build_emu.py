"""Build the host-side SIMT emulation of the engine (test infrastructure only).

Compiles the product's kernel and engine sources unchanged, as C++ for the CPU, against
tests/simt/cuda_runtime.h, with sanitizers, into tests/simt/_build/run_emu_<kind> (the `run` CLI)
or, with main="abi", tests/simt/_build/abi_emu_<kind> (the C-ABI driver tests/simt/abi_main.cpp).
usage: python tests/simt/build_emu.py [asan|tsan|none] [run|abi]
"""
from __future__ import annotations

import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
CSRC = ROOT / "t-fsm_gb300" / "csrc"

SANITIZE = {"asan": ["-fsanitize=address,undefined", "-fno-sanitize-recover=undefined"],
            "tsan": ["-fsanitize=thread"], "none": []}


def _compile(kind: str, src: Path, obj: Path, headers: list[Path]) -> None:
    """One translation unit to an object (skipped while it is newer than its source and headers)."""
    if obj.exists() and all(d.stat().st_mtime <= obj.stat().st_mtime for d in [src, *headers]):
        return
    cmd = ["g++", "-std=c++20", "-O1", "-g", "-pthread", "-DTFSM_SIMT_EMULATION", "-I", str(HERE), "-I", str(CSRC),
           *SANITIZE[kind], "-x", "c++", "-c", str(src), "-o", str(obj)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(" ".join(cmd) + "\n" + r.stderr[-4000:])


def build(kind: str = "asan", main: str = "run") -> Path:
    from concurrent.futures import ThreadPoolExecutor

    out_dir = HERE / "_build"
    obj_dir = out_dir / f"obj_{kind}"
    obj_dir.mkdir(parents=True, exist_ok=True)
    exe = out_dir / f"{main}_emu_{kind}"
    entry = CSRC / "run_main.cpp" if main == "run" else HERE / "abi_main.cpp"
    srcs = [CSRC / "cuda" / "kernels.cu", CSRC / "engine.cu", CSRC / "noalloc.cu", CSRC / "miner.cpp",
            CSRC / "capi.cpp", entry, HERE / "costmodel_stub.cpp"]
    headers = list(CSRC.rglob("*.h*")) + list(CSRC.rglob("*.cuh")) + [HERE / "cuda_runtime.h",
                                                                      ROOT / "include" / "tfsm.h"]
    objs = [obj_dir / (s.parent.name + "_" + s.name + ".o") for s in srcs]
    with ThreadPoolExecutor(max_workers=len(srcs)) as ex:  # the units compile in parallel
        for f in [ex.submit(_compile, kind, s, o, headers) for s, o in zip(srcs, objs)]:
            f.result()
    if exe.exists() and all(o.stat().st_mtime <= exe.stat().st_mtime for o in objs):
        return exe
    cmd = ["g++", "-pthread", *SANITIZE[kind], *map(str, objs), "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(" ".join(cmd) + "\n" + r.stderr[-4000:])
    return exe


if __name__ == "__main__":
    print(build(sys.argv[1] if len(sys.argv) > 1 else "asan", sys.argv[2] if len(sys.argv) > 2 else "run"))
