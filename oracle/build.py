"""ORACLE (test infrastructure): builds oracle/_build/liboracle.so with g++.

The shared library holds the CPU task executor, the CPU DMRG sweep and the determinant
FCI of this directory, linked with the product's host-side task compiler sources
(chemps2_gb300/csrc/host/*.cpp, plain C++ without CUDA). Only the tests, the smoke check
and the benchmark's CPU baseline load it.
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

HERE = Path(__file__).resolve().parent
HOST = HERE.parent / "chemps2_gb300" / "csrc" / "host"
BUILD = HERE / "_build"
LIB = BUILD / "liboracle.so"
FLAGS = ["-std=c++17", "-O3", "-fPIC", "-Wall", "-fno-fast-math", "-pthread"]


def _sources() -> list[Path]:
    return sorted(HERE.glob("*.cpp")) + sorted(HOST.glob("*.cpp"))


def _headers_mtime() -> float:
    t = 0.0
    for d in (HERE, HOST, HOST / "chemps2"):
        for p in d.glob("*"):
            if p.suffix in (".h", ".hpp", ".inc"):
                t = max(t, p.stat().st_mtime)
    return t


def build(verbose: bool = False) -> Path:
    BUILD.mkdir(parents=True, exist_ok=True)
    hdr = _headers_mtime()
    objs, todo = [], []
    for src in _sources():
        tag = "host_" if src.parent == HOST else ""
        obj = BUILD / f"{tag}{src.stem}.o"
        objs.append(obj)
        if not obj.exists() or obj.stat().st_mtime < max(src.stat().st_mtime, hdr):
            todo.append((src, obj))

    def cc(pair):
        src, obj = pair
        cmd = ["g++", *FLAGS, "-I", str(HOST), "-I", str(HERE), "-c", str(src), "-o", str(obj)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"oracle compile failed: {' '.join(cmd)}\n{r.stderr}")

    with ThreadPoolExecutor(max_workers=min(16, os.cpu_count() or 4)) as ex:
        list(ex.map(cc, todo))
    if todo or not LIB.exists():
        tmp = BUILD / "liboracle.so.tmp"
        cmd = ["g++", "-shared", "-pthread", "-o", str(tmp), *map(str, objs)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"oracle link failed: {r.stderr}")
        os.replace(tmp, LIB)
    if verbose:
        print(f"[oracle] compiled {len(todo)} units -> {LIB}", file=sys.stderr)
    return LIB


if __name__ == "__main__":
    print(build(verbose=True))
