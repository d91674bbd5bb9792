"""Builds the native library libchemps2_gb300.so in-tree (chemps2_gb300/_lib/).

Every translation unit (host C++ task compiler, DMRG driver, C-ABI, CUDA kernels) is
compiled by nvcc for sm_103a only, in parallel, and linked with cuSOLVER (FP64
eigensolver of the truncation step). Objects go to chemps2_gb300/_build/; a unit is
rebuilt when it or any header under csrc/ is newer than its object.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIBDIR = PKG / "_lib"
LIBNAME = "libchemps2_gb300.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall"]


def nvcc() -> str:
    exe = shutil.which("nvcc")
    if exe:
        return exe
    cand = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda")) / "bin" / "nvcc"
    if cand.exists():
        return str(cand)
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build chemps2_gb300")


def sources() -> list[Path]:
    out = []
    for p in sorted(CSRC.rglob("*")):
        if p.suffix in (".cpp", ".cu") and "test" not in p.parts:
            out.append(p)
    return out


def _newest_header() -> float:
    t = 0.0
    for p in CSRC.rglob("*"):
        if p.suffix in (".h", ".hpp", ".cuh", ".inc"):
            t = max(t, p.stat().st_mtime)
    hdr = PKG.parent / "include"
    for p in hdr.glob("*.h"):
        t = max(t, p.stat().st_mtime)
    return t


def _compile(src: Path, obj: Path, compiler: str) -> None:
    obj.parent.mkdir(parents=True, exist_ok=True)
    cmd = [compiler, *FLAGS, *ARCH, "-I", str(CSRC), "-I", str(CSRC / "host"), "-c", str(src), "-o", str(obj)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compilation failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")


def build(verbose: bool = False, jobs: int | None = None) -> Path:
    compiler = nvcc()
    hdr_t = _newest_header()
    objs = []
    todo = []
    for src in sources():
        rel = src.relative_to(CSRC)
        obj = BUILD / rel.with_suffix(rel.suffix + ".o")
        objs.append(obj)
        if not obj.exists() or obj.stat().st_mtime < max(src.stat().st_mtime, hdr_t):
            todo.append((src, obj))
    jobs = jobs or min(16, os.cpu_count() or 4)
    with ThreadPoolExecutor(max_workers=jobs) as ex:
        futs = [ex.submit(_compile, s, o, compiler) for s, o in todo]
        for f in futs:
            f.result()
    if verbose:
        print(f"[chemps2_gb300] compiled {len(todo)} of {len(objs)} units", file=sys.stderr)
    LIBDIR.mkdir(parents=True, exist_ok=True)
    lib = LIBDIR / LIBNAME
    if todo or not lib.exists():
        tmp = LIBDIR / (LIBNAME + ".tmp")
        cmd = [compiler, "-shared", *ARCH, "-o", str(tmp), *map(str, objs), "-lcusolver", "-lcublas"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, lib)
    return lib


if __name__ == "__main__":
    print(build(verbose=True))
