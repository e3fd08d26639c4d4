"""Builds libtangerine_gb300.so in-tree: CUDA kernels for sm_103a plus the C++ host
runtime, one object per source compiled in parallel, cudart linked statically.

Host C++ is compiled with -ffp-contract=off and the kernels with -fmad=false: no
multiply-add is ever fused, so the host's clip decisions and the GPU's distances round
exactly like Tangerine's x86-64 Release build.
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
OUT = PKG / "_build"
LIB = PKG / "libtangerine_gb300.so"
INCLUDE = PKG.parent / "include"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc() -> str:
    cand = os.environ.get("NVCC") or shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return cand


def _cuda_home() -> Path:
    return Path(_nvcc()).resolve().parent.parent


def sources():
    cu = sorted((CSRC / "kernels").glob("*.cu"))
    cpp = sorted((CSRC / "host").glob("*.cpp"))
    return cu, cpp


def _compile(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("compile failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stderr


def build(verbose: bool = False, force: bool = False, extra_nvcc=()) -> Path:
    cu, cpp = sources()
    headers = list((CSRC).rglob("*.hpp")) + list((CSRC).rglob("*.cuh")) + list(INCLUDE.glob("*.h"))
    newest = max(p.stat().st_mtime for p in cu + cpp + headers + [Path(__file__)])
    if LIB.exists() and not force and LIB.stat().st_mtime > newest:
        return LIB
    OUT.mkdir(parents=True, exist_ok=True)
    nvcc = _nvcc()
    cuda = _cuda_home()
    jobs = []
    objs = []
    for src in cu:
        obj = OUT / (src.stem + ".cu.o")
        objs.append(obj)
        jobs.append([nvcc, *ARCH, "-lineinfo", "-O3", "-std=c++17", "-fmad=false", "-Xptxas", "-v",
                     "-Xcompiler", "-fPIC,-ffp-contract=off", *extra_nvcc, "-c", str(src), "-o", str(obj)])
    cxx = os.environ.get("CXX", "g++")
    for src in cpp:
        obj = OUT / (src.stem + ".o")
        objs.append(obj)
        jobs.append([cxx, "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-fno-fast-math", "-pthread",
                     f"-I{cuda / 'include'}", "-c", str(src), "-o", str(obj)])
    with cf.ThreadPoolExecutor(max_workers=min(16, os.cpu_count() or 4)) as ex:
        logs = list(ex.map(_compile, jobs))
    if verbose:
        for log in logs:
            if log.strip():
                print(log, file=sys.stderr)
    (OUT / "ptxas.log").write_text("\n".join(logs))
    tmp = LIB.with_suffix(".so.tmp")
    link = [nvcc, *ARCH, "-shared", "-cudart", "static", "-o", str(tmp), *map(str, objs),
            "-Xlinker", "--exclude-libs,ALL", "-lpthread"]
    _compile(link)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
