"""Builds the Lua modelling surface (tg_lua.cpp) against a Lua 5.4 source tree: the Lua
core and standard libraries compiled from that tree, the surface, and a runner executable
(tangerine_gb300/lua/_build/tg_lua) linked to libtangerine_gb300.so.

Where no Lua source tree is given (TANGERINE_LUA_SRC, or a `lua` directory passed in),
nothing is built and `build()` returns None: the library itself does not depend on Lua.
"""

from __future__ import annotations

import concurrent.futures as cf
import os
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
PKG = HERE.parent
if str(PKG.parent) not in sys.path:
    sys.path.insert(0, str(PKG.parent))
OUT = HERE / "_build"
RUNNER = OUT / "tg_lua"
# The interpreter and compiler mains are not part of the library.
SKIP = {"lua.c", "luac.c", "onelua.c"}


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("compile failed:\n" + " ".join(map(str, cmd)) + "\n" + r.stdout + r.stderr)


def build(lua_src: str | os.PathLike | None = None, force: bool = False) -> Path | None:
    src = Path(lua_src or os.environ.get("TANGERINE_LUA_SRC", ""))
    if not str(src) or not (src / "lua.h").exists():
        return None
    from tangerine_gb300 import build as B
    lib = B.build()
    core = sorted(p for p in src.glob("*.c") if p.name not in SKIP)
    mine = HERE / "tg_lua.cpp"
    newest = max(p.stat().st_mtime for p in core + [mine, Path(__file__), PKG.parent / "include" / "tangerine_gb300.h", lib])
    if RUNNER.exists() and not force and RUNNER.stat().st_mtime > newest:
        return RUNNER
    OUT.mkdir(parents=True, exist_ok=True)
    cc, cxx = os.environ.get("CC", "gcc"), os.environ.get("CXX", "g++")
    jobs, objs = [], []
    for c in core:
        o = OUT / (c.stem + ".o")
        objs.append(o)
        jobs.append([cc, "-O2", "-std=gnu99", "-DLUA_USE_LINUX", "-w", "-c", str(c), "-o", str(o)])
    o = OUT / "tg_lua.o"
    objs.append(o)
    jobs.append([cxx, "-O2", "-std=c++17", "-ffp-contract=off", f"-I{src}", "-c", str(mine), "-o", str(o)])
    with cf.ThreadPoolExecutor(max_workers=min(16, os.cpu_count() or 4)) as ex:
        list(ex.map(_run, jobs))
    _run([cxx, "-o", str(RUNNER), *map(str, objs), f"-L{PKG}", "-ltangerine_gb300", f"-Wl,-rpath,{PKG}", "-lm", "-ldl",
          "-pthread"])
    return RUNNER


if __name__ == "__main__":
    print(build(sys.argv[1] if len(sys.argv) > 1 else None, force="-f" in sys.argv))
