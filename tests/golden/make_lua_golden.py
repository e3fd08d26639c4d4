"""Writes tests/golden/lua_models.npz: the trees of Tangerine's own model scripts
(models/*.lua in the reference tree), built by this library's Lua surface
(tangerine_gb300/lua) and stored as tree specs (tg_tree_spec), so that the GPU tests can
export them on the GPU host, which has neither Lua nor the scripts, and compare with the
oracle.  Only scripts that use the modelling functions alone are taken (the others need
the Tangerine application: instancing, materials, random numbers, events).

    python tests/golden/make_lua_golden.py REFERENCE_TREE
"""

from __future__ import annotations

import subprocess
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from tangerine_gb300.lua import build as LB  # noqa: E402

MODELS = ["align", "basic_thing", "color-cube", "flower", "gear", "scale", "shapes", "spiral"]


def main(reference: Path) -> None:
    runner = LB.build(reference / "third_party" / "lua-5.4.4" / "lua")
    if runner is None:
        raise SystemExit("no Lua sources under the reference tree")
    models = reference / "models"
    out = {}
    r = subprocess.run([str(runner), *[f"{m}.lua" for m in MODELS]], cwd=models, capture_output=True, text=True, check=True)
    for line in r.stdout.splitlines():
        name, *words = line.split()
        out[Path(name).stem] = np.array([float(w) for w in words], np.float32)
    np.savez_compressed(Path(__file__).resolve().parent / "lua_models.npz", **out)
    print({k: v.size for k, v in out.items()})


if __name__ == "__main__":
    main(Path(sys.argv[1]))
