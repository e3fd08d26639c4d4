import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
GOLDEN = Path(__file__).resolve().parent / "golden"
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (runs the CUDA kernels)")


@pytest.fixture(scope="session")
def port():
    from oracle import oracle
    oracle.build_port()
    return oracle.port()


@pytest.fixture(scope="session")
def lib():
    """The product library (built in-tree if needed; nvcc cross-compiles without a GPU)."""
    from tangerine_gb300 import build, _lib
    build.build()
    return _lib.load()


def golden_names():
    """The per-tree fixtures (writer_*.npz hold file-writer cases, lua_*.npz the trees of
    the reference's Lua model scripts)."""
    return sorted(p.stem for p in GOLDEN.glob("*.npz") if not p.stem.startswith(("writer_", "lua_")))


@pytest.fixture(scope="session")
def golden():
    return {name: dict(np.load(GOLDEN / f"{name}.npz")) for name in golden_names()}


def sorted_faces(faces):
    f = np.ascontiguousarray(np.asarray(faces, dtype=np.uint64).reshape(-1, 3))
    return np.sort(f.view([("a", "<u8"), ("b", "<u8"), ("c", "<u8")]).ravel())


def canonical_rows(points, normals, colors):
    """Point-cloud rows (position, normal, colour bits) sorted: the reference's threads write
    them in a run-dependent order, every row a function of its voxel alone."""
    cols = [np.ascontiguousarray(points, np.float32).view(np.uint32), np.ascontiguousarray(normals, np.float32).view(np.uint32)]
    if colors is not None:
        cols.append(np.asarray(colors).astype(np.uint32))
    a = np.concatenate(cols, 1)
    return a[np.lexsort(a.T[::-1])]
