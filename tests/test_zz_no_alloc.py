"""tg_export_mesh_noalloc: the mesh export for callers that cannot allocate GPU memory
while running (their device memory is pooled elsewhere, or cudaMalloc's device-wide
synchronisation is off-limits on their thread).  The entry point keeps its scratch in a
fixed device array inside the library and writes into buffers the caller owns; its
results must equal tg_export_mesh's bit for bit (the tolerance of every parity test
here), including on a second call that finds the previous call's data in the shared
scratch array.

This file is collected last so that a run stopping at the first failure has run every
other test first; it also passes on its own in a fresh process."""

import ctypes as C

import numpy as np
import pytest

from tangerine_gb300 import _lib, sdf
from tangerine_gb300 import workloads as W

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _noalloc(prog, grid, vcap, fcap, attributes=True):
    g = sdf._grid(grid)
    dev = torch.device("cuda")
    verts = torch.empty(vcap * 3, dtype=torch.float32, device=dev)
    norms = torch.empty(vcap * 3, dtype=torch.float32, device=dev)
    cols = torch.empty(vcap * 3, dtype=torch.uint8, device=dev)
    faces = torch.empty(fcap * 3, dtype=torch.int32, device=dev)
    cubes = torch.empty(vcap, dtype=torch.int32, device=dev)
    counts = (C.c_uint64 * 2)()
    stream = torch.cuda.current_stream().cuda_stream
    st = _lib.load().tg_export_mesh_noalloc(
        prog.ptr, C.byref(g), 1 if attributes else 0,
        C.c_void_p(verts.data_ptr()), C.c_void_p(norms.data_ptr()), C.c_void_p(cols.data_ptr()),
        C.c_void_p(faces.data_ptr()), C.c_void_p(cubes.data_ptr()), vcap, fcap, counts, C.c_void_p(stream))
    v, f = int(counts[0]), int(counts[1])
    if st != 0:
        return st, (v, f), None
    out = sdf.Mesh(verts[: 3 * v].cpu().numpy().reshape(v, 3), norms[: 3 * v].cpu().numpy().reshape(v, 3),
                   cols[: 3 * v].cpu().numpy().reshape(v, 3) if prog.info().has_paint else None,
                   faces[: 3 * f].cpu().numpy().view(np.uint32).reshape(f, 3),
                   cubes[:v].cpu().numpy().view(np.uint32))
    return st, (v, f), out


def _same(a, b):
    np.testing.assert_array_equal(a.vertices, b.vertices)
    np.testing.assert_array_equal(a.normals, b.normals)
    np.testing.assert_array_equal(a.faces, b.faces)
    np.testing.assert_array_equal(a.cubes, b.cubes)
    if a.colors is None:
        assert b.colors is None
    else:
        np.testing.assert_array_equal(a.colors, b.colors)


def test_noalloc_matches_export_mesh_twice_in_a_row():
    cases = [(W.random_tree(1, 16, ops=W.OPS_UNIFORM4), 100),   # large call first ...
             (W.random_tree(7, 64), 48)]                        # ... then a smaller one over its leftovers
    for spec, res in cases:
        grid = W.export_grid(resolution=res)
        with sdf.compile(sdf.from_spec(spec)) as prog:
            want = prog.export_mesh(grid)
            st, (v, f), got = _noalloc(prog, grid, vcap=want.vertices.shape[0] + 64, fcap=want.faces.shape[0] + 64)
            assert st == 0, _lib.load().tg_last_error()
            assert (v, f) == (want.vertices.shape[0], want.faces.shape[0])
            _same(got, want)


def test_noalloc_rejects_what_does_not_fit():
    spec = W.random_tree(5, 16, ops=W.OPS_UNIFORM4)
    with sdf.compile(sdf.from_spec(spec)) as prog:
        # lattice larger than the fixed scratch array
        st, _, _ = _noalloc(prog, W.export_grid(resolution=300), vcap=16, fcap=16)
        assert st == 6 and b"scratch" in _lib.load().tg_last_error()
        # output capacity too small: the needed sizes come back, then a retry fits
        grid = W.export_grid(resolution=64)
        st, (v, f), _ = _noalloc(prog, grid, vcap=8, fcap=8)
        assert st == 1 and v > 8
        st, (v2, f2), got = _noalloc(prog, grid, vcap=v, fcap=4 * v)
        assert st == 0 and v2 == v
        _same(got, prog.export_mesh(grid))
