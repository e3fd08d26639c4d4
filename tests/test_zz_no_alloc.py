"""tg_export_mesh_noalloc: the mesh export for callers that cannot allocate GPU memory
while running (their device memory is pooled elsewhere, or cudaMalloc's device-wide
synchronisation is off-limits on their thread).  The entry point keeps its scratch in a
fixed device array inside the library and writes into buffers the caller owns; its
results must equal tg_export_mesh's bit for bit (the tolerance of every parity test
here), including on a second call that finds the previous call's data in the shared
scratch array, and a call after the first one on a device must leave the device's free
memory unchanged.

This file is collected last so that a run stopping at the first failure has run every
other test first; it also passes on its own in a fresh process."""

import ctypes as C

import numpy as np
import pytest

from tangerine_gb300 import _lib, sdf
from tangerine_gb300 import workloads as W

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


class _Buffers:
    """Caller-owned device outputs, allocated once (by torch, before the measured calls)."""

    def __init__(self, vcap, fcap):
        dev = torch.device("cuda")
        self.vcap, self.fcap = vcap, fcap
        self.verts = torch.empty(vcap * 3, dtype=torch.float32, device=dev)
        self.norms = torch.empty(vcap * 3, dtype=torch.float32, device=dev)
        self.cols = torch.empty(vcap * 3, dtype=torch.uint8, device=dev)
        self.faces = torch.empty(fcap * 3, dtype=torch.int32, device=dev)
        self.cubes = torch.empty(vcap, dtype=torch.int32, device=dev)


def _ptr(t):
    return C.c_void_p(t.data_ptr()) if t is not None else None


def _call(prog, grid, buf, flags=1, normals=True, colors=True):
    g = sdf._grid(grid)
    counts = (C.c_uint64 * 2)()
    stream = torch.cuda.current_stream().cuda_stream
    st = _lib.load().tg_export_mesh_noalloc(
        prog.ptr, C.byref(g), flags, _ptr(buf.verts), _ptr(buf.norms) if normals else None,
        _ptr(buf.cols) if colors else None, _ptr(buf.faces), _ptr(buf.cubes), buf.vcap, buf.fcap, counts,
        C.c_void_p(stream))
    return st, (int(counts[0]), int(counts[1]))


def _read(prog, buf, v, f, attributes):
    painted = prog.info().has_paint
    return sdf.Mesh(buf.verts[: 3 * v].cpu().numpy().reshape(v, 3),
                    buf.norms[: 3 * v].cpu().numpy().reshape(v, 3) if attributes else None,
                    buf.cols[: 3 * v].cpu().numpy().reshape(v, 3) if attributes and painted else None,
                    buf.faces[: 3 * f].cpu().numpy().view(np.uint32).reshape(f, 3),
                    buf.cubes[:v].cpu().numpy().view(np.uint32))


def _same(got, want, attributes):
    np.testing.assert_array_equal(got.vertices, want.vertices)
    np.testing.assert_array_equal(got.faces, want.faces)
    np.testing.assert_array_equal(got.cubes, want.cubes)
    if attributes:
        np.testing.assert_array_equal(got.normals, want.normals)
        if want.colors is None:
            assert got.colors is None
        else:
            np.testing.assert_array_equal(got.colors, want.colors)


def _free_bytes():
    torch.cuda.synchronize()
    return torch.cuda.mem_get_info()[0]


def test_noalloc_setup_call_reserves_the_scratch():
    # Every pointer NULL: only reserve the array on the current device and cache its address.
    torch.zeros(1, device="cuda")
    st = _lib.load().tg_export_mesh_noalloc(None, None, 0, None, None, None, None, None, 0, 0, None, None)
    assert st == 0, _lib.load().tg_last_error()


def test_noalloc_matches_export_mesh_twice_in_a_row():
    # (tree, resolution, flags): a painted tree with normals and colours, a large lattice
    # first; then a smaller painted one over its leftovers; then an unpainted tree without
    # attributes (normals and colours NULL).
    cases = [(W.random_tree(1, 16, ops=W.OPS_UNIFORM4), 100, 1, True),
             (W.random_tree(7, 64), 48, 1, True),
             (W.random_tree(3, 32, paint=False), 80, 0, False)]
    for spec, res, flags, painted in cases:
        attributes = flags == 1
        grid = W.export_grid(resolution=res)
        with sdf.compile(sdf.from_spec(spec)) as prog:
            assert bool(prog.info().has_paint) == painted
            want = prog.export_mesh(grid, attributes=attributes)
            prog.export_mesh(grid, attributes=attributes, dense=True)   # loads the dense kernels' modules
            buf = _Buffers(want.vertices.shape[0] + 64, want.faces.shape[0] + 64)
            for call in range(2):
                before = _free_bytes()
                st, (v, f) = _call(prog, grid, buf, flags=flags, normals=attributes, colors=attributes)
                after = _free_bytes()
                assert st == 0, _lib.load().tg_last_error()
                assert (v, f) == (want.vertices.shape[0], want.faces.shape[0])
                _same(_read(prog, buf, v, f, attributes), want, attributes)
                if call == 1:
                    assert after == before, f"free device memory changed by {before - after} bytes"


def test_noalloc_rejects_what_does_not_fit():
    spec = W.random_tree(5, 16, ops=W.OPS_UNIFORM4)
    lib = _lib.load()
    with sdf.compile(sdf.from_spec(spec)) as prog:
        small = _Buffers(16, 16)
        # lattice larger than the fixed scratch array
        st, _ = _call(prog, W.export_grid(resolution=300), small)
        assert st == 6 and b"scratch" in lib.tg_last_error()
        # flags this path does not have (brick edge bits)
        grid = W.export_grid(resolution=64)
        st, _ = _call(prog, grid, small, flags=1 | (7 << 8))
        assert st == 6
        # vertex capacity too small: the vertices needed come back, the faces stay unknown
        st, (v, f) = _call(prog, grid, _Buffers(8, 8))
        assert st == 1 and v > 8 and f == 0
        # vertex capacity enough, face capacity too small: the faces needed come back
        st, (v2, f2) = _call(prog, grid, _Buffers(v, 8))
        assert st == 1 and v2 == v and f2 > 8
        buf = _Buffers(v, f2)
        st, (v3, f3) = _call(prog, grid, buf)
        assert st == 0 and (v3, f3) == (v, f2)
        _same(_read(prog, buf, v3, f3, True), prog.export_mesh(grid), True)
