"""The point-cloud export (PointCloudExportThread) and the MagicaVoxel export (VoxExport) on
the GPU, through the C ABI, against the reference fixtures and the CPU oracle.

Everything is bit-exact: kept voxels, refined points, normals, colour bytes, voxel lists and
the .vox file bytes."""

import numpy as np
import pytest

from conftest import canonical_rows, golden_names, sorted_faces
from oracle import oracle as O
from tangerine_gb300 import _lib, sdf
from tangerine_gb300 import workloads as W

pytestmark = pytest.mark.gpu

CLOUD_STEP, CLOUD_REFINE, VOX_GRID, VOX_COLOR = 0.1, 5, 8.0, 3


def bounds_of(prog):
    """The tree's bounds (SDFNode::Bounds) as the program holds them."""
    i = prog.info()
    return np.array(i.bounds_min[:], np.float32), np.array(i.bounds_max[:], np.float32)


@pytest.mark.parametrize("name", golden_names())
def test_point_cloud_matches_reference(lib, golden, name):
    g = golden[name]
    if "cloud_rows" not in g:
        pytest.skip("unbounded tree")
    t = sdf.from_spec(g["spec"])
    with sdf.compile(t) as prog:
        lo, hi = bounds_of(prog)
        m = prog.export_point_cloud(lo, hi, CLOUD_STEP, CLOUD_REFINE)
    assert m.faces.shape[0] == 0
    assert np.all(np.diff(m.cubes.astype(np.int64)) > 0)
    assert (m.colors is not None) == bool(g["cloud_has_color"])
    np.testing.assert_array_equal(canonical_rows(m.vertices, m.normals, m.colors), g["cloud_rows"])


@pytest.mark.parametrize("name", golden_names())
def test_voxels_match_reference(lib, golden, name, tmp_path):
    g = golden[name]
    if "vox_voxels" not in g:
        pytest.skip("unbounded tree")
    t = sdf.from_spec(g["spec"])
    with sdf.compile(t) as prog:
        vox, size, radius = prog.export_voxels(VOX_GRID, VOX_COLOR)
    np.testing.assert_array_equal(vox, g["vox_voxels"])
    assert size == tuple(g["vox_size"]) and np.float32(radius) == g["vox_radius"]
    # ExportMagicaVoxel end to end: the file VoxWriter writes for the cell-order voxels.
    path = tmp_path / "model.vox"
    lib.ExportMagicaVoxel(t.handle, VOX_GRID, VOX_COLOR, str(path).encode())
    assert path.read_bytes() == g["vox_file"].tobytes()


@pytest.mark.parametrize("seed,prims,step,refine", [(2, 64, 0.03, 3), (8, 256, 0.05, 5), (5, 16, (0.04, 0.07, 0.05), 0)])
def test_point_cloud_matches_oracle(lib, port, seed, prims, step, refine):
    """Finer voxels, a per-axis step, and no refinement, in voxel order against the oracle."""
    spec = W.random_tree(seed, prims)
    h = port.build(spec)
    try:
        b = port.bounds(h)
        o = port.octree(h)
        try:
            pts, cells = port.point_cloud(o, b[:3], b[3:], step, refine)
            normals, colors = port.vertex_attributes(o, pts)
        finally:
            port.octree_free(o)
    finally:
        port.free(h)
    with sdf.compile(sdf.from_spec(spec)) as prog:
        m = prog.export_point_cloud(b[:3], b[3:], step, refine)
    assert pts.shape[0] > 500
    np.testing.assert_array_equal(m.cubes, cells.astype(np.uint32))
    np.testing.assert_array_equal(m.vertices, pts)
    np.testing.assert_array_equal(m.normals, normals)
    np.testing.assert_array_equal(m.colors, colors)


@pytest.mark.parametrize("seed,prims,grid,color", [(6, 256, 12.0, -300), (1, 16, 30.0, 254)])
def test_voxels_match_oracle(lib, port, seed, prims, grid, color):
    spec = W.random_tree(seed, prims)
    h = port.build(spec)
    try:
        want, size, radius = port.vox(h, grid, color)
    finally:
        port.free(h)
    with sdf.compile(sdf.from_spec(spec)) as prog:
        vox, gsize, gradius = prog.export_voxels(grid, color)
    assert want.shape[0] > 100
    np.testing.assert_array_equal(vox, want)
    assert gsize == size and np.float32(gradius) == np.float32(radius)


def test_mesh_export_entry(lib, golden, tmp_path):
    """MeshExport: the point cloud written as PLY (scaled), the mesh as PLY and STL, and the
    formats the reference writes nothing for."""
    g = golden["cfg1_seed1"]
    t = sdf.from_spec(g["spec"])
    with sdf.compile(t) as prog:
        lo, hi = bounds_of(prog)
    sdf.mesh_export(t, tmp_path / "cloud.ply", lo, hi, CLOUD_STEP, CLOUD_REFINE, "ply", point_cloud=True, scale=2.0)
    _, p, n, c, f = O.read_ply(tmp_path / "cloud.ply")
    assert f.shape[0] == 0
    rows = canonical_rows(p, n, c)
    want = g["cloud_rows"].copy()
    want[:, :3] = (want[:, :3].view(np.float32) * np.float32(2.0)).view(np.uint32)
    np.testing.assert_array_equal(rows, canonical_rows(want[:, :3].view(np.float32), want[:, 3:6].view(np.float32),
                                                       want[:, 6:9] if want.shape[1] > 6 else None))
    sdf.mesh_export(t, tmp_path / "mesh.ply", lo, hi, 0.05, 0, "ply")
    _, mp, mn, mc, mf = O.read_ply(tmp_path / "mesh.ply")
    assert mp.shape[0] > 100 and mf.shape[0] > 100
    sdf.mesh_export(t, tmp_path / "mesh.stl", lo, hi, 0.05, 0, "stl")
    assert (tmp_path / "mesh.stl").stat().st_size == 84 + 50 * mf.shape[0]
    for fmt, cloud, step in (("vox", False, 0.05), ("stl", True, 0.05), ("ply", False, (0.05, -0.06, 0.05))):
        with pytest.raises(_lib.TangerineError):
            sdf.mesh_export(t, tmp_path / "x", lo, hi, step, 0, fmt, point_cloud=cloud)


def test_async_mesh_export_progress_halt_and_rerun(lib, tmp_path):
    """MeshExport returns at once and writes the same bytes as the synchronous calls; while
    it waits before its write, GetExportProgress reports stage 3 with the generation and
    attribute stages complete; a halt there writes no file and ends the job with
    TG_ERR_CANCELLED; the next export runs to the end."""
    t = sdf.from_spec(W.random_tree(1, 16, ops=W.OPS_UNIFORM4))
    lo, hi, step = (-2.0, -2.0, -2.0), (2.0, 2.0, 2.0), 4.0 / 128
    with sdf.compile(t) as prog:
        sdf.write_ply(prog.export_mesh(sdf.export_grid(lo, hi, step)), tmp_path / "want.ply")
    want = (tmp_path / "want.ply").read_bytes()
    lib.tg_debug_export_pause(3)
    try:
        sdf.mesh_export(t, tmp_path / "a.ply", lo, hi, step, 0, "ply", wait=False)
        assert lib.tg_debug_export_paused(60000) == 1
        assert sdf.export_progress() == (3, 1.0, 0.0, 1.0, 0.0)
        assert not (tmp_path / "a.ply").exists()
        lib.tg_debug_export_pause(0)
        assert sdf.export_result() == 0
        assert sdf.export_progress() == (0, 1.0, 0.0, 1.0, 1.0)
        assert (tmp_path / "a.ply").read_bytes() == want
        lib.tg_debug_export_pause(3)
        sdf.mesh_export(t, tmp_path / "b.ply", lo, hi, step, 0, "ply", wait=False)
        assert lib.tg_debug_export_paused(60000) == 1
        sdf.cancel_export(True)
        assert sdf.export_result() == 7
        assert not (tmp_path / "b.ply").exists()
    finally:
        lib.tg_debug_export_pause(0)
    sdf.mesh_export(t, tmp_path / "c.ply", lo, hi, step, 0, "ply")
    assert (tmp_path / "c.ply").read_bytes() == want


def test_mesh_export_per_axis_step(lib, port, tmp_path):
    """MeshExportThread's vec3 Step: a different step per axis (z with the most cells, so
    the reference's loop order is the plain one), against the oracle's lattice, surface nets
    and attributes; the culled export equals the dense one; MeshExport writes that mesh."""
    spec = W.random_tree(5, 16, ops=W.OPS_UNIFORM4)
    steps = (0.04, 0.05, 0.03)
    grid = W.export_grid(steps=steps)
    g = sdf.export_grid_axes((-2, -2, -2), (2, 2, 2), steps)
    assert (g.nx, g.ny, g.nz) == (grid.sx + 1, grid.sy + 1, grid.sz + 1)
    assert (g.step, g.step_y, g.step_z) == tuple(float(np.float32(s)) for s in steps)
    t = sdf.from_spec(spec)
    with sdf.compile(t) as prog:
        lat = prog.eval_grid(grid)
        m = prog.export_mesh(grid)
        dense = prog.export_mesh(grid, dense=True)
    h = port.build(spec)
    o = port.octree(h)
    try:
        np.testing.assert_array_equal(lat, port.octree_grid(o, grid))
        want = port.surface_nets(o, grid)
        assert want.vertices.shape[0] > 1000
        np.testing.assert_array_equal(m.vertices, want.vertices)
        np.testing.assert_array_equal(m.cubes.astype(np.uint64), want.cubes)
        np.testing.assert_array_equal(sorted_faces(m.faces), sorted_faces(want.faces))
        normals, colors = port.vertex_attributes(o, want.vertices)
        np.testing.assert_array_equal(m.normals, normals)
        np.testing.assert_array_equal(m.colors, colors)
    finally:
        port.octree_free(o)
        port.free(h)
    for a, b in ((m.vertices, dense.vertices), (m.faces, dense.faces), (m.normals, dense.normals), (m.colors, dense.colors)):
        np.testing.assert_array_equal(a, b)
    sdf.mesh_export(t, tmp_path / "axes.ply", (-2, -2, -2), (2, 2, 2), steps, 0, "ply")
    _, p, n, c, f = O.read_ply(tmp_path / "axes.ply")
    np.testing.assert_array_equal(p, m.vertices)
    np.testing.assert_array_equal(n, m.normals)
    np.testing.assert_array_equal(sorted_faces(f), sorted_faces(m.faces))


def test_exports_of_a_tree_that_is_not_lipschitz(lib, port):
    """An ellipsoid brush (its distance estimate is not 1-Lipschitz): the voxel bricks cannot
    be rejected by a bound, so every voxel is tested, with the same voxels as the oracle."""
    spec = np.array([W.ELLIPSOID, 0.5, 0.3, 0.2, W.ROTATE, 0.2, 0.3, 0.1, 0.927, W.PAINT, 1.0, 0.2, 0.1,
                     W.SPHERE, 0.4, W.MOVE, 0.6, 0.1, 0.0, W.PAINT, 0.1, 0.9, 0.2, W.BLEND_UNION, 0.1], np.float32)
    h = port.build(spec)
    try:
        want, size, radius = port.vox(h, 40.0, 7)
        b = port.bounds(h)
        o = port.octree(h)
        try:
            pts, cells = port.point_cloud(o, b[:3], b[3:], 0.02, 2)
        finally:
            port.octree_free(o)
    finally:
        port.free(h)
    with sdf.compile(sdf.from_spec(spec)) as prog:
        vox, gsize, gradius = prog.export_voxels(40.0, 7)
        m = prog.export_point_cloud(b[:3], b[3:], 0.02, 2)
    assert want.shape[0] > 100 and pts.shape[0] > 100
    np.testing.assert_array_equal(vox, want)
    assert gsize == size
    np.testing.assert_array_equal(m.cubes, cells.astype(np.uint32))
    np.testing.assert_array_equal(m.vertices, pts)


def test_staged_copy_wait_runs_out_and_recovers(lib):
    """The bounded wait for a brick's staged program copy (TG_MESH_STAGED), made to run out
    on purpose with no GPU fault: with the test hook a staging warp waits 1 ms on an
    mbarrier that nothing arrives at, records the failure, waits for its own copy and
    leaves; the export fails with "did not complete in time".  With the hook off the staged
    export equals the unstaged one bit for bit."""
    spec = W.random_tree(3, 64)
    grid = W.export_grid(resolution=96)
    with sdf.compile(sdf.from_spec(spec)) as prog:
        want = prog.export_mesh(grid)
        try:
            assert lib.tg_debug_wait_test(0, 1_000_000) == 0
            with pytest.raises(_lib.TangerineError, match="did not complete in time"):
                prog.export_mesh(grid, staged=True)
        finally:
            assert lib.tg_debug_wait_test(0, 0) == 0
        got = prog.export_mesh(grid, staged=True)
        np.testing.assert_array_equal(got.vertices, want.vertices)
        np.testing.assert_array_equal(got.faces, want.faces)
        np.testing.assert_array_equal(got.normals, want.normals)
