"""GPU export path against the CPU oracle and the reference fixtures, through the C ABI.

Integer/byte outputs (active cells, cube indices, faces, colour bytes) and all float
outputs (distances, vertex positions, normals) are required to be bit-exact: the kernels
reproduce the reference's float32 operation order without fused multiply-adds.  The
tolerance the spec allows (1e-5 absolute on distances and vertices) is therefore 0 here."""

import ctypes as C

import numpy as np
import pytest

from conftest import GOLDEN, golden_names, sorted_faces
from oracle import oracle as O
from tangerine_gb300 import _lib, sdf
from tangerine_gb300 import workloads as W

pytestmark = pytest.mark.gpu

EDGES = [(0, 1), (1, 2), (2, 3), (3, 0), (4, 5), (5, 6), (6, 7), (7, 4), (0, 4), (1, 5), (2, 6), (3, 7)]
CORNERS = [(0, 0, 0), (1, 0, 0), (1, 1, 0), (0, 1, 0), (0, 0, 1), (1, 0, 1), (1, 1, 1), (0, 1, 1)]


def grid_of(g):
    x0, y0, z0, step, sx, sy, sz = g["grid"]
    return W.ExportGrid(float(x0), float(y0), float(z0), float(step), int(sx), int(sy), int(sz))


def lattice_points(grid, i, j, k):
    f = np.float32
    x = f(grid.x0) + i.astype(f) * f(grid.step)
    y = f(grid.y0) + j.astype(f) * f(grid.step)
    z = f(grid.z0) + k.astype(f) * f(grid.step)
    return np.stack([x, y, z], 1).astype(f)


def vertices_from_corners(grid, i, j, k, v):
    """FirstLoopInnerThunk's vertex in float32 (surface_nets.cpp:915-965), vectorised."""
    f = np.float32
    fi, fj, fk = i.astype(f), j.astype(f), k.astype(f)
    s = [np.zeros(len(i), f) for _ in range(3)]
    n = np.zeros(len(i), f)
    for a, b in EDGES:
        s1, s2 = v[:, a], v[:, b]
        bip = (s1 >= 0) != (s2 >= 0)
        with np.errstate(divide="ignore", invalid="ignore"):
            t = (f(0) - s1) / (s2 - s1)
        for ax, base in enumerate((fi, fj, fk)):
            p1 = base + f(CORNERS[a][ax])
            p2 = base + f(CORNERS[b][ax])
            s[ax] = np.where(bip, s[ax] + (p1 + t * (p2 - p1)), s[ax])
        n = n + bip.astype(f)
    out = []
    for ax, (o, cells) in enumerate(((grid.x0, grid.sx), (grid.y0, grid.sy), (grid.z0, grid.sz))):
        o, fs = f(o), f(cells)
        mx = o + fs * f(grid.step)
        c = s[ax] / n
        out.append(o + (mx - o) * (c - f(0)) / (fs - f(0)))
    return np.stack(out, 1).astype(f)


@pytest.mark.parametrize("name", golden_names())
def test_export_matches_reference_fixture(lib, golden, name):
    g = golden[name]
    tree = sdf.from_spec(g["spec"])
    if "octree_nodes" not in g:
        with pytest.raises(_lib.TangerineError):
            sdf.compile(tree)
        return
    with sdf.compile(tree) as prog:
        np.testing.assert_array_equal(prog.eval_points(g["points"]), g["octree_eval"])
        m = prog.export_mesh(grid_of(g))
        # Vertex order is the reference's serial order (cells in x, y, z order).
        np.testing.assert_array_equal(m.vertices, g["mesh_vertices"])
        np.testing.assert_array_equal(m.cubes.astype(np.uint64), g["mesh_cubes"])
        np.testing.assert_array_equal(sorted_faces(m.faces), sorted_faces(g["mesh_faces"]))
        np.testing.assert_array_equal(m.normals, g["mesh_normals"])
        if prog.info().has_paint:
            np.testing.assert_array_equal(m.colors, g["mesh_colors"])
        else:
            assert m.colors is None


@pytest.mark.parametrize("seed", [1, 5, 9])
def test_lattice_matches_oracle_config1(lib, port, seed):
    """16-primitive seeded tree, FP32 over a 128^3 export grid (131^3 lattice points)."""
    spec = W.random_tree(seed, 16, ops=W.OPS_UNIFORM4)
    grid = W.export_grid(resolution=128)
    with sdf.compile(sdf.from_spec(spec)) as prog:
        got = prog.eval_grid(grid)
        m = prog.export_mesh(grid)
    h = port.build(spec)
    o = port.octree(h)
    try:
        np.testing.assert_array_equal(got, port.octree_grid(o, grid))
        want = port.surface_nets(o, grid)
        np.testing.assert_array_equal(m.vertices, want.vertices)
        np.testing.assert_array_equal(m.cubes.astype(np.uint64), want.cubes)
        np.testing.assert_array_equal(sorted_faces(m.faces), sorted_faces(want.faces))
        normals, colors = port.vertex_attributes(o, want.vertices)
        np.testing.assert_array_equal(m.normals, normals)
        np.testing.assert_array_equal(m.colors, colors)
    finally:
        port.octree_free(o)
        port.free(h)


def test_full_size_export_properties(lib, port):
    """256-primitive tree on the 512^3 export grid: sampled lattice values, vertices,
    normals and colours against the oracle, plus mesh invariants over every face."""
    spec = W.random_tree(1, 256)
    grid = W.export_grid(resolution=512)
    rng = np.random.RandomState(0)
    with sdf.compile(sdf.from_spec(spec)) as prog:
        lat = prog.eval_grid(grid)
        m = prog.export_mesh(grid)
    h = port.build(spec)
    o = port.octree(h)
    try:
        n = grid.sx + 1
        idx = rng.randint(0, n, (20000, 3))
        pts = lattice_points(grid, idx[:, 0], idx[:, 1], idx[:, 2])
        np.testing.assert_array_equal(lat[idx[:, 2], idx[:, 1], idx[:, 0]], port.octree_eval(o, pts))

        V = m.vertices.shape[0]
        assert V > 100000
        # active cells: exactly those whose corners straddle zero
        cubes = m.cubes.astype(np.int64)
        assert np.all(np.diff(cubes) > 0)
        sample = rng.choice(V, 5000, replace=False)
        c = cubes[sample]
        i, j, k = c % grid.sx, (c // grid.sx) % grid.sy, c // (grid.sx * grid.sy)
        corner_vals = np.stack([port.octree_eval(o, lattice_points(grid, i + dx, j + dy, k + dz))
                                for dx, dy, dz in CORNERS], 1)
        pos = corner_vals >= 0
        assert np.all(pos.any(1) & ~pos.all(1))
        np.testing.assert_array_equal(m.vertices[sample], vertices_from_corners(grid, i, j, k, corner_vals))
        normals, colors = port.vertex_attributes(o, m.vertices[sample])
        np.testing.assert_array_equal(m.normals[sample], normals)
        np.testing.assert_array_equal(m.colors[sample], colors)

        F = m.faces.astype(np.int64)
        assert F.shape[0] % 2 == 0 and F.max() < V
        # every triangle joins its first vertex's cube to cubes one step below it
        d = cubes[F[:, 1:]] - cubes[F[:, :1]]
        allowed = {-1, -grid.sx, -grid.sx * grid.sy, -1 - grid.sx, -1 - grid.sx * grid.sy,
                   -grid.sx - grid.sx * grid.sy}
        assert set(np.unique(d).tolist()) <= allowed
    finally:
        port.octree_free(o)
        port.free(h)


def test_full_size_mesh_matches_oracle(lib, port):
    """The headline export in full: 256-primitive tree (seed 1) on the 512^3 export grid
    (515^3 lattice points).  Every lattice distance, every vertex (in the reference's serial
    order), cube index, face, normal and colour byte of the GPU's culled export against the
    oracle's surface nets (FirstLoopInnerThunk / SecondLoopThunk, surface_nets.cpp:864-1121)
    and its per-vertex Gradient + GetMaterial (export.cpp:283-317) on all host cores.  The
    end-to-end call (tg_export_tree: tree handle in, host mesh out, bricks classified on the
    root cell's program during the compile) gives the same mesh."""
    spec = W.random_tree(1, 256)
    grid = W.export_grid(resolution=512)
    tree = sdf.from_spec(spec)
    with sdf.compile(tree) as prog:
        m = prog.export_mesh(grid)
        lat = prog.eval_grid(grid)
    e = sdf.export_tree(tree, (-2, -2, -2), (2, 2, 2), 4.0 / 512)
    h = port.build(spec)
    o = port.octree(h)
    try:
        np.testing.assert_array_equal(lat, port.octree_grid(o, grid))
        del lat
        want = port.surface_nets(o, grid)
        assert want.vertices.shape[0] > 1000000
        normals, colors = port.vertex_attributes(o, want.vertices)
        for got in (m, e):
            np.testing.assert_array_equal(got.vertices, want.vertices)
            np.testing.assert_array_equal(got.cubes.astype(np.uint64), want.cubes)
            np.testing.assert_array_equal(sorted_faces(got.faces), sorted_faces(want.faces))
            np.testing.assert_array_equal(got.normals, normals)
            np.testing.assert_array_equal(got.colors, colors)
        np.testing.assert_array_equal(e.faces, m.faces)
    finally:
        port.octree_free(o)
        port.free(h)


@pytest.mark.parametrize("brick", [1, 4, 7, 15])
def test_culled_export_equals_dense_export(lib, brick):
    """Brick culling skips only bricks that provably hold no surface: same mesh, bit for bit."""
    for seed, prims, res in ((1, 16, 128), (3, 256, 96)):
        spec = W.random_tree(seed, prims, ops=W.OPS_UNIFORM4 if prims == 16 else W.OPS_60_20_10_10)
        grid = W.export_grid(resolution=res)
        with sdf.compile(sdf.from_spec(spec)) as prog:
            dense = prog.export_mesh(grid, dense=True)
            culled = prog.export_mesh(grid, brick=brick)
            bricks, active = sdf.last_export_stats()
        assert 0 < active <= bricks
        for a, b in ((dense.vertices, culled.vertices), (dense.faces, culled.faces), (dense.normals, culled.normals),
                     (dense.colors, culled.colors), (dense.cubes, culled.cubes)):
            np.testing.assert_array_equal(a, b)


def test_culled_export_full_size(lib):
    spec = W.random_tree(1, 256)
    grid = W.export_grid(resolution=512)
    with sdf.compile(sdf.from_spec(spec)) as prog:
        dense = prog.export_mesh(grid, dense=True)
        culled = prog.export_mesh(grid)
        bricks, active = sdf.last_export_stats()
        staged = prog.export_mesh(grid, staged=True)
        staged4 = prog.export_mesh(grid, staged=True, lanes=4, brick=15)
    assert active < bricks // 3
    for m in (culled, staged, staged4):
        for a, b in ((dense.vertices, m.vertices), (dense.faces, m.faces), (dense.normals, m.normals),
                     (dense.colors, m.colors)):
            np.testing.assert_array_equal(a, b)


def _spec(which):
    if isinstance(which, str):
        return np.load(GOLDEN / f"{which}.npz", allow_pickle=False)["spec"]
    seed, n, ops = which
    return W.random_tree(seed, n, **({"ops": ops} if ops is not None else {}))


# (tree, lattice min, max, step): trees with blends, stencils and paint, a non-Lipschitz
# ellipsoid (nothing may be culled), a single brush, the 256-brush workload on a ragged
# brick grid, and lattices that reach past the root cube on some sides.
EXPORT_TREE_CASES = [
    ((5, 16, W.OPS_UNIFORM4), (-2, -2, -2), (2, 2, 2), 4.0 / 64),
    ((1, 256, None), (-2, -2, -2), (2, 2, 2), 4.0 / 150),
    ((3, 64, None), (-2.5, -1.0, -2.0), (1.0, 2.5, 2.0), 0.045),
    ((7, 1, None), (-1.5, -1.5, -1.5), (1.5, 1.5, 1.5), 0.05),
    ("ellipsoid_cone", (-2, -2, -2), (2, 2, 2), 4.0 / 80),
    ("stencil_align", (-2, -2, -2), (2, 2, 2), 4.0 / 90),
    ("scaled_blend", (-2.2, -1.7, -2.0), (1.9, 2.3, 1.6), 0.04),
    ("coninder_flate_scale", (-2, -2, -2), (2, 2, 2), 4.0 / 70),
]


@pytest.mark.parametrize("case", range(len(EXPORT_TREE_CASES)))
def test_export_tree_matches_program_export(lib, case):
    """tg_export_tree classifies the bricks on the root cell's program while the host is
    still building the octree, and the list pass descends the kept bricks itself: its mesh
    must be the program export's (holder-cell classification) and the dense export's, bit
    for bit."""
    which, lo, hi, step = EXPORT_TREE_CASES[case]
    t = sdf.from_spec(_spec(which))
    sdf.profile_enable(True)
    sdf.profile_reset()
    try:
        a = sdf.export_tree(t, lo, hi, step)
        _, early = sdf.profile_read("classify_root")
        _, late = sdf.profile_read("classify_bricks")
    finally:
        sdf.profile_enable(False)
    assert (early, late) == (1, 0)
    grid = sdf.export_grid(lo, hi, step)
    with sdf.compile(t) as prog:
        b = prog.export_mesh(grid)
        dense = prog.export_mesh(grid, dense=True)
    assert a.vertices.shape[0] > 0
    for m in (b, dense):
        for x, y in ((a.vertices, m.vertices), (a.cubes, m.cubes), (a.faces, m.faces), (a.normals, m.normals),
                     (a.colors, m.colors)):
            np.testing.assert_array_equal(x, y)


def test_export_tree_of_a_tree_without_octree_then_recovers(lib):
    """The root is clipped (and its early brick test launched) before the build finds that
    every octant clips away: the call fails as SDFOctree::Create would, and the next export
    is whole."""
    t = sdf.from_spec(W.random_tree(100010, 8))
    with pytest.raises(_lib.TangerineError):
        sdf.export_tree(t, (-2, -2, -2), (2, 2, 2), 4.0 / 64)
    u = sdf.from_spec(W.random_tree(5, 16, ops=W.OPS_UNIFORM4))
    a = sdf.export_tree(u, (-2, -2, -2), (2, 2, 2), 4.0 / 64)
    with sdf.compile(u) as prog:
        b = prog.export_mesh(sdf.export_grid((-2, -2, -2), (2, 2, 2), 4.0 / 64), dense=True)
    for x, y in ((a.vertices, b.vertices), (a.faces, b.faces), (a.normals, b.normals), (a.colors, b.colors)):
        np.testing.assert_array_equal(x, y)


def test_ply_file_layout(lib, golden, tmp_path):
    g = golden["cfg1_seed1"]
    with sdf.compile(sdf.from_spec(g["spec"])) as prog:
        m = prog.export_mesh(grid_of(g))
        path = tmp_path / "m.ply"
        sdf.write_ply(m, path)
    header, v, n, c, f = O.read_ply(path)
    assert header.startswith("ply\nformat binary_little_endian 1.0\ncomment Created by Tangerine\n")
    np.testing.assert_array_equal(v, g["mesh_vertices"])
    np.testing.assert_array_equal(n, g["mesh_normals"])
    np.testing.assert_array_equal(c, g["mesh_colors"])
    np.testing.assert_array_equal(sorted_faces(f), sorted_faces(g["mesh_faces"]))


def test_stl_normals_are_centroid_gradients(lib, port, tmp_path):
    spec = W.random_tree(1, 16, ops=W.OPS_UNIFORM4)
    grid = W.export_grid(resolution=40)
    with sdf.compile(sdf.from_spec(spec)) as prog:
        m = prog.export_mesh(grid)
        path = tmp_path / "m.stl"
        sdf.write_stl(prog, m, path)
    data = path.read_bytes()
    assert data[:29] == b"STL generated by TangerineCSG" and data[29:80] == b"\0" * 51
    count = int(np.frombuffer(data[80:84], "<u4")[0])
    assert count == m.faces.shape[0]
    rec = np.frombuffer(data[84:84 + 50 * count], dtype=[("n", "<f4", 3), ("v", "<f4", (3, 3)), ("a", "<u2")])
    tri = m.vertices[m.faces.astype(np.int64)]
    np.testing.assert_array_equal(rec["v"], tri)
    center = ((tri[:, 0] + tri[:, 1]) + tri[:, 2]) / np.float32(3.0)
    h = port.build(spec)
    o = port.octree(h)
    try:
        np.testing.assert_array_equal(rec["n"], port.octree_gradient(o, center))
    finally:
        port.octree_free(o)
        port.free(h)


def test_edge_cases(lib):
    # lattice far from the model: no active cell
    t = sdf.sphere(0.5)
    with sdf.compile(t) as prog:
        empty = prog.export_mesh(_lib.Grid(5.0, 5.0, 5.0, 0.1, 16, 16, 16))
        assert empty.vertices.shape == (0, 3) and empty.faces.shape == (0, 3)
        # smallest lattice: one cell straddling the surface
        one = prog.export_mesh(_lib.Grid(0.4, -0.05, -0.05, 0.2, 2, 2, 2))
        assert one.vertices.shape == (1, 3) and one.faces.shape == (0, 3)
        # everything inside
        inside = prog.export_mesh(_lib.Grid(-0.1, -0.1, -0.1, 0.05, 5, 5, 5))
        assert inside.vertices.shape[0] == 0
        with pytest.raises(_lib.TangerineError):
            prog.export_mesh(_lib.Grid(0, 0, 0, 0.1, 1, 4, 4))
        with pytest.raises(_lib.TangerineError):
            prog.export_mesh(_lib.Grid(0, 0, 0, -0.1, 4, 4, 4))
    with pytest.raises(_lib.TangerineError):
        sdf.compile(sdf.plane(0, 0, 1))


def test_float_blend_term_equals_double(lib):
    """The GPU's float evaluation of the smooth-blend term returns exactly the reference's
    double expression rounded to float wherever it does not defer to the double path."""
    from tangerine_gb300 import _lib
    counts = np.zeros(3, np.uint64)
    _lib.check(lib.tg_debug_blend_check(1 << 26, 12345, _lib.as_ptr(counts)), "tg_debug_blend_check")
    checked, mismatches, fallbacks = (int(c) for c in counts)
    assert mismatches == 0, counts
    assert checked > (1 << 26)          # most inputs take the float path


def test_paired_arithmetic_equals_scalar(lib):
    """The interpreters evaluate two points per FADD2 / FMUL2 instruction; every lane must
    equal the scalar float32 operation bit for bit: single adds and multiplies on arbitrary
    finite bit patterns (subnormals included), a product then a sum (never fused), and the
    brush formulas and affine transform on realistic points."""
    counts = np.zeros(10, np.uint64)
    _lib.check(lib.tg_debug_pair_check(1 << 22, 777, _lib.as_ptr(counts)), "tg_debug_pair_check")
    names = ["add", "mul", "mul+add", "sphere", "box", "torus", "cylinder", "plane", "affine"]
    assert int(counts[0]) == 1 << 22
    bad = {n: int(c) for n, c in zip(names, counts[1:]) if c}
    assert not bad, f"lanes differing from the scalar operations: {bad}"


LUA_MODELS = sorted(np.load(GOLDEN / "lua_models.npz").files)


@pytest.mark.parametrize("name", LUA_MODELS)
def test_lua_model_export_matches_oracle(lib, port, name):
    """Tangerine's own model scripts (models/*.lua), built by the Lua surface and stored as
    tree specs: the GPU lattice and mesh (vertices, cubes, faces, normals, colours) against
    the oracle's, on a cube lattice of 96 cells around the model."""
    spec = np.load(GOLDEN / "lua_models.npz")[name]
    with sdf.compile(sdf.from_spec(spec)) as prog:
        info = prog.info()
        half = float(np.max(np.abs(np.concatenate([info.bounds_min[:], info.bounds_max[:]])))) * 1.05
        grid = W.export_grid(lo=(-half,) * 3, hi=(half,) * 3, resolution=96)
        lat = prog.eval_grid(grid)
        m = prog.export_mesh(grid)
    h = port.build(spec)
    o = port.octree(h)
    try:
        np.testing.assert_array_equal(lat, port.octree_grid(o, grid))
        want = port.surface_nets(o, grid)
        assert want.vertices.shape[0] > 100
        np.testing.assert_array_equal(m.vertices, want.vertices)
        np.testing.assert_array_equal(m.cubes.astype(np.uint64), want.cubes)
        np.testing.assert_array_equal(sorted_faces(m.faces), sorted_faces(want.faces))
        normals, colors = port.vertex_attributes(o, want.vertices)
        np.testing.assert_array_equal(m.normals, normals)
        if colors is None:
            assert m.colors is None
        else:
            np.testing.assert_array_equal(m.colors, colors)
    finally:
        port.octree_free(o)
        port.free(h)


@pytest.mark.parametrize("lanes,staged", [(1, False), (2, False), (4, False), (2, True), (4, True)])
def test_culled_export_on_ragged_grids(lib, lanes, staged):
    """Lattices whose sides are not multiples of the brick edge and differ per axis, with
    per-axis steps: every brick size, lane count and staging gives the dense export's mesh
    bit for bit (the last bricks of each axis are cut by the lattice end)."""
    spec = W.random_tree(9, 64, ops=W.OPS_60_20_10_10)
    grids = [_lib.Grid(-1.9, -1.7, -2.0, 0.061, 53, 37, 61),
             _lib.Grid(-2.0, -1.5, -1.2, 0.05, 71, 44, 30, 0.07, 0.09)]
    with sdf.compile(sdf.from_spec(spec)) as prog:
        for grid in grids:
            dense = prog.export_mesh(grid, dense=True)
            assert dense.vertices.shape[0] > 0
            for brick in (1, 3, 4, 7, 10, 11, 15, 32):
                culled = prog.export_mesh(grid, brick=brick, lanes=lanes, staged=staged)
                for a, b in ((dense.vertices, culled.vertices), (dense.faces, culled.faces),
                             (dense.normals, culled.normals), (dense.colors, culled.colors), (dense.cubes, culled.cubes)):
                    np.testing.assert_array_equal(a, b)
