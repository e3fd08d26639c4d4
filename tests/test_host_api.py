"""Host-side logic of the product library against the reference fixtures: the tree API,
program words and the export octree are computed on the CPU and must be bit-exact.
No kernel runs here."""

import ctypes as C
import re

import numpy as np
import pytest

from conftest import ROOT, golden_names
from tangerine_gb300 import _lib, sdf
from tangerine_gb300 import workloads as W


def test_every_declared_symbol_is_exported(lib):
    header = (ROOT / "include" / "tangerine_gb300.h").read_text()
    declared = re.findall(r"^TANGERINE_API\s+[^;(]*?\b(\w+)\s*\(", header, flags=re.M)
    assert len(declared) >= 45
    for name in declared:
        assert hasattr(lib, name), name
        assert name in _lib.SIGNATURES, name


@pytest.mark.parametrize("name", golden_names())
def test_tree_api_matches_reference(lib, golden, name):
    g = golden[name]
    t = sdf.from_spec(g["spec"])
    np.testing.assert_array_equal(t.reference_words(), g["words"])
    got = np.array([t.eval(*p) for p in g["points"][:256]], np.float32)
    np.testing.assert_array_equal(got, g["eval"][:256])
    for i in range(0, 256, 16):
        hit, travel, pos = t.ray_march(g["ray_origins"][i], g["ray_dirs"][i], 256, 1e-4)
        assert hit == bool(g["ray_hit"][i])
        assert np.float32(travel) == g["ray_travel"][i]
        np.testing.assert_array_equal(np.array(pos, np.float32), g["ray_position"][i])


@pytest.mark.parametrize("name", golden_names())
def test_host_octree_matches_reference(lib, golden, name):
    g = golden[name]
    t = sdf.from_spec(g["spec"])
    dump = t.debug_octree()
    if "octree_nodes" not in g:
        assert dump is None
        return
    cells, children, words = dump
    np.testing.assert_array_equal(cells, g["octree_nodes"])
    np.testing.assert_array_equal(children, g["octree_children"])
    np.testing.assert_array_equal(words, g["octree_words"])


@pytest.mark.parametrize("name", golden_names())
def test_root_program_is_node_zero_program(lib, golden, name):
    """tg_export_tree runs the exact brick test on the root cell's program as soon as the
    root is clipped, before the octree below it exists: that program must be the one the
    finished compile gives node 0 (pivot, clip radius with its non-Lipschitz sign, and
    every record)."""
    g = golden[name]
    t = sdf.from_spec(g["spec"])
    q, d = C.c_int64(), C.c_int32()
    st = lib.tg_debug_root_program_check(t.handle, C.byref(q), C.byref(d))
    if "octree_nodes" not in g:
        assert st == 2   # TG_ERR_UNBOUNDED: no octree, so no export either
        return
    assert st == 0, lib.tg_last_error()
    assert q.value >= 2 and d.value >= 1


@pytest.mark.parametrize("name", golden_names())
def test_deferred_surface_programs_give_the_whole_image(lib, golden, name):
    """tg_export_tree compiles without the surface programs, uploads, and emits them into
    the staged image while the GPU runs the first stages; the finished image must be the
    whole compile's, record for record."""
    g = golden[name]
    t = sdf.from_spec(g["spec"])
    st = lib.tg_debug_deferred_surfaces_check(t.handle)
    if "octree_nodes" not in g:
        assert st == 2
        return
    assert st == 0, lib.tg_last_error()


def test_deferred_surface_programs_random_trees(lib):
    for ops in (None, W.OPS_UNIFORM4):
        for seed in range(10):
            for n in (1, 3, 17, 96, 256):
                t = sdf.from_spec(W.random_tree(seed, n, **({} if ops is None else {"ops": ops})))
                st = lib.tg_debug_deferred_surfaces_check(t.handle)
                assert st == (0 if sdf.has_export_octree(t) else 2), (seed, n, lib.tg_last_error())


@pytest.mark.parametrize("ops", [None, "uniform4"])
def test_root_program_is_node_zero_program_random_trees(lib, ops):
    q, d = C.c_int64(), C.c_int32()
    kw = {} if ops is None else {"ops": W.OPS_UNIFORM4}
    for seed in range(12):
        for n in (1, 2, 9, 64, 256):
            t = sdf.from_spec(W.random_tree(seed, n, **kw))
            st = lib.tg_debug_root_program_check(t.handle, C.byref(q), C.byref(d))
            if not sdf.has_export_octree(t):
                assert st == 2
                continue
            assert st == 0, (seed, n, lib.tg_last_error())


def test_operators_take_over_operands(lib):
    a = sdf.sphere(0.5)
    b = sdf.box(0.3, 0.3, 0.3).move(0.4, 0, 0)
    u = sdf.union(a, b)
    assert a.handle.value is None and b.handle.value is None
    assert u.eval(0, 0, 0) == pytest.approx(-0.5)
    assert u.finite()


def test_clip_tree_semantics(lib):
    t = sdf.union(sdf.sphere(0.5), sdf.sphere(0.5).move(3, 0, 0))
    near = t.clip((0, 0, 0), 0.6)
    assert near is not None
    assert near.eval(3, 0, 0) == pytest.approx(2.5)       # far sphere clipped away
    assert t.clip((10, 10, 10), 0.1) is None


def test_plane_only_tree_has_no_octree(lib):
    t = sdf.plane(0, 0, 1)
    assert not t.finite()
    assert t.debug_octree() is None


def test_malformed_spec_is_rejected(lib):
    with pytest.raises(_lib.TangerineError):
        sdf.from_spec(np.array([W.UNION], np.float32))
    with pytest.raises(_lib.TangerineError):
        sdf.from_spec(np.array([W.SPHERE, 0.5, W.SPHERE, 0.2], np.float32))
    with pytest.raises(_lib.TangerineError):
        sdf.from_spec(np.array([99.0], np.float32))


def test_export_lattice_matches_mesh_export_thread(lib):
    for res, cells in ((128, 130), (512, 514), (1024, 1026)):
        g = sdf.export_grid((-2, -2, -2), (2, 2, 2), 4.0 / res)
        assert (g.nx, g.ny, g.nz) == (cells + 1,) * 3
        w = W.export_grid(resolution=res)
        assert (w.sx, w.x0, w.step) == (cells, g.x0, g.step)


@pytest.mark.parametrize("name", golden_names())
def test_host_meshing_octree_matches_reference(lib, golden, name):
    """Sodapop's two-stage meshing octree, built by the product's host code."""
    g = golden[name]
    dump = sdf.from_spec(g["spec"]).debug_octree(meshing=True)
    if "meshing_nodes" not in g:
        assert dump is None
        return
    cells, children, words = dump
    np.testing.assert_array_equal(cells, g["meshing_nodes"])
    np.testing.assert_array_equal(children, g["meshing_children"])
    np.testing.assert_array_equal(words, g["meshing_words"])


def _point_cache_boxes(nodes, grid):
    """The reference's aligned leaf boxes (sodapop.cpp:630-633) in float32 arithmetic, for
    the terminus cells that hold an evaluator, in depth-first order."""
    f = np.float32
    origin, step = grid[0:3].astype(f), grid[3:6].astype(f)
    leaves = nodes[(nodes[:, 9] == 1) & (nodes[:, 10] == 1)]
    lo = np.floor(np.maximum(f(0), leaves[:, 3:6] - origin) / step)
    hi = np.ceil((leaves[:, 6:9] - origin) / step)
    return np.stack([lo[:, 0], hi[:, 0], lo[:, 1], hi[:, 1], lo[:, 2], hi[:, 2]], 1).astype(np.int64)


@pytest.mark.parametrize("name", golden_names())
def test_sodapop_plan_matches_reference(lib, golden, name):
    """The meshing lattice and point-cache boxes the product hands its kernels."""
    g = golden[name]
    if "meshing_nodes" not in g:
        pytest.skip("no octree for this tree")
    grid, boxes = sdf.from_spec(g["spec"]).sodapop_plan(float(g["soda_density"]))
    np.testing.assert_array_equal(grid[:9], g["soda_grid"])
    sx, sy, sz = (int(v) for v in g["soda_grid"][6:9])
    cells = sx * sy * sz
    bucket = min(64, cells)
    limit = (cells + bucket - 1) // bucket * bucket
    assert int(grid[9]) == limit and int(grid[10]) == (limit - 1) // (sx * sy) + 2
    np.testing.assert_array_equal(boxes, _point_cache_boxes(g["meshing_nodes"], g["soda_grid"]))


@pytest.mark.parametrize("name", golden_names())
def test_vox_writer_matches_voxwriter(lib, golden, name, tmp_path):
    """The product's MagicaVoxel writer against the bytes VoxWriter wrote for the same voxels
    added in the same (cell) order."""
    g = golden[name]
    if "vox_file" not in g:
        pytest.skip("unbounded tree")
    path = tmp_path / "out.vox"
    sdf.write_vox(g["vox_voxels"], g["vox_size"], path)
    assert path.read_bytes() == g["vox_file"].tobytes()


def test_vox_writer_splits_large_volumes(lib, tmp_path):
    """More than 126 voxels a side: several cubes, their translations, and the empty file."""
    from oracle import oracle as O
    rng = np.random.RandomState(3)
    pts = np.unique(rng.randint(0, 300, (4000, 3)), axis=0)
    order = np.lexsort((pts[:, 0], pts[:, 1], pts[:, 2]))
    vox = np.concatenate([pts[order], np.full((len(order), 1), 7)], 1).astype(np.int32)
    sdf.write_vox(vox, (300, 300, 300), tmp_path / "big.vox")
    version, models, trans = O.read_vox(tmp_path / "big.vox")
    assert version == 150 and len(models) == len(trans) == 27
    assert sum(m[1].shape[0] for m in models) == vox.shape[0]
    assert all(m[0] == (127, 127, 127) for m in models)
    sdf.write_vox(np.zeros((0, 4), np.int32), (4, 4, 4), tmp_path / "empty.vox")
    assert O.read_vox(tmp_path / "empty.vox")[1] == []
    R = O.reference()
    if R is None:
        return      # VoxWriter itself is only here where the reference sources are
    for name, v, size in (("big", vox, (300, 300, 300)), ("empty", np.zeros((0, 4), np.int32), (4, 4, 4)),
                          ("shuffled", vox[rng.permutation(len(vox))], (300, 200, 150))):
        R.vox_write(v, size, tmp_path / f"ref_{name}.vox")
        sdf.write_vox(v, size, tmp_path / f"own_{name}.vox")
        assert (tmp_path / f"own_{name}.vox").read_bytes() == (tmp_path / f"ref_{name}.vox").read_bytes(), name


def test_drawable_writer_matches_reference(lib, golden, tmp_path):
    """MeshExport(Path, UseBaseColor, ...) over two placed Sodapop drawables: the product's
    PLY and STL bytes against the reference's gather and writers."""
    from conftest import GOLDEN
    w = np.load(GOLDEN / "writer_drawables.npz")
    drawables = []
    for name in ("cfg1_seed1", "stencil_align"):
        g = golden[name]
        drawables.append(sdf.SodapopDrawable(g["soda_positions"], g["soda_normals"], g["soda_colors"],
                                             g["soda_faces"].astype(np.uint32), np.zeros(0, np.uint32), g["soda_grid"]))
    for fmt in ("ply", "stl"):
        sdf.write_drawables(drawables, tmp_path / f"out.{fmt}", frames=w["frames"], fmt=fmt, scale=float(w["scale"]))
        assert (tmp_path / f"out.{fmt}").read_bytes() == w[f"{fmt}_bytes"].tobytes(), fmt


def test_tree_whose_octants_all_clip_away_has_no_octree(lib, port):
    """A tree whose root cube's eight octants all clip away leaves the root without an
    evaluator: SDFOctree::Create returns nullptr, and so does the host build."""
    spec = W.random_tree(100010, 8)
    h = port.build(spec)
    try:
        assert port.octree(h) is None
        # Sodapop's depth-limited first stage keeps the root's evaluator.
        mo = port.meshing_octree(h)
        want = port.octree_dump(mo)
        port.octree_free(mo)
    finally:
        port.free(h)
    t = sdf.from_spec(spec)
    assert t.finite() and not sdf.has_export_octree(t)
    assert t.debug_octree() is None
    got = t.debug_octree(meshing=True)
    for a, b in zip(got, want):
        np.testing.assert_array_equal(a, b)
    a, b = C.c_double(), C.c_double()
    assert lib.tg_debug_compile_seconds(t.handle, 0, C.byref(a), C.byref(b)) == 2   # TG_ERR_UNBOUNDED


def test_compiles_release_their_clipped_trees_whatever_the_order(lib):
    """The octree's clipped trees borrow the nodes of the tree they were clipped from and
    are released on a background thread after the compile: freeing the tree at once,
    compiling trees back to back, and clipping a tree that is then freed all leave every
    result intact (the host compile only: no device here)."""
    a, b = C.c_double(), C.c_double()
    for seed in range(12):
        spec = W.random_tree(seed, 64 if seed % 2 else 16)
        t = sdf.from_spec(spec)
        want = t.eval(0.1, 0.2, 0.3)
        for _ in range(3):
            assert lib.tg_debug_compile_seconds(t.handle, seed % 2, C.byref(a), C.byref(b)) == 0
        near = t.clip((0.1, 0.2, 0.3), 0.5)
        dump = t.debug_octree()
        del t                                    # the caller's tree goes first
        if near is not None:
            assert near.eval(0.1, 0.2, 0.3) == want   # an owned clip outlives its source
        again = sdf.from_spec(spec).debug_octree()
        for x, y in zip(dump, again):
            np.testing.assert_array_equal(x, y)


def test_process_exits_cleanly_with_releases_pending(lib):
    """Compiles hand their octrees to a background release thread; a process that exits
    right after compiling must still exit at once and cleanly (the pool joins its threads
    after running what is queued)."""
    import subprocess
    import sys
    code = ("import ctypes as C, sys; sys.path.insert(0, %r)\n"
            "from tangerine_gb300 import _lib, sdf, workloads as W\n"
            "lib = _lib.load(); a, b = C.c_double(), C.c_double()\n"
            "for s in range(8):\n"
            "    t = sdf.from_spec(W.random_tree(s, 128))\n"
            "    assert lib.tg_debug_compile_seconds(t.handle, 0, C.byref(a), C.byref(b)) == 0\n"
            "print('ok')\n") % str(ROOT)
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr[-2000:]
    assert r.stdout.strip().endswith("ok")
