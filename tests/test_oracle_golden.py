"""The C restatement (oracle/port) against fixtures written by Tangerine's own code.

Everything here is bit-exact: the oracle keeps the reference's float operation order."""

import numpy as np
import pytest

from conftest import canonical_rows, golden_names, sorted_faces
from tangerine_gb300 import workloads as W


@pytest.mark.parametrize("name", golden_names())
def test_tree_semantics(port, golden, name):
    g = golden[name]
    h = port.build(g["spec"])
    try:
        np.testing.assert_array_equal(port.compile(h), g["words"])
        assert port.stack_size(h) == int(g["stack_size"])
        np.testing.assert_array_equal(port.bounds(h), g["bounds"])
        np.testing.assert_array_equal(port.bounds(h, inner=True), g["inner_bounds"])
        np.testing.assert_array_equal(port.eval(h, g["points"]), g["eval"])
        np.testing.assert_array_equal(port.interp_eval(h, g["points"]), g["interp_eval"])
        np.testing.assert_array_equal(port.gradient(h, g["points"][:512]), g["gradient"])
        np.testing.assert_array_equal(port.color(h, g["points"][:512]), g["color"])
        hit, travel, pos = port.raymarch(h, g["ray_origins"], g["ray_dirs"], iterations=256, epsilon=1e-4, threads=1)
        np.testing.assert_array_equal(hit, g["ray_hit"])
        np.testing.assert_array_equal(travel, g["ray_travel"])
        np.testing.assert_array_equal(pos, g["ray_position"])
    finally:
        port.free(h)


@pytest.mark.parametrize("name", golden_names())
def test_octree_and_mesh(port, golden, name):
    g = golden[name]
    if "octree_nodes" not in g:
        pytest.skip("no octree for this tree")
    h = port.build(g["spec"])
    o = port.octree(h)
    try:
        nodes, children, words = port.octree_dump(o)
        np.testing.assert_array_equal(nodes, g["octree_nodes"])
        np.testing.assert_array_equal(children, g["octree_children"])
        np.testing.assert_array_equal(words, g["octree_words"])
        np.testing.assert_array_equal(port.octree_eval(o, g["points"]), g["octree_eval"])
        x0, y0, z0, step, sx, sy, sz = g["grid"]
        grid = W.ExportGrid(float(x0), float(y0), float(z0), float(step), int(sx), int(sy), int(sz))
        for faithful in (False, True):
            m = port.surface_nets(o, grid, threads=2, faithful=faithful)
            np.testing.assert_array_equal(m.vertices, g["mesh_vertices"])
            np.testing.assert_array_equal(m.cubes, g["mesh_cubes"])
            np.testing.assert_array_equal(sorted_faces(m.faces), sorted_faces(g["mesh_faces"]))
        normals, colors = port.vertex_attributes(o, g["mesh_vertices"], threads=2)
        np.testing.assert_array_equal(normals, g["mesh_normals"])
        if colors is not None:
            np.testing.assert_array_equal(colors, g["mesh_colors"])
    finally:
        port.octree_free(o)
        port.free(h)


def test_planted_mistake_is_caught(port, golden):
    """Primitive sizes 0.1% off in the oracle's input must change what the checks compare."""
    g = golden["cfg1_seed1"]
    spec = np.array(g["spec"], np.float32)
    i = 0
    while i < spec.size:
        op = int(spec[i])
        if op <= W.CONINDER:
            spec[i + 1] *= np.float32(1.001)
        i += 1 + W.ARITY[op]
    h = port.build(spec)
    try:
        assert not np.array_equal(port.eval(h, g["points"]), g["eval"])
        assert not np.array_equal(port.compile(h), g["words"])
    finally:
        port.free(h)


@pytest.mark.parametrize("name", golden_names())
def test_sodapop_meshing_job(port, golden, name):
    """Sodapop's meshing octree and drawable (MeshingJob::NaiveSurfaceNets) against the
    reference's serial replay: vertices, normals and colours in cell order, faces as a set
    (the reference's face order follows its own vertex traversal)."""
    g = golden[name]
    if "meshing_nodes" not in g:
        pytest.skip("no octree for this tree")
    h = port.build(g["spec"])
    try:
        mo = port.meshing_octree(h)
        try:
            nodes, children, words = port.octree_dump(mo)
        finally:
            port.octree_free(mo)
        np.testing.assert_array_equal(nodes, g["meshing_nodes"])
        np.testing.assert_array_equal(children, g["meshing_children"])
        np.testing.assert_array_equal(words, g["meshing_words"])
        d = port.sodapop(h, density=float(g["soda_density"]))
        np.testing.assert_array_equal(d.grid, g["soda_grid"])
        np.testing.assert_array_equal(d.positions, g["soda_positions"])
        np.testing.assert_array_equal(d.normals, g["soda_normals"])
        np.testing.assert_array_equal(d.colors, g["soda_colors"])
        np.testing.assert_array_equal(sorted_faces(d.faces), sorted_faces(g["soda_faces"]))
    finally:
        port.free(h)


CLOUD_STEP, CLOUD_REFINE, VOX_GRID, VOX_COLOR = 0.1, 5, 8.0, 3


@pytest.mark.parametrize("name", golden_names())
def test_point_cloud_and_voxels(port, golden, name):
    """PointCloudExportThread (with the refinement and WritePLY's attributes) and VoxExport's
    voxel test against the reference."""
    g = golden[name]
    if "cloud_rows" not in g:
        pytest.skip("unbounded tree")
    h = port.build(g["spec"])
    try:
        b = port.bounds(h)
        o = port.octree(h)
        try:
            pts, cells = port.point_cloud(o, b[:3], b[3:], CLOUD_STEP, CLOUD_REFINE)
            normals, colors = port.vertex_attributes(o, pts)
        finally:
            port.octree_free(o)
        assert np.all(np.diff(cells) > 0)
        assert (colors is not None) == bool(g["cloud_has_color"])
        np.testing.assert_array_equal(canonical_rows(pts, normals, colors), g["cloud_rows"])
        vox, size, radius = port.vox(h, VOX_GRID, VOX_COLOR)
        np.testing.assert_array_equal(vox, g["vox_voxels"])
        assert size == tuple(g["vox_size"]) and np.float32(radius) == g["vox_radius"]
    finally:
        port.free(h)


@pytest.mark.parametrize("name", golden_names())
def test_framed_ray_casts(port, golden, name):
    """Lua's magnet cast and SDFModel::RayMarch (mouse picking on a placed model)."""
    g = golden[name]
    h = port.build(g["spec"])
    try:
        hit, travel, pos = port.ray_query(h, 1, g["ray_origins"], g["magnet_targets"], iterations=100, epsilon=1e-3)
        np.testing.assert_array_equal(hit, g["magnet_hit"])
        np.testing.assert_array_equal(travel, g["magnet_travel"])
        np.testing.assert_array_equal(pos, g["magnet_position"])
        hit, travel, pos = port.ray_query(h, 2, g["ray_origins"], g["ray_dirs"], frame=g["pick_frame"])
        np.testing.assert_array_equal(hit, g["pick_hit"])
        np.testing.assert_array_equal(travel, g["pick_travel"])
        np.testing.assert_array_equal(pos, g["pick_position"])
    finally:
        port.free(h)
