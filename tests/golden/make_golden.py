"""Writes the golden fixtures in this folder from Tangerine's own CPU code.

Run here, where the reference sources are: it builds oracle/_ref/libtangerine_ref.so
(``make -C oracle ref``) and records, for a handful of seeded and hand-made CSG trees,
what the reference computes: program words, the export octree, point distances,
gradients and colours, naive-surface-nets meshes on small export lattices (with the
reference's gradient normals and colours per vertex), RayMarch hits, and Sodapop's meshing
job (its octree and its drawable at a reduced density).  The reference
sources do not travel to the GPU host; these fixtures do.

    python tests/golden/make_golden.py
"""

from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from oracle import oracle as O  # noqa: E402
from tangerine_gb300 import workloads as W  # noqa: E402

OUT = Path(__file__).resolve().parent
# Sodapop::Populate meshes at 20 samples per unit; 6 keeps the fixtures small.
SODAPOP_DENSITY = 6.0
# PointCloudExportThread at 0.1-unit voxels with the app's 5 refinement steps; VoxExport at
# 8 voxels per unit with colour index 3.
CLOUD_STEP, CLOUD_REFINE = 0.1, 5
# A model placement for picking: rotation (w, x, y, z) 35 degrees about y, translation, scale.
_q = W.axis_quaternion(1, 35)
PICK_FRAME = np.array([_q[3], _q[0], _q[1], _q[2], 0.3, -0.2, 0.15, 1.25], np.float32)
VOX_GRID, VOX_COLOR = 8.0, 3


def exotic_specs():
    X = W
    q = W.axis_quaternion
    return {
        "ellipsoid_cone": [X.ELLIPSOID, .5, .3, .7, X.ROTATE, *q(0, 30), X.PAINT, .2, .4, .6,
                           X.CONE, .4, .8, X.MOVE, .3, .1, -.2, X.PAINT, .9, .1, .1, X.BLEND_INTER, .15],
        "coninder_flate_scale": [X.CONINDER, .3, .5, .9, X.SCALE, 1.3, X.FLATE, .1, X.BOX, .3, .2, .4, X.ROTATE, *q(2, 47),
                                 X.PAINT, .5, .5, .1, X.BLEND_DIFF, .2, X.MOVE, .1, .2, .3],
        "plane_inter": [X.SPHERE, .8, X.PAINT, 1, 0, 0, X.PLANE, .3, 1., .2, X.PAINT, 0, 1, 0, X.INTER,
                        X.TORUS, .6, .2, X.ROTATE, *q(1, 20), X.UNION],
        "stencil_align": [X.BOX, .6, .5, .4, X.PAINT, .1, .2, .3, X.SPHERE, .5, X.MOVE, .4, 0, 0, X.STENCIL, 1, .7, .8, .9,
                          X.ALIGN, -1, 0, 1, X.CYLINDER, .2, .8, X.SCALE, .7, X.UNION],
        "scaled_blend": [X.SPHERE, .5, X.SPHERE, .4, X.MOVE, .5, 0, 0, X.BLEND_UNION, .2, X.SCALE, 1.7,
                         X.ROTATE, *q(2, 33), X.TORUS, .5, .1, X.DIFF],
        "unpainted_union": [X.BOX, .5, .5, .5, X.SPHERE, .6, X.MOVE, .3, .3, .3, X.UNION],
    }


def cases():
    out = {}
    for seed in (1, 5, 9):
        out[f"cfg1_seed{seed}"] = (W.random_tree(seed, 16, ops=W.OPS_UNIFORM4), 48)
    out["mix64_seed7"] = (W.random_tree(7, 64), 40)
    for name, spec in exotic_specs().items():
        out[name] = (np.asarray(spec, np.float32), 40)
    return out


def canonical_rows(points, normals, colors):
    """Point-cloud rows sorted by their bits: the reference's threads write them in a
    run-dependent order."""
    cols = [points.view(np.uint32), normals.view(np.uint32)]
    if colors is not None:
        cols.append(colors.astype(np.uint32))
    a = np.concatenate(cols, 1)
    return a[np.lexsort(a.T[::-1])]


def voxel_cubes(path):
    """The multiset of (model size, sorted voxel records) of a .vox file: independent of
    the order in which a writer was given the voxels."""
    _, models, _ = O.read_vox(path)
    keys = []
    for size, vox in models:
        v = vox[np.lexsort(vox.T[::-1])]
        keys.append((size, v.tobytes()))
    return sorted(keys)


def add_point_cloud_and_voxels(R, h, b, rec):
    import tempfile
    with tempfile.TemporaryDirectory() as d:
        R.point_cloud_file(h, b[:3], b[3:], CLOUD_STEP, CLOUD_REFINE, f"{d}/cloud.ply")
        _, p, n, c, _ = O.read_ply(f"{d}/cloud.ply")
        rec["cloud_rows"] = canonical_rows(p, n, c)
        rec["cloud_has_color"] = np.int32(c is not None)
        vox, size, radius = R.vox_serial(h, VOX_GRID, VOX_COLOR, f"{d}/serial.vox")
        R.vox_file(h, VOX_GRID, VOX_COLOR, f"{d}/threaded.vox")
        # The shipped, threaded VoxExport must hold the same cubes of voxels as the serial
        # replay (its cube order and one translation follow the threads' timing).
        assert voxel_cubes(f"{d}/serial.vox") == voxel_cubes(f"{d}/threaded.vox")
        rec["vox_voxels"] = vox
        rec["vox_size"] = np.array(size, np.int32)
        rec["vox_radius"] = np.float32(radius)
        rec["vox_file"] = np.frombuffer(Path(f"{d}/serial.vox").read_bytes(), np.uint8)


def main():
    R = O.reference()
    if R is None:
        raise SystemExit("the reference sources are not available here")
    rng = np.random.RandomState(1234)
    points = rng.uniform(-2.0, 2.0, (2048, 3)).astype(np.float32)
    ray_o = W.camera_poses(77, 256, radius=4.0)
    ray_d = (rng.uniform(-0.3, 0.3, (256, 3)) - ray_o / 4.0).astype(np.float32)
    magnet_targets = rng.uniform(-0.6, 0.6, (256, 3)).astype(np.float32)
    for name, (spec, res) in cases().items():
        h = R.build(spec)
        rec = {"spec": spec, "points": points, "resolution": np.int32(res)}
        rec["words"] = R.compile(h)
        rec["stack_size"] = np.int32(R.stack_size(h))
        rec["bounds"] = R.bounds(h)
        rec["inner_bounds"] = R.bounds(h, inner=True)
        rec["eval"] = R.eval(h, points)
        rec["interp_eval"] = R.interp_eval(h, points)
        rec["gradient"] = R.gradient(h, points[:512])
        rec["color"] = R.color(h, points[:512])
        hit, travel, pos = R.raymarch(h, ray_o, ray_d, iterations=256, epsilon=1e-4, threads=1)
        rec.update(ray_origins=ray_o, ray_dirs=ray_d, ray_hit=hit, ray_travel=travel, ray_position=pos)
        # Lua's magnet cast toward targets near the origin, and SDFModel::RayMarch on the tree
        # placed with a rotation, translation and scale.
        hit, travel, pos = R.ray_query(h, 1, ray_o, magnet_targets, iterations=100, epsilon=1e-3)
        rec.update(magnet_targets=magnet_targets, magnet_hit=hit, magnet_travel=travel, magnet_position=pos)
        hit, travel, pos = R.ray_query(h, 2, ray_o, ray_d, frame=PICK_FRAME)
        rec.update(pick_frame=PICK_FRAME, pick_hit=hit, pick_travel=travel, pick_position=pos)
        o = R.octree(h)
        if o is not None:
            nodes, children, words = R.octree_dump(o)
            rec.update(octree_nodes=nodes, octree_children=children, octree_words=words)
            rec["octree_eval"] = R.octree_eval(o, points)
            g = W.export_grid(resolution=res)
            m = R.surface_nets(o, g, threads=1)
            rec["grid"] = np.array([g.x0, g.y0, g.z0, g.step, g.sx, g.sy, g.sz], np.float64)
            rec["mesh_vertices"] = m.vertices
            rec["mesh_cubes"] = m.cubes
            rec["mesh_faces"] = m.faces
            rec["mesh_normals"] = R.octree_gradient(o, m.vertices)
            rec["mesh_colors"] = R.octree_color(o, m.vertices)
            R.octree_free(o)
        if R.has_finite_bounds(h):
            add_point_cloud_and_voxels(R, h, R.bounds(h), rec)
        mo = R.meshing_octree(h)
        if mo is not None:
            nodes, children, words = R.octree_dump(mo)
            rec.update(meshing_nodes=nodes, meshing_children=children, meshing_words=words)
            R.octree_free(mo)
            d = R.sodapop(h, density=SODAPOP_DENSITY)
            rec.update(soda_density=np.float32(SODAPOP_DENSITY), soda_grid=d.grid, soda_positions=d.positions,
                       soda_normals=d.normals, soda_colors=d.colors, soda_faces=d.faces.astype(np.uint32))
        R.free(h)
        np.savez_compressed(OUT / f"{name}.npz", **rec)
        print(name, "vertices", rec.get("mesh_vertices", np.zeros((0, 3))).shape[0])


def drawables_fixture(R):
    """Two Sodapop drawables from the fixtures, placed by two frames, written by the
    reference's MeshExport(Path, UseBaseColor=True, ...) gather and writers."""
    import tempfile
    recs = [np.load(OUT / f"{n}.npz") for n in ("cfg1_seed1", "stencil_align")]   # tree fixtures written above
    drawables = [(r["soda_positions"], r["soda_normals"], r["soda_colors"], r["soda_faces"]) for r in recs]
    frames = np.stack([PICK_FRAME, np.array([1, 0, 0, 0, -1.5, 2.0, 0.25, 0.5], np.float32)])
    out = {"frames": frames, "scale": np.float32(1.5)}
    with tempfile.TemporaryDirectory() as d:
        for fmt in ("ply", "stl"):
            R.write_drawables(drawables, frames, f"{d}/out.{fmt}", fmt=fmt, scale=1.5)
            out[f"{fmt}_bytes"] = np.frombuffer(Path(f"{d}/out.{fmt}").read_bytes(), np.uint8)
    np.savez_compressed(OUT / "writer_drawables.npz", **out)


if __name__ == "__main__":
    main()
    drawables_fixture(O.reference())
