"""GPU sphere tracing against SDFNode::RayMarch (reference fixtures and the CPU oracle).

Exact form: the reference's step sequence, so hits, travel and positions must be
bit-identical, and so must the full-tree gradient normals and colours of an exact render.
Octree-bounded form: different (conservative) steps, so it stops at a different point
within the hit epsilon of the surface: hit masks must agree on all but grazing rays and
depths within DEPTH_TOL where both hit."""

import numpy as np
import pytest

from conftest import golden_names
from tangerine_gb300 import sdf
from tangerine_gb300 import workloads as W

pytestmark = pytest.mark.gpu

DEPTH_TOL = 2e-3          # octree-bounded vs exact depth, same ray, both hitting
EPS = 1e-4
STEPS = 256


@pytest.mark.parametrize("name", golden_names())
def test_ray_march_matches_reference(lib, golden, name):
    g = golden[name]
    tree = sdf.from_spec(g["spec"])
    if "octree_nodes" not in g:
        pytest.skip("unbounded tree: no program")
    with sdf.compile(tree) as prog:
        hit, travel, pos = prog.ray_march(g["ray_origins"], g["ray_dirs"], STEPS, EPS)
    np.testing.assert_array_equal(hit, g["ray_hit"])
    np.testing.assert_array_equal(travel, g["ray_travel"])
    np.testing.assert_array_equal(pos, g["ray_position"])


@pytest.mark.parametrize("seed,prims", [(1, 16), (2, 256)])
def test_render_exact_and_bounded(lib, port, seed, prims):
    spec = W.random_tree(seed, prims, ops=W.OPS_UNIFORM4 if prims == 16 else W.OPS_60_20_10_10)
    width, height = 48, 32
    poses = W.camera_poses(seed, 2, radius=4.0)
    cams = sdf.cameras(poses, fov_y_degrees=60.0)
    tan_half = cams[0].tan_half_fov
    with sdf.compile(sdf.from_spec(spec)) as prog:
        d_exact, n_exact, c_exact = prog.render(cams, width, height, STEPS, EPS, exact=True)
        d_fast, n_fast, c_fast = prog.render(cams, width, height, STEPS, EPS, exact=False)
    h = port.build(spec)
    try:
        for i, p in enumerate(poses):
            o, d = W.camera_rays(p, width, height, tan_half)
            hit, travel, pos = port.raymarch(h, o, d, STEPS, EPS, threads=0)
            np.testing.assert_array_equal(d_exact[i].reshape(-1), travel)
            normals = np.zeros((hit.size, 3), np.float32)
            colors = np.zeros((hit.size, 3), np.uint8)
            if hit.any():
                normals[hit] = port.gradient(h, pos[hit])
                colors[hit] = port.color(h, pos[hit])
            np.testing.assert_array_equal(n_exact[i].reshape(-1, 3), normals)
            np.testing.assert_array_equal(c_exact[i].reshape(-1, 3), colors)

            fast_hit = np.isfinite(d_fast[i].reshape(-1))
            assert np.mean(fast_hit != hit) <= 0.01
            both = fast_hit & hit
            assert both.sum() > 0
            assert np.max(np.abs(d_fast[i].reshape(-1)[both] - travel[both])) <= DEPTH_TOL
    finally:
        port.free(h)
