"""Batched point queries on the whole tree (Lua's eval / gradient, EvalTree) and the app's
framed ray casts (Lua's magnet cast, SDFModel::RayMarch picking), on the GPU against the
reference fixtures.  Bit-exact."""

import numpy as np
import pytest

from conftest import golden_names
from tangerine_gb300 import sdf

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", golden_names())
def test_point_and_ray_queries(lib, golden, name):
    g = golden[name]
    t = sdf.from_spec(g["spec"])
    try:
        prog = sdf.compile(t)
    except Exception:
        pytest.skip("no octree for this tree")
    with prog:
        np.testing.assert_array_equal(prog.eval_tree(g["points"]), g["eval"])
        np.testing.assert_array_equal(prog.gradient_tree(g["points"][:512]), g["gradient"])
        hit, travel, pos = prog.ray_query(1, g["ray_origins"], g["magnet_targets"], iterations=100, epsilon=1e-3)
        np.testing.assert_array_equal(hit, g["magnet_hit"].astype(bool))
        np.testing.assert_array_equal(travel, g["magnet_travel"])
        np.testing.assert_array_equal(pos, g["magnet_position"])
        # The picking cast ignores the caller's iteration count and epsilon, as the reference.
        hit, travel, pos = prog.ray_query(2, g["ray_origins"], g["ray_dirs"], frame=g["pick_frame"], iterations=3, epsilon=0.5)
        np.testing.assert_array_equal(hit, g["pick_hit"].astype(bool))
        np.testing.assert_array_equal(travel, g["pick_travel"])
        np.testing.assert_array_equal(pos, g["pick_position"])
        hit, travel, pos = prog.ray_query(0, g["ray_origins"], g["ray_dirs"], iterations=256, epsilon=1e-4)
        np.testing.assert_array_equal(hit, g["ray_hit"].astype(bool))
        np.testing.assert_array_equal(travel, g["ray_travel"])
