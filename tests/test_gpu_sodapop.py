"""Sodapop's meshing job on the GPU (tg_sodapop_mesh) against the reference fixtures and
the CPU oracle.

Positions, normals, cell numbers and faces are bit-exact.  Colours are MaterialPBRBR's
RGB x (D + F/4) with D = pow(max(dot(N, H), 0), 2): the kernels square with one correctly
rounded product where the reference calls the C library's powf, which may round the square
the other way, so colours are compared within 2 ulp (one for the square, one carried
through the sum and the product)."""

import numpy as np
import pytest

from conftest import golden_names, sorted_faces
from tangerine_gb300 import _lib, sdf
from tangerine_gb300 import workloads as W

pytestmark = pytest.mark.gpu

COLOR_ULP = 2


def check_against(d, positions, normals, colors, faces, grid, ordered_faces):
    np.testing.assert_array_equal(d.grid, grid)
    np.testing.assert_array_equal(d.positions, positions)
    np.testing.assert_array_equal(d.normals, normals)
    np.testing.assert_array_max_ulp(d.colors, colors, maxulp=COLOR_ULP)
    assert np.all(d.colors[:, 3] == 1.0)
    if ordered_faces:
        np.testing.assert_array_equal(d.faces.astype(np.uint64), np.asarray(faces, np.uint64))
    else:
        np.testing.assert_array_equal(sorted_faces(d.faces), sorted_faces(faces))


@pytest.mark.parametrize("name", golden_names())
def test_sodapop_matches_reference(lib, golden, name):
    g = golden[name]
    t = sdf.from_spec(g["spec"])
    if "soda_grid" not in g:
        with pytest.raises(_lib.TangerineError):
            t.sodapop_mesh(6.0)
        return
    d = t.sodapop_mesh(float(g["soda_density"]))
    check_against(d, g["soda_positions"], g["soda_normals"], g["soda_colors"], g["soda_faces"], g["soda_grid"], False)
    assert np.all(np.diff(d.cells.astype(np.int64)) > 0)
    sx, sy, sz = (int(v) for v in g["soda_grid"][6:9])
    assert int(d.cells[-1]) < ((sx * sy * sz + 63) // 64) * 64


@pytest.mark.parametrize("seed,prims,density", [(3, 64, 20.0), (11, 256, 20.0), (4, 16, 33.5)])
def test_sodapop_matches_oracle_at_full_density(lib, port, seed, prims, density):
    """Sodapop's own density (20 samples per unit) and a fractional one (floored to 33)."""
    spec = W.random_tree(seed, prims)
    h = port.build(spec)
    try:
        want = port.sodapop(h, density=density)
    finally:
        port.free(h)
    d = sdf.from_spec(spec).sodapop_mesh(density)
    assert d.positions.shape[0] > 100
    check_against(d, want.positions, want.normals, want.colors, want.faces, want.grid, True)


def test_sodapop_small_and_tiny_lattices(lib, port):
    """Shapes far smaller than the lattice's 8-samples-per-axis floor: one octree cell, and
    a lattice whose steps differ per axis."""
    for spec in (np.array([W.SPHERE, 0.01], np.float32), np.array([W.BOX, 0.05, 0.3, 0.05], np.float32)):
        h = port.build(spec)
        try:
            want = port.sodapop(h, density=1.0)
        finally:
            port.free(h)
        d = sdf.from_spec(spec).sodapop_mesh(1.0)
        check_against(d, want.positions, want.normals, want.colors, want.faces, want.grid, True)


def test_sodapop_rejects_unbounded_and_bad_density(lib):
    with pytest.raises(_lib.TangerineError):
        sdf.plane(0, 0, 1).sodapop_mesh(20.0)
    with pytest.raises(_lib.TangerineError):
        sdf.sphere(0.5).sodapop_mesh(float("nan"))
