"""The Lua modelling surface (tangerine/lua_sdf.cpp) over the C ABI, on the host: the
reference's argument semantics (diameters halved, n-ary operators folding left, the blend
threshold last, transforms returning new trees), the whole-tree queries, and the tree specs
of Tangerine's own model scripts that tests/golden/lua_models.npz holds (the GPU tests
export those against the oracle).  The Lua runner builds only where Lua 5.4 sources are
present; without them these tests skip."""

import ctypes as C
import subprocess

import numpy as np
import pytest

from conftest import GOLDEN
from oracle import oracle as O
from tangerine_gb300 import _lib, sdf
from tangerine_gb300 import workloads as W
from tangerine_gb300.lua import build as LB

LUA_SRC = O.REFERENCE_SOURCES / "third_party" / "lua-5.4.4" / "lua"


@pytest.fixture(scope="module")
def runner(lib):
    r = LB.build(LUA_SRC)
    if r is None:
        pytest.skip("no Lua 5.4 sources on this host")
    return r


def run(runner, tmp_path, script, name="m.lua"):
    p = tmp_path / name
    p.write_text(script)
    out = subprocess.run([str(runner), str(p)], capture_output=True, text=True)
    line = out.stdout.strip()
    assert out.returncode == 0 and " error:" not in line, line
    return np.array([float(w) for w in line.split()[1:]], np.float32)


def brushes(spec):
    """(op, params, rotation wxyz, translation, scale, paint or None) per brush, in order."""
    out, i = [], 0
    while i < spec.size:
        op = int(spec[i])
        ar = W.ARITY[op]
        if op <= W.CONINDER:
            rec = [op, tuple(spec[i + 1:i + 1 + ar]), None, None, None, None]
            out.append(rec)
        elif op == W.TRANSFORM:
            t = spec[i + 1:i + 9]
            out[-1][2:5] = [tuple(t[:4]), tuple(t[4:7]), float(t[7])]
        elif op == W.PAINT:
            out[-1][5] = tuple(spec[i + 1:i + 4])
        i += 1 + ar
    return out


def ops(spec):
    i, seq = 0, []
    while i < spec.size:
        op = int(spec[i])
        if W.UNION <= op <= W.BLEND_INTER:
            seq.append((op, float(spec[i + 1]) if op >= W.BLEND_UNION else None))
        i += 1 + W.ARITY[op]
    return seq


def test_sizes_are_diameters(runner, tmp_path):
    f32 = np.float32
    spec = run(runner, tmp_path, "model = union(sphere(2), cube(3), box(1, 2, 4), torus(2, .5), cylinder(1, 3), "
                                 "cone(2, 3), coninder(2, 1, 3), ellipsoid(1, 2, 3))")
    got = [(b[0], b[1]) for b in brushes(spec)]
    assert sorted(got) == sorted([
        (W.SPHERE, (f32(1.0),)), (W.BOX, (f32(1.5),) * 3), (W.BOX, (f32(0.5), f32(1.0), f32(2.0))),
        (W.TORUS, (f32(0.75), f32(0.25))), (W.CYLINDER, (f32(0.5), f32(1.5))), (W.CONE, (f32(1.0), f32(3.0))),
        (W.CONINDER, (f32(1.0), f32(0.5), f32(3.0))), (W.ELLIPSOID, (f32(0.5), f32(1.0), f32(1.5)))])


def test_operators_fold_left_and_blend_takes_the_last_argument(runner, tmp_path):
    spec = run(runner, tmp_path, "model = sphere(1):union(sphere(2), sphere(3)):blend_diff(cube(1), cube(2), 0.25)")
    assert ops(spec) == [(W.UNION, None), (W.UNION, None), (W.BLEND_DIFF, 0.25), (W.BLEND_DIFF, 0.25)]


def test_transforms_return_new_trees(runner, tmp_path):
    spec = run(runner, tmp_path, "local a = sphere(1)\nlocal b = a:move_x(2):paint(1, 0, 0)\n"
                                 "local c = a:rotate_z(90):move(0, 1, 0):paint_over('#00ff00')\nmodel = union(a, b, c)")
    (_, _, ra, ta, _, pa), (_, _, rb, tb, _, pb), (_, _, rc, tc, _, pc) = brushes(spec)
    assert ta == (0, 0, 0) and pa is None and ra == (1, 0, 0, 0)
    assert tb == (2, 0, 0) and pb == (1, 0, 0)
    assert tc == (0, 1, 0) and pc == (0, 1, 0) and abs(rc[0] - np.sqrt(0.5)) < 1e-6 and abs(rc[3] - np.sqrt(0.5)) < 1e-6


def test_whole_tree_queries(runner, tmp_path):
    run(runner, tmp_path, """
local s = sphere(2)
assert(math.abs(s:eval(2, 0, 0) - 1) < 1e-6)
local g = s:gradient(0, 3, 0)
assert(math.abs(g[2] - 1) < 1e-3 and math.abs(g[1]) < 1e-3)
local hit = s:ray_cast(-5, 0, 0, 1, 0, 0)
assert(hit and math.abs(hit[1] + 1) < 1e-2)
assert(s:ray_cast(-5, 3, 0, 1, 0, 0) == nil)
local m = s:magnet(0, 0, 5, 0, 0, 0)
assert(m and math.abs(m[3] - 1) < 1e-2)
model = s
""")


def test_errors_come_back_as_lua_errors(runner, tmp_path):
    p = tmp_path / "bad.lua"
    p.write_text("model = sphere('x')")
    out = subprocess.run([str(runner), str(p)], capture_output=True, text=True)
    assert out.returncode == 1 and " error:" in out.stdout


def test_reference_model_specs_round_trip(lib):
    """Every fixture rebuilds (BuildTreeFromSpec) into a tree whose spec is the fixture."""
    fx = np.load(GOLDEN / "lua_models.npz")
    for name in fx.files:
        spec = fx[name]
        t = sdf.from_spec(spec)
        n = lib.tg_tree_spec(t.handle, None, 0)
        back = np.empty(n, np.float32)
        lib.tg_tree_spec(t.handle, _lib.as_ptr(back), n)
        np.testing.assert_array_equal(back, spec, err_msg=name)


def test_reference_models_build_as_in_the_fixture(runner):
    models = O.REFERENCE_SOURCES / "models"
    if not models.exists():
        pytest.skip("the reference's model scripts are not on this host")
    fx = np.load(GOLDEN / "lua_models.npz")
    out = subprocess.run([str(runner), *[f"{n}.lua" for n in fx.files]], cwd=models, capture_output=True, text=True,
                         check=True)
    for line in out.stdout.splitlines():
        name, *words = line.split()
        np.testing.assert_array_equal(np.array([float(w) for w in words], np.float32), fx[name.rsplit(".", 1)[0]])
