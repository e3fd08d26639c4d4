"""Seeded synthetic CSG workloads.

Trees are emitted as *tree specs*: postfix float32 word streams that name the same
constructors and mutators as Tangerine's C++ API (``SDF::Sphere``, ``SDF::Union``,
``SDFNode::Move``/``Rotate``/``ApplyMaterial``; tangerine/sdf_evaluator.h:223-264) and the
C ABI (tangerine/c_sdf.cpp:86-178).  ``tangerine_gb300.sdf.from_spec`` replays a spec
through this library's C ABI; the CPU oracles replay the same words, so every
implementation starts from identical float inputs.

Random numbers: ``std::mt19937`` seeded with the integer seed (numpy's legacy seeding is
the same generator), raw 32-bit words mapped to floats in [0, 1) by ``(w >> 8) * 2**-24``.
Rotations are given to the tree as explicit quaternions (rounded from float64 sin/cos of
the half angle), so no platform libm enters the tree.
"""

from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

# Spec op codes (shared with oracle/ref_harness.cpp and oracle/port/tg_oracle.c).
SPHERE, ELLIPSOID, BOX, TORUS, CYLINDER, PLANE, CONE, CONINDER = range(1, 9)
UNION, DIFF, INTER, BLEND_UNION, BLEND_DIFF, BLEND_INTER, FLATE = range(9, 16)
MOVE, ROTATE, SCALE, PAINT, ALIGN, STENCIL, TRANSFORM = range(16, 23)

ARITY = {
    SPHERE: 1, ELLIPSOID: 3, BOX: 3, TORUS: 2, CYLINDER: 2, PLANE: 3, CONE: 2, CONINDER: 3,
    UNION: 0, DIFF: 0, INTER: 0, BLEND_UNION: 1, BLEND_DIFF: 1, BLEND_INTER: 1, FLATE: 1,
    MOVE: 3, ROTATE: 4, SCALE: 1, PAINT: 3, ALIGN: 3, STENCIL: 4, TRANSFORM: 8,
}


class _Words:
    """mt19937 raw words -> uniform floats (w >> 8) * 2**-24."""

    def __init__(self, seed: int):
        self._bits = np.random.RandomState(seed & 0xFFFFFFFF)._bit_generator
        self._buf = np.empty(0, dtype=np.uint64)
        self._pos = 0

    def u(self) -> float:
        if self._pos >= self._buf.size:
            self._buf = self._bits.random_raw(4096)
            self._pos = 0
        w = int(self._buf[self._pos])
        self._pos += 1
        return float(w >> 8) * (2.0 ** -24)

    def uniform(self, lo: float, hi: float) -> float:
        return lo + (hi - lo) * self.u()


def axis_quaternion(axis: int, degrees: float) -> tuple[float, float, float, float]:
    """(x, y, z, w) of a rotation about one axis, as SDF::RotateX/Y/Z build it
    (sdf_evaluator.cpp:1180-1202: half angle, quat(cos, sin*axis))."""
    half = math.radians(degrees) * 0.5
    s, c = math.sin(half), math.cos(half)
    q = [0.0, 0.0, 0.0, c]
    q[axis] = s
    return tuple(float(np.float32(v)) for v in q)  # type: ignore[return-value]


OPS_UNIFORM4 = ((UNION, 0.25), (DIFF, 0.25), (INTER, 0.25), (BLEND_UNION, 0.25))
OPS_60_20_10_10 = ((UNION, 0.60), (DIFF, 0.20), (INTER, 0.10), (BLEND_UNION, 0.10))


def _emit_primitive(rng: _Words, out: list, paint: bool) -> None:
    kind = min(int(rng.u() * 4), 3)
    cx, cy, cz = (rng.uniform(-1.0, 1.0) for _ in range(3))
    if kind == 0:
        out += [SPHERE, rng.uniform(0.1, 0.5)]
    elif kind == 1:
        out += [BOX, rng.uniform(0.1, 0.5), rng.uniform(0.1, 0.5), rng.uniform(0.1, 0.5)]
    elif kind == 2:
        major = rng.uniform(0.1, 0.5)
        out += [TORUS, major, major * rng.uniform(0.2, 0.5)]
    else:
        out += [CYLINDER, rng.uniform(0.1, 0.5), rng.uniform(0.1, 0.5)]
    for axis in range(3):
        out += [ROTATE, *axis_quaternion(axis, rng.uniform(0.0, 360.0))]
    out += [MOVE, cx, cy, cz]
    if paint:
        out += [PAINT, rng.u(), rng.u(), rng.u()]


def _pick(rng: _Words, table) -> int:
    x = rng.u()
    acc = 0.0
    for op, w in table:
        acc += w
        if x < acc:
            return op
    return table[-1][0]


def random_tree(seed: int, primitives: int, ops=OPS_60_20_10_10, max_depth: int = 12,
                blend_k=(0.02, 0.1), paint: bool = True) -> np.ndarray:
    """Seeded CSG tree of `primitives` leaves (sphere/box/torus/cylinder, centres U(-1,1)^3,
    sizes U(0.1,0.5) in SDF:: units, random Euler rotations, per-primitive sRGB paint),
    joined by a random binary split whose depth never exceeds `max_depth`."""
    if primitives < 1:
        raise ValueError("a tree needs at least one primitive")
    if primitives > 2 ** (max_depth - 1):
        raise ValueError("too many primitives for the depth limit")
    rng = _Words(seed)
    out: list = []

    def build(n: int, depth: int) -> None:
        if n == 1:
            _emit_primitive(rng, out, paint)
            return
        cap = 2 ** (depth - 2)          # most leaves a child subtree may hold
        lo = max(1, n - cap)
        hi = min(n - 1, cap)
        left = lo + min(int(rng.u() * (hi - lo + 1)), hi - lo)
        op = _pick(rng, ops)
        k = rng.uniform(*blend_k) if op in (BLEND_UNION, BLEND_DIFF, BLEND_INTER) else None
        build(left, depth - 1)
        build(n - left, depth - 1)
        out.append(op)
        if k is not None:
            out.append(k)

    build(primitives, max_depth)
    return np.asarray(out, dtype=np.float32)


def spec_primitive_count(spec: np.ndarray) -> int:
    i, n = 0, 0
    while i < spec.size:
        op = int(spec[i])
        if op <= CONINDER:
            n += 1
        i += 1 + ARITY[op]
    return n


@dataclass(frozen=True)
class ExportGrid:
    """The lattice MeshExportThread builds (tangerine/export.cpp:324-337): the lower bound
    moves down by two steps and each axis gets ceil((max - min) / step) cells."""
    x0: float
    y0: float
    z0: float
    step: float
    sx: int
    sy: int
    sz: int
    step_y: float = 0.0          # 0: same as step (MeshExport's vec3 Step may differ per axis)
    step_z: float = 0.0

    @property
    def steps(self) -> tuple[float, float, float]:
        return (self.step, self.step_y or self.step, self.step_z or self.step)

    @property
    def corners(self) -> int:
        return (self.sx + 1) * (self.sy + 1) * (self.sz + 1)

    @property
    def cells(self) -> int:
        return self.sx * self.sy * self.sz


def export_grid(lo=(-2.0, -2.0, -2.0), hi=(2.0, 2.0, 2.0), step: float | None = None,
                resolution: int | None = None, steps=None) -> ExportGrid:
    """`steps`: one step per axis instead of `step` (MeshExport's vec3 Step)."""
    f32 = np.float32
    if steps is None:
        if step is None:
            step = float(f32(f32(hi[0]) - f32(lo[0])) / f32(resolution))
        steps = (step, step, step)
    st = [f32(v) for v in steps]
    mins = [f32(f32(v) - f32(s * f32(2.0))) for v, s in zip(lo, st)]
    extent = [int(math.ceil(float(f32(f32(f32(h) - m) / s)))) for h, m, s in zip(hi, mins, st)]
    if st[0] == st[1] == st[2]:
        return ExportGrid(float(mins[0]), float(mins[1]), float(mins[2]), float(st[0]), *extent)
    return ExportGrid(float(mins[0]), float(mins[1]), float(mins[2]), float(st[0]), *extent, float(st[1]), float(st[2]))


def camera_poses(seed: int, count: int, radius: float = 4.0):
    """Seeded camera positions on a sphere around the origin (uniform on the sphere)."""
    rng = _Words(seed)
    poses = []
    for _ in range(count):
        z = rng.uniform(-1.0, 1.0)
        a = rng.uniform(0.0, 2.0 * math.pi)
        r = math.sqrt(max(0.0, 1.0 - z * z))
        poses.append((radius * r * math.cos(a), radius * r * math.sin(a), radius * z))
    return np.asarray(poses, dtype=np.float32)


def camera_rays(position, width: int, height: int, tan_half: float):
    """The ray tg_render casts through every pixel of a camera at `position` looking at the
    origin with +z up, in float32 with the renderer's operation order: origins and
    unnormalised directions, row-major over pixels."""
    f32 = np.float32

    def normalize(v):
        d = (v[0] * v[0] + v[1] * v[1]) + v[2] * v[2]
        s = f32(1.0) / np.sqrt(f32(d))
        return np.array([v[0] * s, v[1] * s, v[2] * s], np.float32)

    def cross(a, b):
        return np.array([a[1] * b[2] - b[1] * a[2], a[2] * b[0] - b[2] * a[0], a[0] * b[1] - b[0] * a[1]], np.float32)

    pos = np.asarray(position, np.float32)
    fwd = normalize(np.zeros(3, np.float32) - pos)
    right = normalize(cross(fwd, np.array([0, 0, 1], np.float32)))
    up = cross(right, fwd)
    x = np.arange(width, dtype=np.float32)[None, :].repeat(height, 0)
    y = np.arange(height, dtype=np.float32)[:, None].repeat(width, 1)
    aspect = f32(width) / f32(height)
    u = ((f32(2.0) * (x + f32(0.5)) / f32(width)) - f32(1.0)) * f32(tan_half) * aspect
    v = (f32(1.0) - f32(2.0) * (y + f32(0.5)) / f32(height)) * f32(tan_half)
    d = np.stack([(fwd[i] + right[i] * u) + up[i] * v for i in range(3)], -1).astype(np.float32)
    return np.broadcast_to(pos, d.shape).copy().reshape(-1, 3), d.reshape(-1, 3)


BATCH_RESOLUTIONS = (64, 128, 192, 256, 384)


def batch_workload(seed: int, count: int = 512, min_prims: int = 4, max_prims: int = 1024,
                   resolutions=BATCH_RESOLUTIONS, valid=None):
    """Independent seeded trees for the batched export: primitive counts log-uniform in
    [min_prims, max_prims], grid resolution uniform over `resolutions` (cells per axis of
    [-2, 2]^3).  Returns [(tree seed, primitive count, resolution)].  `valid(spec)`, when
    given, rejects trees (an intersection or difference can leave nothing); a rejected
    model takes the next tree seed of its own sequence."""
    rng = _Words(seed * 7919 + 17)
    out = []
    lo, hi = math.log(min_prims), math.log(max_prims)
    for i in range(count):
        prims = int(round(math.exp(rng.uniform(lo, hi))))
        prims = max(min_prims, min(max_prims, prims))
        res = resolutions[min(len(resolutions) - 1, int(rng.uniform(0.0, float(len(resolutions)))))]
        tree_seed = seed * 100000 + i
        if valid is not None:
            attempt = 0
            while not valid(random_tree(tree_seed, prims)):
                attempt += 1
                tree_seed = seed * 100000 + i + 1000003 * attempt
        out.append((tree_seed, prims, res))
    return out
