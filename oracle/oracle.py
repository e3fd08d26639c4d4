"""Test infrastructure only: ctypes bindings for the two CPU checkers.

* ``port()`` -- oracle/port/tg_oracle.c, the C restatement of Tangerine's CPU export path
  (builds anywhere, including the GPU host).
* ``reference()`` -- Tangerine's own CPU code compiled from its sources by
  ``make -C oracle ref`` (only where the reference sources are present).

Only tests/, the smoke check and bench.py's CPU-baseline leg import this module.
"""

from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
PORT_SO = HERE / "_build" / "libtg_oracle.so"
REF_SO = HERE / "_ref" / "libtangerine_ref.so"


def _reference_sources() -> Path:
    """Where Tangerine's sources are: TANGERINE_REFERENCE, else the build recipe's REF
    (oracle/Makefile, the one place that names this machine's copy)."""
    env = os.environ.get("TANGERINE_REFERENCE")
    if env:
        return Path(env)
    for line in (HERE / "Makefile").read_text().splitlines():
        if line.startswith("REF ?="):
            return Path(line.split("?=", 1)[1].strip())
    return HERE / "_ref" / "no-reference"


REFERENCE_SOURCES = _reference_sources()

_f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
_u8p = np.ctypeslib.ndpointer(np.uint8, flags="C_CONTIGUOUS")
_u32p = np.ctypeslib.ndpointer(np.uint32, flags="C_CONTIGUOUS")


def build_port() -> Path:
    subprocess.run(["make", "-s", "-C", str(HERE), "port"], check=True)
    return PORT_SO


def build_reference() -> Path | None:
    if not (REFERENCE_SOURCES / "tangerine" / "sdf_evaluator.cpp").exists():
        return None
    subprocess.run(["make", "-s", "-C", str(HERE), "ref", f"REF={REFERENCE_SOURCES}", "-j8"], check=True)
    return REF_SO


class Mesh:
    """An exported mesh: vertices (V,3) f32, active cube index per vertex (V,) u64,
    faces (F,3) u64 vertex indices, optional normals (V,3) f32 and colours (V,3) u8."""

    def __init__(self, vertices, cubes, faces, normals=None, colors=None, seconds=0.0):
        self.vertices = vertices
        self.cubes = cubes
        self.faces = faces
        self.normals = normals
        self.colors = colors
        self.seconds = seconds


class Drawable:
    """Sodapop's meshing output: positions, gradient normals (V,3) f32, colours (V,4) f32
    (material Eval with the normal as view), faces (F,3), and the meshing grid
    (x, y, z, dx, dy, dz, sx, sy, sz)."""

    def __init__(self, positions, normals, colors, faces, grid):
        self.positions = positions
        self.normals = normals
        self.colors = colors
        self.faces = faces
        self.grid = grid


def _steps(grid):
    """Per-axis steps of an export grid (one step for all axes unless it has step_y/z)."""
    s = grid.step
    return s, (getattr(grid, "step_y", 0.0) or s), (getattr(grid, "step_z", 0.0) or s)


def _vec3(v):
    return np.ascontiguousarray(np.broadcast_to(np.asarray(v, np.float32), (3,)))


class CpuOracle:
    def __init__(self, path: Path, prefix: str):
        self.path = Path(path)
        self.prefix = prefix
        self.lib = C.CDLL(str(path))
        self._bind()

    def _fn(self, name, res, args):
        f = getattr(self.lib, self.prefix + name)
        f.restype = res
        f.argtypes = args
        return f

    def _bind(self):
        vp, i64, f, i = C.c_void_p, C.c_int64, C.c_float, C.c_int
        self._build = self._fn("build", vp, [_f32p, i])
        self._free = self._fn("free", None, [vp])
        self._free_buffer = self._fn("free_buffer", None, [vp])
        self._stack_size = self._fn("stack_size", i, [vp])
        self._has_paint = self._fn("has_paint", i, [vp])
        self._finite = self._fn("has_finite_bounds", i, [vp])
        self._leaf_count = self._fn("leaf_count", i, [vp])
        self._bounds = self._fn("bounds", None, [vp, _f32p, i])
        self._eval = self._fn("eval", None, [vp, i64, _f32p, _f32p])
        self._gradient = self._fn("gradient", None, [vp, i64, _f32p, _f32p])
        self._color = self._fn("color", None, [vp, i64, _f32p, _u8p])
        self._compile = self._fn("compile", i, [vp, _u32p, i])
        self._interp = self._fn("interp_eval", None, [vp, i64, _f32p, _f32p])
        self._clip = self._fn("clip", vp, [vp, f, f, f, f])
        self._equal = self._fn("equal", i, [vp, vp])
        self._oct_create = self._fn("octree_create", vp, [vp, f, i, i])
        self._mesh_oct_create = self._fn("meshing_octree_create", vp, [vp])
        self._oct_free = self._fn("octree_free", None, [vp])
        self._oct_dump = self._fn("octree_dump", i, [vp, C.POINTER(C.POINTER(C.c_float)), C.POINTER(C.POINTER(C.c_int32)),
                                                      C.POINTER(C.POINTER(C.c_uint32)), C.POINTER(C.c_int)])
        self._oct_eval = self._fn("octree_eval", None, [vp, i64, _f32p, i, _f32p])
        self._oct_grad = self._fn("octree_gradient", None, [vp, i64, _f32p, _f32p])
        self._oct_color = self._fn("octree_color", None, [vp, i64, _f32p, _u8p])
        fpp = C.POINTER(C.POINTER(C.c_float))
        self._sodapop = self._fn("sodapop", i64, [vp, f, fpp, fpp, fpp, C.POINTER(C.POINTER(C.c_uint64)),
                                                  C.POINTER(C.c_int64), _f32p])
        self._oct_grid = None
        self._raymarch = None
        self._i32pp = C.POINTER(C.POINTER(C.c_int32))
        self._ray_query = self._fn("ray_query", None, [vp, i, _f32p, i64, _f32p, _f32p, i, f, _u8p, _f32p, _f32p])

    # -- trees ----------------------------------------------------------------------
    def build(self, spec) -> int:
        spec = np.ascontiguousarray(spec, dtype=np.float32)
        h = self._build(spec, spec.size)
        if not h:
            raise ValueError("malformed tree spec")
        return h

    def free(self, h):
        self._free(h)

    def stack_size(self, h):
        return self._stack_size(h)

    def has_paint(self, h):
        return bool(self._has_paint(h))

    def has_finite_bounds(self, h):
        return bool(self._finite(h))

    def leaf_count(self, h):
        return self._leaf_count(h)

    def bounds(self, h, inner=False):
        out = np.zeros(6, np.float32)
        self._bounds(h, out, int(inner))
        return out

    @staticmethod
    def _pts(points):
        return np.ascontiguousarray(np.asarray(points, np.float32).reshape(-1, 3))

    def eval(self, h, points):
        p = self._pts(points)
        out = np.empty(p.shape[0], np.float32)
        self._eval(h, p.shape[0], p, out)
        return out

    def gradient(self, h, points):
        p = self._pts(points)
        out = np.empty_like(p)
        self._gradient(h, p.shape[0], p, out)
        return out

    def color(self, h, points):
        p = self._pts(points)
        out = np.empty(p.shape, np.uint8)
        self._color(h, p.shape[0], p, out)
        return out

    def compile(self, h):
        n = self._compile(h, np.zeros(1, np.uint32), 0)
        out = np.zeros(n, np.uint32)
        self._compile(h, out, n)
        return out

    def interp_eval(self, h, points):
        p = self._pts(points)
        out = np.empty(p.shape[0], np.float32)
        self._interp(h, p.shape[0], p, out)
        return out

    def clip(self, h, point, radius):
        return self._clip(h, float(point[0]), float(point[1]), float(point[2]), float(radius)) or None

    def equal(self, a, b):
        return bool(self._equal(a, b))

    def ray_query(self, h, mode, origins, dirs, frame=None, iterations=100, epsilon=1e-3):
        """mode 1: Lua's magnet cast (dirs are targets); mode 2: SDFModel::RayMarch in the
        model frame (quat w x y z, translation xyz, scale)."""
        o = self._pts(origins)
        d = self._pts(dirs)
        n = o.shape[0]
        fr = np.ascontiguousarray(np.zeros(8, np.float32) if frame is None else np.asarray(frame, np.float32))
        hit = np.empty(n, np.uint8)
        travel = np.empty(n, np.float32)
        pos = np.empty((n, 3), np.float32)
        self._ray_query(h, int(mode), fr, n, o, d, int(iterations), float(epsilon), hit, travel, pos)
        return hit, travel, pos

    # -- octree ---------------------------------------------------------------------
    def octree(self, h, target=0.25, coalesce=True, max_depth=-1):
        o = self._oct_create(h, target, int(coalesce), max_depth)
        return o or None

    def meshing_octree(self, h):
        """Sodapop's meshing octree: Create(.25, false, 3), then each incomplete cell
        populated with Populate(false, 3, -1) (sodapop.cpp:565-569)."""
        return self._mesh_oct_create(h) or None

    def sodapop(self, h, density=20.0) -> Drawable:
        """MeshingJob::NaiveSurfaceNets (sodapop.cpp:562-897), serially, without the vertex
        shuffle; vertices in grid-index order."""
        P, N, Cl = C.POINTER(C.c_float)(), C.POINTER(C.c_float)(), C.POINTER(C.c_float)()
        F = C.POINTER(C.c_uint64)()
        nf = C.c_int64()
        grid = np.zeros(9, np.float32)
        nv = self._sodapop(h, float(density), C.byref(P), C.byref(N), C.byref(Cl), C.byref(F), C.byref(nf), grid)
        if nv < 0:
            return None

        def take(ptr, n, k, dtype):
            return np.ctypeslib.as_array(ptr, shape=(max(1, n) * k,))[: n * k].reshape(n, k).astype(dtype).copy()

        d = Drawable(take(P, nv, 3, np.float32), take(N, nv, 3, np.float32), take(Cl, nv, 4, np.float32),
                     take(F, nf.value, 3, np.uint64), grid)
        for b in (P, N, Cl, F):
            self._free_buffer(C.cast(b, C.c_void_p))
        return d

    def octree_free(self, o):
        self._oct_free(o)

    def octree_dump(self, o):
        nodes = C.POINTER(C.c_float)()
        children = C.POINTER(C.c_int32)()
        words = C.POINTER(C.c_uint32)()
        wc = C.c_int()
        n = self._oct_dump(o, C.byref(nodes), C.byref(children), C.byref(words), C.byref(wc))
        N = np.ctypeslib.as_array(nodes, shape=(n * 14,)).reshape(n, 14).copy()
        Ch = np.ctypeslib.as_array(children, shape=(n * 8,)).reshape(n, 8).copy()
        W = np.ctypeslib.as_array(words, shape=(max(1, wc.value),))[: wc.value].copy()
        for b in (nodes, children, words):
            self._free_buffer(C.cast(b, C.c_void_p))
        return N, Ch, W

    def octree_eval(self, o, points, exact=True):
        p = self._pts(points)
        out = np.empty(p.shape[0], np.float32)
        self._oct_eval(o, p.shape[0], p, int(exact), out)
        return out

    def octree_gradient(self, o, points):
        p = self._pts(points)
        out = np.empty_like(p)
        self._oct_grad(o, p.shape[0], p, out)
        return out

    def octree_color(self, o, points):
        p = self._pts(points)
        out = np.empty(p.shape, np.uint8)
        self._oct_color(o, p.shape[0], p, out)
        return out


class PortOracle(CpuOracle):
    def __init__(self, path: Path = PORT_SO):
        super().__init__(path, "tgo_")
        vp, i64, f, i = C.c_void_p, C.c_int64, C.c_float, C.c_int
        self._oct_grid = self._fn("octree_grid", None, [vp, f, f, f, f, f, f, i64, i64, i64, i, _f32p])
        self._sn = self._fn("surface_nets", i64, [vp, f, f, f, f, f, f, i64, i64, i64, i, i,
                                                  C.POINTER(C.POINTER(C.c_float)), C.POINTER(C.POINTER(C.c_uint64)),
                                                  C.POINTER(C.POINTER(C.c_uint64)), C.POINTER(C.c_int64), C.POINTER(C.c_double)])
        self._attrs = self._fn("vertex_attributes", None, [vp, i64, _f32p, i, _f32p, C.c_void_p])
        self._oct_paint = self._fn("octree_has_paint", i, [vp])
        self._raymarch = self._fn("raymarch", None, [vp, i64, _f32p, _f32p, i, f, i, _u8p, _f32p, _f32p])
        self._cloud = self._fn("point_cloud", i64, [vp, _f32p, _f32p, _f32p, i, C.POINTER(C.POINTER(C.c_float)), self._i32pp])
        self._vox = self._fn("vox", i64, [vp, f, i, C.POINTER(C.c_int32), C.POINTER(C.c_float), self._i32pp])
        self._hw = self._fn("hardware_threads", i, [])

    def hardware_threads(self):
        return self._hw()

    def octree_grid(self, o, grid, threads=0):
        nx, ny, nz = grid.sx + 1, grid.sy + 1, grid.sz + 1
        out = np.empty(nx * ny * nz, np.float32)
        self._oct_grid(o, grid.x0, grid.y0, grid.z0, *_steps(grid), nx, ny, nz, threads, out)
        return out.reshape(nz, ny, nx)

    def surface_nets(self, o, grid, threads=0, faithful=False) -> Mesh:
        V = C.POINTER(C.c_float)()
        Cb = C.POINTER(C.c_uint64)()
        F = C.POINTER(C.c_uint64)()
        nf = C.c_int64()
        secs = C.c_double()
        nv = self._sn(o, grid.x0, grid.y0, grid.z0, *_steps(grid), grid.sx, grid.sy, grid.sz,
                      threads, int(faithful), C.byref(V), C.byref(Cb), C.byref(F), C.byref(nf), C.byref(secs))
        if nv < 0:
            raise ValueError("grid with a strictly longest axis is not restated")
        verts = np.ctypeslib.as_array(V, shape=(max(1, nv) * 3,))[: nv * 3].reshape(nv, 3).copy()
        cubes = np.ctypeslib.as_array(Cb, shape=(max(1, nv),))[:nv].copy()
        faces = np.ctypeslib.as_array(F, shape=(max(1, nf.value) * 3,))[: nf.value * 3].reshape(nf.value, 3).copy()
        for b in (V, Cb, F):
            self._free_buffer(C.cast(b, C.c_void_p))
        return Mesh(verts, cubes, faces, seconds=secs.value)

    def vertex_attributes(self, o, vertices, threads=0):
        v = self._pts(vertices)
        normals = np.empty_like(v)
        colors = np.empty(v.shape, np.uint8) if self._oct_paint(o) else None
        self._attrs(o, v.shape[0], v, threads, normals,
                    colors.ctypes.data_as(C.c_void_p) if colors is not None else None)
        return normals, colors

    def export_mesh(self, spec, grid, threads=0, faithful=False) -> Mesh:
        """Octree(0.25) -> surface nets -> gradient normals + colours, as MeshExportThread
        and WritePLY(Octree, ...) do (export.cpp:283-381)."""
        h = self.build(spec)
        try:
            o = self.octree(h)
            if o is None:
                raise ValueError("tree has infinite or empty bounds")
            try:
                m = self.surface_nets(o, grid, threads, faithful)
                m.normals, m.colors = self.vertex_attributes(o, m.vertices, threads)
                return m
            finally:
                self.octree_free(o)
        finally:
            self.free(h)

    def raymarch(self, h, origins, dirs, iterations=100, epsilon=1e-3, threads=0):
        o = self._pts(origins)
        d = self._pts(dirs)
        n = o.shape[0]
        hit = np.empty(n, np.uint8)
        travel = np.empty(n, np.float32)
        pos = np.empty((n, 3), np.float32)
        self._raymarch(h, n, o, d, iterations, epsilon, threads, hit, travel, pos)
        return hit.astype(bool), travel, pos


    def point_cloud(self, o, lo, hi, step, refine):
        """PointCloudExportThread's points in cell order (export.cpp:384-480): (points, cells)."""
        P = C.POINTER(C.c_float)()
        I = C.POINTER(C.c_int32)()
        n = self._cloud(o, _vec3(lo), _vec3(hi), _vec3(step), int(refine), C.byref(P), C.byref(I))
        pts = np.ctypeslib.as_array(P, shape=(max(1, n) * 3,))[: n * 3].reshape(n, 3).copy()
        cells = np.ctypeslib.as_array(I, shape=(max(1, n),))[:n].copy()
        for b in (P, I):
            self._free_buffer(C.cast(b, C.c_void_p))
        return pts, cells

    def vox(self, h, grid_size, color_index=0):
        """VoxExport's voxels in cell order (magica.cpp:27-69): ((n, 4) x y z colour, size, radius)."""
        V = C.POINTER(C.c_int32)()
        size = (C.c_int32 * 3)()
        radius = C.c_float()
        n = self._vox(h, float(grid_size), int(color_index), size, C.byref(radius), C.byref(V))
        vox = np.ctypeslib.as_array(V, shape=(max(1, n) * 4,))[: n * 4].reshape(n, 4).copy()
        self._free_buffer(C.cast(V, C.c_void_p))
        return vox, tuple(size), float(radius.value)


class ReferenceOracle(CpuOracle):
    def __init__(self, path: Path = REF_SO):
        super().__init__(path, "ref_")
        vp, i64, f, i = C.c_void_p, C.c_int64, C.c_float, C.c_int
        self._oct_grid = self._fn("octree_grid", None, [vp, f, f, f, f, f, f, i64, i64, i64, _f32p])
        self._sn = self._fn("surface_nets", i64, [vp, f, f, f, f, f, f, i64, i64, i64, i,
                                                  C.POINTER(C.POINTER(C.c_float)), C.POINTER(C.POINTER(C.c_uint64)),
                                                  C.POINTER(C.POINTER(C.c_uint64)), C.POINTER(C.c_int64), C.POINTER(C.c_double)])
        self._export_file = self._fn("mesh_export_file", None, [vp, f, f, f, f, f, f, f, i, C.c_char_p])
        self._cloud_file = self._fn("point_cloud_file", None, [vp, _f32p, _f32p, _f32p, i, f, C.c_char_p])
        self._vox_file = self._fn("vox_file", None, [vp, f, i, C.c_char_p])
        self._vox_write = self._fn("vox_write", None, [C.POINTER(C.c_int32), i64, C.POINTER(C.c_int32), C.c_char_p])
        self._write_drawables = self._fn("write_drawables", None, [i, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                                                   C.c_void_p, C.c_void_p, i, f, C.c_char_p])
        self._vox_serial = self._fn("vox_serial", i64, [vp, f, i, C.c_char_p, self._i32pp, C.POINTER(C.c_int32),
                                                        C.POINTER(C.c_float)])
        self._raymarch = self._fn("raymarch", None, [vp, i64, _f32p, _f32p, i, f, i, _u8p, _f32p, _f32p])
        self._attrs = self._fn("vertex_attributes", None, [vp, i64, _f32p, i, _f32p, C.c_void_p])
        self._oct_paint = self._fn("octree_has_paint", i, [vp])
        self._hw = self._fn("hardware_threads", i, [])

    def octree_grid(self, o, grid):
        nx, ny, nz = grid.sx + 1, grid.sy + 1, grid.sz + 1
        out = np.empty(nx * ny * nz, np.float32)
        self._oct_grid(o, grid.x0, grid.y0, grid.z0, *_steps(grid), nx, ny, nz, out)
        return out.reshape(nz, ny, nx)

    def hardware_threads(self):
        return self._hw()

    def vertex_attributes(self, o, vertices, threads=0):
        """WritePLY(Octree, ...)'s per-vertex Gradient + GetMaterial colour bytes on Pool()
        (threads=0) or that many threads."""
        v = self._pts(vertices)
        normals = np.empty_like(v)
        colors = np.empty(v.shape, np.uint8) if self._oct_paint(o) else None
        self._attrs(o, v.shape[0], v, threads, normals, colors.ctypes.data_as(C.c_void_p) if colors is not None else None)
        return normals, colors

    def surface_nets(self, o, grid, threads=1) -> Mesh:
        V = C.POINTER(C.c_float)()
        Cb = C.POINTER(C.c_uint64)()
        F = C.POINTER(C.c_uint64)()
        nf = C.c_int64()
        secs = C.c_double()
        nv = self._sn(o, grid.x0, grid.y0, grid.z0, *_steps(grid), grid.sx, grid.sy, grid.sz,
                      threads, C.byref(V), C.byref(Cb), C.byref(F), C.byref(nf), C.byref(secs))
        verts = np.ctypeslib.as_array(V, shape=(max(1, nv) * 3,))[: nv * 3].reshape(nv, 3).copy()
        cubes = np.ctypeslib.as_array(Cb, shape=(max(1, nv),))[:nv].copy()
        faces = np.ctypeslib.as_array(F, shape=(max(1, nf.value) * 3,))[: nf.value * 3].reshape(nf.value, 3).copy()
        for b in (V, Cb, F):
            self._free_buffer(C.cast(b, C.c_void_p))
        return Mesh(verts, cubes, faces, seconds=secs.value)

    def export_file(self, h, lo, hi, step, path, fmt="ply"):
        self._export_file(h, *[float(v) for v in lo], *[float(v) for v in hi], float(step),
                          1 if fmt == "ply" else 0, str(path).encode())

    def point_cloud_file(self, h, lo, hi, step, refine, path, scale=1.0):
        """PointCloudExportThread writing its PLY (threaded: rows in run-dependent order)."""
        self._cloud_file(h, _vec3(lo), _vec3(hi), _vec3(step), int(refine), float(scale), str(path).encode())

    def vox_file(self, h, grid_size, color_index, path):
        """VoxExport as shipped (threaded)."""
        self._vox_file(h, float(grid_size), int(color_index), str(path).encode())

    def write_drawables(self, drawables, frames, path, fmt="ply", scale=1.0):
        """MeshExport(Path, UseBaseColor=True, ...) over (positions, normals, colors rgba,
        faces) tuples placed by frames (8 floats each), through the reference's writers."""
        vc = np.array([len(d[0]) for d in drawables], np.int64)
        ic = np.array([d[3].size for d in drawables], np.int64)
        P = np.ascontiguousarray(np.concatenate([d[0] for d in drawables]).astype(np.float32))
        N = np.ascontiguousarray(np.concatenate([d[1] for d in drawables]).astype(np.float32))
        Cl = np.ascontiguousarray(np.concatenate([d[2] for d in drawables]).astype(np.float32))
        I = np.ascontiguousarray(np.concatenate([d[3].reshape(-1) for d in drawables]).astype(np.uint32))
        Fr = np.ascontiguousarray(np.asarray(frames, np.float32).reshape(-1, 8))
        ptr = lambda a: a.ctypes.data_as(C.c_void_p)
        self._write_drawables(len(drawables), ptr(vc), ptr(ic), ptr(P), ptr(N), ptr(Cl), ptr(I), ptr(Fr),
                              0 if fmt == "stl" else 1, float(scale), str(path).encode())

    def vox_write(self, voxels, size, path):
        """VoxWriter fed (x, y, z, colour) rows in order, saved to path."""
        v = np.ascontiguousarray(np.asarray(voxels, np.int32).reshape(-1, 4))
        sz = (C.c_int32 * 3)(*[int(x) for x in size])
        self._vox_write(v.ctypes.data_as(C.POINTER(C.c_int32)), v.shape[0], sz, str(path).encode())

    def vox_serial(self, h, grid_size, color_index=0, path=None):
        """VoxExport run serially in cell order through VoxWriter: ((n, 4) voxels, size, radius)."""
        V = C.POINTER(C.c_int32)()
        size = (C.c_int32 * 3)()
        radius = C.c_float()
        n = self._vox_serial(h, float(grid_size), int(color_index), (str(path) if path else "").encode(), C.byref(V), size,
                             C.byref(radius))
        vox = np.ctypeslib.as_array(V, shape=(max(1, n) * 4,))[: n * 4].reshape(n, 4).copy()
        self._free_buffer(C.cast(V, C.c_void_p))
        return vox, tuple(size), float(radius.value)

    def raymarch(self, h, origins, dirs, iterations=100, epsilon=1e-3, threads=0):
        o = self._pts(origins)
        d = self._pts(dirs)
        n = o.shape[0]
        hit = np.empty(n, np.uint8)
        travel = np.empty(n, np.float32)
        pos = np.empty((n, 3), np.float32)
        self._raymarch(h, n, o, d, iterations, epsilon, threads, hit, travel, pos)
        return hit.astype(bool), travel, pos


def port() -> PortOracle:
    if not PORT_SO.exists():
        build_port()
    return PortOracle()


def reference() -> ReferenceOracle | None:
    if not REF_SO.exists():
        if build_reference() is None:
            return None
    return ReferenceOracle()


def read_ply(path):
    """Parses the binary PLY that WritePLY (tangerine/export.cpp:198-280) writes."""
    data = Path(path).read_bytes()
    end = data.index(b"end_header\n") + len(b"end_header\n")
    header = data[:end].decode()
    nv = nf = 0
    color = "property uchar red" in header
    for line in header.splitlines():
        if line.startswith("element vertex"):
            nv = int(line.split()[-1])
        if line.startswith("element face"):
            nf = int(line.split()[-1])
    vdt = [("p", "<f4", 3), ("n", "<f4", 3)] + ([("c", "u1", 3)] if color else [])
    vert = np.frombuffer(data, dtype=np.dtype(vdt), count=nv, offset=end)
    off = end + vert.nbytes
    fdt = np.dtype([("k", "u1"), ("i", "<u4", 3)])
    faces = np.frombuffer(data, dtype=fdt, count=nf, offset=off)
    return header, vert["p"].copy(), vert["n"].copy(), (vert["c"].copy() if color else None), faces["i"].astype(np.uint64)


def read_vox(path):
    """Parses a MagicaVoxel file as VoxWriter writes it (voxwriter/VoxWriter.cpp): version,
    the models' (size, (n, 4) uint8 voxels x y z colour) in file order, and each shape
    transform's "_t" translation in scene order."""
    data = Path(path).read_bytes()
    assert data[:4] == b"VOX "
    version = int.from_bytes(data[4:8], "little")
    assert data[8:12] == b"MAIN"
    pos = 20
    models, translations = [], []
    size = None
    while pos < len(data):
        cid = data[pos:pos + 4]
        content = int.from_bytes(data[pos + 4:pos + 8], "little")
        body = data[pos + 12:pos + 12 + content]
        if cid == b"SIZE":
            size = tuple(int.from_bytes(body[i:i + 4], "little", signed=True) for i in (0, 4, 8))
        elif cid == b"XYZI":
            n = int.from_bytes(body[:4], "little")
            models.append((size, np.frombuffer(body[4:4 + 4 * n], np.uint8).reshape(n, 4).copy()))
        elif cid == b"nTRN":
            q = 4
            nattr = int.from_bytes(body[q:q + 4], "little"); q += 4
            for _ in range(2 * nattr):
                q += 4 + int.from_bytes(body[q:q + 4], "little")
            q += 16
            nframes = int.from_bytes(body[q - 4:q], "little")
            for _ in range(nframes):
                nkeys = int.from_bytes(body[q:q + 4], "little"); q += 4
                kv = []
                for _ in range(2 * nkeys):
                    ln = int.from_bytes(body[q:q + 4], "little")
                    kv.append(body[q + 4:q + 4 + ln].decode()); q += 4 + ln
                d = dict(zip(kv[::2], kv[1::2]))
                if "_t" in d:
                    translations.append(tuple(int(v) for v in d["_t"].split()))
        pos += 12 + content
    return version, models, translations
