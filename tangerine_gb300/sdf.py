"""Python face of the engine: CSG trees through Tangerine's C API and GPU export through
the tg_* entry points (include/tangerine_gb300.h).

    tree = sdf.from_spec(workloads.random_tree(1, 256))
    with sdf.compile(tree) as prog:
        mesh = prog.export_mesh(workloads.export_grid(resolution=512))
"""

from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _lib
from ._lib import check, load


@dataclass
class SodapopDrawable:
    """Sodapop's drawable buffers: positions, gradient normals, shaded RGBA colours, triangle
    indices, each vertex's cell number, and the lattice (origin xyz, step xyz, cells xyz)."""
    positions: np.ndarray
    normals: np.ndarray
    colors: np.ndarray
    faces: np.ndarray
    cells: np.ndarray
    grid: np.ndarray
    compile_seconds: float = 0.0
    gpu_seconds: float = 0.0


class Tree:
    """A reference-counted CSG tree handle (c_sdf.cpp's `void*` trees)."""

    def __init__(self, handle):
        if not handle:
            raise _lib.TangerineError(load().tg_last_error().decode() or "null tree")
        self.handle = C.c_void_p(handle)

    def __del__(self):
        h = getattr(self, "handle", None)
        if h and h.value and _lib._LIB is not None:
            _lib._LIB.DiscardTree(h)
            self.handle = C.c_void_p(None)

    def _give(self):
        """Hands this handle's reference to an operator (the Python object is emptied)."""
        h = self.handle
        self.handle = C.c_void_p(None)
        return h

    def eval(self, x, y, z) -> float:
        return load().EvalTree(self.handle, x, y, z)

    def clip(self, point, radius):
        h = load().ClipTree(self.handle, float(point[0]), float(point[1]), float(point[2]), float(radius))
        return Tree(h) if h else None

    def ray_march(self, start, direction, iterations=100, epsilon=1e-3):
        r = load().RayMarchTree(self.handle, *map(float, start), *map(float, direction), iterations, epsilon)
        return bool(r.Hit), float(r.Travel), tuple(r.Position)

    def finite(self) -> bool:
        return bool(load().TreeHasFiniteBounds(self.handle))

    def move(self, x, y, z):
        load().MoveTree(self.handle, x, y, z)
        return self

    def rotate(self, x, y, z, w):
        load().RotateTree(self.handle, x, y, z, w)
        return self

    def align(self, x, y, z):
        load().AlignTree(self.handle, x, y, z)
        return self

    def scale(self, s):
        load().ScaleTree(self.handle, s)
        return self

    def paint(self, r, g, b):
        load().PaintTree(r, g, b, self.handle)
        return self

    def debug_octree(self, meshing=False):
        """Host-built export octree (or Sodapop's meshing octree) in the oracle's dump
        layout: (cells, children, words)."""
        lib = load()
        fn = lib.tg_debug_meshing_octree if meshing else lib.tg_debug_octree
        wc = C.c_int64()
        n = fn(self.handle, None, None, 0, None, 0, C.byref(wc))
        if n < 0:
            return None
        cells = np.zeros((n, 14), np.float32)
        kids = np.zeros((n, 8), np.int32)
        words = np.zeros(max(1, wc.value), np.uint32)
        fn(self.handle, _lib.as_ptr(cells), _lib.as_ptr(kids), n, _lib.as_ptr(words), wc.value, C.byref(wc))
        return cells, kids, words[: wc.value]

    def sodapop_plan(self, density=20.0):
        """Host-side plan of the meshing job: (grid[11], leaf boxes (n, 6) int64)."""
        lib = load()
        grid = np.zeros(11, np.float32)
        n = C.c_int64()
        check(lib.tg_debug_sodapop_plan(self.handle, float(density), _lib.as_ptr(grid), None, 0, C.byref(n)))
        boxes = np.zeros((max(1, n.value), 6), np.int64)
        check(lib.tg_debug_sodapop_plan(self.handle, float(density), _lib.as_ptr(grid), _lib.as_ptr(boxes), n.value, C.byref(n)))
        return grid, boxes[: n.value]

    def sodapop_mesh(self, density=20.0, stream=None) -> "SodapopDrawable":
        """Sodapop's meshing job (MeshingJob::NaiveSurfaceNets, sodapop.cpp:562-897) on the
        GPU; vertices in cell-number order."""
        lib = load()
        d = _lib.Drawable()
        check(lib.tg_sodapop_mesh(self.handle, float(density), C.byref(d), stream))
        try:
            nv, nf = int(d.vertex_count), int(d.face_count)

            def take(ptr, n, k, dtype):
                if n == 0:
                    return np.zeros((0, k), dtype)
                return np.ctypeslib.as_array(ptr, shape=(n * k,)).reshape(n, k).astype(dtype, copy=True)

            out = SodapopDrawable(
                positions=take(d.positions, nv, 3, np.float32), normals=take(d.normals, nv, 3, np.float32),
                colors=take(d.colors, nv, 4, np.float32), faces=take(d.faces, nf, 3, np.uint32),
                cells=take(d.cells, nv, 1, np.uint32).reshape(-1),
                grid=np.array([*d.grid_origin, *d.grid_step, *d.grid_cells], np.float32),
                compile_seconds=float(d.compile_seconds), gpu_seconds=float(d.gpu_seconds))
        finally:
            lib.tg_drawable_free(C.byref(d))
        return out

    def reference_words(self) -> np.ndarray:
        lib = load()
        n = lib.tg_tree_reference_words(self.handle, None, 0)
        out = np.zeros(n, np.uint32)
        lib.tg_tree_reference_words(self.handle, _lib.as_ptr(out), n)
        return out


def sphere(r): return Tree(load().MakeSphereBrush(r))
def ellipsoid(x, y, z): return Tree(load().MakeEllipsoidBrush(x, y, z))
def box(x, y, z): return Tree(load().MakeBoxBrush(x, y, z))
def torus(major, minor): return Tree(load().MakeTorusBrush(major, minor))
def cylinder(r, e): return Tree(load().MakeCylinderBrush(r, e))
def plane(x, y, z): return Tree(load().MakePlaneOperand(x, y, z))
def cone(r, h): return Tree(load().MakeConeBrush(r, h))
def coninder(rl, rh, h): return Tree(load().MakeConinderBrush(rl, rh, h))
def union(a: Tree, b: Tree): return Tree(load().MakeUnionOp(a._give(), b._give()))
def diff(a: Tree, b: Tree): return Tree(load().MakeDiffOp(a._give(), b._give()))
def inter(a: Tree, b: Tree): return Tree(load().MakeInterOp(a._give(), b._give()))
def blend_union(k, a: Tree, b: Tree): return Tree(load().MakeBlendUnionOp(k, a._give(), b._give()))
def blend_diff(k, a: Tree, b: Tree): return Tree(load().MakeBlendDiffOp(k, a._give(), b._give()))
def blend_inter(k, a: Tree, b: Tree): return Tree(load().MakeBlendInterOp(k, a._give(), b._give()))
def flate(a: Tree, r): return Tree(load().MakeFlateOp(a._give(), r))
def stencil(a: Tree, mask: Tree, rgb, negative=False):
    return Tree(load().MakeStencilOp(a._give(), mask._give(), *map(float, rgb), bool(negative)))


def has_export_octree(tree: "Tree") -> bool:
    """Whether the tree has finite, non-empty bounds (SDFOctree::Create would succeed);
    host-only, no GPU needed."""
    return load().tg_debug_octree(tree.handle, None, None, 0, None, 0, None) >= 0


def from_spec(spec) -> Tree:
    spec = np.ascontiguousarray(spec, dtype=np.float32)
    return Tree(load().BuildTreeFromSpec(_lib.as_ptr(spec), int(spec.size)))


@dataclass
class Mesh:
    vertices: np.ndarray          # (V, 3) float32
    normals: np.ndarray           # (V, 3) float32
    colors: np.ndarray | None     # (V, 3) uint8
    faces: np.ndarray             # (F, 3) uint32
    cubes: np.ndarray             # (V,) uint32


def _grid(g) -> _lib.Grid:
    if isinstance(g, _lib.Grid):
        return g
    # workloads.ExportGrid: cells -> lattice points
    return _lib.Grid(g.x0, g.y0, g.z0, g.step, g.sx + 1, g.sy + 1, g.sz + 1, getattr(g, "step_y", 0.0),
                     getattr(g, "step_z", 0.0))


def _flags(attributes=True, dense=False, brick=0, lanes=0, surrogate_only=False, staged=False) -> int:
    return ((1 if attributes else 0) | (2 if dense else 0) | ((int(brick) & 0xFF) << 8) | ((int(lanes) & 0xF) << 16)
            | ((1 << 20) if surrogate_only else 0) | ((1 << 21) if staged else 0))


def last_export_stats():
    """(bricks, evaluated bricks) of the last culled export."""
    b, a = C.c_int64(), C.c_int64()
    load().tg_last_export_stats(C.byref(b), C.byref(a))
    return b.value, a.value


def last_export_bricks():
    """(brick indices evaluated by the last culled export, brick edge in cells)."""
    b = C.c_int()
    n = load().tg_last_export_bricks(None, 0, C.byref(b))
    out = np.empty(max(n, 0), np.uint32)
    if n > 0:
        load().tg_last_export_bricks(_lib.as_ptr(out), n, C.byref(b))
    return out, b.value


def last_export_timing():
    """Host seconds of the last tg_export_tree: (compile, upload, gpu, copy)."""
    v = [C.c_double() for _ in range(4)]
    load().tg_last_export_timing(*[C.byref(x) for x in v])
    return tuple(x.value for x in v)


class _HostBlocks:
    """Owns the host blocks of one tg_mesh (pinned memory the library reuses): they go back
    to the library with tg_mesh_free once no array views them."""

    def __init__(self, hm: _lib.HostMesh):
        self.hm = hm

    def __del__(self):
        try:
            load().tg_mesh_free(C.byref(self.hm))
        except Exception:   # interpreter shutdown
            pass


def _take_mesh(hm: _lib.HostMesh) -> Mesh:
    """The mesh's arrays view the library's host blocks without a copy."""
    v, f = int(hm.vertex_count), int(hm.face_count)
    owner = _HostBlocks(hm)

    def arr(ptr, n, ctype, dtype):
        if n == 0 or not ptr:
            return np.zeros(0, dtype)
        buf = (ctype * n).from_address(C.addressof(ptr.contents))
        buf._owner = owner
        return np.frombuffer(buf, dtype)

    return Mesh(arr(hm.vertices, v * 3, C.c_float, np.float32).reshape(v, 3),
                arr(hm.normals, v * 3, C.c_float, np.float32).reshape(v, 3),
                arr(hm.colors, v * 3, C.c_uint8, np.uint8).reshape(v, 3) if hm.colors else None,
                arr(hm.faces, f * 3, C.c_uint32, np.uint32).reshape(f, 3),
                arr(hm.cubes, v, C.c_uint32, np.uint32))


class Program:
    """A tree compiled for the GPU: export octree + per-cell record programs."""

    def __init__(self, tree: Tree):
        self.ptr = C.c_void_p()
        check(load().tg_compile(tree.handle, C.byref(self.ptr)), "tg_compile")

    def close(self):
        if self.ptr and self.ptr.value:
            load().tg_program_free(self.ptr)
            self.ptr = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        if _lib._LIB is not None:
            self.close()

    def info(self) -> _lib.ProgramInfo:
        out = _lib.ProgramInfo()
        check(load().tg_program_get_info(self.ptr, C.byref(out)), "tg_program_get_info")
        return out

    def eval_grid(self, grid, out=None, stream=None) -> np.ndarray:
        g = _grid(grid)
        if out is None:
            out = np.empty((g.nz, g.ny, g.nx), np.float32)
        check(load().tg_eval_grid(self.ptr, C.byref(g), _lib.as_ptr(out), 0, stream), "tg_eval_grid")
        return out

    def eval_grid_device(self, grid, device_ptr: int, stream=None) -> None:
        g = _grid(grid)
        check(load().tg_eval_grid(self.ptr, C.byref(g), C.c_void_p(device_ptr), 1, stream), "tg_eval_grid")

    def eval_points(self, points, stream=None) -> np.ndarray:
        p = np.ascontiguousarray(np.asarray(points, np.float32).reshape(-1, 3))
        out = np.empty(p.shape[0], np.float32)
        check(load().tg_eval_points(self.ptr, _lib.as_ptr(p), p.shape[0], _lib.as_ptr(out), stream), "tg_eval_points")
        return out

    def export_mesh(self, grid, attributes=True, dense=False, brick=0, lanes=0, stream=None, staged=False) -> Mesh:
        g = _grid(grid)
        hm = _lib.HostMesh()
        check(load().tg_export_mesh(self.ptr, C.byref(g), _flags(attributes, dense, brick, lanes, staged=staged), C.byref(hm),
                                    stream),
              "tg_export_mesh")
        return _take_mesh(hm)

    def export_mesh_device(self, grid, attributes=True, dense=False, brick=0, lanes=0, stream=None, staged=False) -> _lib.DeviceMesh:
        g = _grid(grid)
        dm = _lib.DeviceMesh()
        check(load().tg_export_mesh_device(self.ptr, C.byref(g), _flags(attributes, dense, brick, lanes, staged=staged), C.byref(dm), stream),
              "tg_export_mesh_device")
        return dm

    def export_point_cloud(self, lo, hi, step, refine=5, attributes=True, stream=None) -> Mesh:
        """PointCloudExportThread on the GPU: points in voxel order (cubes = voxel numbers)."""
        v3 = lambda v: np.ascontiguousarray(np.broadcast_to(np.asarray(v, np.float32), (3,)))
        lo, hi, step = v3(lo), v3(hi), v3(step)
        hm = _lib.HostMesh()
        check(load().tg_export_point_cloud(self.ptr, _lib.as_ptr(lo), _lib.as_ptr(hi), _lib.as_ptr(step), int(refine),
                                           _flags(attributes, False, 0, 0), C.byref(hm), stream), "tg_export_point_cloud")
        return _take_mesh(hm)

    def export_voxels(self, grid_size, color_index=0, stream=None):
        """VoxExport's voxels on the GPU: ((n, 4) int32 x y z colour, size, radius)."""
        lib = load()
        v = _lib.Voxels()
        check(lib.tg_export_voxels(self.ptr, float(grid_size), int(color_index), C.byref(v), stream), "tg_export_voxels")
        try:
            n = int(v.count)
            vox = (np.ctypeslib.as_array(v.voxels, shape=(n * 4,)).reshape(n, 4).copy() if n else np.zeros((0, 4), np.int32))
            return vox, tuple(v.size), float(v.radius)
        finally:
            lib.tg_voxels_free(C.byref(v))


def write_drawables(drawables, path, frames=None, fmt="ply", scale=1.0):
    """MeshExport(Path, UseBaseColor=True, ...) over Sodapop drawables placed by frames
    (8 floats each: rotation w x y z, translation xyz, scale)."""
    keep = []
    arr = (_lib.Drawable * max(1, len(drawables)))()
    for i, d in enumerate(drawables):
        p = np.ascontiguousarray(d.positions, np.float32)
        n = np.ascontiguousarray(d.normals, np.float32)
        c = np.ascontiguousarray(d.colors, np.float32)
        f = np.ascontiguousarray(d.faces, np.uint32)
        keep += [p, n, c, f]
        arr[i].vertex_count = p.shape[0]
        arr[i].face_count = f.shape[0]
        arr[i].positions = p.ctypes.data_as(C.POINTER(C.c_float))
        arr[i].normals = n.ctypes.data_as(C.POINTER(C.c_float))
        arr[i].colors = c.ctypes.data_as(C.POINTER(C.c_float))
        arr[i].faces = f.ctypes.data_as(C.POINTER(C.c_uint32))
    fr = None if frames is None else np.ascontiguousarray(np.asarray(frames, np.float32).reshape(-1, 8))
    check(load().tg_write_drawables(arr, None if fr is None else _lib.as_ptr(fr), len(drawables), str(path).encode(),
                                    0 if fmt == "stl" else 1, float(scale)), "tg_write_drawables")


def write_vox(voxels, size, path):
    """The MagicaVoxel file VoxWriter writes for these voxels (x, y, z, colour) in order."""
    vox = np.ascontiguousarray(np.asarray(voxels, np.int32).reshape(-1, 4))
    v = _lib.Voxels()
    v.count = vox.shape[0]
    v.voxels = vox.ctypes.data_as(C.POINTER(C.c_int32))
    v.size[:] = [int(s) for s in size]
    check(load().tg_write_vox(C.byref(v), str(path).encode()), "tg_write_vox")


def mesh_export(tree: "Tree", path, lo, hi, step, refine=5, fmt="ply", point_cloud=False, scale=1.0, wait=True):
    """MeshExport (export.h:37): starts the export on the library's export thread; with
    wait (default) returns once the file is written (raising if the job failed)."""
    v3 = lambda v: np.ascontiguousarray(np.broadcast_to(np.asarray(v, np.float32), (3,)))
    lo, hi, step = v3(lo), v3(hi), v3(step)
    check(load().MeshExport(tree.handle, str(path).encode(), _lib.as_ptr(lo), _lib.as_ptr(hi), _lib.as_ptr(step), int(refine),
                            {"stl": 0, "ply": 1, "vox": 2}[fmt], bool(point_cloud), float(scale)), "MeshExport")
    if wait:
        check(load().tg_export_result(1), "MeshExport job")


def export_progress():
    """GetExportProgress: (stage, generation, refinement, secondary, write)."""
    p = load().GetExportProgress()
    return p.Stage, p.Generation, p.Refinement, p.Secondary, p.Write


def cancel_export(halt: bool):
    load().CancelExport(bool(halt))


def export_result(wait=True) -> int:
    """The last MeshExport job's status (tg_export_result)."""
    return int(load().tg_export_result(1 if wait else 0))


def _program_ray_march(self, origins, dirs, iterations=100, epsilon=1e-3, stream=None):
    """SDFNode::RayMarch on the GPU: (hit, travel, position) per ray."""
    o = np.ascontiguousarray(np.asarray(origins, np.float32).reshape(-1, 3))
    d = np.ascontiguousarray(np.asarray(dirs, np.float32).reshape(-1, 3))
    n = o.shape[0]
    hit = np.empty(n, np.uint8)
    travel = np.empty(n, np.float32)
    pos = np.empty((n, 3), np.float32)
    check(load().tg_ray_march(self.ptr, _lib.as_ptr(o), _lib.as_ptr(d), n, iterations, epsilon, _lib.as_ptr(hit),
                              _lib.as_ptr(travel), _lib.as_ptr(pos), stream), "tg_ray_march")
    return hit.astype(bool), travel, pos


def _program_ray_query(self, mode, origins, dirs, frame=None, iterations=100, epsilon=1e-3, stream=None):
    """mode 1: Lua's magnet cast (dirs are targets); mode 2: SDFModel::RayMarch in the model
    frame (quat w x y z, translation xyz, scale)."""
    o = np.ascontiguousarray(np.asarray(origins, np.float32).reshape(-1, 3))
    d = np.ascontiguousarray(np.asarray(dirs, np.float32).reshape(-1, 3))
    fr = np.ascontiguousarray(np.zeros(8, np.float32) if frame is None else np.asarray(frame, np.float32).reshape(8))
    n = o.shape[0]
    hit = np.empty(n, np.uint8)
    travel = np.empty(n, np.float32)
    pos = np.empty((n, 3), np.float32)
    check(load().tg_ray_query(self.ptr, int(mode), _lib.as_ptr(fr), _lib.as_ptr(o), _lib.as_ptr(d), n, iterations, epsilon,
                              _lib.as_ptr(hit), _lib.as_ptr(travel), _lib.as_ptr(pos), stream), "tg_ray_query")
    return hit.astype(bool), travel, pos


def _program_eval_tree(self, points, stream=None):
    """SDFNode::Eval on the whole tree per point (Lua's eval), on the GPU."""
    p = np.ascontiguousarray(np.asarray(points, np.float32).reshape(-1, 3))
    out = np.empty(p.shape[0], np.float32)
    check(load().tg_eval_tree_points(self.ptr, _lib.as_ptr(p), p.shape[0], _lib.as_ptr(out), stream), "tg_eval_tree_points")
    return out


def _program_gradient_tree(self, points, stream=None):
    """SDFNode::Gradient on the whole tree per point (Lua's gradient), on the GPU."""
    p = np.ascontiguousarray(np.asarray(points, np.float32).reshape(-1, 3))
    out = np.empty((p.shape[0], 3), np.float32)
    check(load().tg_gradient_tree_points(self.ptr, _lib.as_ptr(p), p.shape[0], _lib.as_ptr(out), stream), "tg_gradient_tree_points")
    return out


def cameras(positions, target=(0.0, 0.0, 0.0), up=(0.0, 0.0, 1.0), fov_y_degrees=60.0):
    """tg_camera array looking at `target` from each position."""
    import math
    arr = (_lib.Camera * len(positions))()
    t = float(np.float32(math.tan(math.radians(fov_y_degrees) * 0.5)))
    for i, p in enumerate(positions):
        arr[i].position[:] = [float(v) for v in p]
        arr[i].target[:] = [float(v) for v in target]
        arr[i].up[:] = [float(v) for v in up]
        arr[i].tan_half_fov = t
    return arr


def _program_render(self, cams, width, height, steps=256, epsilon=1e-4, exact=False, stream=None):
    """(depth, normals, colors) images, one per camera."""
    n = len(cams)
    depth = np.empty((n, height, width), np.float32)
    normals = np.empty((n, height, width, 3), np.float32)
    colors = np.empty((n, height, width, 3), np.uint8)
    check(load().tg_render(self.ptr, cams, n, width, height, steps, epsilon, 1 if exact else 0, _lib.as_ptr(depth),
                           _lib.as_ptr(normals), _lib.as_ptr(colors), 0, stream), "tg_render")
    return depth, normals, colors


Program.ray_march = _program_ray_march
Program.ray_query = _program_ray_query
Program.eval_tree = _program_eval_tree
Program.gradient_tree = _program_gradient_tree
Program.render = _program_render


def compile(tree: Tree) -> Program:  # noqa: A001 - mirrors tg_compile
    return Program(tree)


def export_tree(tree: Tree, lo, hi, step, stream=None) -> Mesh:
    lo = np.asarray(lo, np.float32)
    hi = np.asarray(hi, np.float32)
    hm = _lib.HostMesh()
    check(load().tg_export_tree(tree.handle, _lib.as_ptr(lo), _lib.as_ptr(hi), float(step), C.byref(hm), stream),
          "tg_export_tree")
    return _take_mesh(hm)


def export_grid(lo, hi, step) -> _lib.Grid:
    lo = np.asarray(lo, np.float32)
    hi = np.asarray(hi, np.float32)
    g = _lib.Grid()
    check(load().tg_export_grid(_lib.as_ptr(lo), _lib.as_ptr(hi), float(step), C.byref(g)), "tg_export_grid")
    return g


def export_grid_axes(lo, hi, steps) -> _lib.Grid:
    """tg_export_grid_axes: MeshExportThread's lattice with a step per axis."""
    v3 = lambda v: np.ascontiguousarray(np.asarray(v, np.float32).reshape(3))
    lo, hi, st = v3(lo), v3(hi), v3(steps)
    g = _lib.Grid()
    check(load().tg_export_grid_axes(_lib.as_ptr(lo), _lib.as_ptr(hi), _lib.as_ptr(st), C.byref(g)), "tg_export_grid_axes")
    return g


def write_ply(mesh: Mesh, path, scale=1.0):
    hm = _host_mesh_view(mesh)
    check(load().tg_write_ply(C.byref(hm), str(path).encode(), scale), "tg_write_ply")


def write_stl(program: Program, mesh: Mesh, path, scale=1.0):
    hm = _host_mesh_view(mesh)
    check(load().tg_write_stl(program.ptr, C.byref(hm), str(path).encode(), scale, None), "tg_write_stl")


def _host_mesh_view(mesh: Mesh) -> _lib.HostMesh:
    """A tg_mesh that points into the numpy arrays (kept alive by `mesh`)."""
    hm = _lib.HostMesh()
    hm.vertex_count = mesh.vertices.shape[0]
    hm.face_count = mesh.faces.shape[0]
    mesh.vertices = np.ascontiguousarray(mesh.vertices, np.float32)
    mesh.normals = np.ascontiguousarray(mesh.normals, np.float32)
    mesh.faces = np.ascontiguousarray(mesh.faces, np.uint32)
    hm.vertices = mesh.vertices.ctypes.data_as(C.POINTER(C.c_float))
    hm.normals = mesh.normals.ctypes.data_as(C.POINTER(C.c_float))
    hm.faces = mesh.faces.ctypes.data_as(C.POINTER(C.c_uint32))
    if mesh.colors is not None:
        mesh.colors = np.ascontiguousarray(mesh.colors, np.uint8)
        hm.colors = mesh.colors.ctypes.data_as(C.POINTER(C.c_uint8))
    return hm


def profile_enable(on=True):
    load().tg_profile_enable(1 if on else 0)


def profile_reset():
    load().tg_profile_reset()


def profile_read(kernel: str):
    ms = C.c_double()
    n = C.c_int64()
    load().tg_profile_read(kernel.encode(), C.byref(ms), C.byref(n))
    return ms.value, n.value


def surrogate_options(**kw) -> _lib.SurrogateOptions:
    """tg_surrogate_options with the library defaults, fields overridden by keyword."""
    o = _lib.SurrogateOptions()
    load().tg_surrogate_default_options(C.byref(o))
    for k, v in kw.items():
        if k in ("domain_min", "domain_max"):
            getattr(o, k)[:] = [float(x) for x in v]
        else:
            setattr(o, k, v)
    return o


class Surrogate:
    """Learned distance bound of one tree (tg_surrogate_*): hash grid + 3x64 network on the
    tensor cores, trained by the library's own kernels."""

    def __init__(self, options: _lib.SurrogateOptions | None = None, **kw):
        if options is None:
            options = surrogate_options(**kw)
        self.ptr = C.c_void_p()
        check(load().tg_surrogate_create(C.byref(options), C.byref(self.ptr)), "tg_surrogate_create")
        info = self.info()
        self.table_floats = int(info.table_floats)
        self.mlp_floats = int(info.mlp_floats)

    def close(self):
        if self.ptr and self.ptr.value:
            load().tg_surrogate_free(self.ptr)
            self.ptr = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        if _lib._LIB is not None:
            self.close()

    def info(self) -> _lib.SurrogateInfo:
        out = _lib.SurrogateInfo()
        check(load().tg_surrogate_get_info(self.ptr, C.byref(out)), "tg_surrogate_get_info")
        return out

    def fit(self, program: Program, stream=None) -> _lib.SurrogateInfo:
        check(load().tg_surrogate_fit(self.ptr, program.ptr, stream), "tg_surrogate_fit")
        return self.info()

    def params(self):
        table = np.empty(self.table_floats, np.float32)
        mlp = np.empty(self.mlp_floats, np.float32)
        check(load().tg_surrogate_get_params(self.ptr, _lib.as_ptr(table), _lib.as_ptr(mlp)), "tg_surrogate_get_params")
        return table, mlp

    def set_params(self, table=None, mlp=None):
        t = None if table is None else np.ascontiguousarray(table, np.float32)
        m = None if mlp is None else np.ascontiguousarray(mlp, np.float32)
        check(load().tg_surrogate_set_params(self.ptr, None if t is None else _lib.as_ptr(t),
                                             None if m is None else _lib.as_ptr(m)), "tg_surrogate_set_params")

    def save(self) -> bytes:
        """Checkpoint: parameters, Adam moments, step count, info and held-out record."""
        n = load().tg_surrogate_save(self.ptr, None, 0)
        if n < 0:
            raise _lib.TangerineError(load().tg_last_error().decode())
        buf = C.create_string_buffer(int(n))
        if load().tg_surrogate_save(self.ptr, buf, n) != n:
            raise _lib.TangerineError(load().tg_last_error().decode())
        return buf.raw

    def restore(self, data: bytes):
        """Restores a checkpoint (save()) of a surrogate with the same grid options."""
        check(load().tg_surrogate_load(self.ptr, data, len(data)), "tg_surrogate_load")

    def eval(self, points, stream=None) -> np.ndarray:
        p = np.ascontiguousarray(np.asarray(points, np.float32).reshape(-1, 3))
        out = np.empty(p.shape[0], np.float32)
        check(load().tg_surrogate_eval(self.ptr, _lib.as_ptr(p), p.shape[0], _lib.as_ptr(out), 0, stream), "tg_surrogate_eval")
        return out

    def gradients(self, samples):
        """(table_grad, mlp_grad, summed squared error) of the mean squared error."""
        s = np.ascontiguousarray(np.asarray(samples, np.float32).reshape(-1, 4))
        tg_ = np.empty(self.table_floats, np.float32)
        mg = np.empty(self.mlp_floats, np.float32)
        loss = C.c_float()
        check(load().tg_surrogate_gradients(self.ptr, _lib.as_ptr(s), s.shape[0], _lib.as_ptr(tg_), _lib.as_ptr(mg),
                                            C.byref(loss)), "tg_surrogate_gradients")
        return tg_, mg, loss.value

    def train(self, samples, steps, stream=None):
        s = np.ascontiguousarray(np.asarray(samples, np.float32).reshape(-1, 4))
        check(load().tg_surrogate_train(self.ptr, _lib.as_ptr(s), s.shape[0], int(steps), stream), "tg_surrogate_train")

    def margin(self, radius) -> float:
        """The margin the culled export uses for bricks whose ball has this radius."""
        m = C.c_float()
        check(load().tg_surrogate_margin(self.ptr, float(radius), C.byref(m)), "tg_surrogate_margin")
        return m.value

    def set_margin(self, margin):
        check(load().tg_surrogate_set_margin(self.ptr, float(margin)), "tg_surrogate_set_margin")

    def render(self, program: Program, cams, width, height, steps=256, epsilon=1e-4, stream=None):
        """(depth, normals, colors) with network steps and exact final steps."""
        n = len(cams)
        depth = np.empty((n, height, width), np.float32)
        normals = np.empty((n, height, width, 3), np.float32)
        colors = np.empty((n, height, width, 3), np.uint8)
        check(load().tg_render_surrogate(program.ptr, self.ptr, cams, n, width, height, steps, epsilon, _lib.as_ptr(depth),
                                         _lib.as_ptr(normals), _lib.as_ptr(colors), 0, stream), "tg_render_surrogate")
        return depth, normals, colors

    def export_mesh(self, program: Program, grid, attributes=True, brick=0, lanes=0, only=False, stream=None) -> Mesh:
        """only: the network alone decides (no exact test of the bricks it keeps)."""
        g = _grid(grid)
        hm = _lib.HostMesh()
        check(load().tg_export_mesh_surrogate(program.ptr, self.ptr, C.byref(g), _flags(attributes, False, brick, lanes, only),
                                              C.byref(hm), stream), "tg_export_mesh_surrogate")
        return _take_mesh(hm)

    def export_mesh_device(self, program: Program, grid, attributes=True, brick=0, lanes=0, only=False,
                           stream=None) -> _lib.DeviceMesh:
        g = _grid(grid)
        dm = _lib.DeviceMesh()
        check(load().tg_export_mesh_surrogate_device(program.ptr, self.ptr, C.byref(g),
                                                     _flags(attributes, False, brick, lanes, only), C.byref(dm), stream),
              "tg_export_mesh_surrogate_device")
        return dm


def last_render_steps():
    """(network iterations, exact steps) of the last network-stepped render."""
    a, b = C.c_uint64(), C.c_uint64()
    load().tg_last_render_steps(C.byref(a), C.byref(b))
    return a.value, b.value


def debug_mma(mode: int, a, b) -> np.ndarray:
    """tg_debug_mma: the tensor-core product through the network kernels' operand layouts."""
    a = np.ascontiguousarray(a, np.float32)
    b = np.ascontiguousarray(b, np.float32)
    n = 144 if mode == 1 else 64
    d = np.zeros((128, n), np.float32)
    check(load().tg_debug_mma(int(mode), _lib.as_ptr(a), _lib.as_ptr(b), _lib.as_ptr(d)), "tg_debug_mma")
    return d


class Batch:
    """Many programs exported together by one persistent launch (tg_batch_*).  The programs
    must stay open while the batch lives."""

    def __init__(self, programs, grids, attributes=True):
        self.programs = list(programs)
        n = len(self.programs)
        arr = (C.c_void_p * n)(*[p.ptr.value for p in self.programs])
        gs = (_lib.Grid * n)(*[_grid(g) for g in grids])
        self.ptr = C.c_void_p()
        check(load().tg_batch_create(arr, gs, n, 1 if attributes else 0, C.byref(self.ptr)), "tg_batch_create")
        self.count = n

    def close(self):
        if self.ptr and self.ptr.value:
            load().tg_batch_free(self.ptr)
            self.ptr = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        if _lib._LIB is not None:
            self.close()

    def autotune(self, stream=None):
        check(load().tg_batch_autotune(self.ptr, stream), "tg_batch_autotune")

    def set_tuning(self, bricks=None, lanes=None):
        b = None if bricks is None else np.ascontiguousarray(bricks, np.int32)
        l = None if lanes is None else np.ascontiguousarray(lanes, np.int32)
        check(load().tg_batch_set_tuning(self.ptr, None if b is None else _lib.as_ptr(b), None if l is None else _lib.as_ptr(l)),
              "tg_batch_set_tuning")

    def tuning(self):
        b = np.empty(self.count, np.int32)
        l = np.empty(self.count, np.int32)
        check(load().tg_batch_get_tuning(self.ptr, _lib.as_ptr(b), _lib.as_ptr(l)), "tg_batch_get_tuning")
        return b, l

    def set_surrogates(self, nets, only=False):
        """Cull model m's bricks with nets[m] (a fitted Surrogate or None for the exact test);
        with only=False the bricks a network keeps also take the exact test."""
        arr = (C.c_void_p * max(1, len(nets)))(*[(n.ptr.value if n is not None else None) for n in nets])
        self._nets = list(nets)       # the networks must outlive the runs
        check(load().tg_batch_set_surrogates(self.ptr, arr, len(nets), (1 << 20) if only else 0), "tg_batch_set_surrogates")

    def run(self, stream=None):
        check(load().tg_batch_run(self.ptr, stream), "tg_batch_run")

    def reserve(self, vertices, faces):
        check(load().tg_batch_reserve(self.ptr, int(vertices), int(faces)), "tg_batch_reserve")

    def info(self) -> _lib.BatchInfo:
        out = _lib.BatchInfo()
        check(load().tg_batch_get_info(self.ptr, C.byref(out)), "tg_batch_get_info")
        return out

    def mesh(self, model: int, stream=None) -> Mesh:
        hm = _lib.HostMesh()
        check(load().tg_batch_mesh(self.ptr, int(model), C.byref(hm), stream), "tg_batch_mesh")
        return _take_mesh(hm)

    def mesh_device(self, model: int) -> _lib.DeviceMesh:
        dm = _lib.DeviceMesh()
        check(load().tg_batch_mesh_device(self.ptr, int(model), C.byref(dm)), "tg_batch_mesh_device")
        return dm
