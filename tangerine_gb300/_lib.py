"""ctypes binding of libtangerine_gb300.so (the C ABI in include/tangerine_gb300.h).

The library must have been built (``tangerine_gb300.build.build()``); loading fails
loudly otherwise -- there is no CPU fallback.
"""

from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

LIB_PATH = Path(__file__).resolve().parent / "libtangerine_gb300.so"


class RayHit(C.Structure):
    _fields_ = [("Hit", C.c_bool), ("Travel", C.c_float), ("Position", C.c_float * 3)]


class Grid(C.Structure):
    _fields_ = [("x0", C.c_float), ("y0", C.c_float), ("z0", C.c_float), ("step", C.c_float),
                ("nx", C.c_int64), ("ny", C.c_int64), ("nz", C.c_int64), ("step_y", C.c_float), ("step_z", C.c_float)]


class Camera(C.Structure):
    _fields_ = [("position", C.c_float * 3), ("target", C.c_float * 3), ("up", C.c_float * 3), ("tan_half_fov", C.c_float)]


class ProgramInfo(C.Structure):
    _fields_ = [("octree_cells", C.c_int32), ("code_quads", C.c_int32), ("materials", C.c_int32),
                ("has_paint", C.c_int32), ("max_stack", C.c_int32),
                ("bounds_min", C.c_float * 3), ("bounds_max", C.c_float * 3),
                ("compile_seconds", C.c_double), ("distance_quads", C.c_int64)]


class HostMesh(C.Structure):
    _fields_ = [("vertex_count", C.c_uint64), ("face_count", C.c_uint64),
                ("vertices", C.POINTER(C.c_float)), ("normals", C.POINTER(C.c_float)),
                ("colors", C.POINTER(C.c_uint8)), ("faces", C.POINTER(C.c_uint32)),
                ("cubes", C.POINTER(C.c_uint32))]


class DeviceMesh(C.Structure):
    _fields_ = [("vertex_count", C.c_uint64), ("face_count", C.c_uint64),
                ("vertices", C.c_void_p), ("normals", C.c_void_p), ("colors", C.c_void_p),
                ("faces", C.c_void_p), ("cubes", C.c_void_p)]


class SurrogateOptions(C.Structure):
    _fields_ = [("log2_table", C.c_int), ("base_resolution", C.c_int), ("max_resolution", C.c_int),
                ("domain_min", C.c_float * 3), ("domain_max", C.c_float * 3), ("clamp", C.c_float),
                ("samples", C.c_int64), ("band", C.c_float), ("batch", C.c_int64), ("steps", C.c_int),
                ("learning_rate", C.c_float), ("validation", C.c_int64), ("safety", C.c_float), ("seed", C.c_uint64)]


class SurrogateInfo(C.Structure):
    _fields_ = [("max_error", C.c_float), ("p99_error", C.c_float), ("mean_error", C.c_float), ("margin", C.c_float),
                ("final_loss", C.c_float), ("data_seconds", C.c_double), ("train_seconds", C.c_double),
                ("samples", C.c_int64), ("steps", C.c_int), ("resolutions", C.c_int * 16), ("table_size", C.c_uint32),
                ("dense_levels", C.c_uint32), ("table_floats", C.c_int64), ("mlp_floats", C.c_int64)]


class BatchInfo(C.Structure):
    _fields_ = [("models", C.c_int64), ("samples", C.c_int64), ("bricks", C.c_int64), ("bricks_evaluated", C.c_int64),
                ("vertices", C.c_int64), ("faces", C.c_int64), ("graph", C.c_int), ("blocks", C.c_int), ("reruns", C.c_int),
                ("autotune_seconds", C.c_double), ("device_bytes", C.c_int64)]


class Drawable(C.Structure):
    _fields_ = [("vertex_count", C.c_uint64), ("face_count", C.c_uint64),
                ("positions", C.POINTER(C.c_float)), ("normals", C.POINTER(C.c_float)),
                ("colors", C.POINTER(C.c_float)), ("faces", C.POINTER(C.c_uint32)),
                ("cells", C.POINTER(C.c_uint32)), ("grid_origin", C.c_float * 3), ("grid_step", C.c_float * 3),
                ("grid_cells", C.c_int64 * 3), ("compile_seconds", C.c_double), ("gpu_seconds", C.c_double)]


class ExportProgress(C.Structure):
    _fields_ = [("Stage", C.c_int), ("Generation", C.c_float), ("Refinement", C.c_float), ("Secondary", C.c_float),
                ("Write", C.c_float)]


class Voxels(C.Structure):
    _fields_ = [("count", C.c_uint64), ("voxels", C.POINTER(C.c_int32)), ("size", C.c_int32 * 3), ("radius", C.c_float)]


# Every exported symbol with its signature: (restype, argtypes).
_vp, _f, _i, _i64, _u32 = C.c_void_p, C.c_float, C.c_int, C.c_int64, C.c_uint32
SIGNATURES = {
    "EvalTree": (_f, [_vp, _f, _f, _f]),
    "ClipTree": (_vp, [_vp, _f, _f, _f, _f]),
    "RayMarchTree": (RayHit, [_vp, _f, _f, _f, _f, _f, _f, _i, _f]),
    "DiscardTree": (None, [_vp]),
    "TreeHasFiniteBounds": (C.c_bool, [_vp]),
    "MoveTree": (None, [_vp, _f, _f, _f]),
    "RotateTree": (None, [_vp, _f, _f, _f, _f]),
    "AlignTree": (None, [_vp, _f, _f, _f]),
    "PaintTree": (None, [_f, _f, _f, _vp]),
    "MakeSphereBrush": (_vp, [_f]),
    "MakeEllipsoidBrush": (_vp, [_f, _f, _f]),
    "MakeBoxBrush": (_vp, [_f, _f, _f]),
    "MakeTorusBrush": (_vp, [_f, _f]),
    "MakeCylinderBrush": (_vp, [_f, _f]),
    "MakePlaneOperand": (_vp, [_f, _f, _f]),
    "MakeUnionOp": (_vp, [_vp, _vp]),
    "MakeDiffOp": (_vp, [_vp, _vp]),
    "MakeInterOp": (_vp, [_vp, _vp]),
    "MakeBlendUnionOp": (_vp, [_f, _vp, _vp]),
    "MakeBlendDiffOp": (_vp, [_f, _vp, _vp]),
    "MakeBlendInterOp": (_vp, [_f, _vp, _vp]),
    "MakeConeBrush": (_vp, [_f, _f]),
    "MakeConinderBrush": (_vp, [_f, _f, _f]),
    "MakeFlateOp": (_vp, [_vp, _f]),
    "MakeStencilOp": (_vp, [_vp, _vp, _f, _f, _f, C.c_bool]),
    "ScaleTree": (None, [_vp, _f]),
    "BuildTreeFromSpec": (_vp, [_vp, _i]),
    "tg_tree_spec": (_i64, [_vp, _vp, _i64]),
    "CopyTree": (_vp, [_vp]),
    "GradientTree": (None, [_vp, _f, _f, _f, _vp]),
    "PaintOverTree": (None, [_f, _f, _f, _vp]),
    "RotateTreeX": (None, [_vp, _f]),
    "RotateTreeY": (None, [_vp, _f]),
    "RotateTreeZ": (None, [_vp, _f]),
    "ExportSTL": (None, [_vp, _f, _i, C.c_char_p]),
    "ExportPLY": (None, [_vp, _f, _i, C.c_char_p]),
    "tg_compile": (_i, [_vp, C.POINTER(_vp)]),
    "tg_program_free": (None, [_vp]),
    "tg_program_get_info": (_i, [_vp, C.POINTER(ProgramInfo)]),
    "tg_tree_reference_words": (_i64, [_vp, _vp, _i64]),
    "tg_debug_octree": (_i64, [_vp, _vp, _vp, _i64, _vp, _i64, C.POINTER(_i64)]),
    "tg_debug_meshing_octree": (_i64, [_vp, _vp, _vp, _i64, _vp, _i64, C.POINTER(_i64)]),
    "tg_debug_compile_seconds": (_i, [_vp, _i, C.POINTER(C.c_double), C.POINTER(C.c_double)]),
    "tg_debug_root_program_check": (_i, [_vp, C.POINTER(C.c_int64), C.POINTER(C.c_int32)]),
    "tg_debug_deferred_surfaces_check": (_i, [_vp]),
    "tg_debug_sodapop_plan": (_i, [_vp, _f, _vp, _vp, _i64, C.POINTER(_i64)]),
    "tg_sodapop_mesh": (_i, [_vp, _f, C.POINTER(Drawable), _vp]),
    "tg_export_point_cloud": (_i, [_vp, _vp, _vp, _vp, _i, _u32, C.POINTER(HostMesh), _vp]),
    "tg_export_voxels": (_i, [_vp, _f, _i, C.POINTER(Voxels), _vp]),
    "tg_voxels_free": (None, [C.POINTER(Voxels)]),
    "tg_write_vox": (_i, [C.POINTER(Voxels), C.c_char_p]),
    "ExportMagicaVoxel": (None, [_vp, _f, _i, C.c_char_p]),
    "MeshExport": (_i, [_vp, C.c_char_p, _vp, _vp, _vp, _i, _i, C.c_bool, _f]),
    "GetExportProgress": (ExportProgress, []),
    "CancelExport": (None, [C.c_bool]),
    "tg_export_result": (_i, [_i]),
    "tg_debug_export_pause": (None, [_i]),
    "tg_debug_export_paused": (_i, [_i]),
    "tg_export_grid_axes": (_i, [_vp, _vp, _vp, C.POINTER(Grid)]),
    "tg_ray_query": (_i, [_vp, _i, _vp, _vp, _vp, _i64, _i, _f, _vp, _vp, _vp, _vp]),
    "tg_eval_tree_points": (_i, [_vp, _vp, _i64, _vp, _vp]),
    "tg_gradient_tree_points": (_i, [_vp, _vp, _i64, _vp, _vp]),
    "tg_drawable_free": (None, [C.POINTER(Drawable)]),
    "tg_write_drawables": (_i, [_vp, _vp, _i, C.c_char_p, _i, _f]),
    "tg_export_grid": (_i, [_vp, _vp, _f, C.POINTER(Grid)]),
    "tg_eval_grid": (_i, [_vp, C.POINTER(Grid), _vp, _i, _vp]),
    "tg_eval_points": (_i, [_vp, _vp, _i64, _vp, _vp]),
    "tg_export_mesh": (_i, [_vp, C.POINTER(Grid), _u32, C.POINTER(HostMesh), _vp]),
    "tg_export_mesh_device": (_i, [_vp, C.POINTER(Grid), _u32, C.POINTER(DeviceMesh), _vp]),
    "tg_mesh_free": (None, [C.POINTER(HostMesh)]),
    "tg_export_mesh_noalloc": (_i, [_vp, C.POINTER(Grid), _u32, _vp, _vp, _vp, _vp, _vp, C.c_uint64, C.c_uint64,
                                    C.POINTER(C.c_uint64), _vp]),
    "tg_export_tree": (_i, [_vp, _vp, _vp, _f, C.POINTER(HostMesh), _vp]),
    "tg_ray_march": (_i, [_vp, _vp, _vp, _i64, _i, _f, _vp, _vp, _vp, _vp]),
    "tg_render": (_i, [_vp, C.POINTER(Camera), _i, _i, _i, _i, _f, _u32, _vp, _vp, _vp, _i, _vp]),
    "tg_write_ply": (_i, [C.POINTER(HostMesh), C.c_char_p, _f]),
    "tg_write_stl": (_i, [_vp, C.POINTER(HostMesh), C.c_char_p, _f, _vp]),
    "tg_last_export_stats": (_i, [C.POINTER(_i64), C.POINTER(_i64)]),
    "tg_last_export_bricks": (_i64, [_vp, _i64, C.POINTER(_i)]),
    "tg_last_export_timing": (_i, [C.POINTER(C.c_double)] * 4),
    "tg_profile_enable": (None, [_i]),
    "tg_profile_read": (_i, [C.c_char_p, C.POINTER(C.c_double), C.POINTER(_i64)]),
    "tg_profile_reset": (None, []),
    "tg_measure_fp32_peak": (_i, [C.POINTER(C.c_double), _vp]),
    "tg_batch_create": (_i, [C.POINTER(_vp), C.POINTER(Grid), _i, _u32, C.POINTER(_vp)]),
    "tg_batch_free": (None, [_vp]),
    "tg_batch_autotune": (_i, [_vp, _vp]),
    "tg_batch_set_tuning": (_i, [_vp, _vp, _vp]),
    "tg_batch_get_tuning": (_i, [_vp, _vp, _vp]),
    "tg_batch_set_surrogates": (_i, [_vp, _vp, _i, _u32]),
    "tg_batch_run": (_i, [_vp, _vp]),
    "tg_batch_cancel": (_i, [_vp, _i]),
    "tg_batch_debug_barrier": (_i, [_vp, C.c_uint64, _i, C.c_uint64]),
    "tg_debug_wait_test": (_i, [_i, C.c_uint64]),
    "tg_surrogate_save": (_i64, [_vp, _vp, _i64]),
    "tg_surrogate_load": (_i, [_vp, _vp, _i64]),
    "tg_batch_reserve": (_i, [_vp, C.c_uint64, C.c_uint64]),
    "tg_batch_get_info": (_i, [_vp, C.POINTER(BatchInfo)]),
    "tg_batch_mesh": (_i, [_vp, _i, C.POINTER(HostMesh), _vp]),
    "tg_batch_mesh_device": (_i, [_vp, _i, C.POINTER(DeviceMesh)]),
    "tg_surrogate_default_options": (None, [C.POINTER(SurrogateOptions)]),
    "tg_surrogate_create": (_i, [C.POINTER(SurrogateOptions), C.POINTER(_vp)]),
    "tg_surrogate_free": (None, [_vp]),
    "tg_surrogate_fit": (_i, [_vp, _vp, _vp]),
    "tg_surrogate_get_info": (_i, [_vp, C.POINTER(SurrogateInfo)]),
    "tg_surrogate_get_params": (_i, [_vp, _vp, _vp]),
    "tg_surrogate_set_params": (_i, [_vp, _vp, _vp]),
    "tg_surrogate_eval": (_i, [_vp, _vp, _i64, _vp, _i, _vp]),
    "tg_surrogate_gradients": (_i, [_vp, _vp, _i64, _vp, _vp, _vp]),
    "tg_surrogate_train": (_i, [_vp, _vp, _i64, _i, _vp]),
    "tg_surrogate_set_margin": (_i, [_vp, _f]),
    "tg_surrogate_margin": (_i, [_vp, _f, C.POINTER(_f)]),
    "tg_export_mesh_surrogate": (_i, [_vp, _vp, C.POINTER(Grid), _u32, C.POINTER(HostMesh), _vp]),
    "tg_export_mesh_surrogate_device": (_i, [_vp, _vp, C.POINTER(Grid), _u32, C.POINTER(DeviceMesh), _vp]),
    "tg_render_surrogate": (_i, [_vp, _vp, C.POINTER(Camera), _i, _i, _i, _i, _f, _vp, _vp, _vp, _i, _vp]),
    "tg_last_render_steps": (_i, [C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)]),
    "tg_debug_mma": (_i, [_i, _vp, _vp, _vp]),
    "tg_debug_blend_check": (_i, [C.c_uint64, C.c_uint64, _vp]),
    "tg_debug_pair_check": (_i, [C.c_uint64, C.c_uint64, _vp]),
    "tg_last_error": (C.c_char_p, []),
    "tg_version": (C.c_char_p, []),
}

_LIB = None


def load(path: Path | str | None = None) -> C.CDLL:
    """Loads the in-tree library and binds every entry point; raises if it is missing."""
    global _LIB
    if _LIB is not None and path is None:
        return _LIB
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise RuntimeError(f"{p} is not built: run tangerine_gb300.build.build() (the GPU path has no fallback)")
    lib = C.CDLL(str(p))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _LIB = lib
    return lib


class TangerineError(RuntimeError):
    pass


def check(status: int, what: str = "") -> None:
    if status != 0:
        msg = load().tg_last_error()
        raise TangerineError(f"{what or 'call'} failed (status {status}): {msg.decode() if msg else ''}")


def as_ptr(a: np.ndarray) -> C.c_void_p:
    return C.c_void_p(a.ctypes.data)
