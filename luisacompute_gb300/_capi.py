"""ctypes binding of the C ABI declared in include/lcx_accel.h."""
from __future__ import annotations

import ctypes
import os
import re
from ctypes import POINTER, c_char_p, c_double, c_int, c_size_t, c_uint8, c_uint32, c_uint64, c_void_p
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent
HEADER = ROOT / "include" / "lcx_accel.h"
LIB_PATH = Path(__file__).resolve().parent / "_lib" / "liblcx_accel.so"

LCX_OK = 0
LCX_ERR_INVALID_ARG = -1
LCX_MOTION_MATRIX = 0
LCX_MOTION_SRT = 1
LCX_ERR_OOM = -2
LCX_ERR_NOT_BUILT = -3
LCX_ERR_TIMEOUT = -4
LCX_ERR_CUDA = -5
LCX_ERR_DEPTH = -6
ERROR_NAMES = {0: "LCX_OK", -1: "LCX_ERR_INVALID_ARG", -2: "LCX_ERR_OOM", -3: "LCX_ERR_NOT_BUILT",
               -4: "LCX_ERR_TIMEOUT", -5: "LCX_ERR_CUDA", -6: "LCX_ERR_DEPTH"}

HINT_FAST_TRACE, HINT_FAST_BUILD = 0, 1
REQUEST_PREFER_UPDATE, REQUEST_FORCE_BUILD = 0, 1
NODES_FP32, NODES_QUANT8 = 0, 1
HOST_AUTO, HOST_STAGED, HOST_DIRECT, HOST_STREAMED = 0, 1, 2, 3
MOD_PRIMITIVE, MOD_TRANSFORM, MOD_OPAQUE_ON, MOD_OPAQUE_OFF, MOD_VISIBILITY, MOD_USER_ID = 1, 2, 4, 8, 16, 32


class LcxAccelOption(ctypes.Structure):
    _fields_ = [("hint", c_uint32), ("allow_compaction", c_uint8), ("allow_update", c_uint8),
                ("_pad", c_uint8 * 2)]


class LcxMeshBuildCommand(ctypes.Structure):
    _fields_ = [("request", c_uint32), ("_pad", c_uint32), ("vertex_buffer", c_uint64),
                ("vertex_buffer_offset", c_size_t), ("vertex_buffer_size", c_size_t), ("vertex_stride", c_size_t),
                ("triangle_buffer", c_uint64), ("triangle_buffer_offset", c_size_t),
                ("triangle_buffer_size", c_size_t)]


class LcxTraceJob(ctypes.Structure):
    _fields_ = [("accel", c_uint64), ("rays", c_void_p), ("out", c_void_p), ("ray_count", c_uint32),
                ("mask", c_uint32), ("any", c_uint32), ("_pad", c_uint32)]


class LcxPtMesh(ctypes.Structure):
    _fields_ = [("vertices", c_void_p), ("vertex_stride", c_uint64), ("triangles", c_void_p), ("albedo", c_void_p)]


class LcxPtParams(ctypes.Structure):
    _fields_ = [("width", c_uint32), ("height", c_uint32), ("spp", c_uint32), ("max_bounces", c_uint32),
                ("rr_start", c_uint32), ("seed", c_uint32), ("eye", ctypes.c_float * 3),
                ("target", ctypes.c_float * 3), ("up", ctypes.c_float * 3), ("tan_half_fov", ctypes.c_float),
                ("light_pos", ctypes.c_float * 3), ("light_intensity", ctypes.c_float * 3),
                ("env", ctypes.c_float * 3)]


class LcxProceduralBuildCommand(ctypes.Structure):
    _fields_ = [("request", c_uint32), ("_pad", c_uint32), ("aabb_buffer", c_uint64),
                ("aabb_buffer_offset", c_size_t), ("aabb_buffer_size", c_size_t)]


class LcxCurveBuildCommand(ctypes.Structure):
    _fields_ = [("request", c_uint32), ("basis", c_uint32), ("cp_buffer", c_uint64), ("cp_buffer_offset", c_size_t),
                ("cp_stride", c_size_t), ("cp_count", c_size_t), ("seg_buffer", c_uint64),
                ("seg_buffer_offset", c_size_t), ("seg_count", c_size_t)]


CURVE_PIECEWISE_LINEAR, CURVE_CUBIC_BSPLINE, CURVE_CATMULL_ROM, CURVE_BEZIER = 0, 1, 2, 3


class LcxInstanceBuffer(ctypes.Structure):
    _fields_ = [("states", c_void_p), ("count", c_uint32), ("_pad", c_uint32)]


class LcxMotionOption(ctypes.Structure):
    _fields_ = [("keyframe_count", c_uint32), ("time_start", ctypes.c_float), ("time_end", ctypes.c_float),
                ("vanish_start", c_uint8), ("vanish_end", c_uint8), ("mode", c_uint8), ("_pad", c_uint8)]


class LcxAccelView(ctypes.Structure):
    _fields_ = [("tlas_nodes", c_void_p), ("instances", c_void_p), ("stack_need", c_uint32), ("motion", c_uint32)]


class LcxRay(ctypes.Structure):
    _fields_ = [("origin", ctypes.c_float * 3), ("t_min", ctypes.c_float), ("direction", ctypes.c_float * 3),
                ("t_max", ctypes.c_float)]


class LcxTriangleHit(ctypes.Structure):
    _fields_ = [("inst", c_uint32), ("prim", c_uint32), ("bary", ctypes.c_float * 2), ("committed_ray_t", ctypes.c_float),
                ("_pad", c_uint32)]


class LcxMat4(ctypes.Structure):
    _fields_ = [("m", ctypes.c_float * 16)]


class LcxCpuCommittedHit(ctypes.Structure):
    _fields_ = [("inst", c_uint32), ("prim", c_uint32), ("bary", ctypes.c_float * 2), ("hit_type", c_uint32),
                ("committed_ray_t", ctypes.c_float)]


class LcxCpuRayQuery(ctypes.Structure):
    """defs::RayQuery (the reference's cpu_kernel_defs/src/lib.rs:127-141), 128 B."""
    _fields_ = [("hit", LcxCpuCommittedHit), ("_a", ctypes.c_uint8 * 8), ("ray", LcxRay), ("mask", c_uint32),
                ("cur_committed_ray_t", ctypes.c_float), ("cur_triangle_hit", LcxTriangleHit),
                ("cur_procedural_inst", c_uint32), ("cur_procedural_prim", c_uint32), ("cur_commited", ctypes.c_bool),
                ("terminate_on_first", ctypes.c_bool), ("terminated", ctypes.c_bool), ("_b", ctypes.c_uint8 * 5),
                ("user_data", c_void_p), ("accel", c_void_p)]


LcxCpuHitCallback = ctypes.CFUNCTYPE(None, ctypes.POINTER(LcxCpuRayQuery))
CpuTraceClosest = ctypes.CFUNCTYPE(LcxTriangleHit, c_void_p, ctypes.POINTER(LcxRay), c_uint32)
CpuTraceAny = ctypes.CFUNCTYPE(ctypes.c_bool, c_void_p, ctypes.POINTER(LcxRay), c_uint32)
CpuSetU32 = ctypes.CFUNCTYPE(None, c_void_p, c_uint32, c_uint32)
CpuSetTransform = ctypes.CFUNCTYPE(None, c_void_p, c_uint32, ctypes.POINTER(LcxMat4))
CpuGetTransform = ctypes.CFUNCTYPE(LcxMat4, c_void_p, c_uint32)
CpuGetU32 = ctypes.CFUNCTYPE(c_uint32, c_void_p, c_uint32)
CpuRayQueryFn = ctypes.CFUNCTYPE(None, c_void_p, ctypes.POINTER(LcxCpuRayQuery), LcxCpuHitCallback,
                                 LcxCpuHitCallback)


class LcxCpuAccel(ctypes.Structure):
    """The CPU backend's per-ray accel table (defs::Accel, cpu_kernel_defs/src/lib.rs:111-125)."""
    _fields_ = [("handle", c_void_p), ("trace_closest", CpuTraceClosest), ("trace_any", CpuTraceAny),
                ("set_instance_visibility", CpuSetU32), ("set_instance_transform", CpuSetTransform),
                ("set_instance_user_id", CpuSetU32), ("instance_transform", CpuGetTransform),
                ("instance_user_id", CpuGetU32), ("instance_visibility_mask", CpuGetU32),
                ("ray_query", CpuRayQueryFn)]


class LcxPtStats(ctypes.Structure):
    _fields_ = [("closest_rays", c_uint64), ("any_rays", c_uint64), ("bounces", c_uint32), ("ms", ctypes.c_float),
                ("launches", c_uint32), ("_pad", c_uint32)]


class LcxAccelStats(ctypes.Structure):
    _fields_ = [("node_count", c_uint64), ("leaf_prim_count", c_uint64), ("device_bytes", c_uint64),
                ("depth", c_uint32), ("max_blas_depth", c_uint32), ("sah_cost", c_double),
                ("wide_sah_cost", c_double), ("refits", c_uint64)]


_SIGS = {
    "lcx_device_init": (c_int, [c_int]),
    "lcx_last_error_string": (c_char_p, []),
    "lcx_version": (c_uint32, []),
    "lcx_mesh_create": (c_int, [POINTER(LcxAccelOption), POINTER(c_uint64)]),
    "lcx_mesh_destroy": (c_int, [c_uint64]),
    "lcx_mesh_build": (c_int, [c_uint64, POINTER(LcxMeshBuildCommand), c_void_p]),
    "lcx_mesh_stats": (c_int, [c_uint64, POINTER(LcxAccelStats)]),
    "lcx_mesh_build_batch": (c_int, [c_void_p, c_void_p, c_uint32, c_void_p]),
    "lcx_set_build_tuning": (c_int, [c_uint32, c_uint32]),
    "lcx_get_build_tuning": (c_int, [POINTER(c_uint32), POINTER(c_uint32)]),
    "lcx_set_build_morton": (c_int, [c_uint32, c_uint32, c_uint32]),
    "lcx_accel_device_view": (c_int, [c_uint64, POINTER(LcxAccelView)]),
    "lcx_procedural_create": (c_int, [POINTER(LcxAccelOption), POINTER(c_uint64)]),
    "lcx_procedural_destroy": (c_int, [c_uint64]),
    "lcx_procedural_build": (c_int, [c_uint64, POINTER(LcxProceduralBuildCommand), c_void_p]),
    "lcx_curve_create": (c_int, [POINTER(LcxAccelOption), POINTER(c_uint64)]),
    "lcx_curve_destroy": (c_int, [c_uint64]),
    "lcx_curve_build": (c_int, [c_uint64, POINTER(LcxCurveBuildCommand), c_void_p]),
    "lcx_get_build_morton": (c_int, [POINTER(c_uint32), POINTER(c_uint32), POINTER(c_uint32)]),
    "lcx_set_trace_reorder": (c_int, [c_uint32, c_uint32]),
    "lcx_set_trace_stack": (c_int, [c_uint32]),
    "lcx_trace_closest_host": (c_int, [c_uint64, c_void_p, c_uint32, c_uint32, c_void_p, c_uint32, c_void_p]),
    "lcx_trace_any_host": (c_int, [c_uint64, c_void_p, c_uint32, c_uint32, c_void_p, c_uint32, c_void_p]),
    "lcx_set_host_access": (c_int, [c_uint32]),
    "lcx_trace_jobs_motion": (c_int, [c_void_p, c_void_p, c_uint32, c_uint32, c_void_p]),
    "lcx_get_host_access": (c_int, [POINTER(c_uint32), POINTER(c_uint32)]),
    "lcx_release_scratch": (c_int, []),
    "lcx_set_host_chunk": (c_int, [c_uint32]),
    "lcx_accel_instance_buffer": (c_int, [c_uint64, POINTER(LcxInstanceBuffer)]),
    "lcx_set_build_split": (c_int, [ctypes.c_float]),
    "lcx_get_build_split": (c_int, [POINTER(ctypes.c_float)]),
    "lcx_set_build_fill": (c_int, [c_uint32]),
    "lcx_set_build_tlas_sah": (c_int, [c_uint32]),
    "lcx_get_build_tlas_sah": (c_int, [POINTER(c_uint32)]),
    "lcx_set_build_collapse": (c_int, [c_uint32]),
    "lcx_get_build_collapse": (c_int, [POINTER(c_uint32)]),
    "lcx_set_build_blas_sah": (c_int, [c_uint32]),
    "lcx_get_build_blas_sah": (c_int, [POINTER(c_uint32)]),
    "lcx_get_build_kernel_launches": (c_int, [POINTER(c_uint64)]),
    "lcx_get_build_fill": (c_int, [POINTER(c_uint32)]),
    "lcx_mesh_build_batch_reserve": (c_int, [c_void_p, c_void_p, c_uint32, c_void_p]),
    "lcx_mesh_reserve_batch": (c_int, [c_void_p, c_void_p, c_uint32, c_void_p]),
    "lcx_mesh_create_motion": (c_int, [c_void_p, c_void_p, POINTER(c_uint64)]),
    "lcx_curve_create_motion": (c_int, [c_void_p, c_void_p, POINTER(c_uint64)]),
    "lcx_motion_instance_create": (c_int, [c_uint64, c_void_p, POINTER(c_uint64)]),
    "lcx_motion_instance_destroy": (c_int, [c_uint64]),
    "lcx_motion_instance_set_keyframes": (c_int, [c_uint64, c_void_p, c_uint32]),
    "lcx_motion_instance_build": (c_int, [c_uint64, c_void_p]),
    "lcx_trace_closest_motion": (c_int, [c_uint64, c_void_p, c_void_p, c_uint32, c_uint32, c_void_p, c_uint32,
                                         c_void_p]),
    "lcx_trace_any_motion": (c_int, [c_uint64, c_void_p, c_void_p, c_uint32, c_uint32, c_void_p, c_uint32, c_void_p]),
    "lcx_set_refit_sync": (c_int, [c_uint32]),
    "lcx_get_trace_stack": (c_int, [POINTER(c_uint32)]),
    "lcx_accel_cpu_table": (c_int, [c_uint64, POINTER(LcxCpuAccel)]),
    "lcx_set_trace_step_bound": (c_int, [c_uint32]),
    "lcx_get_trace_step_bound": (c_int, [POINTER(c_uint32)]),
    "lcx_get_trace_reorder": (c_int, [POINTER(c_uint32), POINTER(c_uint32)]),
    "lcx_accel_create": (c_int, [POINTER(LcxAccelOption), POINTER(c_uint64)]),
    "lcx_accel_destroy": (c_int, [c_uint64]),
    "lcx_accel_build": (c_int, [c_uint64, c_uint32, c_uint32, c_void_p, c_size_t, c_int, c_void_p]),
    "lcx_accel_stats": (c_int, [c_uint64, POINTER(LcxAccelStats)]),
    "lcx_trace_closest": (c_int, [c_uint64, c_void_p, c_uint32, c_uint32, c_void_p, c_void_p]),
    "lcx_trace_any": (c_int, [c_uint64, c_void_p, c_uint32, c_uint32, c_void_p, c_void_p]),
    "lcx_trace_closest_ex": (c_int, [c_uint64, c_void_p, c_uint32, c_uint32, c_void_p, c_uint32, c_void_p]),
    "lcx_trace_any_ex": (c_int, [c_uint64, c_void_p, c_uint32, c_uint32, c_void_p, c_uint32, c_void_p]),
    "lcx_trace_closest_counts": (c_int, [c_uint64, c_void_p, c_uint32, c_uint32, c_void_p, c_void_p, c_uint32,
                                         c_void_p]),
    "lcx_set_trace_tuning": (c_int, [c_uint32, c_uint32, c_uint32]),
    "lcx_check_trace_errors": (c_int, []),
    "lcx_trace_jobs": (c_int, [c_void_p, c_uint32, c_uint32, c_void_p]),
    "lcx_pt_render": (c_int, [c_uint64, c_void_p, c_uint32, c_void_p, c_void_p, c_uint32, c_void_p, c_void_p,
                              c_void_p, c_void_p, c_void_p]),
    "lcx_trace_closest_noalloc": (c_int, [c_uint64, c_void_p, c_uint32, c_uint32, c_void_p, c_void_p]),
    "lcx_get_trace_tuning": (c_int, [POINTER(c_uint32), POINTER(c_uint32), POINTER(c_uint32)]),
}


def declared_symbols(header: Path = HEADER) -> list:
    """Function names declared with LCX_API in a header."""
    text = header.read_text()
    return sorted(set(re.findall(r"LCX_API\s+[\w\s\*]+?\b(lcx_\w+)\s*\(", text)))


class LcxError(RuntimeError):
    def __init__(self, code: int, where: str, message: str):
        super().__init__(f"{where}: {ERROR_NAMES.get(code, code)}: {message}")
        self.code = code


_lib = None


def load(path: Path | None = None) -> ctypes.CDLL:
    """Load liblcx_accel.so.  Raises if the library has not been built: there
    is no fallback implementation of this path."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path else Path(os.environ.get("LCX_ACCEL_LIB", LIB_PATH))
    if not p.exists():
        raise RuntimeError(f"{p} is missing: build it with luisacompute_gb300.build.build() "
                           "(the GB300 kernels are the only implementation of this path)")
    lib = ctypes.CDLL(str(p))
    for name, (res, args) in _SIGS.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib


def check(code: int, where: str):
    if code != LCX_OK:
        msg = load().lcx_last_error_string()
        raise LcxError(code, where, msg.decode() if msg else "")
