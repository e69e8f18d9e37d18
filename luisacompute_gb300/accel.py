"""Python host mirror of LuisaCompute's Mesh / Accel API over the C ABI.

Names, arguments and error behaviour follow the reference:
  * ``Mesh(vertices, triangles)`` + ``Mesh.build(request)``   — include/luisa/runtime/rtx/mesh.h:19-141,
    src/runtime/rtx/mesh.cpp:6-12 (borrowed vertex/triangle buffers, stride multiple of 16)
  * ``Accel.emplace_back(mesh, transform, visibility_mask, opaque, user_id)``,
    ``set_transform_on_update``, ``set_visibility_on_update``, ``set_opaque_on_update``,
    ``set_user_id_on_update``, ``pop_back``, ``build(request, update_instance_buffer_only)``
    — include/luisa/runtime/rtx/accel.h:21-134, src/runtime/rtx/accel.cpp:68-249
  * ``Accel.trace_closest(rays, mask)`` / ``trace_any`` — batched forms of the DSL builtins
    ``intersect`` / ``intersect_any`` (src/dsl/rtx/accel.cpp:120-150).
Device memory is torch CUDA tensors; the work runs in liblcx_accel.so.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _capi
from ._capi import (CURVE_BEZIER, CURVE_CATMULL_ROM, CURVE_CUBIC_BSPLINE, CURVE_PIECEWISE_LINEAR, HINT_FAST_BUILD,
                    HINT_FAST_TRACE, MOD_OPAQUE_OFF, MOD_OPAQUE_ON, MOD_PRIMITIVE, MOD_TRANSFORM, MOD_USER_ID,
                    MOD_VISIBILITY, NODES_FP32, NODES_QUANT8, REQUEST_FORCE_BUILD, REQUEST_PREFER_UPDATE,
                    LcxAccelOption, LcxAccelStats, LcxMeshBuildCommand, check)
from .scenes import MOD_DTYPE

__all__ = ["AccelOption", "Mesh", "ProceduralPrimitive", "Curve", "Accel", "HINT_FAST_TRACE", "HINT_FAST_BUILD",
           "REQUEST_FORCE_BUILD", "REQUEST_PREFER_UPDATE", "NODES_FP32", "NODES_QUANT8", "CURVE_PIECEWISE_LINEAR",
           "CURVE_CUBIC_BSPLINE", "CURVE_CATMULL_ROM", "CURVE_BEZIER", "stream_handle"]


def _torch():
    import torch
    return torch


def stream_handle(stream) -> int | None:
    """cudaStream_t of a torch stream (None = the current torch stream)."""
    torch = _torch()
    if stream is None:
        stream = torch.cuda.current_stream()
    return int(stream.cuda_stream) if hasattr(stream, "cuda_stream") else int(stream)


class AccelOption:
    """include/luisa/runtime/rhi/resource.h:94-125 (hint, allow_compaction, allow_update)."""

    def __init__(self, hint: int = HINT_FAST_TRACE, allow_compaction: bool = True, allow_update: bool = False):
        self.hint, self.allow_compaction, self.allow_update = hint, allow_compaction, allow_update

    def c(self) -> LcxAccelOption:
        return LcxAccelOption(self.hint, int(self.allow_compaction), int(self.allow_update))


def _as_affine(transform) -> np.ndarray:
    """4x4 (column vectors, as float4x4 rows here in row-major numpy) or 3x4 -> row-major 3x4
    (the packing of Modification::set_transform, include/luisa/runtime/rhi/command.h:557-571)."""
    m = np.asarray(transform, np.float32)
    if m.shape == (4, 4):
        m = m[:3, :]
    return np.ascontiguousarray(m.reshape(12), np.float32)


class Mesh:
    """A BLAS over borrowed device vertex/triangle buffers."""

    def __init__(self, vertices, triangles, option: AccelOption | None = None, vertex_stride: int | None = None,
                 motion_keyframes: int = 0, time_start: float = 0.0, time_end: float = 1.0,
                 vanish_start: bool = False, vanish_end: bool = False):
        """motion_keyframes >= 2: keyframed vertices (lcx_mesh_create_motion); `vertices` then holds
        that many copies of the vertex set back to back."""
        torch = _torch()
        self.lib = _capi.load()
        self.vertices, self.triangles = vertices, triangles
        if not (vertices.is_cuda and triangles.is_cuda):
            raise ValueError("Mesh buffers must be CUDA tensors")
        stride = vertex_stride or vertices.stride(0) * vertices.element_size()
        self.vertex_stride = stride
        self.vertex_size = vertices.shape[0] * stride
        self.triangle_size = triangles.numel() * triangles.element_size()
        if triangles.dtype not in (torch.int32, torch.uint32) or triangles.numel() % 3 != 0:
            raise ValueError("triangles must be a (T, 3) int32/uint32 tensor")
        h = ctypes.c_uint64(0)
        if motion_keyframes >= 2:
            mo = _capi.LcxMotionOption(motion_keyframes, time_start, time_end, int(vanish_start), int(vanish_end), 0, 0)
            check(self.lib.lcx_mesh_create_motion(ctypes.byref((option or AccelOption()).c()), ctypes.byref(mo),
                                                  ctypes.byref(h)), "lcx_mesh_create_motion")
        else:
            check(self.lib.lcx_mesh_create(ctypes.byref((option or AccelOption()).c()), ctypes.byref(h)),
                  "lcx_mesh_create")
        self.handle = h.value

    def build(self, request: int = REQUEST_FORCE_BUILD, stream=None) -> "Mesh":
        cmd = LcxMeshBuildCommand(request, 0, self.vertices.data_ptr(), 0, self.vertex_size, self.vertex_stride,
                                  self.triangles.data_ptr(), 0, self.triangle_size)
        check(self.lib.lcx_mesh_build(self.handle, ctypes.byref(cmd), stream_handle(stream)), "lcx_mesh_build")
        return self

    def stats(self) -> LcxAccelStats:
        s = LcxAccelStats()
        check(self.lib.lcx_mesh_stats(self.handle, ctypes.byref(s)), "lcx_mesh_stats")
        return s

    def destroy(self):
        if getattr(self, "handle", 0):
            check(self.lib.lcx_mesh_destroy(self.handle), "lcx_mesh_destroy")
            self.handle = 0

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass


class ProceduralPrimitive:
    """A BLAS over AABBs (include/luisa/runtime/rtx/procedural_primitive.h): ``aabbs`` is an (N, 6)
    float32 CUDA tensor of (min xyz, max xyz) records, borrowed like a mesh's buffers.  Instanced by
    an Accel like a Mesh; only lcx::ray_query (user kernels) reports its candidates."""

    def __init__(self, aabbs, option: AccelOption | None = None):
        torch = _torch()
        self.lib = _capi.load()
        if not aabbs.is_cuda or aabbs.dtype != torch.float32 or aabbs.dim() != 2 or aabbs.shape[1] != 6 \
                or not aabbs.is_contiguous():
            raise ValueError("aabbs must be a contiguous (N, 6) float32 CUDA tensor")
        self.aabbs = aabbs
        h = ctypes.c_uint64(0)
        check(self.lib.lcx_procedural_create(ctypes.byref((option or AccelOption()).c()), ctypes.byref(h)),
              "lcx_procedural_create")
        self.handle = h.value

    def build(self, request: int = REQUEST_FORCE_BUILD, stream=None) -> "ProceduralPrimitive":
        cmd = _capi.LcxProceduralBuildCommand(request, 0, self.aabbs.data_ptr(), 0, self.aabbs.numel() * 4)
        check(self.lib.lcx_procedural_build(self.handle, ctypes.byref(cmd), stream_handle(stream)),
              "lcx_procedural_build")
        return self

    def stats(self) -> LcxAccelStats:
        s = LcxAccelStats()
        check(self.lib.lcx_mesh_stats(self.handle, ctypes.byref(s)), "lcx_mesh_stats")
        return s

    def destroy(self):
        if getattr(self, "handle", 0):
            check(self.lib.lcx_procedural_destroy(self.handle), "lcx_procedural_destroy")
            self.handle = 0

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass


class Curve:
    """A BLAS over curve segments (include/luisa/runtime/rtx/curve.h): ``control_points`` is an (N, 4)
    float32 CUDA tensor of (x, y, z, radius) records, ``segments`` a uint32 / int32 CUDA tensor with the
    first control point of each segment; ``basis`` is one of CURVE_PIECEWISE_LINEAR, CURVE_CUBIC_BSPLINE,
    CURVE_CATMULL_ROM, CURVE_BEZIER.  Both buffers are borrowed like a mesh's.  Instanced by an Accel like
    a Mesh; hits on it report prim = segment, bary = (u, -1).  motion_keyframes >= 2: keyframed control
    points (lcx_curve_create_motion); ``control_points`` then holds that many copies back to back and
    ``segments`` index one copy."""

    def __init__(self, basis: int, control_points, segments, option: AccelOption | None = None,
                 motion_keyframes: int = 0, time_start: float = 0.0, time_end: float = 1.0,
                 vanish_start: bool = False, vanish_end: bool = False):
        torch = _torch()
        self.lib = _capi.load()
        if not control_points.is_cuda or control_points.dtype != torch.float32 or control_points.dim() != 2 \
                or control_points.shape[1] != 4 or not control_points.is_contiguous():
            raise ValueError("control_points must be a contiguous (N, 4) float32 CUDA tensor")
        if not segments.is_cuda or segments.dtype not in (torch.int32, torch.uint32) or segments.dim() != 1 \
                or not segments.is_contiguous():
            raise ValueError("segments must be a contiguous 1-D int32 / uint32 CUDA tensor")
        self.basis = int(basis)
        self.control_points = control_points
        self.segments = segments
        h = ctypes.c_uint64(0)
        if motion_keyframes >= 2:
            mo = _capi.LcxMotionOption(motion_keyframes, time_start, time_end, int(vanish_start), int(vanish_end), 0, 0)
            check(self.lib.lcx_curve_create_motion(ctypes.byref((option or AccelOption()).c()), ctypes.byref(mo),
                                                   ctypes.byref(h)), "lcx_curve_create_motion")
        else:
            check(self.lib.lcx_curve_create(ctypes.byref((option or AccelOption()).c()), ctypes.byref(h)),
                  "lcx_curve_create")
        self.handle = h.value

    def build(self, request: int = REQUEST_FORCE_BUILD, stream=None) -> "Curve":
        cmd = _capi.LcxCurveBuildCommand(request, self.basis, self.control_points.data_ptr(), 0, 16,
                                         self.control_points.shape[0], self.segments.data_ptr(), 0,
                                         self.segments.numel())
        check(self.lib.lcx_curve_build(self.handle, ctypes.byref(cmd), stream_handle(stream)), "lcx_curve_build")
        return self

    def stats(self) -> LcxAccelStats:
        s = LcxAccelStats()
        check(self.lib.lcx_mesh_stats(self.handle, ctypes.byref(s)), "lcx_mesh_stats")
        return s

    def destroy(self):
        if getattr(self, "handle", 0):
            check(self.lib.lcx_curve_destroy(self.handle), "lcx_curve_destroy")
            self.handle = 0

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass


class Accel:
    """A TLAS over instanced meshes; modifications are staged and sent by build()."""

    def __init__(self, option: AccelOption | None = None):
        self.lib = _capi.load()
        h = ctypes.c_uint64(0)
        check(self.lib.lcx_accel_create(ctypes.byref((option or AccelOption()).c()), ctypes.byref(h)),
              "lcx_accel_create")
        self.handle = h.value
        self._count = 0
        self._mods: dict = {}
        self._meshes: dict = {}  # keeps Python Mesh objects alive while referenced

    def __len__(self):
        return self._count

    def _mod(self, index: int) -> np.ndarray:
        if index not in self._mods:
            m = np.zeros(1, MOD_DTYPE)[0]
            m["index"] = index
            self._mods[index] = m
        return self._mods[index]

    def emplace_back(self, mesh: Mesh, transform=None, visibility_mask: int = 0xFF, opaque: bool = True,
                     user_id: int = 0) -> int:
        index = self._count
        m = self._mod(index)
        m["primitive"] = mesh.handle
        m["affine"] = _as_affine(np.eye(4) if transform is None else transform)
        m["vis_mask"] = visibility_mask & 0xFF
        m["user_id"] = user_id
        m["flags"] = (MOD_PRIMITIVE | MOD_TRANSFORM | MOD_VISIBILITY | MOD_USER_ID |
                      (MOD_OPAQUE_ON if opaque else MOD_OPAQUE_OFF))
        self._meshes[index] = mesh
        self._count += 1
        return index

    def emplace_back_many(self, meshes, affines: np.ndarray, masks=None):
        """Bulk emplace_back: meshes[i] with row-major 3x4 affines[i]."""
        n = len(meshes)
        base = self._count
        arr = np.zeros(n, MOD_DTYPE)
        arr["index"] = np.arange(base, base + n)
        arr["primitive"] = [m.handle for m in meshes]
        arr["affine"] = np.asarray(affines, np.float32).reshape(n, 12)
        arr["vis_mask"] = 0xFF if masks is None else np.asarray(masks) & 0xFF
        arr["flags"] = MOD_PRIMITIVE | MOD_TRANSFORM | MOD_VISIBILITY | MOD_USER_ID | MOD_OPAQUE_ON
        for i in range(n):
            self._mods[base + i] = arr[i]
            self._meshes[base + i] = meshes[i]
        self._count += n

    def pop_back(self):
        if self._count == 0:
            return  # the reference only warns (src/runtime/rtx/accel.cpp:108-110)
        self._count -= 1
        self._mods.pop(self._count, None)
        self._meshes.pop(self._count, None)

    def set(self, index: int, mesh, transform=None, visibility_mask: int = 0xFF, opaque: bool = True,
            user_id: int = 0):
        """Replace instance ``index`` (src/runtime/rtx/accel.cpp:114-131, 163-178): its primitive (a Mesh,
        Curve, ProceduralPrimitive or MotionInstance), transform, mask, opacity and user id."""
        self._check_index(index)
        m = self._mod(index)
        m["primitive"] = mesh.handle
        m["affine"] = _as_affine(np.eye(4) if transform is None else transform)
        m["vis_mask"] = visibility_mask & 0xFF
        m["user_id"] = user_id
        m["flags"] = (MOD_PRIMITIVE | MOD_TRANSFORM | MOD_VISIBILITY | MOD_USER_ID |
                      (MOD_OPAQUE_ON if opaque else MOD_OPAQUE_OFF))
        self._meshes[index] = mesh

    def set_mesh_on_update(self, index: int, mesh: Mesh):
        """Replace only the primitive of instance ``index`` (the reference's set_mesh / set_curve /
        set_procedural_primitive / set_motion_instance, accel.cpp:179-193)."""
        self._check_index(index)
        m = self._mod(index)
        m["primitive"] = mesh.handle
        m["flags"] |= MOD_PRIMITIVE
        self._meshes[index] = mesh

    set_mesh = set_curve = set_procedural_primitive = set_motion_instance = set_mesh_on_update

    def set_transform_on_update(self, index: int, transform):
        self._check_index(index)
        m = self._mod(index)
        m["affine"] = _as_affine(transform)
        m["flags"] |= MOD_TRANSFORM

    def set_visibility_on_update(self, index: int, visibility_mask: int):
        self._check_index(index)
        m = self._mod(index)
        m["vis_mask"] = visibility_mask & 0xFF
        m["flags"] |= MOD_VISIBILITY

    def set_opaque_on_update(self, index: int, opaque: bool):
        self._check_index(index)
        m = self._mod(index)
        m["flags"] = (m["flags"] & ~(MOD_OPAQUE_ON | MOD_OPAQUE_OFF)) | (MOD_OPAQUE_ON if opaque else MOD_OPAQUE_OFF)

    def set_user_id_on_update(self, index: int, user_id: int):
        self._check_index(index)
        m = self._mod(index)
        m["user_id"] = user_id
        m["flags"] |= MOD_USER_ID

    def _check_index(self, index: int):
        if not 0 <= index < self._count:
            raise IndexError(f"instance index {index} out of range [0, {self._count})")

    def build(self, request: int = REQUEST_FORCE_BUILD, update_instance_buffer_only: bool = False,
              stream=None) -> "Accel":
        mods = np.array([self._mods[k] for k in sorted(self._mods)], MOD_DTYPE) if self._mods else \
            np.zeros(0, MOD_DTYPE)
        ptr = mods.ctypes.data if mods.size else None
        check(self.lib.lcx_accel_build(self.handle, self._count, request, ptr, mods.size,
                                       int(update_instance_buffer_only), stream_handle(stream)), "lcx_accel_build")
        self._mods.clear()
        return self

    def stats(self) -> LcxAccelStats:
        s = LcxAccelStats()
        check(self.lib.lcx_accel_stats(self.handle, ctypes.byref(s)), "lcx_accel_stats")
        return s

    # ------------------------------------------------------------ queries
    @staticmethod
    def _rays_ptr(rays):
        if not rays.is_cuda or not rays.is_contiguous() or rays.numel() * rays.element_size() % 32 != 0:
            raise ValueError("rays must be a contiguous CUDA tensor of 32-byte Ray records")
        return rays.data_ptr(), rays.numel() * rays.element_size() // 32

    def trace_closest(self, rays, mask: int = 0xFF, out=None, layout: int = NODES_QUANT8, stream=None,
                      counts=None):
        """Closest hits as an (N, 6) int32 tensor of TriangleHit records (view floats with
        ``hits_view``)."""
        torch = _torch()
        ptr, n = self._rays_ptr(rays)
        if out is None:
            out = torch.empty((n, 6), dtype=torch.int32, device=rays.device)
        if counts is not None:
            check(self.lib.lcx_trace_closest_counts(self.handle, ptr, n, mask, out.data_ptr(), counts.data_ptr(),
                                                    layout, stream_handle(stream)), "lcx_trace_closest_counts")
        else:
            check(self.lib.lcx_trace_closest_ex(self.handle, ptr, n, mask, out.data_ptr(), layout,
                                                stream_handle(stream)), "lcx_trace_closest")
        return out

    def trace_closest_motion(self, rays, times=None, mask: int = 0xFF, out=None, layout: int = NODES_QUANT8,
                             stream=None):
        """lcx_trace_closest_motion: rays with a time each (a float32 CUDA tensor, None = 0)."""
        torch = _torch()
        ptr, n = self._rays_ptr(rays)
        if out is None:
            out = torch.empty((n, 6), dtype=torch.int32, device=rays.device)
        tp = 0 if times is None else times.data_ptr()
        check(self.lib.lcx_trace_closest_motion(self.handle, ptr, tp or None, n, mask, out.data_ptr(), layout,
                                                stream_handle(stream)), "lcx_trace_closest_motion")
        return out

    def trace_any_motion(self, rays, times=None, mask: int = 0xFF, out=None, layout: int = NODES_QUANT8,
                         stream=None):
        torch = _torch()
        ptr, n = self._rays_ptr(rays)
        if out is None:
            out = torch.empty(n, dtype=torch.uint8, device=rays.device)
        tp = 0 if times is None else times.data_ptr()
        check(self.lib.lcx_trace_any_motion(self.handle, ptr, tp or None, n, mask, out.data_ptr(), layout,
                                            stream_handle(stream)), "lcx_trace_any_motion")
        return out

    def trace_any(self, rays, mask: int = 0xFF, out=None, layout: int = NODES_QUANT8, stream=None):
        torch = _torch()
        ptr, n = self._rays_ptr(rays)
        if out is None:
            out = torch.empty(n, dtype=torch.uint8, device=rays.device)
        check(self.lib.lcx_trace_any_ex(self.handle, ptr, n, mask, out.data_ptr(), layout, stream_handle(stream)),
              "lcx_trace_any")
        return out

    def instance_buffer(self):
        """lcx_accel_instance_buffer: the instance records for device-side edits
        (include/lcx/accel_instances.cuh)."""
        b = _capi.LcxInstanceBuffer()
        check(self.lib.lcx_accel_instance_buffer(self.handle, ctypes.byref(b)), "lcx_accel_instance_buffer")
        return b

    # ------------------------------------------------- host-buffer queries
    @staticmethod
    def _host_ptr(buf, rec: int, what: str):
        """(address, records) of a contiguous host buffer: a CPU torch tensor (pinned for
        overlapped copies) or a numpy array."""
        if isinstance(buf, np.ndarray):
            if not buf.flags.c_contiguous or buf.nbytes % rec:
                raise ValueError(f"{what}: contiguous array of {rec}-byte records expected")
            return buf.ctypes.data, buf.nbytes // rec
        if buf.is_cuda or not buf.is_contiguous() or buf.numel() * buf.element_size() % rec:
            raise ValueError(f"{what}: contiguous CPU tensor of {rec}-byte records expected")
        return buf.data_ptr(), buf.numel() * buf.element_size() // rec

    def trace_closest_host(self, rays, out, mask: int = 0xFF, layout: int = NODES_QUANT8, stream=None):
        """lcx_trace_closest_host: rays and hits in host memory; `out` is complete once `stream`
        (default: the current torch stream) is synchronised."""
        rp, n = self._host_ptr(rays, 32, "rays")
        hp, m = self._host_ptr(out, 24, "hits")
        if m < n:
            raise ValueError("hit buffer smaller than the ray count")
        check(self.lib.lcx_trace_closest_host(self.handle, rp, n, mask, hp, layout, stream_handle(stream)),
              "lcx_trace_closest_host")
        return out

    def trace_any_host(self, rays, out, mask: int = 0xFF, layout: int = NODES_QUANT8, stream=None):
        rp, n = self._host_ptr(rays, 32, "rays")
        op, m = self._host_ptr(out, 1, "occluded")
        if m < n:
            raise ValueError("occluded buffer smaller than the ray count")
        check(self.lib.lcx_trace_any_host(self.handle, rp, n, mask, op, layout, stream_handle(stream)),
              "lcx_trace_any_host")
        return out

    def destroy(self):
        if getattr(self, "handle", 0):
            check(self.lib.lcx_accel_destroy(self.handle), "lcx_accel_destroy")
            self.handle = 0

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass


class MotionInstance:
    """A motion instance (include/luisa/runtime/rtx/motion_instance.h) of a built mesh: matrix
    keyframes (row-major 3x4 or 4x4 each) spaced evenly over [time_start, time_end].  An Accel
    instances it like a mesh (``emplace_back``); traces move it at each ray's time
    (``trace_closest_motion``)."""

    def __init__(self, mesh: Mesh, keyframes, time_start: float = 0.0, time_end: float = 1.0,
                 vanish_start: bool = False, vanish_end: bool = False, stream=None, srt: bool = False):
        self.lib = _capi.load()
        self.mesh = mesh
        self.srt = srt  # keyframes are 16-float SRT records (pivot, quaternion, scale, shear, translation)
        keys = self._pack(keyframes)
        opt = _capi.LcxMotionOption(keys.shape[0], time_start, time_end, int(vanish_start), int(vanish_end),
                                    _capi.LCX_MOTION_SRT if srt else _capi.LCX_MOTION_MATRIX, 0)
        h = ctypes.c_uint64(0)
        check(self.lib.lcx_motion_instance_create(mesh.handle, ctypes.byref(opt), ctypes.byref(h)),
              "lcx_motion_instance_create")
        self.handle = h.value
        self.set_keyframes(keys)
        self.build(stream)

    def _pack(self, keyframes) -> np.ndarray:
        if self.srt:
            return np.ascontiguousarray(np.asarray(keyframes, np.float32).reshape(-1, 16))
        return np.ascontiguousarray(np.stack([_as_affine(k) for k in keyframes]), np.float32)

    def set_keyframes(self, keyframes):
        keys = self._pack(keyframes)
        check(self.lib.lcx_motion_instance_set_keyframes(self.handle, keys.ctypes.data, keys.shape[0]),
              "lcx_motion_instance_set_keyframes")
        self.keys = keys

    def build(self, stream=None) -> "MotionInstance":
        check(self.lib.lcx_motion_instance_build(self.handle, stream_handle(stream)), "lcx_motion_instance_build")
        return self

    def destroy(self):
        if getattr(self, "handle", 0):
            check(self.lib.lcx_motion_instance_destroy(self.handle), "lcx_motion_instance_destroy")
            self.handle = 0

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass


def build_meshes(meshes, request: int = REQUEST_FORCE_BUILD, stream=None):
    """Build many meshes with one lcx_mesh_build_batch call (one sort, one LBVH pass,
    one collapse and one emit for all of them)."""
    lib = _capi.load()
    n = len(meshes)
    handles = (ctypes.c_uint64 * n)(*[m.handle for m in meshes])
    cmds = (LcxMeshBuildCommand * n)()
    for i, m in enumerate(meshes):
        cmds[i] = LcxMeshBuildCommand(request, 0, m.vertices.data_ptr(), 0, m.vertex_size, m.vertex_stride,
                                      m.triangles.data_ptr(), 0, m.triangle_size)
    check(lib.lcx_mesh_build_batch(handles, cmds, n, stream_handle(stream)), "lcx_mesh_build_batch")
    return meshes


def reserve_meshes(meshes, stream=None, build: bool = True):
    """lcx_mesh_build_batch_reserve: build the batch and keep room to rebuild it in place (later
    ``build_meshes`` calls of the same meshes over the same buffers, capturable in CUDA graphs).
    build=False: lcx_mesh_reserve_batch, the room only; the first ``build_meshes`` of the batch is
    then already the in-place build and can itself be captured."""
    lib = _capi.load()
    n = len(meshes)
    handles = (ctypes.c_uint64 * n)(*[m.handle for m in meshes])
    cmds = (LcxMeshBuildCommand * n)()
    for i, m in enumerate(meshes):
        cmds[i] = LcxMeshBuildCommand(REQUEST_FORCE_BUILD, 0, m.vertices.data_ptr(), 0, m.vertex_size,
                                      m.vertex_stride, m.triangles.data_ptr(), 0, m.triangle_size)
    fn = lib.lcx_mesh_build_batch_reserve if build else lib.lcx_mesh_reserve_batch
    check(fn(handles, cmds, n, stream_handle(stream)), fn.__name__)
    return meshes


def set_refit_sync(sync: bool):
    """Refit mode of later PREFER_UPDATE mesh builds: True synchronises once to report bad
    indices from the call; False only enqueues kernels (capturable in a CUDA graph) and leaves
    errors for ``lcx_check_trace_errors``."""
    check(_capi.load().lcx_set_refit_sync(1 if sync else 0), "lcx_set_refit_sync")


def hits_to_numpy(hits) -> np.ndarray:
    """(N, 6) int32 device tensor -> numpy TriangleHit records."""
    from .scenes import HIT_DTYPE
    return hits.cpu().numpy().view(HIT_DTYPE).reshape(-1)


def rays_to_device(rays: np.ndarray, device="cuda"):
    torch = _torch()
    return torch.from_numpy(np.ascontiguousarray(rays).view(np.float32).reshape(-1, 8)).to(device)


def mesh_from_data(md, device="cuda", option: AccelOption | None = None) -> Mesh:
    torch = _torch()
    v = torch.from_numpy(np.ascontiguousarray(md.vertices, np.float32)).to(device)
    t = torch.from_numpy(np.ascontiguousarray(md.triangles).astype(np.int32)).to(device)
    return Mesh(v, t, option)


def accel_from_scene(scene, device="cuda", option: AccelOption | None = None, stream=None, batch: bool = False):
    """Build every mesh and one TLAS for a scenes.Scene; returns (accel, meshes).
    batch=True builds all meshes with one lcx_mesh_build_batch call."""
    if batch:
        meshes = build_meshes([mesh_from_data(m, device, option) for m in scene.meshes], stream=stream)
    else:
        meshes = [mesh_from_data(m, device, option).build(stream=stream) for m in scene.meshes]
    acc = Accel(option)
    acc.emplace_back_many([meshes[i] for i in scene.inst_mesh], scene.inst_affine, scene.inst_mask)
    acc.build(stream=stream)
    return acc, meshes
