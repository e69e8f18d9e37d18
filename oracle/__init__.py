"""CPU oracle for the Mesh/Accel path — TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py (its cpu_baseline leg and
the ``--impl reference`` arm) may load this module; the product never does.
It wraps liblcx_oracle.so (lcx_oracle.cpp), a C++ restatement of the
reference CPU backend's semantics for trace_closest / trace_any
(src/rust/luisa_compute_backend_impl/src/cpu/accel.rs:449-535) with a
binned-SAH BVH, the FP32 watertight triangle test and an FP64 adjudicator.
Parity against the reference's own outputs is unpinned: the reference ships
no golden vectors for this path and its CPU backend (Rust + Embree) cannot
be built here.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from ctypes import POINTER, c_double, c_float, c_int, c_size_t, c_uint32, c_void_p
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "liblcx_oracle.so"
F64_DTYPE = np.dtype([("hit", "<i4"), ("pad", "<i4"), ("t", "<f8"), ("u", "<f8"), ("v", "<f8"),
                      ("min_bary", "<f8")])

_lib = None


def build():
    r = subprocess.run(["make", "-s", "-C", str(HERE)], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{r.stdout}\n{r.stderr}")
    return LIB


def load():
    global _lib
    if _lib is None:
        if not LIB.exists():
            build()
        lib = ctypes.CDLL(str(LIB))
        lib.lcxo_mesh_create.restype = c_void_p
        lib.lcxo_mesh_create.argtypes = [c_void_p, c_size_t, c_size_t, c_void_p, c_size_t, c_int, c_int]
        lib.lcxo_mesh_destroy.argtypes = [c_void_p]
        lib.lcxo_mesh_sah.restype = c_double
        lib.lcxo_mesh_sah.argtypes = [c_void_p]
        lib.lcxo_mesh_depth.restype = c_uint32
        lib.lcxo_mesh_depth.argtypes = [c_void_p]
        lib.lcxo_accel_create.restype = c_void_p
        lib.lcxo_accel_create.argtypes = [c_size_t, POINTER(c_void_p), c_void_p, c_void_p]
        lib.lcxo_accel_destroy.argtypes = [c_void_p]
        for name in ("lcxo_trace_closest", "lcxo_brute_closest"):
            getattr(lib, name).argtypes = [c_void_p, c_void_p, c_size_t, c_uint32, c_void_p, c_int]
        lib.lcxo_trace_any.argtypes = [c_void_p, c_void_p, c_size_t, c_uint32, c_void_p, c_int]
        lib.lcxo_fp64_closest.argtypes = [c_void_p, c_void_p, c_size_t, c_uint32, c_void_p, c_void_p, c_int]
        lib.lcxo_fp64_eval.argtypes = [c_void_p, c_void_p, c_size_t, c_void_p, c_void_p, c_void_p]
        lib.lcxo_affine_inverse.argtypes = [c_void_p, c_void_p]
        lib.lcxo_trace_motion.argtypes = [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_size_t, c_uint32,
                                          c_int, c_void_p, c_void_p, c_int]
        lib.lcxo_pathtrace.argtypes = [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_int]
        lib.lcxo_curve_create.restype = c_void_p
        lib.lcxo_curve_create.argtypes = [c_void_p, c_size_t, c_size_t, c_void_p, c_size_t, c_uint32]
        lib.lcxo_curve_destroy.argtypes = [c_void_p]
        lib.lcxo_curve_pieces.restype = c_uint32
        lib.lcxo_curve_pieces.argtypes = [c_void_p, c_size_t]
        lib.lcxo_trace_curves.argtypes = [c_void_p, c_void_p, c_void_p, c_size_t, c_void_p, c_size_t, c_uint32, c_int,
                                          c_void_p, c_void_p, c_int]
        lib.lcxo_curve_create_motion.restype = c_void_p
        lib.lcxo_curve_create_motion.argtypes = [c_void_p, c_size_t, c_size_t, c_uint32, c_void_p, c_size_t, c_uint32,
                                                 c_float, c_float, c_uint32]
        lib.lcxo_trace_curves_t.argtypes = [c_void_p, c_void_p, c_void_p, c_size_t, c_void_p, c_void_p, c_size_t,
                                            c_uint32, c_int, c_void_p, c_void_p, c_int]
        lib.lcxo_intersect_triangle.restype = c_int
        lib.lcxo_intersect_triangle.argtypes = [c_void_p, c_void_p, c_float, c_float, c_void_p, c_void_p, c_void_p,
                                                POINTER(c_float), POINTER(c_float), POINTER(c_float)]
        _lib = lib
    return _lib


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(c_void_p)


class LcxoMotion(ctypes.Structure):
    _fields_ = [("keys", ctypes.POINTER(ctypes.c_float)), ("count", ctypes.c_uint32), ("t0", ctypes.c_float),
                ("t1", ctypes.c_float), ("flags", ctypes.c_uint32)]


class LcxoMeshMotion(ctypes.Structure):
    _fields_ = [("verts", ctypes.POINTER(ctypes.c_float)), ("stride_floats", ctypes.c_size_t),
                ("vcount", ctypes.c_uint32), ("keys", ctypes.c_uint32), ("tris", ctypes.POINTER(ctypes.c_uint32)),
                ("tri_count", ctypes.c_uint32), ("t0", ctypes.c_float), ("t1", ctypes.c_float),
                ("flags", ctypes.c_uint32)]


class OracleScene:
    """A scene (scenes.Scene) built on the CPU: one binned-SAH BVH per mesh, one over instances."""

    def __init__(self, scene, leaf_size: int = 4, bins: int = 32):
        from luisacompute_gb300.scenes import HIT_DTYPE  # noqa: F401  (layout shared with the product)
        lib = load()
        self.lib = lib
        self._keep = []
        self.meshes = []
        for md in scene.meshes:
            v = np.ascontiguousarray(md.vertices, np.float32)
            t = np.ascontiguousarray(md.triangles, np.uint32)
            self._keep += [v, t]
            self.meshes.append(lib.lcxo_mesh_create(_ptr(v), v.shape[1], v.shape[0], _ptr(t), t.shape[0],
                                                    leaf_size, bins))
        n = scene.instance_count
        arr = (c_void_p * n)(*[self.meshes[i] for i in scene.inst_mesh])
        aff = np.ascontiguousarray(scene.inst_affine, np.float32)
        masks = np.ascontiguousarray(scene.inst_mask, np.uint32)
        self._keep += [aff, masks]
        self.accel = lib.lcxo_accel_create(n, arr, _ptr(aff), _ptr(masks))

    def mesh_sah(self, i: int) -> float:
        return float(self.lib.lcxo_mesh_sah(self.meshes[i]))

    def trace_closest(self, rays: np.ndarray, mask: int = 0xFF, threads: int = 0) -> np.ndarray:
        from luisacompute_gb300.scenes import HIT_DTYPE
        rays = np.ascontiguousarray(rays)
        hits = np.zeros(rays.shape[0], HIT_DTYPE)
        self.lib.lcxo_trace_closest(self.accel, _ptr(rays), rays.shape[0], mask, _ptr(hits), threads)
        return hits

    def brute_closest(self, rays: np.ndarray, mask: int = 0xFF, threads: int = 0) -> np.ndarray:
        from luisacompute_gb300.scenes import HIT_DTYPE
        rays = np.ascontiguousarray(rays)
        hits = np.zeros(rays.shape[0], HIT_DTYPE)
        self.lib.lcxo_brute_closest(self.accel, _ptr(rays), rays.shape[0], mask, _ptr(hits), threads)
        return hits

    def trace_motion(self, rays: np.ndarray, times: np.ndarray, motion: list, mask: int = 0xFF, any_hit: bool = False,
                     threads: int = 0, mesh_motion: list | None = None):
        """Rays with per-ray times over the scene whose instance i moves by motion[i] = (keys (k, 12),
        or (k, 16) SRT records with flags bit 2, float32, t0, t1, flags) or stays static (None);
        lcxo_trace_motion."""
        from luisacompute_gb300.scenes import HIT_DTYPE
        import ctypes
        rays = np.ascontiguousarray(rays)
        times = np.ascontiguousarray(times, np.float32)
        arr = (LcxoMotion * len(motion))()
        keep = []
        for i, mo in enumerate(motion):
            if mo is None:
                continue
            keys = np.ascontiguousarray(mo[0], np.float32).reshape(-1, 16 if mo[3] & 4 else 12)
            keep.append(keys)
            arr[i] = LcxoMotion(keys.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), keys.shape[0], mo[1], mo[2], mo[3])
        marr = None
        if mesh_motion is not None:  # per instance: (vertices (keys*V, >=3) float32, keys, triangles, t0, t1, flags)
            marr = (LcxoMeshMotion * len(mesh_motion))()
            for i, mm in enumerate(mesh_motion):
                if mm is None:
                    continue
                verts = np.ascontiguousarray(mm[0], np.float32)
                tris = np.ascontiguousarray(mm[2], np.uint32).reshape(-1, 3)
                keep += [verts, tris]
                marr[i] = LcxoMeshMotion(verts.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), verts.shape[1],
                                         verts.shape[0] // mm[1], mm[1],
                                         tris.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)), tris.shape[0],
                                         mm[3], mm[4], mm[5])
        hits = np.zeros(rays.shape[0], HIT_DTYPE)
        occ = np.zeros(rays.shape[0], np.uint8)
        self.lib.lcxo_trace_motion(self.accel, arr, marr, _ptr(rays), _ptr(times), rays.shape[0], mask,
                                   int(any_hit), _ptr(hits), _ptr(occ), threads)
        return occ if any_hit else hits

    def trace_any(self, rays: np.ndarray, mask: int = 0xFF, threads: int = 0) -> np.ndarray:
        rays = np.ascontiguousarray(rays)
        occ = np.zeros(rays.shape[0], np.uint8)
        self.lib.lcxo_trace_any(self.accel, _ptr(rays), rays.shape[0], mask, _ptr(occ), threads)
        return occ

    def fp64_closest(self, rays: np.ndarray, mask: int = 0xFF, threads: int = 0):
        from luisacompute_gb300.scenes import HIT_DTYPE
        rays = np.ascontiguousarray(rays)
        hits = np.zeros(rays.shape[0], HIT_DTYPE)
        t64 = np.zeros(rays.shape[0], np.float64)
        self.lib.lcxo_fp64_closest(self.accel, _ptr(rays), rays.shape[0], mask, _ptr(hits), _ptr(t64), threads)
        return hits, t64

    def fp64_eval(self, rays: np.ndarray, inst: np.ndarray, prim: np.ndarray) -> np.ndarray:
        rays = np.ascontiguousarray(rays)
        inst = np.ascontiguousarray(inst, np.uint32)
        prim = np.ascontiguousarray(prim, np.uint32)
        out = np.zeros(rays.shape[0], F64_DTYPE)
        self.lib.lcxo_fp64_eval(self.accel, _ptr(rays), rays.shape[0], _ptr(inst), _ptr(prim), _ptr(out))
        return out

    def pathtrace(self, scene, albedo, prm, threads: int = 0):
        """CPU restatement of lcx_pt_render: (image HxWx3, first-bounce hits)."""
        from luisacompute_gb300.scenes import HIT_DTYPE
        arrs = [np.ascontiguousarray(albedo[m], np.float32) for m in scene.inst_mesh]
        self._keep += arrs
        ptrs = (c_void_p * len(arrs))(*[a.ctypes.data for a in arrs])
        img = np.zeros(prm.height * prm.width * 3, np.float32)
        hits = np.zeros(prm.width * prm.height * prm.spp, HIT_DTYPE)
        self.lib.lcxo_pathtrace(self.accel, ptrs, ctypes.byref(prm), _ptr(img), _ptr(hits), threads)
        return img.reshape(prm.height, prm.width, 3), hits

    def close(self):
        if self.accel:
            self.lib.lcxo_accel_destroy(self.accel)
            self.accel = None
        for m in self.meshes:
            self.lib.lcxo_mesh_destroy(m)
        self.meshes = []

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class OracleCurve:
    """One curve (lcxo_curve_create): control points (N, 4) float32, segment starts (uint32), basis 0..3."""

    def __init__(self, control_points: np.ndarray, segments: np.ndarray, basis: int, keyframes: int = 1,
                 time_start: float = 0.0, time_end: float = 1.0, vanish_start: bool = False, vanish_end: bool = False):
        self.lib = load()
        self.cps = np.ascontiguousarray(control_points, np.float32).reshape(-1, 4)
        self.segs = np.ascontiguousarray(segments, np.uint32).reshape(-1)
        keys = max(int(keyframes), 1)
        flags = (1 if vanish_start else 0) | (2 if vanish_end else 0)
        self.handle = self.lib.lcxo_curve_create_motion(_ptr(self.cps), 4, self.cps.shape[0] // keys, keys,
                                                        _ptr(self.segs), self.segs.size, int(basis), time_start,
                                                        time_end, flags)
        if not self.handle:
            raise ValueError("a curve segment runs past the control points")

    def pieces(self) -> np.ndarray:
        return np.array([self.lib.lcxo_curve_pieces(self.handle, i) for i in range(self.segs.size)], np.uint32)

    def close(self):
        if getattr(self, "handle", None):
            self.lib.lcxo_curve_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def trace_curves(instances: list, o2w: np.ndarray, masks, rays: np.ndarray, mask: int = 0xFF, any_hit: bool = False,
                 threads: int = 0, times: np.ndarray | None = None):
    """Brute-force closest / any hit over the curve instances (entries of ``instances`` that are None are
    skipped: a mixed scene's mesh instances are traced with OracleScene and merged by the caller)."""
    from luisacompute_gb300.scenes import HIT_DTYPE
    lib = load()
    n_inst = len(instances)
    handles = (c_void_p * n_inst)(*[c.handle if c is not None else None for c in instances])
    o2w = np.ascontiguousarray(o2w, np.float32).reshape(n_inst, 12)
    masks = np.ascontiguousarray(np.broadcast_to(np.asarray(masks, np.uint32), (n_inst,)))
    rays = np.ascontiguousarray(rays)
    hits = np.zeros(rays.shape[0], HIT_DTYPE)
    occ = np.zeros(rays.shape[0], np.uint8)
    tp = None
    if times is not None:
        times = np.ascontiguousarray(times, np.float32)
        tp = _ptr(times)
    lib.lcxo_trace_curves_t(handles, _ptr(o2w), _ptr(masks), n_inst, _ptr(rays), tp, rays.shape[0], mask,
                            int(any_hit), _ptr(hits), _ptr(occ), threads)
    return occ if any_hit else hits


def affine_inverse(o2w: np.ndarray) -> np.ndarray:
    o2w = np.ascontiguousarray(o2w, np.float32).reshape(12)
    out = np.zeros(12, np.float32)
    load().lcxo_affine_inverse(_ptr(o2w), _ptr(out))
    return out


def intersect_triangle(o, d, tmin, tmax, v0, v1, v2):
    """FP32 watertight test of one ray against one triangle: (hit, t, u, v)."""
    arrs = [np.ascontiguousarray(x, np.float32) for x in (o, d, v0, v1, v2)]
    t, u, v = c_float(0), c_float(0), c_float(0)
    hit = load().lcxo_intersect_triangle(_ptr(arrs[0]), _ptr(arrs[1]), tmin, tmax, _ptr(arrs[2]), _ptr(arrs[3]),
                                         _ptr(arrs[4]), ctypes.byref(t), ctypes.byref(u), ctypes.byref(v))
    return bool(hit), t.value, u.value, v.value


def adjudicate(scene_oracle: OracleScene, rays: np.ndarray, got: np.ndarray, want: np.ndarray,
               rel_t: float = 1e-6, edge_eps: float = 1e-5) -> dict:
    """Classify every ray whose (inst, prim) differs between ``got`` and ``want`` with FP64:
    a near-tie in t (relative difference of the two FP64 hit distances <= rel_t) or an
    edge/vertex-grazing hit (FP64 min barycentric of either triangle within edge_eps of 0).
    Returns counts and the indices left unexplained."""
    diff = np.nonzero((got["inst"] != want["inst"]) | (got["prim"] != want["prim"]))[0]
    out = {"rays": int(rays.shape[0]), "disagree": int(diff.size), "near_tie": 0, "grazing": 0,
           "unexplained": []}
    if diff.size == 0:
        return out
    r = rays[diff]
    eg = scene_oracle.fp64_eval(r, got["inst"][diff], got["prim"][diff])
    ew = scene_oracle.fp64_eval(r, want["inst"][diff], want["prim"][diff])
    g_miss = got["inst"][diff] == 0xFFFFFFFF
    w_miss = want["inst"][diff] == 0xFFFFFFFF
    for k in range(diff.size):
        if not g_miss[k] and not w_miss[k]:
            t0, t1 = eg["t"][k], ew["t"][k]
            if abs(t0 - t1) <= rel_t * max(abs(t0), abs(t1), 1e-30):
                out["near_tie"] += 1
                continue
        mb = []
        if not g_miss[k]:
            mb.append(abs(eg["min_bary"][k]))
        if not w_miss[k]:
            mb.append(abs(ew["min_bary"][k]))
        if mb and min(mb) <= edge_eps:
            out["grazing"] += 1
            continue
        out["unexplained"].append(int(diff[k]))
    return out
