"""The CPU backend's per-ray accel table (defs::Accel, the reference's
src/rust/luisa_compute_cpu_kernel_defs/src/lib.rs:111-125) over the GPU path: lcx_accel_cpu_table.

Called through the function pointers as generated CPU-backend code would call them: trace_closest
and trace_any equal the batched calls' records bit for bit; ray_query with host callbacks gives
lcx_trace_closest's record when every candidate is committed, the oracle's record on the cut scene
for an alpha cutout, and a hit exactly when trace_any does for a terminate-on-first query; the
instance getters return what the setters wrote (column-major Mat4)."""
import ctypes

import numpy as np
import pytest

from luisacompute_gb300 import _capi
from luisacompute_gb300 import scenes as S

CUT = 3


def test_table_layout_and_bad_handle(lcx):
    """CPU only: the structs have the reference's sizes and offsets; an unknown handle is refused."""
    assert ctypes.sizeof(_capi.LcxCpuRayQuery) == 128 and ctypes.sizeof(_capi.LcxCpuAccel) == 80
    assert _capi.LcxCpuRayQuery.ray.offset == 32 and _capi.LcxCpuRayQuery.cur_triangle_hit.offset == 72
    assert _capi.LcxCpuRayQuery.cur_commited.offset == 104 and _capi.LcxCpuRayQuery.accel.offset == 120
    t = _capi.LcxCpuAccel()
    assert lcx.lcx_accel_cpu_table(987654321, ctypes.byref(t)) == _capi.LCX_ERR_INVALID_ARG


def _aligned(cls, keep):
    """A zeroed instance of ctypes struct `cls` at a 16-byte aligned address (kept alive in `keep`)."""
    buf = np.zeros(ctypes.sizeof(cls) + 16, np.uint8)
    keep.append(buf)
    addr = (buf.ctypes.data + 15) & ~15
    return cls.from_address(addr)


def _ray(rec, keep):
    r = _aligned(_capi.LcxRay, keep)
    r.origin[:] = rec["o"].tolist()
    r.t_min = float(rec["tmin"])
    r.direction[:] = rec["d"].tolist()
    r.t_max = float(rec["tmax"])
    return r


@pytest.mark.gpu
def test_per_ray_table(lcx, oracle_mod):
    import torch
    from luisacompute_gb300.accel import accel_from_scene, hits_to_numpy, rays_to_device
    scene = S.terrain_scene(n=64, sphere_count=8, sphere_subdiv=3)
    acc, meshes = accel_from_scene(scene)
    rays = np.concatenate([S.terrain_rays(scene, 300, seed=81), S.terrain_shadow_rays(scene, 200, seed=82)])
    d = rays_to_device(rays)
    want = hits_to_numpy(acc.trace_closest(d))
    want_any = acc.trace_any(d).cpu().numpy()
    torch.cuda.synchronize()
    tab = _capi.LcxCpuAccel()
    _capi.check(lcx.lcx_accel_cpu_table(acc.handle, ctypes.byref(tab)), "lcx_accel_cpu_table")
    keep = []
    got = np.zeros(rays.shape[0], S.HIT_DTYPE)
    occ = np.zeros(rays.shape[0], np.uint8)
    for i in range(rays.shape[0]):
        r = _ray(rays[i], keep)
        h = tab.trace_closest(tab.handle, ctypes.byref(r), 0xFF)
        got[i] = (h.inst, h.prim, (h.bary[0], h.bary[1]), h.committed_ray_t, h._pad)
        occ[i] = 1 if tab.trace_any(tab.handle, ctypes.byref(r), 0xFF) else 0
    assert np.array_equal(got.view(np.uint8), want.view(np.uint8))
    assert np.array_equal(occ, want_any)
    assert (want["inst"] != S.MISS).sum() > 50

    # ray_query: commit every candidate = trace_closest; cutout = the oracle on the cut scene
    state = {"cut": False}

    def on_tri(rq):
        c = rq.contents.cur_triangle_hit
        rq.contents.cur_commited = not (state["cut"] and c.prim % CUT == 0)

    def on_proc(rq):
        rq.contents.cur_commited = False

    cb_t, cb_p = _capi.LcxCpuHitCallback(on_tri), _capi.LcxCpuHitCallback(on_proc)
    meshes_cut, keeps = [], []
    for m in scene.meshes:
        k = np.nonzero(np.arange(m.tri_count) % CUT != 0)[0].astype(np.uint32)
        keeps.append(k)
        meshes_cut.append(S.MeshData(m.vertices, m.triangles[k]))
    cut = oracle_mod.OracleScene(S.Scene(meshes_cut, scene.inst_mesh, scene.inst_affine, scene.inst_mask))
    want_cut = cut.trace_closest(rays)
    for i in range(want_cut.shape[0]):
        if want_cut["inst"][i] != S.MISS:
            want_cut["prim"][i] = keeps[scene.inst_mesh[want_cut["inst"][i]]][want_cut["prim"][i]]
    for cutting, ref in ((False, want), (True, want_cut)):
        state["cut"] = cutting
        for i in range(rays.shape[0]):
            rq = _aligned(_capi.LcxCpuRayQuery, keep)
            rq.hit.inst = rq.hit.prim = 0xFFFFFFFF
            rq.hit.committed_ray_t = float(rays["tmax"][i])
            r = _ray(rays[i], keep)
            ctypes.memmove(ctypes.addressof(rq) + 32, ctypes.addressof(r), 32)
            rq.mask = 0xFF
            tab.ray_query(tab.handle, ctypes.byref(rq), cb_t, cb_p)
            w = ref[i]
            assert (rq.hit.inst, rq.hit.prim) == (int(w["inst"]), int(w["prim"])), (cutting, i)
            if w["inst"] != S.MISS:
                assert rq.hit.hit_type == 1
                assert np.float32(rq.hit.committed_ray_t) == w["t"]
                assert (np.float32(rq.hit.bary[0]), np.float32(rq.hit.bary[1])) == (w["bary"][0], w["bary"][1])
    # terminate on first: a hit exactly when trace_any reports one
    state["cut"] = False
    for i in range(rays.shape[0]):
        rq = _aligned(_capi.LcxCpuRayQuery, keep)
        rq.hit.inst = rq.hit.prim = 0xFFFFFFFF
        r = _ray(rays[i], keep)
        ctypes.memmove(ctypes.addressof(rq) + 32, ctypes.addressof(r), 32)
        rq.mask = 0xFF
        rq.terminate_on_first = True
        tab.ray_query(tab.handle, ctypes.byref(rq), cb_t, cb_p)
        assert (rq.hit.inst != 0xFFFFFFFF) == bool(want_any[i]), i

    # instances: setters then getters (edits apply at the next build)
    m = _aligned(_capi.LcxMat4, keep)
    cols = np.arange(16, dtype=np.float32).reshape(4, 4)
    cols[:, 3] = [0, 0, 0, 1]  # the last row of the column-major matrix
    m.m[:] = cols.reshape(-1).tolist()
    tab.set_instance_transform(tab.handle, 2, ctypes.byref(m))
    back = tab.instance_transform(tab.handle, 2)
    assert list(back.m) == m.m[:]
    tab.set_instance_visibility(tab.handle, 3, 0x0F)
    assert tab.instance_visibility_mask(tab.handle, 3) == 0x0F
    tab.set_instance_user_id(tab.handle, 4, 1234)
    assert tab.instance_user_id(tab.handle, 4) == 1234
    assert tab.instance_user_id(tab.handle, 10_000) == 0 and b"out of range" in lcx.lcx_last_error_string()
