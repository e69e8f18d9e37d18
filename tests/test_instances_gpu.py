"""Device-side instance edits (include/lcx/accel_instances.cuh; the reference's
Accel::set_instance_transform / visibility / opacity / user_id and getters in kernels,
src/backends/cuda/cuda_builtin/cuda_device_resource.h:1450-1512).

tests/cuda/instance_kernels.cu is compiled here as a user would compile it. A kernel moves every
instance and hides some; the next lcx_accel_build (a TLAS refit with PREFER_UPDATE, or a rebuild)
must give the oracle's records on the edited scene bit for bit."""
import ctypes
import subprocess
from pathlib import Path

import numpy as np
import pytest

from luisacompute_gb300 import scenes as S

pytestmark = pytest.mark.gpu
ROOT = Path(__file__).resolve().parent.parent


@pytest.fixture(scope="module")
def ik(tmp_path_factory):
    from luisacompute_gb300 import build as B
    out = tmp_path_factory.mktemp("ik") / "libik.so"
    subprocess.run([B.nvcc_path(), B.ARCH, "-O3", "-std=c++17", "-shared", "-Xcompiler", "-fPIC", "-cudart", "shared",
                    f"-I{ROOT / 'include'}", "-o", str(out), str(ROOT / "tests/cuda/instance_kernels.cu")],
                   check=True, capture_output=True)
    lib = ctypes.CDLL(str(out))
    lib.inst_edit.restype = ctypes.c_int
    lib.inst_edit.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint32, ctypes.c_void_p]
    lib.inst_read.restype = ctypes.c_int
    lib.inst_read.argtypes = [ctypes.c_void_p, ctypes.c_uint32] + [ctypes.c_void_p] * 4
    lib.inst_motion_key.restype = ctypes.c_int
    lib.inst_motion_key.argtypes = [ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint32] + [ctypes.c_void_p] * 3
    return lib


def _buffer(acc):
    from luisacompute_gb300 import _capi
    b = _capi.LcxInstanceBuffer()
    _capi.check(_capi.load().lcx_accel_instance_buffer(acc.handle, ctypes.byref(b)), "lcx_accel_instance_buffer")
    return b


def _read(ik, buf, n):
    import torch
    aff = torch.zeros((n, 12), dtype=torch.float32, device="cuda")
    masks, uids, opq = (torch.zeros(n, dtype=torch.int32, device="cuda") for _ in range(3))
    assert ik.inst_read(ctypes.byref(buf), n, aff.data_ptr(), masks.data_ptr(), uids.data_ptr(), opq.data_ptr()) == 0
    torch.cuda.synchronize()
    return aff.cpu().numpy(), masks.cpu().numpy().astype(np.uint32), uids.cpu().numpy(), opq.cpu().numpy()


def test_device_instance_edits(lcx, oracle_mod, ik):
    import torch
    from luisacompute_gb300 import _capi
    from luisacompute_gb300.accel import (REQUEST_PREFER_UPDATE, AccelOption, accel_from_scene, hits_to_numpy,
                                          rays_to_device)
    scene = S.terrain_scene(n=128, sphere_count=48, sphere_subdiv=3)
    acc, _ = accel_from_scene(scene, option=AccelOption(allow_update=True))
    n = scene.instance_count
    buf = _buffer(acc)
    assert buf.count == n
    aff0, masks0, uids0, opq0 = _read(ik, buf, n + 3)
    assert np.array_equal(aff0[:n], scene.inst_affine) and np.all(masks0[:n] == scene.inst_mask & 0xFF)
    assert np.all(uids0[:n] == 0) and np.all(opq0[:n] == 1)
    ident = np.array([1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0], np.float32)
    assert np.all(aff0[n:] == ident) and np.all(masks0[n:] == 0xFF) and np.all(opq0[n:] == 1)  # out of range
    # the kernel edits: spheres move and hide at random, the terrain (instance 0) stays
    rng = np.random.default_rng(21)
    aff = scene.inst_affine.copy()
    aff[1:, [3, 7, 11]] += rng.normal(0.0, 0.05, (n - 1, 3)).astype(np.float32)
    masks = np.full(n, 0xFF, np.uint32)
    masks[1 + rng.choice(n - 1, 10, replace=False)] = 0x02
    d_aff = torch.from_numpy(aff).cuda()
    d_masks = torch.from_numpy(masks.astype(np.int32)).cuda()
    assert ik.inst_edit(ctypes.byref(buf), d_aff.data_ptr(), d_masks.data_ptr(), n,
                        torch.cuda.current_stream().cuda_stream) == 0
    got_aff, got_masks, got_uids, got_opq = _read(ik, buf, n)
    assert np.array_equal(got_aff, aff) and np.array_equal(got_masks, masks)
    assert np.array_equal(got_uids, 1000 + np.arange(n)) and np.array_equal(got_opq, np.arange(n) % 2)
    rays = S.terrain_rays(scene, 120_000, seed=22)
    edited = S.Scene(scene.meshes, scene.inst_mesh, aff, masks)
    osc = oracle_mod.OracleScene(edited)
    # refit, then a rebuild: both see the kernel's edits; ray mask 0x01 skips the hidden spheres
    acc.build(request=REQUEST_PREFER_UPDATE)
    assert acc.stats().refits == 1
    for build in ("refit", "rebuild"):
        if build == "rebuild":
            acc.build()
            assert acc.stats().refits == 0
        for mask in (0xFF, 0x01):
            got = hits_to_numpy(acc.trace_closest(rays_to_device(rays), mask=mask))
            want = osc.trace_closest(rays, mask=mask)
            assert np.array_equal(got.view(np.uint8), want.view(np.uint8)), (build, mask)
    _capi.check(lcx.lcx_check_trace_errors(), "trace errors")
    bad = _capi.LcxInstanceBuffer()
    from luisacompute_gb300.accel import Accel
    empty = Accel()
    assert lcx.lcx_accel_instance_buffer(empty.handle, ctypes.byref(bad)) == _capi.LCX_ERR_NOT_BUILT
    assert lcx.lcx_accel_instance_buffer(acc.handle, None) == _capi.LCX_ERR_INVALID_ARG


def test_instance_edits_in_cuda_graph(lcx, oracle_mod, ik):
    """A frame of rigid animation captured once: the user kernel writes the instances from a device
    array, the TLAS is refit and rays are traced; each replay, after the array changes, matches the
    oracle on that frame's transforms."""
    import torch
    from luisacompute_gb300 import _capi
    from luisacompute_gb300.accel import (REQUEST_PREFER_UPDATE, AccelOption, accel_from_scene, hits_to_numpy,
                                          rays_to_device)
    scene = S.terrain_scene(n=96, sphere_count=32, sphere_subdiv=3)
    acc, _ = accel_from_scene(scene, option=AccelOption(allow_update=True))
    n = scene.instance_count
    buf = _buffer(acc)
    rays = S.terrain_rays(scene, 60_000, seed=23)
    d_rays = rays_to_device(rays)
    out = torch.empty((rays.shape[0], 6), dtype=torch.int32, device="cuda")
    d_aff = torch.from_numpy(scene.inst_affine.copy()).cuda()
    d_masks = torch.full((n,), 0xFF, dtype=torch.int32, device="cuda")
    acc.build(request=REQUEST_PREFER_UPDATE)
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):  # the kernel goes on the capturing stream
        assert ik.inst_edit(ctypes.byref(buf), d_aff.data_ptr(), d_masks.data_ptr(), n,
                            torch.cuda.current_stream().cuda_stream) == 0
        acc.build(request=REQUEST_PREFER_UPDATE)
        acc.trace_closest(d_rays, out=out)
    rng = np.random.default_rng(24)
    for frame in range(3):
        aff = scene.inst_affine.copy()
        aff[1:, [3, 7, 11]] += rng.normal(0.0, 0.08, (n - 1, 3)).astype(np.float32)
        d_aff.copy_(torch.from_numpy(aff))
        g.replay()
        torch.cuda.synchronize()
        want = oracle_mod.OracleScene(S.Scene(scene.meshes, scene.inst_mesh, aff, scene.inst_mask)).trace_closest(rays)
        assert np.array_equal(hits_to_numpy(out).view(np.uint8), want.view(np.uint8)), frame
    _capi.check(lcx.lcx_check_trace_errors(), "trace errors")


def test_device_motion_keyframe_edits(lcx, oracle_mod, ik):
    """instance_motion_matrix / set_instance_motion_matrix (include/luisa/dsl/rtx/accel.h:69-110) from
    a user kernel: keyframe 1 of every matrix motion instance is read and replaced; static instances
    and the SRT one report no matrix keyframe and keep theirs.  After a TLAS refit the traces match
    the oracle with the new keyframes, bit for bit."""
    import torch
    from luisacompute_gb300.accel import (REQUEST_PREFER_UPDATE, Accel, AccelOption, MotionInstance, hits_to_numpy,
                                          mesh_from_data, rays_to_device)
    rng = np.random.default_rng(61)
    data = S.icosphere(3, radius=0.5)
    mesh = mesh_from_data(data).build()
    n_static, n_motion = 2, 3
    static_aff = S.affine_rows(S.random_rotations(n_static, rng), np.ones(n_static), rng.uniform(-1, 1, (n_static, 3)))
    keys = [S.affine_rows(S.random_rotations(2, rng), np.ones(2), rng.uniform(-1, 1, (2, 3))) for _ in range(n_motion)]
    motions = [MotionInstance(mesh, k.reshape(-1, 3, 4), 0.0, 1.0) for k in keys]
    srt = np.zeros((2, 16), np.float32)
    srt[:, 6] = 1.0      # identity quaternion (x, y, z, w at 3..6)
    srt[:, 7:10] = 1.0   # unit scale
    srt[1, 13:16] = [0.5, 0.0, 0.0]
    srt_mo = MotionInstance(mesh, srt, 0.0, 1.0, srt=True)
    acc = Accel(AccelOption(allow_update=True))
    for i in range(n_static):
        acc.emplace_back(mesh, static_aff[i].reshape(3, 4))
    for mo in motions:
        acc.emplace_back(mo)
    acc.emplace_back(srt_mo)
    acc.build()
    n = n_static + n_motion + 1
    new = S.affine_rows(S.random_rotations(n, rng), np.ones(n), rng.uniform(-1, 1, (n, 3)))
    d_new = torch.from_numpy(new).cuda()
    old = torch.full((n, 12), -7.0, dtype=torch.float32, device="cuda")
    found = torch.zeros(n, dtype=torch.int32, device="cuda")
    buf = _buffer(acc)
    assert ik.inst_motion_key(ctypes.byref(buf), n, 1, d_new.data_ptr(), old.data_ptr(), found.data_ptr()) == 0
    torch.cuda.synchronize()
    assert list(found.cpu().numpy()) == [0, 0, 1, 1, 1, 0]
    old_np = old.cpu().numpy()
    for j in range(n_motion):
        assert np.array_equal(old_np[n_static + j], keys[j][1])
    assert np.all(old_np[[0, 1, n - 1]] == -7.0)
    # a key past the count changes nothing
    assert ik.inst_motion_key(ctypes.byref(buf), n, 2, d_new.data_ptr(), old.data_ptr(), found.data_ptr()) == 0
    torch.cuda.synchronize()
    assert not found.cpu().numpy().any()
    acc.build(request=REQUEST_PREFER_UPDATE)
    specs = [None] * n_static + [(np.stack([keys[j][0], new[n_static + j]]), 0.0, 1.0, 0) for j in range(n_motion)]
    specs.append((srt, 0.0, 1.0, 4))
    scene = S.Scene([data], np.zeros(n, np.int64),
                    np.concatenate([static_aff, np.tile(np.eye(3, 4, dtype=np.float32).reshape(1, 12), (n - n_static, 1))]),
                    np.full(n, 0xFF, np.uint32))
    rays = S.sphere_rays(50_000, [-1.6] * 3, [1.6] * 3, seed=62)
    times = rng.uniform(0.0, 1.0, rays.shape[0]).astype(np.float32)
    want = oracle_mod.OracleScene(scene).trace_motion(rays, times, specs)
    got = hits_to_numpy(acc.trace_closest_motion(rays_to_device(rays), torch.from_numpy(times).cuda()))
    assert np.array_equal(got.view(np.uint8), want.view(np.uint8))
    assert np.isin(np.arange(n_static, n_static + n_motion), got["inst"]).all()
