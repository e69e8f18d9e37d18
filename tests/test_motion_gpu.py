"""Motion instances (MotionInstance, include/luisa/runtime/rtx/motion_instance.h; the DSL's
intersect_motion / intersect_any_motion with a time per ray, include/luisa/dsl/rtx/accel.h:47-48).

Matrix keyframes are interpolated per element at each ray's time and inverted with the static
instances' FP32 sequence; the oracle restates both (lcxo_trace_motion), so the records must be the
same bit for bit, for times inside, before and after the motion range (clamped, or vanished when
the motion asks for it) and NaN times, with matrix and SRT keyframes."""
import ctypes

import numpy as np
import pytest

from luisacompute_gb300 import scenes as S

pytestmark = pytest.mark.gpu


def _keyframes(rng, k, spread=1.0):
    return S.affine_rows(S.random_rotations(k, rng), rng.uniform(0.2, 0.5, k), rng.uniform(-spread, spread, (k, 3)))


def _setup(rng, allow_update=False):
    import torch
    from luisacompute_gb300.accel import Accel, AccelOption, MotionInstance, mesh_from_data
    datas = [S.icosphere(3), S.displaced_mesh(3_000, rng), S.grid_mesh(20, 20)]
    meshes = [mesh_from_data(d).build() for d in datas]
    n_static, n_motion = 5, 7
    inst_mesh = np.array([i % 3 for i in range(n_static + n_motion)])
    aff = _keyframes(rng, n_static + n_motion)
    motion_specs = [None] * n_static
    motions = []
    for j in range(n_motion):
        k = 2 + j % 3
        keys = _keyframes(rng, k)
        t0, t1 = (0.0, 1.0) if j % 2 == 0 else (0.25, 0.75)
        flags = j % 4  # bit 0: vanish before, bit 1: vanish after
        mo = MotionInstance(meshes[inst_mesh[n_static + j]], keys.reshape(-1, 3, 4), t0, t1,
                            vanish_start=bool(flags & 1), vanish_end=bool(flags & 2))
        motions.append(mo)
        motion_specs.append((keys, t0, t1, flags))
    acc = Accel(AccelOption(allow_update=allow_update))
    for i in range(n_static):
        acc.emplace_back(meshes[inst_mesh[i]], aff[i].reshape(3, 4))
    for j, mo in enumerate(motions):
        acc.emplace_back(mo)
    acc.build()
    torch.cuda.synchronize()
    scene = S.Scene(datas, inst_mesh, aff, np.full(n_static + n_motion, 0xFF, np.uint32))
    return scene, acc, meshes, motions, motion_specs


def _rays_times(rng, n, seed):
    rays = S.sphere_rays(n, [-1.5] * 3, [1.5] * 3, seed=seed)
    times = rng.uniform(-0.3, 1.3, n).astype(np.float32)
    times[:16] = np.nan
    times[16:32] = [0.0, 1.0, 0.25, 0.75] * 4
    return rays, times


def test_motion_instances_match_oracle(lcx, oracle_mod):
    import torch
    from luisacompute_gb300.accel import hits_to_numpy, rays_to_device
    rng = np.random.default_rng(51)
    scene, acc, meshes, motions, specs = _setup(rng)
    osc = oracle_mod.OracleScene(scene)
    rays, times = _rays_times(rng, 60_000, 52)
    want = osc.trace_motion(rays, times, specs)
    want_any = osc.trace_motion(rays, times, specs, any_hit=True)
    assert (want["inst"] >= 5).sum() > 500 and (want["inst"] < 5).sum() > 500  # moving and static hits
    d_rays, d_times = rays_to_device(rays), torch.from_numpy(times).cuda()
    for layout in (0, 1):
        got = hits_to_numpy(acc.trace_closest_motion(d_rays, d_times, layout=layout))
        assert np.array_equal(got.view(np.uint8), want.view(np.uint8)), layout
        occ = acc.trace_any_motion(d_rays, d_times, layout=layout).cpu().numpy()
        assert np.array_equal(occ, want_any), layout
    # calls without times (and the plain trace calls) use time 0
    zero = osc.trace_motion(rays, np.zeros(rays.shape[0], np.float32), specs)
    for got in (acc.trace_closest_motion(d_rays), acc.trace_closest(d_rays)):
        assert np.array_equal(hits_to_numpy(got).view(np.uint8), zero.view(np.uint8))
    # a static-only result differs: the motion moved something
    assert not np.array_equal(want.view(np.uint8), zero.view(np.uint8))
    from luisacompute_gb300 import _capi
    _capi.check(lcx.lcx_check_trace_errors(), "trace errors")


def test_motion_keyframe_rebuild_refit_and_errors(lcx, oracle_mod):
    import torch
    from luisacompute_gb300 import _capi
    from luisacompute_gb300.accel import REQUEST_PREFER_UPDATE, hits_to_numpy, rays_to_device
    rng = np.random.default_rng(53)
    scene, acc, meshes, motions, specs = _setup(rng, allow_update=True)
    rays, times = _rays_times(rng, 30_000, 54)
    d_rays, d_times = rays_to_device(rays), torch.from_numpy(times).cuda()
    # new keyframes: traces of the accel fail until it is built again; a refit takes them
    keys = _keyframes(rng, motions[2].keys.shape[0])
    motions[2].set_keyframes(keys.reshape(-1, 3, 4))
    motions[2].build()
    specs[5 + 2] = (keys, specs[5 + 2][1], specs[5 + 2][2], specs[5 + 2][3])
    with pytest.raises(_capi.LcxError):
        acc.trace_closest_motion(d_rays, d_times)
    acc.build(request=REQUEST_PREFER_UPDATE)
    assert acc.stats().refits == 1
    want = oracle_mod.OracleScene(scene).trace_motion(rays, times, specs)
    got = hits_to_numpy(acc.trace_closest_motion(d_rays, d_times))
    assert np.array_equal(got.view(np.uint8), want.view(np.uint8))
    # device views and multi-job launches take motion accels (lcx::ray_query_motion: test_ray_query_gpu.py)
    v = _capi.LcxAccelView()
    assert lcx.lcx_accel_device_view(acc.handle, ctypes.byref(v)) == _capi.LCX_OK and v.motion == 1
    out = torch.empty((16, 6), dtype=torch.int32, device="cuda")
    job = (_capi.LcxTraceJob * 1)(_capi.LcxTraceJob(acc.handle, d_rays.data_ptr(), out.data_ptr(), 16, 0xFF, 0, 0))
    assert lcx.lcx_trace_jobs(job, 1, 1, None) == _capi.LCX_OK  # time 0 (lcx_trace_jobs_motion takes times)
    h = ctypes.c_uint64(0)
    for opt in (_capi.LcxMotionOption(1, 0.0, 1.0, 0, 0, 0, 0), _capi.LcxMotionOption(2, 1.0, 1.0, 0, 0, 0, 0),
                _capi.LcxMotionOption(2, 0.0, 1.0, 0, 0, 2, 0)):
        assert lcx.lcx_motion_instance_create(meshes[0].handle, ctypes.byref(opt), ctypes.byref(h)) == \
            _capi.LCX_ERR_INVALID_ARG
    assert lcx.lcx_motion_instance_set_keyframes(motions[0].handle, keys.ctypes.data, 99) == _capi.LCX_ERR_INVALID_ARG
    # a destroyed motion instance: the accel's traces fail (its memory stays with the accel)
    motions[1].destroy()
    with pytest.raises(_capi.LcxError):
        acc.trace_closest_motion(d_rays, d_times)
    with pytest.raises(_capi.LcxError):
        acc.build()


def _srt_keyframes(rng, k):
    """k SRT records: pivot, unit-ish quaternion (not normalised: the product normalises), scale,
    shear, translation."""
    v = np.zeros((k, 16), np.float32)
    v[:, 0:3] = rng.uniform(-0.2, 0.2, (k, 3))
    q = rng.normal(0.0, 1.0, (k, 4))
    v[:, 3:7] = q * rng.uniform(0.5, 2.0, (k, 1))
    v[:, 7:10] = rng.uniform(0.15, 0.45, (k, 3))
    v[:, 10:13] = rng.uniform(-0.1, 0.1, (k, 3))
    v[:, 13:16] = rng.uniform(-1.0, 1.0, (k, 3))
    return v


def test_srt_motion_matches_oracle(lcx, oracle_mod):
    import torch
    from luisacompute_gb300.accel import Accel, MotionInstance, hits_to_numpy, mesh_from_data, rays_to_device
    rng = np.random.default_rng(55)
    datas = [S.icosphere(3), S.displaced_mesh(2_000, rng)]
    meshes = [mesh_from_data(d).build() for d in datas]
    n = 10
    inst_mesh = np.arange(n) % 2
    specs, motions = [], []
    acc = Accel()
    for j in range(n):
        keys = _srt_keyframes(rng, 2 + j % 3)
        t0, t1 = (0.0, 1.0) if j % 2 == 0 else (0.2, 0.9)
        flags = (j % 4) | 4
        mo = MotionInstance(meshes[inst_mesh[j]], keys, t0, t1, vanish_start=bool(flags & 1),
                            vanish_end=bool(flags & 2), srt=True)
        motions.append(mo)
        specs.append((keys, t0, t1, flags))
        acc.emplace_back(mo)
    acc.build()
    scene = S.Scene(datas, inst_mesh, np.tile(S.IDENTITY, (n, 1)), np.full(n, 0xFF, np.uint32))
    osc = oracle_mod.OracleScene(scene)
    rays, times = _rays_times(rng, 50_000, 56)
    want = osc.trace_motion(rays, times, specs)
    want_any = osc.trace_motion(rays, times, specs, any_hit=True)
    assert (want["inst"] != S.MISS).sum() > 1000
    d_rays, d_times = rays_to_device(rays), torch.from_numpy(times).cuda()
    for layout in (0, 1):
        got = hits_to_numpy(acc.trace_closest_motion(d_rays, d_times, layout=layout))
        assert np.array_equal(got.view(np.uint8), want.view(np.uint8)), layout
        assert np.array_equal(acc.trace_any_motion(d_rays, d_times, layout=layout).cpu().numpy(), want_any)
    from luisacompute_gb300 import _capi
    _capi.check(lcx.lcx_check_trace_errors(), "trace errors")


def test_keyframed_vertices_match_oracle(lcx, oracle_mod):
    """A mesh with keyframed vertices (the vertex buffer holds 3 copies of the vertices), instanced
    with static transforms and through a motion instance (both motions at once), next to a static
    mesh: the oracle's records bit for bit, closest and any, both layouts; the plain calls use time 0."""
    import torch
    from luisacompute_gb300.accel import Accel, Mesh, MotionInstance, hits_to_numpy, mesh_from_data, rays_to_device
    rng = np.random.default_rng(57)
    base = S.icosphere(3)
    keys = 3
    frames = []
    for k in range(keys):
        v = base.vertices.copy()
        v[:, :3] = v[:, :3] * np.float32(0.6 + 0.2 * k) + rng.normal(0.0, 0.02, (v.shape[0], 3)).astype(np.float32)
        v[:, :3] += np.float32(0.3 * k)
        frames.append(v)
    stacked = np.ascontiguousarray(np.concatenate(frames), np.float32)
    t0, t1, flags = 0.1, 0.9, 2  # vanishes after t1
    mesh = Mesh(torch.from_numpy(stacked).cuda(), torch.from_numpy(base.triangles.astype(np.int32)).cuda(),
                motion_keyframes=keys, time_start=t0, time_end=t1, vanish_end=True).build()
    other = S.displaced_mesh(2_000, rng)
    static = mesh_from_data(other).build()
    aff = _keyframes(rng, 4, spread=0.8)
    acc = Accel()
    acc.emplace_back(mesh, aff[0].reshape(3, 4))
    acc.emplace_back(mesh, aff[1].reshape(3, 4))
    acc.emplace_back(static, aff[2].reshape(3, 4))
    ikeys = _keyframes(rng, 2, spread=0.5)
    mo = MotionInstance(mesh, ikeys.reshape(-1, 3, 4), 0.0, 1.0)
    acc.emplace_back(mo)
    acc.build()
    first = S.MeshData(frames[0], base.triangles)
    scene = S.Scene([first, other], np.array([0, 0, 1, 0]), np.concatenate([aff[:3], S.IDENTITY[None]]),
                    np.full(4, 0xFF, np.uint32))
    osc = oracle_mod.OracleScene(scene)
    vm = (stacked, keys, base.triangles, t0, t1, flags)
    mesh_motion = [vm, vm, None, vm]
    specs = [None, None, None, (ikeys, 0.0, 1.0, 0)]
    rays, times = _rays_times(rng, 40_000, 58)
    want = osc.trace_motion(rays, times, specs, mesh_motion=mesh_motion)
    want_any = osc.trace_motion(rays, times, specs, any_hit=True, mesh_motion=mesh_motion)
    assert np.isin([0, 1, 2, 3], want["inst"]).all()
    d_rays, d_times = rays_to_device(rays), torch.from_numpy(times).cuda()
    for layout in (0, 1):
        got = hits_to_numpy(acc.trace_closest_motion(d_rays, d_times, layout=layout))
        assert np.array_equal(got.view(np.uint8), want.view(np.uint8)), layout
        assert np.array_equal(acc.trace_any_motion(d_rays, d_times, layout=layout).cpu().numpy(), want_any)
    zero = osc.trace_motion(rays, np.zeros(rays.shape[0], np.float32), specs, mesh_motion=mesh_motion)
    assert np.array_equal(hits_to_numpy(acc.trace_closest(d_rays)).view(np.uint8), zero.view(np.uint8))
    from luisacompute_gb300 import _capi
    _capi.check(lcx.lcx_check_trace_errors(), "trace errors")
    # a vertex buffer that is not whole keyframes, and refit, are refused
    bad = Mesh(torch.from_numpy(stacked[:-1]).cuda(), torch.from_numpy(base.triangles.astype(np.int32)).cuda(),
               motion_keyframes=keys)
    with pytest.raises(_capi.LcxError):
        bad.build()
    from luisacompute_gb300.accel import AccelOption
    with pytest.raises(_capi.LcxError):
        Mesh(torch.from_numpy(stacked).cuda(), torch.from_numpy(base.triangles.astype(np.int32)).cuda(),
             AccelOption(allow_update=True), motion_keyframes=keys)


def test_motion_in_multi_job_launches(lcx, oracle_mod):
    """lcx_trace_jobs_motion: jobs on a motion accel (each with its own ray times) and on a static
    accel share one launch per kind; every job equals its own lcx_trace_closest_motion /
    lcx_trace_any_motion call bit for bit, and plain lcx_trace_jobs traces the motion accel at
    time 0."""
    import torch
    from luisacompute_gb300 import _capi
    from luisacompute_gb300.accel import Accel, hits_to_numpy, mesh_from_data, rays_to_device
    rng = np.random.default_rng(57)
    scene, acc, meshes, motions, specs = _setup(rng)
    static = Accel()
    static.emplace_back(mesh_from_data(S.icosphere(3)).build())
    static.build()
    lib = _capi.load()
    n = 30_000
    rays = [rays_to_device(_rays_times(rng, n, 60 + k)[0]) for k in range(3)]
    times = [torch.from_numpy(_rays_times(rng, n, 70 + k)[1]).cuda() for k in range(3)]
    outs = [torch.empty((n, 6), dtype=torch.int32, device="cuda") for _ in range(2)]
    occ = torch.empty(n, dtype=torch.uint8, device="cuda")
    jobs = (_capi.LcxTraceJob * 3)(
        _capi.LcxTraceJob(acc.handle, rays[0].data_ptr(), outs[0].data_ptr(), n, 0xFF, 0, 0),
        _capi.LcxTraceJob(static.handle, rays[1].data_ptr(), outs[1].data_ptr(), n, 0xFF, 0, 0),
        _capi.LcxTraceJob(acc.handle, rays[2].data_ptr(), occ.data_ptr(), n, 0xFF, 1, 0))
    tptr = (ctypes.c_void_p * 3)(times[0].data_ptr(), None, times[2].data_ptr())
    for layout in (0, 1):
        _capi.check(lib.lcx_trace_jobs_motion(jobs, tptr, 3, layout, None), "lcx_trace_jobs_motion")
        torch.cuda.synchronize()
        want0 = hits_to_numpy(acc.trace_closest_motion(rays[0], times[0], layout=layout))
        assert np.array_equal(hits_to_numpy(outs[0]).view(np.uint8), want0.view(np.uint8))
        want1 = hits_to_numpy(static.trace_closest(rays[1], layout=layout))
        assert np.array_equal(hits_to_numpy(outs[1]).view(np.uint8), want1.view(np.uint8))
        assert torch.equal(occ, acc.trace_any_motion(rays[2], times[2], layout=layout))
    _capi.check(lib.lcx_trace_jobs(jobs, 3, 1, None), "lcx_trace_jobs")
    torch.cuda.synchronize()
    want0 = hits_to_numpy(acc.trace_closest_motion(rays[0], layout=1))  # time 0
    assert np.array_equal(hits_to_numpy(outs[0]).view(np.uint8), want0.view(np.uint8))
