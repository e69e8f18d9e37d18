"""Per-ray trace_closest / trace_any called from inside a user kernel (include/lcx/trace.cuh): the
form of the reference's lc_accel_trace_closest / lc_accel_trace_any
(src/backends/cuda/cuda_builtin/cuda_device_resource.h:1784-1829), which LuisaCompute kernels
such as src/tests/test_path_tracing.cpp:165-250 call once per thread.

tests/cuda/trace_kernels.cu is compiled here as a user would compile it (local short stack, and
16 shared-memory entries per thread).  Its records must equal the oracle's bit for bit on the
icosphere primary rays and on the full terrain scene, for closest and any hit; with motion
instances and curves they must equal the batched calls' (which the motion and curve tests check
against the oracle).  Loop mode 3 runs the same device functions as a launch form of the plain
entry points (one ray per thread), checked through the C ABI, with and without ray reordering."""
import ctypes
import subprocess
from pathlib import Path

import numpy as np
import pytest

from luisacompute_gb300 import scenes as S

pytestmark = pytest.mark.gpu
ROOT = Path(__file__).resolve().parent.parent


@pytest.fixture(scope="module")
def tk(tmp_path_factory):
    from luisacompute_gb300 import build as B
    out = tmp_path_factory.mktemp("tk") / "libtk.so"
    subprocess.run([B.nvcc_path(), B.ARCH, "-O3", "-std=c++17", "-shared", "-Xcompiler", "-fPIC", "-cudart", "shared",
                    f"-I{ROOT / 'include'}", "-o", str(out), str(ROOT / "tests/cuda/trace_kernels.cu")],
                   check=True, capture_output=True)
    lib = ctypes.CDLL(str(out))
    for name in ("tk_closest", "tk_any"):
        fn = getattr(lib, name)
        fn.restype = ctypes.c_int
        fn.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint32,
                       ctypes.c_uint32, ctypes.c_void_p]
    return lib


def _view(acc):
    from luisacompute_gb300 import _capi
    v = _capi.LcxAccelView()
    _capi.check(_capi.load().lcx_accel_device_view(acc.handle, ctypes.byref(v)), "lcx_accel_device_view")
    return v


def _device_closest(tk, acc, d_rays, variant, mask=0xFF, d_times=None):
    import torch
    from luisacompute_gb300.accel import hits_to_numpy
    n = d_rays.shape[0]
    hits = torch.full((n, 6), -7, dtype=torch.int32, device="cuda")
    view = _view(acc)
    tp = d_times.data_ptr() if d_times is not None else None
    assert tk.tk_closest(ctypes.byref(view), d_rays.data_ptr(), tp, n, mask, variant, hits.data_ptr()) == 0
    return hits_to_numpy(hits)


def _device_any(tk, acc, d_rays, variant, mask=0xFF, d_times=None):
    import torch
    n = d_rays.shape[0]
    occ = torch.full((n,), 7, dtype=torch.uint8, device="cuda")
    view = _view(acc)
    tp = d_times.data_ptr() if d_times is not None else None
    assert tk.tk_any(ctypes.byref(view), d_rays.data_ptr(), tp, n, mask, variant, occ.data_ptr()) == 0
    return occ.cpu().numpy()


def _same(a, b):
    return np.array_equal(a.view(np.uint8), b.view(np.uint8))


@pytest.fixture(scope="module")
def full_terrain(oracle_mod):
    scene = S.terrain_scene()
    return scene, oracle_mod.OracleScene(scene)


def test_icosphere_primary_rays(lcx, oracle_mod, tk):
    """Config 1: the 81,920-triangle icosphere, 1024x1024 jittered pinhole rays."""
    from luisacompute_gb300.accel import accel_from_scene, rays_to_device
    scene = S.icosphere_scene(6)
    rays = S.primary_rays_icosphere(1024, 1024)
    osc = oracle_mod.OracleScene(scene)
    want = osc.trace_closest(rays)
    acc, _m = accel_from_scene(scene)
    d = rays_to_device(rays)
    for variant in (0, 1):
        assert _same(_device_closest(tk, acc, d, variant), want), variant
        assert np.array_equal(_device_any(tk, acc, d, variant), (want["inst"] != S.MISS).astype(np.uint8))


def test_full_terrain(lcx, oracle_mod, tk, full_terrain):
    """Config 2 at full size: 2^20 incoherent rays (closest) and 2^20 shadow rays (any), and
    instance masks, against the oracle."""
    from luisacompute_gb300.accel import accel_from_scene, rays_to_device
    scene, osc = full_terrain
    acc, _m = accel_from_scene(scene)
    rays = S.terrain_rays(scene, 1 << 20, seed=4)
    d = rays_to_device(rays)
    want = osc.trace_closest(rays)
    for variant in (0, 1):
        assert _same(_device_closest(tk, acc, d, variant), want), variant
    shadow = S.terrain_shadow_rays(scene, 1 << 20, seed=5)
    want_any = osc.trace_any(shadow)
    ds = rays_to_device(shadow)
    for variant in (0, 1):
        assert np.array_equal(_device_any(tk, acc, ds, variant), want_any), variant


def test_masks(lcx, oracle_mod, tk):
    from luisacompute_gb300.accel import accel_from_scene, rays_to_device
    scene = S.terrain_scene(n=128, sphere_count=64, sphere_subdiv=3)
    scene.inst_mask = np.array([0x01] + [0x02, 0x04] * 32, np.uint32)
    rays = S.terrain_rays(scene, 50_000, seed=7)
    osc = oracle_mod.OracleScene(scene)
    acc, _m = accel_from_scene(scene)
    d = rays_to_device(rays)
    for mask in (0xFF, 0x01, 0x06, 0x00):
        want = osc.trace_closest(rays, mask)
        assert _same(_device_closest(tk, acc, d, 1, mask=mask), want), mask
        assert np.array_equal(_device_any(tk, acc, d, 0, mask=mask), (want["inst"] != S.MISS).astype(np.uint8))


def test_motion_and_curves_equal_batched_calls(lcx, tk):
    """Moving instances (per-ray times, and time 0 for the plain forms) and round curves: the
    device functions equal lcx_trace_closest(_motion) / lcx_trace_any(_motion) bit for bit."""
    import torch
    from luisacompute_gb300.accel import Accel, Curve, MotionInstance, hits_to_numpy, mesh_from_data, rays_to_device
    rng = np.random.default_rng(61)
    datas = [S.icosphere(3), S.displaced_mesh(3_000, rng)]
    meshes = [mesh_from_data(m).build() for m in datas]
    cps = S.hair_curves(64, 10, rng)
    segs = S.curve_segments(64, 10, 2)
    cv = Curve(2, torch.from_numpy(cps).cuda(), torch.from_numpy(segs.astype(np.int32)).cuda()).build()
    acc = Accel()
    aff = S.affine_rows(S.random_rotations(4, rng), rng.uniform(0.3, 0.6, 4), rng.uniform(-1, 1, (4, 3)))
    for i in range(2):
        acc.emplace_back(meshes[i], aff[i].reshape(3, 4))
    acc.emplace_back(cv, aff[2].reshape(3, 4))
    keys = S.affine_rows(S.random_rotations(3, rng), rng.uniform(0.2, 0.5, 3), rng.uniform(-1, 1, (3, 3)))
    mo = MotionInstance(meshes[1], keys.reshape(-1, 3, 4), 0.0, 1.0, vanish_end=True)
    acc.emplace_back(mo)
    acc.build()
    rays = S.sphere_rays(80_000, [-1.5] * 3, [1.5] * 3, seed=62)
    times = rng.uniform(-0.2, 1.2, rays.shape[0]).astype(np.float32)
    d, dt = rays_to_device(rays), torch.from_numpy(times).cuda()
    want_t = hits_to_numpy(acc.trace_closest_motion(d, dt))
    want_0 = hits_to_numpy(acc.trace_closest(d))
    any_t = acc.trace_any_motion(d, dt).cpu().numpy()
    any_0 = acc.trace_any(d).cpu().numpy()
    torch.cuda.synchronize()
    assert (want_t["inst"] == 2).sum() > 50 and (want_t["inst"] == 3).sum() > 50  # curves and the moving mesh
    for variant in (0, 1):
        assert _same(_device_closest(tk, acc, d, variant, d_times=dt), want_t), variant
        assert _same(_device_closest(tk, acc, d, variant), want_0), variant
        assert np.array_equal(_device_any(tk, acc, d, variant, d_times=dt), any_t), variant
        assert np.array_equal(_device_any(tk, acc, d, variant), any_0), variant


@pytest.mark.parametrize("reorder", [0, 6])
def test_loop_mode_3_through_the_c_abi(lcx, oracle_mod, full_terrain, reorder):
    """lcx_set_trace_tuning(mode 3): the plain entry points launch one thread per ray through the
    device functions; records equal the oracle's (closest, any), with and without reordering."""
    import torch
    from luisacompute_gb300 import _capi
    from luisacompute_gb300.accel import accel_from_scene, hits_to_numpy, rays_to_device
    lib = _capi.load()
    scene, osc = full_terrain
    acc, _m = accel_from_scene(scene)
    rays = S.terrain_rays(scene, 1 << 19, seed=14)
    shadow = S.terrain_shadow_rays(scene, 1 << 19, seed=15)
    k = [ctypes.c_uint32(0) for _ in range(3)]
    _capi.check(lib.lcx_get_trace_tuning(*[ctypes.byref(x) for x in k]), "get")
    rb, rm = ctypes.c_uint32(0), ctypes.c_uint32(0)
    _capi.check(lib.lcx_get_trace_reorder(ctypes.byref(rb), ctypes.byref(rm)), "get")
    _capi.check(lib.lcx_set_trace_tuning(k[0].value, k[1].value, 3), "mode 3")
    _capi.check(lib.lcx_set_trace_reorder(reorder, 1024), "reorder")
    try:
        got = hits_to_numpy(acc.trace_closest(rays_to_device(rays)))
        occ = acc.trace_any(rays_to_device(shadow)).cpu().numpy()
        torch.cuda.synchronize()
        _capi.check(lib.lcx_check_trace_errors(), "errors")
    finally:
        _capi.check(lib.lcx_set_trace_tuning(k[0].value, k[1].value, k[2].value), "restore")
        _capi.check(lib.lcx_set_trace_reorder(rb.value, rm.value), "restore")
    assert _same(got, osc.trace_closest(rays))
    assert np.array_equal(occ, osc.trace_any(shadow))
