"""lcx_trace_closest_noalloc: the trace entry point for callers that cannot allocate device
memory (applications that reserve HBM at start-up, plugins whose host framework owns all
device allocations, loops that must not hit cudaMalloc's implicit synchronisation).

Called through the C ABI and compared bit for bit with lcx_trace_closest, the regular entry
point (the same exactness the other parity tests demand), on two calls in a row: the
static scratch array keeps the previous call's counter, so the second call checks that the
entry point clears it.  Also checks that the calls leave the device's free memory unchanged.
Also runs it in loop mode 0, and checks that its kernel-side bounds reach
lcx_check_trace_errors.  Kept in its own file, collected last.
"""
import ctypes

import numpy as np
import pytest

from luisacompute_gb300 import scenes as S

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def small_scene(lcx):
    from luisacompute_gb300.accel import accel_from_scene, rays_to_device
    scene = S.terrain_scene(n=128, sphere_count=64, sphere_subdiv=3)
    acc, meshes = accel_from_scene(scene)
    rays = S.terrain_rays(scene, 300_000, seed=21)
    return acc, meshes, rays_to_device(rays), rays.shape[0]


@pytest.mark.parametrize("mode", [2, 0])
def test_noalloc_matches_regular_entry_point(lcx, small_scene, mode):
    """In the default loop structure (mode 2, deferred triangle batches) and in mode 0."""
    import torch
    from luisacompute_gb300 import _capi
    from luisacompute_gb300.accel import stream_handle

    lib = _capi.load()
    acc, _meshes, d_rays, n = small_scene
    st = stream_handle(None)
    knobs = [ctypes.c_uint32(0) for _ in range(3)]
    _capi.check(lib.lcx_get_trace_tuning(*[ctypes.byref(k) for k in knobs]), "lcx_get_trace_tuning")
    _capi.check(lib.lcx_set_trace_tuning(knobs[0].value, knobs[1].value, mode), "lcx_set_trace_tuning")
    try:
        want = torch.empty((n, 6), dtype=torch.int32, device="cuda")
        _capi.check(lib.lcx_trace_closest(acc.handle, d_rays.data_ptr(), n, 0xFF, want.data_ptr(), st),
                    "lcx_trace_closest")
        torch.cuda.synchronize()
        expected = want.cpu().numpy()
        assert (expected[:, 0] != -1).sum() > 1000  # the rays hit something

        outs = [torch.full((n, 6), -7, dtype=torch.int32, device="cuda") for _ in range(3)]
        # the first call on this device looks up the scratch array's address
        _capi.check(lib.lcx_trace_closest_noalloc(acc.handle, d_rays.data_ptr(), n, 0xFF, outs[0].data_ptr(), st),
                    "lcx_trace_closest_noalloc")
        torch.cuda.synchronize()
        free_before = torch.cuda.mem_get_info()[0]
        for out in outs[1:]:  # two more calls in a row on the same static scratch
            _capi.check(lib.lcx_trace_closest_noalloc(acc.handle, d_rays.data_ptr(), n, 0xFF, out.data_ptr(), st),
                        "lcx_trace_closest_noalloc")
        torch.cuda.synchronize()
        free_after = torch.cuda.mem_get_info()[0]
        for out in outs:
            assert np.array_equal(out.cpu().numpy(), expected)
        assert free_after == free_before
        _capi.check(lib.lcx_check_trace_errors(), "lcx_check_trace_errors")
    finally:
        _capi.check(lib.lcx_set_trace_tuning(*[k.value for k in knobs]), "lcx_set_trace_tuning")


def test_noalloc_reports_kernel_bounds(lcx, small_scene):
    """A step bound of 3 ends the rays early on a valid scene (the kernel returns normally); the
    flag the kernel leaves in the static scratch reaches lcx_check_trace_errors as
    LCX_ERR_TIMEOUT, and the next check is clean."""
    import torch
    from luisacompute_gb300 import _capi
    from luisacompute_gb300.accel import stream_handle

    lib = _capi.load()
    acc, _meshes, d_rays, n = small_scene
    assert lib.lcx_check_trace_errors() == _capi.LCX_OK
    out = torch.empty((n, 6), dtype=torch.int32, device="cuda")
    _capi.check(lib.lcx_set_trace_step_bound(3), "lcx_set_trace_step_bound")
    try:
        _capi.check(lib.lcx_trace_closest_noalloc(acc.handle, d_rays.data_ptr(), n, 0xFF, out.data_ptr(),
                                                  stream_handle(None)), "lcx_trace_closest_noalloc")
        torch.cuda.synchronize()
    finally:
        _capi.check(lib.lcx_set_trace_step_bound(0), "lcx_set_trace_step_bound")
    assert lib.lcx_check_trace_errors() == _capi.LCX_ERR_TIMEOUT
    assert lib.lcx_check_trace_errors() == _capi.LCX_OK


def test_noalloc_rejects_oversize_and_bad_handle(lcx):
    from luisacompute_gb300 import _capi
    lib = _capi.load()
    rc = lib.lcx_trace_closest_noalloc(0, None, 1, 0xFF, None, None)
    assert rc == _capi.LCX_ERR_INVALID_ARG
    import torch
    from luisacompute_gb300.accel import accel_from_scene
    acc, _m = accel_from_scene(S.icosphere_scene(1))
    buf = torch.zeros(64, dtype=torch.float32, device="cuda")
    rc = lib.lcx_trace_closest_noalloc(acc.handle, buf.data_ptr(), (1 << 31) + 1, 0xFF, buf.data_ptr(), None)
    assert rc == _capi.LCX_ERR_INVALID_ARG
    assert b"maximum" in lib.lcx_last_error_string()
    torch.cuda.synchronize()
