"""Failure paths on the GPU, in forms that fault, trap or hang nothing.

* The per-ray step bound: lowered to a few steps with lcx_set_trace_step_bound, it ends the
  rays of a valid scene early; the kernels return normally and lcx_check_trace_errors reports
  LCX_ERR_TIMEOUT for every trace form (closest and any hit, loop modes 2 and 0, multi-job
  launches).  With the default bound restored the same calls equal the oracle again.
* Serving: a scene larger than the whole HBM budget is refused (its requests fail with the
  budget error, every other request is served as it is alone), and a request cancelled while
  its chunks are running stops taking launches without disturbing the others.
"""
import ctypes

import numpy as np
import pytest

from luisacompute_gb300 import scenes as S

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def scene_and_rays(lcx):
    from luisacompute_gb300.accel import accel_from_scene, rays_to_device
    scene = S.terrain_scene(n=128, sphere_count=64, sphere_subdiv=3)
    acc, meshes = accel_from_scene(scene)
    rays = S.terrain_rays(scene, 100_000, seed=31)
    return scene, acc, meshes, rays, rays_to_device(rays)


def _tuning(lib):
    from luisacompute_gb300 import _capi
    k = [ctypes.c_uint32(0) for _ in range(3)]
    _capi.check(lib.lcx_get_trace_tuning(*[ctypes.byref(x) for x in k]), "lcx_get_trace_tuning")
    return [x.value for x in k]


@pytest.mark.parametrize("mode", [2, 0])
def test_step_bound_reports_timeout(scene_and_rays, oracle_mod, mode):
    import torch
    from luisacompute_gb300 import _capi
    from luisacompute_gb300.accel import hits_to_numpy
    lib = _capi.load()
    scene, acc, _m, rays, d = scene_and_rays
    old = _tuning(lib)
    _capi.check(lib.lcx_set_trace_tuning(old[0], old[1], mode), "lcx_set_trace_tuning")
    try:
        assert lib.lcx_check_trace_errors() == _capi.LCX_OK
        _capi.check(lib.lcx_set_trace_step_bound(3), "lcx_set_trace_step_bound")
        try:
            acc.trace_closest(d)
            torch.cuda.synchronize()
            assert lib.lcx_check_trace_errors() == _capi.LCX_ERR_TIMEOUT
            assert b"step bound" in lib.lcx_last_error_string()
            acc.trace_any(d)
            torch.cuda.synchronize()
            assert lib.lcx_check_trace_errors() == _capi.LCX_ERR_TIMEOUT
            # multi-job launch
            out = torch.empty((rays.shape[0], 6), dtype=torch.int32, device="cuda")
            jobs = (_capi.LcxTraceJob * 1)()
            jobs[0] = _capi.LcxTraceJob(acc.handle, d.data_ptr(), out.data_ptr(), rays.shape[0], 0xFF, 0, 0)
            _capi.check(lib.lcx_trace_jobs(jobs, 1, 1, None), "lcx_trace_jobs")
            torch.cuda.synchronize()
            assert lib.lcx_check_trace_errors() == _capi.LCX_ERR_TIMEOUT
        finally:
            _capi.check(lib.lcx_set_trace_step_bound(0), "lcx_set_trace_step_bound")
        # the default bound: clean, and the records equal the oracle's
        got = hits_to_numpy(acc.trace_closest(d))
        torch.cuda.synchronize()
        assert lib.lcx_check_trace_errors() == _capi.LCX_OK
        want = oracle_mod.OracleScene(scene).trace_closest(rays)
        assert np.array_equal(got.view(np.uint8), want.view(np.uint8))
    finally:
        _capi.check(lib.lcx_set_trace_tuning(*old), "lcx_set_trace_tuning")


def _clone(reqs):
    from luisacompute_gb300 import serving as V
    return [V.Request(r.rid, r.arrival, r.scene, r.rays, r.any_hit, r.new_scene) for r in reqs]


def test_serving_budget_refusal(lcx):
    """An upload whose scene alone exceeds the budget fails with the budget error; the other
    requests (including ones that force evictions) equal their results served alone."""
    from luisacompute_gb300 import serving as V
    scenes, reqs = V.make_workload(n_scenes=4, n_requests=30, rate_hz=3000.0, tri_lo=2_000, tri_hi=30_000,
                                   ray_lo=500, ray_hi=20_000, new_scene_frac=0.0, seed=8)
    budget = 8 << 20
    rng = np.random.default_rng(3)
    big = S.displaced_mesh(200_000, rng)
    assert V.SceneStore.estimate(big) > budget
    reqs[10] = V.Request(10, reqs[10].arrival, 1000, reqs[10].rays, False, big)
    mix = V.ContinuousServer(V.SceneStore(scenes, budget), slots=3, max_batch_rays=16_384, min_chunk=1_024)
    done = mix.run(_clone(reqs))
    assert mix.failed == 1
    failed = [r for r in done if r.error is not None]
    assert [r.rid for r in failed] == [10] and "budget" in failed[0].error
    got = V.results(done)
    alone = V.PlainServer(V.SceneStore(scenes, budget))
    ref = alone.run(_clone(reqs))
    assert [r.rid for r in ref if r.error is not None] == [10]
    want = V.results(ref)
    for r, a, b in zip(done, got, want):
        if r.error is None:
            assert np.array_equal(a.view(np.uint8), b.view(np.uint8)), f"request {r.rid}"
    assert V.latency_stats(done)["requests"] == len(reqs) - 1


def test_serving_cancel_mid_flight(lcx):
    """A 400k-ray request split into 16k-ray chunks is cancelled from the serving loop as its
    first chunk launches: it stops taking launches, the chunks it launched hold the alone results
    for their rays, and every other request equals its result served alone."""
    from luisacompute_gb300 import serving as V
    scenes, reqs = V.make_workload(n_scenes=4, n_requests=30, rate_hz=3000.0, tri_lo=2_000, tri_hi=30_000,
                                   ray_lo=500, ray_hi=20_000, new_scene_frac=0.0, seed=9)
    big_rays = S.sphere_rays(400_000, [-1.3] * 3, [1.3] * 3, seed=12)
    reqs[5] = V.Request(5, reqs[5].arrival, reqs[5].scene, big_rays, False, None)

    def on_launch(server, batch):
        if any(r.rid == 5 for r, _, _ in batch):
            server.cancel(5)

    mix = V.ContinuousServer(V.SceneStore(scenes, 1 << 40), slots=3, max_batch_rays=16_384, min_chunk=1_024,
                             on_launch=on_launch)
    done = mix.run(_clone(reqs))
    big = next(r for r in done if r.rid == 5)
    assert big.cancelled and big.done > 0 and mix.cancelled == 1
    launched = sorted((f, n) for _, _, pieces in mix.timeline for rid, f, n in pieces if rid == 5)
    end = 0
    for f, n in launched:  # chunks are taken in order: a prefix of the rays
        assert f == end
        end += n
    assert 0 < end < big_rays.shape[0]
    got = V.results(done)
    want = V.results(V.PlainServer(V.SceneStore(scenes, 1 << 40)).run(_clone(reqs)))
    for r, a, b in zip(done, got, want):
        if r.rid == 5:
            assert np.array_equal(a[:end].view(np.uint8), b[:end].view(np.uint8))
        else:
            assert np.array_equal(a.view(np.uint8), b.view(np.uint8)), f"request {r.rid}"
