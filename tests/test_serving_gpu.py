"""Serving: every request's result is the same served alone (one request at a time) and in the
continuous-batching mix (shared launches, overlapping streams, LRU eviction, scene uploads)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("max_batch_rays,min_chunk,direct", [(60_000, 1 << 16, None), (16_384, 1_024, None),
                                                              (16_384, 1_024, False)])
def test_mix_equals_alone(lcx, oracle_mod, max_batch_rays, min_chunk, direct):
    """With the small cap, requests of up to 40k rays are split into chunks across launches
    and streams; every result must still equal the request served alone, with the kernels reading
    and writing the requests' pinned buffers directly (the default on a coherent host link) and
    through device copies (direct=False)."""
    from luisacompute_gb300 import scenes as S
    from luisacompute_gb300 import serving as V
    scenes, reqs = V.make_workload(n_scenes=6, n_requests=60, rate_hz=3000.0, tri_lo=2_000, tri_hi=60_000,
                                   ray_lo=500, ray_hi=40_000, new_scene_frac=0.15, seed=5)
    assert any(r.new_scene is not None for r in reqs)
    # a small budget forces evictions and rebuilds on demand
    budget = 12 << 20
    mix = V.ContinuousServer(V.SceneStore(scenes, budget), slots=3, max_batch_rays=max_batch_rays,
                             min_chunk=min_chunk, direct_host=direct)
    got = V.results(mix.run([V.Request(r.rid, r.arrival, r.scene, r.rays, r.any_hit, r.new_scene) for r in reqs]))
    assert mix.store.evictions > 0
    if max_batch_rays >= 40_000:
        assert mix.batches < len(reqs)  # requests share launches
    else:
        assert mix.chunks > len(reqs)  # some requests were split
    alone = V.PlainServer(V.SceneStore(scenes, 1 << 40))
    want = V.results(alone.run([V.Request(r.rid, r.arrival, r.scene, r.rays, r.any_hit, r.new_scene)
                                for r in reqs]))
    for r, a, b in zip(sorted(reqs, key=lambda q: q.arrival), got, want):
        assert np.array_equal(a.view(np.uint8), b.view(np.uint8)), f"request {r.rid}"
    # and against the oracle for a few closest-hit requests
    checked = 0
    for r, a in zip(sorted(reqs, key=lambda q: q.arrival), got):
        if r.any_hit or checked >= 4:
            continue
        md = r.new_scene if r.new_scene is not None else scenes[r.scene]
        sc = S.Scene([md], np.zeros(1, np.int64), S.IDENTITY[None].copy(), np.full(1, 0xFF, np.uint32))
        want_o = oracle_mod.OracleScene(sc).trace_closest(r.rays)
        assert np.array_equal(a.view(np.uint8), want_o.view(np.uint8))
        checked += 1
    assert checked == 4


def test_trace_jobs_equals_single_calls(lcx):
    import torch
    from luisacompute_gb300 import _capi
    from luisacompute_gb300 import scenes as S
    from luisacompute_gb300.accel import accel_from_scene, hits_to_numpy, rays_to_device
    lib = _capi.load()
    accs = []
    for k in range(3):
        sc = S.Scene([S.icosphere(3 + k)], np.zeros(1, np.int64), S.IDENTITY[None].copy(), np.full(1, 0xFF, np.uint32))
        accs.append(accel_from_scene(sc))
    ray_sets = [S.sphere_rays(n, [-1.5] * 3, [1.5] * 3, seed=40 + i) for i, n in enumerate([1, 777, 5000, 33, 20000])]
    d_rays = [rays_to_device(r) for r in ray_sets]
    outs, jobs = [], (_capi.LcxTraceJob * len(ray_sets))()
    for i, d in enumerate(d_rays):
        anyhit = i % 2 == 1
        o = torch.zeros(d.shape[0] * (1 if anyhit else 6), dtype=torch.uint8 if anyhit else torch.int32, device="cuda")
        outs.append(o)
        jobs[i] = _capi.LcxTraceJob(accs[i % 3][0].handle, d.data_ptr(), o.data_ptr(), d.shape[0], 0xFF,
                                    1 if anyhit else 0, 0)
    import ctypes
    old = [ctypes.c_uint32(0) for _ in range(3)]
    _capi.check(lib.lcx_get_trace_tuning(*old), "get")
    try:
        # single calls in loop mode 0 are the reference; the multi-job launch runs in mode 2
        # (deferred triangle batches, the default for quantised nodes) and in mode 0
        _capi.check(lib.lcx_set_trace_tuning(old[0].value, 0, 0), "mode 0")
        want = {}
        for layout in (0, 1):
            for i, d in enumerate(d_rays):
                acc = accs[i % 3][0]
                want[layout, i] = (acc.trace_any(d, layout=layout).cpu() if i % 2 == 1 else
                                   hits_to_numpy(acc.trace_closest(d, layout=layout)).view(np.uint8))
        for mode, post in ((2, 0), (2, 3), (0, 0)):
            _capi.check(lib.lcx_set_trace_tuning(old[0].value, post, mode), "mode")
            for layout in (0, 1):
                for o in outs:
                    o.zero_()
                _capi.check(lib.lcx_trace_jobs(jobs, len(ray_sets), layout, None), "lcx_trace_jobs")
                torch.cuda.synchronize()
                for i, d in enumerate(d_rays):
                    if i % 2 == 1:
                        assert torch.equal(outs[i].cpu(), want[layout, i]), (mode, layout, i)
                    else:
                        assert np.array_equal(hits_to_numpy(outs[i].view(-1, 6)).view(np.uint8), want[layout, i]), \
                            (mode, layout, i)
    finally:
        _capi.check(lib.lcx_set_trace_tuning(old[0].value, old[1].value, old[2].value), "restore")
    _capi.check(lib.lcx_check_trace_errors(), "errors")
