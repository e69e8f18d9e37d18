"""The autotuner on a small scene: it measures every candidate, leaves the best applied, and
no knob it sets changes a hit record (checked against the oracle)."""
import numpy as np
import pytest

from luisacompute_gb300 import scenes as S

pytestmark = pytest.mark.gpu


def test_autotune_small_scene(lcx, oracle_mod, tmp_path):
    import torch
    from luisacompute_gb300 import autotune as A
    from luisacompute_gb300.accel import accel_from_scene, hits_to_numpy, rays_to_device
    scene = S.terrain_scene(n=128, sphere_count=16, sphere_subdiv=3)
    rays = S.terrain_rays(scene, 60_000, seed=31)
    shadow = S.terrain_shadow_rays(scene, 30_000, seed=32)
    want = oracle_mod.OracleScene(scene).trace_closest(rays)
    old = A.current()
    try:
        res = A.tune(scene, rays_to_device(rays), rays_to_device(shadow), reps=1,
                     build_space={"leaf_max": [1, 3], "width": [4]},
                     trace_space={"refill": [1, 8], "short_stack": [8, 24], "mode": [1], "reorder_bits": [6]})
        # start + 3 build candidates + the re-build of the winner + 6 traversal candidates
        assert len(res.trials) == 11
        assert A.current() == res.config
        assert res.tuned_ms <= res.default_ms * 1.5
        acc, _ = accel_from_scene(scene)
        got = hits_to_numpy(acc.trace_closest(rays_to_device(rays)))
        torch.cuda.synchronize()
        assert np.array_equal(got.view(np.uint8), want.view(np.uint8))
        path = tmp_path / "tune.json"
        A.save(path, scene, res)
        A.apply(old)
        assert A.load(path, scene) == res.config and A.current() == res.config
    finally:
        A.apply(old)
