"""Wavefront path tracing: the GPU frame equals the CPU restatement's bit for bit (same random
numbers, same FP32 sequence, bit-exact traversal), and its first-bounce hits equal the oracle's
closest hits on the same camera rays."""
import numpy as np
import pytest

from luisacompute_gb300 import scenes as S

pytestmark = pytest.mark.gpu


def _check(scene, prm, oracle_mod):
    from luisacompute_gb300 import pathtrace as PT
    from luisacompute_gb300.accel import accel_from_scene
    acc, meshes = accel_from_scene(scene)
    alb = PT.albedos(scene)
    img, hits, st = PT.render(scene, acc, meshes, alb, prm, first_hits=True)
    assert st.bounces >= 1 and st.closest_rays >= prm.width * prm.height * prm.spp
    osc = oracle_mod.OracleScene(scene)
    cimg, chits = osc.pathtrace(scene, alb, prm)
    assert np.array_equal(hits.view(np.uint8), chits.view(np.uint8))
    rmse = float(np.sqrt(np.mean((img - cimg) ** 2)))
    assert rmse == 0.0, rmse
    assert np.isfinite(img).all() and img.mean() > 0.0
    return img, st


def test_icosphere_frame(lcx, oracle_mod):
    from luisacompute_gb300 import pathtrace as PT
    _check(S.icosphere_scene(4), PT.params(width=96, height=64, spp=2), oracle_mod)


def test_terrain_frame_multibounce(lcx, oracle_mod):
    from luisacompute_gb300 import pathtrace as PT
    scene = S.terrain_scene(n=64, sphere_count=24, sphere_subdiv=2)
    prm = PT.params(width=80, height=48, spp=2, eye=(0.0, 0.8, 2.4))
    img, st = _check(scene, prm, oracle_mod)
    assert st.bounces >= 4 and st.any_rays > 0
