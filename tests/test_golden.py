"""Golden vectors: the Cornell box of the reference's path-tracing tests
(src/tests/common/cornell_box.h, src/tests/test_path_tracing.cpp:40-104) with seeded rays.

The fixture (tests/golden/cornell_box.npz, made by tests/golden/make_golden.py) holds the
oracle's answers.  The CPU tests pin the oracle to them, so a change of compiler, CPU
architecture or oracle code that moves one bit fails here; the GPU tests require the CUDA
path to reproduce them bit for bit through the C ABI, for both node layouts, with the
meshes sharing one vertex buffer as the reference test's meshes do.
"""
import numpy as np
import pytest

from luisacompute_gb300 import scenes as S
from tests.golden import make_golden as G


@pytest.fixture(scope="module")
def golden():
    return G.load()


def _same(a, b):
    return a.tobytes() == b.tobytes()


def test_fixture_shape(golden):
    scene, _, albedo, prm, z = golden
    assert [str(n) for n in z["group_names"]] == ["floor", "ceiling", "backWall", "rightWall", "leftWall",
                                                  "shortBox", "tallBox", "light"]
    assert scene.instanced_triangles() == 36 and len(albedo) == 8
    assert z["pt_image"].shape == (prm["height"], prm["width"], 3)
    # Every camera ray meets the box; the light's quad faces down and the point light sits below it.
    assert (z["hits_camera"]["inst"] != S.MISS).all()


def test_oracle_reproduces_golden(oracle_mod, golden):
    scene, mscene, albedo, prm, z = golden
    orc = oracle_mod.OracleScene(scene)
    assert _same(orc.trace_closest(z["rays_camera"]), z["hits_camera"])
    assert _same(orc.trace_closest(z["rays_incoherent"]), z["hits_incoherent"])
    assert _same(orc.brute_closest(z["rays_incoherent"]), z["hits_incoherent"])
    assert _same(orc.trace_any(z["rays_shadow"]), z["occluded_shadow"])
    morc = oracle_mod.OracleScene(mscene)
    assert _same(morc.trace_closest(z["rays_incoherent"], mask=0x55), z["hits_mask55"])
    assert _same(morc.trace_any(z["rays_shadow"], mask=0x55), z["occluded_mask55"])
    from luisacompute_gb300 import pathtrace as P
    image, first = orc.pathtrace(scene, albedo, P.params(**prm), threads=2)
    assert _same(image, z["pt_image"]) and _same(first, z["pt_first_hits"])


def _gpu_scene(scene, masks=None):
    """The fixture's meshes over ONE shared device vertex buffer (as the reference test builds them)."""
    import torch
    from luisacompute_gb300.accel import Accel, Mesh
    v = torch.from_numpy(scene.meshes[0].vertices).cuda()
    meshes = [Mesh(v, torch.from_numpy(m.triangles.astype(np.int32)).cuda()).build() for m in scene.meshes]
    acc = Accel()
    acc.emplace_back_many(meshes, scene.inst_affine, scene.inst_mask if masks is None else masks)
    acc.build()
    return acc, meshes


@pytest.mark.gpu
@pytest.mark.parametrize("layout", [0, 1])
def test_gpu_reproduces_golden_queries(lcx, golden, layout):
    import torch
    from luisacompute_gb300.accel import hits_to_numpy, rays_to_device
    scene, mscene, _, _, z = golden
    acc, meshes = _gpu_scene(scene)
    for rays, want in (("rays_camera", "hits_camera"), ("rays_incoherent", "hits_incoherent")):
        got = hits_to_numpy(acc.trace_closest(rays_to_device(z[rays]), layout=layout))
        assert _same(got, z[want]), rays
    occ = acc.trace_any(rays_to_device(z["rays_shadow"]), layout=layout).cpu().numpy()
    assert _same(occ, z["occluded_shadow"])
    macc, mmeshes = _gpu_scene(mscene)
    got = hits_to_numpy(macc.trace_closest(rays_to_device(z["rays_incoherent"]), mask=0x55, layout=layout))
    assert _same(got, z["hits_mask55"])
    occ = macc.trace_any(rays_to_device(z["rays_shadow"]), mask=0x55, layout=layout).cpu().numpy()
    assert _same(occ, z["occluded_mask55"])
    assert lcx.lcx_check_trace_errors() == 0
    torch.cuda.synchronize()


@pytest.mark.gpu
def test_gpu_reproduces_golden_pathtrace(lcx, golden):
    from luisacompute_gb300 import pathtrace as P
    scene, _, albedo, prm, z = golden
    acc, meshes = _gpu_scene(scene)
    image, first, _ = P.render(scene, acc, meshes, albedo, P.params(**prm), first_hits=True)
    assert _same(first, z["pt_first_hits"])
    assert _same(image, z["pt_image"])
