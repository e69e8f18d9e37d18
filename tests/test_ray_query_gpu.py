"""RayQuery with per-candidate callbacks in a user kernel (include/lcx/ray_query.cuh; reference
include/luisa/dsl/rtx/ray_query.h:17-240 and the alpha-cutout path tracer
src/tests/test_path_tracing_cutout.cpp).

tests/cuda/ray_query_kernels.cu is compiled here as a user would compile it. Committing every
candidate must give lcx_trace_closest's records bit for bit. An alpha cutout (triangles with
prim % 3 == 0 transparent) must give the oracle's records on the scene with those triangles
removed, mapped back to the original prim ids."""
import ctypes
import subprocess
from pathlib import Path

import numpy as np
import pytest

from luisacompute_gb300 import scenes as S

pytestmark = pytest.mark.gpu
ROOT = Path(__file__).resolve().parent.parent
CUT = 3


@pytest.fixture(scope="module")
def rq(tmp_path_factory):
    from luisacompute_gb300 import build as B
    out = tmp_path_factory.mktemp("rq") / "librq.so"
    subprocess.run([B.nvcc_path(), B.ARCH, "-O3", "-std=c++17", "-shared", "-Xcompiler", "-fPIC", "-cudart", "shared",
                    f"-I{ROOT / 'include'}", "-o", str(out), str(ROOT / "tests/cuda/ray_query_kernels.cu")],
                   check=True, capture_output=True)
    lib = ctypes.CDLL(str(out))
    lib.rq_run.restype = ctypes.c_int
    lib.rq_run.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32,
                           ctypes.c_void_p, ctypes.c_void_p]
    return lib


def _view(acc):
    from luisacompute_gb300 import _capi
    v = _capi.LcxAccelView()
    _capi.check(_capi.load().lcx_accel_device_view(acc.handle, ctypes.byref(v)), "lcx_accel_device_view")
    return v


def _cut_scene(scene):
    """The scene without the transparent triangles, and per mesh the original prim id of each kept one."""
    keeps, meshes = [], []
    for m in scene.meshes:
        keep = np.nonzero(np.arange(m.tri_count) % CUT != 0)[0].astype(np.uint32)
        keeps.append(keep)
        meshes.append(S.MeshData(m.vertices, m.triangles[keep]))
    return S.Scene(meshes, scene.inst_mesh, scene.inst_affine, scene.inst_mask), keeps


def test_ray_query_commit_all_and_cutout(lcx, oracle_mod, rq):
    import torch
    from luisacompute_gb300.accel import accel_from_scene, hits_to_numpy, rays_to_device
    scene = S.terrain_scene(n=128, sphere_count=16, sphere_subdiv=3)
    rays = np.concatenate([S.terrain_rays(scene, 50_000, seed=41), S.terrain_shadow_rays(scene, 30_000, seed=42)])
    acc, meshes = accel_from_scene(scene)
    view = _view(acc)
    d = rays_to_device(rays)
    n = rays.shape[0]
    hits = torch.empty((n, 6), dtype=torch.int32, device="cuda")
    occ = torch.zeros(n, dtype=torch.uint8, device="cuda")
    # commit everything: lcx_trace_closest bit for bit
    assert rq.rq_run(ctypes.byref(view), d.data_ptr(), n, 0, CUT, hits.data_ptr(), None) == 0
    want = hits_to_numpy(acc.trace_closest(d))
    assert np.array_equal(hits_to_numpy(hits).view(np.uint8), want.view(np.uint8))
    # alpha cutout, closest: the oracle on the cut scene, prim ids mapped back
    cut_scene, keeps = _cut_scene(scene)
    osc = oracle_mod.OracleScene(cut_scene)
    want = osc.trace_closest(rays)
    hit = want["inst"] != S.MISS
    for i in np.nonzero(hit)[0]:
        want["prim"][i] = keeps[scene.inst_mesh[want["inst"][i]]][want["prim"][i]]
    assert rq.rq_run(ctypes.byref(view), d.data_ptr(), n, 1, CUT, hits.data_ptr(), None) == 0
    got = hits_to_numpy(hits)
    assert np.array_equal(got.view(np.uint8), want.view(np.uint8))
    assert np.all(got["prim"][hit] % CUT != 0) and hit.mean() > 0.2
    # alpha cutout, any hit
    assert rq.rq_run(ctypes.byref(view), d.data_ptr(), n, 2, CUT, None, occ.data_ptr()) == 0
    torch.cuda.synchronize()
    assert np.array_equal(occ.cpu().numpy(), osc.trace_any(rays))


def test_device_view_follows_accel_state(lcx):
    import torch
    from luisacompute_gb300 import _capi
    from luisacompute_gb300.accel import accel_from_scene
    scene = S.icosphere_scene(3)
    acc, meshes = accel_from_scene(scene)
    v = _view(acc)
    assert v.tlas_nodes and v.instances and 3 <= v.stack_need <= 32
    meshes[0].build()  # the mesh changed: the accel (and its view) is stale until rebuilt
    out = _capi.LcxAccelView()
    assert _capi.load().lcx_accel_device_view(acc.handle, ctypes.byref(out)) == _capi.LCX_ERR_NOT_BUILT
    acc.build()
    assert _view(acc).tlas_nodes
    torch.cuda.synchronize()
