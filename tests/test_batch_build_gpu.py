"""Batched BLAS builds (lcx_mesh_build_batch) and build knobs: results must equal the oracle's
bit for bit, whatever the batch composition or node width."""
import ctypes

import numpy as np
import pytest

from luisacompute_gb300 import scenes as S

pytestmark = pytest.mark.gpu


def batch_scene(seed=0, count=24):
    rng = np.random.default_rng(seed)
    meshes = S.batch_meshes(count, lo=1, hi=3000, seed=seed)
    meshes.insert(3, S.MeshData(np.zeros((3, 4), np.float32), np.zeros((0, 3), np.uint32)))  # empty
    meshes.insert(7, S.MeshData(np.array([[0, 0, 0, 0], [1, 0, 0, 0], [0, 1, 0, 0]], np.float32),
                                np.array([[0, 1, 2]], np.uint32)))  # one triangle
    n = len(meshes)
    rot = S.random_rotations(n, rng)
    aff = S.affine_rows(rot, np.exp(rng.uniform(np.log(0.05), np.log(0.4), n)), rng.uniform(-1, 1, (n, 3)))
    return S.Scene(meshes, np.arange(n), aff, np.full(n, 0xFF, np.uint32))


def run(scene, rays, batch):
    import torch
    from luisacompute_gb300.accel import accel_from_scene, hits_to_numpy, rays_to_device
    acc, meshes = accel_from_scene(scene, batch=batch)
    d = rays_to_device(rays)
    out = [hits_to_numpy(acc.trace_closest(d, layout=l)) for l in (0, 1)]
    torch.cuda.synchronize()
    return out, acc, meshes


def test_batch_equals_oracle_and_single(lcx, oracle_mod):
    scene = batch_scene()
    lo, hi = scene.bounds()
    rays = S.sphere_rays(100_000, lo, hi, seed=3)
    want = oracle_mod.OracleScene(scene).trace_closest(rays)
    (bq, bf), acc_b, meshes_b = run(scene, rays, True)
    (sq, sf), acc_s, meshes_s = run(scene, rays, False)
    for got in (bq, bf, sq, sf):
        assert np.array_equal(got.view(np.uint8), want.view(np.uint8))
    assert (want["inst"] != S.MISS).sum() > 1000
    # per-mesh stats agree between the batch and single builds up to the Morton precision a batch
    # gives up for its segment ids (19 instead of 21 bits per axis at 26 meshes)
    for mb, ms in zip(meshes_b, meshes_s):
        a, b = mb.stats(), ms.stats()
        assert a.leaf_prim_count == b.leaf_prim_count and abs(int(a.depth) - int(b.depth)) <= 1
        assert abs(a.sah_cost - b.sah_cost) <= 0.05 * max(1.0, b.sah_cost)
        assert abs(int(a.node_count) - int(b.node_count)) <= 0.05 * max(1, b.node_count)


@pytest.mark.parametrize("leaf_max,width", [(1, 8), (3, 8), (2, 4), (2, 2), (3, 6)])
def test_build_knobs_do_not_change_results(lcx, oracle_mod, leaf_max, width):
    from luisacompute_gb300 import _capi
    lib = _capi.load()
    scene = S.terrain_scene(n=96, sphere_count=32, sphere_subdiv=3)
    rays = np.concatenate([S.terrain_rays(scene, 60_000, seed=31), S.terrain_shadow_rays(scene, 20_000, seed=32)])
    osc = oracle_mod.OracleScene(scene)
    want = osc.trace_closest(rays)
    old = [ctypes.c_uint32(0), ctypes.c_uint32(0)]
    _capi.check(lib.lcx_get_build_tuning(*old), "get")
    try:
        _capi.check(lib.lcx_set_build_tuning(leaf_max, width), "set")
        (q, f), acc, meshes = run(scene, rays, True)
    finally:
        _capi.check(lib.lcx_set_build_tuning(old[0].value, old[1].value), "set")
    assert np.array_equal(q.view(np.uint8), want.view(np.uint8))
    assert np.array_equal(f.view(np.uint8), want.view(np.uint8))


def test_batch_rebuild_keeps_shared_block_alive(lcx, oracle_mod):
    """Rebuilding one mesh of a batch alone must not free the others' BVHs."""
    import torch
    from luisacompute_gb300.accel import Accel, build_meshes, hits_to_numpy, mesh_from_data, rays_to_device
    scene = batch_scene(seed=5, count=8)
    meshes = build_meshes([mesh_from_data(m) for m in scene.meshes])
    meshes[0].build()  # leaves the batch's block
    acc = Accel()
    acc.emplace_back_many([meshes[i] for i in scene.inst_mesh], scene.inst_affine, scene.inst_mask)
    acc.build()
    lo, hi = scene.bounds()
    rays = S.sphere_rays(50_000, lo, hi, seed=9)
    got = hits_to_numpy(acc.trace_closest(rays_to_device(rays)))
    torch.cuda.synchronize()
    want = oracle_mod.OracleScene(scene).trace_closest(rays)
    assert np.array_equal(got.view(np.uint8), want.view(np.uint8))
