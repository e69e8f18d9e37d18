"""BLAS refit (PREFER_UPDATE on meshes created with allow_update; the reference's OptiX update
path, src/backends/cuda/cuda_mesh.cpp:42-67, exercised by src/tests/test_rtx.cpp:92-137).

A refit keeps the topology and recomputes triangle records and boxes from the new buffers. Hit
records never depend on topology, so after a refit they must equal the oracle's on the new
geometry bit for bit, exactly as after a full build."""
import numpy as np
import pytest

from luisacompute_gb300 import scenes as S

pytestmark = pytest.mark.gpu


def _scene(meshes):
    n = len(meshes)
    return S.Scene(meshes, np.arange(n), np.tile(S.IDENTITY, (n, 1)), np.full(n, 0xFF, np.uint32))


def _device(meshes, allow_update=True):
    import torch
    from luisacompute_gb300.accel import AccelOption, Mesh
    opt = AccelOption(allow_update=allow_update)
    out = []
    for md in meshes:
        v = torch.from_numpy(np.ascontiguousarray(md.vertices, np.float32)).cuda()
        t = torch.from_numpy(np.ascontiguousarray(md.triangles).astype(np.int32)).cuda()
        out.append(Mesh(v, t, opt))
    return out


def _accel(meshes):
    from luisacompute_gb300.accel import Accel
    acc = Accel()
    acc.emplace_back_many(meshes, np.tile(S.IDENTITY, (len(meshes), 1)))
    acc.build()
    return acc


def _check(oracle_mod, acc, datas, rays):
    import torch
    from luisacompute_gb300 import _capi
    from luisacompute_gb300.accel import hits_to_numpy, rays_to_device
    want = oracle_mod.OracleScene(_scene(datas)).trace_closest(rays)
    for layout in (0, 1):
        got = hits_to_numpy(acc.trace_closest(rays_to_device(rays), layout=layout))
        torch.cuda.synchronize()
        assert np.array_equal(got.view(np.uint8), want.view(np.uint8)), f"layout {layout}"
    _capi.check(_capi.load().lcx_check_trace_errors(), "trace errors")


def _deform(md, rng, sigma, scale=1.0, shift=(0.0, 0.0, 0.0)):
    v = md.vertices.copy()
    v[:, :3] = v[:, :3] * np.float32(scale) + np.asarray(shift, np.float32)
    v[:, :3] += rng.standard_normal((v.shape[0], 3)).astype(np.float32) * np.float32(sigma)
    return S.MeshData(v, md.triangles.copy())


def test_refit_single_mesh(lcx, oracle_mod):
    import torch
    from luisacompute_gb300 import _capi
    from luisacompute_gb300.accel import REQUEST_PREFER_UPDATE, rays_to_device
    rng = np.random.default_rng(3)
    md = S.displaced_mesh(20_000, rng)
    (mesh,) = _device([md])
    mesh.build()
    nodes = mesh.stats().node_count
    acc = _accel([mesh])
    rays = S.sphere_rays(60_000, [-1.3] * 3, [1.3] * 3, seed=31)
    _check(oracle_mod, acc, [md], rays)
    # unchanged vertices: a refit reproduces the same answers
    mesh.build(request=REQUEST_PREFER_UPDATE)
    assert mesh.stats().refits == 1 and mesh.stats().node_count == nodes
    with pytest.raises(_capi.LcxError):  # the accel over the refit mesh is stale until rebuilt
        acc.trace_closest(rays_to_device(rays[:16]))
    acc.build()
    _check(oracle_mod, acc, [md], rays)
    # small, then large deformations, written into the same device buffer
    for sigma, scale, shift in ((0.005, 1.0, (0, 0, 0)), (0.05, 1.7, (0.3, -0.2, 0.1))):
        md = _deform(md, rng, sigma, scale, shift)
        mesh.vertices.copy_(torch.from_numpy(md.vertices).cuda())
        mesh.build(request=REQUEST_PREFER_UPDATE)
        acc.build()
        _check(oracle_mod, acc, [md], S.sphere_rays(60_000, [-2.5] * 3, [2.5] * 3, seed=32))
    assert mesh.stats().refits == 3 and mesh.stats().node_count == nodes


def test_refit_new_index_buffer(lcx, oracle_mod):
    """Same triangle count, different indices: the refit reads each prim's new indices."""
    import torch
    from luisacompute_gb300.accel import REQUEST_PREFER_UPDATE
    rng = np.random.default_rng(4)
    md = S.displaced_mesh(5_000, rng)
    (mesh,) = _device([md])
    mesh.build()
    perm = rng.permutation(md.triangles.shape[0])
    md2 = S.MeshData(md.vertices.copy(), md.triangles[perm].copy())
    mesh.triangles.copy_(torch.from_numpy(md2.triangles.astype(np.int32)).cuda())
    mesh.build(request=REQUEST_PREFER_UPDATE)
    assert mesh.stats().refits == 1
    acc = _accel([mesh])
    _check(oracle_mod, acc, [md2], S.sphere_rays(40_000, [-1.3] * 3, [1.3] * 3, seed=33))


def test_refit_batch_and_fallbacks(lcx, oracle_mod):
    """A batch built together is refit together; a partial batch, a changed triangle count or a
    mesh without allow_update is rebuilt instead -- with the same answers either way."""
    import torch
    from luisacompute_gb300.accel import REQUEST_PREFER_UPDATE, build_meshes
    rng = np.random.default_rng(5)
    datas = [S.displaced_mesh(int(n), rng) for n in (300, 3_000, 12_000, 800, 40_000)]
    meshes = build_meshes(_device(datas))
    rays = S.sphere_rays(80_000, [-1.5] * 3, [1.5] * 3, seed=34)
    datas = [_deform(md, rng, 0.01) for md in datas]
    for m, md in zip(meshes, datas):
        m.vertices.copy_(torch.from_numpy(md.vertices).cuda())
    build_meshes(meshes, request=REQUEST_PREFER_UPDATE)
    assert all(m.stats().refits == 1 for m in meshes)
    _check(oracle_mod, _accel(meshes), datas, rays)
    # only two of the block's meshes: rebuilt, not refit
    datas[1] = _deform(datas[1], rng, 0.01)
    datas[3] = _deform(datas[3], rng, 0.01)
    for i in (1, 3):
        meshes[i].vertices.copy_(torch.from_numpy(datas[i].vertices).cuda())
    build_meshes([meshes[1], meshes[3]], request=REQUEST_PREFER_UPDATE)
    assert meshes[1].stats().refits == 0 and meshes[3].stats().refits == 0
    _check(oracle_mod, _accel(meshes), datas, rays)
    # no allow_update: PREFER_UPDATE rebuilds
    (plain,) = _device([datas[2]], allow_update=False)
    plain.build()
    plain.build(request=REQUEST_PREFER_UPDATE)
    assert plain.stats().refits == 0
    _check(oracle_mod, _accel([plain]), [datas[2]], rays)
