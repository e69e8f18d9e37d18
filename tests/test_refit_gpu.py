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


# ------------------------------------------------------------------ TLAS refit
# PREFER_UPDATE on an accel created with allow_update (src/backends/cuda/cuda_accel.cpp:261-320:
# update unless the instance count or an instance's primitive changed). The refit recomputes the
# instance boxes and records from the current transforms, masks and meshes; hit records must equal
# the oracle's on the new scene bit for bit.

def _check_scene(oracle_mod, acc, scene, rays, layouts=(0, 1)):
    import torch
    from luisacompute_gb300 import _capi
    from luisacompute_gb300.accel import hits_to_numpy, rays_to_device
    want = oracle_mod.OracleScene(scene).trace_closest(rays)
    for layout in layouts:
        got = hits_to_numpy(acc.trace_closest(rays_to_device(rays), layout=layout))
        torch.cuda.synchronize()
        assert np.array_equal(got.view(np.uint8), want.view(np.uint8)), f"layout {layout}"
    _capi.check(_capi.load().lcx_check_trace_errors(), "trace errors")
    return want


def _placements(rng, n, spread=1.5):
    return S.affine_rows(S.random_rotations(n, rng), rng.uniform(0.15, 0.4, n), rng.uniform(-spread, spread, (n, 3)))


def test_tlas_refit_moving_instances(lcx, oracle_mod):
    import torch
    from luisacompute_gb300.accel import REQUEST_PREFER_UPDATE, Accel, AccelOption, build_meshes
    rng = np.random.default_rng(11)
    datas = [S.displaced_mesh(int(n), rng) for n in (1_500, 6_000, 400)]
    meshes = build_meshes(_device(datas))
    n = 300
    inst_mesh = np.arange(n) % 3
    aff = _placements(rng, n)
    masks = np.full(n, 0xFF, np.uint32)
    acc = Accel(AccelOption(allow_update=True))
    acc.emplace_back_many([meshes[i] for i in inst_mesh], aff)
    acc.build()
    nodes = acc.stats().node_count
    rays = S.sphere_rays(80_000, [-2.0] * 3, [2.0] * 3, seed=41)
    _check_scene(oracle_mod, acc, S.Scene(datas, inst_mesh, aff, masks), rays)
    # move every instance a little, hide a few: refit twice
    for step in (1, 2):
        aff = aff.copy()
        aff[:, [3, 7, 11]] += rng.normal(0.0, 0.1, (n, 3)).astype(np.float32)
        for i in range(n):
            acc.set_transform_on_update(i, aff[i].reshape(3, 4))
        hidden = rng.choice(n, 20, replace=False)
        masks[:] = 0xFF
        masks[hidden] = 0
        for i in range(n):
            acc.set_visibility_on_update(i, int(masks[i]))
        acc.build(request=REQUEST_PREFER_UPDATE)
        st = acc.stats()
        assert st.refits == step and st.node_count == nodes
        _check_scene(oracle_mod, acc, S.Scene(datas, inst_mesh, aff, masks), rays)
    # the instances' meshes are refit: the TLAS refit takes their new boxes
    datas = [_deform(md, rng, 0.02, 1.3) for md in datas]
    for m, md in zip(meshes, datas):
        m.vertices.copy_(torch.from_numpy(md.vertices).cuda())
    build_meshes(meshes, request=REQUEST_PREFER_UPDATE)
    assert all(m.stats().refits == 1 for m in meshes)
    acc.build(request=REQUEST_PREFER_UPDATE)
    assert acc.stats().refits == 3
    _check_scene(oracle_mod, acc, S.Scene(datas, inst_mesh, aff, masks), rays)
    # an instance's primitive changed: rebuilt, as cuda_accel.cpp:184-185
    inst_mesh = inst_mesh.copy()
    inst_mesh[0] = 1
    acc.set_mesh_on_update(0, meshes[1])
    acc.build(request=REQUEST_PREFER_UPDATE)
    assert acc.stats().refits == 0
    _check_scene(oracle_mod, acc, S.Scene(datas, inst_mesh, aff, masks), rays)
    # a later PREFER_UPDATE refits again
    acc.build(request=REQUEST_PREFER_UPDATE)
    assert acc.stats().refits == 1
    # FORCE_BUILD and an accel without allow_update rebuild
    acc.build()
    assert acc.stats().refits == 0
    plain = Accel(AccelOption(allow_update=False))
    plain.emplace_back_many([meshes[i] for i in inst_mesh], aff, masks)
    plain.build()
    plain.build(request=REQUEST_PREFER_UPDATE)
    assert plain.stats().refits == 0
    _check_scene(oracle_mod, plain, S.Scene(datas, inst_mesh, aff, masks), rays, layouts=(0,))


def test_async_refit_reports_errors(lcx, oracle_mod):
    """With lcx_set_refit_sync(0) a refit only enqueues kernels; a bad index is reported by the
    next lcx_check_trace_errors, and the flag is cleared after the report."""
    import torch
    from luisacompute_gb300 import _capi
    from luisacompute_gb300.accel import REQUEST_PREFER_UPDATE, set_refit_sync
    rng = np.random.default_rng(12)
    md = S.displaced_mesh(3_000, rng)
    (mesh,) = _device([md])
    mesh.build()
    set_refit_sync(False)
    try:
        md = _deform(md, rng, 0.01)
        mesh.vertices.copy_(torch.from_numpy(md.vertices).cuda())
        mesh.build(request=REQUEST_PREFER_UPDATE)
        assert mesh.stats().refits == 1
        assert lcx.lcx_check_trace_errors() == 0
        _check(oracle_mod, _accel([mesh]), [md], S.sphere_rays(30_000, [-1.3] * 3, [1.3] * 3, seed=42))
        # one index past the vertex count: the refit kernel flags it (and skips the read)
        bad = md.triangles.astype(np.int32).copy()
        bad[7, 1] = md.vertices.shape[0]
        mesh.triangles.copy_(torch.from_numpy(bad).cuda())
        mesh.build(request=REQUEST_PREFER_UPDATE)  # returns at once
        assert lcx.lcx_check_trace_errors() == _capi.LCX_ERR_INVALID_ARG
        assert lcx.lcx_check_trace_errors() == 0
    finally:
        set_refit_sync(True)


@pytest.mark.filterwarnings("ignore:The CUDA Graph is empty")  # the refused captures end empty
def test_refit_frame_in_cuda_graph(lcx, oracle_mod):
    """An animation frame captured once in a CUDA graph and replayed: a torch kernel writes each
    mesh's new vertices, the BLASes and the TLAS are refit and rays are traced. Between replays
    the host moves instances with update_instance_buffer_only; every replay must match the oracle
    on the frame's vertices (read back) and transforms. Calls that cannot be captured (a build,
    synchronous refit) fail with an error instead of breaking the capture silently."""
    import torch
    from luisacompute_gb300 import _capi
    from luisacompute_gb300.accel import (REQUEST_PREFER_UPDATE, Accel, AccelOption, build_meshes, hits_to_numpy,
                                          rays_to_device, set_refit_sync)
    rng = np.random.default_rng(13)
    datas = [S.displaced_mesh(int(n), rng) for n in (2_000, 7_000, 600)]
    meshes = build_meshes(_device(datas))
    n = 120
    inst_mesh = np.arange(n) % 3
    aff = _placements(rng, n)
    acc = Accel(AccelOption(allow_update=True))
    acc.emplace_back_many([meshes[i] for i in inst_mesh], aff)
    acc.build()
    rays = S.sphere_rays(50_000, [-2.0] * 3, [2.0] * 3, seed=43)
    d_rays = rays_to_device(rays)
    out = torch.empty((rays.shape[0], 6), dtype=torch.int32, device="cuda")
    base = [m.vertices.clone() for m in meshes]
    disp = []
    for md in datas:
        d = np.zeros_like(md.vertices)
        d[:, :3] = rng.normal(0.0, 0.02, (md.vertices.shape[0], 3))
        disp.append(torch.from_numpy(d).cuda())
    phase = torch.zeros(1, device="cuda")
    old_bits, old_min = ctypes_pair(lcx.lcx_get_trace_reorder)
    _capi.check(lcx.lcx_set_trace_reorder(0, old_min), "reorder off")
    set_refit_sync(False)
    try:
        # a first refit outside the capture puts the segment table on the device
        build_meshes(meshes, request=REQUEST_PREFER_UPDATE)
        acc.build(request=REQUEST_PREFER_UPDATE)
        torch.cuda.synchronize()
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            for m, b, d in zip(meshes, base, disp):
                m.vertices.copy_(b + d * phase)
            build_meshes(meshes, request=REQUEST_PREFER_UPDATE)
            acc.build(request=REQUEST_PREFER_UPDATE)
            acc.trace_closest(d_rays, out=out)
        for frame, p in enumerate((0.0, 1.0, -2.5, 4.0)):
            if frame >= 2:  # move a third of the instances between replays
                aff = aff.copy()
                moved = rng.choice(n, n // 3, replace=False)
                aff[moved, 3] += rng.normal(0.0, 0.2, moved.size).astype(np.float32)
                for i in moved:
                    acc.set_transform_on_update(int(i), aff[i].reshape(3, 4))
                acc.build(update_instance_buffer_only=True)
            phase.fill_(p)
            g.replay()
            torch.cuda.synchronize()
            frame_datas = [S.MeshData(m.vertices.cpu().numpy(), md.triangles) for m, md in zip(meshes, datas)]
            want = oracle_mod.OracleScene(S.Scene(frame_datas, inst_mesh, aff, np.full(n, 0xFF, np.uint32))) \
                .trace_closest(rays)
            got = hits_to_numpy(out)
            assert np.array_equal(got.view(np.uint8), want.view(np.uint8)), f"frame {frame}"
            assert (got["inst"] != 0xFFFFFFFF).mean() > 0.05
            _capi.check(lcx.lcx_check_trace_errors(), "trace / refit errors")
        # what cannot be captured is refused before any work is enqueued
        for call in (lambda: acc.build(), lambda: (set_refit_sync(True), build_meshes(
                meshes, request=REQUEST_PREFER_UPDATE))):
            g2 = torch.cuda.CUDAGraph()
            with pytest.raises(_capi.LcxError):
                with torch.cuda.graph(g2):
                    call()
            set_refit_sync(False)
    finally:
        set_refit_sync(True)
        _capi.check(lcx.lcx_set_trace_reorder(old_bits, old_min), "reorder restore")


def ctypes_pair(fn):
    import ctypes
    a, b = ctypes.c_uint32(), ctypes.c_uint32()
    _ = fn(ctypes.byref(a), ctypes.byref(b))
    return a.value, b.value


def test_reserved_batch_rebuild_in_cuda_graph(lcx, oracle_mod):
    """lcx_mesh_build_batch_reserve, then full rebuilds of the batch in place (no host sync): first
    uncaptured after the vertices moved, then captured in a CUDA graph with a torch kernel that
    writes the vertices and a TLAS refit, replayed over several frames.  A rebuild gives a new
    topology for the new vertices; every frame must match the oracle on that frame's vertices."""
    import torch
    from luisacompute_gb300 import _capi
    from luisacompute_gb300.accel import (REQUEST_PREFER_UPDATE, Accel, AccelOption, build_meshes, hits_to_numpy,
                                          rays_to_device, reserve_meshes)
    rng = np.random.default_rng(61)
    datas = [S.displaced_mesh(int(n), rng) for n in (500, 4_000, 20_000, 1_200)]
    meshes = reserve_meshes(_device(datas, allow_update=False))
    n = len(meshes)
    aff = _placements(rng, n, spread=1.0)
    acc = Accel(AccelOption(allow_update=True))
    acc.emplace_back_many(meshes, aff)
    acc.build()
    rays = S.sphere_rays(50_000, [-2.0] * 3, [2.0] * 3, seed=62)
    masks = np.full(n, 0xFF, np.uint32)
    _check_scene(oracle_mod, acc, S.Scene(datas, np.arange(n), aff, masks), rays)
    nodes_before = [int(m.stats().node_count) for m in meshes]
    # an uncaptured in-place rebuild after large deformations
    datas = [_deform(md, rng, 0.08, 1.4) for md in datas]
    for m, md in zip(meshes, datas):
        m.vertices.copy_(torch.from_numpy(md.vertices).cuda())
    build_meshes(meshes)
    acc.build(request=REQUEST_PREFER_UPDATE)
    _check_scene(oracle_mod, acc, S.Scene(datas, np.arange(n), aff, masks), rays)
    assert [int(m.stats().node_count) for m in meshes] == nodes_before  # the reserving build's figures
    # captured: vertices from a device phase, rebuild, TLAS refit, trace
    base = [m.vertices.clone() for m in meshes]
    disp = []
    for md in datas:
        d = np.zeros_like(md.vertices)
        d[:, :3] = rng.normal(0.0, 0.05, (md.vertices.shape[0], 3))
        disp.append(torch.from_numpy(d).cuda())
    phase = torch.zeros(1, device="cuda")
    d_rays = rays_to_device(rays)
    out = torch.empty((rays.shape[0], 6), dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        for m, b, d in zip(meshes, base, disp):
            m.vertices.copy_(b + d * phase)
        build_meshes(meshes)
        acc.build(request=REQUEST_PREFER_UPDATE)
        acc.trace_closest(d_rays, out=out)
    for p in (0.0, 1.0, -2.0, 3.0):
        phase.fill_(p)
        g.replay()
        torch.cuda.synchronize()
        frame = [S.MeshData(m.vertices.cpu().numpy(), md.triangles) for m, md in zip(meshes, datas)]
        want = oracle_mod.OracleScene(S.Scene(frame, np.arange(n), aff, masks)).trace_closest(rays)
        assert np.array_equal(hits_to_numpy(out).view(np.uint8), want.view(np.uint8)), p
        _capi.check(lcx.lcx_check_trace_errors(), "rebuild / trace errors")
    # other buffers: no longer the reserved batch, so an ordinary build
    moved = [m.vertices.clone() for m in meshes]
    for m, v in zip(meshes, moved):
        m.vertices = v
    build_meshes(meshes)
    acc.build()
    frame = [S.MeshData(v.cpu().numpy(), md.triangles) for v, md in zip(moved, datas)]
    _check_scene(oracle_mod, acc, S.Scene(frame, np.arange(n), aff, masks), rays, layouts=(1,))


def test_first_build_in_cuda_graph(lcx, oracle_mod):
    """lcx_mesh_reserve_batch allocates the room of a reserved batch and builds nothing; the
    batch's first build is then captured in a CUDA graph (no host sync, no allocation of its own)
    and replayed.  The TLAS built afterwards traces the oracle's records; a replay after the
    vertices moved rebuilds the trees in place, and a TLAS rebuild traces the new vertices."""
    import torch
    from luisacompute_gb300 import _capi
    from luisacompute_gb300.accel import Accel, build_meshes, reserve_meshes
    rng = np.random.default_rng(71)
    datas = [S.displaced_mesh(int(n), rng) for n in (700, 9_000, 30_000, 2_500, 64)]
    meshes = reserve_meshes(_device(datas, allow_update=False), build=False)
    assert all(int(m.stats().node_count) == 0 for m in meshes)  # reserved, not built
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        build_meshes(meshes)  # the first build of these meshes, inside the capture
    g.replay()
    torch.cuda.synchronize()
    _capi.check(lcx.lcx_check_trace_errors(), "in-graph build errors")
    n = len(meshes)
    aff = _placements(rng, n, spread=1.0)
    masks = np.full(n, 0xFF, np.uint32)
    acc = Accel()
    acc.emplace_back_many(meshes, aff)
    acc.build()
    rays = S.sphere_rays(40_000, [-2.0] * 3, [2.0] * 3, seed=72)
    _check_scene(oracle_mod, acc, S.Scene(datas, np.arange(n), aff, masks), rays)
    # move the vertices, replay the same graph, rebuild the TLAS: the new geometry
    datas = [_deform(md, rng, 0.08, 1.3) for md in datas]
    for m, md in zip(meshes, datas):
        m.vertices.copy_(torch.from_numpy(md.vertices).cuda())
    g.replay()
    acc.build()
    _check_scene(oracle_mod, acc, S.Scene(datas, np.arange(n), aff, masks), rays)
