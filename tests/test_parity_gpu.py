"""GPU parity: the sm_103a kernels (through the C ABI) against the CPU oracle.

The closest-hit rule keeps (t, inst, prim) minimal, and the GPU repeats the oracle's FP32
operation sequence for the instance transform and the watertight test, so the expected
result is bit-exact equality of every TriangleHit record; any disagreement is reported
with the FP64 adjudicator's classification.
"""
import numpy as np
import pytest

from luisacompute_gb300 import scenes as S

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch_cuda():
    import torch
    assert torch.cuda.is_available()
    return torch


def gpu_scene(scene, option=None):
    from luisacompute_gb300.accel import accel_from_scene
    return accel_from_scene(scene, option=option)


def no_kernel_errors():
    from luisacompute_gb300 import _capi
    _capi.check(_capi.load().lcx_check_trace_errors(), "lcx_check_trace_errors")


def trace(acc, rays, layout, mask=0xFF):
    from luisacompute_gb300.accel import hits_to_numpy, rays_to_device
    import torch
    d = rays_to_device(rays)
    h = acc.trace_closest(d, mask=mask, layout=layout)
    torch.cuda.synchronize()
    no_kernel_errors()
    return hits_to_numpy(h)


def trace_any(acc, rays, layout, mask=0xFF):
    from luisacompute_gb300.accel import rays_to_device
    import torch
    d = rays_to_device(rays)
    o = acc.trace_any(d, mask=mask, layout=layout)
    torch.cuda.synchronize()
    no_kernel_errors()
    return o.cpu().numpy()


def assert_bit_exact(oracle_mod, osc, rays, got, want):
    if np.array_equal(got.view(np.uint8), want.view(np.uint8)):
        return
    rep = oracle_mod.adjudicate(osc, rays, got, want)
    same_id = (got["inst"] == want["inst"]) & (got["prim"] == want["prim"])
    field_diff = int((~np.all(got.view(np.uint32).reshape(-1, 6)[:, :5] == want.view(np.uint32).reshape(-1, 6)[:, :5],
                              axis=1) & same_id).sum())
    raise AssertionError(f"GPU != oracle: {rep['disagree']} id mismatches (near-tie {rep['near_tie']}, grazing "
                         f"{rep['grazing']}, unexplained {len(rep['unexplained'])}), {field_diff} field mismatches")


@pytest.mark.parametrize("layout", [0, 1])
def test_icosphere_primary_rays(torch_cuda, lcx, oracle_mod, layout):
    """Icosphere subdivided 6 times (81,920 triangles), 1024x1024 jittered pinhole rays."""
    scene = S.icosphere_scene(6)
    rays = S.primary_rays_icosphere(1024, 1024)
    osc = oracle_mod.OracleScene(scene)
    want = osc.trace_closest(rays)
    acc, _ = gpu_scene(scene)
    got = trace(acc, rays, layout)
    assert_bit_exact(oracle_mod, osc, rays, got, want)
    assert 0.2 < (got["inst"] != S.MISS).mean() < 0.6


def small_terrain():
    return S.terrain_scene(n=128, sphere_count=64, sphere_subdiv=3)


@pytest.mark.parametrize("layout", [0, 1])
def test_terrain_incoherent(torch_cuda, lcx, oracle_mod, layout):
    scene = small_terrain()
    rays = S.terrain_rays(scene, 200_000, seed=4)
    osc = oracle_mod.OracleScene(scene)
    want = osc.trace_closest(rays)
    acc, _ = gpu_scene(scene)
    got = trace(acc, rays, layout)
    assert_bit_exact(oracle_mod, osc, rays, got, want)
    assert (got["inst"] > 0).sum() > 100  # some sphere instances are hit


@pytest.mark.parametrize("layout", [0, 1])
def test_terrain_shadow_any(torch_cuda, lcx, oracle_mod, layout):
    scene = small_terrain()
    rays = S.terrain_shadow_rays(scene, 200_000, seed=5)
    osc = oracle_mod.OracleScene(scene)
    want = osc.trace_any(rays)
    acc, _ = gpu_scene(scene)
    got = trace_any(acc, rays, layout)
    assert np.array_equal(got, want)
    assert 0.05 < want.mean() < 0.95


@pytest.fixture(scope="module")
def full_terrain(oracle_mod):
    """The headline scene at full size: the 1024x1024 heightfield (2,093,058 triangles) and 256
    instances of a 20,480-triangle icosphere, with its oracle."""
    scene = S.terrain_scene()
    return scene, oracle_mod.OracleScene(scene)


@pytest.mark.parametrize("layout", [1, 0])
def test_full_terrain_closest_and_any(torch_cuda, lcx, oracle_mod, full_terrain, layout):
    """The full headline scene, 2^20 incoherent rays of the headline distribution (closest hit)
    and 2^20 shadow rays (any hit), both node layouts, bit for bit against the oracle."""
    scene, osc = full_terrain
    acc, _ = gpu_scene(scene)
    rays = S.terrain_rays(scene, 1 << 20, seed=4)
    got = trace(acc, rays, layout)
    assert_bit_exact(oracle_mod, osc, rays, got, osc.trace_closest(rays))
    assert (got["inst"] > 0).sum() > 1000  # the instanced spheres are hit
    shadow = S.terrain_shadow_rays(scene, 1 << 20, seed=5)
    occ = trace_any(acc, shadow, layout)
    want = osc.trace_any(shadow)
    assert np.array_equal(occ, want)
    assert 0.05 < want.mean() < 0.95


def test_masks(torch_cuda, lcx, oracle_mod):
    scene = small_terrain()
    scene.inst_mask = np.array([0x01] + [0x02, 0x04] * 32, np.uint32)
    rays = S.terrain_rays(scene, 50_000, seed=7)
    osc = oracle_mod.OracleScene(scene)
    acc, _ = gpu_scene(scene)
    for mask in (0xFF, 0x01, 0x02, 0x06, 0x00):
        got = trace(acc, rays, 1, mask)
        want = osc.trace_closest(rays, mask)
        assert_bit_exact(oracle_mod, osc, rays, got, want)
        if mask == 0:
            assert np.all(got["inst"] == S.MISS)
        occ = trace_any(acc, rays, 1, mask)
        assert np.array_equal(occ.astype(bool), want["inst"] != S.MISS)


def test_layouts_identical_and_counts(torch_cuda, lcx):
    import torch
    scene = small_terrain()
    rays = S.terrain_rays(scene, 100_000, seed=9)
    from luisacompute_gb300.accel import rays_to_device, hits_to_numpy
    acc, _ = gpu_scene(scene)
    d = rays_to_device(rays)
    hq = hits_to_numpy(acc.trace_closest(d, layout=1))
    hf = hits_to_numpy(acc.trace_closest(d, layout=0))
    assert np.array_equal(hq.view(np.uint8), hf.view(np.uint8))
    counts = torch.zeros((rays.shape[0], 3), dtype=torch.int32, device="cuda")
    hc = hits_to_numpy(acc.trace_closest(d, layout=1, counts=counts))
    assert np.array_equal(hq.view(np.uint8), hc.view(np.uint8))
    c = counts.cpu().numpy()
    assert c[:, 0].min() >= 1 and c[:, 1].mean() > 1


def test_miss_record_and_t_range(torch_cuda, lcx, oracle_mod):
    scene = S.icosphere_scene(3)
    acc, _ = gpu_scene(scene)
    rays = np.zeros(6, S.RAY_DTYPE)
    rays["o"] = [[0, 0, 3], [0, 0, 3], [0, 0, 3], [0, 0, 3], [5, 5, 5], [0, 0, 0]]
    rays["d"] = [[0, 0, -1], [0, 0, -1], [0, 0, -1], [0, 0, 1], [1, 0, 0], [0, 1, 0]]
    rays["tmin"] = [0, 0, 2.5, 0, 0, 0]
    rays["tmax"] = [1e30, 1.5, 1e30, 1e30, 7.0, 1e30]
    got = trace(acc, rays, 1)
    osc = oracle_mod.OracleScene(scene)
    want = osc.trace_closest(rays)
    assert np.array_equal(got.view(np.uint8), want.view(np.uint8))
    assert got["inst"][0] == 0 and abs(got["t"][0] - 2.0) < 2e-2       # front face
    assert got["inst"][1] == S.MISS and got["t"][1] == np.float32(1.5)  # t_max clips
    assert got["inst"][2] == 0 and abs(got["t"][2] - 4.0) < 2e-2       # t_min skips the front face
    assert got["inst"][3] == S.MISS and got["inst"][4] == S.MISS
    assert got["inst"][5] == 0 and abs(got["t"][5] - 1.0) < 2e-2       # origin inside, back face hit


def test_edge_cases(torch_cuda, lcx, oracle_mod):
    """Empty mesh, single triangle, degenerate triangles, scaled/rotated instances."""
    import torch
    from luisacompute_gb300.accel import Accel, mesh_from_data
    empty = S.MeshData(np.zeros((3, 4), np.float32), np.zeros((0, 3), np.uint32))
    single = S.MeshData(np.array([[0, 0, 0, 0], [1, 0, 0, 0], [0, 1, 0, 0]], np.float32),
                        np.array([[0, 1, 2]], np.uint32))
    degen = S.MeshData(np.array([[0, 0, 0, 0], [1, 0, 0, 0], [2, 0, 0, 0], [0, 1, 0, 0]], np.float32),
                       np.array([[0, 1, 2], [0, 0, 0], [0, 1, 3]], np.uint32))
    rng = np.random.default_rng(11)
    aff = np.concatenate([S.IDENTITY[None],
                          S.affine_rows(S.random_rotations(3, rng), np.array([0.5, 2.0, 1e-3]),
                                        rng.uniform(-1, 1, (3, 3)))])
    scene = S.Scene([empty, single, degen], np.array([0, 1, 2, 1]), aff, np.full(4, 0xFF, np.uint32))
    osc = oracle_mod.OracleScene(scene)
    meshes = [mesh_from_data(m).build() for m in scene.meshes]
    acc = Accel()
    for i in range(4):
        acc.emplace_back(meshes[scene.inst_mesh[i]], scene.inst_affine[i].reshape(3, 4))
    acc.build()
    rays = S.sphere_rays(100_000, [-2, -2, -2], [2, 2, 2], seed=12)
    # aim half the rays at the instances' triangles
    tgt = rng.uniform(-1, 1, (50_000, 3)).astype(np.float32)
    d = tgt - rays["o"][:50_000]
    rays["d"][:50_000] = d / np.linalg.norm(d, axis=1, keepdims=True)
    got = trace(acc, rays, 1)
    want = osc.trace_closest(rays)
    assert_bit_exact(oracle_mod, osc, rays, got, want)
    assert np.all(got["inst"] != 0)  # the empty mesh is never hit
    torch.cuda.synchronize()


def test_errors(torch_cuda, lcx):
    import torch
    from luisacompute_gb300 import LcxError
    from luisacompute_gb300.accel import Accel, Mesh, mesh_from_data
    from luisacompute_gb300._capi import LCX_ERR_INVALID_ARG, LCX_ERR_NOT_BUILT
    acc = Accel()
    with pytest.raises(LcxError) as e:
        acc.build()  # no instances (src/runtime/rtx/accel.cpp:72-73)
    assert e.value.code == LCX_ERR_INVALID_ARG
    rays = torch.zeros((4, 8), dtype=torch.float32, device="cuda")
    m = mesh_from_data(S.icosphere(1))
    acc.emplace_back(m)
    with pytest.raises(LcxError) as e:
        acc.build()  # mesh not built (accel.rs:356-358)
    assert e.value.code == LCX_ERR_NOT_BUILT
    m.build()
    acc.emplace_back(m)
    acc.build()
    acc.trace_closest(rays)
    # rebuilt mesh invalidates the TLAS until the accel is rebuilt
    m.build()
    with pytest.raises(LcxError) as e:
        acc.trace_closest(rays)
    assert e.value.code == LCX_ERR_NOT_BUILT
    acc.build()
    acc.trace_closest(rays)
    # vertex stride must be a multiple of 16 (src/runtime/rtx/mesh.cpp:44-45)
    v = torch.zeros((12, 3), dtype=torch.float32, device="cuda")
    t = torch.zeros((4, 3), dtype=torch.int32, device="cuda")
    with pytest.raises(LcxError) as e:
        Mesh(v, t).build()
    assert e.value.code == LCX_ERR_INVALID_ARG
    # triangle index out of range
    v4 = torch.zeros((3, 4), dtype=torch.float32, device="cuda")
    bad = torch.tensor([[0, 1, 7]], dtype=torch.int32, device="cuda")
    with pytest.raises(LcxError) as e:
        Mesh(v4, bad).build()
    assert e.value.code == LCX_ERR_INVALID_ARG
    torch.cuda.synchronize()


def test_instance_updates(torch_cuda, lcx, oracle_mod):
    """set_transform / set_visibility / update_instance_buffer_only / pop_back."""
    from luisacompute_gb300.accel import Accel, mesh_from_data
    sph = S.icosphere(3)
    m = mesh_from_data(sph).build()
    acc = Accel()
    acc.emplace_back(m, np.eye(4))
    acc.emplace_back(m, np.array([[1, 0, 0, 3], [0, 1, 0, 0], [0, 0, 1, 0]], np.float32))
    acc.build()
    rays = np.zeros(2, S.RAY_DTYPE)
    rays["o"] = [[0, 0, 5], [3, 0, 5]]
    rays["d"] = [[0, 0, -1], [0, 0, -1]]
    rays["tmax"] = 1e30
    h = trace(acc, rays, 1)
    assert list(h["inst"]) == [0, 1]
    acc.set_visibility_on_update(1, 0)
    acc.build(update_instance_buffer_only=True)
    assert list(trace(acc, rays, 1)["inst"]) == [0, 1]  # TLAS not rebuilt yet
    acc.build()
    assert list(trace(acc, rays, 1)["inst"]) == [0, S.MISS]
    acc.set_visibility_on_update(1, 0xFF)
    acc.set_transform_on_update(0, np.array([[1, 0, 0, 0], [0, 1, 0, 0], [0, 0, 1, -10]], np.float32))
    acc.build()
    h = trace(acc, rays, 1)
    assert h["inst"][1] == 1 and h["inst"][0] == 0 and abs(h["t"][0] - 14.0) < 1e-2
    acc.pop_back()
    acc.build()
    assert list(trace(acc, rays, 1)["inst"]) == [0, S.MISS]


@pytest.mark.parametrize("layout", [0, 1])
def test_axis_aligned_exact_ties(torch_cuda, lcx, oracle_mod, layout):
    """Rays along the axes through the vertices and edges of an integer grid (every hit is a
    shared edge or vertex; the smallest (inst, prim) among equal t must win), plus rays lying
    in the grid plane."""
    n = 9
    xs = np.arange(n, dtype=np.float32) - 4.0
    X, Z = np.meshgrid(xs, xs, indexing="xy")
    v = np.zeros((n * n, 4), np.float32)
    v[:, 0], v[:, 2] = X.ravel(), Z.ravel()
    idx = np.arange(n * n).reshape(n, n)
    a, b, c, d = idx[:-1, :-1].ravel(), idx[:-1, 1:].ravel(), idx[1:, :-1].ravel(), idx[1:, 1:].ravel()
    tris = np.concatenate([np.stack([a, c, b], 1), np.stack([b, c, d], 1)]).astype(np.uint32)
    grid = S.MeshData(v, tris)
    aff = np.stack([S.IDENTITY, S.IDENTITY.copy()])
    aff[1, 7] = 2.0  # a second copy 2 units above
    scene = S.Scene([grid], np.array([0, 0]), aff, np.full(2, 0xFF, np.uint32))
    g = np.arange(-8, 9, dtype=np.float32) * 0.5
    px, pz = np.meshgrid(g, g)
    m = px.size
    rays = np.zeros(3 * m, S.RAY_DTYPE)
    rays["o"][:m, 0], rays["o"][:m, 1], rays["o"][:m, 2] = px.ravel(), 5.0, pz.ravel()
    rays["d"][:m] = [0, -1, 0]
    rays["o"][m:2 * m, 0], rays["o"][m:2 * m, 1], rays["o"][m:2 * m, 2] = px.ravel(), -5.0, pz.ravel()
    rays["d"][m:2 * m] = [0, 1, 0]
    rays["o"][2 * m:, 0], rays["o"][2 * m:, 2] = -6.0, pz.ravel()
    rays["d"][2 * m:] = [1, 0, 0]
    rays["tmax"] = 1e30
    osc = oracle_mod.OracleScene(scene)
    want = osc.trace_closest(rays)
    assert np.array_equal(want.view(np.uint8), osc.brute_closest(rays).view(np.uint8))
    acc, _ = gpu_scene(scene)
    got = trace(acc, rays, layout)
    assert_bit_exact(oracle_mod, osc, rays, got, want)
    assert (got["inst"][:2 * m] != S.MISS).sum() >= 2 * 15 * 15


@pytest.mark.parametrize("layout", [0, 1])
def test_identity_instances(torch_cuda, lcx, oracle_mod, layout):
    """Identity and translated instances of a flat grid whose zero coordinates are partly -0 (the
    same geometry, signed zeros), against rays with +0 / -0 direction components and with origins
    on the grid's plane (signed zeros through the instance transform, the slab reciprocals and the
    watertight test): the oracle's records bit for bit.  (A grid folded by moving vertices onto
    zero coordinates is not a fit: its overlapping coplanar triangles meet a ray at t values that
    differ by rounding, and the oracle's own BVH then disagrees with its brute-force answer.)"""
    rng = np.random.default_rng(71)
    grid = S.grid_mesh(25, 25)
    v = grid.vertices.copy()
    v[::3, 1] = -0.0                                          # y = 0 everywhere: -0 on a third
    zx = np.nonzero(v[:, 0] == 0.0)[0]
    v[zx[::2], 0] = -0.0                                      # half of the x = 0 column
    zz = np.nonzero(v[:, 2] == 0.0)[0]
    v[zz[1::2], 2] = -0.0                                     # half of the z = 0 row
    mesh = S.MeshData(v, grid.triangles)
    aff = np.stack([S.IDENTITY, S.IDENTITY.copy()])
    aff[1, 3] = 3.0  # a translated copy
    scene = S.Scene([mesh, S.icosphere(2)], np.array([0, 0, 1]), np.concatenate([aff, S.IDENTITY[None]]),
                    np.full(3, 0xFF, np.uint32))
    lo, hi = scene.bounds()
    rays = S.sphere_rays(60_000, lo, hi, seed=72)
    k = rays.shape[0] // 4
    rays["d"][:k, 0] = 0.0                       # +0 direction components
    rays["d"][k:2 * k, 2] = -0.0                 # -0 direction components
    rays["o"][2 * k:3 * k, 1] = rng.choice([0.0, -0.0], k).astype(np.float32)  # origins on the plane
    osc = oracle_mod.OracleScene(scene)
    want = osc.trace_closest(rays)
    assert np.array_equal(want.view(np.uint8), osc.brute_closest(rays).view(np.uint8))
    acc, _ = gpu_scene(scene)
    got = trace(acc, rays, layout)
    assert_bit_exact(oracle_mod, osc, rays, got, want)
    assert (want["inst"] != S.MISS).mean() > 0.3
    no_kernel_errors()


@pytest.mark.parametrize("refill,postpone,mode", [(1, 0, 0), (8, 8, 0), (16, 12, 0), (32, 32, 0), (4, 20, 0),
                                                  (4, 0, 1), (16, 0, 1), (1, 8, 1),
                                                  (4, 0, 2), (1, 1, 2), (8, 16, 2), (32, 32, 2), (2, 5, 2),
                                                  (4, 0, 3)])
def test_tuning_does_not_change_results(torch_cuda, lcx, oracle_mod, refill, postpone, mode):
    import ctypes
    from luisacompute_gb300 import _capi
    lib = _capi.load()
    scene = small_terrain()
    rays = np.concatenate([S.terrain_rays(scene, 100_000, seed=13), S.terrain_shadow_rays(scene, 50_000, seed=14)])
    osc = oracle_mod.OracleScene(scene)
    want = osc.trace_closest(rays)
    want_any = osc.trace_any(rays)
    acc, _ = gpu_scene(scene)
    old = [ctypes.c_uint32(0) for _ in range(3)]
    _capi.check(lib.lcx_get_trace_tuning(*old), "get")
    try:
        _capi.check(lib.lcx_set_trace_tuning(refill, postpone, mode), "set")
        for layout in (0, 1):
            got = trace(acc, rays, layout)
            assert np.array_equal(got.view(np.uint8), want.view(np.uint8))
            assert np.array_equal(trace_any(acc, rays, layout), want_any)
    finally:
        _capi.check(lib.lcx_set_trace_tuning(old[0].value, old[1].value, old[2].value), "set")


@pytest.mark.parametrize("bits", [1, 6, 9])
def test_ray_reorder_does_not_change_results(torch_cuda, lcx, oracle_mod, bits):
    """Reordered calls (sorted by octant and origin cell) give the oracle's records bit for bit,
    for closest, any, both layouts, the counting kernel and a call below min_rays."""
    import ctypes
    from luisacompute_gb300 import _capi
    from luisacompute_gb300.accel import hits_to_numpy, rays_to_device
    lib = _capi.load()
    scene = small_terrain()
    rays = np.concatenate([S.terrain_rays(scene, 100_000, seed=15), S.terrain_shadow_rays(scene, 50_000, seed=16)])
    osc = oracle_mod.OracleScene(scene)
    want = osc.trace_closest(rays)
    want_any = osc.trace_any(rays)
    acc, _ = gpu_scene(scene)
    tune = [ctypes.c_uint32(0) for _ in range(3)]
    _capi.check(lib.lcx_get_trace_tuning(*tune), "get")

    def counts_mode0():
        # loop mode 0: a ray's walk does not depend on its neighbours (in mode 2 the queued
        # triangle tests, and so the best t that culls nodes, depend on the warp's other rays)
        _capi.check(lib.lcx_set_trace_tuning(tune[0].value, 0, 0), "set")
        try:
            c = torch_cuda.zeros((rays.shape[0], 3), dtype=torch_cuda.int32, device="cuda")
            acc.trace_closest(rays_to_device(rays), layout=1, counts=c)
            return c
        finally:
            _capi.check(lib.lcx_set_trace_tuning(tune[0].value, tune[1].value, tune[2].value), "set")

    plain_counts = counts_mode0()
    old = [ctypes.c_uint32(0) for _ in range(2)]
    _capi.check(lib.lcx_get_trace_reorder(*old), "get")
    try:
        _capi.check(lib.lcx_set_trace_reorder(bits, 0), "set")
        for layout in (0, 1):
            got = trace(acc, rays, layout)
            assert np.array_equal(got.view(np.uint8), want.view(np.uint8))
            assert np.array_equal(trace_any(acc, rays, layout), want_any)
        assert torch_cuda.equal(counts_mode0(), plain_counts)
        # the default loop structure's counting build gives the oracle's records
        counts = torch_cuda.zeros_like(plain_counts)
        got = hits_to_numpy(acc.trace_closest(rays_to_device(rays), layout=1, counts=counts))
        assert np.array_equal(got.view(np.uint8), want.view(np.uint8))
        assert counts[:, 0].min() >= 1
        _capi.check(lib.lcx_set_trace_reorder(bits, rays.shape[0] + 1), "set")  # below min_rays: not reordered
        assert np.array_equal(trace(acc, rays, 1).view(np.uint8), want.view(np.uint8))
        assert lib.lcx_set_trace_reorder(10, 0) == _capi.LCX_ERR_INVALID_ARG
    finally:
        _capi.check(lib.lcx_set_trace_reorder(old[0].value, old[1].value), "set")
    no_kernel_errors()


@pytest.mark.parametrize("chunk,access", [(1 << 14, 1), (1 << 20, 1), (1 << 20, 0), (1 << 20, 2), (1 << 20, 3)])
def test_host_buffer_traces(torch_cuda, lcx, oracle_mod, chunk, access):
    """lcx_trace_closest_host / lcx_trace_any_host (rays and results in host memory): the oracle's
    records bit for bit, for pinned and pageable buffers, both layouts, on a side stream, in every
    host access mode: staged (chunked through device staging with copies overlapped; a ray count
    that is not a multiple of the chunk, with 2^14 13 chunks through the 4-slot ring), direct (the
    kernel reads and writes the pinned host buffers itself), auto (direct at this size) and streamed
    (pinned quantised-node calls streamed, the others staged); the empty call is a no-op."""
    from luisacompute_gb300 import _capi
    lib = _capi.load()
    _capi.check(lib.lcx_set_host_access(access), "host access")
    scene = small_terrain()
    rays = np.concatenate([S.terrain_rays(scene, 150_000, seed=17), S.terrain_shadow_rays(scene, 50_003, seed=18)])
    osc = oracle_mod.OracleScene(scene)
    want = osc.trace_closest(rays)
    want_any = osc.trace_any(rays)
    acc, _ = gpu_scene(scene)
    _capi.check(lib.lcx_set_host_chunk(chunk), "chunk")
    try:
        side = torch_cuda.cuda.Stream()
        for layout in (0, 1):
            # pinned torch tensors
            h_rays = torch_cuda.from_numpy(rays.view(np.float32).reshape(-1, 8)).pin_memory()
            h_hits = torch_cuda.full((rays.shape[0], 6), -7, dtype=torch_cuda.int32).pin_memory()
            h_occ = torch_cuda.full((rays.shape[0],), 9, dtype=torch_cuda.uint8).pin_memory()
            acc.trace_closest_host(h_rays, h_hits, layout=layout, stream=side)
            acc.trace_any_host(h_rays, h_occ, layout=layout, stream=side)
            side.synchronize()
            got = h_hits.numpy().view(want.dtype).reshape(-1)
            assert_bit_exact(oracle_mod, osc, rays, got, want)
            assert np.array_equal(h_occ.numpy(), want_any)
            # pageable numpy arrays on the current stream
            got2 = np.zeros_like(want)
            occ2 = np.zeros(rays.shape[0], np.uint8)
            acc.trace_closest_host(np.ascontiguousarray(rays), got2, layout=layout)
            acc.trace_any_host(np.ascontiguousarray(rays), occ2, layout=layout)
            torch_cuda.cuda.synchronize()
            assert np.array_equal(got2.view(np.uint8), want.view(np.uint8))
            assert np.array_equal(occ2, want_any)
        # pinned buffers at odd offsets: the direct path steps aside for the staged one
        raw_rays = torch_cuda.empty(rays.nbytes + 8, dtype=torch_cuda.uint8).pin_memory()
        raw_rays[8:] = torch_cuda.from_numpy(rays.view(np.uint8).reshape(-1))
        raw_hits = torch_cuda.zeros(want.nbytes + 4, dtype=torch_cuda.uint8).pin_memory()
        _capi.check(lib.lcx_trace_closest_host(acc.handle, raw_rays.data_ptr() + 8, rays.shape[0], 0xFF,
                                               raw_hits.data_ptr() + 4, 1, None), "odd offsets")
        torch_cuda.cuda.synchronize()
        assert np.array_equal(raw_hits.numpy()[4:], want.view(np.uint8).reshape(-1))
        empty = np.zeros(0, rays.dtype)
        acc.trace_closest_host(empty, np.zeros(0, want.dtype))
        with pytest.raises(ValueError):
            acc.trace_closest_host(rays, np.zeros(10, want.dtype))
        assert lib.lcx_trace_closest_host(acc.handle, rays.ctypes.data, 16, 0xFF, None, 1, None) \
            == _capi.LCX_ERR_INVALID_ARG
        assert lib.lcx_set_host_chunk(100) == _capi.LCX_ERR_INVALID_ARG
        assert lib.lcx_set_host_access(4) == _capi.LCX_ERR_INVALID_ARG
    finally:
        _capi.check(lib.lcx_set_host_chunk(1 << 22), "chunk")
        _capi.check(lib.lcx_set_host_access(_capi.HOST_AUTO), "host access")
    no_kernel_errors()


_SERIALIZED_SCRIPT = """
import sys, time
sys.path.insert(0, {root!r})
import numpy as np, torch
from luisacompute_gb300 import scenes as S, _capi
from luisacompute_gb300.accel import accel_from_scene, rays_to_device, hits_to_numpy
lib = _capi.load()
_capi.check(lib.lcx_set_host_access(3), "streamed")
scene = S.terrain_scene(n=128, sphere_count=64, sphere_subdiv=3)
rays = S.terrain_rays(scene, 400_003, seed=41)
acc, _ = accel_from_scene(scene)
want = hits_to_numpy(acc.trace_closest(rays_to_device(rays)))
h_rays = torch.from_numpy(rays.view(np.float32).reshape(-1, 8)).pin_memory()
h_hits = torch.full((rays.shape[0], 6), -7, dtype=torch.int32).pin_memory()
t = time.perf_counter()
acc.trace_closest_host(h_rays, h_hits)
torch.cuda.synchronize()
dt = time.perf_counter() - t
_capi.check(lib.lcx_check_trace_errors(), "errors")
assert np.array_equal(h_hits.numpy().view(np.uint8).reshape(-1), want.view(np.uint8).reshape(-1))
assert dt < 5.0, dt
print("OK", dt)
"""


def test_host_streamed_serialized_launches(torch_cuda, lcx):
    """With launches serialised (CUDA_LAUNCH_BLOCKING=1, in a child process) a streamed host
    trace would wait for copies enqueued after its launch returned; it takes the staged path
    instead, promptly and with the device path's records."""
    import os
    import subprocess
    import sys
    from pathlib import Path
    root = str(Path(__file__).resolve().parent.parent)
    env = dict(os.environ, CUDA_LAUNCH_BLOCKING="1")
    r = subprocess.run([sys.executable, "-c", _SERIALIZED_SCRIPT.format(root=root)], env=env, capture_output=True,
                       text=True, timeout=300)
    assert r.returncode == 0 and "OK" in r.stdout, r.stdout[-2000:] + r.stderr[-2000:]


def test_host_streamed_concurrent(torch_cuda, lcx, oracle_mod):
    """Two host threads tracing host buffers at once on their own streams: one call holds the
    device's streamed-trace state, the other takes the staged path meanwhile; both give the
    oracle's records bit for bit."""
    import threading
    from luisacompute_gb300 import _capi
    lib = _capi.load()
    _capi.check(lib.lcx_set_host_access(3), "host access")
    scene = small_terrain()
    rays = S.terrain_rays(scene, 400_003, seed=37)
    osc = oracle_mod.OracleScene(scene)
    want = osc.trace_closest(rays)
    acc, _ = gpu_scene(scene)
    h_rays = torch_cuda.from_numpy(rays.view(np.float32).reshape(-1, 8)).pin_memory()
    outs = [torch_cuda.full((rays.shape[0], 6), -7, dtype=torch_cuda.int32).pin_memory() for _ in range(2)]
    errors = []

    def worker(k):
        try:
            s = torch_cuda.cuda.Stream()
            for _ in range(4):
                acc.trace_closest_host(h_rays, outs[k], stream=s)
            s.synchronize()
        except Exception as e:  # reported below
            errors.append(e)

    try:
        ts = [threading.Thread(target=worker, args=(k,)) for k in range(2)]
        for t in ts:
            t.start()
        for t in ts:
            t.join()
        assert not errors, errors
        for k in range(2):
            assert_bit_exact(oracle_mod, osc, rays, outs[k].numpy().view(want.dtype).reshape(-1), want)
    finally:
        _capi.check(lib.lcx_set_host_access(_capi.HOST_AUTO), "host access")
    no_kernel_errors()


@pytest.mark.parametrize("access", [3, 0])
def test_host_streamed_traces(torch_cuda, lcx, oracle_mod, access):
    """Streamed host-buffer traces (LCX_HOST_STREAMED, and auto above 2^18 rays): one traversal
    launch over the call takes each 2^17-ray copy chunk as its flag arrives while finished chunks
    are copied out; 700,001 rays are five full chunks and a partial one.  Closest and any hit, the
    oracle's records bit for bit, back to back on one side stream and then on the current stream
    (each call waits for the last one's kernel before it reuses the marks)."""
    from luisacompute_gb300 import _capi
    lib = _capi.load()
    _capi.check(lib.lcx_set_host_access(access), "host access")
    scene = small_terrain()
    rays = np.concatenate([S.terrain_rays(scene, 600_000, seed=27), S.terrain_shadow_rays(scene, 100_001, seed=28)])
    osc = oracle_mod.OracleScene(scene)
    want = osc.trace_closest(rays)
    want_any = osc.trace_any(rays)
    acc, _ = gpu_scene(scene)
    try:
        h_rays = torch_cuda.from_numpy(rays.view(np.float32).reshape(-1, 8)).pin_memory()
        for stream in (torch_cuda.cuda.Stream(), None):
            h_hits = torch_cuda.full((rays.shape[0], 6), -7, dtype=torch_cuda.int32).pin_memory()
            h_occ = torch_cuda.full((rays.shape[0],), 9, dtype=torch_cuda.uint8).pin_memory()
            acc.trace_closest_host(h_rays, h_hits, stream=stream)
            acc.trace_any_host(h_rays, h_occ, stream=stream)
            acc.trace_closest_host(h_rays, h_hits, stream=stream)  # again over the same buffers
            torch_cuda.cuda.synchronize()
            got = h_hits.numpy().view(want.dtype).reshape(-1)
            assert_bit_exact(oracle_mod, osc, rays, got, want)
            assert np.array_equal(h_occ.numpy(), want_any)
    finally:
        _capi.check(lib.lcx_set_host_access(_capi.HOST_AUTO), "host access")
    no_kernel_errors()


@pytest.mark.parametrize("fraction", [1.0, 4.0])
def test_triangle_splitting_keeps_results(torch_cuda, lcx, oracle_mod, fraction):
    """Split builds (FAST_TRACE, extra references with clipped boxes) give the oracle's records bit
    for bit: on a displaced mesh (long overlapping triangles, many splits), the terrain with its
    instanced spheres, and a batch of meshes built together; the references cover every triangle
    (no hit is lost) and the reference counts are the same in a batch as alone."""
    import ctypes
    from luisacompute_gb300 import _capi
    from luisacompute_gb300.accel import build_meshes, mesh_from_data
    lib = _capi.load()
    old = ctypes.c_float(0.0)
    _capi.check(lib.lcx_get_build_split(ctypes.byref(old)), "get")
    rng = np.random.default_rng(31)
    soup = S.displaced_mesh(150_000, rng)
    soup_scene = S.Scene([soup], np.array([0]), S.IDENTITY[None, :].copy(), np.array([0xFF], np.uint32))
    try:
        _capi.check(lib.lcx_set_build_split(ctypes.c_float(fraction)), "set")
        for scene, rays in ((soup_scene, S.sphere_rays(100_000, [-1.3] * 3, [1.3] * 3, seed=32)),
                            (small_terrain(), S.terrain_rays(small_terrain(), 100_000, seed=33))):
            osc = oracle_mod.OracleScene(scene)
            want, want_any = osc.trace_closest(rays), osc.trace_any(rays)
            acc, meshes = gpu_scene(scene)
            assert sum(int(m.stats().leaf_prim_count) for m in meshes) > sum(m.tri_count for m in scene.meshes)
            for layout in (0, 1):
                assert_bit_exact(oracle_mod, osc, rays, trace(acc, rays, layout), want)
                assert np.array_equal(trace_any(acc, rays, layout), want_any)
        # per-mesh reference counts do not depend on batching
        datas = [S.displaced_mesh(int(t), rng) for t in (2_000, 30_000, 500)]
        alone = [mesh_from_data(d).build() for d in datas]
        batch = build_meshes([mesh_from_data(d) for d in datas])
        for a, b in zip(alone, batch):
            assert a.stats().leaf_prim_count == b.stats().leaf_prim_count
    finally:
        _capi.check(lib.lcx_set_build_split(old), "restore")
    no_kernel_errors()
