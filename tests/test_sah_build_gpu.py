"""Binned-SAH binary trees (the BLAS builder of FAST_TRACE meshes, lcx_set_build_blas_sah, and the
TLAS builder, lcx_set_build_tlas_sah): hit records never depend on the tree, so with the SAH
builder on they must equal the oracle's bit for bit, as with the LBVH; the SAH of the tree must be
lower than the LBVH's on a heightfield.  The cases reach both phases of the builder: ranges of more
than 1024 items (split level by level over the whole build) and of at most 1024 (one block per
range), their boundary (1024 / 1025 / 2049 triangles), coincident centroids (median splits),
invalid triangles (empty boxes), and batches mixing small, large and empty meshes."""
import ctypes

import numpy as np
import pytest

from luisacompute_gb300 import scenes as S

pytestmark = pytest.mark.gpu


class _Knob:
    """Sets lcx_set_build_<name> for the duration of a with-block."""

    def __init__(self, name, value):
        from luisacompute_gb300 import _capi
        self.lib, self.name, self.value = _capi.load(), name, value

    def __enter__(self):
        from luisacompute_gb300 import _capi
        old = ctypes.c_uint32(0)
        _capi.check(getattr(self.lib, f"lcx_get_build_{self.name}")(ctypes.byref(old)), "get")
        self.old = old.value
        _capi.check(getattr(self.lib, f"lcx_set_build_{self.name}")(self.value), "set")

    def __exit__(self, *exc):
        from luisacompute_gb300 import _capi
        _capi.check(getattr(self.lib, f"lcx_set_build_{self.name}")(self.old), "restore")


def _strip(n_tris, rng, jitter=0.0):
    """n_tris small triangles along a noisy strip (uneven spacing, so SAH splits are uneven)."""
    x = np.cumsum(rng.exponential(1.0, n_tris)).astype(np.float32)
    x = x / x[-1] * 4.0 - 2.0
    v = np.zeros((3 * n_tris, 4), np.float32)
    base = np.stack([x, rng.uniform(-0.3, 0.3, n_tris), rng.uniform(-0.3, 0.3, n_tris)], 1).astype(np.float32)
    for k in range(3):
        v[k::3, :3] = base + rng.uniform(-0.02, 0.02, (n_tris, 3)).astype(np.float32)
    if jitter:
        v[:, :3] += rng.standard_normal((3 * n_tris, 3)).astype(np.float32) * np.float32(jitter)
    t = np.arange(3 * n_tris, dtype=np.uint32).reshape(-1, 3)
    return S.MeshData(v, t)


def _scene(meshes, rng):
    n = len(meshes)
    aff = S.affine_rows(S.random_rotations(n, rng), np.exp(rng.uniform(np.log(0.3), np.log(1.0), n)),
                        rng.uniform(-1, 1, (n, 3)))
    return S.Scene(meshes, np.arange(n), aff, np.full(n, 0xFF, np.uint32))


def _trace(scene, rays, batch):
    import torch
    from luisacompute_gb300 import _capi
    from luisacompute_gb300.accel import accel_from_scene, hits_to_numpy, rays_to_device
    acc, meshes = accel_from_scene(scene, batch=batch)
    d = rays_to_device(rays)
    got = hits_to_numpy(acc.trace_closest(d))
    occ = acc.trace_any(d).cpu().numpy()
    torch.cuda.synchronize()
    _capi.check(_capi.load().lcx_check_trace_errors(), "trace errors")
    return got, occ, acc, meshes


def _aimed(scene, n, seed):
    """Rays from random points of the scene's box, each aimed at the centroid of a random triangle
    of a random instance."""
    lo, hi = scene.bounds()
    rng = np.random.default_rng(seed)
    rays = S.sphere_rays(n, lo, hi, seed=seed)
    inst = np.array([i for i in range(scene.instance_count) if scene.meshes[scene.inst_mesh[i]].tri_count > 0])
    pick = inst[rng.integers(0, inst.size, n)]
    tgt = np.zeros((n, 3))
    for i in np.unique(pick):
        sel = pick == i
        m = scene.meshes[scene.inst_mesh[i]]
        t = rng.integers(0, m.tri_count, int(sel.sum()))
        v = m.vertices[:, :3].astype(np.float64)
        c = v[m.triangles[t].astype(np.int64)].mean(axis=1)
        a = scene.inst_affine[i].astype(np.float64).reshape(3, 4)
        tgt[sel] = c @ a[:, :3].T + a[:, 3]
    d = tgt - rays["o"]
    rays["d"] = (d / np.linalg.norm(d, axis=1, keepdims=True)).astype(np.float32)
    return rays


@pytest.mark.parametrize("batch", [False, True])
def test_sah_blas_sizes_and_degenerates(lcx, oracle_mod, batch):
    rng = np.random.default_rng(21)
    meshes = [_strip(n, rng) for n in (1, 2, 3, 31, 1024, 1025, 2049, 5000)]
    # 3000 coincident triangles (every centroid equal: no bin boundary separates them)
    one = _strip(1, rng)
    meshes.append(S.MeshData(one.vertices.copy(), np.zeros((3000, 3), np.uint32) + np.arange(3, dtype=np.uint32)))
    meshes.insert(4, S.MeshData(np.zeros((3, 4), np.float32), np.zeros((0, 3), np.uint32)))  # empty
    scene = _scene(meshes, rng)
    rays = _aimed(scene, 120_000, seed=22)
    osc = oracle_mod.OracleScene(scene)
    want, want_occ = osc.trace_closest(rays), osc.trace_any(rays)
    for sah in (1, 0):
        with _Knob("blas_sah", sah):
            got, occ, _, meshes_d = _trace(scene, rays, batch)
        assert np.array_equal(got.view(np.uint8), want.view(np.uint8)), f"blas_sah {sah}"
        assert np.array_equal(occ, want_occ), f"blas_sah {sah}"
        for md, m in zip(meshes, meshes_d):
            assert int(m.stats().leaf_prim_count) == md.triangles.shape[0]
    assert (want["inst"] != S.MISS).mean() > 0.5


def test_sah_blas_invalid_triangles(lcx):
    """2500 triangles, every fifth with a vertex at NaN (an item with an empty box): the SAH and
    LBVH trees place every triangle and give the same hits."""
    rng = np.random.default_rng(26)
    good = _strip(2500, rng)
    bad = S.MeshData(good.vertices.copy(), good.triangles.copy())
    bad.vertices[0:3 * 2500:15, 0] = np.nan
    good_scene = _scene([good], rng)
    scene = S.Scene([bad], good_scene.inst_mesh, good_scene.inst_affine, good_scene.inst_mask)
    rays = _aimed(good_scene, 50_000, seed=27)
    res = []
    for sah in (1, 0):
        with _Knob("blas_sah", sah):
            got, occ, _, meshes_d = _trace(scene, rays, False)
        assert int(meshes_d[0].stats().leaf_prim_count) == 2500
        res.append((got, occ))
    assert np.array_equal(res[0][0].view(np.uint8), res[1][0].view(np.uint8))
    assert np.array_equal(res[0][1], res[1][1])
    assert (res[0][0]["inst"] != S.MISS).mean() > 0.3


def test_sah_lowers_the_heightfield_sah(lcx, oracle_mod):
    """On a 256 x 256 heightfield (130k triangles: large ranges, then one-block ranges) the SAH
    builder's binary tree has a lower SAH than the LBVH's, and the hits are the oracle's."""
    from luisacompute_gb300.accel import Accel, hits_to_numpy, mesh_from_data, rays_to_device
    import torch
    md = S.heightfield(256, seed=2)
    scene = S.Scene([md], np.array([0]), S.IDENTITY[None].copy(), np.full(1, 0xFF, np.uint32))
    rays = S.terrain_rays(scene, 100_000, seed=23)
    want = oracle_mod.OracleScene(scene).trace_closest(rays)
    sah = {}
    for on in (1, 0):
        with _Knob("blas_sah", on):
            m = mesh_from_data(md).build()
        acc = Accel()
        acc.emplace_back(m, S.IDENTITY.reshape(3, 4))
        acc.build()
        got = hits_to_numpy(acc.trace_closest(rays_to_device(rays)))
        torch.cuda.synchronize()
        assert np.array_equal(got.view(np.uint8), want.view(np.uint8)), f"blas_sah {on}"
        st = m.stats()
        sah[on] = st.sah_cost
        assert int(st.leaf_prim_count) == md.triangles.shape[0]
    assert sah[1] < 0.95 * sah[0], sah


def test_fast_build_meshes_keep_the_lbvh(lcx):
    """FAST_BUILD meshes are built by the LBVH whatever the knob: same SAH either way."""
    import torch
    from luisacompute_gb300.accel import HINT_FAST_BUILD, AccelOption, Mesh
    md = S.heightfield(128, seed=3)
    v = torch.from_numpy(np.ascontiguousarray(md.vertices)).cuda()
    t = torch.from_numpy(md.triangles.astype(np.int32)).cuda()
    out = []
    for on in (1, 0):
        with _Knob("blas_sah", on):
            m = Mesh(v, t, AccelOption(hint=HINT_FAST_BUILD)).build()
        torch.cuda.synchronize()
        out.append(m.stats().sah_cost)
    assert out[0] == out[1]


@pytest.mark.parametrize("count", [900, 3000])
def test_sah_tlas_many_instances(lcx, oracle_mod, count):
    """TLAS over `count` instances (3000: ranges above 1024 instances), a tenth of them stacked on
    one spot (coincident centroids); hits equal the oracle's with the SAH TLAS on and off."""
    import torch
    from luisacompute_gb300.accel import Accel, hits_to_numpy, mesh_from_data, rays_to_device
    rng = np.random.default_rng(24)
    datas = [S.icosphere(1), _strip(40, rng)]
    meshes = [mesh_from_data(m).build() for m in datas]
    pick = rng.integers(0, 2, count)
    trans = rng.uniform(-3, 3, (count, 3))
    trans[: count // 10] = 0.5
    aff = S.affine_rows(S.random_rotations(count, rng), np.exp(rng.uniform(np.log(0.05), np.log(0.2), count)), trans)
    scene = S.Scene(datas, pick, aff, np.full(count, 0xFF, np.uint32))
    rays = _aimed(scene, 60_000, seed=25)
    want = oracle_mod.OracleScene(scene).trace_closest(rays)
    for on in (1, 0):
        with _Knob("tlas_sah", on):
            acc = Accel()
            acc.emplace_back_many([meshes[i] for i in pick], aff)
            acc.build()
        got = hits_to_numpy(acc.trace_closest(rays_to_device(rays)))
        torch.cuda.synchronize()
        assert np.array_equal(got.view(np.uint8), want.view(np.uint8)), f"tlas_sah {on}"
        assert int(acc.stats().leaf_prim_count) == count
    assert (want["inst"] != S.MISS).mean() > 0.5


@pytest.mark.parametrize("batch", [False, True])
def test_dp_collapse(lcx, oracle_mod, batch):
    """The collapse by dynamic program (lcx_set_build_collapse 1, the default) against the greedy one
    (0): the oracle's records bit for bit either way, on uneven meshes alone and in one batch, and
    fewer wide nodes on a heightfield, whose wide-tree SAH is no higher."""
    import torch
    from luisacompute_gb300.accel import Accel, mesh_from_data
    rng = np.random.default_rng(31)
    meshes = [_strip(n, rng) for n in (2, 17, 700, 3000)] + [S.heightfield(64, seed=4), S.icosphere(3)]
    scene = _scene(meshes, rng)
    rays = _aimed(scene, 80_000, seed=32)
    osc = oracle_mod.OracleScene(scene)
    want, want_occ = osc.trace_closest(rays), osc.trace_any(rays)
    for mode in (1, 0):
        with _Knob("collapse", mode):
            got, occ, _, _ = _trace(scene, rays, batch)
        assert np.array_equal(got.view(np.uint8), want.view(np.uint8)), f"collapse {mode}"
        assert np.array_equal(occ, want_occ), f"collapse {mode}"
    md = S.heightfield(192, seed=5)
    stats = {}
    for mode in (1, 0):
        with _Knob("collapse", mode):
            m = mesh_from_data(md).build()
        torch.cuda.synchronize()
        st = m.stats()
        assert int(st.leaf_prim_count) == md.triangles.shape[0]
        stats[mode] = (int(st.node_count), st.wide_sah_cost)
    assert stats[1][0] < 0.9 * stats[0][0], stats
    assert stats[1][1] <= stats[0][1] * 1.01, stats


def test_release_scratch(lcx, oracle_mod):
    """Builds take their scratch from a pool that keeps freed memory for the next build;
    lcx_release_scratch hands it back to the driver.  Builds before and after it give the oracle's
    records, and a build right after it maps its scratch again."""
    from luisacompute_gb300 import _capi
    lib = _capi.load()
    rng = np.random.default_rng(31)
    scene = _scene([_strip(3000, rng), _strip(1500, rng, jitter=0.01)], rng)
    rays = _aimed(scene, 20_000, seed=32)
    osc = oracle_mod.OracleScene(scene)
    want = osc.trace_closest(rays)
    for step in range(2):
        got, _, _, _ = _trace(scene, rays, batch=True)
        assert np.array_equal(got.view(np.uint8), want.view(np.uint8))
        assert lib.lcx_release_scratch() == _capi.LCX_OK
