"""CPU tests of the oracle: known-answer triangle tests, FP64 agreement, BVH == brute force."""
import numpy as np
import pytest

from luisacompute_gb300 import scenes as S


def test_watertight_known_answers(oracle_mod):
    # unit right triangle in z = 0, rays along -z
    v0, v1, v2 = [0, 0, 0], [1, 0, 0], [0, 1, 0]
    hit, t, u, v = oracle_mod.intersect_triangle([0.25, 0.25, 1], [0, 0, -1], 0.0, 1e30, v0, v1, v2)
    assert hit and t == 1.0 and u == 0.25 and v == 0.25
    # p = (1-u-v) v0 + u v1 + v v2 (src/dsl/rtx/hit.cpp:7-20)
    hit, t, u, v = oracle_mod.intersect_triangle([0.5, 0.125, 2], [0, 0, -1], 0.0, 1e30, v0, v1, v2)
    assert hit and t == 2.0 and u == 0.5 and v == 0.125
    # back face is not culled (src/backends/cuda/cuda_mesh.cpp:15-16)
    hit, t, _, _ = oracle_mod.intersect_triangle([0.25, 0.25, -1], [0, 0, 1], 0.0, 1e30, v0, v1, v2)
    assert hit and t == 1.0
    # outside, behind, t range
    assert not oracle_mod.intersect_triangle([1.0, 1.0, 1], [0, 0, -1], 0.0, 1e30, v0, v1, v2)[0]
    assert not oracle_mod.intersect_triangle([0.25, 0.25, 1], [0, 0, 1], 0.0, 1e30, v0, v1, v2)[0]
    assert not oracle_mod.intersect_triangle([0.25, 0.25, 1], [0, 0, -1], 0.0, 0.5, v0, v1, v2)[0]
    assert not oracle_mod.intersect_triangle([0.25, 0.25, 1], [0, 0, -1], 1.5, 1e30, v0, v1, v2)[0]
    # t range is closed: t == t_max and t == t_min are hits
    assert oracle_mod.intersect_triangle([0.25, 0.25, 1], [0, 0, -1], 0.0, 1.0, v0, v1, v2)[0]
    assert oracle_mod.intersect_triangle([0.25, 0.25, 1], [0, 0, -1], 1.0, 1e30, v0, v1, v2)[0]
    # degenerate triangle never hits
    assert not oracle_mod.intersect_triangle([0.5, 0.0, 1], [0, 0, -1], 0.0, 1e30, v0, v1, [2, 0, 0])[0]


def test_watertight_shared_edge(oracle_mod):
    """A ray through the shared edge of two triangles hits at least one of them."""
    a, b, c, d = [0, 0, 0], [1, 0, 0], [0, 1, 0], [1, 1, 0]
    rng = np.random.default_rng(0)
    for _ in range(2000):
        s = rng.random()
        p = np.array([1 - s, s, 0.0]) + rng.normal(0, 1e-3, 3) * [0, 0, 0]
        o = p + np.array([0, 0, 1.0]) + rng.normal(0, 0.3, 3) * [1, 1, 0]
        dvec = p - o
        h1 = oracle_mod.intersect_triangle(o, dvec, 0.0, 1e30, a, b, c)[0]
        h2 = oracle_mod.intersect_triangle(o, dvec, 0.0, 1e30, b, d, c)[0]
        assert h1 or h2


def test_affine_inverse(oracle_mod):
    rng = np.random.default_rng(1)
    rot = S.random_rotations(20, rng)
    aff = S.affine_rows(rot, np.exp(rng.uniform(-3, 1, 20)), rng.normal(0, 3, (20, 3)))
    for m in aff:
        w = oracle_mod.affine_inverse(m).astype(np.float64).reshape(3, 4)
        M = np.vstack([m.astype(np.float64).reshape(3, 4), [0, 0, 0, 1]])
        W = np.vstack([w, [0, 0, 0, 1]])
        np.testing.assert_allclose(W @ M, np.eye(4), atol=2e-5)
    ident = oracle_mod.affine_inverse(S.IDENTITY)
    assert np.array_equal(ident, S.IDENTITY)


def small_instanced_scene(seed=0):
    sphere = S.icosphere(2)
    grid = S.heightfield(17, seed=seed)
    rng = np.random.default_rng(seed)
    rot = S.random_rotations(6, rng)
    aff = np.concatenate([S.IDENTITY[None], S.affine_rows(rot, rng.uniform(0.05, 0.3, 6),
                                                          rng.uniform(-0.8, 0.8, (6, 3)))])
    return S.Scene([grid, sphere], np.array([0] + [1] * 6), aff,
                   np.array([0xFF, 0x01, 0x02, 0xFF, 0x04, 0xFF, 0xFF], np.uint32))


@pytest.mark.parametrize("mask", [0xFF, 0x01, 0x02, 0x00])
def test_bvh_equals_brute_force(oracle_mod, mask):
    scene = small_instanced_scene()
    o = oracle_mod.OracleScene(scene)
    lo, hi = scene.bounds()
    rays = S.sphere_rays(4000, lo, hi, seed=3)
    got = o.trace_closest(rays, mask)
    want = o.brute_closest(rays, mask)
    assert np.array_equal(got.view(np.uint8), want.view(np.uint8))
    occ = o.trace_any(rays, mask)
    assert np.array_equal(occ.astype(bool), want["inst"] != S.MISS)
    if mask == 0:
        assert np.all(want["inst"] == S.MISS)


def test_miss_record(oracle_mod):
    scene = small_instanced_scene()
    o = oracle_mod.OracleScene(scene)
    rays = np.zeros(3, S.RAY_DTYPE)
    rays["o"] = [10, 10, 10]
    rays["d"] = [1, 0, 0]
    rays["tmax"] = [1e30, 7.0, 0.5]
    h = o.trace_closest(rays)
    # {~0u, ~0u, (0,0), t_max} (accel.rs:501-507)
    assert np.all(h["inst"] == S.MISS) and np.all(h["prim"] == S.MISS)
    assert np.all(h["bary"] == 0) and np.array_equal(h["t"], rays["tmax"])


def test_fp64_agrees(oracle_mod):
    scene = small_instanced_scene(1)
    o = oracle_mod.OracleScene(scene)
    lo, hi = scene.bounds()
    rays = S.sphere_rays(4000, lo, hi, seed=5)
    got = o.trace_closest(rays)
    h64, t64 = o.fp64_closest(rays)
    rep = oracle_mod.adjudicate(o, rays, got, h64)
    assert rep["unexplained"] == []
    both = (got["inst"] != S.MISS) & (got["inst"] == h64["inst"]) & (got["prim"] == h64["prim"])
    # FP32 t error scales with the coordinates of the (instance-transformed) ray, ~1e-7 of the
    # scene extent (~1 here), not with t: hits closer than 0.1 are measured against 0.1
    rel = np.abs(got["t"][both] - t64[both]) / np.maximum(t64[both], 0.1)
    assert rel.max() <= 1e-5


def test_camera_icosphere_small(oracle_mod):
    scene = S.icosphere_scene(3)
    o = oracle_mod.OracleScene(scene)
    rays = S.camera_rays(64, 64)
    h = o.trace_closest(rays)
    hit = h["inst"] != S.MISS
    assert 0.2 < hit.mean() < 0.6
    # hit points lie on the unit sphere (within the faceting of a subdiv-3 icosphere)
    p = rays["o"][hit] + rays["d"][hit] * h["t"][hit, None]
    r = np.linalg.norm(p, axis=1)
    assert np.all((r > 0.98) & (r <= 1.0 + 1e-5))


def test_bvh_equals_brute_axis_aligned(oracle_mod):
    """Axis-aligned rays through icosphere vertices and along grid planes: the BVH walk must not
    cull boxes whose faces contain the ray (zero direction components)."""
    scene = S.icosphere_scene(3)
    o = oracle_mod.OracleScene(scene)
    v = scene.meshes[0].vertices[:, :3]
    axes = np.eye(3, dtype=np.float32)
    rays = np.zeros(6 * v.shape[0] + 6, S.RAY_DTYPE)
    k = 0
    for a in range(3):
        for sgn in (1.0, -1.0):
            d = axes[a] * sgn
            rays["o"][k:k + v.shape[0]] = v - 3.0 * d
            rays["d"][k:k + v.shape[0]] = d
            k += v.shape[0]
            rays["o"][k], rays["d"][k] = 0.0, d  # from the centre
            k += 1
    rays["tmax"] = 1e30
    got = o.trace_closest(rays)
    want = o.brute_closest(rays)
    assert np.array_equal(got.view(np.uint8), want.view(np.uint8))
    assert np.all(want["inst"] == 0)
