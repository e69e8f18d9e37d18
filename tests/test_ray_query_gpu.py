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
    lib.rq_run_motion.restype = ctypes.c_int
    lib.rq_run_motion.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint32,
                                  ctypes.c_void_p]
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


def _sphere_aabbs(n, rng):
    c = rng.uniform(-1.0, 1.0, (n, 3))
    r = rng.uniform(0.03, 0.15, n)
    return np.concatenate([c - r[:, None], c + r[:, None]], 1).astype(np.float32)


def _spheres_fp64(rays, aabbs, affines):
    """Closest sphere hit per ray in FP64: (t, inst, prim), inf / ~0 for a miss."""
    lo, hi = aabbs[:, :3].astype(np.float64), aabbs[:, 3:].astype(np.float64)
    cen, rad = 0.5 * (lo + hi), 0.5 * (hi[:, 0] - lo[:, 0])
    best_t = np.full(rays.shape[0], np.inf)
    best_i = np.full(rays.shape[0], S.MISS, np.uint32)
    best_p = np.full(rays.shape[0], S.MISS, np.uint32)
    o, d = rays["o"].astype(np.float64), rays["d"].astype(np.float64)
    tmin, tmax = rays["tmin"].astype(np.float64), rays["tmax"].astype(np.float64)
    for inst, aff in enumerate(affines):
        a = aff.astype(np.float64).reshape(3, 4)
        inv = np.linalg.inv(a[:, :3])
        oo = (o - a[:, 3]) @ inv.T
        dd = d @ inv.T
        for s0 in range(0, rays.shape[0], 4096):
            sl = slice(s0, s0 + 4096)
            oc = oo[sl, None, :] - cen[None]
            A = (dd[sl] ** 2).sum(1)[:, None]
            B = (oc * dd[sl, None, :]).sum(2)
            C = (oc ** 2).sum(2) - rad[None] ** 2
            disc = B * B - A * C
            sq = np.sqrt(np.maximum(disc, 0.0))
            t0, t1 = (-B - sq) / A, (-B + sq) / A
            t = np.where(t0 >= tmin[sl, None], t0, t1)
            ok = (disc >= 0) & (t >= tmin[sl, None]) & (t < tmax[sl, None])
            t = np.where(ok, t, np.inf)
            j = t.argmin(1)
            tj = t[np.arange(t.shape[0]), j]
            better = tj < best_t[sl]
            best_t[sl] = np.where(better, tj, best_t[sl])
            best_i[sl] = np.where(better, inst, best_i[sl])
            best_p[sl] = np.where(better, j, best_p[sl])
    return best_t, best_i, best_p


def test_procedural_primitives(lcx, oracle_mod, rq):
    import torch
    from luisacompute_gb300.accel import Accel, ProceduralPrimitive, hits_to_numpy, mesh_from_data, rays_to_device
    rng = np.random.default_rng(51)
    aabbs = _sphere_aabbs(300, rng)
    prim = ProceduralPrimitive(torch.from_numpy(aabbs).cuda()).build()
    tri = S.icosphere(3, radius=0.4)
    mesh = mesh_from_data(tri).build()
    affines = [S.affine_rows(S.random_rotations(1, rng), np.array([1.5]), np.array([[0.2, -0.1, 0.3]]))[0],
               np.array([1, 0, 0, 0.5, 0, 1, 0, -0.4, 0, 0, 1, 0.1], np.float32)]
    acc = Accel()
    acc.emplace_back(prim, affines[0])
    acc.emplace_back(prim, affines[1])
    acc.emplace_back(mesh, S.IDENTITY)
    acc.build()
    rays = S.sphere_rays(20_000, [-2.0] * 3, [2.0] * 3, seed=52)
    d = rays_to_device(rays)
    n = rays.shape[0]
    # plain traces do not see procedural instances: the oracle with those slots invisible
    oscene = S.Scene([tri, S.icosphere(1)], np.array([1, 1, 0]), np.stack(affines + [S.IDENTITY]).astype(np.float32),
                     np.array([0, 0, 0xFF], np.uint32))
    osc = oracle_mod.OracleScene(oscene)
    tri_hits = hits_to_numpy(acc.trace_closest(d))
    assert np.array_equal(tri_hits.view(np.uint8), osc.trace_closest(rays).view(np.uint8))
    assert np.array_equal(acc.trace_any(d).cpu().numpy(), osc.trace_any(rays))
    # ray_query with triangles and spheres: the closer of the two, spheres checked against FP64
    hits = torch.empty((n, 6), dtype=torch.int32, device="cuda")
    assert rq.rq_run(ctypes.byref(_view(acc)), d.data_ptr(), n, 3, 1, hits.data_ptr(), None) == 0
    got = hits_to_numpy(hits)
    st, si, sp = _spheres_fp64(rays, aabbs, affines)
    tt = np.where(tri_hits["inst"] != S.MISS, tri_hits["t"].astype(np.float64), np.inf)
    sphere_first = st < tt
    with np.errstate(invalid="ignore"):  # inf - inf where both miss
        clear = ~(np.abs(st - tt) <= 1e-4 * np.minimum(st, tt))  # not a near-tie between the two kinds
    kind = got["pad"]
    # FP32 and FP64 may disagree on a grazing ray's discriminant: allow a handful of those
    assert (kind[clear & sphere_first & np.isfinite(st)] != 2).sum() <= 5
    assert (kind[clear & ~sphere_first & np.isfinite(tt)] != 1).sum() <= 5
    assert (kind[~np.isfinite(st) & ~np.isfinite(tt)] != 0).sum() <= 5
    sel = clear & sphere_first & np.isfinite(st) & (kind == 2)
    assert sel.sum() > 1000
    same = (got["inst"][sel] == si[sel]) & (got["prim"][sel] == sp[sel])
    assert same.mean() > 0.999  # the rest: two spheres at nearly equal distance
    # the callback's FP32 quadratic loses digits for near-tangent rays (catastrophic cancellation)
    rel = np.abs(got["t"][sel][same] - st[sel][same]) / np.maximum(st[sel][same], 1e-3)
    assert np.median(rel) < 1e-6 and rel.max() < 2e-3
    tri_sel = clear & ~sphere_first & np.isfinite(tt) & (kind == 1)
    for f in ("inst", "prim", "t"):
        assert np.array_equal(got[f][tri_sel], tri_hits[f][tri_sel])


def test_curves_as_surface_candidates(lcx, rq):
    """Curve segments reach the candidate callback as surface candidates (bary_v = -1); committing
    every candidate gives lcx_trace_closest's records bit for bit, curve and triangle hits alike,
    and a cutout of every curve segment leaves only the triangles."""
    import torch
    from luisacompute_gb300.accel import Accel, Curve, hits_to_numpy, mesh_from_data, rays_to_device
    rng = np.random.default_rng(77)
    cps = S.hair_curves(80, 10, rng)
    segs = S.curve_segments(80, 10, 2)
    cv = Curve(2, torch.from_numpy(cps).cuda(), torch.from_numpy(segs.astype(np.int32)).cuda()).build()
    mesh = mesh_from_data(S.icosphere(3, radius=0.7)).build()
    acc = Accel()
    acc.emplace_back(cv)
    acc.emplace_back(mesh)
    acc.build()
    rays = S.sphere_rays(60_000, [-1.5] * 3, [1.5] * 3, seed=78)
    d = rays_to_device(rays)
    n = rays.shape[0]
    hits = torch.empty((n, 6), dtype=torch.int32, device="cuda")
    assert rq.rq_run(ctypes.byref(_view(acc)), d.data_ptr(), n, 0, CUT, hits.data_ptr(), None) == 0
    got = hits_to_numpy(hits)
    want = hits_to_numpy(acc.trace_closest(d))
    assert np.array_equal(got.view(np.uint8), want.view(np.uint8))
    on_curve = got["inst"] == 0
    assert on_curve.sum() > 500 and (got["inst"] == 1).sum() > 500
    assert np.all(got["bary"][on_curve, 1] == -1.0)


def test_ray_query_motion(lcx, rq):
    """lcx::ray_query_motion (the reference's traverse_motion, include/luisa/dsl/rtx/accel.h:49-50):
    committing every candidate at each ray's time gives lcx_trace_closest_motion's records bit for
    bit, on an accel with static and moving instances, a keyframed mesh and a keyframed curve; the
    plain query on the same view passes over everything that moves."""
    import torch
    from luisacompute_gb300.accel import (Accel, Curve, Mesh, MotionInstance, hits_to_numpy, mesh_from_data,
                                          rays_to_device)
    rng = np.random.default_rng(91)
    sphere = S.icosphere(3, radius=0.4)
    mesh = mesh_from_data(sphere).build()
    keys = S.affine_rows(S.random_rotations(3, rng), np.array([1.0, 1.2, 0.8]),
                         rng.uniform(-0.6, 0.6, (3, 3))).reshape(3, 3, 4)
    mo = MotionInstance(mesh, keys, 0.0, 1.0, vanish_end=True)
    v0 = sphere.vertices.copy()
    v1 = v0.copy()
    v1[:, 1] += 0.5
    kv = torch.from_numpy(np.concatenate([v0, v1])).cuda()
    kt = torch.from_numpy(sphere.triangles.astype(np.int32)).cuda()
    kmesh = Mesh(kv, kt, motion_keyframes=2).build()
    cps = S.hair_curves(32, 8, rng)
    moved = cps.copy()
    moved[:, 0] += 0.3
    kc = Curve(2, torch.from_numpy(np.concatenate([cps, moved])).cuda(),
               torch.from_numpy(S.curve_segments(32, 8, 2).astype(np.int32)).cuda(), motion_keyframes=2).build()
    acc = Accel()
    acc.emplace_back(mesh, np.array([[1, 0, 0, 0.8], [0, 1, 0, 0], [0, 0, 1, 0]], np.float32))
    acc.emplace_back(mo)
    acc.emplace_back(kmesh, np.array([[1, 0, 0, -0.8], [0, 1, 0, 0], [0, 0, 1, 0]], np.float32))
    acc.emplace_back(kc)
    acc.build()
    view = _view(acc)
    assert view.motion == 1
    rays = S.sphere_rays(60_000, [-1.5] * 3, [1.5] * 3, seed=92)
    times = rng.uniform(-0.2, 1.2, rays.shape[0]).astype(np.float32)
    d, dt = rays_to_device(rays), torch.from_numpy(times).cuda()
    n = rays.shape[0]
    hits = torch.empty((n, 6), dtype=torch.int32, device="cuda")
    assert rq.rq_run_motion(ctypes.byref(view), d.data_ptr(), dt.data_ptr(), n, hits.data_ptr()) == 0
    got = hits_to_numpy(hits)
    want = hits_to_numpy(acc.trace_closest_motion(d, dt))
    assert np.array_equal(got.view(np.uint8), want.view(np.uint8))
    for inst in range(4):
        assert (got["inst"] == inst).sum() > 200, inst
    # the plain query sees the static instance only
    assert rq.rq_run(ctypes.byref(view), d.data_ptr(), n, 0, CUT, hits.data_ptr(), None) == 0
    plain = hits_to_numpy(hits)
    assert set(np.unique(plain["inst"])) <= {0, 0xFFFFFFFF} and (plain["inst"] == 0).sum() > 200
