"""Accuracy of the GPU hit records against an FP64 evaluation, per workload.

The oracle's FP64 traversal (double-precision instance transform and triangle test,
oracle/lcx_oracle.cpp) gives the reference answer.  Per workload the test asserts the
tolerances of the path (>= 99.999 % of rays agree on (inst, prim); every disagreement is an
FP64 near-tie within 1e-6 relative in t or an edge/vertex-grazing hit; t and the hit point
within 1e-5 relative) and prints one JSON line of statistics.

t is measured relative to max(t64, 0.1 x scene extent): FP32 rounding of the transformed ray
and of the vertices is relative to the coordinates (the scene is about 2 units across), not to
t, so hits very close to the ray origin carry an absolute error of ~1e-7 of the extent.  The
pure relative error |dt|/t64 is reported beside it.

Barycentrics: an FP32 test works in coordinates relative to the ray origin (or a vertex), so
the absolute error of (u, v) is about eps x distance / triangle size: ~1e-4 for the 0.002-wide
terrain triangles seen from across the scene, for any FP32 ray/triangle test, Embree's
included.  The geometric accuracy is the hit point p = (1-u-v) v0 + u v1 + v v2: its FP32 error
|p32 - p64| (with FP64 vertices) relative to max(t64, 0.1 x extent) is bounded by 1e-5 here.
The raw (u, v) error distribution is reported beside it.

Conditioning: the test divides by a determinant proportional to |cos| of the angle between ray
and triangle normal, so rounding is amplified ~1/|cos| for grazing rays.  The bounds are
asserted for hits with |cos| >= 0.05; the statistics over all hits are reported.
"""
import json

import numpy as np
import pytest

from luisacompute_gb300 import scenes as S

pytestmark = pytest.mark.gpu


def _gpu_hits(scene, rays, layout):
    import torch
    from luisacompute_gb300.accel import accel_from_scene, hits_to_numpy, rays_to_device
    acc, meshes = accel_from_scene(scene)
    h = hits_to_numpy(acc.trace_closest(rays_to_device(rays), layout=layout))
    torch.cuda.synchronize()
    return h


def _stats(oracle_mod, scene, rays, got, name):
    osc = oracle_mod.OracleScene(scene)
    h64, t64 = osc.fp64_closest(rays)
    rep = oracle_mod.adjudicate(osc, rays, got, h64)
    same = (got["inst"] == h64["inst"]) & (got["prim"] == h64["prim"])
    hit = same & (got["inst"] != S.MISS)
    lo, hi = scene.bounds()
    ext = float(np.max(np.asarray(hi) - np.asarray(lo)))
    # barycentrics of the agreed hits, in FP64, for the bary error
    e64 = osc.fp64_eval(rays[hit], got["inst"][hit], got["prim"][hit])
    dt = np.abs(got["t"][hit].astype(np.float64) - t64[hit])
    rel_floor = dt / np.maximum(t64[hit], 0.1 * ext)
    rel = dt / np.maximum(t64[hit], 1e-30)
    dbary = np.maximum(np.abs(got["bary"][hit, 0].astype(np.float64) - e64["u"]),
                       np.abs(got["bary"][hit, 1].astype(np.float64) - e64["v"]))
    cos, e1, e2 = _hit_geometry(scene, rays[hit], got["inst"][hit], got["prim"][hit])
    du = (got["bary"][hit, 0].astype(np.float64) - e64["u"])[:, None]
    dv = (got["bary"][hit, 1].astype(np.float64) - e64["v"])[:, None]
    dp = np.linalg.norm(du * e1 + dv * e2, axis=1) / np.maximum(t64[hit], 0.1 * ext)
    steep = cos >= 0.05
    bad = (rel_floor > 1e-5) | (dp > 1e-5)
    out = {"workload": name, "rays": int(rays.shape[0]), "hits": int(hit.sum()),
           "id_agreement": float(same.mean()), "disagree": rep["disagree"], "near_tie": rep["near_tie"],
           "grazing": rep["grazing"], "unexplained": len(rep["unexplained"]),
           "t_rel_floored_max": float(rel_floor.max()), "t_rel_floored_p9999": float(np.quantile(rel_floor, 0.9999)),
           "t_rel_median": float(np.median(rel)), "t_rel_p9999": float(np.quantile(rel, 0.9999)),
           "t_rel_max": float(rel.max()), "bary_abs_median": float(np.median(dbary)),
           "bary_abs_p9999": float(np.quantile(dbary, 0.9999)), "bary_abs_max": float(dbary.max()),
           "point_rel_median": float(np.median(dp)), "point_rel_p9999": float(np.quantile(dp, 0.9999)),
           "point_rel_max": float(dp.max()), "hits_beyond_1e-5": int(bad.sum()),
           "max_abs_cos_beyond_1e-5": float(cos[bad].max()) if bad.any() else None,
           "steep_hits": int(steep.sum()), "steep_t_rel_floored_max": float(rel_floor[steep].max()),
           "steep_point_rel_max": float(dp[steep].max()), "scene_extent": ext}
    print("ACCURACY " + json.dumps(out))
    assert out["unexplained"] == 0
    # both conditions: at least 99.999 % of rays agree, and every disagreement is explained
    assert out["id_agreement"] >= 0.99999
    assert rep["disagree"] == rep["near_tie"] + rep["grazing"]
    assert out["steep_t_rel_floored_max"] <= 1e-5
    assert out["steep_point_rel_max"] <= 1e-5
    return out


def _hit_geometry(scene, rays, inst, prim):
    """World-space FP64 geometry of each hit triangle: |cos| of the angle between the ray and
    the normal, and the edges v1 - v0, v2 - v0."""
    cos = np.zeros(rays.shape[0])
    e1 = np.zeros((rays.shape[0], 3))
    e2 = np.zeros((rays.shape[0], 3))
    d = rays["d"].astype(np.float64)
    for i in np.unique(inst):
        sel = inst == i
        m = scene.meshes[scene.inst_mesh[i]]
        a = scene.inst_affine[i].astype(np.float64).reshape(3, 4)
        v = m.vertices[m.triangles[prim[sel]].astype(np.int64), :3].astype(np.float64) @ a[:, :3].T + a[:, 3]
        e1[sel] = v[:, 1] - v[:, 0]
        e2[sel] = v[:, 2] - v[:, 0]
        n = np.cross(e1[sel], e2[sel])
        dd = d[sel]
        cos[sel] = np.abs((n * dd).sum(1)) / (np.linalg.norm(n, axis=1) * np.linalg.norm(dd, axis=1))
    return cos, e1, e2


@pytest.mark.parametrize("layout", [1, 0])
def test_icosphere_primary_vs_fp64(lcx, oracle_mod, layout):
    """1024x1024 jittered pinhole rays at an 81,920-triangle icosphere."""
    scene = S.icosphere_scene(6)
    rays = S.primary_rays_icosphere()
    _stats(oracle_mod, scene, rays, _gpu_hits(scene, rays, layout), f"icosphere primary, layout {layout}")


@pytest.mark.parametrize("layout", [1, 0])
def test_terrain_incoherent_vs_fp64(lcx, oracle_mod, layout):
    """The terrain + 256 instanced spheres scene, 262,144 incoherent rays of the headline distribution."""
    scene = S.terrain_scene()
    rays = S.terrain_rays(scene, 262_144, seed=4)
    _stats(oracle_mod, scene, rays, _gpu_hits(scene, rays, layout), f"terrain incoherent, layout {layout}")


def test_batch_meshes_vs_fp64(lcx, oracle_mod):
    """Displaced icospheres and grids of the batched-build and serving scenes, one instance each."""
    rng = np.random.default_rng(21)
    meshes = [S.displaced_mesh(int(n), rng) for n in (300, 5_000, 60_000)]
    n = len(meshes)
    scene = S.Scene(meshes, np.arange(n), np.tile(S.IDENTITY, (n, 1)), np.full(n, 0xFF, np.uint32))
    rays = S.sphere_rays(200_000, *scene.bounds(), seed=22)
    _stats(oracle_mod, scene, rays, _gpu_hits(scene, rays, 1), "displaced meshes")
