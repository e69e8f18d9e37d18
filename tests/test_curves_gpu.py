"""Curves (Curve, include/luisa/runtime/rtx/curve.h; CurveBasis, include/luisa/runtime/rhi/curve_basis.h:11-24;
CurveBuildCommand, include/luisa/runtime/rhi/command.h:446-486).

A segment is the union of balls along its curve (round curves, as the reference's Embree and OptiX
paths use, cpu/accel.rs:150-156 and cuda_curve.cpp:45-51); cubic segments are traced as the round
cones between the balls at u = k/pieces.  The oracle (lcxo_trace_curves) picks the same pieces with
the kernels' FP32 sequence and intersects them in FP64, so records agree except on rays that graze
a silhouette within FP32 rounding: the tests bound the share of such rays and the t / u errors.
Hit records follow the reference's curve convention: prim = segment, bary = (u, -1)
(include/luisa/runtime/rtx/hit.h:29-30, cpu/accel.rs:491-494)."""
import numpy as np
import pytest

from luisacompute_gb300 import scenes as S

pytestmark = pytest.mark.gpu

INV = 0xFFFFFFFF
BASES = (0, 1, 2, 3)


def _aimed_rays(rng, targets, n, centre, radius=3.0, jitter=0.03):
    """Rays from a sphere around ``centre`` toward jittered points of ``targets`` (many hits and
    many near misses), plus a quarter of incoherent rays starting inside the scene's box."""
    k = n - n // 4
    tgt = targets[rng.integers(0, targets.shape[0], k)] + rng.normal(0.0, jitter, (k, 3))
    o = rng.standard_normal((k, 3))
    o = centre + radius * o / np.linalg.norm(o, axis=1, keepdims=True)
    d = tgt - o
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    rays = np.zeros(n, S.RAY_DTYPE)
    rays["o"][:k] = o
    rays["d"][:k] = d
    rays["tmax"][:k] = 1e30
    lo, hi = targets.min(0), targets.max(0)
    rays[k:] = S.sphere_rays(n - k, lo, hi, seed=int(rng.integers(1 << 30)))
    return rays


def _check(got, want, min_hits=0.15, max_mismatch=2e-3, curve_inst=None):
    hg, hw = got["inst"] != INV, want["inst"] != INV
    n = got.shape[0]
    assert hw.mean() >= min_hits, hw.mean()
    mism = hg != hw
    assert mism.mean() <= max_mismatch, (int(mism.sum()), n)
    both = hg & hw
    tg, tw = got["t"][both].astype(np.float64), want["t"][both].astype(np.float64)
    terr = np.abs(tg - tw) / (1e-4 + 1e-5 * np.abs(tw))
    assert np.quantile(terr, 0.999) <= 1.0 and terr.max() <= 50.0, (np.quantile(terr, 0.999), terr.max())
    same = (got["inst"][both] == want["inst"][both]) & (got["prim"][both] == want["prim"][both])
    assert same.mean() >= 0.995, same.mean()
    assert np.all(terr[~same] <= 50.0)  # another segment only at a near-tie
    du = np.abs(got["bary"][both, 0][same] - want["bary"][both, 0][same])
    assert np.quantile(du, 0.999) <= 2e-3 and du.max() <= 5e-2, (np.quantile(du, 0.999), du.max())
    on_curve = hg if curve_inst is None else hg & np.isin(got["inst"], curve_inst)
    assert np.all(got["bary"][on_curve, 1] == -1.0)
    miss = ~hg
    assert np.all(got["prim"][miss] == INV) and np.all(got["bary"][miss] == 0.0)


def _curve_scene(rng, basis, n_curves=96, n_cp=10):
    import torch
    from luisacompute_gb300.accel import Accel, Curve
    cps = S.hair_curves(n_curves, n_cp, rng)
    segs = S.curve_segments(n_curves, n_cp, basis)
    cv = Curve(basis, torch.from_numpy(cps).cuda(), torch.from_numpy(segs.astype(np.int32)).cuda()).build()
    aff = np.stack([np.eye(3, 4, dtype=np.float32).reshape(12),
                    S.affine_rows(S.random_rotations(1, rng), np.array([0.7]), np.array([[2.5, 0.0, 0.0]]))[0],
                    S.affine_rows(S.random_rotations(1, rng), np.array([1.3]), np.array([[0.0, -2.5, 0.5]]))[0]])
    masks = np.array([0xFF, 0x0F, 0xF0], np.uint32)
    acc = Accel()
    for i in range(3):
        acc.emplace_back(cv, aff[i].reshape(3, 4), visibility_mask=int(masks[i]))
    acc.build()
    torch.cuda.synchronize()
    world = np.concatenate([cps[:, :3] @ aff[i].reshape(3, 4)[:, :3].T + aff[i].reshape(3, 4)[:, 3]
                            for i in range(3)])
    return cps, segs, cv, acc, aff, masks, world


@pytest.mark.parametrize("basis", BASES)
def test_curve_bases_match_oracle(lcx, oracle_mod, basis):
    from luisacompute_gb300.accel import hits_to_numpy, rays_to_device
    rng = np.random.default_rng(700 + basis)
    cps, segs, cv, acc, aff, masks, world = _curve_scene(rng, basis)
    oc = oracle_mod.OracleCurve(cps, segs, basis)
    if basis != 0:
        assert oc.pieces().max() > 1  # bent strands are traced as several cones
    rays = _aimed_rays(rng, world, 120_000, world.mean(0))
    d_rays = rays_to_device(rays)
    for mask in (0xFF, 0x0F):
        want = oracle_mod.trace_curves([oc] * 3, aff, masks, rays, mask=mask)
        want_any = oracle_mod.trace_curves([oc] * 3, aff, masks, rays, mask=mask, any_hit=True)
        for layout in (0, 1):
            got = hits_to_numpy(acc.trace_closest(d_rays, mask=mask, layout=layout))
            _check(got, want, min_hits=0.1)
            occ = acc.trace_any(d_rays, mask=mask, layout=layout).cpu().numpy()
            assert (occ != want_any).mean() <= 2e-3
            assert np.array_equal(occ.astype(bool), got["inst"] != INV) or (
                (occ.astype(bool) != (got["inst"] != INV)).mean() <= 1e-3)
    if mask == 0x0F:
        assert not np.any(got["inst"] == 2)  # instance 2's mask 0xF0 never meets ray mask 0x0F


def test_curve_open_ends_and_caps(lcx, oracle_mod):
    """One straight strand along x (radius 0.1) per basis: rays straight down at x = 0.5 hit the side
    (t = 0.9, u = 0.5); at x = 1.05 and x = -0.05 only the end balls lie below them, which linear
    segments have (spherical caps) and open cubic ones do not; a ray starting inside misses."""
    import torch
    from luisacompute_gb300.accel import Accel, Curve, hits_to_numpy, rays_to_device
    rays = np.zeros(4, S.RAY_DTYPE)
    rays["o"] = [[0.5, 1, 0], [1.05, 1, 0], [-0.05, 1, 0], [0.5, 0, 0]]
    rays["d"] = [0, -1, 0]
    rays["tmax"] = 1e30
    pts = {0: [[0, 0, 0, 0.1], [1, 0, 0, 0.1]],
           3: [[0, 0, 0, 0.1], [1 / 3, 0, 0, 0.1], [2 / 3, 0, 0, 0.1], [1, 0, 0, 0.1]],
           1: [[-1, 0, 0, 0.1], [0, 0, 0, 0.1], [1, 0, 0, 0.1], [2, 0, 0, 0.1]],  # B-spline: x runs 0..1
           2: [[-1, 0, 0, 0.1], [0, 0, 0, 0.1], [1, 0, 0, 0.1], [2, 0, 0, 0.1]]}
    for basis, p in pts.items():
        cps = np.array(p, np.float32)
        cv = Curve(basis, torch.from_numpy(cps).cuda(), torch.zeros(1, dtype=torch.int32).cuda()).build()
        acc = Accel()
        acc.emplace_back(cv)
        acc.build()
        got = hits_to_numpy(acc.trace_closest(rays_to_device(rays)))
        want = oracle_mod.trace_curves([oracle_mod.OracleCurve(cps, np.zeros(1), basis)],
                                       np.eye(3, 4, dtype=np.float32).reshape(1, 12), 0xFF, rays)
        assert np.array_equal(got["inst"], want["inst"]), basis
        assert got["inst"][0] == 0 and abs(got["t"][0] - 0.9) < 1e-5 and abs(got["bary"][0, 0] - 0.5) < 1e-4
        assert got["bary"][0, 1] == -1.0
        capped = basis == 0
        assert (got["inst"][1] == 0) == capped and (got["inst"][2] == 0) == capped, basis
        if capped:
            assert abs(got["t"][1] - (1 - np.sqrt(0.01 - 0.0025))) < 1e-5 and got["bary"][1, 0] == 1.0
            assert got["bary"][2, 0] == 0.0
        assert got["inst"][3] == INV  # starts inside the strand


def test_curves_with_meshes_and_errors(lcx, oracle_mod):
    import torch
    from luisacompute_gb300 import LcxError
    from luisacompute_gb300.accel import Accel, Curve, hits_to_numpy, mesh_from_data, rays_to_device
    import ctypes
    rng = np.random.default_rng(711)
    basis = 2
    cps = S.hair_curves(64, 8, rng, lo=(-1.2, -1.2, -1.2), hi=(1.2, 1.2, 1.2))
    segs = S.curve_segments(64, 8, basis)
    d_cps = torch.from_numpy(cps).cuda()
    cv = Curve(basis, d_cps, torch.from_numpy(segs.astype(np.int32)).cuda()).build()
    sphere = S.icosphere(4, radius=0.8)
    mesh = mesh_from_data(sphere).build()
    acc = Accel()
    acc.emplace_back(mesh)
    acc.emplace_back(cv)
    ident = np.eye(3, 4, dtype=np.float32).reshape(12)
    shifted = ident.copy()
    shifted[3] = 0.4
    acc.emplace_back(cv, shifted.reshape(3, 4))
    acc.build()
    rays = _aimed_rays(rng, np.concatenate([cps[:, :3], sphere.vertices[:, :3]]), 80_000, np.zeros(3))
    d_rays = rays_to_device(rays)
    got = hits_to_numpy(acc.trace_closest(d_rays))
    # oracle: the mesh instance alone (curve slots masked off), the curve instances alone, then the
    # closest of the two with ties to the smaller instance id
    osc = oracle_mod.OracleScene(S.Scene([sphere], np.zeros(3, np.int64), np.stack([ident, ident, shifted]),
                                         np.array([0xFF, 0, 0], np.uint32)))
    wm = osc.trace_closest(rays)
    oc = oracle_mod.OracleCurve(cps, segs, basis)
    wc = oracle_mod.trace_curves([None, oc, oc], np.stack([ident, ident, shifted]), 0xFF, rays)
    take_c = (wc["t"] < wm["t"]) | ((wc["t"] == wm["t"]) & (wc["inst"] < wm["inst"]))
    want = np.where(take_c, wc, wm)
    _check(got, want, min_hits=0.3, curve_inst=[1, 2])
    assert (got["inst"] == 0).sum() > 1000 and (got["inst"] >= 1).sum() > 1000
    tri = got["inst"] == 0
    assert np.all(got["bary"][tri, 1] >= 0.0)  # triangle hits keep their barycentrics
    # a rebuild with moved control points: the accel must be rebuilt, then it sees them
    d_cps[:, 0] += 0.25
    cv.build()
    with pytest.raises(LcxError):
        acc.trace_closest(d_rays)
    acc.build()
    got2 = hits_to_numpy(acc.trace_closest(d_rays))
    cps2 = d_cps.cpu().numpy()
    wc2 = oracle_mod.trace_curves([None, oracle_mod.OracleCurve(cps2, segs, basis)] * 1 +
                                  [oracle_mod.OracleCurve(cps2, segs, basis)], np.stack([ident, ident, shifted]),
                                  0xFF, rays)
    take_c = (wc2["t"] < wm["t"]) | ((wc2["t"] == wm["t"]) & (wc2["inst"] < wm["inst"]))
    _check(got2, np.where(take_c, wc2, wm), min_hits=0.3, curve_inst=[1, 2])
    # a segment whose control points run past the buffer is an error, and the old tree stays usable
    bad = torch.from_numpy(np.array([0, cps.shape[0] - 2], np.int32)).cuda()
    cv_bad = Curve(basis, d_cps, bad)
    with pytest.raises(LcxError):
        cv_bad.build()
    bad_lin = Curve(0, d_cps, torch.from_numpy(np.array([cps.shape[0] - 1], np.int32)).cuda())
    with pytest.raises(LcxError):
        bad_lin.build()
    assert np.array_equal(hits_to_numpy(acc.trace_closest(d_rays)).view(np.uint8), got2.view(np.uint8))
    # Accel.set swaps instance 1 from the curve to a moved copy of the sphere: its hits become triangle hits
    away = ident.copy()
    away[3] = 1.5
    acc.set(1, mesh, away.reshape(3, 4))
    acc.build()
    got3 = hits_to_numpy(acc.trace_closest(d_rays))
    on1 = got3["inst"] == 1
    assert on1.sum() > 100 and np.all(got3["bary"][on1, 1] >= 0.0)
    acc.set_curve(1, cv)
    acc.set_transform_on_update(1, ident.reshape(3, 4))
    acc.build()
    assert np.array_equal(hits_to_numpy(acc.trace_closest(d_rays)).view(np.uint8), got2.view(np.uint8))


def test_curve_motion_instance(lcx, oracle_mod):
    """A motion instance of a curve: at time tau the matrix is the per-element interpolation of its
    keyframes, so the oracle traces the curve with that matrix."""
    import torch
    from luisacompute_gb300.accel import Accel, Curve, MotionInstance, hits_to_numpy, rays_to_device
    rng = np.random.default_rng(731)
    basis = 1
    cps = S.hair_curves(48, 9, rng)
    segs = S.curve_segments(48, 9, basis)
    cv = Curve(basis, torch.from_numpy(cps).cuda(), torch.from_numpy(segs.astype(np.int32)).cuda()).build()
    k0 = np.eye(3, 4, dtype=np.float32)
    k1 = k0.copy()
    k1[:, 3] = [0.6, -0.2, 0.1]
    mo = MotionInstance(cv, np.stack([k0, k1]), 0.0, 1.0)
    acc = Accel()
    acc.emplace_back(mo)
    acc.build()
    tau = 0.25
    m = (k0 + np.float32(tau) * (k1 - k0)).reshape(12)
    world = cps[:, :3] + m.reshape(3, 4)[:, 3]
    rays = _aimed_rays(rng, world, 60_000, world.mean(0))
    times = torch.full((rays.shape[0],), tau, dtype=torch.float32, device="cuda")
    got = hits_to_numpy(acc.trace_closest_motion(rays_to_device(rays), times))
    want = oracle_mod.trace_curves([oracle_mod.OracleCurve(cps, segs, basis)], m.reshape(1, 12), 0xFF, rays)
    _check(got, want, min_hits=0.1)


def test_keyframed_curves_match_oracle(lcx, oracle_mod):
    """Curves with keyframed control points (three keyframes, each a perturbed copy of the strands):
    traced at times inside, before and after the range and NaN, with and without vanishing, under an
    instance transform, against the oracle's interpolation of the Bezier points."""
    import torch
    from luisacompute_gb300.accel import Accel, Curve, hits_to_numpy, rays_to_device
    rng = np.random.default_rng(741)
    basis, n_curves, n_cp, keys = 2, 48, 9, 3
    base = S.hair_curves(n_curves, n_cp, rng)
    frames = [base]
    for _ in range(keys - 1):  # each later keyframe moves every control point a little (radii kept)
        jitter = np.zeros_like(base)
        jitter[:, :3] = rng.normal(0.0, 0.05, (base.shape[0], 3))
        frames.append(base + jitter)
    cps = np.concatenate(frames).astype(np.float32)
    segs = S.curve_segments(n_curves, n_cp, basis)
    d_cps = torch.from_numpy(cps).cuda()
    d_segs = torch.from_numpy(segs.astype(np.int32)).cuda()
    aff = S.affine_rows(S.random_rotations(1, rng), np.array([1.1]), np.array([[0.2, -0.1, 0.3]]))[0]
    rays = _aimed_rays(rng, base[:, :3] @ aff.reshape(3, 4)[:, :3].T + aff.reshape(3, 4)[:, 3], 60_000,
                       aff.reshape(3, 4)[:, 3])
    times = rng.uniform(-0.3, 1.3, rays.shape[0]).astype(np.float32)
    times[:16] = np.nan
    d_rays, d_times = rays_to_device(rays), torch.from_numpy(times).cuda()
    for vanish in (False, True):
        cv = Curve(basis, d_cps, d_segs, motion_keyframes=keys, time_start=0.0, time_end=1.0,
                   vanish_start=vanish, vanish_end=vanish).build()
        acc = Accel()
        acc.emplace_back(cv, aff.reshape(3, 4))
        acc.build()
        oc = oracle_mod.OracleCurve(cps, segs, basis, keyframes=keys, vanish_start=vanish, vanish_end=vanish)
        want = oracle_mod.trace_curves([oc], aff.reshape(1, 12), 0xFF, rays, times=times)
        got = hits_to_numpy(acc.trace_closest_motion(d_rays, d_times))
        _check(got, want, min_hits=0.05)
        occ = acc.trace_any_motion(d_rays, d_times).cpu().numpy()
        want_any = oracle_mod.trace_curves([oc], aff.reshape(1, 12), 0xFF, rays, times=times, any_hit=True)
        assert (occ != want_any).mean() <= 2e-3
        outside = (times < 0.0) | (times > 1.0)
        if vanish:
            assert np.all(got["inst"][outside] == INV)
        else:
            assert np.any(got["inst"][outside] != INV)
    # the control point count must be a whole number of keyframes
    from luisacompute_gb300 import LcxError
    with pytest.raises(LcxError):
        Curve(basis, d_cps[:-1], d_segs, motion_keyframes=keys).build()


def test_curves_in_multi_job_launches(lcx):
    """lcx_trace_jobs with a curve accel among its jobs: the group runs the curve kernel, and every
    job's records equal its own lcx_trace_closest / lcx_trace_any call, bit for bit."""
    import ctypes
    import torch
    from luisacompute_gb300 import _capi
    from luisacompute_gb300.accel import Accel, Curve, hits_to_numpy, mesh_from_data, rays_to_device
    rng = np.random.default_rng(751)
    cps = S.hair_curves(64, 9, rng)
    cv = Curve(1, torch.from_numpy(cps).cuda(),
               torch.from_numpy(S.curve_segments(64, 9, 1).astype(np.int32)).cuda()).build()
    curves = Accel()
    curves.emplace_back(cv)
    curves.build()
    mesh = mesh_from_data(S.icosphere(4, radius=0.9)).build()
    tris = Accel()
    tris.emplace_back(mesh)
    tris.build()
    rays = [rays_to_device(_aimed_rays(rng, cps[:, :3], 40_000, np.zeros(3))) for _ in range(2)]
    outs = [torch.empty((40_000, 6), dtype=torch.int32, device="cuda") for _ in range(2)]
    occ = torch.empty(40_000, dtype=torch.uint8, device="cuda")
    jobs = (_capi.LcxTraceJob * 3)(
        _capi.LcxTraceJob(curves.handle, rays[0].data_ptr(), outs[0].data_ptr(), 40_000, 0xFF, 0, 0),
        _capi.LcxTraceJob(tris.handle, rays[1].data_ptr(), outs[1].data_ptr(), 40_000, 0xFF, 0, 0),
        _capi.LcxTraceJob(curves.handle, rays[1].data_ptr(), occ.data_ptr(), 40_000, 0xFF, 1, 0))
    for layout in (0, 1):
        _capi.check(_capi.load().lcx_trace_jobs(jobs, 3, layout, None), "lcx_trace_jobs")
        torch.cuda.synchronize()
        for k, acc in enumerate((curves, tris)):
            want = hits_to_numpy(acc.trace_closest(rays[k], layout=layout))
            assert np.array_equal(hits_to_numpy(outs[k]).view(np.uint8), want.view(np.uint8)), (layout, k)
        assert torch.equal(occ, curves.trace_any(rays[1], layout=layout))
    assert (hits_to_numpy(outs[0])["inst"] == 0).mean() > 0.1


def test_curve_edge_cases(lcx, oracle_mod):
    """A curve with no segments (its instance is empty), a strand of zero radius (never hit), and a
    segment with NaN control points (never hit; the other segments of the same curve still are)."""
    import torch
    from luisacompute_gb300.accel import Accel, Curve, hits_to_numpy, rays_to_device
    empty = Curve(0, torch.zeros((2, 4), dtype=torch.float32, device="cuda"),
                  torch.zeros(0, dtype=torch.int32, device="cuda")).build()
    assert empty.stats().leaf_prim_count == 0
    thin = np.array([[0, 0, 0, 0.0], [1, 0, 0, 0.0]], np.float32)
    thin_cv = Curve(0, torch.from_numpy(thin).cuda(), torch.zeros(1, dtype=torch.int32, device="cuda")).build()
    pts = np.array([[0, 0, 0, 0.1], [1, 0, 0, 0.1], [np.nan, 0, 0, 0.1], [3, 0, 0, 0.1]], np.float32)
    nan_cv = Curve(0, torch.from_numpy(pts).cuda(), torch.arange(3, dtype=torch.int32, device="cuda")).build()
    acc = Accel()
    acc.emplace_back(empty)
    acc.emplace_back(thin_cv, np.array([[1, 0, 0, 0], [0, 1, 0, 0], [0, 0, 1, 2]], np.float32))
    acc.emplace_back(nan_cv)
    acc.build()
    rays = np.zeros(4, S.RAY_DTYPE)
    rays["o"] = [[0.5, 1, 0], [1.5, 1, 0], [2.5, 1, 0], [0.5, 1, 2]]
    rays["d"] = [0, -1, 0]
    rays["tmax"] = 1e30
    got = hits_to_numpy(acc.trace_closest(rays_to_device(rays)))
    assert got["inst"][0] == 2 and got["prim"][0] == 0 and abs(got["t"][0] - 0.9) < 1e-5
    assert list(got["inst"][1:]) == [0xFFFFFFFF] * 3  # NaN segments, and the zero-radius strand
