"""The curve oracle (lcxo_trace_curves) against closed-form cases, and the segment tables of
luisacompute_gb300.scenes (CPU only).

Closed forms: a ray straight down onto a horizontal strand of radius r meets its side at
t = height - r; past an end it meets only the end ball (linear segments: spherical caps,
include/luisa/runtime/rhi/curve_basis.h:12-13; cubic ones are open there, :14-22); a round cone
from radius ra to rb over length L has its side at rho = (ra - s sin) / cos with sin = (ra - rb) / L."""
import numpy as np

from luisacompute_gb300 import scenes as S

INV = 0xFFFFFFFF
IDENT = np.eye(3, 4, dtype=np.float32).reshape(1, 12)


def _rays(origins, d=(0.0, -1.0, 0.0), tmin=0.0, tmax=1e30):
    r = np.zeros(len(origins), S.RAY_DTYPE)
    r["o"] = origins
    r["d"] = d
    r["tmin"] = tmin
    r["tmax"] = tmax
    return r


def test_linear_strand_side_caps_and_inside(oracle_mod):
    c = oracle_mod.OracleCurve(np.array([[0, 0, 0, 0.1], [1, 0, 0, 0.1]], np.float32), np.array([0]), 0)
    h = oracle_mod.trace_curves([c], IDENT, 0xFF, _rays([[0.5, 1, 0], [1.05, 1, 0], [2, 1, 0], [0.5, 0, 0]]))
    assert list(h["inst"]) == [0, 0, INV, INV]
    assert abs(h["t"][0] - 0.9) < 1e-6 and abs(h["bary"][0, 0] - 0.5) < 1e-6 and h["bary"][0, 1] == -1.0
    assert abs(h["t"][1] - (1.0 - np.sqrt(0.01 - 0.0025))) < 1e-6 and h["bary"][1, 0] == 1.0
    assert h["t"][2] == np.float32(1e30) and h["prim"][2] == INV
    occ = oracle_mod.trace_curves([c], IDENT, 0xFF, _rays([[0.5, 1, 0], [2, 1, 0]]), any_hit=True)
    assert list(occ) == [1, 0]
    # t range: the side at t = 0.9 lies outside [0, 0.85]
    assert oracle_mod.trace_curves([c], IDENT, 0xFF, _rays([[0.5, 1, 0]], tmax=0.85))["inst"][0] == INV


def test_cubic_strand_is_open_at_free_ends(oracle_mod):
    pts = np.array([[0, 0, 0, 0.1], [1 / 3, 0, 0, 0.1], [2 / 3, 0, 0, 0.1], [1, 0, 0, 0.1]], np.float32)
    c = oracle_mod.OracleCurve(pts, np.array([0]), 3)
    assert c.pieces()[0] == 1  # straight: one cone
    h = oracle_mod.trace_curves([c], IDENT, 0xFF, _rays([[0.5, 1, 0], [1.05, 1, 0], [-0.05, 1, 0]]))
    assert list(h["inst"]) == [0, INV, INV]
    # two Bezier segments sharing a point: the joint keeps its ball, the free ends stay open
    pts2 = np.concatenate([pts, pts[1:] + np.array([1, 0, 0, 0], np.float32)])
    c2 = oracle_mod.OracleCurve(pts2, np.array([0, 3]), 3)
    h2 = oracle_mod.trace_curves([c2], IDENT, 0xFF, _rays([[1.0, 1, 0], [2.05, 1, 0], [1.5, 1, 0]]))
    assert h2["inst"][0] == 0 and h2["inst"][1] == INV and h2["prim"][2] == 1


def test_tapered_cone_side(oracle_mod):
    ra, rb, L = 0.2, 0.1, 1.0
    c = oracle_mod.OracleCurve(np.array([[0, 0, 0, ra], [L, 0, 0, rb]], np.float32), np.array([0]), 0)
    h = oracle_mod.trace_curves([c], IDENT, 0xFF, _rays([[0.5, 1, 0]]))
    sn = (ra - rb) / L
    cs = np.sqrt(1 - sn * sn)
    rho = (ra - 0.5 * sn) / cs
    assert abs(h["t"][0] - (1 - rho)) < 1e-6
    assert abs(h["bary"][0, 0] - (0.5 - rho * sn / cs) / L) < 1e-6


def test_bases_agree_on_a_shared_strand(oracle_mod):
    """B-spline and Catmull-Rom control points chosen so that both describe the same straight strand
    as the Bezier one: the same rays hit at the same t and u."""
    line = np.array([[-1, 0, 0, 0.1], [0, 0, 0, 0.1], [1, 0, 0, 0.1], [2, 0, 0, 0.1]], np.float32)
    rays = _rays([[x, 1, 0] for x in np.linspace(0.05, 0.95, 19)])
    ref = oracle_mod.trace_curves([oracle_mod.OracleCurve(line[1:3], np.array([0]), 0)],
                                  IDENT, 0xFF, rays)
    for basis in (1, 2):
        h = oracle_mod.trace_curves([oracle_mod.OracleCurve(line, np.array([0]), basis)], IDENT, 0xFF, rays)
        assert np.all(h["inst"] == 0)
        assert np.allclose(h["t"], ref["t"], atol=1e-6) and np.allclose(h["bary"][:, 0], ref["bary"][:, 0], atol=1e-6)


def test_piece_count_tracks_bending(oracle_mod):
    rng = np.random.default_rng(3)
    cps = S.hair_curves(8, 10, rng)
    straight = oracle_mod.OracleCurve(np.array([[0, 0, 0, 0.01], [0.1, 0, 0, 0.01], [0.2, 0, 0, 0.01],
                                                [0.3, 0, 0, 0.01]], np.float32), np.array([0]), 3)
    assert straight.pieces()[0] == 1
    bent = oracle_mod.OracleCurve(cps, S.curve_segments(8, 10, 2), 2).pieces()
    assert bent.min() >= 1 and bent.max() <= 32 and bent.max() > 1


def test_bad_segment_is_rejected(oracle_mod):
    import pytest
    cps = np.zeros((5, 4), np.float32)
    with pytest.raises(ValueError):
        oracle_mod.OracleCurve(cps, np.array([2]), 1)  # needs control points 2..5


def test_curve_segment_tables():
    assert list(S.curve_segments(2, 4, 0)) == [0, 1, 2, 4, 5, 6]
    assert list(S.curve_segments(2, 5, 1)) == [0, 1, 5, 6]
    assert list(S.curve_segments(1, 7, 3)) == [0, 3]
    cps = S.hair_curves(3, 6, np.random.default_rng(1))
    assert cps.shape == (18, 4) and cps.dtype == np.float32 and np.all(cps[:, 3] > 0)


def test_keyframed_strand_moves_and_vanishes(oracle_mod):
    """Two keyframes one unit apart in y: at time tau the strand's top lies at y = tau + r; with
    vanish_end the strand is gone after the range, without it the last keyframe holds."""
    cps = np.array([[0, 0, 0, 0.1], [1, 0, 0, 0.1], [0, 1, 0, 0.1], [1, 1, 0, 0.1]], np.float32)
    times = np.array([0.0, 0.5, 1.5, -1.0], np.float32)
    rays = _rays([[0.5, 3, 0]] * 4)
    gone = oracle_mod.OracleCurve(cps, np.array([0]), 0, keyframes=2, vanish_end=True)
    h = oracle_mod.trace_curves([gone], IDENT, 0xFF, rays, times=times)
    assert list(h["inst"]) == [0, 0, INV, 0]
    assert np.allclose(h["t"][[0, 1, 3]], [2.9, 2.4, 2.9], atol=1e-6)
    held = oracle_mod.OracleCurve(cps, np.array([0]), 0, keyframes=2)
    assert abs(oracle_mod.trace_curves([held], IDENT, 0xFF, rays, times=times)["t"][2] - 1.9) < 1e-6
