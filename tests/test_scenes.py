"""CPU tests of the synthetic workload generators (sizes named by the benchmark configs)."""
import numpy as np

from luisacompute_gb300 import scenes as S


def test_record_layouts():
    assert S.RAY_DTYPE.itemsize == 32 and S.HIT_DTYPE.itemsize == 24 and S.MOD_DTYPE.itemsize == 80


def test_icosphere_counts():
    for s, (nv, nt) in {0: (12, 20), 5: (10242, 20480), 6: (40962, 81920)}.items():
        m = S.icosphere(s)
        assert m.vertices.shape == (nv, 4) and m.triangles.shape == (nt, 3)
        r = np.linalg.norm(m.vertices[:, :3], axis=1)
        assert np.allclose(r, 1.0, atol=1e-6)
        assert m.triangles.max() < nv


def test_heightfield_counts():
    m = S.heightfield(1024)
    assert m.triangles.shape[0] == 2_093_058 and m.vertices.shape[0] == 1024 * 1024
    h = m.vertices[:, 1]
    assert -0.2 <= h.min() and h.max() <= 0.2 and h.std() > 0.01


def test_terrain_scene():
    sc = S.terrain_scene(n=64)
    assert sc.instance_count == 257 and sc.meshes[1].tri_count == 20480
    scale = np.linalg.norm(sc.inst_affine[1:].reshape(-1, 3, 4)[:, :, 0], axis=1)
    assert np.all((scale >= 0.01 - 1e-6) & (scale <= 0.1 + 1e-6))


def test_rays():
    r = S.camera_rays(32, 16)
    assert r.shape == (512,) and np.allclose(np.linalg.norm(r["d"], axis=1), 1, atol=1e-6)
    assert np.all(r["o"] == np.float32([0, 0, 3]))
    s = S.sphere_rays(1000, [-1, -1, -1], [1, 1, 1], seed=4)
    assert np.all(np.abs(s["o"]) <= 1) and np.all(s["tmax"] == np.float32(1e30))
    sh = S.shadow_rays(100, [-1, -1, -1], [1, 1, 1], [0, 2, 0], seed=5)
    end = sh["o"] + sh["d"] * sh["tmax"][:, None]
    assert np.allclose(end, [0, 2, 0], atol=1e-5)


def test_batch_meshes_small():
    ms = S.batch_meshes(16, seed=6)
    assert len(ms) == 16
    for m in ms:
        assert m.triangles.max() < m.vertices.shape[0]
