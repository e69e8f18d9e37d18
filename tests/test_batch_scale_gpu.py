"""The batched-build workload at full scale: all 4096 meshes (log-uniform 64..262,144 triangles,
135M triangles) built with one lcx_mesh_build_batch, and a TLAS over 100,000 random affine
instances of them -- the configuration the batched-build benchmark times.

The oracle cannot hold the whole scene in a test's time, so a sample of 48 instances carries
visibility mask 0x01 and every other instance 0xFE: rays with mask 0x01 see exactly the sample
through the full TLAS, and the oracle builds a scene of the sample alone.  The GPU's records
(instance ids are TLAS slots) must equal the oracle's (mapped back to slots) bit for bit, for
closest and any hit; mask 0xFF rays through the same instances check that the other instances
are really there."""
import numpy as np
import pytest

from luisacompute_gb300 import scenes as S

pytestmark = pytest.mark.gpu


def _aimed_rays(rng, centres, radii, per):
    """`per` rays at each instance: origins on a sphere of 3 radii around it, aimed at a point
    within one radius of its centre."""
    n = centres.shape[0] * per
    c = np.repeat(centres, per, axis=0)
    r = np.repeat(radii, per)[:, None]
    u = rng.standard_normal((n, 3))
    u /= np.linalg.norm(u, axis=1, keepdims=True)
    o = c + 3.0 * r * u
    target = c + r * rng.uniform(-1, 1, (n, 3))
    d = target - o
    rays = np.zeros(n, S.RAY_DTYPE)
    rays["o"] = o.astype(np.float32)
    rays["d"] = d.astype(np.float32)
    rays["tmin"] = 0.0
    rays["tmax"] = 1e30
    return rays


def test_4096_meshes_and_100k_instances(lcx, oracle_mod):
    import torch
    from luisacompute_gb300.accel import Accel, build_meshes, hits_to_numpy, mesh_from_data, rays_to_device
    datas = S.batch_meshes(4096, seed=6)
    meshes = [mesh_from_data(m) for m in datas]
    build_meshes(meshes)
    rng = np.random.default_rng(7)
    n_inst = 100_000
    pick = rng.integers(0, len(meshes), n_inst)
    scale = np.exp(rng.uniform(np.log(0.5), np.log(2.0), n_inst))
    aff = S.affine_rows(S.random_rotations(n_inst, rng), scale, rng.uniform(-50, 50, (n_inst, 3)))
    sample = np.sort(rng.choice(n_inst, 48, replace=False))
    masks = np.full(n_inst, 0xFE, np.uint32)
    masks[sample] = 0x01
    acc = Accel()
    acc.emplace_back_many([meshes[i] for i in pick], aff, masks)
    acc.build()
    torch.cuda.synchronize()
    assert int(acc.stats().leaf_prim_count) == n_inst

    # the sample alone, on the CPU
    uniq, local = np.unique(pick[sample], return_inverse=True)
    osc = oracle_mod.OracleScene(S.Scene([datas[u] for u in uniq], local, aff[sample],
                                         np.full(sample.size, 0xFF, np.uint32)))
    centres = aff[sample].reshape(-1, 3, 4)[:, :, 3].astype(np.float64)
    rays = _aimed_rays(rng, centres, 1.2 * scale[sample], 2000)
    d = rays_to_device(rays)
    got = hits_to_numpy(acc.trace_closest(d, mask=0x01))
    occ = acc.trace_any(d, mask=0x01).cpu().numpy()
    every = hits_to_numpy(acc.trace_closest(d, mask=0xFF))
    torch.cuda.synchronize()
    from luisacompute_gb300 import _capi
    _capi.check(lcx.lcx_check_trace_errors(), "lcx_check_trace_errors")
    want = osc.trace_closest(rays)
    hit = want["inst"] != S.MISS
    want["inst"][hit] = sample[want["inst"][hit]]  # oracle instance k is TLAS slot sample[k]
    assert np.array_equal(got.view(np.uint8), want.view(np.uint8))
    assert np.array_equal(occ, osc.trace_any(rays))
    assert hit.mean() > 0.3
    # with every instance visible, some rays end on instances outside the sample, never farther
    other = every["inst"] != S.MISS
    assert (~np.isin(every["inst"][other], sample)).sum() > 0
    assert np.all(every["t"][hit] <= got["t"][hit])
