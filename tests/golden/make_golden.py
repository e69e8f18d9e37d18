"""Generates tests/golden/cornell_box.npz: seeded inputs and the oracle's outputs on the
Cornell box of the reference's own tests.

Run from the repository root, with the path of a LuisaCompute checkout (required):

    python tests/golden/make_golden.py path/to/LuisaCompute

Scene.  The geometry is the OBJ text that LuisaCompute's path-tracing tests embed
(src/tests/common/cornell_box.h; "Released into the Public Domain" by its authors,
Cardenas and McGuire, Williams College 2011).  As in src/tests/test_path_tracing.cpp:40-92,
every `g` group becomes one mesh over ONE shared vertex buffer, each placed by an identity
instance, in file order (floor, ceiling, backWall, rightWall, leftWall, shortBox, tallBox,
light).  Quads are split as fans, (a, b, c) and (a, c, d).  The camera follows that test
(eye (-0.01, 0.995, 5.0) looking down -z, 27.8 degree vertical field of view).

Outputs.  The hit records come from the oracle (oracle/, the CPU restatement of the
reference's CPU-backend ray queries).  The reference itself cannot run here, so these
vectors pin the oracle (across compilers and CPU architectures) and the CUDA path to one
fixed set of answers; they are not outputs of the reference.
"""
from __future__ import annotations

import json
import re
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from luisacompute_gb300 import scenes as S  # noqa: E402

OUT = Path(__file__).resolve().parent / "cornell_box.npz"
EYE = (-0.01, 0.995, 5.0)
TARGET = (-0.01, 0.995, 0.0)
FOV_DEG = 27.8
LIGHT = (-0.005, 1.90, -0.03)  # just under the ceiling light's quad
PT = dict(width=48, height=48, spp=2, max_bounces=6, rr_start=3, seed=7, eye=EYE, target=TARGET,
          up=(0.0, 1.0, 0.0), fov_deg=FOV_DEG, light_pos=LIGHT, light_intensity=(3.4, 2.4, 0.8),
          env=(0.02, 0.02, 0.03))
# Mean reflectance of each group's colour in the reference test (test_path_tracing.cpp:95-104).
GROUP_ALBEDO = {"floor": 0.705, "ceiling": 0.705, "backWall": 0.705, "rightWall": 0.227,
                "leftWall": 0.248, "shortBox": 0.705, "tallBox": 0.705, "light": 0.0}


def parse_obj(text: str):
    """OBJ subset of the fixture: `v x y z`, `g name`, `f` with negative (relative) indices."""
    verts, groups = [], []
    for line in text.splitlines():
        tok = line.split()
        if not tok or tok[0].startswith("#"):
            continue
        if tok[0] == "v":
            verts.append([float(x) for x in tok[1:4]])
        elif tok[0] == "g":
            groups.append((tok[1], []))
        elif tok[0] == "f":
            idx = [int(x.split("/")[0]) for x in tok[1:]]
            idx = [i - 1 if i > 0 else len(verts) + i for i in idx]
            for k in range(1, len(idx) - 1):
                groups[-1][1].append((idx[0], idx[k], idx[k + 1]))
    v = np.zeros((len(verts), 4), np.float32)
    v[:, :3] = np.asarray(verts, np.float32)
    return v, [(name, np.asarray(tris, np.uint32)) for name, tris in groups]


def cornell_scene(vertices: np.ndarray, groups, masks=None) -> S.Scene:
    meshes = [S.MeshData(vertices, tris) for _, tris in groups]
    n = len(meshes)
    aff = np.tile(S.IDENTITY, (n, 1))
    mk = np.full(n, 0xFF, np.uint32) if masks is None else np.asarray(masks, np.uint32)
    return S.Scene(meshes, np.arange(n), aff, mk, name="cornell_box")


def rays_for(scene: S.Scene):
    lo, hi = scene.bounds()
    cam = S.camera_rays(64, 64, eye=EYE, target=TARGET, fov_deg=FOV_DEG, seed=11)
    inc = S.sphere_rays(4096, lo, hi, seed=12)
    sh = S.shadow_rays(4096, lo, hi, LIGHT, seed=13)
    return cam, inc, sh


def main(ref_root: Path):
    import oracle
    from luisacompute_gb300 import pathtrace as P
    oracle.build()
    src = (ref_root / "src/tests/common/cornell_box.h").read_text()
    text = re.search(r'R"\((.*)\)"', src, re.S).group(1)
    vertices, groups = parse_obj(text)
    scene = cornell_scene(vertices, groups)
    cam, inc, sh = rays_for(scene)
    orc = oracle.OracleScene(scene)
    hits_cam = orc.trace_closest(cam)
    hits_inc = orc.trace_closest(inc)
    occ_sh = orc.trace_any(sh)
    # Masks: instance i visible to ray-mask bit i only; the rays carry 0b0101_0101.
    mscene = cornell_scene(vertices, groups, masks=[1 << i for i in range(len(groups))])
    morc = oracle.OracleScene(mscene)
    hits_mask = morc.trace_closest(inc, mask=0x55)
    occ_mask = morc.trace_any(sh, mask=0x55)
    albedo = [np.full(t.shape[0], GROUP_ALBEDO[name], np.float32) for name, t in groups]
    prm = P.params(**PT)
    image, first = orc.pathtrace(scene, albedo, prm)
    np.savez_compressed(
        OUT, vertices=vertices, group_names=np.array([g[0] for g in groups]),
        tri_counts=np.array([g[1].shape[0] for g in groups], np.uint32),
        triangles=np.concatenate([g[1] for g in groups]), albedo=np.concatenate(albedo),
        rays_camera=cam, hits_camera=hits_cam, rays_incoherent=inc, hits_incoherent=hits_inc,
        rays_shadow=sh, occluded_shadow=occ_sh, hits_mask55=hits_mask, occluded_mask55=occ_mask,
        pt_params=np.array(json.dumps(PT)), pt_image=image, pt_first_hits=first)
    print(f"wrote {OUT} ({OUT.stat().st_size} B): {len(groups)} meshes, {vertices.shape[0]} vertices, "
          f"{sum(g[1].shape[0] for g in groups)} triangles; camera hits "
          f"{int((hits_cam['inst'] != S.MISS).sum())}/{cam.shape[0]}, occluded {int(occ_sh.sum())}/{sh.shape[0]}")


def load():
    """The fixture as (scene, masked scene, arrays) for the tests."""
    z = np.load(OUT, allow_pickle=False)
    names = [str(x) for x in z["group_names"]]
    off = np.concatenate([[0], np.cumsum(z["tri_counts"].astype(np.int64))])
    groups = [(names[i], z["triangles"][off[i]:off[i + 1]]) for i in range(len(names))]
    v = z["vertices"]
    scene = cornell_scene(v, groups)
    mscene = cornell_scene(v, groups, masks=[1 << i for i in range(len(groups))])
    albedo = [z["albedo"][off[i]:off[i + 1]] for i in range(len(names))]
    return scene, mscene, albedo, json.loads(str(z["pt_params"])), z


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py <path of the LuisaCompute checkout>")
    main(Path(sys.argv[1]))
