"""Wavefront diffuse path tracing through lcx_pt_render (a caller of the Mesh/Accel path)."""
from __future__ import annotations

import ctypes
import math

import numpy as np

from . import _capi
from . import scenes as S
from .accel import stream_handle


def albedos(scene: S.Scene, seed: int = 7):
    """One grey Lambert albedo per triangle, uniform in [0.2, 0.8] (per mesh, seeded)."""
    rng = np.random.default_rng(seed)
    return [rng.uniform(0.2, 0.8, m.tri_count).astype(np.float32) for m in scene.meshes]


def params(width=1920, height=1080, spp=4, max_bounces=8, rr_start=3, seed=7, eye=(0.0, 0.0, 3.0),
           target=(0.0, 0.0, 0.0), up=(0.0, 1.0, 0.0), fov_deg=45.0, light_pos=(0.25, 1.0, -0.25),
           light_intensity=(4.0, 3.8, 3.5), env=(0.18, 0.22, 0.3)) -> _capi.LcxPtParams:
    p = _capi.LcxPtParams()
    p.width, p.height, p.spp, p.max_bounces, p.rr_start, p.seed = width, height, spp, max_bounces, rr_start, seed
    p.eye[:] = eye
    p.target[:] = target
    p.up[:] = up
    p.tan_half_fov = math.tan(math.radians(fov_deg) * 0.5)
    p.light_pos[:] = light_pos
    p.light_intensity[:] = light_intensity
    p.env[:] = env
    return p


def albedos_to_device(albedo_host):
    """The per-mesh albedo arrays as CUDA tensors, for repeated `render` calls."""
    import torch
    return [torch.from_numpy(np.ascontiguousarray(a, np.float32)).cuda() for a in albedo_host]


def render(scene: S.Scene, acc, meshes, albedo_host, prm, first_hits: bool = False, stream=None):
    """Renders `scene` (already built as `acc` over `meshes`); returns (image HxWx3 float32,
    first-bounce hits or None, LcxPtStats).  `albedo_host` holds one float32 array per mesh:
    numpy arrays are uploaded for this call, CUDA tensors (see `albedos_to_device`) are used
    in place."""
    import torch
    lib = _capi.load()
    dev_alb = [a if isinstance(a, torch.Tensor) else torch.from_numpy(a).cuda() for a in albedo_host]
    mt = (_capi.LcxPtMesh * len(meshes))()
    for i, m in enumerate(meshes):
        mt[i] = _capi.LcxPtMesh(m.vertices.data_ptr(), m.vertex_stride, m.triangles.data_ptr(), dev_alb[i].data_ptr())
    inst_mesh = np.ascontiguousarray(scene.inst_mesh, np.uint32)
    inst_o2w = np.ascontiguousarray(scene.inst_affine, np.float32)
    img = torch.empty(prm.height * prm.width * 3, dtype=torch.float32, device="cuda")
    n = prm.width * prm.height * prm.spp
    fh = torch.empty((n, 6), dtype=torch.int32, device="cuda") if first_hits else None
    st = _capi.LcxPtStats()
    _capi.check(lib.lcx_pt_render(acc.handle, mt, len(meshes), inst_mesh.ctypes.data, inst_o2w.ctypes.data,
                                  len(inst_mesh), ctypes.byref(prm), img.data_ptr(),
                                  fh.data_ptr() if fh is not None else None, ctypes.byref(st),
                                  stream_handle(stream)), "lcx_pt_render")
    torch.cuda.synchronize()
    image = img.cpu().numpy().reshape(prm.height, prm.width, 3)
    hits = fh.cpu().numpy().view(S.HIT_DTYPE).reshape(-1) if fh is not None else None
    return image, hits, st


def write_pfm(path, image: np.ndarray):
    """Little-endian PFM (bottom row first), the headless output of a render."""
    h, w, _ = image.shape
    with open(path, "wb") as f:
        f.write(f"PF\n{w} {h}\n-1.0\n".encode())
        f.write(np.ascontiguousarray(image[::-1], np.float32).tobytes())
