"""Autotuner for the build and traversal knobs of the Mesh/Accel path.

It measures, on the caller's own scene and rays, and picks:

* build knobs (``lcx_set_build_tuning`` / ``lcx_set_build_morton``):
  - node width: children per wide node, 2..8;
  - leaf size: items per leaf slot, 1..3 (the collapse schedule: subtrees of at most this many
    triangles become leaf slots, everything larger is opened);
  - BLAS builder of FAST_TRACE meshes: binned SAH or Morton LBVH (``lcx_set_build_blas_sah``);
  - collapse to wide nodes: dynamic program or greedy (``lcx_set_build_collapse``);
  - Morton normalisation of BLAS centroids (LBVH builds): by the largest extent ("cube") or per axis;
  - triangle splitting of FAST_TRACE meshes: extra references as a fraction of the triangles.
* traversal knobs (``lcx_set_trace_tuning`` / ``lcx_set_trace_stack`` / ``lcx_set_trace_reorder``):
  - ray-pool refill threshold: the number of idle lanes at which a warp takes new rays, 1..32;
  - shared-memory stack depth: 8, 16 or 24 entries per thread;
  - loop structure: 2 (deferred triangle batches, the default), 0 (node + its items per step),
    1 (speculative while-while) or 3 (one ray per thread through the device-side trace functions);
  - mode 2's flush size (``postpone``): 0 (24 closest / 16 any), 12 or 32 queued tests;
  - ray reordering: off, or sorted by octant and 7-bit origin Morton cell.

Search: coordinate descent, build knobs first (each trial builds every mesh with one batched
build plus the TLAS), then traversal knobs on the best build.  A trial's score is

    trace_ms(sample) * rays_per_build / sample_rays + build_ms

so ``rays_per_build=None`` (a static scene) ranks by traversal time alone, and a small value
favours fast builds (serving many short-lived scenes).  Traversal time is the median over
``reps`` CUDA-event timings of closest-hit (plus any-hit when ``any_rays`` is given) with the
L2 flushed before each.  Knobs never change results: every setting gives the same hit records.
The tuned values stay applied (they are process-wide settings of the library) and are returned
with the table of trials; ``save``/``load`` keep them in a JSON file keyed by GPU and scene size.
"""
from __future__ import annotations

import ctypes
import json
import math
import time
from dataclasses import asdict, dataclass, field, replace
from pathlib import Path

from . import _capi
from .accel import NODES_QUANT8, Accel, build_meshes, mesh_from_data

BUILD_SPACE = {"blas_sah": [1, 0], "collapse": [1, 0], "leaf_max": [1, 2, 3], "width": [8, 6, 4],
               "blas_cube": [1, 0], "split": [0.0, 1.0, 3.0]}
TRACE_SPACE = {"refill": [1, 2, 4, 8, 16, 32], "short_stack": [8, 16, 24], "mode": [2, 0, 1, 3], "postpone": [0, 12, 32],
               "reorder_bits": [0, 7]}


@dataclass
class Config:
    leaf_max: int = 0  # 0: from the AccelOption hint
    width: int = 8
    blas_cube: int = 1
    refill: int = 4
    short_stack: int = 16
    mode: int = 2
    reorder_bits: int = 0
    postpone: int = 0
    split: float = 0.0
    blas_sah: int = 1
    collapse: int = 1


@dataclass
class TuneResult:
    config: Config
    default_ms: float
    tuned_ms: float
    trials: list = field(default_factory=list)
    seconds: float = 0.0

    def to_json(self) -> dict:
        return {"config": asdict(self.config), "default_ms": self.default_ms, "tuned_ms": self.tuned_ms,
                "speedup": self.default_ms / self.tuned_ms if self.tuned_ms > 0 else None,
                "trials": len(self.trials), "seconds": self.seconds}


def _u32(n):
    return [ctypes.c_uint32(0) for _ in range(n)]


def current() -> Config:
    """The knob values the library uses now."""
    lib = _capi.load()
    lm, w = _u32(2)
    _capi.check(lib.lcx_get_build_tuning(lm, w), "lcx_get_build_tuning")
    bc, tc, sb = _u32(3)
    _capi.check(lib.lcx_get_build_morton(bc, tc, sb), "lcx_get_build_morton")
    rf, pp, md = _u32(3)
    _capi.check(lib.lcx_get_trace_tuning(rf, pp, md), "lcx_get_trace_tuning")
    (ss,) = _u32(1)
    _capi.check(lib.lcx_get_trace_stack(ss), "lcx_get_trace_stack")
    rb, rm = _u32(2)
    _capi.check(lib.lcx_get_trace_reorder(rb, rm), "lcx_get_trace_reorder")
    sp = ctypes.c_float(0.0)
    _capi.check(lib.lcx_get_build_split(ctypes.byref(sp)), "lcx_get_build_split")
    (bs,) = _u32(1)
    _capi.check(lib.lcx_get_build_blas_sah(bs), "lcx_get_build_blas_sah")
    (cm,) = _u32(1)
    _capi.check(lib.lcx_get_build_collapse(cm), "lcx_get_build_collapse")
    return Config(lm.value, w.value, bc.value, rf.value, ss.value, md.value, rb.value, pp.value,
                  round(sp.value, 6), bs.value, cm.value)


def apply(cfg: Config):
    """Sets every knob of ``cfg`` (builds and traces issued afterwards use them)."""
    lib = _capi.load()
    bc, tc, sb = _u32(3)
    _capi.check(lib.lcx_get_build_morton(bc, tc, sb), "lcx_get_build_morton")
    rb, rm = _u32(2)
    _capi.check(lib.lcx_get_trace_reorder(rb, rm), "lcx_get_trace_reorder")
    _capi.check(lib.lcx_set_build_tuning(cfg.leaf_max, cfg.width), "lcx_set_build_tuning")
    _capi.check(lib.lcx_set_build_morton(cfg.blas_cube, tc.value, sb.value), "lcx_set_build_morton")
    _capi.check(lib.lcx_set_build_split(ctypes.c_float(cfg.split)), "lcx_set_build_split")
    _capi.check(lib.lcx_set_build_blas_sah(cfg.blas_sah), "lcx_set_build_blas_sah")
    _capi.check(lib.lcx_set_build_collapse(cfg.collapse), "lcx_set_build_collapse")
    _capi.check(lib.lcx_set_trace_tuning(cfg.refill, cfg.postpone, cfg.mode), "lcx_set_trace_tuning")
    _capi.check(lib.lcx_set_trace_stack(cfg.short_stack), "lcx_set_trace_stack")
    _capi.check(lib.lcx_set_trace_reorder(cfg.reorder_bits, rm.value), "lcx_set_trace_reorder")


class _Bench:
    """The scene's meshes on the device, builds under a config, timed traces."""

    def __init__(self, scene, rays, any_rays, reps, layout):
        import torch
        self.torch = torch
        self.scene = scene
        self.meshes = [mesh_from_data(m) for m in scene.meshes]
        self.rays, self.any_rays = rays, any_rays
        n = rays.shape[0]
        self.hits = torch.empty((n, 6), dtype=torch.int32, device="cuda")
        self.occ = torch.empty(any_rays.shape[0] if any_rays is not None else 1, dtype=torch.uint8, device="cuda")
        self.flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
        self.reps, self.layout = reps, layout
        self.acc = None

    def _events(self, fn):
        t = self.torch
        e0, e1 = t.cuda.Event(enable_timing=True), t.cuda.Event(enable_timing=True)
        e0.record()
        fn()
        e1.record()
        t.cuda.synchronize()
        return e0.elapsed_time(e1)

    def build(self):
        def run():
            build_meshes(self.meshes)
            acc = Accel()
            acc.emplace_back_many([self.meshes[i] for i in self.scene.inst_mesh], self.scene.inst_affine,
                                  self.scene.inst_mask)
            acc.build()
            self.acc_new = acc
        ms = self._events(run)
        if self.acc is not None:
            self.acc.destroy()
        self.acc = self.acc_new
        return ms

    def trace(self):
        def one():
            self.acc.trace_closest(self.rays, out=self.hits, layout=self.layout)
            if self.any_rays is not None:
                self.acc.trace_any(self.any_rays, out=self.occ, layout=self.layout)
        one()  # warm-up (kernel selection, reorder scratch pool)
        times = []
        for _ in range(self.reps):
            self.flush.zero_()
            times.append(self._events(one))
        times.sort()
        return times[len(times) // 2]

    def close(self):
        if self.acc is not None:
            self.acc.destroy()
        for m in self.meshes:
            m.destroy()


def tune(scene, rays, any_rays=None, *, rays_per_build=None, reps: int = 3, layout: int = NODES_QUANT8,
         build_space: dict | None = None, trace_space: dict | None = None, log=None) -> TuneResult:
    """Tunes the knobs for ``scene`` (scenes.Scene) and the device ray tensors ``rays``
    (closest) and ``any_rays`` (any hit, optional).  Leaves the best configuration applied."""
    t_start = time.perf_counter()
    build_space = BUILD_SPACE if build_space is None else build_space
    trace_space = TRACE_SPACE if trace_space is None else trace_space
    n_sample = rays.shape[0] + (any_rays.shape[0] if any_rays is not None else 0)
    scale = (rays_per_build / n_sample) if rays_per_build else None
    B = _Bench(scene, rays, any_rays, reps, layout)
    trials = []

    def score(cfg, rebuild):
        apply(cfg)
        b_ms = B.build() if rebuild else float("nan")
        t_ms = B.trace()
        s = t_ms * scale + b_ms if scale is not None else t_ms
        trials.append({**asdict(cfg), "build_ms": b_ms, "trace_ms": t_ms, "score": s})
        if log:
            log(f"autotune {asdict(cfg)} build {b_ms:.2f} ms trace {t_ms:.3f} ms")
        return s

    try:
        start = current()
        if start.leaf_max == 0:
            start = replace(start, leaf_max=2)
        best, best_s = start, score(start, True)
        default_ms = trials[-1]["trace_ms"]
        for knob, values in build_space.items():
            for v in values:
                if getattr(best, knob) == v:
                    continue
                cand = replace(best, **{knob: v})
                s = score(cand, True)
                if s < best_s:
                    best, best_s = cand, s
        score(best, True)  # the winning build stays resident for the traversal stage
        best_s = trials[-1]["score"]
        for knob, values in trace_space.items():
            for v in values:
                if getattr(best, knob) == v:
                    continue
                cand = replace(best, **{knob: v})
                s = score(cand, False)
                if s < best_s:
                    best, best_s = cand, s
        apply(best)
        tuned_ms = min(t["trace_ms"] for t in trials if all(t[k] == v for k, v in asdict(best).items()))
    finally:
        B.close()
    return TuneResult(best, default_ms, tuned_ms, trials, time.perf_counter() - t_start)


def signature(scene) -> str:
    """GPU name + log2 buckets of triangle and instance counts."""
    import torch
    tris = sum(m.tri_count for m in scene.meshes)
    return (f"{torch.cuda.get_device_name()}|tris2^{int(math.log2(max(tris, 1)))}"
            f"|inst2^{int(math.log2(max(scene.instance_count, 1)))}")


def save(path, scene, result: TuneResult):
    p = Path(path)
    data = json.loads(p.read_text()) if p.exists() else {}
    data[signature(scene)] = asdict(result.config)
    p.write_text(json.dumps(data, indent=1, sort_keys=True))


def load(path, scene) -> Config | None:
    """The saved configuration for this GPU and scene size, applied; None if there is none."""
    p = Path(path)
    if not p.exists():
        return None
    cfg = json.loads(p.read_text()).get(signature(scene))
    if cfg is None:
        return None
    c = Config(**cfg)
    apply(c)
    return c


def tune_batch_build(datas, *, sample: int = 512, reps: int = 3, sah_slack: float = 0.10,
                     space: dict | None = None, log=None) -> TuneResult:
    """Tunes the build knobs for batched BLAS builds (``lcx_mesh_build_batch``) on the first
    ``sample`` meshes of ``datas`` (scenes.MeshData): among every point of the grid ``space``
    (BLAS builder x leaf size x node width x Morton normalisation) whose mean wide-BVH SAH is within
    ``sah_slack`` of the best one, the fastest build wins.  Build time is the median of
    ``reps`` CUDA-event timings.  Leaves the winner applied; ``default_ms`` / ``tuned_ms`` are
    the build times of the starting and the chosen configuration."""
    import itertools

    import torch
    t_start = time.perf_counter()
    # triangle splitting is a traversal-quality knob: on displaced meshes it wins the SAH
    # criterion at several times the build time, so batched builds keep it at its current value
    space = {k: v for k, v in BUILD_SPACE.items() if k != "split"} if space is None else space
    meshes = [mesh_from_data(m) for m in datas[:sample]]
    start = current()
    trials = []
    try:
        keys = list(space)
        grid = [dict(zip(keys, vals)) for vals in itertools.product(*(space[k] for k in keys))]
        for point in grid:
            cfg = replace(start, **point)
            apply(cfg)
            build_meshes(meshes)  # warm-up
            times = []
            for _ in range(reps):
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record()
                build_meshes(meshes)
                e1.record()
                torch.cuda.synchronize()
                times.append(e0.elapsed_time(e1))
            times.sort()
            sah = [m.stats().wide_sah_cost for m in meshes]
            trials.append({**asdict(cfg), "build_ms": times[len(times) // 2], "mean_wide_sah": float(sum(sah) / len(sah))})
            if log:
                log(f"autotune build {point}: {trials[-1]['build_ms']:.2f} ms, SAH {trials[-1]['mean_wide_sah']:.3f}")
        best_sah = min(t["mean_wide_sah"] for t in trials)
        ok = [t for t in trials if t["mean_wide_sah"] <= best_sah * (1.0 + sah_slack)]
        win = min(ok, key=lambda t: t["build_ms"])
        best = Config(**{k: win[k] for k in asdict(start)})
        apply(best)
        ref = replace(start, leaf_max=start.leaf_max or 1)
        default = [t for t in trials if all(t[k] == v for k, v in asdict(ref).items())]
        default_ms = default[0]["build_ms"] if default else float("nan")
    finally:
        for m in meshes:
            m.destroy()
    return TuneResult(best, default_ms, win["build_ms"], trials, time.perf_counter() - t_start)
