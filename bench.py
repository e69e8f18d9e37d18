"""Benchmark of the Mesh/Accel hot path on GB300.

Default workload: terrain heightfield (2,093,058 triangles) + 256 instanced 20,480-triangle
icospheres (~7.34 M instanced triangles), 8,388,608 incoherent rays (origins uniform in the
scene box, directions uniform on the sphere), trace_closest.  Metric: Grays/s.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

One step = one trace_closest batch over all rays.  `value` times the kernel with rays
resident in HBM; `e2e` times the same call with the rays in pinned host memory, copied
in and the hits copied out inside the timed region.  `--impl reference` times the CPU
restatement of the reference CPU backend's trace_closest on all host cores (the reference
itself, Rust + Embree, cannot be built here).
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import re
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

from luisacompute_gb300 import scenes as S  # noqa: E402

METRIC = "Grays/s closest-hit (incoherent, ~7M tris)"
UNIT = "Grays/s"
RAYS = 8_388_608
WORKLOAD = ("terrain 1024x1024 heightfield (2,093,058 tris) + 256 instances of a 20,480-tri icosphere "
            "(7,335,938 instanced tris); 8,388,608 incoherent rays; trace_closest")


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--rays", type=int, default=RAYS)
    ap.add_argument("--layout", type=int, default=1, help="0 = FP32 nodes, 1 = 8-bit quantised nodes")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-extra", action="store_true")
    ap.add_argument("--no-autotune", action="store_true",
                    help="skip the autotuner (build and traversal knobs stay at their defaults)")
    ap.add_argument("--workload", default="terrain",
                    choices=["terrain", "batch_build", "serving", "pathtrace", "curves"],
                    help="terrain: the headline trace_closest benchmark; batch_build: 4096 BLAS builds; "
                         "serving: continuous batching vs one request at a time; "
                         "pathtrace: wavefront path tracing 1920x1080x4spp; curves: hair strands as round curves")
    ap.add_argument("--requests", type=int, default=2000)
    ap.add_argument("--rate", type=float, default=800.0, help="serving: Poisson arrival rate (requests/s)")
    ap.add_argument("--warm-split", type=float, default=3.0,
                    help="serving: triangle-splitting fraction for the scenes built before requests arrive "
                         "(0: none; 3.0 measured p99 4.5-4.7 ms against 10.1 ms without)")
    ap.add_argument("--budget-gb", type=float, default=8.0, help="serving: HBM budget for scenes")
    ap.add_argument("--meshes", type=int, default=4096)
    ap.add_argument("--builder", default="auto", choices=["auto", "sah", "lbvh"],
                    help="batch_build: the BLAS builder of the FAST_TRACE meshes (auto: the autotuner's "
                         "choice, or the library default with --no-autotune)")
    ap.add_argument("--instances", type=int, default=100_000)
    return ap.parse_args()


def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("LOCAL_RANK", 0)), int(os.environ.get("WORLD_SIZE", 1))


def make_workload(n_rays):
    scene = S.terrain_scene()
    rays = S.terrain_rays(scene, n_rays, seed=4)
    return scene, rays


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms while running."""
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.thread.join(timeout=2)

    def summary(self):
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            p = [x.strip() for x in line.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                mx = max(mx, float(p[2]))
            except ValueError:
                continue
            for k, name in enumerate(names):
                if p[5 + k].lower().startswith("active"):
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx or None,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peak():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured (MEASURED_PEAKS.json hbm_gbs, STREAM-style copy)"
    return 6800.0, "fallback (6.8 TB/s)"


def ncu_traffic_per_ray(layout):
    """DRAM bytes per ray of the traversal kernel from the committed ncu summary, or None."""
    f = ROOT / "profiles" / ("trace_closest_quant8_terrain.md" if layout == 1 else "trace_closest_fp32_terrain.md")
    if not f.exists():
        return None
    m = re.search(r"dram_bytes_per_ray:\s*([0-9.]+)", f.read_text())
    return float(m.group(1)) if m else None


def cpu_baseline(osc, rays, build_s, budget_s=12.0, threads=0):
    """The oracle (CPU restatement, all host threads) on a bounded sample of the same rays.
    Returns the baseline record and the oracle's hits for the first ``n`` rays (the sample)."""
    cores = threads or os.cpu_count()
    pilot = rays[:65536]
    t0 = time.perf_counter()
    osc.trace_closest(pilot, threads=cores)
    dt = time.perf_counter() - t0
    n = int(min(rays.shape[0], max(65536, 65536 * budget_s / max(dt, 1e-6))))
    sample = rays[:n]
    t0 = time.perf_counter()
    hits = osc.trace_closest(sample, threads=cores)
    dt = time.perf_counter() - t0
    return {"value": n / dt / 1e9, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": f"first {n} of the {rays.shape[0]} incoherent rays, oracle BVH build excluded "
                      f"({build_s:.1f} s)"}, hits


def closest_parity(oracle_mod, osc, rays, got, want):
    """Every record of ``got`` (GPU) against ``want`` (oracle, same rays): bit-exact records, and
    the (inst, prim) disagreements classified in FP64 as near-ties or grazing hits."""
    g = got.view(np.uint32).reshape(-1, 6)[:, :5]
    w = want.view(np.uint32).reshape(-1, 6)[:, :5]
    exact = np.all(g == w, axis=1)
    rep = oracle_mod.adjudicate(osc, rays, got, want)
    same_id = (got["inst"] == want["inst"]) & (got["prim"] == want["prim"])
    other = same_id & ~exact  # same triangle, different t or barycentric bits
    t_rel = 0.0
    if other.any():
        tg, tw = got["t"][other].astype(np.float64), want["t"][other].astype(np.float64)
        t_rel = float(np.max(np.abs(tg - tw) / np.maximum(np.abs(tw), 1e-30)))
    return {"rays": int(rays.shape[0]), "bit_exact": float(exact.mean()), "bit_exact_rays": int(exact.sum()),
            "id_agreement": float(same_id.mean()), "disagree": rep["disagree"], "near_tie": rep["near_tie"],
            "grazing": rep["grazing"], "unexplained": len(rep["unexplained"]),
            "same_id_other_bits": int(other.sum()), "same_id_t_rel_max": t_rel}


def headline_parity(osc, rays, dev_hits, host_hits, baseline_hits, shadow=None, occ=None, fp32_equal=None):
    """Parity of the bench's own outputs at the full headline size, against the oracle: the
    device-resident run (`value`), the host-buffer run (`e2e`) and, when given, the any-hit run on
    the shadow rays.  The oracle's hits of the timed cpu_baseline sample are reused; the rest of
    the rays are traced here, untimed."""
    import oracle as oracle_mod
    t0 = time.perf_counter()
    n0 = baseline_hits.shape[0]
    want = baseline_hits
    if n0 < rays.shape[0]:
        want = np.concatenate([baseline_hits, osc.trace_closest(rays[n0:])])
    out = {"oracle": "oracle/lcx_oracle.cpp (FP32 restatement of accel.rs:449-535, binned-SAH BVH); "
                     "mismatches classified by its FP64 evaluator",
           "closest": closest_parity(oracle_mod, osc, rays, dev_hits, want),
           "closest_e2e": closest_parity(oracle_mod, osc, rays, host_hits, want)}
    if shadow is not None and occ is not None:
        want_occ = osc.trace_any(shadow)
        agree = occ.astype(bool) == want_occ.astype(bool)
        out["any"] = {"rays": int(shadow.shape[0]), "bit_exact": float(agree.mean()),
                      "disagree": int((~agree).sum()), "occluded_frac": float(want_occ.mean())}
    if fp32_equal is not None:
        out["fp32_nodes_records_equal_quant8"] = bool(fp32_equal)
    out["check_s"] = time.perf_counter() - t0
    return out


def _event_ms(fn, reps, stream):
    """Mean ms per call of fn() by CUDA events on `stream` (synchronised on both sides)."""
    import torch
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(reps):
        fn()
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / reps


def leg_per_thread(acc, d_rays, d_hits, n, stream, reps=5):
    """Loop mode 3 on the headline rays: one ray per thread through lcx::trace_closest, the
    per-ray device call a user megakernel makes (include/lcx/trace.cuh)."""
    import ctypes
    from luisacompute_gb300 import _capi
    lib = _capi.load()
    k = [ctypes.c_uint32(0) for _ in range(3)]
    _capi.check(lib.lcx_get_trace_tuning(*[ctypes.byref(x) for x in k]), "lcx_get_trace_tuning")
    _capi.check(lib.lcx_set_trace_tuning(k[0].value, k[1].value, 3), "lcx_set_trace_tuning")
    try:
        for _ in range(3):
            acc.trace_closest(d_rays, out=d_hits)
        ms = _event_ms(lambda: acc.trace_closest(d_rays, out=d_hits), reps, stream)
    finally:
        _capi.check(lib.lcx_set_trace_tuning(k[0].value, k[1].value, k[2].value), "lcx_set_trace_tuning")
    return {"grays_per_s": n / (ms * 1e-3) / 1e9, "ms": ms,
            "what": "loop mode 3: one ray per thread, each calling lcx::trace_closest (include/lcx/trace.cuh) with "
                    "a 16-entry shared short stack, as a user megakernel does; same rays and records as `value`"}


def leg_multi_job(scene_acc, stream, jobs=2048, lo=256, hi=8192, seed=23):
    """Many small closest-hit jobs against several resident scenes: one lcx_trace_jobs launch
    (the batched form) against one lcx_trace_closest per job in sequence (the plain
    one-job-at-a-time path, each job on the best single kernel, loop mode 2), the latter captured
    in a CUDA graph and replayed so that host overhead is not counted against it."""
    import torch
    from luisacompute_gb300 import _capi
    from luisacompute_gb300.accel import accel_from_scene, rays_to_device, stream_handle
    lib = _capi.load()
    rng = np.random.default_rng(seed)
    scenes = [S.icosphere_scene(k) for k in (3, 4, 5)] + [S.terrain_scene(n=256, sphere_count=16, sphere_subdiv=3)]
    built = [accel_from_scene(s) for s in scenes]
    accs = [scene_acc] + [a for a, _ in built]
    counts = np.exp(rng.uniform(np.log(lo), np.log(hi), jobs)).astype(np.int64)
    first = np.concatenate([[0], np.cumsum(counts)[:-1]])
    total = int(counts.sum())
    d_rays = rays_to_device(S.sphere_rays(total, [-1.5] * 3, [1.5] * 3, seed=seed + 1))
    hits_a = torch.empty((total, 6), dtype=torch.int32, device="cuda")
    hits_b = torch.empty_like(hits_a)
    pick = rng.integers(0, len(accs), jobs)
    table = (_capi.LcxTraceJob * jobs)()
    for j in range(jobs):
        table[j] = _capi.LcxTraceJob(accs[pick[j]].handle, d_rays.data_ptr() + int(first[j]) * 32,
                                     hits_a.data_ptr() + int(first[j]) * 24, int(counts[j]), 0xFF, 0, 0)
    sh = stream_handle(stream)

    def batched():
        _capi.check(lib.lcx_trace_jobs(table, jobs, 1, sh), "lcx_trace_jobs")

    def one_at_a_time(h):
        for j in range(jobs):
            _capi.check(lib.lcx_trace_closest(accs[pick[j]].handle, d_rays.data_ptr() + int(first[j]) * 32,
                                              int(counts[j]), 0xFF, hits_b.data_ptr() + int(first[j]) * 24, h),
                        "lcx_trace_closest")

    for _ in range(3):
        batched()
    batched_ms = _event_ms(batched, 5, stream)
    one_at_a_time(sh)
    torch.cuda.synchronize()
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph):  # captured on torch's capture stream
        one_at_a_time(stream_handle(torch.cuda.current_stream()))
    for _ in range(2):
        graph.replay()
    plain_ms = _event_ms(graph.replay, 5, stream)
    equal = bool(torch.equal(hits_a, hits_b))
    del graph
    return {"jobs": jobs, "rays": total, "scenes": len(accs), "batched_ms": batched_ms, "one_at_a_time_ms": plain_ms,
            "batched_grays_per_s": total / (batched_ms * 1e-3) / 1e9,
            "one_at_a_time_grays_per_s": total / (plain_ms * 1e-3) / 1e9,
            "ratio": plain_ms / batched_ms, "records_equal": equal,
            "what": f"{jobs} closest-hit jobs of {lo}..{hi} rays (log-uniform) against {len(accs)} resident scenes "
                    "(the headline scene, icospheres of 1,280 / 5,120 / 20,480 triangles, a small terrain): one "
                    "lcx_trace_jobs launch (host preparation included) vs one lcx_trace_closest per job in "
                    "sequence, replayed from a CUDA graph (no host overhead counted against it)"}


def leg_batch_build(stream, count=512):
    """Batched BLAS build of a 512-mesh sample of the batched-build workload (log-uniform
    64..262,144 triangles, 1 % Gaussian displacement): Mtris/s of one lcx_mesh_build_batch."""
    from luisacompute_gb300.accel import build_meshes, mesh_from_data
    datas = S.batch_meshes(count, seed=6)
    meshes = [mesh_from_data(m) for m in datas]
    total = sum(m.tri_count for m in datas)
    for _ in range(3):
        build_meshes(meshes)
    ms = _event_ms(lambda: build_meshes(meshes), 5, stream)
    sah = float(np.mean([m.stats().wide_sah_cost for m in meshes]))
    # the same build with the Morton LBVH in place of the binned-SAH builder
    from luisacompute_gb300 import _capi
    lib = _capi.load()
    old = ctypes.c_uint32(0)
    _capi.check(lib.lcx_get_build_blas_sah(ctypes.byref(old)), "blas_sah")
    _capi.check(lib.lcx_set_build_blas_sah(1 - old.value), "blas_sah")
    try:
        build_meshes(meshes)
        ms_other = _event_ms(lambda: build_meshes(meshes), 5, stream)
        sah_other = float(np.mean([m.stats().wide_sah_cost for m in meshes]))
    finally:
        _capi.check(lib.lcx_set_build_blas_sah(old.value), "blas_sah")
    # the same meshes reserved without a build (lcx_mesh_reserve_batch): their first build captured in a
    # CUDA graph, replayed
    import torch
    from luisacompute_gb300.accel import Mesh, reserve_meshes
    res = reserve_meshes([Mesh(m.vertices, m.triangles) for m in meshes], build=False)
    torch.cuda.synchronize()
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph):
        build_meshes(res)
    for _ in range(2):
        graph.replay()
    gms = _event_ms(graph.replay, 5, stream)
    del graph, res
    names = ("sah", "lbvh") if old.value else ("lbvh", "sah")
    return {"meshes": count, "triangles": int(total), "ms": ms, "mtris_per_s": total / (ms * 1e-3) / 1e6,
            "builder": names[0], "mean_wide_sah": sah,
            f"{names[1]}_ms": ms_other, f"{names[1]}_mean_wide_sah": sah_other,
            "graph_first_build_ms": gms, "graph_first_build_mtris_per_s": total / (gms * 1e-3) / 1e6,
            "what": "one lcx_mesh_build_batch over the sample per step (its host sync for the node count included), "
                    "default build knobs; graph_first_build: the sample reserved without a build and its first "
                    "build captured in a CUDA graph (no host sync, Morton LBVH), per replay"}


def leg_pathtrace(scene, acc, meshes, stream, steps=5):
    """Wavefront path tracing of the headline scene, 1920x1080, 4 spp, <= 8 bounces."""
    import torch
    from luisacompute_gb300 import pathtrace as PT
    alb = PT.albedos_to_device(PT.albedos(scene))
    prm = PT.params(width=1920, height=1080, spp=4, max_bounces=8, rr_start=3, eye=(0.0, 0.8, 2.4))
    for _ in range(3):
        PT.render(scene, acc, meshes, alb, prm)
    times, st = [], None
    for _ in range(steps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        _, _, st = PT.render(scene, acc, meshes, alb, prm, stream=stream)
        e1.record(stream)
        torch.cuda.synchronize()
        times.append(e0.elapsed_time(e1))
    ms = float(np.median(times))
    return {"ms_per_frame": ms, "rays_closest": int(st.closest_rays), "rays_any": int(st.any_rays),
            "grays_per_s": (st.closest_rays + st.any_rays) / (ms * 1e-3) / 1e9,
            "what": "lcx_pt_render, 1920x1080x4 spp, <= 8 bounces, RR from 3, per-bounce host syncs included"}


def leg_serving(requests=300, rate=800.0, n_scenes=16):
    """A short serving mix: continuous batching against one request at a time on the same trace."""
    import torch
    from luisacompute_gb300 import serving as V
    scenes, reqs = V.make_workload(n_scenes=n_scenes, n_requests=requests, rate_hz=rate, tri_hi=1_000_000,
                                   ray_pool=12)
    budget = 8 << 30

    def clone():
        return [V.Request(r.rid, r.arrival, r.scene, r.rays, r.any_hit, r.new_scene) for r in reqs]

    V.ContinuousServer(V.SceneStore(scenes, budget), slots=4).run(clone()[:8])  # warm pools and modules
    torch.cuda.synchronize()
    store = V.SceneStore(scenes, budget)
    store.warm(sorted(scenes), split=3.0)
    cont = V.ContinuousServer(store, slots=4)
    rc = cont.run(clone())
    torch.cuda.synchronize()
    store_p = V.SceneStore(scenes, budget)
    store_p.warm(sorted(scenes), split=3.0)
    rp = V.PlainServer(store_p).run(clone())
    c, p = V.latency_stats(rc), V.latency_stats(rp)
    slow = sorted(rc, key=lambda r: r.arrival - r.done)[:3]  # the slowest requests, for the tail
    worst = [{"rid": r.rid, "rays": int(r.rays.shape[0]), "any": bool(r.any_hit), "upload": r.new_scene is not None,
              "arrival_ms": r.arrival * 1e3, "wait_ms": (r.dispatched - r.arrival) * 1e3,
              "run_ms": (r.done - r.dispatched) * 1e3} for r in slow]
    return {"continuous": {"p50_ms": c["p50_ms"], "p99_ms": c["p99_ms"], "grays_per_s": c["grays_per_s"],
                           "queries_0.5M_to_2M_rays": c["queries_0.5M_to_2M_rays"], "slowest": worst,
                           "batches": cont.batches, "builds": store.builds, "evictions": store.evictions},
            "one_at_a_time": {"p50_ms": p["p50_ms"], "p99_ms": p["p99_ms"], "grays_per_s": p["grays_per_s"],
                              "queries_0.5M_to_2M_rays": p["queries_0.5M_to_2M_rays"]},
            "what": f"{requests} Poisson requests at {rate:g}/s, {n_scenes} resident scenes of 10k..1M triangles "
                    "(split-built), 1k..4M rays, half camera half incoherent, half closest half any, 8% uploads"}


def run_batch_build(args):
    """4096 meshes, triangle counts log-uniform in [64, 262144] (icospheres or grids with 1 % Gaussian
    vertex displacement), built with one lcx_mesh_build_batch call per step; then a TLAS over
    100,000 random affine instances.  Metric: Mtris/s of the batched BLAS build.  The build knobs
    (leaf size, node width, Morton normalisation) are autotuned on the first 512 meshes first."""
    import torch
    from luisacompute_gb300 import build as B
    B.build()
    from luisacompute_gb300.accel import Accel, build_meshes, mesh_from_data
    t0 = time.perf_counter()
    datas = S.batch_meshes(args.meshes, seed=6)
    gen_s = time.perf_counter() - t0
    total = sum(m.tri_count for m in datas)
    tuned = None
    from luisacompute_gb300 import _capi
    if args.builder != "auto":  # a fixed builder, and the autotuner's other knobs
        _capi.check(_capi.load().lcx_set_build_blas_sah(1 if args.builder == "sah" else 0), "builder")
    if not args.no_autotune:
        from luisacompute_gb300 import autotune
        space = None
        if args.builder != "auto":
            space = {k: v for k, v in autotune.BUILD_SPACE.items() if k not in ("split", "blas_sah")}
        tuned = autotune.tune_batch_build(datas, sample=512, space=space).to_json()
    meshes = [mesh_from_data(m) for m in datas]
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream()

    def timed(fn, reps):
        """Mean seconds per call: CUDA events on the current stream (each batched build also
        synchronises once on the host for its node count, inside the timed span)."""
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / 1e3 / reps

    for _ in range(max(3, args.warmup)):
        build_meshes(meshes)
    lib = _capi.load()
    sah_on = ctypes.c_uint32(0)
    _capi.check(lib.lcx_get_build_blas_sah(ctypes.byref(sah_on)), "builder")
    builder_name = "binned SAH" if sah_on.value else "Morton LBVH"
    launches0 = ctypes.c_uint64(0)
    _capi.check(lib.lcx_get_build_kernel_launches(ctypes.byref(launches0)), "launch count")
    with ClockSampler(0) as clocks:
        batch_s = timed(lambda: build_meshes(meshes), args.steps)
    launches1 = ctypes.c_uint64(0)
    _capi.check(lib.lcx_get_build_kernel_launches(ctypes.byref(launches1)), "launch count")
    launches = int(launches1.value - launches0.value)
    # one-by-one on the first 256 meshes (each lcx_mesh_build synchronises once)
    sub = meshes[:256]
    sub_tris = sum(m.triangles.shape[0] for m in sub)
    single_s = timed(lambda: [m.build() for m in sub], 1)
    batch_sub_s = timed(lambda: build_meshes(sub), 3)
    # TLAS over random affine instances of the meshes
    rng = np.random.default_rng(7)
    pick = rng.integers(0, len(meshes), args.instances)
    aff = S.affine_rows(S.random_rotations(args.instances, rng), np.exp(rng.uniform(np.log(0.5), np.log(2.0),
                                                                                    args.instances)),
                        rng.uniform(-50, 50, (args.instances, 3)))
    acc = Accel()
    acc.emplace_back_many([meshes[i] for i in pick], aff)
    tlas_first_s = timed(lambda: acc.build(), 1)
    tlas_s = timed(lambda: acc.build(), 3)
    st = acc.stats()
    wide = [m.stats().wide_sah_cost for m in meshes]
    # refit (PREFER_UPDATE on meshes created with allow_update) of the whole batch, same buffers
    from luisacompute_gb300.accel import REQUEST_PREFER_UPDATE, AccelOption, Mesh
    upd = [Mesh(m.vertices, m.triangles, AccelOption(allow_update=True)) for m in meshes]
    build_meshes(upd)
    upd_build_s = timed(lambda: build_meshes(upd), 3)
    build_meshes(upd, request=REQUEST_PREFER_UPDATE)
    refit_s = timed(lambda: build_meshes(upd, request=REQUEST_PREFER_UPDATE), 5)
    refits = int(upd[0].stats().refits)
    # the same refit without host synchronisation, a TLAS refit over the 100,000 instances, and
    # both captured once as a CUDA graph and replayed (a rigid or skinned animation frame)
    from luisacompute_gb300.accel import set_refit_sync
    set_refit_sync(False)
    try:
        refit_async_s = timed(lambda: build_meshes(upd, request=REQUEST_PREFER_UPDATE), 5)
        uacc = Accel(AccelOption(allow_update=True))
        uacc.emplace_back_many([upd[i] for i in pick], aff)
        uacc.build()
        tlas_rebuild_s = timed(lambda: uacc.build(), 3)
        uacc.build(request=REQUEST_PREFER_UPDATE)
        tlas_refit_s = timed(lambda: uacc.build(request=REQUEST_PREFER_UPDATE), 5)
        tlas_refits = int(uacc.stats().refits)
        torch.cuda.synchronize()
        graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(graph):
            build_meshes(upd, request=REQUEST_PREFER_UPDATE)
            uacc.build(request=REQUEST_PREFER_UPDATE)
        graph.replay()
        graph_s = timed(graph.replay, 5)
        from luisacompute_gb300 import _capi
        _capi.check(_capi.load().lcx_check_trace_errors(), "refit errors")
    finally:
        set_refit_sync(True)
    del graph, uacc, upd
    # a reserved batch: full rebuilds in place with no host synchronisation, also as a CUDA graph
    from luisacompute_gb300.accel import reserve_meshes
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    res = reserve_meshes([Mesh(m.vertices, m.triangles) for m in meshes])
    torch.cuda.synchronize()
    res_bytes = max(0, free0 - torch.cuda.mem_get_info()[0])  # the reserved block, about
    reserved_s = timed(lambda: build_meshes(res), 5)
    graph_b = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph_b):
        build_meshes(res)
    graph_b.replay()
    graph_rebuild_s = timed(graph_b.replay, 5)
    _capi.check(_capi.load().lcx_check_trace_errors(), "rebuild errors")
    del graph_b, res
    # gpu_launches: our kernels in the timed loop, from the library's build-launch counter (the
    # LBVH: tri_prep, morton, lbvh, binary_sah, collapse_init, collapse, emit; the SAH builder: its
    # seed and mark, four kernels per level of ranges above 1,024 items, the per-range blocks and
    # the segment keys in place of morton and lbvh; CUB's sort and scan are library kernels)
    line = {"metric": "Mtris/s batched BLAS build (4096 meshes)", "value": total / batch_s / 1e6, "unit": "Mtris/s",
            "n_gpus": 1, "steps": args.steps, "warmup": max(3, args.warmup), "ms_per_step": batch_s * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded)",
            "config": {"workload": f"{len(meshes)} meshes, {total} triangles, counts log-uniform [64, 262144], "
                                   "icosphere or grid with 1% Gaussian displacement; one lcx_mesh_build_batch per step",
                       "generation_s": gen_s, "blas_builder": builder_name,
                       "l2": "inputs (vertices + indices, ~2.6 GB) and outputs exceed the 129 MB L2"},
            "clocks": clocks.summary(), "gpu_launches": launches,
            "extra": {"one_by_one_mtris_s_first_256": sub_tris / single_s / 1e6,
                      "batched_mtris_s_first_256": sub_tris / batch_sub_s / 1e6,
                      "mean_wide_sah": float(np.mean(wide)),
                      "refit": {"build_ms": upd_build_s * 1e3, "refit_ms": refit_s * 1e3,
                                "refit_mtris_s": total / refit_s / 1e6, "refits_counted": refits,
                                "refit_async_ms": refit_async_s * 1e3,
                                "tlas_rebuild_ms": tlas_rebuild_s * 1e3, "tlas_refit_ms": tlas_refit_s * 1e3,
                                "tlas_refits_counted": tlas_refits,
                                "graph_frame_ms": graph_s * 1e3,
                                "reserved_rebuild_ms": reserved_s * 1e3,
                                "reserved_graph_rebuild_ms": graph_rebuild_s * 1e3,
                                "reserved_graph_rebuild_mtris_s": total / graph_rebuild_s / 1e6,
                                "reserved_block_gib": res_bytes / 2**30,
                                "what": "the same 4096 meshes created with allow_update: one batched build vs "
                                        "one batched PREFER_UPDATE (refit in place, topology kept; refit_ms "
                                        "synchronises once for errors, refit_async_ms does not); a TLAS over "
                                        "the 100,000 instances rebuilt vs refit; graph_frame_ms = BLAS refit of "
                                        "all 4096 meshes + TLAS refit captured as one CUDA graph, per replay; "
                                        "reserved_*: the 4096 meshes reserved (lcx_mesh_build_batch_reserve) and "
                                        "fully rebuilt in place with no host sync, plain and as a CUDA graph"},
                      "tlas_instances": args.instances, "tlas_build_ms": tlas_s * 1e3,
                      "tlas_first_build_ms": tlas_first_s * 1e3,
                      "tlas": {"nodes": int(st.node_count), "depth": int(st.depth), "sah": st.sah_cost,
                               "wide_sah": st.wide_sah_cost}}}
    if tuned is not None:
        line["config"]["autotune"] = tuned
    if not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline_build(datas, meshes, rng)
    print(json.dumps(line), flush=True)
    return 0


def cpu_baseline_build(datas, meshes, rng, count=16):
    """The oracle's binned-SAH build (32 bins, leaf size 4, one thread) timed on a sample of the
    batch, with its SAH beside the SAH of our build of the same meshes."""
    import oracle
    oracle.build()
    lib = oracle.load()
    sample = rng.choice(len(meshes), count, replace=False)
    sah, tris, secs = [], 0, 0.0
    for i in sample:
        md = datas[i]
        v = np.ascontiguousarray(md.vertices)
        tt = np.ascontiguousarray(md.triangles)
        t = time.perf_counter()
        om = lib.lcxo_mesh_create(v.ctypes.data, 4, v.shape[0], tt.ctypes.data, tt.shape[0], 4, 32)
        secs += time.perf_counter() - t
        tris += md.tri_count
        ms = meshes[i].stats()
        sah.append({"tris": int(md.tri_count), "oracle_binned_sah": float(lib.lcxo_mesh_sah(om)),
                    "ours_binary": ms.sah_cost, "ours_wide": ms.wide_sah_cost, "ours_depth": int(ms.depth)})
        lib.lcxo_mesh_destroy(om)
    ratio = float(np.median([x["ours_binary"] / x["oracle_binned_sah"] for x in sah]))
    return {"value": tris / secs / 1e6, "unit": "Mtris/s", "cores": 1, "kind": "port",
            "sample": f"{count} meshes of the batch ({tris} triangles), oracle binned-SAH build",
            "sah_sample": sah, "median_sah_ratio_ours_to_oracle_binned": ratio,
            "ours_builder": "the timed build's (autotuned: binned SAH or Morton LBVH)"}


def run_serving(args):
    """64 resident scenes (log-uniform 10k..4M triangles), Poisson-arriving requests (log-uniform
    1k..4M rays, half coherent camera rays, half incoherent; half closest, half any), 8 % upload a
    new scene; HBM budget with LRU eviction.  Continuous batching vs one request at a time on the
    same arrival trace."""
    import torch
    from luisacompute_gb300 import build as B
    B.build()
    from luisacompute_gb300 import serving as V
    budget = int(args.budget_gb * (1 << 30))
    runs = {}
    for rate in (args.rate, 4 * args.rate):
        t0 = time.perf_counter()
        scenes, reqs = V.make_workload(n_scenes=64, n_requests=args.requests, rate_hz=rate, ray_pool=24)
        gen_s = time.perf_counter() - t0

        def clone():
            return [V.Request(r.rid, r.arrival, r.scene, r.rays, r.any_hit, r.new_scene) for r in reqs]

        # warm both paths (module load, pinned pools, allocator) on a short prefix
        V.ContinuousServer(V.SceneStore(scenes, budget), slots=4).run(clone()[:8])
        V.PlainServer(V.SceneStore(scenes, budget)).run(clone()[:8])
        torch.cuda.synchronize()
        store_c = V.SceneStore(scenes, budget)
        store_c.warm(sorted(scenes), split=args.warm_split)  # the 64 scenes are resident before requests arrive
        cont = V.ContinuousServer(store_c, slots=4)
        with ClockSampler(0) as clocks:
            rc = cont.run(clone())
        torch.cuda.synchronize()
        store_p = V.SceneStore(scenes, budget)
        store_p.warm(sorted(scenes), split=args.warm_split)
        rp = V.PlainServer(store_p).run(clone())
        runs[rate] = {"rate_hz": rate, "generation_s": gen_s,
                      "continuous": {**V.latency_stats(rc), "batches": cont.batches, "chunks": cont.chunks,
                                     "trace_launches": cont.trace_launches,
                                     "builds": store_c.builds, "evictions": store_c.evictions},
                      "plain_one_at_a_time": {**V.latency_stats(rp), "builds": store_p.builds,
                                              "evictions": store_p.evictions},
                      "clocks": clocks.summary()}
    base = runs[args.rate]
    line = {"metric": "serving p99 latency (ms) of 0.5M-2M-ray queries, continuous batching",
            "value": base["continuous"]["queries_0.5M_to_2M_rays"]["p99_ms"], "unit": "ms",
            "n_gpus": 1, "steps": 1, "warmup": 1, "ms_per_step": base["continuous"]["span_s"] * 1e3,
            "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded)",
            "config": {"workload": f"64 resident scenes log-uniform 10k..4M tris, {args.requests} Poisson requests, "
                                   "1k..4M rays (half camera, half incoherent; half closest, half any), "
                                   f"8% upload a new scene, HBM budget {args.budget_gb:g} GiB, 4 stream slots, "
                                   "<= 1M rays per launch, <= 2M rays in flight, fewest-remaining-rays first",
                       "resident_scene_split": args.warm_split,
                       "host_buffers": "pinned; read and written by the kernels directly on a coherent host link"},
            "runs": list(runs.values()), "clocks": base["clocks"],
            "gpu_launches": base["continuous"]["trace_launches"]}
    print(json.dumps(line), flush=True)
    return 0


def run_pathtrace(args):
    """Wavefront diffuse path tracing, 1920x1080, 4 spp, up to 8 bounces, Russian roulette from bounce
    3, point light + constant environment, grey albedo U[0.2, 0.8] per triangle (seed 7), on the
    terrain scene (heightfield + 256 instanced spheres) and on the icosphere scene.  A frame is timed
    with CUDA events around lcx_pt_render (its per-bounce host synchronisations included).  The
    cpu_baseline leg renders the same frame with the CPU restatement and compares first-bounce hits
    per path and the image (RMSE)."""
    import torch
    from luisacompute_gb300 import build as B
    B.build()
    from luisacompute_gb300 import pathtrace as PT
    from luisacompute_gb300.accel import accel_from_scene
    stream = torch.cuda.current_stream()
    out, launches = [], 0
    steps = max(1, args.steps)
    for name, scene, eye in (("terrain + 256 instanced spheres", S.terrain_scene(), (0.0, 0.8, 2.4)),
                             ("icosphere subdiv 6", S.icosphere_scene(6), (0.0, 0.0, 3.0))):
        acc, meshes = accel_from_scene(scene)
        alb = PT.albedos(scene)
        d_alb = PT.albedos_to_device(alb)
        prm = PT.params(width=1920, height=1080, spp=4, max_bounces=8, rr_start=3, eye=eye)
        for _ in range(max(3, args.warmup)):
            PT.render(scene, acc, meshes, d_alb, prm)
        times, stats = [], None
        with ClockSampler(0) as clocks:
            for _ in range(steps):
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                img, _, stats = PT.render(scene, acc, meshes, d_alb, prm, stream=stream)
                e1.record(stream)
                torch.cuda.synchronize()
                times.append(e0.elapsed_time(e1) / 1e3)
                launches += int(stats.launches) if not out else 0
        frame = float(np.median(times))
        row = {"scene": name, "s_per_frame": frame, "ms_per_frame_render_kernels": stats.ms,
               "rays_closest": int(stats.closest_rays), "rays_any": int(stats.any_rays),
               "bounces": int(stats.bounces), "launches_per_frame": int(stats.launches),
               "grays_per_s": (stats.closest_rays + stats.any_rays) / frame / 1e9,
               "image_mean": float(img.mean()), "clocks": clocks.summary()}
        if not args.no_cpu_baseline:
            row["cpu_baseline"] = cpu_baseline_pathtrace(scene, acc, meshes, alb, prm)
        out.append(row)
    line = {"metric": "s/frame wavefront path tracing 1920x1080x4spp (terrain scene)",
            "value": out[0]["s_per_frame"], "unit": "s", "n_gpus": 1, "steps": steps,
            "warmup": max(3, args.warmup), "ms_per_step": out[0]["s_per_frame"] * 1e3,
            "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded)",
            "config": {"workload": "wavefront diffuse path tracing, 1920x1080, 4 spp, <= 8 bounces, RR from 3, "
                                   "shadow rays via trace_any, compaction between bounces",
                       "l2": "8.3M paths: rays (265 MB), hits and path state exceed the 129 MB L2"},
            "gpu_launches": launches, "scenes": out}
    if "cpu_baseline" in out[0]:
        line["cpu_baseline"] = out[0]["cpu_baseline"]
    print(json.dumps(line), flush=True)
    return 0


def run_curves(args):
    """Round curves: 20,000 hair strands of 16 control points each (random smooth walks in [-1, 1]^3,
    step 0.05, radius tapering 0.004 -> 0.001), as Catmull-Rom (260,000 segments) and piecewise
    linear (300,000 segments) curves; 1024x1024 camera rays and 2^20 incoherent rays, closest hit,
    timed with CUDA events per trace call.  The cpu_baseline leg runs the curve oracle (brute force
    over the segments with box culling, FP64 intersection) on a sample of the camera rays and
    reports the hit agreement with the GPU records."""
    import torch
    from luisacompute_gb300 import build as B
    B.build()
    from luisacompute_gb300.accel import Accel, Curve, hits_to_numpy, rays_to_device
    stream = torch.cuda.current_stream()
    rng = np.random.default_rng(17)
    cps = S.hair_curves(20_000, 16, rng, step=0.05, radius=(0.004, 0.001))
    d_cps = torch.from_numpy(cps).cuda()
    cam = S.camera_rays(1024, 1024, eye=(0.0, 0.0, 4.0), target=(0.0, 0.0, 0.0))
    inc = S.sphere_rays(1 << 20, [-1.5] * 3, [1.5] * 3, seed=18)
    steps, warm = max(1, args.steps), max(3, args.warmup)
    rows, launches = [], 0
    with ClockSampler(0) as clocks:
        for basis, name in ((2, "catmull-rom"), (0, "piecewise linear")):
            segs = S.curve_segments(20_000, 16, basis)
            cv = Curve(basis, d_cps, torch.from_numpy(segs.astype(np.int32)).cuda())
            cv.build()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            cv.build()
            torch.cuda.synchronize()
            build_s = time.perf_counter() - t0
            acc = Accel()
            acc.emplace_back(cv)
            acc.build()
            row = {"basis": name, "segments": int(segs.size), "build_s": build_s}
            for kind, rays in (("camera", cam), ("incoherent", inc)):
                d = rays_to_device(rays)
                out = acc.trace_closest(d)
                for _ in range(warm):
                    acc.trace_closest(d, out=out)
                ms = []
                for _ in range(steps):
                    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                    e0.record(stream)
                    acc.trace_closest(d, out=out)
                    e1.record(stream)
                    torch.cuda.synchronize()
                    ms.append(e0.elapsed_time(e1))
                    launches += 1
                h = hits_to_numpy(out)
                row[kind] = {"grays_per_s": rays.shape[0] / (float(np.median(ms)) * 1e-3) / 1e9,
                             "ms": float(np.median(ms)), "hit_frac": float((h["inst"] != 0xFFFFFFFF).mean())}
                if kind == "camera" and basis == 2 and not args.no_cpu_baseline:
                    row["cpu_baseline"] = cpu_baseline_curves(cps, segs, basis, cam, h)
            rows.append(row)
    first = rows[0]
    line = {"metric": "Grays/s closest-hit on round curves (hair, Catmull-Rom, camera rays)",
            "value": first["camera"]["grays_per_s"], "unit": "Grays/s", "n_gpus": 1, "steps": steps, "warmup": warm,
            "ms_per_step": first["camera"]["ms"], "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic (seeded)",
            "config": {"workload": "20,000 strands x 16 control points, Catmull-Rom (260,000 segments) and linear; "
                                   "1024x1024 camera rays and 2^20 incoherent rays; trace_closest",
                       "l2": "curve BLAS and control points stay resident; rays 32 MiB, hits 24 MiB per call"},
            "gpu_launches": launches, "clocks": clocks.summary(), "bases": rows}
    if "cpu_baseline" in first:
        line["cpu_baseline"] = first["cpu_baseline"]
    print(json.dumps(line), flush=True)
    return 0


def cpu_baseline_curves(cps, segs, basis, rays, gpu_hits, sample=4096):
    """The curve oracle on the first ``sample`` rays, all host cores; hit agreement with the GPU."""
    import oracle
    oracle.build()
    oc = oracle.OracleCurve(cps, segs, basis)
    t0 = time.perf_counter()
    want = oracle.trace_curves([oc], np.eye(3, 4, dtype=np.float32).reshape(1, 12), 0xFF, rays[:sample])
    cpu_s = time.perf_counter() - t0
    got = gpu_hits[:sample]
    agree = float(((got["inst"] == 0xFFFFFFFF) == (want["inst"] == 0xFFFFFFFF)).mean())
    return {"value": sample / cpu_s / 1e9, "unit": "Grays/s", "cores": os.cpu_count(), "kind": "port",
            "sample": f"first {sample} camera rays; brute force over all segments with box culling (no BVH), "
                      "FP64 intersection", "hit_agreement": agree}


def cpu_baseline_pathtrace(scene, acc, meshes, alb, prm):
    """The CPU restatement of the wavefront tracer on all host cores, one frame, with the GPU
    frame's first-bounce hits and image compared against it."""
    from luisacompute_gb300 import pathtrace as PT
    import oracle
    oracle.build()
    img, hits, _ = PT.render(scene, acc, meshes, alb, prm, first_hits=True)
    t0 = time.perf_counter()
    osc = oracle.OracleScene(scene)
    cimg, chits = osc.pathtrace(scene, alb, prm)
    cpu_s = time.perf_counter() - t0
    agree = float((hits.view(np.uint32).reshape(-1, 6)[:, :2] == chits.view(np.uint32).reshape(-1, 6)[:, :2]).all(1).mean())
    return {"value": cpu_s, "unit": "s", "cores": os.cpu_count(), "kind": "port",
            "sample": "one full frame (BVH build included)", "first_hit_agreement": agree,
            "image_rmse_vs_gpu": float(np.sqrt(np.mean((img - cimg) ** 2)))}


def run_reference(args):
    rank, _, world = dist_env()
    if rank != 0:
        return 0
    scene, rays = make_workload(args.rays)
    import oracle
    oracle.build()
    osc = oracle.OracleScene(scene)
    cores = os.cpu_count()
    pilot = rays[:32768]
    t0 = time.perf_counter()
    osc.trace_closest(pilot, threads=cores)
    per_ray = (time.perf_counter() - t0) / pilot.shape[0]
    # each step is a bounded sample so that warmup + steps take about 90 s in total
    n = int(min(rays.shape[0], max(32768, 90.0 / max(per_ray, 1e-12) / max(1, args.steps + args.warmup))))
    sample = rays[:n]
    for _ in range(args.warmup):
        osc.trace_closest(sample, threads=cores)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        osc.trace_closest(sample, threads=cores)
    dt = time.perf_counter() - t0
    value = n * args.steps / dt / 1e9
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": dt / args.steps * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
            "impl": "reference",
            "config": {"workload": WORKLOAD, "rays_per_step": n},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": f"first {n} of {rays.shape[0]} rays per step; the reference CPU backend "
                                       "(Rust + Embree) is not buildable here, so its restatement is timed"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "batch_build":
        return run_batch_build(args)
    if args.workload == "serving":
        return run_serving(args)
    if args.workload == "pathtrace":
        return run_pathtrace(args)
    if args.workload == "curves":
        return run_curves(args)
    import torch
    rank, local_rank, world = dist_env()
    if world > 1:
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local_rank)
    from luisacompute_gb300 import build as B
    B.build()
    from luisacompute_gb300.accel import accel_from_scene, rays_to_device

    scene, rays = make_workload(args.rays)
    n = rays.shape[0]
    stream = torch.cuda.current_stream()
    tuned = None
    if not args.no_autotune:
        # knobs picked on a separate sample of the same distribution (1M rays, other seed)
        from luisacompute_gb300 import autotune
        sample = rays_to_device(S.terrain_rays(scene, min(n, 1 << 20), seed=40))
        tuned = autotune.tune(scene, sample, layout=args.layout).to_json()
        del sample
    t0 = time.perf_counter()
    acc, meshes = accel_from_scene(scene)
    torch.cuda.synchronize()
    build_wall_s = time.perf_counter() - t0
    d_rays = rays_to_device(rays)
    d_hits = torch.empty((n, 6), dtype=torch.int32, device="cuda")

    def barrier():
        if world > 1:
            import torch.distributed as dist
            dist.barrier()

    # counting pass (not timed): algorithmic bytes per ray
    counts = torch.zeros((n, 3), dtype=torch.int32, device="cuda")
    acc.trace_closest(d_rays, out=d_hits, layout=args.layout, counts=counts)
    torch.cuda.synchronize()
    c = counts.double().mean(0).cpu().numpy()
    del counts
    node_bytes = 80 if args.layout == 1 else 208
    bytes_per_ray = 32 + 24 + c[0] * node_bytes + c[1] * 48 + c[2] * 80
    import ctypes
    from luisacompute_gb300 import _capi
    knobs = [ctypes.c_uint32(0) for _ in range(3)]
    _capi.check(_capi.load().lcx_get_trace_tuning(*knobs), "lcx_get_trace_tuning")
    deferred = knobs[2].value == 2 and args.layout == 1  # loop mode 2 runs quantised-node calls
    kernel_name = ("k_trace_deferred<quant8, closest> (loop mode 2)" if deferred else
                   f"k_trace<{'quant8' if args.layout == 1 else 'fp32'}, closest> (loop mode {knobs[2].value})")

    for _ in range(max(3, args.warmup)):
        acc.trace_closest(d_rays, out=d_hits, layout=args.layout)
    torch.cuda.synchronize()
    barrier()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local_rank) as clocks:
        torch.cuda.synchronize()
        barrier()
        ev0.record(stream)
        for _ in range(args.steps):
            acc.trace_closest(d_rays, out=d_hits, layout=args.layout)
        ev1.record(stream)
        torch.cuda.synchronize()
        barrier()
    ms = ev0.elapsed_time(ev1)
    if world > 1:
        import torch.distributed as dist
        t = torch.tensor([ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    ms_per_step = ms / args.steps
    value = n * world * args.steps / (ms / 1e3) / 1e9
    from luisacompute_gb300.accel import hits_to_numpy
    dev_hits = hits_to_numpy(d_hits) if rank == 0 else None  # the timed run's records, for the parity check

    # end to end: pinned host rays -> device -> trace -> hits -> pinned host
    h_rays = torch.from_numpy(rays.view(np.float32).reshape(-1, 8)).pin_memory()
    h_hits = torch.empty((n, 6), dtype=torch.int32).pin_memory()
    e2e_steps = max(3, args.steps // 2)

    def serial_step():  # one copy in, one trace, one copy out, in sequence on one stream
        d_rays.copy_(h_rays, non_blocking=True)
        acc.trace_closest(d_rays, out=d_hits, layout=args.layout)
        h_hits.copy_(d_hits, non_blocking=True)

    def host_step():  # lcx_trace_closest_host: streamed, staged or direct host access (auto: streamed here)
        acc.trace_closest_host(h_rays, h_hits, layout=args.layout)

    from luisacompute_gb300 import _capi as C
    lib = C.load()
    mode, coherent = ctypes.c_uint32(0), ctypes.c_uint32(0)
    C.check(lib.lcx_get_host_access(ctypes.byref(mode), ctypes.byref(coherent)), "host access")

    def time_e2e(step):
        for _ in range(3):
            step()
        torch.cuda.synchronize()
        barrier()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(e2e_steps):
            step()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1)

    e2e_serial_ms = time_e2e(serial_step)
    direct_value = None
    if coherent.value:  # the direct path, for comparison
        C.check(lib.lcx_set_host_access(C.HOST_DIRECT), "host access")
        direct_value = n * e2e_steps / (time_e2e(host_step) / 1e3) / 1e9
        C.check(lib.lcx_set_host_access(mode.value), "host access")
    C.check(lib.lcx_set_host_access(C.HOST_STAGED), "host access")  # the staged path, for comparison
    staged_value = n * e2e_steps / (time_e2e(host_step) / 1e3) / 1e9
    C.check(lib.lcx_set_host_access(mode.value), "host access")
    e2e_ms = time_e2e(host_step)
    if world > 1:
        import torch.distributed as dist
        t = torch.tensor([e2e_ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_ms = float(t.item())
    e2e_value = n * world * e2e_steps / (e2e_ms / 1e3) / 1e9

    peak, peak_src = measured_peak()
    achieved = bytes_per_ray * n / (ms_per_step / 1e3) / 1e9
    traffic_pr = ncu_traffic_per_ray(args.layout)
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": max(3, args.warmup), "ms_per_step": ms_per_step, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
            "config": {"workload": WORKLOAD, "rays": n, "instanced_triangles": scene.instanced_triangles(),
                       "node_layout": "quant8" if args.layout == 1 else "fp32",
                       "l2": "rays (256 MiB) and hits (192 MiB) per step exceed the 129 MB L2; the BVH stays resident",
                       "parallelism": "replicas" if world > 1 else "single GPU"},
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(n * 32),
                    "d2h_bytes_per_step": int(n * 24),
                    "path": ("lcx_trace_closest_host via ctypes, pinned host rays and hits: the traversal kernel "
                             "reads the rays from and writes the hits to host memory over the coherent CPU-GPU "
                             "link (NVLink-C2C), no staging copies" if coherent.value and mode.value == C.HOST_DIRECT
                             else "lcx_trace_closest_host via ctypes: pinned host rays and hits, streamed (one "
                                  "traversal launch takes each 2^17-ray copy chunk as it lands; finished chunks are "
                                  "copied out while it runs), all copies in the timed region"),
                    "direct_host_access_value": direct_value,
                    "staged_value": staged_value,
                    "serial_copies_value": n * e2e_steps / (e2e_serial_ms / 1e3) / 1e9},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "peak_source": peak_src,
                         "traffic": None if traffic_pr is None else traffic_pr * n,
                         "traffic_source": None if traffic_pr is None else
                         ("profiles/trace_closest_quant8_terrain.md: ncu dram__bytes_read.sum + dram__bytes_write.sum "
                          "of one full-size launch of this kernel in an earlier capture (per ray, times the rays "
                          "of this run); not measured in this run"),
                         "algorithmic_bytes_per_ray": bytes_per_ray,
                         "visits_per_ray": {"nodes": c[0], "triangles": c[1], "instances": c[2]},
                         "kernel": kernel_name,
                         "visits_from": (f"the counting build of the timed loop structure (loop mode {knobs[2].value}"
                                         f"{', quantised nodes' if args.layout == 1 else ''}) on the same rays, "
                                         "before the timed region")},
            "clocks": clocks.summary(),
            "gpu_launches": args.steps}
    if tuned is not None:
        line["config"]["autotune"] = tuned

    shadow_np = occ_np = fp32_equal = None
    if rank == 0 and not args.no_extra:
        extra = {"build_wall_s_all_meshes_and_tlas": build_wall_s}
        try:
            other = 0 if args.layout == 1 else 1
            for _ in range(3):
                acc.trace_closest(d_rays, out=d_hits, layout=other)
            torch.cuda.synchronize()
            x0, x1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            x0.record(stream)
            for _ in range(5):
                acc.trace_closest(d_rays, out=d_hits, layout=other)
            x1.record(stream)
            torch.cuda.synchronize()
            extra["closest_grays_" + ("fp32" if other == 0 else "quant8")] = n * 5 / (x0.elapsed_time(x1) / 1e3) / 1e9
            fp32_equal = np.array_equal(hits_to_numpy(d_hits).view(np.uint8), dev_hits.view(np.uint8))
            shadow_np = S.terrain_shadow_rays(scene, n, seed=5)
            sh = rays_to_device(shadow_np)
            occ = torch.empty(n, dtype=torch.uint8, device="cuda")
            for _ in range(3):
                acc.trace_any(sh, out=occ, layout=args.layout)
            torch.cuda.synchronize()
            x0.record(stream)
            for _ in range(5):
                acc.trace_any(sh, out=occ, layout=args.layout)
            x1.record(stream)
            torch.cuda.synchronize()
            extra["any_shadow_grays"] = n * 5 / (x0.elapsed_time(x1) / 1e3) / 1e9
            extra["shadow_occluded_frac"] = float(occ.float().mean().item())
            occ_np = occ.cpu().numpy()
            st = acc.stats()
            extra["tlas"] = {"nodes": int(st.node_count), "depth": int(st.depth), "max_blas_depth": int(st.max_blas_depth)}
            ms0 = meshes[0].stats()
            extra["terrain_blas"] = {"nodes": int(ms0.node_count), "depth": int(ms0.depth),
                                     "sah_binary": ms0.sah_cost, "sah_wide": ms0.wide_sah_cost,
                                     "device_mib": ms0.device_bytes / 2**20}
            del sh, occ
        except Exception as e:  # extras never fail the bench
            extra["error"] = repr(e)
        # the other forms, each a bounded leg (a failing leg records its error)
        for name, leg in (("per_thread_device_calls", lambda: leg_per_thread(acc, d_rays, d_hits, n, stream)),
                          ("multi_job_vs_one_at_a_time", lambda: leg_multi_job(acc, stream)),
                          ("batched_build_512_meshes", lambda: leg_batch_build(stream)),
                          ("pathtrace_1080p_4spp", lambda: leg_pathtrace(scene, acc, meshes, stream)),
                          ("serving_short_mix", leg_serving)):
            t0 = time.perf_counter()
            try:
                extra[name] = leg()
            except Exception as e:
                extra[name] = {"error": repr(e)}
            extra[name]["leg_wall_s"] = time.perf_counter() - t0
        line["extra"] = extra

    if rank == 0 and not args.no_cpu_baseline:
        import oracle
        oracle.build()
        t0 = time.perf_counter()
        osc = oracle.OracleScene(scene)
        build_s = time.perf_counter() - t0
        line["cpu_baseline"], base_hits = cpu_baseline(osc, rays, build_s)
        host_hits = h_hits.numpy().view(S.HIT_DTYPE).reshape(-1)
        line["parity"] = headline_parity(osc, rays, dev_hits, host_hits, base_hits, shadow_np, occ_np, fp32_equal)
        osc.close()
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
