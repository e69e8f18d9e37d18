// User-side kernels over lcx::ray_query (include/lcx/ray_query.cuh), built by
// tests/test_ray_query_gpu.py as a small shared library: what an application
// kernel with an alpha-cutout RayQuery looks like.
#include <lcx/ray_query.cuh>

namespace {

// Procedural spheres: the sphere inscribed in each AABB (centre, radius from
// the x extent), intersected in object space; commits the nearest root >= t_min.
__device__ lcx::ProceduralDecision sphere(const lcx::ProceduralCandidate &c) {
    float oc[3], d[3];
    const float r = 0.5f * (c.aabb_max[0] - c.aabb_min[0]);
    for (int k = 0; k < 3; k++) {
        oc[k] = c.obj_origin[k] - 0.5f * (c.aabb_min[k] + c.aabb_max[k]);
        d[k] = c.obj_dir[k];
    }
    const float a = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
    const float b = oc[0] * d[0] + oc[1] * d[1] + oc[2] * d[2];
    const float cc = oc[0] * oc[0] + oc[1] * oc[1] + oc[2] * oc[2] - r * r;
    const float disc = b * b - a * cc;
    if (disc < 0.0f) return lcx::ProceduralDecision{lcx::kSkip, 0.0f};
    const float s = sqrtf(disc);
    float t = (-b - s) / a;
    if (t < c.ray.t_min) t = (-b + s) / a;
    return lcx::ProceduralDecision{lcx::kCommit, t};
}

// mode 0: commit every candidate (= lcx_trace_closest)
// mode 1: cutout closest hit: triangles with prim % cut == 0 are transparent
// mode 2: cutout any hit: the first opaque candidate ends the query
// mode 3: every triangle plus procedural spheres; hits[i]._pad = the hit type
__global__ void k_query(LcxAccelView view, const LcxRay *rays, uint32_t n, uint32_t mode, uint32_t cut,
                        LcxTriangleHit *hits, uint8_t *occluded) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (mode == 3) {
        const lcx::CommittedHit c = lcx::ray_query(
            view, rays[i], 0xffu, [](const lcx::TriangleCandidate &) { return int(lcx::kCommit); }, sphere);
        LcxTriangleHit h;
        h.inst = c.inst;
        h.prim = c.prim;
        h.bary[0] = c.bary_u;
        h.bary[1] = c.bary_v;
        h.committed_ray_t = c.t;
        h._pad = c.type;
        hits[i] = h;
        return;
    }
    const LcxTriangleHit h = lcx::ray_query(view, rays[i], 0xffu, [&](const lcx::TriangleCandidate &c) {
        if (mode == 0) return int(lcx::kCommit);
        if (c.prim % cut == 0u) return int(lcx::kSkip);
        return int(mode == 2 ? lcx::kCommitAndTerminate : lcx::kCommit);
    });
    if (mode == 2)
        occluded[i] = h.inst != 0xffffffffu ? 1u : 0u;
    else
        hits[i] = h;
}

// commit every candidate of a motion query at times[i] (= lcx_trace_closest_motion)
__global__ void k_query_motion(LcxAccelView view, const LcxRay *rays, const float *times, uint32_t n,
                               LcxTriangleHit *hits) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    hits[i] = lcx::ray_query_motion(view, rays[i], times[i], 0xffu,
                                    [](const lcx::TriangleCandidate &) { return int(lcx::kCommit); });
}

}  // namespace

extern "C" __attribute__((visibility("default"))) int rq_run_motion(const LcxAccelView *view, const LcxRay *rays,
                                                                    const float *times, uint32_t n,
                                                                    LcxTriangleHit *hits) {
    if (n == 0) return 0;
    if (!view || !rays || !times || !hits) return -1;
    k_query_motion<<<(n + 127) / 128, 128>>>(*view, rays, times, n, hits);
    if (cudaGetLastError() != cudaSuccess) return -5;
    return cudaDeviceSynchronize() == cudaSuccess ? 0 : -5;
}

extern "C" __attribute__((visibility("default"))) int rq_run(const LcxAccelView *view, const LcxRay *rays, uint32_t n,
                                                             uint32_t mode, uint32_t cut, LcxTriangleHit *hits,
                                                             uint8_t *occluded) {
    if (n == 0) return 0;
    if (!view || !rays || (mode == 2 ? !occluded : !hits) || cut == 0 || mode > 3) return -1;
    k_query<<<(n + 127) / 128, 128>>>(*view, rays, n, mode, cut, hits, occluded);
    if (cudaGetLastError() != cudaSuccess) return -5;
    return cudaDeviceSynchronize() == cudaSuccess ? 0 : -5;
}
