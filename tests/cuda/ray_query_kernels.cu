// User-side kernels over lcx::ray_query (include/lcx/ray_query.cuh), built by
// tests/test_ray_query_gpu.py as a small shared library: what an application
// kernel with an alpha-cutout RayQuery looks like.
#include <lcx/ray_query.cuh>

namespace {

// mode 0: commit every candidate (= lcx_trace_closest)
// mode 1: cutout closest hit: triangles with prim % cut == 0 are transparent
// mode 2: cutout any hit: the first opaque candidate ends the query
__global__ void k_query(LcxAccelView view, const LcxRay *rays, uint32_t n, uint32_t mode, uint32_t cut,
                        LcxTriangleHit *hits, uint8_t *occluded) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
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

}  // namespace

extern "C" __attribute__((visibility("default"))) int rq_run(const LcxAccelView *view, const LcxRay *rays, uint32_t n,
                                                             uint32_t mode, uint32_t cut, LcxTriangleHit *hits,
                                                             uint8_t *occluded) {
    if (n == 0) return 0;
    if (!view || !rays || (mode == 2 ? !occluded : !hits) || cut == 0 || mode > 2) return -1;
    k_query<<<(n + 127) / 128, 128>>>(*view, rays, n, mode, cut, hits, occluded);
    if (cudaGetLastError() != cudaSuccess) return -5;
    return cudaDeviceSynchronize() == cudaSuccess ? 0 : -5;
}
