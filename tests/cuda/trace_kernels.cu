// User-side kernels over lcx::trace_closest / lcx::trace_any
// (include/lcx/trace.cuh), built by tests/test_device_trace_gpu.py as a small
// shared library: what an application kernel that traces one ray per thread
// looks like, compiled the way an application would compile it.
#include <lcx/trace.cuh>

namespace {

// variant 0: local short stack; 1: 16 shared-memory entries per thread
__global__ void k_closest(LcxAccelView view, const LcxRay *rays, const float *times, uint32_t n, uint32_t mask,
                          uint32_t variant, LcxTriangleHit *hits) {
    __shared__ uint2 smem[16 * 128];
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const LcxRay ray = rays[i];
    if (variant == 1) {
        hits[i] = lcx::trace_closest<16>(view, ray, mask, lcx::ShortStack{smem + threadIdx.x, blockDim.x},
                                         times ? times[i] : 0.0f);
    } else {
        hits[i] = times ? lcx::trace_closest_motion(view, ray, times[i], mask) : lcx::trace_closest(view, ray, mask);
    }
}

__global__ void k_any(LcxAccelView view, const LcxRay *rays, const float *times, uint32_t n, uint32_t mask,
                      uint32_t variant, uint8_t *occluded) {
    __shared__ uint2 smem[16 * 128];
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const LcxRay ray = rays[i];
    bool o;
    if (variant == 1)
        o = lcx::trace_any<16>(view, ray, mask, lcx::ShortStack{smem + threadIdx.x, blockDim.x},
                               times ? times[i] : 0.0f);
    else
        o = times ? lcx::trace_any_motion(view, ray, times[i], mask) : lcx::trace_any(view, ray, mask);
    occluded[i] = o ? 1u : 0u;
}

}  // namespace

extern "C" __attribute__((visibility("default"))) int tk_closest(const LcxAccelView *view, const LcxRay *rays,
                                                                 const float *times, uint32_t n, uint32_t mask,
                                                                 uint32_t variant, LcxTriangleHit *hits) {
    if (n == 0) return 0;
    if (!view || !rays || !hits || variant > 1) return -1;
    k_closest<<<(n + 127) / 128, 128>>>(*view, rays, times, n, mask, variant, hits);
    if (cudaGetLastError() != cudaSuccess) return -5;
    return cudaDeviceSynchronize() == cudaSuccess ? 0 : -5;
}

extern "C" __attribute__((visibility("default"))) int tk_any(const LcxAccelView *view, const LcxRay *rays,
                                                             const float *times, uint32_t n, uint32_t mask,
                                                             uint32_t variant, uint8_t *occluded) {
    if (n == 0) return 0;
    if (!view || !rays || !occluded || variant > 1) return -1;
    k_any<<<(n + 127) / 128, 128>>>(*view, rays, times, n, mask, variant, occluded);
    if (cudaGetLastError() != cudaSuccess) return -5;
    return cudaDeviceSynchronize() == cudaSuccess ? 0 : -5;
}
