// noalloc.cu — trace_closest for callers that cannot allocate device memory.
//
// The regular entry points keep their per-call scratch (the persistent-warp
// ray counter and an error word) in a per-device pool that the first call on
// a device creates with cudaMalloc.  Some callers cannot accept that: an
// application that reserves all of its HBM at start-up and forbids later
// allocations, a plugin whose host framework owns every device allocation, or
// a latency-bound loop that must not hit cudaMalloc's implicit device-wide
// synchronisation.  lcx_trace_closest_noalloc serves them: its scratch is the
// file-scope array below, which every GPU that loads this library holds until
// the process exits, and nothing on its path calls cudaMalloc, cudaFree or an
// allocating library routine.
#include <mutex>

#include "lcx_internal.h"

namespace {

// Scratch of the allocation-free trace: word 0 = ray counter, word 1 = error
// flags, the rest reserved.  Every call shares it.
constexpr int kNoAllocScratchWords = 64;  // 256 B
static __device__ __align__(256) uint32_t g_noalloc_scratch[kNoAllocScratchWords];

// Largest ray_count: warps overshoot the 32-bit counter by at most 32 rays
// each, so 2^31 rays keep it from wrapping.
constexpr uint32_t kNoAllocMaxRays = 1u << 31;

constexpr int kMaxDevices = 64;
std::mutex g_setup_mtx;
uint32_t *g_scratch_addr[kMaxDevices] = {};

// Device address of g_noalloc_scratch on the current device.  In host code the
// symbol's name is only a host-side stand-in, never a device address, so it is
// looked up once per device with that device current.  The address is kept for
// the life of the process: after cudaDeviceReset (a new primary context) the
// entry point must not be called again in that process.
int scratch_address(uint32_t **out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return lcx::record_error(LCX_ERR_CUDA, cudaGetErrorString(e));
    if (dev < 0 || dev >= kMaxDevices) return lcx::record_error(LCX_ERR_INVALID_ARG, "device index out of range");
    std::lock_guard<std::mutex> lk(g_setup_mtx);
    if (g_scratch_addr[dev] == nullptr) {
        void *ptr = nullptr;
        e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
        if (e != cudaSuccess || ptr == nullptr) {
            cudaGetLastError();
            return lcx::record_error(LCX_ERR_CUDA, e != cudaSuccess ? cudaGetErrorString(e)
                                                                    : "cudaGetSymbolAddress returned null");
        }
        g_scratch_addr[dev] = static_cast<uint32_t *>(ptr);
    }
    *out = g_scratch_addr[dev];
    return LCX_OK;
}

}  // namespace

namespace lcx {

// The kernel-side error flags (stack overflow, step bound) the allocation-free
// trace left in its scratch on the current device, cleared as they are read;
// 0 when it never ran there.  lcx_check_trace_errors calls it after its device
// synchronisation, so no call of the entry point is in flight.
int noalloc_take_errors(uint32_t *flags) {
    *flags = 0;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return record_error(LCX_ERR_CUDA, cudaGetErrorString(e));
    if (dev < 0 || dev >= kMaxDevices) return LCX_OK;
    uint32_t *addr = nullptr;
    {
        std::lock_guard<std::mutex> lk(g_setup_mtx);
        addr = g_scratch_addr[dev];
    }
    if (addr == nullptr) return LCX_OK;
    e = cudaMemcpy(flags, addr + 1, sizeof(uint32_t), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && *flags != 0u) e = cudaMemset(addr + 1, 0, sizeof(uint32_t));
    if (e != cudaSuccess) {
        cudaGetLastError();
        return record_error(LCX_ERR_CUDA, cudaGetErrorString(e));
    }
    return LCX_OK;
}

}  // namespace lcx

extern "C" int lcx_trace_closest_noalloc(uint64_t accel, const LcxRay *d_rays, uint32_t ray_count, uint32_t mask,
                                         LcxTriangleHit *d_hits, void *stream) {
    lcx::TraceParams p;
    std::shared_lock<std::shared_mutex> life(lcx::lifetime_mutex());  // until the kernel is enqueued
    if (int r = lcx::trace_params_for(accel, d_rays, ray_count, mask, d_hits, kNoAllocMaxRays, p)) return r;
    if (ray_count == 0) return LCX_OK;
    uint32_t *scratch = nullptr;
    if (int r = scratch_address(&scratch)) return r;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    // the array keeps the previous call's counter: clear it (and the error word)
    cudaError_t e = cudaMemsetAsync(scratch, 0, 2 * sizeof(uint32_t), st);
    if (e == cudaSuccess) {
        p.pool = scratch;
        e = lcx::launch_trace(p, LCX_NODES_QUANT8, false, false, st);
    }
    if (e != cudaSuccess) {
        cudaGetLastError();
        return lcx::record_error(LCX_ERR_CUDA, cudaGetErrorString(e));
    }
    return LCX_OK;
}
