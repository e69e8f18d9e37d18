// reorder.cu — ray reordering for trace calls.
//
// Before the traversal the rays of a call are sorted by a 32-bit key: the
// direction octant above the Morton code of the origin's cell in the scene box
// (the TLAS root's bounds, `bits` per axis).  The traversal then takes rays in
// that order through a permutation, so the lanes of a warp start in the same
// region heading the same way and share their first TLAS and BLAS nodes in L1.
// Results are written to each ray's own slot, and the closest-hit rules make a
// ray's record independent of which rays it runs beside, so the output is the
// same bit for bit with or without reordering.
//
// Scratch (keys, permutation, CUB temporary storage) comes from a per-device
// stream-ordered memory pool (scratch_pool, also used by the path tracer) and
// is released on the call's stream after the traversal, so concurrent calls on
// different streams never share it.
#include <cub/device/device_radix_sort.cuh>

#include <cstdio>
#include <mutex>

#include "lcx_internal.h"

namespace lcx {
namespace {

int cuda_error(cudaError_t e, const char *what) {
    char buf[256];
    snprintf(buf, sizeof(buf), "%s: %s", what, cudaGetErrorString(e));
    return record_error(LCX_ERR_CUDA, buf);
}

#define RO_CUDA(call, what)                                 \
    do {                                                    \
        cudaError_t e_ = (call);                            \
        if (e_ != cudaSuccess) return cuda_error(e_, what); \
    } while (0)

__device__ __forceinline__ uint32_t spread10(uint32_t x) {  // bit i -> bit 3i, i < 10
    x &= 0x3ffu;
    x = (x | (x << 16)) & 0x030000FFu;
    x = (x | (x << 8)) & 0x0300F00Fu;
    x = (x | (x << 4)) & 0x030C30C3u;
    x = (x | (x << 2)) & 0x09249249u;
    return x;
}

__global__ void k_ray_keys(const Ray *rays, uint32_t n, const Node8F *root, uint32_t bits, uint32_t *keys,
                           uint32_t *vals) {
    __shared__ float box[6];
    if (threadIdx.x == 0) {
        // union of the root's child boxes (Node8F planes: lo_x[8] hi_x[8] lo_y[8] ...; meta bytes in word 50..51)
        const float *pl = reinterpret_cast<const float *>(root);
        const uint32_t *hdr = reinterpret_cast<const uint32_t *>(root) + 48;
        float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
        for (int s = 0; s < 8; s++) {
            if (((hdr[2 + (s >> 2)] >> (8 * (s & 3))) & 0xffu) == 0u) continue;
            for (int k = 0; k < 3; k++) {
                lo[k] = fminf(lo[k], pl[16 * k + s]);
                hi[k] = fmaxf(hi[k], pl[16 * k + 8 + s]);
            }
        }
        for (int k = 0; k < 3; k++) {
            const bool ok = lo[k] <= hi[k];
            box[k] = ok ? lo[k] : 0.0f;
            box[3 + k] = ok && hi[k] > lo[k] ? float(1u << bits) / (hi[k] - lo[k]) : 0.0f;
        }
    }
    __syncthreads();
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 *rp = reinterpret_cast<const float4 *>(rays + i);
    const float4 r0 = __ldg(rp), r1 = __ldg(rp + 1);
    const float o[3] = {r0.x, r0.y, r0.z};
    const uint32_t qmax = (1u << bits) - 1u;
    uint32_t q[3];
#pragma unroll
    for (int k = 0; k < 3; k++) {
        const float f = (o[k] - box[k]) * box[3 + k];  // NaN origins land in cell 0
        q[k] = f > 0.0f ? min(uint32_t(fminf(f, float(qmax))), qmax) : 0u;
    }
    const uint32_t oct = (r1.x < 0.0f ? 4u : 0u) | (r1.y < 0.0f ? 2u : 0u) | (r1.z < 0.0f ? 1u : 0u);
    keys[i] = (oct << (3 * bits)) | (spread10(q[0]) << 2) | (spread10(q[1]) << 1) | spread10(q[2]);
    vals[i] = i;
}

struct PoolEntry {
    int device = -1;
    cudaMemPool_t pool = nullptr;
};
std::mutex g_pool_mtx;
PoolEntry g_pools[64];

}  // namespace

// A memory pool of our own per device that keeps freed blocks for reuse.
int scratch_pool(cudaMemPool_t *out) {
    int dev = 0;
    RO_CUDA(cudaGetDevice(&dev), "cudaGetDevice");
    if (dev < 0 || dev >= 64) return record_error(LCX_ERR_INVALID_ARG, "device ordinal out of range");
    std::lock_guard<std::mutex> lk(g_pool_mtx);
    PoolEntry &e = g_pools[dev];
    if (!e.pool) {
        cudaMemPoolProps props{};
        props.allocType = cudaMemAllocationTypePinned;
        props.location.type = cudaMemLocationTypeDevice;
        props.location.id = dev;
        RO_CUDA(cudaMemPoolCreate(&e.pool, &props), "cudaMemPoolCreate");
        uint64_t keep = ~0ull;
        RO_CUDA(cudaMemPoolSetAttribute(e.pool, cudaMemPoolAttrReleaseThreshold, &keep), "pool release threshold");
        e.device = dev;
    }
    *out = e.pool;
    return LCX_OK;
}

int reorder_begin(const Ray *rays, uint32_t n, const Node8F *tlas_root, uint32_t bits, cudaStream_t st,
                  ReorderScratch *rs) {
    *rs = ReorderScratch{};
    if (bits < 1 || bits > 9) return record_error(LCX_ERR_INVALID_ARG, "reorder bits out of range 1..9");
    cudaMemPool_t pool;
    if (int r = scratch_pool(&pool)) return r;
    size_t temp = 0;
    RO_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, temp, static_cast<const uint32_t *>(nullptr),
                                             static_cast<uint32_t *>(nullptr), static_cast<const uint32_t *>(nullptr),
                                             static_cast<uint32_t *>(nullptr), int(n), 0, int(3 * bits + 3), st),
             "reorder sort size");
    const size_t arr = (size_t(n) * 4 + 255) & ~size_t(255);
    const size_t total = 4 * arr + temp;
    void *mem = nullptr;
    RO_CUDA(cudaMallocFromPoolAsync(&mem, total, pool, st), "reorder scratch");
    char *base = static_cast<char *>(mem);
    uint32_t *kin = reinterpret_cast<uint32_t *>(base), *kout = reinterpret_cast<uint32_t *>(base + arr);
    uint32_t *vin = reinterpret_cast<uint32_t *>(base + 2 * arr), *vout = reinterpret_cast<uint32_t *>(base + 3 * arr);
    k_ray_keys<<<(n + 255) / 256, 256, 0, st>>>(rays, n, tlas_root, bits, kin, vin);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess)
        e = cub::DeviceRadixSort::SortPairs(base + 4 * arr, temp, kin, kout, vin, vout, int(n), 0, int(3 * bits + 3),
                                            st);
    if (e != cudaSuccess) {
        cudaFreeAsync(mem, st);
        return cuda_error(e, "ray reorder");
    }
    rs->mem = mem;
    rs->order = vout;
    return LCX_OK;
}

int reorder_end(ReorderScratch *rs, cudaStream_t st) {
    if (!rs->mem) return LCX_OK;
    const cudaError_t e = cudaFreeAsync(rs->mem, st);
    rs->mem = nullptr;
    rs->order = nullptr;
    if (e != cudaSuccess) return cuda_error(e, "reorder scratch release");
    return LCX_OK;
}

}  // namespace lcx
