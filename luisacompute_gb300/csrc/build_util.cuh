// build_util.cuh — device helpers shared by the BVH build translation units
// (build.cu: boxes, Morton codes, LBVH, collapse, emit; sah.cu: binned-SAH trees).
#pragma once

#include <cfloat>
#include <cstdint>

#include "lcx_internal.h"

namespace lcx {
namespace {

constexpr uint32_t kLeafBit = 0x80000000u;  // a binary-tree child that is an item (its sorted position)
constexpr int kSahBins = 16;                 // centroid bins per axis of the binned-SAH builds

inline unsigned blocks_for(uint64_t n, unsigned bs) { return unsigned((n + bs - 1) / bs); }

__device__ __forceinline__ bool box_empty(const float4 &lo, const float4 &hi) {
    return !(lo.x <= hi.x && lo.y <= hi.y && lo.z <= hi.z);
}

__device__ __forceinline__ float box_area(const float4 &lo, const float4 &hi) {
    if (box_empty(lo, hi)) return 0.0f;
    const float dx = hi.x - lo.x, dy = hi.y - lo.y, dz = hi.z - lo.z;
    return 2.0f * (dx * dy + dy * dz + dz * dx);
}

// Segment of global item i: binary search over the segment table.
__device__ __forceinline__ uint32_t segment_of(const SegInput *segs, uint32_t nseg, uint32_t i) {
    uint32_t lo = 0, hi = nseg - 1;
    while (lo < hi) {
        const uint32_t mid = (lo + hi + 1) >> 1;
        if (segs[mid].item_offset <= i)
            lo = mid;
        else
            hi = mid - 1;
    }
    return lo;
}

// Centroid of an item box; an empty box (an invalid item) counts as the origin.
__device__ __forceinline__ float3 centroid_of(const float4 &l, const float4 &h) {
    if (box_empty(l, h)) return make_float3(0.0f, 0.0f, 0.0f);
    return make_float3(0.5f * (l.x + h.x), 0.5f * (l.y + h.y), 0.5f * (l.z + h.z));
}
__device__ __forceinline__ float axis_of(const float3 &c, int k) { return k == 0 ? c.x : (k == 1 ? c.y : c.z); }
__device__ __forceinline__ float area3(const float3 &l, const float3 &h) {
    if (!(l.x <= h.x && l.y <= h.y && l.z <= h.z)) return 0.0f;
    const float dx = h.x - l.x, dy = h.y - l.y, dz = h.z - l.z;
    return 2.0f * (dx * dy + dy * dz + dz * dx);
}

}  // namespace
}  // namespace lcx
