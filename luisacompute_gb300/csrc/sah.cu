// sah.cu — binned-SAH binary trees for FAST_TRACE BLAS builds and for TLAS builds.
//
// The reference hands its builds to Embree (src/rust/luisa_compute_backend_impl/src/cpu/accel.rs:
// 58-61 asks for RTC_BUILD_QUALITY_HIGH on FAST_TRACE meshes) and to OptiX
// (src/backends/cuda/cuda_primitive.cpp:20-113 with OPTIX_BUILD_FLAG_PREFER_FAST_TRACE), both
// SAH builders.  This is the top-down binned SAH of Wald (2007, "On fast Construction of
// SAH-based Bounding Volume Hierarchies"): every range of items is split at the bin boundary of
// least cost A_L N_L + A_R N_R over 16 centroid bins on each axis, down to single items.  The
// tree is written in the layout the LBVH pass writes (items reordered so that every node covers
// a contiguous range, the internal node splitting [a, m) | [m, b) at index m - 1, leaves as
// sorted positions, segment roots in segctl[kSegRoot]), so the binary SAH, bounding spheres,
// collapse and emit passes run on it unchanged.
//
// Large ranges (more than kSahChunk items) are split level by level, every segment of the build
// at once:
//   k_sah_bin      bins the items of every large range: a block takes kSahChunk consecutive
//                  positions, which meet at most two large ranges, bins them into per-warp
//                  shared-memory bins (one reduced update when the warp's items share a bin),
//                  and merges those into the range's bins with global atomics;
//   k_sah_split    one warp per large range: prefix and suffix sweeps over its bins, the split of
//                  least cost (the position median when no bin boundary separates the items),
//                  the internal node, and the two child ranges (large ones to the next level, the
//                  others to the list of small ranges);
//   k_sah_flag     marks the items that go left; an exclusive scan of the marks (CUB) places
//   k_sah_scatter  every item: a stable partition of the item ids.
// Small ranges: k_sah_small, one block per range, builds the whole subtree in shared memory with
// one warp per open range.
//
// A large range's bins cover its box (its items' centroids lie inside it); small ranges bin over
// their exact centroid bounds.  The bin of an item is computed by one function from the same
// stored origin and scale in k_sah_bin and k_sah_flag, so the counts the split is chosen from are
// the counts the partition produces; the scatter still checks every destination against its
// range and flags a mismatch, and any flagged error rebuilds the tree with the LBVH.
#include <cub/device/device_scan.cuh>

#include <algorithm>
#include <cfloat>

#include "build_util.cuh"
#include "lcx_internal.h"

namespace lcx {
namespace {

#ifndef LCX_SAH_CHUNK
// items of the ranges one block builds (k_sah_small): terrain BLAS 4.86 / 4.83 / 5.51 ms and a
// 1024-mesh batch 57.0 / 58.2 / 71.6 ms at 1024 / 512 / 256, traversal the same
#define LCX_SAH_CHUNK 1024
#endif
constexpr uint32_t kSahChunk = LCX_SAH_CHUNK;                  // large ranges hold more items
constexpr uint32_t kBinWords = 7;                              // count, lo xyz, hi xyz (ordered-uint floats)
constexpr uint32_t kTaskBinWords = 3 * kSahBins * kBinWords;  // 336 words of bins per range
constexpr uint32_t kTaskWords = 16;
// Depth bounds: from level kSahMedianLevel of the large ranges, and from level kSahSmallMedian
// within a small range, ranges split at the position median, so the tree stays within
// kSahMedianLevel + 21 + kSahSmallMedian + 10 binary levels whatever the input.
constexpr uint32_t kSahMedianLevel = 32;
constexpr uint32_t kSahMaxLevels = kSahMedianLevel + 40;
constexpr uint32_t kSahSmallMedian = 24;
constexpr uint32_t kBinThreads = 256, kBinWarps = kBinThreads / 32;
constexpr uint32_t kSmallThreads = 128, kSmallWarps = kSmallThreads / 32;
#ifndef LCX_SAH_THREAD_RANGE
#define LCX_SAH_THREAD_RANGE 16
#endif
constexpr uint32_t kThreadRange = LCX_SAH_THREAD_RANGE;  // ranges of at most this many items: one thread
// bins per axis in the small ranges' warps: 8 built the terrain BLAS 3 % faster but made the
// 257-instance TLAS SAH 15.2 -> 15.8 and traversal 1.5 % slower
constexpr int kSmallBins = kSahBins;

// control words: small-range count, large-range counts of the two level parities, error bits
enum : uint32_t { kCtrSmall = 0, kCtrLarge = 1, kCtrErr = 3, kCtrWords = 8 };
enum : uint32_t { kSahErrScatter = 1u, kSahErrCap = 2u, kSahErrSmall = 4u };
// large-range record: [a, b), parent node + 1 (0: the segment root), side (the segment for a
// root), bin origin and scale per axis, then the split: axis (3 = position median), bin, m, and
// the child ranges' records in the next level (kInvalid: small)
enum : uint32_t {
    kTA = 0,
    kTB = 1,
    kTParent = 2,
    kTSide = 3,
    kTLo = 4,
    kTScale = 7,
    kTAxis = 10,
    kTBin = 11,
    kTM = 12,
    kTLeft = 13,
    kTRight = 14,
};

struct SahLayout {
    uint32_t *ctr, *small, *task[2], *bins[2];
    uint32_t *pos_task[2];  // range record of every position (kInvalid: not in a large range)
    uint32_t *flags, *scan, *seg_task;
    uint32_t cap;  // large ranges per level: disjoint, each above kSahChunk items
};

// Carves the SAH build's arrays out of the LBVH scratch it does not use: the collapse's
// descriptor words (12 per item) hold the control words, the small ranges (4 words each, at most
// one per item) and the large ranges with their bins; the Morton keys hold the range of every
// position (two levels), the sorted keys the marks and their scan; the collapse queue the large
// range of every segment at level 0.
SahLayout sah_layout(const BuildScratch &s) {
    SahLayout L;
    const uint32_t n = s.n;
    L.cap = n / (kSahChunk + 1);
    uint32_t *w = s.desc;
    L.ctr = w;
    w += kCtrWords;
    L.small = w;
    w += 4ull * n;
    for (int p = 0; p < 2; p++) {
        L.task[p] = w;
        w += size_t(kTaskWords) * L.cap;
    }
    for (int p = 0; p < 2; p++) {
        L.bins[p] = w;
        w += size_t(kTaskBinWords) * L.cap;
    }
    uint32_t *keys = reinterpret_cast<uint32_t *>(s.keys);
    L.pos_task[0] = keys;
    L.pos_task[1] = keys + n;
    uint32_t *sorted = reinterpret_cast<uint32_t *>(s.keys_sorted);
    L.flags = sorted;
    L.scan = sorted + n;
    L.seg_task = reinterpret_cast<uint32_t *>(s.queue);
    return L;
}

__device__ __forceinline__ uint32_t bin_init(uint32_t word) {
    const uint32_t k = word % kBinWords;
    return k == 0 ? 0u : (k < 4 ? 0xffffffffu : 0u);
}
__device__ __forceinline__ float bin_lo_of(uint32_t v) { return v == 0xffffffffu ? FLT_MAX : ordered_to_float(v); }
__device__ __forceinline__ float bin_hi_of(uint32_t v) { return v == 0u ? -FLT_MAX : ordered_to_float(v); }

// Bins per unit length over [lo, hi]; 0 (every item in bin 0) for an empty, degenerate or
// non-finite extent.
template <int B = kSahBins>
__device__ __forceinline__ float sah_scale(float lo, float hi) {
    const float e = hi - lo;
    const float s = e > 0.0f ? float(B) / e : 0.0f;
    return isfinite(s) ? s : 0.0f;
}
// The bin of centroid coordinate c: clamped to [0, B - 1]; NaN goes to bin 0.
template <int B = kSahBins>
__device__ __forceinline__ int sah_bin(float c, float lo, float scale) {
    return int(fminf(fmaxf((c - lo) * scale, 0.0f), float(B - 1)));
}

// Adds one item per valid lane to three bins of `bins` (keys[q]: its bin key on axis q; every lane
// of the warp calls).  For each axis whose key the valid lanes share, one lane adds the warp's count
// and box (reduced once for all such axes); on the other axes each valid lane adds its own.
__device__ __forceinline__ void bin_add3(uint32_t *bins, const uint32_t keys[3], bool valid, const float4 &l,
                                         const float4 &h) {
    const unsigned vm = __ballot_sync(~0u, valid);
    if (vm == 0u) return;
    const uint32_t first = __ffs(vm) - 1u;
    bool uni[3];
    bool any = false;
#pragma unroll
    for (int q = 0; q < 3; q++) {
        const uint32_t k0 = __shfl_sync(~0u, keys[q], first);
        uni[q] = __all_sync(~0u, !valid || keys[q] == k0);
        any = any || uni[q];
    }
    float v[6] = {valid ? l.x : FLT_MAX,  valid ? l.y : FLT_MAX,  valid ? l.z : FLT_MAX,
                  valid ? h.x : -FLT_MAX, valid ? h.y : -FLT_MAX, valid ? h.z : -FLT_MAX};
    if (any) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
            for (int q = 0; q < 3; q++) v[q] = fminf(v[q], __shfl_xor_sync(~0u, v[q], o));
#pragma unroll
            for (int q = 3; q < 6; q++) v[q] = fmaxf(v[q], __shfl_xor_sync(~0u, v[q], o));
        }
    }
    const bool leader = (threadIdx.x & 31u) == first;
#pragma unroll
    for (int q = 0; q < 3; q++) {
        if (uni[q] ? leader : valid) {
            uint32_t *b = bins + size_t(keys[q]) * kBinWords;
            atomicAdd(b, uni[q] ? uint32_t(__popc(vm)) : 1u);
            atomicMin(b + 1, float_to_ordered(uni[q] ? v[0] : l.x));
            atomicMin(b + 2, float_to_ordered(uni[q] ? v[1] : l.y));
            atomicMin(b + 3, float_to_ordered(uni[q] ? v[2] : l.z));
            atomicMax(b + 4, float_to_ordered(uni[q] ? v[3] : h.x));
            atomicMax(b + 5, float_to_ordered(uni[q] ? v[4] : h.y));
            atomicMax(b + 6, float_to_ordered(uni[q] ? v[5] : h.z));
        }
    }
}

__device__ __forceinline__ float3 fmin3(const float3 &a, const float3 &b) {
    return make_float3(fminf(a.x, b.x), fminf(a.y, b.y), fminf(a.z, b.z));
}
__device__ __forceinline__ float3 fmax3(const float3 &a, const float3 &b) {
    return make_float3(fmaxf(a.x, b.x), fmaxf(a.y, b.y), fmaxf(a.z, b.z));
}
__device__ __forceinline__ float3 shfl3(const float3 &v, int src, int width = 32) {
    return make_float3(__shfl_sync(~0u, v.x, src, width), __shfl_sync(~0u, v.y, src, width),
                       __shfl_sync(~0u, v.z, src, width));
}
__device__ __forceinline__ float3 shfl_up3(const float3 &v, unsigned d) {
    return make_float3(__shfl_up_sync(~0u, v.x, d, 16), __shfl_up_sync(~0u, v.y, d, 16),
                       __shfl_up_sync(~0u, v.z, d, 16));
}
__device__ __forceinline__ float3 shfl_down3(const float3 &v, unsigned d) {
    return make_float3(__shfl_down_sync(~0u, v.x, d, 16), __shfl_down_sync(~0u, v.y, d, 16),
                       __shfl_down_sync(~0u, v.z, d, 16));
}

// Lane j (and j + 16) of a warp: bins 0..j (prefix) and j..15 (suffix) of one axis.
__device__ __forceinline__ void sweep_axis(const uint32_t *axis_bins, uint32_t &pn, float3 &pl, float3 &ph,
                                           uint32_t &sn, float3 &sl, float3 &sh) {
    const uint32_t j = threadIdx.x & 15u;
    const uint32_t *b = axis_bins + j * kBinWords;
    pn = sn = b[0];
    pl = sl = make_float3(bin_lo_of(b[1]), bin_lo_of(b[2]), bin_lo_of(b[3]));
    ph = sh = make_float3(bin_hi_of(b[4]), bin_hi_of(b[5]), bin_hi_of(b[6]));
#pragma unroll
    for (unsigned d = 1; d < 16; d <<= 1) {
        const uint32_t un = __shfl_up_sync(~0u, pn, d, 16);
        const float3 ul = shfl_up3(pl, d), uh = shfl_up3(ph, d);
        const uint32_t dn = __shfl_down_sync(~0u, sn, d, 16);
        const float3 dl = shfl_down3(sl, d), dh = shfl_down3(sh, d);
        if (j >= d) {
            pn += un;
            pl = fmin3(pl, ul);
            ph = fmax3(ph, uh);
        }
        if (j + d < 16u) {
            sn += dn;
            sl = fmin3(sl, dl);
            sh = fmax3(sh, dh);
        }
    }
}

struct SahSplit {
    int axis;     // -1: no bin boundary separates the items
    int bin;      // items in bins <= bin go left
    uint32_t nl;  // items that go left
    float3 box_l, box_h, left_l, left_h, right_l, right_h;
};

// The split of least cost from a range's bins (3 axes x kSahBins bins x kBinWords words); every
// lane of the warp calls and gets the result.  Ties go to the lower axis, then the lower bin.
__device__ SahSplit best_split(const uint32_t *bins) {
    const uint32_t lane = threadIdx.x & 31u, j = lane & 15u, half = lane >> 4;
    SahSplit r;
    float best = FLT_MAX;
    uint32_t best_key = kInvalid;
    // two sweeps: axis 0 in lanes 0-15 and axis 1 in lanes 16-31, then axis 2 in both halves
    uint32_t pn[2], sn[2];
    float3 pl[2], ph[2], sl[2], sh[2];
#pragma unroll
    for (int it = 0; it < 2; it++) {
        const uint32_t k = it == 0 ? half : 2u;
        sweep_axis(bins + size_t(k) * kSahBins * kBinWords, pn[it], pl[it], ph[it], sn[it], sl[it], sh[it]);
        // split between bins j and j + 1: the suffix from bin j + 1
        const uint32_t rn = __shfl_down_sync(~0u, sn[it], 1, 16);
        const float3 rl = shfl_down3(sl[it], 1), rh = shfl_down3(sh[it], 1);
        const bool ok = j + 1u < uint32_t(kSahBins) && pn[it] > 0u && rn > 0u;
        const float cost = area3(pl[it], ph[it]) * float(pn[it]) + area3(rl, rh) * float(rn);
        if (ok && cost < best) {
            best = cost;
            best_key = k * kSahBins + j;
        }
    }
    r.box_l = shfl3(pl[0], 15);  // axis 0 over all bins: the range's box
    r.box_h = shfl3(ph[0], 15);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const float oc = __shfl_xor_sync(~0u, best, o);
        const uint32_t ok = __shfl_xor_sync(~0u, best_key, o);
        if (oc < best || (oc == best && ok < best_key)) {
            best = oc;
            best_key = ok;
        }
    }
    if (best_key == kInvalid) {
        r.axis = -1;
        r.bin = 0;
        r.nl = 0;
        r.left_l = r.right_l = r.box_l;
        r.left_h = r.right_h = r.box_h;
        return r;
    }
    r.axis = int(best_key / kSahBins);
    r.bin = int(best_key % kSahBins);
    const bool second = r.axis == 2;                           // warp-uniform
    const int src = (r.axis == 1 ? 16 : 0) + r.bin;            // the lane that swept the best split
    const uint32_t p_n = second ? pn[1] : pn[0];
    const float3 p_l = second ? pl[1] : pl[0], p_h = second ? ph[1] : ph[0];
    const float3 s_l = second ? sl[1] : sl[0], s_h = second ? sh[1] : sh[0];
    r.nl = __shfl_sync(~0u, p_n, src);
    r.left_l = shfl3(p_l, src);
    r.left_h = shfl3(p_h, src);
    r.right_l = shfl3(s_l, src + 1);
    r.right_h = shfl3(s_h, src + 1);
    return r;
}

// Links a child (an internal node, or kLeafBit | position) to its parent: `up` = 0 for a segment
// root, else parent node + 1 with the side in bit 31.
__device__ __forceinline__ void link_child(uint32_t up, uint32_t seg, uint32_t child, uint32_t *bin_child,
                                           uint32_t *segctl) {
    if (up == 0u)
        segctl[kSegWords * seg + kSegRoot] = child;
    else
        bin_child[2ull * ((up & 0x7fffffffu) - 1u) + (up >> 31)] = child;
}

// Level 0: a range per non-empty segment, large or small; bins of the large ones cleared.
__global__ void k_sah_seed(const SegInput *segs, uint32_t nseg, uint32_t cap, const uint32_t *segctl_in,
                           uint32_t *ctr, uint32_t *small, uint32_t *task, uint32_t *bins, uint32_t *seg_task) {
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nseg) return;
    const uint32_t a = segs[s].item_offset, cnt = segs[s].item_count;
    uint32_t id = kInvalid;
    if (cnt > kSahChunk) {
        id = atomicAdd(&ctr[kCtrLarge], 1u);
        if (id >= cap) {
            atomicOr(&ctr[kCtrErr], kSahErrCap);
            id = kInvalid;
        } else {
            uint32_t *rec = task + size_t(kTaskWords) * id;
            rec[kTA] = a;
            rec[kTB] = a + cnt;
            rec[kTParent] = 0u;
            rec[kTSide] = s;
            for (int k = 0; k < 3; k++) {  // the segment's centroid bounds
                const float lo = ordered_to_float(segctl_in[kSegWords * s + kSegCenLo + k]);
                const float hi = ordered_to_float(segctl_in[kSegWords * s + kSegCenHi + k]);
                rec[kTLo + k] = __float_as_uint(lo);
                rec[kTScale + k] = __float_as_uint(sah_scale(lo, hi));
            }
            uint32_t *b = bins + size_t(kTaskBinWords) * id;
            for (uint32_t q = 0; q < kTaskBinWords; q++) b[q] = bin_init(q);
        }
    } else if (cnt > 0u) {
        const uint32_t sid = atomicAdd(&ctr[kCtrSmall], 1u);
        uint32_t *r = small + 4ull * sid;
        r[0] = a;
        r[1] = a + cnt;
        r[2] = 0u;
        r[3] = s;
    }
    seg_task[s] = id;
}

__global__ void k_sah_mark(const SegInput *segs, uint32_t nseg, uint32_t n, const uint32_t *seg_task,
                           uint32_t *pos_task, uint32_t *vals) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    pos_task[i] = seg_task[nseg > 1 ? segment_of(segs, nseg, i) : 0u];
    vals[i] = i;
}

__global__ void __launch_bounds__(kBinThreads) k_sah_bin(uint32_t n, const uint32_t *pos_task, const uint32_t *vals,
                                                           const float4 *lo, const float4 *hi, const uint32_t *task,
                                                           uint32_t *bins) {
    __shared__ uint32_t wb[kBinWarps][2 * kTaskBinWords];
    __shared__ uint32_t t_min, t_max;
    constexpr uint32_t kPer = kSahChunk / kBinThreads;
    const uint32_t base = blockIdx.x * kSahChunk;
    uint32_t *flat = &wb[0][0];
    for (uint32_t w = threadIdx.x; w < kBinWarps * 2 * kTaskBinWords; w += kBinThreads) flat[w] = bin_init(w);
    if (threadIdx.x == 0) {
        t_min = kInvalid;
        t_max = 0u;
    }
    __syncthreads();
    uint32_t t[kPer];
    uint32_t lo_t = kInvalid, hi_t = 0u;
#pragma unroll
    for (uint32_t j = 0; j < kPer; j++) {
        const uint32_t i = base + j * kBinThreads + threadIdx.x;
        t[j] = i < n ? pos_task[i] : kInvalid;
        if (t[j] != kInvalid) {
            lo_t = min(lo_t, t[j]);
            hi_t = max(hi_t, t[j]);
        }
    }
    lo_t = __reduce_min_sync(~0u, lo_t);
    hi_t = __reduce_max_sync(~0u, hi_t);
    if ((threadIdx.x & 31u) == 0u && lo_t != kInvalid) {
        atomicMin(&t_min, lo_t);
        atomicMax(&t_max, hi_t);
    }
    __syncthreads();
    const uint32_t t0 = t_min, t1 = t_max;  // the chunk meets at most two large ranges
    if (t0 == kInvalid) return;
    uint32_t *mine = wb[threadIdx.x / 32u];
#pragma unroll 1
    for (uint32_t j = 0; j < kPer; j++) {
        const uint32_t i = base + j * kBinThreads + threadIdx.x;
        const bool valid = t[j] != kInvalid;
        float4 l = make_float4(FLT_MAX, FLT_MAX, FLT_MAX, 0.0f), h = make_float4(-FLT_MAX, -FLT_MAX, -FLT_MAX, 0.0f);
        float3 c = make_float3(0.0f, 0.0f, 0.0f);
        uint32_t slot = 0u;
        const uint32_t *rec = task;
        if (valid) {
            const uint32_t it = vals[i];
            l = lo[it];
            h = hi[it];
            c = centroid_of(l, h);
            slot = t[j] == t0 ? 0u : 1u;
            rec = task + size_t(kTaskWords) * t[j];
        }
        uint32_t keys[3];
#pragma unroll
        for (int k = 0; k < 3; k++) {
            const int b =
                valid ? sah_bin(axis_of(c, k), __uint_as_float(rec[kTLo + k]), __uint_as_float(rec[kTScale + k])) : 0;
            keys[k] = slot * 3u * kSahBins + uint32_t(k) * kSahBins + uint32_t(b);
        }
        bin_add3(mine, keys, valid, l, h);
    }
    __syncthreads();
    for (uint32_t w = threadIdx.x; w < 2 * kTaskBinWords; w += kBinThreads) {
        const uint32_t slot = w / kTaskBinWords, word = w % kTaskBinWords, kind = word % kBinWords;
        if (slot == 1u && t1 == t0) continue;
        uint32_t v = wb[0][w];
        for (uint32_t q = 1; q < kBinWarps; q++) {
            const uint32_t x = wb[q][w];
            v = kind == 0u ? v + x : (kind < 4u ? min(v, x) : max(v, x));
        }
        uint32_t *g = bins + size_t(kTaskBinWords) * (slot ? t1 : t0) + word;
        if (kind == 0u) {
            if (v) atomicAdd(g, v);
        } else if (kind < 4u) {
            if (v != 0xffffffffu) atomicMin(g, v);
        } else if (v != 0u) {
            atomicMax(g, v);
        }
    }
}

// One warp per large range of this level (parity par): the split, the internal node, the links,
// and the child ranges.
__global__ void __launch_bounds__(128) k_sah_split(uint32_t par, uint32_t median, uint32_t cap, uint32_t n,
                                                   uint32_t *ctr, uint32_t *task, const uint32_t *bins,
                                                   uint32_t *task_next, uint32_t *bins_next, uint32_t *small,
                                                   float4 *bin_lo, float4 *bin_hi, uint32_t *bin_child,
                                                   uint32_t *segctl) {
    const uint32_t w = (blockIdx.x * blockDim.x + threadIdx.x) / 32u, lane = threadIdx.x & 31u;
    if (w >= min(ctr[kCtrLarge + par], cap)) return;  // warp-uniform
    uint32_t *rec = task + size_t(kTaskWords) * w;
    const uint32_t a = rec[kTA], b = rec[kTB], p1 = rec[kTParent], side = rec[kTSide];
    const SahSplit sp = best_split(bins + size_t(kTaskBinWords) * w);
    uint32_t axis = sp.axis < 0 || median ? 3u : uint32_t(sp.axis);
    uint32_t m = axis < 3u ? a + sp.nl : a + (b - a) / 2u;
    if (!(m > a && m < b)) {  // cannot happen with consistent bins; keep the tree valid anyway
        axis = 3u;
        m = a + (b - a) / 2u;
    }
    const uint32_t node = m - 1u;
    if (lane == 0) {
        bin_lo[node] = make_float4(sp.box_l.x, sp.box_l.y, sp.box_l.z, __uint_as_float(b - a));
        bin_hi[node] = make_float4(sp.box_h.x, sp.box_h.y, sp.box_h.z, __uint_as_float(a));
        link_child(p1 == 0u ? 0u : (p1 | (side << 31)), side, node, bin_child, segctl);
    }
    uint32_t ids[2];
    for (uint32_t c = 0; c < 2; c++) {
        const uint32_t ca = c ? m : a, cb = c ? b : m;
        uint32_t id = kInvalid;
        if (lane == 0) {
            if (cb - ca > kSahChunk) {
                id = atomicAdd(&ctr[kCtrLarge + (par ^ 1u)], 1u);
                if (id >= cap) {
                    atomicOr(&ctr[kCtrErr], kSahErrCap);
                    id = kInvalid;
                }
            } else {
                const uint32_t sid = atomicAdd(&ctr[kCtrSmall], 1u);
                if (sid < n) {
                    uint32_t *r = small + 4ull * sid;
                    r[0] = ca;
                    r[1] = cb;
                    r[2] = node + 1u;
                    r[3] = c;
                } else {
                    atomicOr(&ctr[kCtrErr], kSahErrCap);
                }
            }
        }
        id = __shfl_sync(~0u, id, 0);
        if (id != kInvalid) {
            if (lane == 0) {
                uint32_t *nr = task_next + size_t(kTaskWords) * id;
                nr[kTA] = ca;
                nr[kTB] = cb;
                nr[kTParent] = node + 1u;
                nr[kTSide] = c;
                const float3 cl = c ? sp.right_l : sp.left_l, ch = c ? sp.right_h : sp.left_h;
                for (int k = 0; k < 3; k++) {
                    if (axis == 3u) {  // a median split: the range's own bin domain
                        nr[kTLo + k] = rec[kTLo + k];
                        nr[kTScale + k] = rec[kTScale + k];
                    } else {  // the child's box
                        nr[kTLo + k] = __float_as_uint(axis_of(cl, k));
                        nr[kTScale + k] = __float_as_uint(sah_scale(axis_of(cl, k), axis_of(ch, k)));
                    }
                }
            }
            uint32_t *nb = bins_next + size_t(kTaskBinWords) * id;
            for (uint32_t q = lane; q < kTaskBinWords; q += 32u) nb[q] = bin_init(q);
        }
        ids[c] = id;
    }
    if (lane == 0) {
        rec[kTAxis] = axis;
        rec[kTBin] = uint32_t(sp.bin);
        rec[kTM] = m;
        rec[kTLeft] = ids[0];
        rec[kTRight] = ids[1];
    }
}

// 1 for the items of large ranges that go left; also clears this level's large-range count
// (read by k_sah_split, reused two levels on).
__global__ void k_sah_flag(uint32_t n, uint32_t par, uint32_t *ctr, const uint32_t *pos_task, const uint32_t *vals,
                           const float4 *lo, const float4 *hi, const uint32_t *task, uint32_t *flags) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i == 0) ctr[kCtrLarge + par] = 0u;
    if (i >= n) return;
    const uint32_t t = pos_task[i];
    uint32_t f = 0u;
    if (t != kInvalid) {
        const uint32_t *rec = task + size_t(kTaskWords) * t;
        const uint32_t axis = rec[kTAxis];
        if (axis >= 3u) {
            f = i < rec[kTM] ? 1u : 0u;
        } else {
            const uint32_t it = vals[i];
            const float3 c = centroid_of(lo[it], hi[it]);
            f = sah_bin(axis_of(c, int(axis)), __uint_as_float(rec[kTLo + axis]), __uint_as_float(rec[kTScale + axis])) <=
                        int(rec[kTBin])
                    ? 1u
                    : 0u;
        }
    }
    flags[i] = f;
}

__global__ void k_sah_scatter(uint32_t n, const uint32_t *pos_task, uint32_t *pos_task_out, const uint32_t *vals,
                              uint32_t *vals_out, const uint32_t *task, const uint32_t *flags, const uint32_t *scan,
                              uint32_t *ctr) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t t = pos_task[i], v = vals[i];
    if (t == kInvalid) {
        vals_out[i] = v;
        pos_task_out[i] = kInvalid;
        return;
    }
    const uint32_t *rec = task + size_t(kTaskWords) * t;
    const uint32_t a = rec[kTA], b = rec[kTB], m = rec[kTM];
    const uint32_t before = scan[i] - scan[a];  // items of the range before i that go left
    const bool left = flags[i] != 0u;
    const uint32_t dst = left ? a + before : m + (i - a - before);
    if (left ? dst >= m : (dst < m || dst >= b)) {
        atomicOr(&ctr[kCtrErr], kSahErrScatter);
        return;
    }
    vals_out[dst] = v;
    pos_task_out[dst] = left ? rec[kTLeft] : rec[kTRight];
}

__device__ __forceinline__ float4 sbox_lo(const float *box, uint32_t p) {
    return make_float4(box[p], box[kSahChunk + p], box[2 * kSahChunk + p], 0.0f);
}
__device__ __forceinline__ float4 sbox_hi(const float *box, uint32_t p) {
    return make_float4(box[3 * kSahChunk + p], box[4 * kSahChunk + p], box[5 * kSahChunk + p], 0.0f);
}

// Sort key of item p on an axis: its box midpoint (the sort only orders the candidates of a
// split, so it needs no agreement with the bins).
__device__ __forceinline__ float sort_key(const float *box, uint32_t p, int axis) {
#if LCX_SAH_SORT_KEY_FULL
    return axis_of(centroid_of(sbox_lo(box, p), sbox_hi(box, p)), axis);
#else
    return 0.5f * (box[axis * kSahChunk + p] + box[(axis + 3) * kSahChunk + p]);
#endif
}

// The subtree of a range of at most kThreadRange items, built by the calling thread alone with the
// exact SAH of every split position: at each node the items are sorted by centroid on each axis
// (a stable insertion sort of the range's order) and swept from both ends.  box: the block's item
// boxes (6 x kSahChunk floats), perm: its order; nodes and links as in the warp levels.
__device__ void thread_subtree(uint32_t ra0, uint32_t rb0, uint32_t up0, uint32_t a, uint32_t ss, uint16_t *perm,
                               const float *box, float4 *bin_lo, float4 *bin_hi, uint32_t *bin_child,
                               uint32_t *segctl) {
    uint32_t st_r[kThreadRange], st_up[kThreadRange];
    float rarea[kThreadRange];
    int sp = 0;
    st_r[sp] = ra0 | (rb0 << 16);
    st_up[sp++] = up0;
    while (sp > 0) {
        --sp;
        const uint32_t ra = st_r[sp] & 0xffffu, rb = st_r[sp] >> 16, up = st_up[sp], k = rb - ra;
        float4 nl = make_float4(FLT_MAX, FLT_MAX, FLT_MAX, 0.0f), nh = make_float4(-FLT_MAX, -FLT_MAX, -FLT_MAX, 0.0f);
        for (uint32_t i = ra; i < rb; i++) {
            const float4 l = sbox_lo(box, perm[i]), h = sbox_hi(box, perm[i]);
            nl = make_float4(fminf(nl.x, l.x), fminf(nl.y, l.y), fminf(nl.z, l.z), 0.0f);
            nh = make_float4(fmaxf(nh.x, h.x), fmaxf(nh.y, h.y), fmaxf(nh.z, h.z), 0.0f);
        }
        float best = FLT_MAX;
        int best_axis = -1;
        uint32_t best_pos = k / 2u;
        for (int axis = 0; axis < 3; axis++) {
            auto key = [&](uint32_t p) { return sort_key(box, p, axis); };
            for (uint32_t i = ra + 1u; i < rb; i++) {  // stable insertion sort by centroid
                const uint16_t p = perm[i];
                const float kp = key(p);
                uint32_t j = i;
                while (j > ra && key(perm[j - 1u]) > kp) {
                    perm[j] = perm[j - 1u];
                    j--;
                }
                perm[j] = p;
            }
            float3 l = make_float3(FLT_MAX, FLT_MAX, FLT_MAX), h = make_float3(-FLT_MAX, -FLT_MAX, -FLT_MAX);
            for (uint32_t i = rb - 1u; i > ra; i--) {  // rarea[j]: items j.. of the range
                const float4 bl = sbox_lo(box, perm[i]), bh = sbox_hi(box, perm[i]);
                l = fmin3(l, make_float3(bl.x, bl.y, bl.z));
                h = fmax3(h, make_float3(bh.x, bh.y, bh.z));
                rarea[i - ra] = area3(l, h);
            }
            l = make_float3(FLT_MAX, FLT_MAX, FLT_MAX);
            h = make_float3(-FLT_MAX, -FLT_MAX, -FLT_MAX);
            for (uint32_t i = ra; i + 1u < rb; i++) {  // split after item i
                const float4 bl = sbox_lo(box, perm[i]), bh = sbox_hi(box, perm[i]);
                l = fmin3(l, make_float3(bl.x, bl.y, bl.z));
                h = fmax3(h, make_float3(bh.x, bh.y, bh.z));
                const uint32_t nleft = i - ra + 1u;
                const float cost = area3(l, h) * float(nleft) + rarea[nleft] * float(k - nleft);
                if (cost < best) {
                    best = cost;
                    best_axis = axis;
                    best_pos = nleft;
                }
            }
        }
        if (best_axis >= 0 && best_axis != 2) {  // back to the order of the best axis
            const int axis = best_axis;
            auto key = [&](uint32_t p) { return sort_key(box, p, axis); };
            for (uint32_t i = ra + 1u; i < rb; i++) {
                const uint16_t p = perm[i];
                const float kp = key(p);
                uint32_t j = i;
                while (j > ra && key(perm[j - 1u]) > kp) {
                    perm[j] = perm[j - 1u];
                    j--;
                }
                perm[j] = p;
            }
        }
        const uint32_t m = ra + best_pos;
        const uint32_t node = a + m - 1u;
        bin_lo[node] = make_float4(nl.x, nl.y, nl.z, __uint_as_float(k));
        bin_hi[node] = make_float4(nh.x, nh.y, nh.z, __uint_as_float(a + ra));
        link_child(up, ss, node, bin_child, segctl);
        if (m - ra == 1u) {
            link_child(node + 1u, ss, kLeafBit | (a + ra), bin_child, segctl);
        } else {
            st_r[sp] = ra | (m << 16);
            st_up[sp++] = node + 1u;
        }
        if (rb - m == 1u) {
            link_child((node + 1u) | (1u << 31), ss, kLeafBit | (a + m), bin_child, segctl);
        } else {
            st_r[sp] = m | (rb << 16);
            st_up[sp++] = (node + 1u) | (1u << 31);
        }
    }
}

// One block per small range (at most kSahChunk items): the item boxes in shared memory, then
// level by level one warp per open range of more than kThreadRange items: exact centroid bounds,
// 16 bins per axis (their union is the node box), the split of least cost (the median when none
// separates the items, and from level kSahSmallMedian on), a stable ballot partition of the
// range's order, the internal node and the links; one-item children become leaves, children of
// 2..kThreadRange items go to a list (in tlist at the range's offset: at most one entry of two
// words per two items) that the block's threads then build one per thread (thread_subtree).
__global__ void __launch_bounds__(kSmallThreads) k_sah_small(uint32_t n, uint32_t *ctr, const uint32_t *small,
                                                             const uint32_t *vals_in, uint32_t *vals_out,
                                                             const float4 *lo, const float4 *hi, float4 *bin_lo,
                                                             float4 *bin_hi, uint32_t *bin_child, uint32_t *segctl,
                                                             uint32_t *tlist) {
    __shared__ float s_box[6][kSahChunk];
    __shared__ uint32_t s_id[kSahChunk];
    __shared__ uint16_t s_perm[2][kSahChunk];      // the order, and each range's partition buffer
    __shared__ uint2 s_rng[2][kSahChunk / 2];      // open ranges: (a | b << 16, up) of this level and the next
    __shared__ uint32_t s_bins[kSmallWarps][kTaskBinWords];
    __shared__ uint32_t s_cnt[2], s_tcnt;
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    const unsigned below = (1u << lane) - 1u;
    const uint32_t total = min(ctr[kCtrSmall], n);
    for (uint32_t t = blockIdx.x; t < total; t += gridDim.x) {
        __syncthreads();  // the previous range's shared data is no longer read
        const uint32_t a = small[4ull * t], b = small[4ull * t + 1], p1 = small[4ull * t + 2], ss = small[4ull * t + 3];
        const uint32_t nt = b - a;
        const uint32_t root_up = p1 == 0u ? 0u : (p1 | (ss << 31));
        if (nt == 0u || nt > kSahChunk || b > n) {
            if (threadIdx.x == 0) atomicOr(&ctr[kCtrErr], kSahErrSmall);
            continue;
        }
        if (nt == 1u) {
            if (threadIdx.x == 0) {
                vals_out[a] = vals_in[a];
                link_child(root_up, ss, kLeafBit | a, bin_child, segctl);
            }
            continue;
        }
        for (uint32_t k = threadIdx.x; k < nt; k += kSmallThreads) {
            const uint32_t id = vals_in[a + k];
            const float4 l = lo[id], h = hi[id];
            s_id[k] = id;
            s_box[0][k] = l.x;
            s_box[1][k] = l.y;
            s_box[2][k] = l.z;
            s_box[3][k] = h.x;
            s_box[4][k] = h.y;
            s_box[5][k] = h.z;
            s_perm[0][k] = uint16_t(k);
        }
        uint32_t *tl = tlist + a;
        if (threadIdx.x == 0) {
            s_cnt[0] = s_cnt[1] = s_tcnt = 0u;
            if (nt > kThreadRange) {
                s_rng[0][0] = make_uint2(nt << 16, root_up);
                s_cnt[0] = 1u;
            } else {
                tl[0] = nt << 16;
                tl[1] = root_up;
                s_tcnt = 1u;
            }
        }
        __syncthreads();
        // a child of 2..kThreadRange items to the thread list, a larger one to the next level
        auto push = [&](uint32_t cur_next, uint32_t ra, uint32_t rb, uint32_t up) {
            if (rb - ra <= kThreadRange) {
                const uint32_t q = atomicAdd(&s_tcnt, 1u);
                if (2u * q + 1u < nt) {
                    tl[2u * q] = ra | (rb << 16);
                    tl[2u * q + 1u] = up;
                } else {
                    atomicOr(&ctr[kCtrErr], kSahErrSmall);
                }
            } else {
                const uint32_t q = atomicAdd(&s_cnt[cur_next], 1u);
                if (q < kSahChunk / 2)
                    s_rng[cur_next][q] = make_uint2(ra | (rb << 16), up);
                else
                    atomicOr(&ctr[kCtrErr], kSahErrSmall);
            }
        };
        uint32_t cur = 0u;
        for (uint32_t level = 0; level < kSahChunk; level++) {
            const uint32_t open = s_cnt[cur];
            if (open == 0u) break;
            for (uint32_t r = warp; r < open; r += kSmallWarps) {
                const uint2 R = s_rng[cur][r];
                const uint32_t ra = R.x & 0xffffu, rb = R.x >> 16, up = R.y, cnt = rb - ra;
                // centroid bounds (the node box comes from the bins)
                float v[6];
#pragma unroll
                for (int q = 0; q < 3; q++) {
                    v[q] = FLT_MAX;
                    v[3 + q] = -FLT_MAX;
                }
                for (uint32_t k = ra + lane; k < rb; k += 32u) {
                    const uint32_t p = s_perm[0][k];
                    const float3 c = centroid_of(sbox_lo(&s_box[0][0], p), sbox_hi(&s_box[0][0], p));
                    v[0] = fminf(v[0], c.x);
                    v[1] = fminf(v[1], c.y);
                    v[2] = fminf(v[2], c.z);
                    v[3] = fmaxf(v[3], c.x);
                    v[4] = fmaxf(v[4], c.y);
                    v[5] = fmaxf(v[5], c.z);
                }
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
                    for (int q = 0; q < 6; q++) {
                        const float x = __shfl_xor_sync(~0u, v[q], o);
                        v[q] = q < 3 ? fminf(v[q], x) : fmaxf(v[q], x);
                    }
                }
                const float cl[3] = {v[0], v[1], v[2]};
                const float sc[3] = {sah_scale<kSmallBins>(v[0], v[3]), sah_scale<kSmallBins>(v[1], v[4]),
                                     sah_scale<kSmallBins>(v[2], v[5])};
                uint32_t *wb = s_bins[warp];
                for (uint32_t q = lane; q < 3u * kSmallBins * kBinWords; q += 32u) wb[q] = bin_init(q);
                __syncwarp();
                for (uint32_t k0 = ra; k0 < rb; k0 += 32u) {
                    const uint32_t k = k0 + lane;
                    const bool valid = k < rb;
                    float4 l = make_float4(FLT_MAX, FLT_MAX, FLT_MAX, 0.0f);
                    float4 h = make_float4(-FLT_MAX, -FLT_MAX, -FLT_MAX, 0.0f);
                    if (valid) {
                        const uint32_t p = s_perm[0][k];
                        l = sbox_lo(&s_box[0][0], p);
                        h = sbox_hi(&s_box[0][0], p);
                    }
                    const float3 c = centroid_of(l, h);
                    uint32_t keys[3];
#pragma unroll
                    for (int q = 0; q < 3; q++)
                        keys[q] = uint32_t(q) * kSmallBins + uint32_t(sah_bin<kSmallBins>(axis_of(c, q), cl[q], sc[q]));
                    bin_add3(wb, keys, valid, l, h);
                }
                __syncwarp();
                const SahSplit sp = best_split(wb);
                __syncwarp();
                // the split's left count is the bins' (the partition below bins by the same function);
                // deep levels, and ranges no bin boundary separates, split at the median
                const int axis = level < kSahSmallMedian ? sp.axis : -1;
                const int bin = sp.bin;
                const uint32_t nl = axis >= 0 ? sp.nl : cnt / 2u;
                auto goes_left = [&](uint32_t k) -> bool {
                    if (axis < 0) return k < ra + cnt / 2u;
                    const uint32_t p = s_perm[0][k];
                    const float3 c = centroid_of(sbox_lo(&s_box[0][0], p), sbox_hi(&s_box[0][0], p));
                    return sah_bin<kSmallBins>(axis_of(c, axis), cl[axis], sc[axis]) <= bin;
                };
                const uint32_t m = ra + nl;
                uint32_t L = 0u, Rn = 0u;
                for (uint32_t k0 = ra; k0 < rb; k0 += 32u) {
                    const uint32_t k = k0 + lane;
                    const bool valid = k < rb;
                    const bool f = valid && goes_left(k);
                    const unsigned bl = __ballot_sync(~0u, f), br = __ballot_sync(~0u, valid && !f);
                    if (valid) {
                        const uint32_t dst = f ? ra + L + __popc(bl & below) : m + Rn + __popc(br & below);
                        if (f ? dst < m : dst < rb) s_perm[1][dst] = s_perm[0][k];
                    }
                    L += __popc(bl);
                    Rn += __popc(br);
                }
                if (L != nl && lane == 0) atomicOr(&ctr[kCtrErr], kSahErrSmall);
                __syncwarp();
                for (uint32_t k = ra + lane; k < rb; k += 32u) s_perm[0][k] = s_perm[1][k];
                __syncwarp();
                const float v_box[6] = {sp.box_l.x, sp.box_l.y, sp.box_l.z, sp.box_h.x, sp.box_h.y, sp.box_h.z};
                if (lane == 0) {
                    const uint32_t node = a + m - 1u;
                    bin_lo[node] = make_float4(v_box[0], v_box[1], v_box[2], __uint_as_float(cnt));
                    bin_hi[node] = make_float4(v_box[3], v_box[4], v_box[5], __uint_as_float(a + ra));
                    link_child(up, ss, node, bin_child, segctl);
                    if (m - ra == 1u)
                        link_child(node + 1u, ss, kLeafBit | (a + ra), bin_child, segctl);
                    else
                        push(cur ^ 1u, ra, m, node + 1u);
                    if (rb - m == 1u)
                        link_child((node + 1u) | (1u << 31), ss, kLeafBit | (a + m), bin_child, segctl);
                    else
                        push(cur ^ 1u, m, rb, (node + 1u) | (1u << 31));
                }
            }
            __syncthreads();
            if (threadIdx.x == 0) s_cnt[cur] = 0u;
            cur ^= 1u;
            __syncthreads();
        }
        const uint32_t tc = min(s_tcnt, nt / 2u);
        for (uint32_t j = threadIdx.x; j < tc; j += kSmallThreads) {
            const uint32_t R = tl[2u * j], up = tl[2u * j + 1u];
            thread_subtree(R & 0xffffu, R >> 16, up, a, ss, s_perm[0], &s_box[0][0], bin_lo, bin_hi, bin_child,
                           segctl);
        }
        __syncthreads();
        for (uint32_t k = threadIdx.x; k < nt; k += kSmallThreads) vals_out[a + k] = s_id[s_perm[0][k]];
    }
}

// Multi-segment builds: the segment bits above bit `shift` of every position's key, which the
// passes after the tree read.
__global__ void k_sah_keys(const SegInput *segs, uint32_t nseg, uint32_t n, uint32_t shift,
                           unsigned long long *keys) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    keys[i] = static_cast<unsigned long long>(segment_of(segs, nseg, i)) << shift;
}

int small_grid() {
    static int grid = 0;
    if (grid == 0) {
        int dev = 0, sms = 0, per_sm = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_sah_small, kSmallThreads, 0);
        grid = sms * (per_sm > 0 ? per_sm : 1);
    }
    return grid;
}

// The binary tree; false in *ok when the device flagged an inconsistency (the caller rebuilds
// with the LBVH).
cudaError_t sah_tree(BuildScratch &s, cudaStream_t st, bool *ok) {
    NvtxRange nr("binned-SAH tree");
    *ok = false;
    const uint32_t n = s.n;
    SahLayout L = sah_layout(s);
    cudaError_t e = cudaMemsetAsync(L.ctr, 0, sizeof(uint32_t) * kCtrWords, st);
    if (e != cudaSuccess) return e;
    note_build_launches(2);
    k_sah_seed<<<blocks_for(s.nseg, 128), 128, 0, st>>>(s.segs, s.nseg, L.cap, s.segctl, L.ctr, L.small, L.task[0],
                                                       L.bins[0], L.seg_task);
    k_sah_mark<<<blocks_for(n, 256), 256, 0, st>>>(s.segs, s.nseg, n, L.seg_task, L.pos_task[0], s.vals);
    uint32_t h[kCtrWords];
    e = cudaMemcpyAsync(h, L.ctr, sizeof(h), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return e;
    uint32_t *vin = s.vals, *vout = s.vals_sorted;
    uint32_t par = 0u;
    for (uint32_t level = 0; h[kCtrErr] == 0u && h[kCtrLarge + par] > 0u; level++) {
        if (level >= kSahMaxLevels) return cudaSuccess;  // cannot happen: median splits from kSahMedianLevel
        NvtxRange lr("SAH level: ranges above 1024 items");
        const uint32_t large = std::min(h[kCtrLarge + par], L.cap);
        note_build_launches(4);
        k_sah_bin<<<blocks_for(n, kSahChunk), kBinThreads, 0, st>>>(n, L.pos_task[par], vin, s.box_lo, s.box_hi,
                                                                    L.task[par], L.bins[par]);
        k_sah_split<<<blocks_for(uint64_t(large) * 32u, 128), 128, 0, st>>>(
            par, level >= kSahMedianLevel ? 1u : 0u, L.cap, n, L.ctr, L.task[par], L.bins[par], L.task[par ^ 1u],
            L.bins[par ^ 1u], L.small, s.bin_lo, s.bin_hi, s.bin_child, s.segctl);
        k_sah_flag<<<blocks_for(n, 256), 256, 0, st>>>(n, par, L.ctr, L.pos_task[par], vin, s.box_lo, s.box_hi,
                                                       L.task[par], L.flags);
        size_t bytes = s.sort_tmp_bytes;
        e = cub::DeviceScan::ExclusiveSum(s.sort_tmp, bytes, L.flags, L.scan, int(n), st);
        if (e != cudaSuccess) return e;
        k_sah_scatter<<<blocks_for(n, 256), 256, 0, st>>>(n, L.pos_task[par], L.pos_task[par ^ 1u], vin, vout,
                                                          L.task[par], L.flags, L.scan, L.ctr);
        std::swap(vin, vout);
        par ^= 1u;
        e = cudaMemcpyAsync(h, L.ctr, sizeof(h), cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) return e;
    }
    if (h[kCtrErr] != 0u) return cudaSuccess;
    const uint32_t nsmall = h[kCtrSmall];
    NvtxRange sr("SAH: one block per range of at most 1024 items");
    if (nsmall > 0u) {
        const uint32_t grid = std::min<uint32_t>(nsmall, uint32_t(small_grid()));
        note_build_launches(1);
        k_sah_small<<<grid, kSmallThreads, 0, st>>>(n, L.ctr, L.small, vin, s.vals_sorted, s.box_lo, s.box_hi, s.bin_lo,
                                                    s.bin_hi, s.bin_child, s.segctl,
                                                    reinterpret_cast<uint32_t *>(s.other));
    }
    if (s.nseg > 1) {
        note_build_launches(1);
        k_sah_keys<<<blocks_for(n, 256), 256, 0, st>>>(s.segs, s.nseg, n, 3 * s.axis_bits, s.keys_sorted);
    }
    e = cudaMemcpyAsync(h, L.ctr, sizeof(h), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return e;
    *ok = h[kCtrErr] == 0u;
    return cudaGetLastError();
}

}  // namespace

size_t sah_scan_temp_bytes(uint32_t n) {
    size_t bytes = 0;
    cub::DeviceScan::ExclusiveSum(nullptr, bytes, static_cast<const uint32_t *>(nullptr),
                                  static_cast<uint32_t *>(nullptr), int(n));
    return bytes;
}

cudaError_t build_tree_sah(BuildScratch &s, const BuildParams &bp, cudaStream_t st) {
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    cudaError_t e = cudaStreamIsCapturing(st, &cs);
    if (e != cudaSuccess) return e;
    if (cs != cudaStreamCaptureStatusNone || s.n == 0) return build_tree_lbvh(s, bp, st);
    bool ok = false;
    e = sah_tree(s, st, &ok);
    if (e != cudaSuccess) return e;
    if (!ok) return build_tree_lbvh(s, bp, st);
    return build_tree_rest(s, bp, st);
}

}  // namespace lcx
