// build.cu — BVH construction kernels for sm_103a.
//
// BLAS (MeshBuildCommand, replacing Embree's rtcCommitScene in
// src/rust/luisa_compute_backend_impl/src/cpu/accel.rs:205-260 and OptiX
// accelBuild in src/backends/cuda/cuda_primitive.cpp:20-113) and TLAS
// (AccelBuildCommand, replacing accel.rs:324-447 and the update_accel kernels
// of src/backends/cuda/cuda_builtin/cuda_builtin_kernels.cu:42-111 plus the
// IAS build of cuda_accel.cpp:26-126) share one pipeline over *segments*: a
// segment is one BVH's items (one mesh's triangles, or a TLAS's instances),
// and a batch of thousands of uneven meshes is built in the same launches as
// a single one:
//
//   prep      item boxes + per-segment centroid bounds   (one thread per item)
//   morton    key = segment id above a Morton code of the centroid
//   sort      key/value radix sort of all items of all segments (CUB, sort.cu)
//   lbvh      one bottom-up pass builds every segment's binary radix tree
//             (Apetrei 2014, "Fast and Simple Agglomerative LBVH
//             Construction"); a thread stops at its segment's root, so trees
//             of different segments never merge
//   collapse  one cooperative launch, level-synchronous over all segments:
//             each wide node opens its largest-area children up to the node
//             width, subtrees of <= leaf_max items become leaf slots, children
//             go to octant slots and internal children get contiguous indices
//   emit      both node layouts and the leaf items of every segment into
//             shared pools; a segment's root is wide node s, its indices are
//             stored relative to it, its items relative to its item offset
#include <cooperative_groups.h>
#include <cooperative_groups/scan.h>

#include <atomic>
#include <cfloat>

#include <cub/device/device_scan.cuh>

#include "build_util.cuh"
#include "lcx_internal.h"

namespace cg = cooperative_groups;

namespace lcx {
namespace {

#ifndef LCX_OCTANT_FAST
#define LCX_OCTANT_FAST 1
#endif
#ifndef LCX_COLLAPSE_AGG
#define LCX_COLLAPSE_AGG 1
#endif
#ifndef LCX_QUANT_MUL
#define LCX_QUANT_MUL 1
#endif
#ifndef LCX_INST_SPHERE
#define LCX_INST_SPHERE 1  // TLAS: intersect a static instance's box with its BLAS sphere's box
#endif
#ifndef LCX_COLLAPSE_BLOCKS
// resident blocks per SM of the cooperative collapse: 512-mesh sample 19.1 / 18.1 / 17.1 ms at
// 2 / 4 / 8, the 4096-mesh batch 134 -> 118 ms at 2 -> 8
#define LCX_COLLAPSE_BLOCKS 8
#endif

constexpr int kPrepBlock = 256;

__device__ __forceinline__ unsigned long long spread21(uint32_t v) {
    unsigned long long x = v & 0x1fffffu;
    x = (x | x << 32) & 0x1f00000000ffffull;
    x = (x | x << 16) & 0x1f0000ff0000ffull;
    x = (x | x << 8) & 0x100f00f00f00f00full;
    x = (x | x << 4) & 0x10c30c30c30c30c3ull;
    x = (x | x << 2) & 0x1249249249249249ull;
    return x;
}

__device__ __forceinline__ double box_area_d(float lx, float ly, float lz, float hx, float hy, float hz) {
    if (!(lx <= hx && ly <= hy && lz <= hz)) return 0.0;
    const double dx = double(hx) - lx, dy = double(hy) - ly, dz = double(hz) - lz;
    return 2.0 * (dx * dy + dy * dz + dz * dx);
}

// out[2 seg] += v from every calling lane: one atomic per warp when the whole
// warp is present and in one segment (a segment's items and nodes are
// contiguous, so that is the common case), else one per lane.
__device__ __forceinline__ void seg_sum(double *out, uint32_t seg, double v) {
    const uint32_t mask = __activemask();
    if (mask == 0xffffffffu && __match_any_sync(mask, seg) == mask) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(mask, v, o);
        if ((threadIdx.x & 31u) == 0u) atomicAdd(&out[2 * seg], v);
    } else {
        atomicAdd(&out[2 * seg], v);
    }
}

// Centroid bounds into the per-segment control words; warps whose lanes share
// a segment reduce first (most warps, as segments are contiguous).
__device__ __forceinline__ void add_centroid(uint32_t seg, bool valid, const float c[3], uint32_t *segctl) {
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t seg0 = __shfl_sync(~0u, seg, 0);
    const bool uniform = __all_sync(~0u, seg == seg0);
    if (uniform) {
#pragma unroll
        for (int k = 0; k < 3; k++) {
            float a = valid ? c[k] : FLT_MAX, b = valid ? c[k] : -FLT_MAX;
            for (int o = 16; o; o >>= 1) {
                a = fminf(a, __shfl_xor_sync(~0u, a, o));
                b = fmaxf(b, __shfl_xor_sync(~0u, b, o));
            }
            if (lane == 0 && a <= b) {
                atomicMin(&segctl[kSegWords * seg0 + kSegCenLo + k], float_to_ordered(a));
                atomicMax(&segctl[kSegWords * seg0 + kSegCenHi + k], float_to_ordered(b));
            }
        }
    } else if (valid) {
#pragma unroll
        for (int k = 0; k < 3; k++) {
            atomicMin(&segctl[kSegWords * seg + kSegCenLo + k], float_to_ordered(c[k]));
            atomicMax(&segctl[kSegWords * seg + kSegCenHi + k], float_to_ordered(c[k]));
        }
    }
}

// Curve builds.  The BLAS items are the cones of the segments (a linear segment
// is one cone, a cubic one `pieces` cones, see bvh_device.cuh), so traversal
// culls cones by their own tight boxes.  k_curve_prep converts each segment to
// Bezier form, picks its cone count and open ends; after an exclusive scan of
// the counts, k_curve_fill names the segment of every cone.  The build's
// SegInput then has vbase = the Bezier array (4 float4 per segment and
// keyframe) followed by vcount u32 cone offsets and vcount u32 metas (cones |
// flags << 8), tbase = the u32 segment of each cone, kind bits 16+ = the
// keyframes (0 or 1: static) and, for keyframed curves, vstride = the address
// of the cones' keyframe balls that the emit fills (2 float4 per cone and
// keyframe).
struct CurveCone {
    float4 c0, c1;  // balls: centre xyz, radius w
    uint32_t seg, k, pieces, flags;
};

__device__ __forceinline__ uint32_t curve_keys(const SegInput &g) { return max(g.kind >> 16, 1u); }

__device__ __forceinline__ CurveCone curve_cone(const SegInput &g, uint32_t item, uint32_t key = 0) {
    const float4 *bez = reinterpret_cast<const float4 *>(g.vbase);
    const uint32_t nseg = g.vcount, keys = curve_keys(g);
    const uint32_t *off = reinterpret_cast<const uint32_t *>(bez + 4ull * keys * nseg);
    const uint32_t *meta = off + nseg;
    const uint32_t s = min(reinterpret_cast<const uint32_t *>(g.tbase)[item], nseg - 1u);
    CurveCone c;
    c.seg = s;
    c.pieces = max(meta[s] & 0xffu, 1u);
    c.flags = meta[s] >> 8;
    c.k = min(item - off[s], c.pieces - 1u);
    float4 p[4];
    for (int k = 0; k < 4; k++) p[k] = bez[4ull * (uint64_t(s) * keys + min(key, keys - 1u)) + k];
    c.c0 = curve_piece_point(p, c.k, c.pieces);
    c.c1 = curve_piece_point(p, c.k + 1, c.pieces);
    return c;
}

// cp_count: control points per keyframe; keyframe j's points follow keyframe j-1's.
__global__ void k_curve_prep(const unsigned char *cps, uint64_t stride, uint32_t cp_count, uint32_t keys,
                             const uint32_t *seg, uint32_t nseg, uint32_t basis, float4 *bez, uint32_t *count,
                             uint32_t *meta, uint32_t *err) {
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nseg) return;
    const uint32_t need = basis == kCurveLinear ? 2u : 4u;
    const uint32_t first = seg[s];
    const bool bad = first > cp_count || cp_count - first < need;
    if (bad) atomicOr(err, 1u);
    uint32_t pieces = 0, flags = 0;
    for (uint32_t key = 0; key < keys; key++) {
        float4 p[4] = {make_float4(0, 0, 0, 0), make_float4(0, 0, 0, 0), make_float4(0, 0, 0, 0),
                       make_float4(0, 0, 0, 0)};
        if (!bad) {
            float4 q[4];
            for (uint32_t k = 0; k < 4; k++) {
                const uint64_t at = uint64_t(key) * cp_count + first + min(k, need - 1);
                const float *cp = reinterpret_cast<const float *>(cps + stride * at);
                q[k] = make_float4(cp[0], cp[1], cp[2], cp[3]);
            }
            curve_to_bezier(basis, q, p);
            pieces = max(pieces, curve_pieces(basis, p));
        }
        for (int k = 0; k < 4; k++) bez[4ull * (uint64_t(s) * keys + key) + k] = p[k];
    }
    if (!bad && basis != kCurveLinear) {  // a cubic curve goes on where the next segment starts at this one's end
        const uint32_t step = basis == kCurveBezier ? 3u : 1u;
        if (!(s > 0 && seg[s - 1] + step == first)) flags |= 1u;
        if (!(s + 1 < nseg && seg[s + 1] == first + step)) flags |= 2u;
    }
    count[s] = pieces;
    meta[s] = pieces | (flags << 8);
}

__global__ void k_curve_fill(const uint32_t *off, const uint32_t *count, uint32_t nseg, uint32_t *cone_seg) {
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nseg) return;
    const uint32_t o = off[s];
    for (uint32_t k = 0; k < count[s]; k++) cone_seg[o + k] = s;
}

__global__ void __launch_bounds__(kPrepBlock) k_tri_prep(const SegInput *segs, uint32_t nseg, uint32_t n, float4 *lo,
                                                         float4 *hi, uint32_t *segctl, uint32_t *ctl) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const bool in = i < n;
    const uint32_t s = in ? segment_of(segs, nseg, i) : 0u;
    float c[3] = {0, 0, 0};
    bool valid = false;
    if (in) {
        const SegInput g = segs[s];
        const uint32_t local = i - g.item_offset;
        float4 l = make_float4(FLT_MAX, FLT_MAX, FLT_MAX, 0.0f), h = make_float4(-FLT_MAX, -FLT_MAX, -FLT_MAX, 0.0f);
        uint32_t i0 = 0, i1 = 0, i2 = 0;
        bool bad = false;
        if ((g.kind & 0xffu) == kSegAabbs) {  // the item box is the AABB record (min xyz, max xyz)
            const float *bx = reinterpret_cast<const float *>(g.vbase + 24ull * local);
            l.x = bx[0];
            l.y = bx[1];
            l.z = bx[2];
            h.x = bx[3];
            h.y = bx[4];
            h.z = bx[5];
        } else if ((g.kind & 0xffu) == kSegCurves) {
            // one cone of a curve segment: the box of its two balls, over the keyframes (a ball
            // interpolated between two keyframes stays inside the union of their boxes)
            for (uint32_t key = 0; key < curve_keys(g); key++) {
                const CurveCone cc = curve_cone(g, local, key);
                l.x = fminf(l.x, fminf(cc.c0.x - cc.c0.w, cc.c1.x - cc.c1.w));
                l.y = fminf(l.y, fminf(cc.c0.y - cc.c0.w, cc.c1.y - cc.c1.w));
                l.z = fminf(l.z, fminf(cc.c0.z - cc.c0.w, cc.c1.z - cc.c1.w));
                h.x = fmaxf(h.x, fmaxf(cc.c0.x + cc.c0.w, cc.c1.x + cc.c1.w));
                h.y = fmaxf(h.y, fmaxf(cc.c0.y + cc.c0.w, cc.c1.y + cc.c1.w));
                h.z = fmaxf(h.z, fmaxf(cc.c0.z + cc.c0.w, cc.c1.z + cc.c1.w));
            }
        } else {
            const uint32_t *t = reinterpret_cast<const uint32_t *>(g.tbase + 12ull * local);
            i0 = t[0];
            i1 = t[1];
            i2 = t[2];
            bad = i0 >= g.vcount || i1 >= g.vcount || i2 >= g.vcount;
        }
        if (bad) {
            atomicOr(&segctl[kSegWords * s + kSegErr], kErrBadIndex);
            atomicOr(&ctl[kCtlErr], kErrBadIndex);
        } else if ((g.kind & 0xffu) == kSegTriangles) {
            // vertex motion (kind >> 8 keyframes): the union over the keyframes bounds the
            // linearly interpolated triangle at every time
            const uint32_t keys = max(g.kind >> 8, 1u);
            for (uint32_t key = 0; key < keys; key++) {
                const uint64_t kb = uint64_t(key) * g.vcount;
                const float4 a = __ldg(reinterpret_cast<const float4 *>(g.vbase + g.vstride * (kb + i0)));
                const float4 b = __ldg(reinterpret_cast<const float4 *>(g.vbase + g.vstride * (kb + i1)));
                const float4 cc = __ldg(reinterpret_cast<const float4 *>(g.vbase + g.vstride * (kb + i2)));
                l.x = fminf(fminf(l.x, a.x), fminf(b.x, cc.x));
                l.y = fminf(fminf(l.y, a.y), fminf(b.y, cc.y));
                l.z = fminf(fminf(l.z, a.z), fminf(b.z, cc.z));
                h.x = fmaxf(fmaxf(h.x, a.x), fmaxf(b.x, cc.x));
                h.y = fmaxf(fmaxf(h.y, a.y), fmaxf(b.y, cc.y));
                h.z = fmaxf(fmaxf(h.z, a.z), fmaxf(b.z, cc.z));
            }
        }
        if (box_empty(l, h)) {
            l = make_float4(FLT_MAX, FLT_MAX, FLT_MAX, 0.0f);
            h = make_float4(-FLT_MAX, -FLT_MAX, -FLT_MAX, 0.0f);
        } else {
            valid = true;
            c[0] = 0.5f * (l.x + h.x);
            c[1] = 0.5f * (l.y + h.y);
            c[2] = 0.5f * (l.z + h.z);
        }
        lo[i] = l;
        hi[i] = h;
    }
    add_centroid(s, valid, c, segctl);
}

// ---------------------------------------------------------------------------
// Triangle splitting (FAST_TRACE builds; the counterpart of the spatial splits
// of Embree's RTC_BUILD_QUALITY_HIGH that the reference's CPU backend asks for,
// cpu/accel.rs:58-61).  A triangle whose box is much larger than the triangle
// (a long diagonal sliver) overlaps many others and is tested by many rays
// that do not hit it.  Before the Morton sort such triangles get several
// references, each with a box around one piece of the triangle, so the tree
// is built over tighter boxes (Karras & Aila, "Fast Parallel Construction of
// High-Quality Bounding Volume Hierarchies", 2013, triangle splitting).
// Every reference of a triangle stores the whole triangle, so a ray tests the
// same triangle with the same arithmetic through any of them: hit records do
// not change, a triangle is only found in more leaves.
//
// Budget: the extra references of a mesh (segment) are at most
// floor(fraction * its triangles), shared out within the mesh in proportion
// to each triangle's weight max(0, A_box - 2 A_tri), quantised to 20 bits of
// the mesh's largest weight so that the counts are deterministic
// (A_box = dx dy + dy dz + dz dx of its box: an axis-aligned right triangle
// scores 0), at most kMaxRefs per triangle.
// Pieces: the triangle's box is split recursively at the midpoint of its
// longest axis; each half is tightened to the box of the triangle clipped to
// it (Sutherland-Hodgman against the half's six planes), padded outward by
// 2^-19 of the coordinate magnitude and cut back to the half.  The halves
// share the split plane exactly and each padded box contains its part of the
// triangle, so the references' boxes cover the whole triangle.
constexpr uint32_t kMaxRefs = 16;

__device__ __forceinline__ float tri_area2(const float4 &a, const float4 &b, const float4 &c) {
    const float ux = b.x - a.x, uy = b.y - a.y, uz = b.z - a.z;
    const float vx = c.x - a.x, vy = c.y - a.y, vz = c.z - a.z;
    const float cx = uy * vz - uz * vy, cy = uz * vx - ux * vz, cz = ux * vy - uy * vx;
    return sqrtf(cx * cx + cy * cy + cz * cz);  // twice the area
}

// Per-segment atomics of the split kernels, one per warp when the warp's items
// share a segment (a single-mesh build would otherwise send every thread's
// atomic to the same word).
__device__ __forceinline__ void seg_add_u64(unsigned long long *a, uint32_t seg, bool in, unsigned long long v) {
    const uint32_t seg0 = __shfl_sync(~0u, seg, 0);
    if (__all_sync(~0u, !in || seg == seg0)) {
        unsigned long long t = in ? v : 0ull;
        for (int o = 16; o; o >>= 1) t += __shfl_xor_sync(~0u, t, o);
        if ((threadIdx.x & 31u) == 0u && t) atomicAdd(&a[seg0], t);
    } else if (in && v) {
        atomicAdd(&a[seg], v);
    }
}
__device__ __forceinline__ void seg_add_u32(uint32_t *a, uint32_t seg, bool in, uint32_t v) {
    const uint32_t seg0 = __shfl_sync(~0u, seg, 0);
    if (__all_sync(~0u, !in || seg == seg0)) {
        uint32_t t = in ? v : 0u;
        for (int o = 16; o; o >>= 1) t += __shfl_xor_sync(~0u, t, o);
        if ((threadIdx.x & 31u) == 0u && t) atomicAdd(&a[seg0], t);
    } else if (in && v) {
        atomicAdd(&a[seg], v);
    }
}
__device__ __forceinline__ void seg_max_u32(uint32_t *a, uint32_t seg, bool in, uint32_t v) {
    const uint32_t seg0 = __shfl_sync(~0u, seg, 0);
    if (__all_sync(~0u, !in || seg == seg0)) {
        uint32_t t = in ? v : 0u;
        for (int o = 16; o; o >>= 1) t = max(t, __shfl_xor_sync(~0u, t, o));
        if ((threadIdx.x & 31u) == 0u && t) atomicMax(&a[seg0], t);
    } else if (in && v) {
        atomicMax(&a[seg], v);
    }
}

__global__ void __launch_bounds__(kPrepBlock) k_split_weight(const SegInput *segs, uint32_t nseg, uint32_t n,
                                                             float *wts, uint32_t *wmax, uint32_t *segctl,
                                                             uint32_t *ctl) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const bool in = i < n;
    const uint32_t s = in ? segment_of(segs, nseg, i) : 0u;
    float w = 0.0f;
    if (in) {
    const SegInput g = segs[s];
    const uint32_t local = i - g.item_offset;
    const uint32_t *t = reinterpret_cast<const uint32_t *>(g.tbase + 12ull * local);
    const uint32_t i0 = t[0], i1 = t[1], i2 = t[2];
    if (i0 >= g.vcount || i1 >= g.vcount || i2 >= g.vcount) {
        atomicOr(&segctl[kSegWords * s + kSegErr], kErrBadIndex);
        atomicOr(&ctl[kCtlErr], kErrBadIndex);
    } else {
        const float4 a = __ldg(reinterpret_cast<const float4 *>(g.vbase + g.vstride * i0));
        const float4 b = __ldg(reinterpret_cast<const float4 *>(g.vbase + g.vstride * i1));
        const float4 c = __ldg(reinterpret_cast<const float4 *>(g.vbase + g.vstride * i2));
        const float dx = fmaxf(fmaxf(a.x, b.x), c.x) - fminf(fminf(a.x, b.x), c.x);
        const float dy = fmaxf(fmaxf(a.y, b.y), c.y) - fminf(fminf(a.y, b.y), c.y);
        const float dz = fmaxf(fmaxf(a.z, b.z), c.z) - fminf(fminf(a.z, b.z), c.z);
        const float abox = dx * dy + dy * dz + dz * dx;
        const float v = abox - tri_area2(a, b, c);  // A_box - 2 A_tri
        w = v > 0.0f && isfinite(v) ? v : 0.0f;
    }
    wts[i] = w;
    }
    seg_max_u32(wmax, s, in, __float_as_uint(w));  // non-negative floats order as their bits
}

// Weights as integers relative to the segment's largest (so the sums, and the
// reference counts, do not depend on the order of the atomics): q in [0, 2^20].
__global__ void __launch_bounds__(kPrepBlock) k_split_quant(const SegInput *segs, uint32_t nseg, uint32_t n,
                                                            float *wts, const uint32_t *wmax,
                                                            unsigned long long *qsum) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const bool in = i < n;
    const uint32_t s = in ? segment_of(segs, nseg, i) : 0u;
    uint32_t q = 0;
    if (in) {
        const float m = __uint_as_float(wmax[s]);
        const float w = wts[i];
        q = m > 0.0f ? uint32_t(fminf(w / m, 1.0f) * 1048576.0f) : 0u;
        reinterpret_cast<uint32_t *>(wts)[i] = q;
    }
    seg_add_u64(qsum, s, in, q);
}

// refs[i] = 1 + this triangle's extra references; seg_refs[s] += refs of segment s.
__global__ void __launch_bounds__(kPrepBlock) k_split_assign(const SegInput *segs, uint32_t nseg, uint32_t n,
                                                             const uint32_t *q, const unsigned long long *qsum,
                                                             float fraction, uint32_t *refs, uint32_t *seg_refs) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const bool in = i < n;
    const uint32_t s = in ? segment_of(segs, nseg, i) : 0u;
    uint32_t extra = 0;
    if (in) {
        const unsigned long long total = qsum[s];
        const unsigned long long budget =
            static_cast<unsigned long long>(floorf(fraction * float(segs[s].item_count)));
        if (total > 0ull) {
            const unsigned long long e = budget * q[i] / total;  // < 2^33 * 2^21
            extra = e >= kMaxRefs - 1 ? kMaxRefs - 1 : uint32_t(e);
        }
        refs[i] = 1u + extra;
    }
    seg_add_u32(seg_refs, s, in, in ? 1u + extra : 0u);
}

// Clip the convex polygon P (n vertices) to the half-space x[axis] >= v (keep_ge) or <= v.
__device__ __forceinline__ int clip_plane(float (*P)[3], int n, float (*Q)[3], int axis, float v, bool keep_ge) {
    int m = 0;
    for (int k = 0; k < n; k++) {
        const float *A = P[k], *B = P[(k + 1) % n];
        const float da = keep_ge ? A[axis] - v : v - A[axis];
        const float db = keep_ge ? B[axis] - v : v - B[axis];
        if (da >= 0.0f) {
            Q[m][0] = A[0];
            Q[m][1] = A[1];
            Q[m][2] = A[2];
            m++;
        }
        if ((da >= 0.0f) != (db >= 0.0f)) {
            const float t = da / (da - db);
            for (int j = 0; j < 3; j++) Q[m][j] = A[j] + t * (B[j] - A[j]);
            Q[m][axis] = v;
            m++;
        }
    }
    return m;
}

// The box of (triangle within [lo, hi]), padded outward and cut back to [lo, hi].
// Returns false if the clipped triangle is empty.
__device__ bool tight_box(const float4 &a, const float4 &b, const float4 &c, const float lo[3], const float hi[3],
                          float tl[3], float th[3]) {
    float P[10][3], Q[10][3];
    P[0][0] = a.x;
    P[0][1] = a.y;
    P[0][2] = a.z;
    P[1][0] = b.x;
    P[1][1] = b.y;
    P[1][2] = b.z;
    P[2][0] = c.x;
    P[2][1] = c.y;
    P[2][2] = c.z;
    int n = 3;
    for (int axis = 0; axis < 3 && n > 0; axis++) {
        n = clip_plane(P, n, Q, axis, lo[axis], true);
        if (n == 0) break;
        n = clip_plane(Q, n, P, axis, hi[axis], false);
    }
    if (n == 0) return false;
    float mag = 0.0f;
    for (int j = 0; j < 3; j++) {
        tl[j] = FLT_MAX;
        th[j] = -FLT_MAX;
        mag = fmaxf(mag, fmaxf(fabsf(lo[j]), fabsf(hi[j])));
    }
    for (int k = 0; k < n; k++)
        for (int j = 0; j < 3; j++) {
            tl[j] = fminf(tl[j], P[k][j]);
            th[j] = fmaxf(th[j], P[k][j]);
        }
    const float pad = mag * 0x1p-19f + 1e-30f;
    for (int j = 0; j < 3; j++) {
        tl[j] = fmaxf(tl[j] - pad, lo[j]);
        th[j] = fminf(th[j] + pad, hi[j]);
    }
    return tl[0] <= th[0] && tl[1] <= th[1] && tl[2] <= th[2];
}

__device__ __forceinline__ void add_centroid_range(uint32_t seg, bool valid, const float cl[3], const float ch[3],
                                                   uint32_t *segctl) {
    if (!valid) return;
#pragma unroll
    for (int k = 0; k < 3; k++) {
        atomicMin(&segctl[kSegWords * seg + kSegCenLo + k], float_to_ordered(cl[k]));
        atomicMax(&segctl[kSegWords * seg + kSegCenHi + k], float_to_ordered(ch[k]));
    }
}

// Writes the references of triangle i: boxes at ref_off[i] .. + refs[i] - 1 (in the
// reference-space item arrays) and their triangle's local index; centroid bounds of
// the reference segments.  tsegs: the triangle-space segment table.
__global__ void __launch_bounds__(kPrepBlock) k_split_emit(const SegInput *tsegs, uint32_t nseg, uint32_t n,
                                                           const uint32_t *refs, const uint32_t *ref_off, float4 *lo,
                                                           float4 *hi, uint32_t *ref_prim, uint32_t *segctl) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t s = segment_of(tsegs, nseg, i);
    const SegInput g = tsegs[s];
    const uint32_t local = i - g.item_offset;
    const uint32_t r = refs[i], base = ref_off[i];
    for (uint32_t k = 0; k < r; k++) ref_prim[base + k] = local;
    const uint32_t *t = reinterpret_cast<const uint32_t *>(g.tbase + 12ull * local);
    const uint32_t i0 = t[0], i1 = t[1], i2 = t[2];
    const float4 E0 = make_float4(FLT_MAX, FLT_MAX, FLT_MAX, 0.0f), E1 = make_float4(-FLT_MAX, -FLT_MAX, -FLT_MAX, 0.0f);
    if (i0 >= g.vcount || i1 >= g.vcount || i2 >= g.vcount) {  // reported by k_split_weight
        for (uint32_t k = 0; k < r; k++) {
            lo[base + k] = E0;
            hi[base + k] = E1;
        }
        return;
    }
    const float4 a = __ldg(reinterpret_cast<const float4 *>(g.vbase + g.vstride * i0));
    const float4 b = __ldg(reinterpret_cast<const float4 *>(g.vbase + g.vstride * i1));
    const float4 c = __ldg(reinterpret_cast<const float4 *>(g.vbase + g.vstride * i2));
    float cl[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, ch[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
    bool any = false;
    // pieces as (box, references) on a small stack; a piece with one reference is written
    float sl[6][3], sh[6][3];
    uint32_t sc[6];
    int sp = 0;
    sl[0][0] = fminf(fminf(a.x, b.x), c.x);
    sl[0][1] = fminf(fminf(a.y, b.y), c.y);
    sl[0][2] = fminf(fminf(a.z, b.z), c.z);
    sh[0][0] = fmaxf(fmaxf(a.x, b.x), c.x);
    sh[0][1] = fmaxf(fmaxf(a.y, b.y), c.y);
    sh[0][2] = fmaxf(fmaxf(a.z, b.z), c.z);
    sc[0] = r;
    sp = 1;
    uint32_t out = 0;
    while (sp > 0) {
        sp--;
        float bl[3] = {sl[sp][0], sl[sp][1], sl[sp][2]}, bh[3] = {sh[sp][0], sh[sp][1], sh[sp][2]};
        const uint32_t cnt = sc[sp];
        const bool valid = bl[0] <= bh[0] && bl[1] <= bh[1] && bl[2] <= bh[2] && isfinite(bl[0] + bl[1] + bl[2]) &&
                           isfinite(bh[0] + bh[1] + bh[2]);
        int axis = 0;
        float ext = bh[0] - bl[0];
        for (int j = 1; j < 3; j++)
            if (bh[j] - bl[j] > ext) {
                ext = bh[j] - bl[j];
                axis = j;
            }
        const float mid = 0.5f * (bl[axis] + bh[axis]);
        if (cnt == 1u || !valid || !(mid > bl[axis] && mid < bh[axis]) || sp + 2 > 6) {
            // one reference gets the box; any others of this piece stay empty
            for (uint32_t k = 0; k < cnt; k++) {
                const bool first = k == 0 && valid;
                lo[base + out] = first ? make_float4(bl[0], bl[1], bl[2], 0.0f) : E0;
                hi[base + out] = first ? make_float4(bh[0], bh[1], bh[2], 0.0f) : E1;
                if (first) {
                    any = true;
                    for (int j = 0; j < 3; j++) {
                        const float cj = 0.5f * (bl[j] + bh[j]);
                        cl[j] = fminf(cl[j], cj);
                        ch[j] = fmaxf(ch[j], cj);
                    }
                }
                out++;
            }
            continue;
        }
        float ll[3] = {bl[0], bl[1], bl[2]}, lh[3] = {bh[0], bh[1], bh[2]};
        float rl[3] = {bl[0], bl[1], bl[2]}, rh[3] = {bh[0], bh[1], bh[2]};
        lh[axis] = mid;
        rl[axis] = mid;
        float tl1[3], th1[3], tl2[3], th2[3];
        const bool okl = tight_box(a, b, c, ll, lh, tl1, th1);
        const bool okr = tight_box(a, b, c, rl, rh, tl2, th2);
        if (!okl || !okr) {  // all of the piece on one side: keep splitting that side
            const float *nl = okl ? tl1 : tl2, *nh = okl ? th1 : th2;
            if (!okl && !okr) {
                nl = bl;
                nh = bh;
            }
            for (int j = 0; j < 3; j++) {
                sl[sp][j] = nl[j];
                sh[sp][j] = nh[j];
            }
            sc[sp] = (okl || okr) ? cnt : 1u;
            sp++;
            if (!okl && !okr)  // cannot happen for a finite triangle; write the rest empty
                for (uint32_t k = 1; k < cnt; k++) {
                    lo[base + out] = E0;
                    hi[base + out] = E1;
                    out++;
                }
            continue;
        }
        const uint32_t cl_n = cnt / 2u, cr_n = cnt - cl_n;
        for (int j = 0; j < 3; j++) {
            sl[sp][j] = tl1[j];
            sh[sp][j] = th1[j];
        }
        sc[sp++] = cl_n;
        for (int j = 0; j < 3; j++) {
            sl[sp][j] = tl2[j];
            sh[sp][j] = th2[j];
        }
        sc[sp++] = cr_n;
    }
    add_centroid_range(s, any, cl, ch, segctl);
}

__global__ void __launch_bounds__(kPrepBlock) k_inst_prep(const InstState *inst, uint32_t n, float4 *lo, float4 *hi,
                                                          float *w2o, uint32_t *segctl) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    float c[3] = {0, 0, 0};
    bool valid = false;
    if (i < n) {
        const InstState &s = inst[i];
        float m[12], w[12];
        const MotionDesc *md = s.motion;
        const bool srt = md != nullptr && (md->flags & 4u);
        if (md != nullptr) {  // a motion instance: keyframe 0 stands in (its w2o is not used)
            if (srt)
                srt_matrix(md->keys, m);
            else
                for (int k = 0; k < 12; k++) m[k] = md->keys[k];
        } else {
#pragma unroll
            for (int k = 0; k < 12; k++) m[k] = s.o2w[k];
        }
        affine_inverse(m, w);
#pragma unroll
        for (int k = 0; k < 12; k++) w2o[12ull * i + k] = w[k];
        float4 l = make_float4(FLT_MAX, FLT_MAX, FLT_MAX, 0.0f), h = make_float4(-FLT_MAX, -FLT_MAX, -FLT_MAX, 0.0f);
        const BlasDesc *d = s.blas;
        if (d != nullptr && (d->valid & 1u)) {
            const float blo[3] = {d->lo[0], d->lo[1], d->lo[2]}, bhi[3] = {d->hi[0], d->hi[1], d->hi[2]};
            float wl[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, wh[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
            // a static instance: its matrix; a motion instance: the union over its keyframes,
            // which bounds the linear interpolation of the matrices (a point moves along the
            // segment between its keyframe positions), padded for the FP32 interpolation
            const uint32_t nkey = srt ? 0u : (md != nullptr ? md->count : 1u);
            const float rel = md != nullptr ? 0x1p-17f : 0x1p-20f;
            // SRT keyframes, per segment: S (scale, shear, pivot; linear in the keyframe
            // values) maps the BLAS box into the union of its two keyframe boxes; any
            // rotation keeps that within the ball of its largest corner distance; the
            // translation moves along the segment between its keyframe values
            for (uint32_t seg = 0; srt && seg + 1 < md->count; seg++) {
                float sl[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, sh[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
                float tl[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, th[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
                for (uint32_t e = 0; e < 2; e++) {
                    const float *v = md->keys + 16ull * (seg + e);
                    // rows of S: (sx, a, b | px), (0, sy, c | py), (0, 0, sz | pz)
                    const float S[12] = {v[7], v[10], v[11], v[0], 0.0f, v[8], v[12], v[1], 0.0f, 0.0f, v[9], v[2]};
                    for (int k = 0; k < 3; k++) {
                        float a = S[4 * k + 3], b = S[4 * k + 3];
                        for (int j = 0; j < 3; j++) {
                            const float e0 = S[4 * k + j] * blo[j], e1 = S[4 * k + j] * bhi[j];
                            a += fminf(e0, e1);
                            b += fmaxf(e0, e1);
                        }
                        sl[k] = fminf(sl[k], a);
                        sh[k] = fmaxf(sh[k], b);
                        tl[k] = fminf(tl[k], v[13 + k]);
                        th[k] = fmaxf(th[k], v[13 + k]);
                    }
                }
                float r2 = 0.0f;
                for (int k = 0; k < 3; k++) {
                    const float c = fmaxf(fabsf(sl[k]), fabsf(sh[k]));
                    r2 += c * c;
                }
                const float r = sqrtf(r2) * (1.0f + 0x1p-16f);
                for (int k = 0; k < 3; k++) {
                    const float pad = (r + fmaxf(fabsf(tl[k]), fabsf(th[k]))) * 0x1p-17f;
                    wl[k] = fminf(wl[k], tl[k] - r - pad);
                    wh[k] = fmaxf(wh[k], th[k] + r + pad);
                }
            }
            // interval arithmetic of the affine map over box [bl, bh], then an outward pad that
            // covers the FP32 rounding of the sums; the world box grows to hold it
            auto add_box = [&](const float bl[3], const float bh[3]) {
#pragma unroll
                for (int k = 0; k < 3; k++) {
                    float a = m[4 * k + 3], b = m[4 * k + 3], mag = fabsf(m[4 * k + 3]);
#pragma unroll
                    for (int j = 0; j < 3; j++) {
                        const float e0 = m[4 * k + j] * bl[j], e1 = m[4 * k + j] * bh[j];
                        a += fminf(e0, e1);
                        b += fmaxf(e0, e1);
                        mag += fmaxf(fabsf(e0), fabsf(e1));
                    }
                    const float pad = mag * rel;
                    wl[k] = fminf(wl[k], a - pad);
                    wh[k] = fmaxf(wh[k], b + pad);
                }
            };
            for (uint32_t key = 0; key < nkey; key++) {
                if (md != nullptr)
                    for (int k = 0; k < 12; k++) m[k] = md->keys[12ull * key + k];
                add_box(blo, bhi);
            }
            // A static instance's box also lies within the box of its BLAS's bounding sphere, mapped:
            // a ball of radius r goes to an ellipsoid whose half-extent on axis k is r times the norm
            // of row k.  The world box is the intersection of the two (a rotated round object's box
            // shrinks by up to sqrt(3) per axis, so fewer rays enter an instance they miss).
            if (LCX_INST_SPHERE && md == nullptr && d->bs_r > 0.0f && isfinite(d->bs_r)) {
                const float c[3] = {0.5f * (blo[0] + bhi[0]), 0.5f * (blo[1] + bhi[1]), 0.5f * (blo[2] + bhi[2])};
#pragma unroll
                for (int k = 0; k < 3; k++) {
                    const float x = __fmaf_rn(m[4 * k], c[0], __fmaf_rn(m[4 * k + 1], c[1], __fmaf_rn(m[4 * k + 2], c[2],
                                                                                             m[4 * k + 3])));
                    const float nr = __fsqrt_ru(__fmaf_ru(m[4 * k], m[4 * k], __fmaf_ru(m[4 * k + 1], m[4 * k + 1],
                                                                                  __fmul_ru(m[4 * k + 2], m[4 * k + 2]))));
                    const float ext = __fmul_ru(d->bs_r, nr);
                    const float mag = fabsf(m[4 * k] * c[0]) + fabsf(m[4 * k + 1] * c[1]) + fabsf(m[4 * k + 2] * c[2]) +
                                      fabsf(m[4 * k + 3]) + ext;
                    const float pad = mag * 0x1p-18f;
                    wl[k] = fmaxf(wl[k], x - ext - pad);
                    wh[k] = fminf(wh[k], x + ext + pad);
                }
            }
            l = make_float4(wl[0], wl[1], wl[2], 0.0f);
            h = make_float4(wh[0], wh[1], wh[2], 0.0f);
            if (box_empty(l, h)) {
                l = make_float4(FLT_MAX, FLT_MAX, FLT_MAX, 0.0f);
                h = make_float4(-FLT_MAX, -FLT_MAX, -FLT_MAX, 0.0f);
            } else {
                valid = true;
                c[0] = 0.5f * (l.x + h.x);
                c[1] = 0.5f * (l.y + h.y);
                c[2] = 0.5f * (l.z + h.z);
            }
        }
        lo[i] = l;
        hi[i] = h;
    }
    add_centroid(0, valid, c, segctl);
}

// Morton key of an item.  With cube = 1 the centroid is normalised by the
// segment's largest centroid extent on every axis (so a flat segment does not
// get as many splits across its thin axis as along its wide ones); with
// cube = 0 each axis by its own extent.  With size_bits > 0 (extended Morton
// codes, Vinkler, Bittner & Havran 2017) the top bits below the segment id
// hold a size class, log2(segment extent / item diagonal), so large items meet
// near the root instead of deep among small neighbours.
__global__ void k_morton(const SegInput *segs, uint32_t nseg, uint32_t n, uint32_t axis_bits, uint32_t size_bits,
                         uint32_t cube, const float4 *lo, const float4 *hi, const uint32_t *segctl,
                         unsigned long long *keys, uint32_t *vals) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t s = nseg > 1 ? segment_of(segs, nseg, i) : 0u;
    const float4 l = lo[i], h = hi[i];
    const uint32_t qmax = (1u << axis_bits) - 1u;
    const uint32_t code_bits = 3 * axis_bits;
    unsigned long long code = (1ull << code_bits) - 1ull;  // empty boxes sort last in their segment
    if (!box_empty(l, h)) {
        const float c[3] = {0.5f * (l.x + h.x), 0.5f * (l.y + h.y), 0.5f * (l.z + h.z)};
        float blo[3], ax[3], ext = 0.0f;
#pragma unroll
        for (int k = 0; k < 3; k++) {
            blo[k] = ordered_to_float(segctl[kSegWords * s + kSegCenLo + k]);
            ax[k] = ordered_to_float(segctl[kSegWords * s + kSegCenHi + k]) - blo[k];
            ext = fmaxf(ext, ax[k]);
        }
        uint32_t q[3];
#pragma unroll
        for (int k = 0; k < 3; k++) {
            const float e = cube ? ext : ax[k];
            float f = e > 0.0f ? (c[k] - blo[k]) / e : 0.0f;
            f = fminf(fmaxf(f, 0.0f), 1.0f);
            q[k] = min(uint32_t(f * float(qmax)), qmax);
        }
        code = spread21(q[0]) << 2 | spread21(q[1]) << 1 | spread21(q[2]);
        if (size_bits) {
            const float dx = h.x - l.x, dy = h.y - l.y, dz = h.z - l.z;
            const float diag = sqrtf(dx * dx + dy * dy + dz * dz);
            const uint32_t cmax = (1u << size_bits) - 1u;
            float cls = ext > 0.0f && diag > 0.0f ? floorf(log2f(ext / diag)) + 1.0f : float(cmax);
            cls = fminf(fmaxf(cls, 0.0f), float(cmax));
            code = (static_cast<unsigned long long>(cls) << (code_bits - size_bits)) | (code >> size_bits);
        }
    }
    keys[i] = (static_cast<unsigned long long>(s) << code_bits) | code;
    vals[i] = i;
}

// delta(a) < delta(b) with delta(i) = (key_i ^ key_i+1, i ^ i+1) in lexicographic order.
__device__ __forceinline__ bool delta_less(const unsigned long long *k, uint32_t a, uint32_t b) {
    const unsigned long long da = k[a] ^ k[a + 1], db = k[b] ^ k[b + 1];
    if (da != db) return da < db;
    return (a ^ (a + 1)) < (b ^ (b + 1));
}

// ---- collapse by dynamic program (Ylitie, Karras & Laine 2017, "Efficient Incoherent Ray
// Traversal on GPUs Through Compressed Wide BVHs"): bottom-up over the binary tree, the cost of
// each subtree given i = 1..width slots of its wide parent -- a leaf slot (at most leaf_max items,
// cost dp_prim x area x items), a wide node of its own (cost area + the best split of `width` slots
// between its children), or for i > 1 the best split of i slots between its children -- and the
// decisions that reach it, which the collapse then follows instead of opening the largest child.
// Costs are in units of the root-independent box area; a node test costs 1.  The LBVH's own
// bottom-up walk runs it for 8-wide nodes (k_lbvh<8>); other trees and widths take a pass of
// their own (k_dp_parents, k_dp_up).

// The costs out[0..W) of a node of box area a over cnt items for 1..W slots, from its children's
// (cl, cr), and its decision word: bits 0..2 the split of W slots when the node is a wide node;
// bits 3(i-1)..3(i-1)+2 for i = 2..W: 0 = take i - 1 slots, else k = the left child's share of
// i slots.  W is a template argument so that every cost stays in registers; out may alias cl or cr.
template <int W>
__device__ __forceinline__ uint32_t dp_up_node(const float *cl, const float *cr, float a, uint32_t cnt, int leaf_max,
                                               float cp, float *out) {
    float dist[W + 1];
    uint32_t dk[W + 1];
#pragma unroll
    for (int j = 2; j <= W; j++) {
        dist[j] = FLT_MAX;
        dk[j] = 0u;
#pragma unroll
        for (int k = 1; k < j; k++) {
            const float v = cl[k - 1] + cr[j - k - 1];
            if (v < dist[j]) {
                dist[j] = v;
                dk[j] = uint32_t(k);
            }
        }
    }
    uint32_t word = 0u;
    float prev;
    if (cnt <= uint32_t(leaf_max)) {
        prev = cp * a * float(cnt);
    } else {
        prev = a + dist[W];
        word = dk[W];
    }
    out[0] = prev;
#pragma unroll
    for (int i = 2; i <= W; i++) {
        if (dist[i] < prev) {
            prev = dist[i];
            word |= dk[i] << (3 * (i - 1));
        }
        out[i - 1] = prev;
    }
    return word;
}

// A node's 8 cost words (slots beyond W repeat the W-slot cost).
template <int W>
__device__ __forceinline__ void dp_store_costs(float *dst, const float *c) {
    float o[8];
#pragma unroll
    for (int i = 0; i < 8; i++) o[i] = c[i < W ? i : W - 1];
    float4 *d4 = reinterpret_cast<float4 *>(dst);
    d4[0] = make_float4(o[0], o[1], o[2], o[3]);
    d4[1] = make_float4(o[4], o[5], o[6], o[7]);
}

// Binary node j (0 <= j < n-1) covers sorted items [first, first + count);
// bin_lo.w / bin_hi.w hold count / first as bits.  A segment's keys differ
// from its neighbours' in the segment bits, so its boundary deltas are larger
// than every inner one and the merges stay inside it; the thread that
// completes the node spanning the whole segment records it as the root.
// W > 0: the same walk also runs the collapse's dynamic program for W-wide nodes (dp_up_node): the
// completing thread holds its own subtree's costs in registers, reads the sibling's, writes the
// node's costs and, over the node's arrival word (which nothing reads after the second arrival),
// its decision word.
template <int W>
__global__ void k_lbvh(const SegInput *segs, uint32_t n, uint32_t seg_shift, const unsigned long long *keys,
                       const uint32_t *vals, const float4 *lo, const float4 *hi, uint32_t *bin_child, float4 *bin_lo,
                       float4 *bin_hi, int32_t *other, uint32_t *segctl, int leaf_max, float cp, float *cost) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t s = seg_shift < 64 ? uint32_t(keys[i] >> seg_shift) : 0u;
    const uint32_t seg_first = segs[s].item_offset;
    const uint32_t seg_last = seg_first + segs[s].item_count - 1;
    uint32_t cur = kLeafBit | i;
    uint32_t l = i, r = i;
    if (l == seg_first && r == seg_last) {
        segctl[kSegWords * s + kSegRoot] = cur;
        return;
    }
    const uint32_t item = vals[i];
    float4 clo = lo[item], chi = hi[item];
    float ccost[W > 0 ? W : 1];
    if constexpr (W > 0) {
        const float v = cp * box_area(clo, chi);
#pragma unroll
        for (int k = 0; k < W; k++) ccost[k] = v;
    }
    for (uint32_t guard = 0; guard < n; guard++) {
        const bool left = (l == 0) || (r != n - 1 && delta_less(keys, r, l - 1));
        const uint32_t parent = left ? r : l - 1;
        bin_child[2 * parent + (left ? 0 : 1)] = cur;
        // acquire-release: publishes this subtree's node (and costs), sees the sibling's
        int32_t prev;
        asm volatile("atom.acq_rel.gpu.global.exch.b32 %0, [%1], %2;"
                     : "=r"(prev)
                     : "l"(other + parent), "r"(left ? int32_t(l) : int32_t(r))
                     : "memory");
        if (prev < 0) return;  // the sibling finishes the parent
        if (left)
            r = uint32_t(prev);
        else
            l = uint32_t(prev);
        const uint32_t sib = __ldcg(&bin_child[2 * parent + (left ? 1 : 0)]);
        float4 slo, shi;
        if (sib & kLeafBit) {
            const uint32_t it = vals[sib & ~kLeafBit];
            slo = lo[it];
            shi = hi[it];
        } else {
            slo = __ldcg(&bin_lo[sib]);
            shi = __ldcg(&bin_hi[sib]);
        }
        clo = make_float4(fminf(clo.x, slo.x), fminf(clo.y, slo.y), fminf(clo.z, slo.z), 0.0f);
        chi = make_float4(fmaxf(chi.x, shi.x), fmaxf(chi.y, shi.y), fmaxf(chi.z, shi.z), 0.0f);
        bin_lo[parent] = make_float4(clo.x, clo.y, clo.z, __uint_as_float(r - l + 1));
        bin_hi[parent] = make_float4(chi.x, chi.y, chi.z, __uint_as_float(l));
        if constexpr (W > 0) {
            float scost[W];
            if (sib & kLeafBit) {
                const float v = cp * box_area(slo, shi);
#pragma unroll
                for (int k = 0; k < W; k++) scost[k] = v;
            } else {
#pragma unroll
                for (int k = 0; k < W; k++) scost[k] = __ldcg(cost + 8ull * sib + k);
            }
            const uint32_t word = left ? dp_up_node<W>(ccost, scost, box_area(clo, chi), r - l + 1, leaf_max, cp, ccost)
                                       : dp_up_node<W>(scost, ccost, box_area(clo, chi), r - l + 1, leaf_max, cp, ccost);
            dp_store_costs<W>(cost + 8ull * parent, ccost);
            other[parent] = int32_t(word);
        }
        cur = parent;
        if (l == seg_first && r == seg_last) {
            segctl[kSegWords * s + kSegRoot] = parent;
            return;
        }
    }
}

struct TreeView {
    const uint32_t *child;
    const float4 *blo, *bhi;
    const float4 *lo, *hi;  // item boxes
    const uint32_t *vals;   // sorted item ids
    const unsigned long long *keys;
    uint32_t seg_shift;     // segment = key >> seg_shift (64: a single segment)
    const uint32_t *dp_dec = nullptr;  // collapse by dynamic program: decisions per binary node (else greedy)
    __device__ __forceinline__ bool leaf(uint32_t id) const { return (id & kLeafBit) != 0; }
    __device__ __forceinline__ uint32_t count(uint32_t id) const {
        return leaf(id) ? 1u : __float_as_uint(blo[id].w);
    }
    __device__ __forceinline__ uint32_t first(uint32_t id) const {
        return leaf(id) ? (id & ~kLeafBit) : __float_as_uint(bhi[id].w);
    }
    __device__ __forceinline__ uint32_t segment(uint32_t id) const {
        return seg_shift < 64 ? uint32_t(keys[first(id)] >> seg_shift) : 0u;
    }
    __device__ __forceinline__ void box(uint32_t id, float4 &l, float4 &h) const {
        if (leaf(id)) {
            const uint32_t it = vals[id & ~kLeafBit];
            l = lo[it];
            h = hi[it];
        } else {
            l = blo[id];
            h = bhi[id];
        }
    }
};

// Arrays of up to 8 entries kept in registers: every access is an unrolled loop over the 8
// positions, so a run-time index never sends the array to local memory (whose traffic, for the
// whole grid's threads, leaves L1).
template <typename T>
__device__ __forceinline__ T get8(const T (&a)[8], int i) {
    T v = a[0];
#pragma unroll
    for (int j = 1; j < 8; j++)
        if (i == j) v = a[j];
    return v;
}
template <typename T>
__device__ __forceinline__ void set8(T (&a)[8], int i, T v) {
#pragma unroll
    for (int j = 0; j < 8; j++)
        if (i == j) a[j] = v;
}

// Open up to `width` children of binary node b, assign them to octant slots
// and allocate their wide-node / item ranges.  desc: 12 words per wide node
// (binary node, child base, item base, segment, 8 slot children).
// fill: slots still free once no child can become a wide node are filled by
// splitting leaf slots (largest area first) into finer ones -- no new wide
// node, the node test costs the same, and a ray tests fewer triangles.
__device__ void collapse_node(const TreeView &tv, const SegInput *segs, uint32_t b, uint32_t w, uint32_t seg,
                              int leaf_max, int width, int fill, uint32_t *desc, uint2 *qout, uint32_t *ctl,
                              uint32_t *segctl, int level) {
    uint32_t C[8];
    float A[8];
#pragma unroll
    for (int k = 0; k < 8; k++) {
        C[k] = kInvalid;
        A[k] = 0.0f;
    }
    int nC;
    if (tv.leaf(b)) {
        C[0] = b;
        nC = 1;
    } else {
        C[0] = tv.child[2 * b];
        C[1] = tv.child[2 * b + 1];
        nC = 2;
    }
    const uint32_t kw = (tv.dp_dec != nullptr && !tv.leaf(b)) ? (tv.dp_dec[b] & 7u) : 0u;
    if (kw != 0u) {
        // the dynamic program's choice: `width` slots split kw | width - kw between b's children, each
        // side expanded by its own decisions (a subtree given i slots either takes i - 1, or splits
        // i = k + (i - k) between its children)
        uint32_t sn[8], si[8];
        const uint32_t c0 = C[0], c1 = C[1];
        nC = 0;
        int sp = 2;
        sn[0] = c1;
        si[0] = uint32_t(width) - kw;
        sn[1] = c0;
        si[1] = kw;
        while (sp > 0 && nC < 8) {
            --sp;
            uint32_t nd = get8(sn, sp), i = get8(si, sp);
            for (int guard = 0; guard < 16; guard++) {
                if (tv.leaf(nd) || i <= 1u) {
                    set8(C, nC, nd);
                    nC++;
                    break;
                }
                const uint32_t d = (tv.dp_dec[nd] >> (3u * (i - 1u))) & 7u;
                if (d == 0u || d >= i) {
                    i--;  // fewer slots serve this subtree as well
                    continue;
                }
                if (sp < 8) {
                    set8(sn, sp, tv.child[2 * nd + 1]);
                    set8(si, sp, i - d);
                    sp++;
                }
                nd = tv.child[2 * nd];
                i = d;
            }
        }
    } else {
#pragma unroll
        for (int k = 0; k < 8; k++) {
            if (k < nC) {
                float4 l, h;
                tv.box(C[k], l, h);
                A[k] = box_area(l, h);
            }
        }
    }
    // greedy (kw == 0): open the largest child that can become a wide node; with `fill`, then the
    // largest splittable leaf slot
    for (int pass = 0; pass < 2 && kw == 0u; pass++) {
        if (pass == 1 && !fill) break;
        while (nC < width) {
            int best = -1;
            float best_a = -1.0f;
#pragma unroll
            for (int k = 0; k < 8; k++) {
                if (k < nC && !tv.leaf(C[k]) && (pass == 1 || tv.count(C[k]) > uint32_t(leaf_max)) && A[k] > best_a) {
                    best_a = A[k];
                    best = k;
                }
            }
            if (best < 0) break;
            const uint32_t x = get8(C, best);
            const uint32_t xl = tv.child[2 * x], xr = tv.child[2 * x + 1];
            set8(C, best, xl);
            set8(C, nC, xr);
            float4 l, h;
            tv.box(xl, l, h);
            set8(A, best, box_area(l, h));
            tv.box(xr, l, h);
            set8(A, nC, box_area(l, h));
            nC++;
        }
    }
    // octant slot assignment: greedy on dot(child centroid - node centroid, octant diagonal)
    float4 nl, nh;
    tv.box(b, nl, nh);
    const float pc[3] = {0.5f * (nl.x + nh.x), 0.5f * (nl.y + nh.y), 0.5f * (nl.z + nh.z)};
    const bool node_empty = box_empty(nl, nh);
    float ox[8], oy[8], oz[8];
#pragma unroll
    for (int k = 0; k < 8; k++) {
        ox[k] = oy[k] = oz[k] = 0.0f;
        if (k < nC) {
            float4 l, h;
            tv.box(C[k], l, h);
            if (!(box_empty(l, h) || node_empty)) {
                ox[k] = 0.5f * (l.x + h.x) - pc[0];
                oy[k] = 0.5f * (l.y + h.y) - pc[1];
                oz[k] = 0.5f * (l.z + h.z) - pc[2];
            }
        }
    }
    uint32_t slot_child[8];
#pragma unroll
    for (int s = 0; s < 8; s++) slot_child[s] = kInvalid;
    // Each child's best slot is the octant of its offset's signs (it maximises the dot product with
    // the octant diagonal).  When those octants are distinct, the greedy assignment below gives
    // exactly them, so it is skipped (nodes of a few children).
    uint32_t pref_word = 0, pref_used = 0;  // child k's octant in bits 3k..3k+2
    bool distinct = LCX_OCTANT_FAST != 0;
#pragma unroll
    for (int k = 0; k < 8; k++) {
        if (k < nC) {
            const uint32_t pref = (ox[k] < 0.0f ? 1u : 0u) | (oy[k] < 0.0f ? 2u : 0u) | (oz[k] < 0.0f ? 4u : 0u);
            // a zero or NaN component ties two slots: leave those nodes to the greedy
            const bool clear = fabsf(ox[k]) > 0.0f && fabsf(oy[k]) > 0.0f && fabsf(oz[k]) > 0.0f;
            distinct = distinct && clear && !(pref_used >> pref & 1u);
            pref_used |= 1u << pref;
            pref_word |= pref << (3 * k);
        }
    }
    if (distinct) {
#pragma unroll
        for (int k = 0; k < 8; k++)
            if (k < nC) set8(slot_child, int((pref_word >> (3 * k)) & 7u), C[k]);
    } else {
        // the largest dot(offset, octant diagonal) over the free (child, slot) pairs, first in
        // child-major order on ties, nC times
        uint32_t used_slots = 0, used_children = 0;
        for (int it = 0; it < nC; it++) {
            float best = -INFINITY;
            int bk = -1, bs = -1;
#pragma unroll
            for (int k = 0; k < 8; k++) {
#pragma unroll
                for (int s = 0; s < 8; s++) {
                    if (k < nC && !(used_children >> k & 1u) && !(used_slots >> s & 1u)) {
                        const float sc = ((s & 1) ? -ox[k] : ox[k]) + ((s & 2) ? -oy[k] : oy[k]) +
                                         ((s & 4) ? -oz[k] : oz[k]);
                        const float cst = sc == sc ? sc : -FLT_MAX;  // NaN never blocks an assignment
                        if (bk < 0 || cst > best) {
                            best = cst;
                            bk = k;
                            bs = s;
                        }
                    }
                }
            }
            used_children |= 1u << bk;
            used_slots |= 1u << bs;
            set8(slot_child, bs, get8(C, bk));
        }
    }
    uint32_t n_int = 0, n_items = 0;
    for (int s = 0; s < 8; s++) {
        const uint32_t c = slot_child[s];
        if (c == kInvalid) continue;
        const uint32_t cnt = tv.count(c);
        if (!tv.leaf(c) && cnt > uint32_t(leaf_max))
            n_int++;
        else
            n_items += cnt;
    }
    uint32_t *sc = segctl + kSegWords * seg;
    // The global counters take every node of the level: one atomic per group of lanes that reach
    // this point together (a prefix over their counts gives each lane its range), instead of one
    // per lane on the same two addresses.
#if LCX_COLLAPSE_AGG
    cg::coalesced_group g = cg::coalesced_threads();
    const uint32_t incl = cg::inclusive_scan(g, n_int);
    const uint32_t total = g.shfl(incl, g.size() - 1);
    uint32_t wbase = 0, qb = 0;
    if (g.thread_rank() == g.size() - 1 && total) {
        wbase = atomicAdd(&ctl[kCtlWideCount], total);
        qb = atomicAdd(&ctl[kCtlLevel + level + 1], total);
    }
    wbase = g.shfl(wbase, g.size() - 1);
    qb = g.shfl(qb, g.size() - 1);
    const uint32_t child_base = n_int ? wbase + incl - n_int : 0u;
    const uint32_t qbase = n_int ? qb + incl - n_int : 0u;
#else
    const uint32_t child_base = n_int ? atomicAdd(&ctl[kCtlWideCount], n_int) : 0u;
    const uint32_t qbase = n_int ? atomicAdd(&ctl[kCtlLevel + level + 1], n_int) : 0u;
#endif
    const uint32_t item_base = n_items ? segs[seg].item_offset + atomicAdd(&sc[kSegItems], n_items) : 0u;
    if (n_int) atomicAdd(&sc[kSegNodes], n_int);
    atomicMax(&sc[kSegDepth], uint32_t(level + 1));
    uint32_t *d = desc + 12ull * w;
    d[0] = b;
    d[1] = child_base;
    d[2] = item_base;
    d[3] = seg;
    uint32_t rank = 0;
    for (int s = 0; s < 8; s++) {
        const uint32_t c = slot_child[s];
        d[4 + s] = c;
        if (c != kInvalid && !tv.leaf(c) && tv.count(c) > uint32_t(leaf_max)) {
            qout[qbase + rank] = make_uint2(c, child_base + rank);
            rank++;
        }
    }
}

// Parent of every item and internal binary node (kInvalid: none, a segment root).
__global__ void k_dp_parents(TreeView tv, const SegInput *segs, uint32_t nseg, uint32_t n, uint32_t *parent_item,
                             uint32_t *parent_node) {
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j + 1u >= n) return;
    const uint32_t s = segment_of(segs, nseg, j);
    if (j + 1u >= segs[s].item_offset + segs[s].item_count) return;  // not an internal node
#pragma unroll
    for (int side = 0; side < 2; side++) {
        const uint32_t c = tv.child[2ull * j + side];
        if (c & kLeafBit) {
            if ((c & ~kLeafBit) < n) parent_item[c & ~kLeafBit] = j;
        } else if (c < n) {
            parent_node[c] = j;
        }
    }
}

// The costs of child c for 1..8 slots (a leaf item: one leaf slot, whatever the slots).
template <int W>
__device__ __forceinline__ void dp_child_costs(const TreeView &tv, uint32_t c, float cp, const float *cost,
                                               float out[W]) {
    if (tv.leaf(c)) {
        float4 l, h;
        tv.box(c, l, h);
        const float v = cp * box_area(l, h);
#pragma unroll
        for (int i = 0; i < W; i++) out[i] = v;
    } else {
#pragma unroll
        for (int i = 0; i < W; i++) out[i] = __ldcg(cost + 8ull * c + i);
    }
}

// The costs and decisions of internal node nd from its children's (dp_up_node).
template <int W>
__device__ __forceinline__ void dp_node(const TreeView &tv, uint32_t nd, int leaf_max, float cp, float *cost,
                                        uint32_t *dec) {
    float cl[W], cr[W], out[W];
    dp_child_costs<W>(tv, tv.child[2ull * nd], cp, cost, cl);
    dp_child_costs<W>(tv, tv.child[2ull * nd + 1], cp, cost, cr);
    float4 l, h;
    tv.box(nd, l, h);
    dec[nd] = dp_up_node<W>(cl, cr, box_area(l, h), tv.count(nd), leaf_max, cp, out);
    dp_store_costs<W>(cost + 8ull * nd, out);
}

// One thread per item walks up; the second arrival at a node computes it (its other subtree is
// done).  The arrival is an acquire-release atomic: it publishes the costs this thread wrote and
// makes the sibling's visible.
template <int W>
__global__ void __launch_bounds__(256) k_dp_up(TreeView tv, uint32_t n, int leaf_max, float cp,
                                               const uint32_t *parent_item, const uint32_t *parent_node,
                                               uint32_t *arrivals, float *cost, uint32_t *dec) {
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    uint32_t nd = parent_item[p];
    for (uint32_t guard = 0; guard < n && nd < n; guard++) {
        uint32_t old;
        asm volatile("atom.acq_rel.gpu.global.add.u32 %0, [%1], 1;" : "=r"(old) : "l"(arrivals + nd) : "memory");
        if (old == 0u) return;
        dp_node<W>(tv, nd, leaf_max, cp, cost, dec);
        nd = parent_node[nd];
    }
}

template <int W>
void launch_dp_up(const TreeView &tv, uint32_t n, int leaf_max, float cp, const uint32_t *parent_item,
                  const uint32_t *parent_node, uint32_t *arrivals, float *cost, uint32_t *dec, cudaStream_t st) {
    k_dp_up<W><<<blocks_for(n, 256), 256, 0, st>>>(tv, n, leaf_max, cp, parent_item, parent_node, arrivals, cost,
                                                   dec);
}

void launch_dp_up_width(int width, const TreeView &tv, uint32_t n, int leaf_max, float cp,
                        const uint32_t *parent_item, const uint32_t *parent_node, uint32_t *arrivals, float *cost,
                        uint32_t *dec, cudaStream_t st) {
    switch (width) {
        case 2: launch_dp_up<2>(tv, n, leaf_max, cp, parent_item, parent_node, arrivals, cost, dec, st); break;
        case 3: launch_dp_up<3>(tv, n, leaf_max, cp, parent_item, parent_node, arrivals, cost, dec, st); break;
        case 4: launch_dp_up<4>(tv, n, leaf_max, cp, parent_item, parent_node, arrivals, cost, dec, st); break;
        case 5: launch_dp_up<5>(tv, n, leaf_max, cp, parent_item, parent_node, arrivals, cost, dec, st); break;
        case 6: launch_dp_up<6>(tv, n, leaf_max, cp, parent_item, parent_node, arrivals, cost, dec, st); break;
        case 7: launch_dp_up<7>(tv, n, leaf_max, cp, parent_item, parent_node, arrivals, cost, dec, st); break;
        default: launch_dp_up<8>(tv, n, leaf_max, cp, parent_item, parent_node, arrivals, cost, dec, st); break;
    }
}

// Level 0 tasks: the root of every non-empty segment s becomes wide node s.
__global__ void k_collapse_init(const SegInput *segs, uint32_t nseg, uint32_t *segctl, uint2 *q0, uint32_t *desc,
                                uint32_t *ctl) {
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s == 0) ctl[kCtlWideCount] = nseg;
    if (s >= nseg) return;
    desc[12ull * s + 3] = s;  // keeps the root slot of an empty segment identifiable
    if (segs[s].item_count == 0) return;
    const uint32_t pos = atomicAdd(&ctl[kCtlLevel + 0], 1u);
    q0[pos] = make_uint2(segctl[kSegWords * s + kSegRoot], s);
    segctl[kSegWords * s + kSegNodes] = 1u;
}

#ifndef LCX_COLLAPSE_MINB
// resident blocks per SM the collapse is compiled for (its arrays live in registers): 1024-mesh
// sample 28.8 / 28.7 / 28.5 / 28.5 ms at 1 / 4 / 5 / 6, against 32.8 ms with the arrays in
// local memory
#define LCX_COLLAPSE_MINB 5
#endif
__global__ void __launch_bounds__(128, LCX_COLLAPSE_MINB)
    k_collapse(TreeView tv, const SegInput *segs, int leaf_max, int width, int fill, uint32_t *desc,
                           uint2 *q0, uint2 *q1, uint32_t *ctl, uint32_t *segctl) {
    cg::grid_group grid = cg::this_grid();
    int level = 0;
    for (; level < kMaxLevels; level++) {
        const uint32_t cnt = __ldcg(&ctl[kCtlLevel + level]);
        if (cnt == 0) break;
        const uint2 *qin = (level & 1) ? q1 : q0;
        uint2 *qout = (level & 1) ? q0 : q1;
        for (unsigned long long t = grid.thread_rank(); t < cnt; t += grid.size()) {
            const uint2 task = qin[t];
            const uint32_t seg = tv.segment(task.x);
            collapse_node(tv, segs, task.x, task.y, seg, leaf_max, width, fill, desc, qout, ctl, segctl, level);
        }
        grid.sync();
    }
    if (grid.thread_rank() == 0) {
        ctl[kCtlDepth] = uint32_t(level);
        if (level == kMaxLevels && __ldcg(&ctl[kCtlLevel + kMaxLevels]) != 0) atomicOr(&ctl[kCtlErr], kErrTooDeep);
    }
}

// ---- emit
__device__ __forceinline__ uint32_t quant_exp(float lo, float hi) {
    const float x = __fdiv_ru(__fsub_ru(hi, lo), kQuantRange);
    const uint32_t bits = __float_as_uint(x);
    uint32_t b = bits >> 23;
    if (b == 0) return 1u;  // zero or subnormal extent: 2^-126
    if (bits & 0x7fffffu) b += 1;
    return min(b, 254u);
}

// Quantisation frame of a node box: per-axis exponents and the origin one
// step below the box (rounded down).  Shared by the emit and the refit.
__device__ __forceinline__ void quant_frame(const float4 &nl, const float4 &nh, uint32_t ex[3], float p[3]) {
    const bool node_empty = box_empty(nl, nh);
    ex[0] = node_empty ? 127u : quant_exp(nl.x, nh.x);
    ex[1] = node_empty ? 127u : quant_exp(nl.y, nh.y);
    ex[2] = node_empty ? 127u : quant_exp(nl.z, nh.z);
    p[0] = node_empty ? 0.0f : __fsub_rd(nl.x, __uint_as_float(ex[0] << 23));
    p[1] = node_empty ? 0.0f : __fsub_rd(nl.y, __uint_as_float(ex[1] << 23));
    p[2] = node_empty ? 0.0f : __fsub_rd(nl.z, __uint_as_float(ex[2] << 23));
}

// Outward 8-bit bounds of a non-empty child box in the frame (ex, p): exact
// outward bounds, then one more step outward on each side.
__device__ __forceinline__ void quant_child(const float cl[3], const float ch[3], const uint32_t ex[3], const float p[3],
                                            uint32_t ql[3], uint32_t qh[3], uint32_t *ctl) {
#pragma unroll
    for (int k = 0; k < 3; k++) {
        // e is a power of two, so 1 / e is exact (2^-127 included, as a subnormal) and x * (1 / e)
        // has the exact value of x / e: with the same directed rounding the two give the same bits,
        // and the multiplication is far cheaper than a directed division
#if LCX_QUANT_MUL
        const float inv_e = __frcp_rn(__uint_as_float(ex[k] << 23));
        float a = floorf(__fmul_rd(__fsub_rd(cl[k], p[k]), inv_e)) - 1.0f;
        float z = ceilf(__fmul_ru(__fsub_ru(ch[k], p[k]), inv_e)) + 1.0f;
#else
        const float e = __uint_as_float(ex[k] << 23);
        float a = floorf(__fdiv_rd(__fsub_rd(cl[k], p[k]), e)) - 1.0f;
        float z = ceilf(__fdiv_ru(__fsub_ru(ch[k], p[k]), e)) + 1.0f;
#endif
        if (!(a >= -1.0f) || !(z <= 255.0f)) atomicOr(&ctl[kCtlErr], kErrQuant);
        ql[k] = uint32_t(fminf(fmaxf(a, 0.0f), 255.0f));
        qh[k] = uint32_t(fminf(fmaxf(z, 0.0f), 255.0f));
    }
}

// Writes wide node w (both layouts, indices relative to its segment) and its
// leaf items; accumulates the segment's wide SAH (sum of node areas + leaf
// areas x counts) into sah[2 seg], its root area into sah[2 seg + 1].
// rtab (optional, meshes built for refit): entry c = parent of wide node c plus
// one in the low word (0 for a root), (segment << 3 | slot in the parent) in
// the high word; written by the parent for each internal child, by the root
// for itself.
template <class ItemWriter>
__device__ void emit_node(const TreeView &tv, const SegInput *segs, const uint32_t *desc, uint32_t w, Node8Q *qn,
                          Node8F *fn, int leaf_max, uint32_t *ctl, double *sah, unsigned long long *rtab,
                          ItemWriter &&write_item, float4 &node_lo, float4 &node_hi) {
    const uint32_t *d = desc + 12ull * w;
    const uint32_t b = d[0], child_base = d[1], item_base = d[2], seg = d[3];
    const uint32_t root = seg;  // wide index of the segment's root
    const uint32_t item_offset = segs[seg].item_offset;
    float4 nl, nh;
    tv.box(b, nl, nh);
    node_lo = nl;
    node_hi = nh;
    uint32_t ex[3];
    float p[3];
    quant_frame(nl, nh, ex, p);
    Node8Q q;
    Node8F f;
    q.px = p[0];
    q.py = p[1];
    q.pz = p[2];
    uint32_t meta_lo = 0, meta_hi = 0, imask = 0, offset = 0;
    uint32_t qlo[3][2] = {{0, 0}, {0, 0}, {0, 0}}, qhi[3][2] = {{0, 0}, {0, 0}, {0, 0}};
    double area_acc = box_area_d(nl.x, nl.y, nl.z, nh.x, nh.y, nh.z);
    for (int s = 0; s < 8; s++) {
        const uint32_t c = d[4 + s];
        uint32_t meta = 0;
        float cl[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, ch[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
        uint32_t ql[3] = {255u, 255u, 255u}, qh[3] = {0u, 0u, 0u};
        if (c != kInvalid) {
            float4 l, h;
            tv.box(c, l, h);
            const bool empty = box_empty(l, h);
            const uint32_t cnt = tv.count(c);
            if (!tv.leaf(c) && cnt > uint32_t(leaf_max)) {
                if (rtab != nullptr)
                    rtab[child_base + __popc(imask)] =
                        (static_cast<unsigned long long>((seg << 3) | uint32_t(s)) << 32) | (w + 1u);
                imask |= 1u << s;
                meta = kMetaInternalBase + uint32_t(s);
            } else {
                meta = empty ? 0u : meta_leaf(cnt, offset);
                const uint32_t first = tv.first(c);
                for (uint32_t j = 0; j < cnt; j++)
                    write_item(item_base + offset + j, tv.vals[first + j] - item_offset, seg);
                offset += cnt;
                area_acc += double(cnt) * box_area_d(l.x, l.y, l.z, h.x, h.y, h.z);
            }
            if (!empty) {
                cl[0] = l.x;
                cl[1] = l.y;
                cl[2] = l.z;
                ch[0] = h.x;
                ch[1] = h.y;
                ch[2] = h.z;
                quant_child(cl, ch, ex, p, ql, qh, ctl);
            }
        }
        const int wsel = s >> 2, sh = (s & 3) * 8;
        if (wsel == 0)
            meta_lo |= meta << sh;
        else
            meta_hi |= meta << sh;
#pragma unroll
        for (int k = 0; k < 3; k++) {
            qlo[k][wsel] |= ql[k] << sh;
            qhi[k][wsel] |= qh[k] << sh;
        }
        f.lo_x[s] = cl[0];
        f.lo_y[s] = cl[1];
        f.lo_z[s] = cl[2];
        f.hi_x[s] = ch[0];
        f.hi_y[s] = ch[1];
        f.hi_z[s] = ch[2];
    }
    const uint32_t cb = imask ? child_base - root : 0u;
    const uint32_t ib = offset ? item_base - item_offset : 0u;
    q.exps = ex[0] | (ex[1] << 8) | (ex[2] << 16) | (imask << 24);
    q.child_base = cb;
    q.item_base = ib;
    q.meta_lo = meta_lo;
    q.meta_hi = meta_hi;
    for (int k = 0; k < 2; k++) {
        q.qlo_x[k] = qlo[0][k];
        q.qlo_y[k] = qlo[1][k];
        q.qlo_z[k] = qlo[2][k];
        q.qhi_x[k] = qhi[0][k];
        q.qhi_y[k] = qhi[1][k];
        q.qhi_z[k] = qhi[2][k];
    }
    f.child_base = cb;
    f.item_base = ib;
    f.meta_lo = meta_lo;
    f.meta_hi = meta_hi;
    qn[w] = q;
    fn[w] = f;
    if (rtab != nullptr && w == root) rtab[w] = static_cast<unsigned long long>(seg << 3) << 32;
    if (sah != nullptr) {
        seg_sum(sah, seg, area_acc);
        if (w == root) sah[2 * seg + 1] = box_area_d(nl.x, nl.y, nl.z, nh.x, nh.y, nh.z);
    }
}

__global__ void k_emit_blas(TreeView tv, const SegInput *segs, const uint32_t *desc, uint32_t wide_count,
                            int leaf_max, Node8Q *qn, Node8F *fn, TriRec *tris, const uint32_t *segctl,
                            uint32_t *ctl, double *sah, unsigned long long *rtab, const uint32_t *ref_prim,
                            bool count_on_device) {
    const uint32_t w = blockIdx.x * blockDim.x + threadIdx.x;
    // a build that does not read its node count back: wide_count is the capacity
    // of the output, the collapse's count (never above it) bounds the work
    if (w >= wide_count || (count_on_device && w >= __ldcg(&ctl[kCtlWideCount]))) return;
    const uint32_t seg = desc[12ull * w + 3];
    if (segs[seg].item_count == 0) {  // root slot of an empty segment
        if (w == seg) {
            BlasDesc *bd = segs[seg].desc;
            bd->qnodes = nullptr;
            bd->fnodes = nullptr;
            bd->tris = nullptr;
            bd->node_count = 0;
            bd->tri_count = 0;
            bd->depth = 0;
            bd->bs_r = 0.0f;
            bd->valid = 0;
        }
        return;
    }
    float4 rl, rh;
    emit_node(
        tv, segs, desc, w, qn, fn, leaf_max, ctl, sah, rtab,
        [&](uint32_t pos, uint32_t item, uint32_t s) {
            const SegInput &g = segs[s];
            // a reference of a split build names its triangle (local index of the mesh)
            const uint32_t prim = ref_prim != nullptr ? ref_prim[g.item_offset + item] : item;
            if ((g.kind & 0xffu) == kSegAabbs) {
                const float *bx = reinterpret_cast<const float *>(g.vbase + 24ull * prim);
                tris[pos] = TriRec{make_float4(bx[0], bx[1], bx[2], __uint_as_float(prim)),
                                   make_float4(bx[3], bx[4], bx[5], 0.0f), make_float4(0.0f, 0.0f, 0.0f, 0.0f)};
                return;
            }
            if ((g.kind & 0xffu) == kSegCurves && curve_keys(g) > 1) {  // a keyframed cone
                const uint32_t keys = curve_keys(g);
                float4 *kd = reinterpret_cast<float4 *>(g.vstride) + 2ull * keys * prim;
                CurveCone cc{};
                for (uint32_t key = 0; key < keys; key++) {
                    cc = curve_cone(g, prim, key);
                    kd[2 * key] = cc.c0;
                    kd[2 * key + 1] = cc.c1;
                }
                const MeshMotion *mm = g.desc->motion;
                const unsigned long long ka = reinterpret_cast<unsigned long long>(kd);
                tris[pos] = TriRec{make_float4(mm->t0, mm->t1, __uint_as_float(mm->flags), __uint_as_float(cc.seg)),
                                   make_float4(__uint_as_float(keys), 0.0f, 0.0f, __uint_as_float(kTriCurveMotion)),
                                   make_float4(__uint_as_float(uint32_t(ka)), __uint_as_float(uint32_t(ka >> 32)),
                                               __uint_as_float(cc.k | (cc.pieces << 16)), __uint_as_float(cc.flags))};
                return;
            }
            if ((g.kind & 0xffu) == kSegCurves) {  // a cone: its balls, its place along the segment, open ends
                const CurveCone cc = curve_cone(g, prim);
                tris[pos] = TriRec{make_float4(cc.c0.x, cc.c0.y, cc.c0.z, __uint_as_float(cc.seg)),
                                   make_float4(cc.c1.x, cc.c1.y, cc.c1.z, __uint_as_float(kTriCurve)),
                                   make_float4(cc.c0.w, cc.c1.w, __uint_as_float(cc.k | (cc.pieces << 16)),
                                               __uint_as_float(cc.flags))};
                return;
            }
            if (g.kind >> 8) {  // vertex motion: the motion kernels interpolate the vertices at the ray's time
                const unsigned long long mp = reinterpret_cast<unsigned long long>(g.desc->motion);
                tris[pos] = TriRec{make_float4(0.0f, 0.0f, 0.0f, __uint_as_float(prim)),
                                   make_float4(0.0f, 0.0f, 0.0f, __uint_as_float(kTriMotion)),
                                   make_float4(__uint_as_float(uint32_t(mp)), __uint_as_float(uint32_t(mp >> 32)), 0.0f,
                                               0.0f)};
                return;
            }
            const uint32_t *t = reinterpret_cast<const uint32_t *>(g.tbase + 12ull * prim);
            float4 a = __ldg(reinterpret_cast<const float4 *>(g.vbase + g.vstride * t[0]));
            float4 b = __ldg(reinterpret_cast<const float4 *>(g.vbase + g.vstride * t[1]));
            float4 c = __ldg(reinterpret_cast<const float4 *>(g.vbase + g.vstride * t[2]));
            a.w = __uint_as_float(prim);
            b.w = 0.0f;
            c.w = 0.0f;
            tris[pos] = TriRec{a, b, c};
        },
        rl, rh);
    if (w == seg) {  // the segment's root writes the BLAS descriptor
        const SegInput &g = segs[seg];
        BlasDesc *bd = g.desc;
        const uint32_t *sc = segctl + kSegWords * seg;
        bd->qnodes = qn + seg;
        bd->fnodes = fn + seg;
        bd->tris = tris + g.item_offset;
        bd->node_count = sc[kSegNodes];
        bd->tri_count = g.item_count;
        const bool empty = box_empty(rl, rh);
        bd->lo[0] = rl.x;
        bd->lo[1] = rl.y;
        bd->lo[2] = rl.z;
        bd->hi[0] = rh.x;
        bd->hi[1] = rh.y;
        bd->hi[2] = rh.z;
        bd->depth = sc[kSegDepth];
        // radius: the root of the rounded-up squared distance, rounded up, and a relative pad for
        // the rounding of the corner offsets
        const float r2 = __uint_as_float(sc[kSegRad2]);
        bd->bs_r = (empty || !(r2 > 0.0f) || !isfinite(r2)) ? 0.0f : __fmul_ru(__fsqrt_ru(r2), 1.0f + 0x1p-16f);
        bd->valid = (empty ? 0u : 1u) | ((g.kind & 0xffu) == kSegAabbs ? 2u : 0u) |
                    ((g.kind & 0xffu) == kSegCurves ? 4u : 0u);
    }
}

// TLAS leaf record of instance `id` (its inverse transform from k_inst_prep).
__device__ __forceinline__ InstRec make_inst_rec(uint32_t id, const InstState *inst, const float *w2o) {
    InstRec r;
#pragma unroll
    for (int k = 0; k < 12; k++) r.w2o[k] = w2o[12ull * id + k];
    const InstState &s = inst[id];
    const BlasDesc *d = s.blas;
    const bool ok = d != nullptr && (d->valid & 1u);
    r.qnodes = ok ? d->qnodes : nullptr;
    r.tris = ok ? d->tris : nullptr;
    r.fnodes = ok ? d->fnodes : nullptr;
    r.inst_id = id;
    r.mask = !ok                ? 0u
             : (d->valid & 2u)  ? (((s.mask & 0xffu) << 8) | kInstProcedural)
             : (d->valid & 4u)  ? (((s.mask & 0xffu) << 8) | kInstCurve | (s.motion != nullptr ? kInstMotion : 0u))
             : s.motion != nullptr ? (((s.mask & 0xffu) << 8) | kInstMotion)
                                   : (s.mask & 0xffu);
    if (ok && s.motion != nullptr) {  // the MotionDesc address instead of an inverse
        const unsigned long long a = reinterpret_cast<unsigned long long>(s.motion);
        r.w2o[0] = __uint_as_float(uint32_t(a));
        r.w2o[1] = __uint_as_float(uint32_t(a >> 32));
    }
    return r;
}

__global__ void k_emit_tlas(TreeView tv, const SegInput *segs, const uint32_t *desc, uint32_t wide_count,
                            int leaf_max, const InstState *inst, const float *w2o, Node8Q *qn, Node8F *fn,
                            InstRec *recs, uint32_t *ctl, double *sah, unsigned long long *rtab) {
    const uint32_t w = blockIdx.x * blockDim.x + threadIdx.x;
    if (w >= wide_count) return;
    float4 rl, rh;
    emit_node(
        tv, segs, desc, w, qn, fn, leaf_max, ctl, sah, rtab,
        [&](uint32_t pos, uint32_t id, uint32_t) { recs[pos] = make_inst_rec(id, inst, w2o); },
        rl, rh);
}

__global__ void k_apply_mods(const ModRec *mods, uint32_t count, InstState *inst, uint32_t instance_count) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    const ModRec m = mods[i];
    if (m.index >= instance_count) return;  // validated on the host
    InstState &s = inst[m.index];
    // Modification flags: include/luisa/runtime/rhi/command.h:537-543
    if (m.flags & 1u) {
        s.blas = reinterpret_cast<const BlasDesc *>(m.primitive);
        s.motion = reinterpret_cast<const MotionDesc *>(m.motion);
    }
    if (m.flags & 2u)
        for (int k = 0; k < 12; k++) s.o2w[k] = m.affine[k];
    if (m.flags & 4u) s.opaque = 1u;
    else if (m.flags & 8u) s.opaque = 0u;
    if (m.flags & 16u) s.mask = m.vis_mask & 0xffu;
    if (m.flags & 32u) s.user_id = m.user_id;
}

__global__ void k_init_instances(InstState *inst, uint32_t begin, uint32_t end) {
    const uint32_t i = begin + blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= end) return;
    InstState s;
    const float id[12] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0};
    for (int k = 0; k < 12; k++) s.o2w[k] = id[k];
    s.blas = nullptr;
    s.mask = 0xffu;  // default visibility (accel.rs:289)
    s.user_id = 0;
    s.opaque = 1u;
    s._pad0 = 0;
    s.motion = nullptr;
    inst[i] = s;
}

// SAH of every segment's binary LBVH (C_node = C_item = 1): out[2 s] = sum of
// areas, out[2 s + 1] = root area.
// Also the squared radius of each segment's bounding sphere around its root box centre: the
// farthest item box corner, max-reduced per warp and segment into segctl[kSegRad2].
__global__ void k_binary_sah(uint32_t n, uint32_t seg_shift, const unsigned long long *keys, const uint32_t *vals,
                             const float4 *blo, const float4 *bhi, const float4 *lo, const float4 *hi,
                             const SegInput *segs, uint32_t *segctl, double *out) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t s = seg_shift < 64 ? uint32_t(keys[i] >> seg_shift) : 0u;
    const uint32_t it = vals[i];
    double acc = box_area(lo[it], hi[it]);
    // internal node i splits items i | i+1: it belongs to the segment iff both do
    const uint32_t last = segs[s].item_offset + segs[s].item_count - 1;
    if (i < last) acc += box_area(blo[i], bhi[i]);
    seg_sum(out, s, acc);
    const uint32_t r = segctl[kSegWords * s + kSegRoot];
    if (i == segs[s].item_offset)
        out[2 * s + 1] = (r & kLeafBit) ? box_area(lo[it], hi[it]) : box_area(blo[r], bhi[r]);
    const float4 rl = (r & kLeafBit) ? lo[it] : blo[r], rh = (r & kLeafBit) ? hi[it] : bhi[r];
    const float4 il = lo[it], ih = hi[it];
    uint32_t d2 = 0u;  // non-negative floats order as their bits
    if (!box_empty(il, ih) && !box_empty(rl, rh)) {
        const float cx = 0.5f * (rl.x + rh.x), cy = 0.5f * (rl.y + rh.y), cz = 0.5f * (rl.z + rh.z);
        const float mx = fmaxf(fabsf(il.x - cx), fabsf(ih.x - cx)), my = fmaxf(fabsf(il.y - cy), fabsf(ih.y - cy)),
                    mz = fmaxf(fabsf(il.z - cz), fabsf(ih.z - cz));
        const float q = __fmaf_ru(mx, mx, __fmaf_ru(my, my, __fmul_ru(mz, mz)));
        d2 = isfinite(q) ? __float_as_uint(q) : 0x7f800000u;
    }
    // one atomic per segment present in the warp; every lane that entered takes part in every vote
    // (the mask of each collective names exactly the lanes that execute it)
    const unsigned lanes = __activemask();
    unsigned todo = lanes;
    while (todo) {
        const uint32_t leader = __ffs(todo) - 1u;
        const uint32_t ls = __shfl_sync(lanes, s, leader);
        const uint32_t v = __reduce_max_sync(lanes, s == ls ? d2 : 0u);
        if (threadIdx.x % 32u == leader && v) atomicMax(&segctl[kSegWords * ls + kSegRad2], v);
        todo &= ~__ballot_sync(lanes, s == ls);
    }
}

TreeView make_view(const BuildScratch &s) {
    TreeView tv;
    tv.child = s.bin_child;
    tv.blo = s.bin_lo;
    tv.bhi = s.bin_hi;
    tv.lo = s.box_lo;
    tv.hi = s.box_hi;
    tv.vals = s.vals_sorted;
    tv.keys = s.keys_sorted;
    tv.seg_shift = s.nseg > 1 ? 3 * s.axis_bits : 64;
    return tv;
}

int collapse_grid() {
    static int grid = 0;
    if (grid == 0) {
        int dev = 0, sms = 0, per_sm = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_collapse, 128, 0);
        const int want = LCX_COLLAPSE_BLOCKS;
        grid = sms * (per_sm > want ? want : (per_sm > 0 ? per_sm : 1));
    }
    return grid;
}

cudaError_t build_rest(BuildScratch &s, const BuildParams &bp, cudaStream_t st, bool dp_done = false);

cudaError_t build_common(BuildScratch &s, const BuildParams &bp, cudaStream_t st) {
    NvtxRange nr("LBVH: Morton codes, sort, radix tree");
    const uint32_t n = s.n;
    note_build_launches(1);
    k_morton<<<blocks_for(n, 256), 256, 0, st>>>(s.segs, s.nseg, n, s.axis_bits, bp.size_bits, bp.cube, s.box_lo,
                                                  s.box_hi, s.segctl, s.keys, s.vals);
    cudaError_t e = sort_pairs(s.sort_tmp, s.sort_tmp_bytes, s.keys, s.keys_sorted, s.vals, s.vals_sorted, n,
                               3 * s.axis_bits + s.seg_bits, st);
    if (e != cudaSuccess) return e;
    if (n > 1) {
        e = cudaMemsetAsync(s.other, 0xff, sizeof(int32_t) * (n - 1), st);
        if (e != cudaSuccess) return e;
    }
    const uint32_t shift = s.nseg > 1 ? 3 * s.axis_bits : 64;
    // 8-wide collapse by dynamic program: in the same walk (decisions over the arrival words)
    const bool dp8 = s.dp_cost != nullptr && bp.width == 8 && n > 1;
    note_build_launches(1);
    if (dp8)
        k_lbvh<8><<<blocks_for(n, 256), 256, 0, st>>>(s.segs, n, shift, s.keys_sorted, s.vals_sorted, s.box_lo,
                                                       s.box_hi, s.bin_child, s.bin_lo, s.bin_hi, s.other, s.segctl,
                                                       bp.leaf_max, bp.dp_prim, s.dp_cost);
    else
        k_lbvh<0><<<blocks_for(n, 256), 256, 0, st>>>(s.segs, n, shift, s.keys_sorted, s.vals_sorted, s.box_lo,
                                                       s.box_hi, s.bin_child, s.bin_lo, s.bin_hi, s.other, s.segctl,
                                                       bp.leaf_max, bp.dp_prim, nullptr);
    return build_rest(s, bp, st, dp8);
}

// After the binary tree: its SAH (and the BLAS bounding spheres), then the collapse.
cudaError_t build_rest(BuildScratch &s, const BuildParams &bp, cudaStream_t st, bool dp_done) {
    NvtxRange nr("binary SAH, bounding spheres, collapse");
    const uint32_t n = s.n;
    const uint32_t shift = s.nseg > 1 ? 3 * s.axis_bits : 64;
    note_build_launches(1);
    k_binary_sah<<<blocks_for(n, 256), 256, 0, st>>>(n, shift, s.keys_sorted, s.vals_sorted, s.bin_lo, s.bin_hi,
                                                       s.box_lo, s.box_hi, s.segs, s.segctl, s.bin_sah);
    TreeView tv = make_view(s);
    if (dp_done) {
        tv.dp_dec = reinterpret_cast<const uint32_t *>(s.other);
    } else if (s.dp_cost != nullptr && n > 1) {
        // scratch the tree no longer needs: the Morton keys hold the parents, the unsorted ids the
        // arrival counters, the LBVH's sibling words the decisions
        uint32_t *parent_item = reinterpret_cast<uint32_t *>(s.keys), *parent_node = parent_item + n;
        uint32_t *arrivals = s.vals, *dec = reinterpret_cast<uint32_t *>(s.other);
        cudaError_t e = cudaMemsetAsync(parent_item, 0xff, sizeof(uint32_t) * 2ull * n, st);
        if (e == cudaSuccess) e = cudaMemsetAsync(arrivals, 0, sizeof(uint32_t) * n, st);
        if (e != cudaSuccess) return e;
        note_build_launches(2);
        k_dp_parents<<<blocks_for(n, 256), 256, 0, st>>>(tv, s.segs, s.nseg, n, parent_item, parent_node);
        launch_dp_up_width(bp.width, tv, n, bp.leaf_max, bp.dp_prim, parent_item, parent_node, arrivals, s.dp_cost,
                           dec, st);
        tv.dp_dec = dec;
    }
    note_build_launches(1);
    k_collapse_init<<<blocks_for(s.nseg, 256), 256, 0, st>>>(s.segs, s.nseg, s.segctl, s.queue, s.desc, s.ctl);
    const SegInput *segs = s.segs;
    int lm = bp.leaf_max, width = bp.width, fill = bp.fill ? 1 : 0;
    uint32_t *desc = s.desc;
    uint2 *q0 = s.queue, *q1 = s.queue + s.queue_len;
    uint32_t *ctl = s.ctl, *segctl = s.segctl;
    void *args[] = {&tv, &segs, &lm, &width, &fill, &desc, &q0, &q1, &ctl, &segctl};
    note_build_launches(1);
    return cudaLaunchCooperativeKernel(reinterpret_cast<void *>(k_collapse), dim3(collapse_grid()), dim3(128), args, 0,
                                       st);
}

}  // namespace

uint32_t morton_axis_bits(uint32_t nseg, uint32_t *seg_bits) {
    uint32_t sb = 0;
    while (nseg > 1 && (1u << sb) < nseg) sb++;
    *seg_bits = sb;
    const uint32_t ab = (63 - sb) / 3;
    return ab > 21 ? 21 : ab;
}

namespace {
std::atomic<uint64_t> g_build_launches{0};
}

void note_build_launches(uint32_t k) { g_build_launches.fetch_add(k, std::memory_order_relaxed); }
uint64_t build_launches() { return g_build_launches.load(std::memory_order_relaxed); }

cudaError_t build_tree_tris(BuildScratch &s, const BuildParams &bp, cudaStream_t st) {
    if (s.ref_prim == nullptr) {  // with triangle splitting split_emit has written the item boxes
        note_build_launches(1);
        k_tri_prep<<<blocks_for(s.n, kPrepBlock), kPrepBlock, 0, st>>>(s.segs, s.nseg, s.n, s.box_lo, s.box_hi,
                                                                       s.segctl, s.ctl);
    }
    return bp.blas_sah ? build_tree_sah(s, bp, st) : build_common(s, bp, st);
}

cudaError_t build_tree_lbvh(BuildScratch &s, const BuildParams &bp, cudaStream_t st) { return build_common(s, bp, st); }

cudaError_t build_tree_rest(BuildScratch &s, const BuildParams &bp, cudaStream_t st) { return build_rest(s, bp, st); }

cudaError_t split_count(const SegInput *tsegs, uint32_t nseg, uint32_t n, float fraction, float *wts,
                        unsigned long long *sums, uint32_t *refs, uint32_t *seg_refs, uint32_t *segctl, uint32_t *ctl,
                        cudaStream_t st) {
    uint32_t *wmax = reinterpret_cast<uint32_t *>(sums + nseg);
    cudaError_t e = cudaMemsetAsync(sums, 0, sizeof(unsigned long long) * nseg + sizeof(uint32_t) * nseg, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(seg_refs, 0, sizeof(uint32_t) * nseg, st);
    if (e != cudaSuccess) return e;
    note_build_launches(1);
    k_split_weight<<<blocks_for(n, kPrepBlock), kPrepBlock, 0, st>>>(tsegs, nseg, n, wts, wmax, segctl, ctl);
    note_build_launches(1);
    k_split_quant<<<blocks_for(n, kPrepBlock), kPrepBlock, 0, st>>>(tsegs, nseg, n, wts, wmax, sums);
    note_build_launches(1);
    k_split_assign<<<blocks_for(n, kPrepBlock), kPrepBlock, 0, st>>>(
        tsegs, nseg, n, reinterpret_cast<const uint32_t *>(wts), sums, fraction, refs, seg_refs);
    return cudaGetLastError();
}

cudaError_t exclusive_sum(void *tmp, size_t *tmp_bytes, const uint32_t *in, uint32_t *out, uint32_t n,
                          cudaStream_t st) {
    return cub::DeviceScan::ExclusiveSum(tmp, *tmp_bytes, in, out, int(n), st);
}

cudaError_t curve_prepare(const unsigned char *cps, uint64_t stride, uint32_t cp_count, uint32_t keys,
                          const uint32_t *seg, uint32_t nseg, uint32_t basis, float4 *bez, uint32_t *count,
                          uint32_t *meta, uint32_t *err, cudaStream_t st) {
    if (nseg == 0) return cudaSuccess;
    note_build_launches(1);
    k_curve_prep<<<blocks_for(nseg, kPrepBlock), kPrepBlock, 0, st>>>(cps, stride, cp_count, keys, seg, nseg, basis,
                                                                       bez, count, meta, err);
    return cudaGetLastError();
}

cudaError_t curve_fill(const uint32_t *off, const uint32_t *count, uint32_t nseg, uint32_t *cone_seg,
                       cudaStream_t st) {
    if (nseg == 0) return cudaSuccess;
    note_build_launches(1);
    k_curve_fill<<<blocks_for(nseg, kPrepBlock), kPrepBlock, 0, st>>>(off, count, nseg, cone_seg);
    return cudaGetLastError();
}

cudaError_t split_emit(const SegInput *tsegs, uint32_t nseg, uint32_t n, const uint32_t *refs, const uint32_t *ref_off,
                       BuildScratch &s, uint32_t *ref_prim, cudaStream_t st) {
    note_build_launches(1);
    k_split_emit<<<blocks_for(n, kPrepBlock), kPrepBlock, 0, st>>>(tsegs, nseg, n, refs, ref_off, s.box_lo, s.box_hi,
                                                                   ref_prim, s.segctl);
    s.ref_prim = ref_prim;
    return cudaGetLastError();
}

cudaError_t build_tree_insts(const InstState *inst, BuildScratch &s, const BuildParams &bp, cudaStream_t st) {
    note_build_launches(1);
    k_inst_prep<<<blocks_for(s.n, kPrepBlock), kPrepBlock, 0, st>>>(inst, s.n, s.box_lo, s.box_hi, s.w2o, s.segctl);
    return bp.tlas_sah ? build_tree_sah(s, bp, st) : build_common(s, bp, st);
}

cudaError_t emit_blas(const BuildScratch &s, const BuildParams &bp, uint32_t wide_count, Node8Q *qn, Node8F *fn,
                      TriRec *tris, double *wide_sah, unsigned long long *rtab, cudaStream_t st,
                      bool count_on_device) {
    note_build_launches(1);
    k_emit_blas<<<blocks_for(wide_count, 128), 128, 0, st>>>(make_view(s), s.segs, s.desc, wide_count, bp.leaf_max,
                                                              qn, fn, tris, s.segctl, s.ctl, wide_sah, rtab,
                                                              s.ref_prim, count_on_device);
    return cudaGetLastError();
}

__global__ void k_or_errors(const uint32_t *ctl, uint32_t *into) {
    const uint32_t e = ctl[kCtlErr];
    if (e) atomicOr(&into[kCtlErr], e);
}

cudaError_t report_build_errors(const uint32_t *ctl, uint32_t *into, cudaStream_t st) {
    note_build_launches(1);
    k_or_errors<<<1, 1, 0, st>>>(ctl, into);
    return cudaGetLastError();
}

cudaError_t emit_tlas(const InstState *inst, const BuildScratch &s, const BuildParams &bp, uint32_t wide_count,
                      Node8Q *qn, Node8F *fn, InstRec *recs, double *wide_sah, unsigned long long *rtab,
                      cudaStream_t st) {
    note_build_launches(1);
    k_emit_tlas<<<blocks_for(wide_count, 128), 128, 0, st>>>(make_view(s), s.segs, s.desc, wide_count, bp.leaf_max,
                                                              inst, s.w2o, qn, fn, recs, s.ctl, wide_sah, rtab);
    return cudaGetLastError();
}

cudaError_t apply_modifications(const ModRec *mods, uint32_t count, InstState *inst, uint32_t instance_count,
                                cudaStream_t st) {
    if (count == 0) return cudaSuccess;
    note_build_launches(1);
    k_apply_mods<<<blocks_for(count, 256), 256, 0, st>>>(mods, count, inst, instance_count);
    return cudaGetLastError();
}

cudaError_t init_instances(InstState *inst, uint32_t begin, uint32_t end, cudaStream_t st) {
    if (end <= begin) return cudaSuccess;
    note_build_launches(1);
    k_init_instances<<<blocks_for(end - begin, 256), 256, 0, st>>>(inst, begin, end);
    return cudaGetLastError();
}

// ---- refit: same topology, new vertices
namespace {

// Box of one item from its vertices, as k_tri_prep computes it.
__device__ __forceinline__ void item_box(const float4 &a, const float4 &b, const float4 &c, float l[3], float h[3]) {
    l[0] = fminf(fminf(FLT_MAX, a.x), fminf(b.x, c.x));
    l[1] = fminf(fminf(FLT_MAX, a.y), fminf(b.y, c.y));
    l[2] = fminf(fminf(FLT_MAX, a.z), fminf(b.z, c.z));
    h[0] = fmaxf(fmaxf(-FLT_MAX, a.x), fmaxf(b.x, c.x));
    h[1] = fmaxf(fmaxf(-FLT_MAX, a.y), fmaxf(b.y, c.y));
    h[2] = fmaxf(fmaxf(-FLT_MAX, a.z), fmaxf(b.z, c.z));
}

__device__ __forceinline__ bool box3_empty(const float l[3], const float h[3]) {
    return !(l[0] <= h[0] && l[1] <= h[1] && l[2] <= h[2]);
}

// Bottom-up refit over the wide nodes of one BVH block (a BLAS block or a
// TLAS): a thread starts at a node without internal children, rewrites the
// leaf records of its leaf slots (triangles or AABBs from the segment's
// current buffers, by the prim id each record keeps; TLAS: the instance
// records, from the instance states) and their boxes, takes its node box as
// the union of its slots, writes it into the parent's slot and goes on with
// the parent if it is the last of the parent's internal children to arrive
// (the parent's counter).  Boxes written by other threads are read with ld.cg
// after the counter says they are complete.
struct RefitArgs {
    uint32_t W;
    const unsigned long long *rtab;
    const Node8Q *qn;
    Node8F *fn;
    uint32_t *counters, *ctl;
    // BLAS blocks
    const SegInput *segs;
    uint32_t nseg;
    TriRec *tris;
    // TLAS
    const InstState *inst;
    const float4 *ilo, *ihi;  // instance world boxes (k_inst_prep)
    const float *w2o;
    InstRec *recs;
    uint32_t ninst;
};

template <bool kTlas>
__global__ void k_refit(RefitArgs A) {
    uint32_t w = blockIdx.x * blockDim.x + threadIdx.x;
    if (w >= A.W) return;
    if ((__ldg(&A.qn[w].exps) >> 24) != 0u) return;
    for (int level = 0; level <= kMaxLevels; level++) {
        const unsigned long long te = __ldg(&A.rtab[w]);
        const uint32_t hiw = uint32_t(te >> 32), parent1 = uint32_t(te);
        const uint32_t seg = hiw >> 3, pslot = hiw & 7u;
        if (seg >= (kTlas ? 1u : A.nseg)) {  // cannot happen for a table the build wrote
            atomicOr(&A.ctl[kCtlErr], kErrBadIndex);
            return;
        }
        SegInput g{};
        if (!kTlas) g = A.segs[seg];
        Node8F &f = A.fn[w];
        const uint32_t meta_lo = __ldcg(&f.meta_lo), meta_hi = __ldcg(&f.meta_hi), ib = __ldcg(&f.item_base);
        float nl[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, nh[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
        for (int s = 0; s < 8; s++) {
            const uint32_t meta = ((s < 4 ? meta_lo : meta_hi) >> (8 * (s & 3))) & 0xffu;
            if (meta == 0u) continue;
            float cl[3], ch[3];
            if (meta_internal(meta)) {
                cl[0] = __ldcg(&f.lo_x[s]);
                cl[1] = __ldcg(&f.lo_y[s]);
                cl[2] = __ldcg(&f.lo_z[s]);
                ch[0] = __ldcg(&f.hi_x[s]);
                ch[1] = __ldcg(&f.hi_y[s]);
                ch[2] = __ldcg(&f.hi_z[s]);
            } else {
                cl[0] = cl[1] = cl[2] = FLT_MAX;
                ch[0] = ch[1] = ch[2] = -FLT_MAX;
                const uint32_t cnt = meta_count(meta), off = meta & 31u;
                for (uint32_t j = 0; j < cnt; j++) {
                    float il[3], ih[3];
                    if (kTlas) {
                        const uint32_t pos = ib + off + j;
                        if (pos >= A.ninst) {  // cannot happen for a node the build wrote
                            atomicOr(&A.ctl[kCtlErr], kErrBadIndex);
                            continue;
                        }
                        const uint32_t id = A.recs[pos].inst_id;
                        if (id >= A.ninst) {
                            atomicOr(&A.ctl[kCtlErr], kErrBadIndex);
                            continue;
                        }
                        const float4 l = A.ilo[id], h = A.ihi[id];
                        il[0] = l.x;
                        il[1] = l.y;
                        il[2] = l.z;
                        ih[0] = h.x;
                        ih[1] = h.y;
                        ih[2] = h.z;
                        A.recs[pos] = make_inst_rec(id, A.inst, A.w2o);
                    } else {
                        if (ib + off + j >= g.item_count) {  // cannot happen for a node the build wrote
                            atomicOr(&A.ctl[kCtlErr], kErrBadIndex);
                            continue;
                        }
                        TriRec *r = A.tris + (size_t(g.item_offset) + ib + off + j);
                        const uint32_t prim = __float_as_uint(r->v0.w);
                        if (prim >= g.item_count) {  // cannot happen for a record the build wrote
                            atomicOr(&A.ctl[kCtlErr], kErrBadIndex);
                            continue;
                        }
                        if ((g.kind & 0xffu) == kSegAabbs) {
                            const float *bx = reinterpret_cast<const float *>(g.vbase + 24ull * prim);
                            for (int k = 0; k < 3; k++) {
                                il[k] = bx[k];
                                ih[k] = bx[3 + k];
                            }
                            *r = TriRec{make_float4(il[0], il[1], il[2], __uint_as_float(prim)),
                                        make_float4(ih[0], ih[1], ih[2], 0.0f), make_float4(0.0f, 0.0f, 0.0f, 0.0f)};
                        } else {
                            const uint32_t *t = reinterpret_cast<const uint32_t *>(g.tbase + 12ull * prim);
                            const uint32_t i0 = t[0], i1 = t[1], i2 = t[2];
                            if (i0 >= g.vcount || i1 >= g.vcount || i2 >= g.vcount) {
                                atomicOr(&A.ctl[kCtlErr], kErrBadIndex);
                                continue;
                            }
                            float4 a = __ldg(reinterpret_cast<const float4 *>(g.vbase + g.vstride * i0));
                            float4 b = __ldg(reinterpret_cast<const float4 *>(g.vbase + g.vstride * i1));
                            float4 c = __ldg(reinterpret_cast<const float4 *>(g.vbase + g.vstride * i2));
                            item_box(a, b, c, il, ih);
                            a.w = __uint_as_float(prim);
                            b.w = 0.0f;
                            c.w = 0.0f;
                            *r = TriRec{a, b, c};
                        }
                    }
                    if (!box3_empty(il, ih)) {
#pragma unroll
                        for (int k = 0; k < 3; k++) {
                            cl[k] = fminf(cl[k], il[k]);
                            ch[k] = fmaxf(ch[k], ih[k]);
                        }
                    }
                }
                f.lo_x[s] = cl[0];
                f.lo_y[s] = cl[1];
                f.lo_z[s] = cl[2];
                f.hi_x[s] = ch[0];
                f.hi_y[s] = ch[1];
                f.hi_z[s] = ch[2];
            }
#pragma unroll
            for (int k = 0; k < 3; k++) {
                nl[k] = fminf(nl[k], cl[k]);
                nh[k] = fmaxf(nh[k], ch[k]);
            }
        }
        if (parent1 == 0u) {  // a root: a BLAS root's box for the TLAS builds
            BlasDesc *bd = kTlas ? nullptr : g.desc;
            if (bd != nullptr) {
                const bool empty = box3_empty(nl, nh);
                for (int k = 0; k < 3; k++) {
                    bd->lo[k] = empty ? FLT_MAX : nl[k];
                    bd->hi[k] = empty ? -FLT_MAX : nh[k];
                }
                bd->bs_r = 0.0f;  // the build's sphere no longer bounds the moved items: the box alone
                bd->valid = (empty ? 0u : 1u) | ((g.kind & 0xffu) == kSegAabbs ? 2u : 0u) |
                            ((g.kind & 0xffu) == kSegCurves ? 4u : 0u);
            }
            return;
        }
        const uint32_t parent = parent1 - 1u;
        if (parent >= A.W || pslot > 7u) {  // cannot happen for a table the build wrote
            atomicOr(&A.ctl[kCtlErr], kErrBadIndex);
            return;
        }
        Node8F &pf = A.fn[parent];
        pf.lo_x[pslot] = nl[0];
        pf.lo_y[pslot] = nl[1];
        pf.lo_z[pslot] = nl[2];
        pf.hi_x[pslot] = nh[0];
        pf.hi_y[pslot] = nh[1];
        pf.hi_z[pslot] = nh[2];
        const uint32_t need = __popc(__ldg(&A.qn[parent].exps) >> 24);
        // acquire-release: publishes this slot's box, sees the other slots' when last
        uint32_t arrived;
        asm volatile("atom.acq_rel.gpu.global.add.u32 %0, [%1], 1;" : "=r"(arrived) : "l"(A.counters + parent) : "memory");
        if (arrived + 1u != need) return;
        w = parent;
    }
    atomicOr(&A.ctl[kCtlErr], kErrTooDeep);
}

// Re-encodes the quantised node from the refit FP32 node: node box = union of
// the slot boxes, then the emit's frame and outward child bounds.
__global__ void k_requantize(uint32_t W, Node8Q *qn, const Node8F *fn, uint32_t *ctl) {
    const uint32_t w = blockIdx.x * blockDim.x + threadIdx.x;
    if (w >= W) return;
    const Node8F &f = fn[w];
    float4 nl = make_float4(FLT_MAX, FLT_MAX, FLT_MAX, 0.0f), nh = make_float4(-FLT_MAX, -FLT_MAX, -FLT_MAX, 0.0f);
    for (int s = 0; s < 8; s++) {
        nl.x = fminf(nl.x, f.lo_x[s]);
        nl.y = fminf(nl.y, f.lo_y[s]);
        nl.z = fminf(nl.z, f.lo_z[s]);
        nh.x = fmaxf(nh.x, f.hi_x[s]);
        nh.y = fmaxf(nh.y, f.hi_y[s]);
        nh.z = fmaxf(nh.z, f.hi_z[s]);
    }
    uint32_t ex[3];
    float p[3];
    quant_frame(nl, nh, ex, p);
    Node8Q q = qn[w];
    q.px = p[0];
    q.py = p[1];
    q.pz = p[2];
    q.exps = ex[0] | (ex[1] << 8) | (ex[2] << 16) | (q.exps & 0xff000000u);
    uint32_t qlo[3][2] = {{0, 0}, {0, 0}, {0, 0}}, qhi[3][2] = {{0, 0}, {0, 0}, {0, 0}};
    for (int s = 0; s < 8; s++) {
        const float cl[3] = {f.lo_x[s], f.lo_y[s], f.lo_z[s]}, ch[3] = {f.hi_x[s], f.hi_y[s], f.hi_z[s]};
        uint32_t ql[3] = {255u, 255u, 255u}, qh[3] = {0u, 0u, 0u};
        if (!box3_empty(cl, ch)) quant_child(cl, ch, ex, p, ql, qh, ctl);
        const int wsel = s >> 2, sh = (s & 3) * 8;
        for (int k = 0; k < 3; k++) {
            qlo[k][wsel] |= ql[k] << sh;
            qhi[k][wsel] |= qh[k] << sh;
        }
    }
    for (int k = 0; k < 2; k++) {
        q.qlo_x[k] = qlo[0][k];
        q.qlo_y[k] = qlo[1][k];
        q.qlo_z[k] = qlo[2][k];
        q.qhi_x[k] = qhi[0][k];
        q.qhi_y[k] = qhi[1][k];
        q.qhi_z[k] = qhi[2][k];
    }
    qn[w] = q;
}

}  // namespace

cudaError_t refit_blas(const SegInput *segs, uint32_t nseg, uint32_t W, const unsigned long long *rtab, Node8Q *qn,
                       Node8F *fn, TriRec *tris, uint32_t *counters, uint32_t *ctl, cudaStream_t st) {
    if (W == 0) return cudaSuccess;
    cudaError_t e = cudaMemsetAsync(counters, 0, sizeof(uint32_t) * W, st);
    if (e != cudaSuccess) return e;
    RefitArgs A{};
    A.W = W;
    A.rtab = rtab;
    A.qn = qn;
    A.fn = fn;
    A.counters = counters;
    A.ctl = ctl;
    A.segs = segs;
    A.nseg = nseg;
    A.tris = tris;
    note_build_launches(1);
    k_refit<false><<<blocks_for(W, 128), 128, 0, st>>>(A);
    note_build_launches(1);
    k_requantize<<<blocks_for(W, 128), 128, 0, st>>>(W, qn, fn, ctl);
    return cudaGetLastError();
}

cudaError_t refit_tlas(const InstState *inst, uint32_t n, float4 *ilo, float4 *ihi, float *w2o, uint32_t *segctl,
                       uint32_t W, const unsigned long long *rtab, Node8Q *qn, Node8F *fn, InstRec *recs,
                       uint32_t *counters, uint32_t *ctl, cudaStream_t st) {
    if (W == 0 || n == 0) return cudaSuccess;
    cudaError_t e = cudaMemsetAsync(counters, 0, sizeof(uint32_t) * W, st);
    if (e != cudaSuccess) return e;
    // instance world boxes and inverses, as a build computes them (segctl: scratch)
    note_build_launches(1);
    k_inst_prep<<<blocks_for(n, kPrepBlock), kPrepBlock, 0, st>>>(inst, n, ilo, ihi, w2o, segctl);
    RefitArgs A{};
    A.W = W;
    A.rtab = rtab;
    A.qn = qn;
    A.fn = fn;
    A.counters = counters;
    A.ctl = ctl;
    A.inst = inst;
    A.ilo = ilo;
    A.ihi = ihi;
    A.w2o = w2o;
    A.recs = recs;
    A.ninst = n;
    note_build_launches(1);
    k_refit<true><<<blocks_for(W, 128), 128, 0, st>>>(A);
    note_build_launches(1);
    k_requantize<<<blocks_for(W, 128), 128, 0, st>>>(W, qn, fn, ctl);
    return cudaGetLastError();
}

}  // namespace lcx
