// trace.cuh — trace_closest / trace_any as device functions, called per ray
// from inside a user kernel.
//
// The reference's kernels call the acceleration structure once per ray from
// their own code: the DSL's Accel::intersect / intersect_any
// (src/dsl/rtx/accel.cpp:120-150) become lc_accel_trace_closest /
// lc_accel_trace_any in the CUDA backend
// (src/backends/cuda/cuda_builtin/cuda_device_resource.h:1784-1829) and
// lc_trace_closest / lc_trace_any in the CPU backend
// (src/rust/luisa_compute_backend_impl/src/cpu/codegen/cpp.rs:1334-1350).  A
// megakernel such as src/tests/test_path_tracing.cpp:165-250 traces each
// thread's path segment this way.  These functions are that call for a CUDA
// kernel of the user's own:
//
//   #include <lcx/trace.cuh>              // include/ of this repository
//   __global__ void shade(LcxAccelView v, const LcxRay *rays, LcxTriangleHit *hits, uint32_t n) {
//       const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
//       if (i < n) hits[i] = lcx::trace_closest(v, rays[i], 0xffu);
//   }
//
// The view comes from lcx_accel_device_view() and stays valid until the accel
// is built again or destroyed.  Results are those of lcx_trace_closest /
// lcx_trace_any on the same accel bit for bit: the same quantised-node test,
// instance transform and watertight triangle test, the same (t, inst, prim)
// tie rule, curves traced with the curve test, procedural instances passed
// over, motion instances and keyframed meshes and curves at time 0 (the
// _motion forms take a time per ray).
//
// The walk is the trace kernels' loop mode 0 for one ray per thread: one node
// per step, its triangles tested at once, the node group stack split between
// a short stack and a local-memory rest.  The short stack is either local too
// (the plain forms) or, in the forms taking a ShortStack, kShort entries per
// thread in shared memory the caller's kernel owns: what the persistent trace
// kernels measured fastest (16 entries per thread).  The rare geometry --
// curves, keyframed vertices, moving instances -- runs in functions that are
// not inlined, so a kernel over plain triangle meshes keeps the registers of
// the triangle walk.  Unlike the batched lcx_trace_closest, the calling kernel
// owns the threads: a warp runs until its slowest ray is done, with no refill
// of finished lanes.
#pragma once

#include "lcx/node_test.cuh"
#include "lcx_accel.h"

namespace lcx {

// A thread's short stack in the caller's shared memory: entries
// base[k * stride] for k < kShort (e.g. base = smem + threadIdx.x, stride =
// blockDim.x, for __shared__ uint2 smem[kShort * blockDim.x]).
struct ShortStack {
    uint2 *base;
    uint32_t stride;
};

namespace detail {

// A special leaf item: a cone of a curve (kTriCurve, kTriCurveMotion) or a
// triangle of a keyframed mesh (kTriMotion), at `time`: whether it is hit in
// [tmin, tmax] and the hit's (t, u, v) -- v = -1 for a curve, u its parameter.
// Not inlined: it is rare and register-hungry.  Arguments and result go by
// value, so the caller's ray state stays in registers.
struct ItemHit {
    float t, u, v;
    bool hit;
};
static __device__ __noinline__ ItemHit special_item(float4 a, float4 b, float4 c, float time, WtRay wt, float ox, float oy,
                                             float oz, float dx, float dy, float dz, float tmin, float tmax) {
    ItemHit r{0.0f, 0.0f, 0.0f, false};
    const uint32_t marker = __float_as_uint(b.w);
    if (marker == kTriCurve || marker == kTriCurveMotion) {
        float4 c0 = make_float4(a.x, a.y, a.z, c.x), c1 = make_float4(b.x, b.y, b.z, c.y);
        if (marker == kTriCurveMotion && !curve_motion_cone(a, b, c, time, c0, c1)) return r;
        const uint32_t kn = __float_as_uint(c.z);
        r.hit = curve_piece_entry(make_float3(ox, oy, oz), make_float3(dx, dy, dz), c0, c1, kn & 0xffffu, kn >> 16,
                                  __float_as_uint(c.w), tmin, tmax, r.t, r.u);
        r.v = -1.0f;
        return r;
    }
    // kTriMotion: v2.xy hold the mesh's MeshMotion address
    const MeshMotion *mm = reinterpret_cast<const MeshMotion *>((unsigned long long)__float_as_uint(c.x) |
                                                                ((unsigned long long)__float_as_uint(c.y) << 32));
    if (!motion_triangle(*mm, __float_as_uint(a.w), time, a, b, c)) return r;
    r.hit = wt_intersect(wt, tmin, tmax, a, b, c, r.t, r.u, r.v);
    return r;
}

// World-to-object matrix of a moving instance at `time` (its MotionDesc address
// in the record's first 8 bytes), as three rows; ok = false when it has
// vanished.  Not inlined.
struct W2O {
    float4 r0, r1, r2;
    bool ok;
};
static __device__ __noinline__ W2O moving_w2o(float4 r0, float time) {
    const MotionDesc *md = reinterpret_cast<const MotionDesc *>((unsigned long long)__float_as_uint(r0.x) |
                                                                ((unsigned long long)__float_as_uint(r0.y) << 32));
    W2O o{};
    float m[12], w[12];
    if (!motion_matrix(*md, time, m)) return o;
    affine_inverse(m, w);
    o.r0 = make_float4(w[0], w[1], w[2], w[3]);
    o.r1 = make_float4(w[4], w[5], w[6], w[7]);
    o.r2 = make_float4(w[8], w[9], w[10], w[11]);
    o.ok = true;
    return o;
}

// max_steps: per-ray step bound; a ray that exceeds it ends with the record it
// has and, when err is not null, sets bit 1 of *err.
template <bool kAny, int kShort>
__device__ __forceinline__ void trace_walk(const LcxAccelView &view, const LcxRay &ray, float time, uint32_t mask,
                                           ShortStack ss, LcxTriangleHit &hit, bool &occluded,
                                           uint32_t max_steps = kMaxRaySteps, uint32_t *err = nullptr) {
    static_assert(kShort >= 1, "at least one short-stack entry");
    constexpr int kS = kShort < kStackSize ? kShort : kStackSize;
    constexpr int kDeep = kStackSize - kS;
    uint2 deep[kDeep > 0 ? kDeep : 1];
    const Node8Q *tlas = static_cast<const Node8Q *>(view.tlas_nodes);
    const InstRec *insts = static_cast<const InstRec *>(view.instances);
    const float wox = ray.origin[0], woy = ray.origin[1], woz = ray.origin[2];
    const float wdx = ray.direction[0], wdy = ray.direction[1], wdz = ray.direction[2];
    const float tmin = ray.t_min;
    float best_t = ray.t_max, best_u = 0.0f, best_v = 0.0f;
    uint32_t best_inst = kInvalid, best_prim = kInvalid;
    mask &= 0xffu;
    float ox = wox, oy = woy, oz = woz;
    float dx = wdx, dy = wdy, dz = wdz;  // current-space direction (the curve test reads it)
    float ix = slab_rcp(wdx), iy = slab_rcp(wdy), iz = slab_rcp(wdz);
    uint32_t octinv = octant_inv(wdx, wdy, wdz);
    WtRay wt{};
    int sp = 0, blas_sp = 0;
    bool in_blas = false;
    uint32_t cur_inst = 0;
    const Node8Q *blas = nullptr;
    const TriRec *tris = nullptr;
    uint2 G = (wdx == 0.0f && wdy == 0.0f && wdz == 0.0f) ? make_uint2(0, 0) : root_group(octinv);
    occluded = false;
    // indices are clamped as well as branched on, so a speculated load stays in bounds
    auto push = [&](uint2 g) {
        if (sp < kS) {
            if (kS > 0) ss.base[uint32_t(min(sp, kS - 1)) * ss.stride] = g;
            sp++;
        } else if (kDeep > 0 && sp < kStackSize) {
            deep[min(max(sp - kS, 0), kDeep > 0 ? kDeep - 1 : 0)] = g;
            sp++;
        }
    };
    auto pop = [&]() -> uint2 {
        sp--;
        if (kDeep == 0 || sp < kS) return ss.base[uint32_t(min(max(sp, 0), kS > 0 ? kS - 1 : 0)) * ss.stride];
        return deep[min(max(sp - kS, 0), kDeep > 0 ? kDeep - 1 : 0)];
    };

    for (uint32_t steps = 1;; steps++) {
        if (steps > max_steps) {
            if (err != nullptr) atomicOr(err, 2u);
            break;
        }
        uint2 Gt;
        if (G.y >= 0x01000000u) {  // visit the front child of the node group; push the rest
            const uint32_t key = __ffs(G.y >> 24) - 1u;
            G.y &= ~(1u << (24 + key));
            const uint32_t slot = key ^ octinv;
            const uint32_t child = G.x + __popc(G.y & 0xffu & ((1u << slot) - 1u));
            if (G.y >= 0x01000000u) push(G);
            intersect_q(in_blas ? blas : tlas, child, ox, oy, oz, ix, iy, iz, octinv, tmin, best_t, G, Gt);
        } else {
            Gt = G;
            G = make_uint2(0, 0);
        }
        if (in_blas) {
            while (Gt.y) {  // the node's triangles (or curve cones)
                const uint32_t k = __ffs(Gt.y) - 1u;
                Gt.y &= Gt.y - 1u;
                const float4 *tp = reinterpret_cast<const float4 *>(tris + Gt.x + k);
                const float4 a = __ldg(tp), b = __ldg(tp + 1), c = __ldg(tp + 2);
                float t, u, v;
                if (__float_as_uint(b.w) >= kTriCurveMotion) {
                    const ItemHit ih = special_item(a, b, c, time, wt, ox, oy, oz, dx, dy, dz, tmin, best_t);
                    if (!ih.hit) continue;
                    t = ih.t;
                    u = ih.u;
                    v = ih.v;
                } else if (!wt_intersect(wt, tmin, best_t, a, b, c, t, u, v)) {
                    continue;
                }
                if (kAny) {
                    occluded = true;
                    return;
                }
                const uint32_t prim = __float_as_uint(a.w);
                // t <= best_t here; equal t goes to the smaller (inst, prim)
                if (t < best_t || cur_inst < best_inst || (cur_inst == best_inst && prim < best_prim)) {
                    best_t = t;
                    best_u = u;
                    best_v = v;
                    best_inst = cur_inst;
                    best_prim = prim;
                }
            }
        } else {
            while (Gt.y) {  // enter the first eligible instance; the rest stays on the stack
                const uint32_t k = __ffs(Gt.y) - 1u;
                Gt.y &= Gt.y - 1u;
                const uint4 *ip = reinterpret_cast<const uint4 *>(insts + Gt.x + k);
                const uint4 m4 = __ldg(ip + 4);  // fnodes (x,y), inst id (z), mask (w)
                uint32_t vis = m4.w;
                if (vis & (kInstProcedural | kInstMotion | kInstCurve)) {
                    if (vis & kInstProcedural) continue;  // procedural primitives: RayQuery only
                    vis >>= 8;                            // curve and motion instances: mask in bits 8..15
                }
                if ((vis & mask) == 0u) continue;
                float4 r0 = __ldg(reinterpret_cast<const float4 *>(ip));
                float4 r1 = __ldg(reinterpret_cast<const float4 *>(ip + 1));
                float4 r2 = __ldg(reinterpret_cast<const float4 *>(ip + 2));
                if (m4.w & kInstMotion) {  // the matrix at the ray's time, inverted as a static one is
                    const W2O x = moving_w2o(r0, time);
                    if (!x.ok) continue;  // vanished at this time
                    r0 = x.r0;
                    r1 = x.r1;
                    r2 = x.r2;
                }
                const float w[12] = {r0.x, r0.y, r0.z, r0.w, r1.x, r1.y, r1.z, r1.w, r2.x, r2.y, r2.z, r2.w};
                const uint4 pp = __ldg(ip + 3);  // qnodes (x,y), tris (z,w)
                if (Gt.y) push(Gt);
                if (G.y) push(G);
                transform_point(w, wox, woy, woz, ox, oy, oz);
                transform_dir(w, wdx, wdy, wdz, dx, dy, dz);
                ix = slab_rcp(dx);
                iy = slab_rcp(dy);
                iz = slab_rcp(dz);
                octinv = octant_inv(dx, dy, dz);
                wt = wt_setup(ox, oy, oz, dx, dy, dz);
                blas = reinterpret_cast<const Node8Q *>((unsigned long long)pp.x | ((unsigned long long)pp.y << 32));
                tris = reinterpret_cast<const TriRec *>((unsigned long long)pp.z | ((unsigned long long)pp.w << 32));
                cur_inst = m4.z;
                in_blas = true;
                blas_sp = sp;
                G = root_group(octinv);
                break;
            }
        }
        if (G.y == 0u) {  // leave a finished BLAS, pop, or finish
            if (in_blas && sp == blas_sp) {
                in_blas = false;
                ox = wox;
                oy = woy;
                oz = woz;
                dx = wdx;
                dy = wdy;
                dz = wdz;
                ix = slab_rcp(wdx);
                iy = slab_rcp(wdy);
                iz = slab_rcp(wdz);
                octinv = octant_inv(wdx, wdy, wdz);
            }
            if (sp == 0) break;
            G = pop();
        }
    }
    hit.inst = best_inst;
    hit.prim = best_prim;
    hit.bary[0] = best_u;
    hit.bary[1] = best_v;
    hit.committed_ray_t = best_t;
    hit._pad = 0u;
}

}  // namespace detail

// Closest hit of `ray` against the accel of `view`: the record lcx_trace_closest
// writes for it (miss: {~0u, ~0u, (0, 0), t_max}).  `mask`: instances with
// (mask & instance mask) == 0 are skipped.  The short stack lives in local memory.
__device__ __forceinline__ LcxTriangleHit trace_closest(const LcxAccelView &view, const LcxRay &ray,
                                                        uint32_t mask = 0xffu) {
    uint2 local[8];
    LcxTriangleHit h;
    bool occ;
    detail::trace_walk<false, 8>(view, ray, 0.0f, mask, ShortStack{local, 1u}, h, occ);
    return h;
}

// Whether `ray` hits anything in [t_min, t_max] (lcx_trace_any).
__device__ __forceinline__ bool trace_any(const LcxAccelView &view, const LcxRay &ray, uint32_t mask = 0xffu) {
    uint2 local[8];
    LcxTriangleHit h;
    bool occ;
    detail::trace_walk<true, 8>(view, ray, 0.0f, mask, ShortStack{local, 1u}, h, occ);
    return occ;
}

// The same with a time per ray (lcx_trace_closest_motion / _any_motion): moving
// instances and keyframed meshes and curves at `time`.
__device__ __forceinline__ LcxTriangleHit trace_closest_motion(const LcxAccelView &view, const LcxRay &ray, float time,
                                                               uint32_t mask = 0xffu) {
    uint2 local[8];
    LcxTriangleHit h;
    bool occ;
    detail::trace_walk<false, 8>(view, ray, time, mask, ShortStack{local, 1u}, h, occ);
    return h;
}
__device__ __forceinline__ bool trace_any_motion(const LcxAccelView &view, const LcxRay &ray, float time,
                                                 uint32_t mask = 0xffu) {
    uint2 local[8];
    LcxTriangleHit h;
    bool occ;
    detail::trace_walk<true, 8>(view, ray, time, mask, ShortStack{local, 1u}, h, occ);
    return occ;
}

// With the top kShort stack entries in the caller's shared memory (see ShortStack).
template <int kShort>
__device__ __forceinline__ LcxTriangleHit trace_closest(const LcxAccelView &view, const LcxRay &ray, uint32_t mask,
                                                        ShortStack ss, float time = 0.0f) {
    LcxTriangleHit h;
    bool occ;
    detail::trace_walk<false, kShort>(view, ray, time, mask, ss, h, occ);
    return h;
}
template <int kShort>
__device__ __forceinline__ bool trace_any(const LcxAccelView &view, const LcxRay &ray, uint32_t mask, ShortStack ss,
                                          float time = 0.0f) {
    LcxTriangleHit h;
    bool occ;
    detail::trace_walk<true, kShort>(view, ray, time, mask, ss, h, occ);
    return occ;
}

}  // namespace lcx
