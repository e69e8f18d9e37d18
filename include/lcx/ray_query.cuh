// ray_query.cuh — RayQuery for user CUDA kernels: a closest-hit or any-hit
// query whose candidate triangles are accepted or rejected by user code.
//
// The reference's RayQuery (include/luisa/dsl/rtx/ray_query.h:17-240; CPU
// src/rust/luisa_compute_backend_impl/src/cpu/accel.rs:582-800) calls an
// on-surface-candidate callback that may commit the candidate or terminate
// the query (alpha cutout is the usual use, src/tests/test_path_tracing_cutout.cpp).
// The CUDA-native form is a device function template: the callback is a
// functor inlined into the traversal of the user's own kernel.
//
//   #include <lcx/ray_query.cuh>           // include/ of this repository
//   __global__ void k(LcxAccelView v, const LcxRay *rays, LcxTriangleHit *hits) {
//       const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
//       hits[i] = lcx::ray_query(v, rays[i], 0xffu, [&](const lcx::TriangleCandidate &c) {
//           return alpha(c) > 0.5f ? lcx::kCommit : lcx::kSkip;
//       });
//   }
//
// The view comes from lcx_accel_device_view() (include/lcx_accel.h) and stays
// valid until the accel is built again or destroyed.  The walk is one ray per
// thread with a 32-entry local stack, over the 8-bit quantised nodes, with the
// node test, instance transform and watertight triangle test of the trace
// kernels (and their curve test for curve instances): committing every
// candidate gives lcx_trace_closest's records bit for bit.  Candidates arrive in traversal order, but the committed result is
// the minimum over committed candidates of (t, inst, prim), so it does not
// depend on that order when the decision depends only on the candidate.
#pragma once

#include "lcx/node_test.cuh"
#include "lcx_accel.h"

namespace lcx {

// A surface candidate: a triangle, or a curve segment (bary_v = -1, bary_u =
// the curve parameter; the reference's curve convention, hit.h:29-30).
struct TriangleCandidate {
    uint32_t inst;  // TLAS slot of the instance
    uint32_t prim;  // triangle (segment) index in its mesh (curve)
    float bary_u, bary_v;
    float t;        // distance along the ray (world ray parameter)
};

// What the callback returns for a candidate.
enum CandidateAction : int {
    kSkip = 0,                // ignore it
    kCommit = 1,              // commit it (kept if it is the closest committed so far)
    kCommitAndTerminate = 2,  // commit it and end the query (any-hit queries)
    kTerminate = 3            // end the query without committing it
};

// An AABB of a procedural primitive the ray passes through (the reference's
// ProceduralCandidate, ray_query.h:43-66): the callback intersects its own
// primitive and commits a distance.
struct ProceduralCandidate {
    uint32_t inst, prim;
    float aabb_min[3], aabb_max[3];  // object space, as built
    float obj_origin[3], obj_dir[3]; // the ray in the instance's object space (same t as in world space)
    LcxRay ray;                      // the world ray; t_max = the closest committed distance so far
};
struct ProceduralDecision {
    int action;  // CandidateAction
    float t;     // distance committed with kCommit / kCommitAndTerminate; kept iff t_min <= t < ray.t_max
};

// Committed hit of a query with procedural primitives (the reference's
// CommittedHit, cpu_kernel_defs/src/lib.rs:70-76).
enum HitType : uint32_t { kHitMiss = 0, kHitTriangle = 1, kHitProcedural = 2 };
struct CommittedHit {
    uint32_t inst, prim;
    float bary_u, bary_v;  // triangles only
    uint32_t type;         // HitType
    float t;               // t_max of the ray for a miss
};

// One ray against `view`, triangles, curves and procedural primitives.  `mask`:
// instances with (mask & instance mask) == 0 are skipped.  Returns the closest
// committed hit; a miss is {~0u, ~0u, (0,0), kHitMiss, t_max}.  kMotion: the
// ray has a time (the reference's traverse_motion, include/luisa/dsl/rtx/accel.h:49-50):
// motion instances move, keyframed vertices and control points interpolate, with
// the trace kernels' motion arithmetic.  Without it, motion instances and
// keyframed meshes and curves are passed over (view.motion says whether the
// accel has any).
template <bool kMotion, class OnCandidate, class OnProcedural>
__device__ CommittedHit ray_query_core(const LcxAccelView &view, const LcxRay &ray, float time, uint32_t mask,
                                       OnCandidate &&on_candidate, OnProcedural &&on_procedural) {
    const Node8Q *tlas = static_cast<const Node8Q *>(view.tlas_nodes);
    const InstRec *insts = static_cast<const InstRec *>(view.instances);
    const float wox = ray.origin[0], woy = ray.origin[1], woz = ray.origin[2];
    const float wdx = ray.direction[0], wdy = ray.direction[1], wdz = ray.direction[2];
    const float tmin = ray.t_min;
    float best_t = ray.t_max, best_u = 0.0f, best_v = 0.0f;
    uint32_t best_inst = kInvalid, best_prim = kInvalid, best_type = kHitMiss;
    bool cur_proc = false;
    float odx = 0.0f, ody = 0.0f, odz = 0.0f;  // object-space direction of the current instance
    mask &= 0xffu;

    float ox = wox, oy = woy, oz = woz;
    float ix = slab_rcp(wdx), iy = slab_rcp(wdy), iz = slab_rcp(wdz);
    uint32_t octinv = octant_inv(wdx, wdy, wdz);
    WtRay wt{};
    uint2 stk[kStackSize];
    int sp = 0, blas_sp = 0;
    bool in_blas = false;
    uint32_t cur_inst = 0;
    const Node8Q *blas = nullptr;
    const TriRec *tris = nullptr;
    uint2 G = (wdx == 0.0f && wdy == 0.0f && wdz == 0.0f) ? make_uint2(0, 0) : root_group(octinv);
    bool stop = false;

    for (uint32_t steps = 0; steps < (1u << 22) && !stop; steps++) {
        uint2 Gt;
        if (G.y >= 0x01000000u) {  // visit the front child of the node group
            const uint32_t key = __ffs(G.y >> 24) - 1u;
            G.y &= ~(1u << (24 + key));
            const uint32_t slot = key ^ octinv;
            const uint32_t child = G.x + __popc(G.y & 0xffu & ((1u << slot) - 1u));
            if (G.y >= 0x01000000u && sp < kStackSize) stk[sp++] = G;
            intersect_q(in_blas ? blas : tlas, child, ox, oy, oz, ix, iy, iz, octinv, tmin, best_t, G, Gt);
        } else {
            Gt = G;
            G = make_uint2(0, 0);
        }
        if (in_blas && cur_proc) {
            while (Gt.y && !stop) {  // procedural candidates: AABBs the ray passes through
                const uint32_t k = __ffs(Gt.y) - 1u;
                Gt.y &= Gt.y - 1u;
                const float4 *tp = reinterpret_cast<const float4 *>(tris + Gt.x + k);
                const float4 lo = __ldg(tp), hi = __ldg(tp + 1);
                const float tnx = ((ix < 0.0f ? hi.x : lo.x) - ox) * ix, tfx = ((ix < 0.0f ? lo.x : hi.x) - ox) * ix;
                const float tny = ((iy < 0.0f ? hi.y : lo.y) - oy) * iy, tfy = ((iy < 0.0f ? lo.y : hi.y) - oy) * iy;
                const float tnz = ((iz < 0.0f ? hi.z : lo.z) - oz) * iz, tfz = ((iz < 0.0f ? lo.z : hi.z) - oz) * iz;
                const float tn = fmaxf(fmaxf(tnx, tny), fmaxf(tnz, tmin));
                const float tf = fminf(fminf(tfx, tfy), fminf(tfz, best_t));
                if (!slab_accept(tn, tf)) continue;
                ProceduralCandidate pc;
                pc.inst = cur_inst;
                pc.prim = __float_as_uint(lo.w);
                pc.aabb_min[0] = lo.x;
                pc.aabb_min[1] = lo.y;
                pc.aabb_min[2] = lo.z;
                pc.aabb_max[0] = hi.x;
                pc.aabb_max[1] = hi.y;
                pc.aabb_max[2] = hi.z;
                pc.obj_origin[0] = ox;
                pc.obj_origin[1] = oy;
                pc.obj_origin[2] = oz;
                pc.obj_dir[0] = odx;
                pc.obj_dir[1] = ody;
                pc.obj_dir[2] = odz;
                pc.ray = ray;
                pc.ray.t_max = best_t;
                const ProceduralDecision dec = on_procedural(pc);
                if ((dec.action == kCommit || dec.action == kCommitAndTerminate) && dec.t >= tmin && dec.t < best_t) {
                    best_t = dec.t;
                    best_u = best_v = 0.0f;
                    best_inst = cur_inst;
                    best_prim = pc.prim;
                    best_type = kHitProcedural;
                }
                if (dec.action == kCommitAndTerminate || dec.action == kTerminate) stop = true;
            }
        } else if (in_blas) {
            while (Gt.y && !stop) {  // candidate triangles
                const uint32_t k = __ffs(Gt.y) - 1u;
                Gt.y &= Gt.y - 1u;
                const float4 *tp = reinterpret_cast<const float4 *>(tris + Gt.x + k);
                float4 a = __ldg(tp), b = __ldg(tp + 1), c = __ldg(tp + 2);
                float t, u, v;
                const uint32_t marker = __float_as_uint(b.w);
                if (marker == kTriCurve || marker == kTriCurveMotion) {  // a cone of a curve: the trace kernels' test
                    float4 c0 = make_float4(a.x, a.y, a.z, c.x), c1 = make_float4(b.x, b.y, b.z, c.y);
                    if (marker == kTriCurveMotion && (!kMotion || !curve_motion_cone(a, b, c, time, c0, c1))) continue;
                    const uint32_t kn = __float_as_uint(c.z);
                    if (!curve_piece_entry(make_float3(ox, oy, oz), make_float3(odx, ody, odz), c0, c1, kn & 0xffffu,
                                           kn >> 16, __float_as_uint(c.w), tmin, best_t, t, u))
                        continue;
                    v = -1.0f;
                } else {
                    if (marker == kTriMotion) {  // keyframed vertices: the triangle at the ray's time
                        if (!kMotion) continue;
                        const MeshMotion *mm = reinterpret_cast<const MeshMotion *>(
                            (unsigned long long)__float_as_uint(c.x) | ((unsigned long long)__float_as_uint(c.y) << 32));
                        if (!motion_triangle(*mm, __float_as_uint(a.w), time, a, b, c)) continue;
                    }
                    if (!wt_intersect(wt, tmin, best_t, a, b, c, t, u, v)) continue;
                }
                const uint32_t prim = __float_as_uint(a.w);
                const int act = on_candidate(TriangleCandidate{cur_inst, prim, u, v, t});
                if (act == kCommit || act == kCommitAndTerminate) {
                    if (t < best_t || cur_inst < best_inst || (cur_inst == best_inst && prim < best_prim)) {
                        best_t = t;
                        best_u = u;
                        best_v = v;
                        best_inst = cur_inst;
                        best_prim = prim;
                        best_type = kHitTriangle;
                    }
                }
                if (act == kCommitAndTerminate || act == kTerminate) stop = true;
            }
        } else {
            while (Gt.y) {  // enter the first eligible instance; the rest stays on the stack
                const uint32_t k = __ffs(Gt.y) - 1u;
                Gt.y &= Gt.y - 1u;
                const uint4 *ip = reinterpret_cast<const uint4 *>(insts + Gt.x + k);
                const uint4 m4 = __ldg(ip + 4);  // fnodes (x,y), inst id (z), mask (w)
                const bool proc = (m4.w & kInstProcedural) != 0u;
                // mask in bits 8..15
                const bool shifted = (m4.w & (kInstProcedural | kInstCurve | kInstMotion)) != 0u;
                const bool moving = !proc && (m4.w & kInstMotion) != 0u;
                if ((((shifted ? m4.w >> 8 : m4.w) & 0xffu) & mask) == 0u) continue;
                if (moving && !kMotion) continue;
                const float4 r0 = __ldg(reinterpret_cast<const float4 *>(ip));
                const float4 r1 = __ldg(reinterpret_cast<const float4 *>(ip + 1));
                const float4 r2 = __ldg(reinterpret_cast<const float4 *>(ip + 2));
                float w[12] = {r0.x, r0.y, r0.z, r0.w, r1.x, r1.y, r1.z, r1.w, r2.x, r2.y, r2.z, r2.w};
                if (kMotion && moving) {  // the matrix at the ray's time, inverted as a static one is
                    const MotionDesc *md = reinterpret_cast<const MotionDesc *>(
                        (unsigned long long)__float_as_uint(r0.x) | ((unsigned long long)__float_as_uint(r0.y) << 32));
                    float m[12];
                    if (!motion_matrix(*md, time, m)) continue;  // vanished at this time
                    affine_inverse(m, w);
                }
                const uint4 pp = __ldg(ip + 3);  // qnodes (x,y), tris (z,w)
                if (Gt.y && sp < kStackSize) stk[sp++] = Gt;
                if (G.y && sp < kStackSize) stk[sp++] = G;
                float dx, dy, dz;
                transform_point(w, wox, woy, woz, ox, oy, oz);
                transform_dir(w, wdx, wdy, wdz, dx, dy, dz);
                ix = slab_rcp(dx);
                iy = slab_rcp(dy);
                iz = slab_rcp(dz);
                octinv = octant_inv(dx, dy, dz);
                wt = wt_setup(ox, oy, oz, dx, dy, dz);
                odx = dx;
                ody = dy;
                odz = dz;
                cur_proc = proc;
                blas = reinterpret_cast<const Node8Q *>((unsigned long long)pp.x | ((unsigned long long)pp.y << 32));
                tris = reinterpret_cast<const TriRec *>((unsigned long long)pp.z | ((unsigned long long)pp.w << 32));
                cur_inst = m4.z;
                in_blas = true;
                blas_sp = sp;
                G = root_group(octinv);
                break;
            }
        }
        if (G.y == 0u && !stop) {  // leave a finished BLAS, pop, or finish
            if (in_blas && sp == blas_sp) {
                in_blas = false;
                ox = wox;
                oy = woy;
                oz = woz;
                ix = slab_rcp(wdx);
                iy = slab_rcp(wdy);
                iz = slab_rcp(wdz);
                octinv = octant_inv(wdx, wdy, wdz);
            }
            if (sp == 0) break;
            G = stk[--sp];
        }
    }
    CommittedHit h;
    h.inst = best_inst;
    h.prim = best_prim;
    h.bary_u = best_u;
    h.bary_v = best_v;
    h.type = best_type;
    h.t = best_t;
    return h;
}

template <class OnCandidate, class OnProcedural>
__device__ CommittedHit ray_query(const LcxAccelView &view, const LcxRay &ray, uint32_t mask,
                                  OnCandidate &&on_candidate, OnProcedural &&on_procedural) {
    return ray_query_core<false>(view, ray, 0.0f, mask, on_candidate, on_procedural);
}

// With a time per ray (motion blur): moving instances and keyframed meshes and
// curves at `time`, as lcx_trace_closest_motion traces them.
template <class OnCandidate, class OnProcedural>
__device__ CommittedHit ray_query_motion(const LcxAccelView &view, const LcxRay &ray, float time, uint32_t mask,
                                         OnCandidate &&on_candidate, OnProcedural &&on_procedural) {
    return ray_query_core<true>(view, ray, time, mask, on_candidate, on_procedural);
}

namespace detail {
inline __device__ LcxTriangleHit surface_hit(const CommittedHit &c) {
    LcxTriangleHit h;
    h.inst = c.inst;
    h.prim = c.prim;
    h.bary[0] = c.bary_u;
    h.bary[1] = c.bary_v;
    h.committed_ray_t = c.t;
    h._pad = 0u;
    return h;
}
}  // namespace detail

// Surfaces only (procedural instances are passed over): the TriangleHit
// record of the closest committed triangle or curve.
template <class OnCandidate>
__device__ LcxTriangleHit ray_query(const LcxAccelView &view, const LcxRay &ray, uint32_t mask,
                                    OnCandidate &&on_candidate) {
    return detail::surface_hit(ray_query(view, ray, mask, on_candidate, [](const ProceduralCandidate &) {
        return ProceduralDecision{kSkip, 0.0f};
    }));
}
template <class OnCandidate>
__device__ LcxTriangleHit ray_query_motion(const LcxAccelView &view, const LcxRay &ray, float time, uint32_t mask,
                                           OnCandidate &&on_candidate) {
    return detail::surface_hit(ray_query_motion(view, ray, time, mask, on_candidate, [](const ProceduralCandidate &) {
        return ProceduralDecision{kSkip, 0.0f};
    }));
}

}  // namespace lcx
