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
// kernels: committing every candidate gives lcx_trace_closest's records bit
// for bit.  Candidates arrive in traversal order, but the committed result is
// the minimum over committed candidates of (t, inst, prim), so it does not
// depend on that order when the decision depends only on the candidate.
#pragma once

#include "lcx/node_test.cuh"
#include "lcx_accel.h"

namespace lcx {

struct TriangleCandidate {
    uint32_t inst;  // TLAS slot of the instance
    uint32_t prim;  // triangle index in its mesh
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

// One ray against `view`.  `mask`: instances with (mask & instance mask) == 0
// are skipped.  Returns the closest committed hit, or the miss record
// {~0u, ~0u, (0,0), t_max}.
template <class OnCandidate>
__device__ LcxTriangleHit ray_query(const LcxAccelView &view, const LcxRay &ray, uint32_t mask,
                                    OnCandidate &&on_candidate) {
    const Node8Q *tlas = static_cast<const Node8Q *>(view.tlas_nodes);
    const InstRec *insts = static_cast<const InstRec *>(view.instances);
    const float wox = ray.origin[0], woy = ray.origin[1], woz = ray.origin[2];
    const float wdx = ray.direction[0], wdy = ray.direction[1], wdz = ray.direction[2];
    const float tmin = ray.t_min;
    float best_t = ray.t_max, best_u = 0.0f, best_v = 0.0f;
    uint32_t best_inst = kInvalid, best_prim = kInvalid;
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
        if (in_blas) {
            while (Gt.y && !stop) {  // candidate triangles
                const uint32_t k = __ffs(Gt.y) - 1u;
                Gt.y &= Gt.y - 1u;
                const float4 *tp = reinterpret_cast<const float4 *>(tris + Gt.x + k);
                const float4 a = __ldg(tp), b = __ldg(tp + 1), c = __ldg(tp + 2);
                float t, u, v;
                if (!wt_intersect(wt, tmin, best_t, a, b, c, t, u, v)) continue;
                const uint32_t prim = __float_as_uint(a.w);
                const int act = on_candidate(TriangleCandidate{cur_inst, prim, u, v, t});
                if (act == kCommit || act == kCommitAndTerminate) {
                    if (t < best_t || cur_inst < best_inst || (cur_inst == best_inst && prim < best_prim)) {
                        best_t = t;
                        best_u = u;
                        best_v = v;
                        best_inst = cur_inst;
                        best_prim = prim;
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
                if ((m4.w & mask) == 0u) continue;
                const float4 r0 = __ldg(reinterpret_cast<const float4 *>(ip));
                const float4 r1 = __ldg(reinterpret_cast<const float4 *>(ip + 1));
                const float4 r2 = __ldg(reinterpret_cast<const float4 *>(ip + 2));
                const uint4 pp = __ldg(ip + 3);  // qnodes (x,y), tris (z,w)
                if (Gt.y && sp < kStackSize) stk[sp++] = Gt;
                if (G.y && sp < kStackSize) stk[sp++] = G;
                const float w[12] = {r0.x, r0.y, r0.z, r0.w, r1.x, r1.y, r1.z, r1.w, r2.x, r2.y, r2.z, r2.w};
                float dx, dy, dz;
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
    LcxTriangleHit h;
    h.inst = best_inst;
    h.prim = best_prim;
    h.bary[0] = best_u;
    h.bary[1] = best_v;
    h.committed_ray_t = best_t;
    h._pad = 0u;
    return h;
}

}  // namespace lcx
