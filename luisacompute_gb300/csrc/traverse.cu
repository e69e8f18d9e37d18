// traverse.cu — trace_closest / trace_any over 8-wide BVHs on sm_103a.
//
// Replaces the per-ray OptiX hit-object traversal of the CUDA backend
// (src/backends/cuda/cuda_builtin/cuda_device_resource.h:1742-1829) and the
// per-ray Embree rtcIntersect1 / rtcOccluded1 calls of the CPU backend
// (src/rust/luisa_compute_backend_impl/src/cpu/accel.rs:449-535) with one
// batched kernel:
//   * persistent warps: each warp takes rays from a global counter and, after
//     every traversal step, refills its idle lanes once at least P.refill of
//     them have finished (dynamic ray fetch, Aila & Laine 2009);
//   * a lane whose triangles would be tested by fewer than P.postpone lanes
//     pushes them and keeps walking nodes (postponing, Ylitie et al. 2017);
//   * node groups: a visited node yields the hit mask of its internal
//     children (bits ordered front to back by the ray octant) and the hit
//     mask of its leaf items; a group with hits left is pushed on a per-thread
//     short stack: the top kShortStack entries (8 B each) per thread in shared
//     memory, deeper ones in local memory;
//   * two levels: a TLAS leaf item is an instance; the ray is moved to object
//     space with the exact FP32 sequence of lcx/bvh_device.cuh and the same loop
//     runs over the BLAS; when the stack unwinds to the entry depth the world
//     ray is restored;
//   * 128-bit read-only loads of nodes (5 for Node8Q, 13 for Node8F) and
//     triangles (3 per triangle);
//   * closest hit keeps (t, inst, prim) minimal, so the answer is independent
//     of traversal order; any hit stops at the first accepted triangle.
#include "lcx_internal.h"
#include "lcx/node_test.cuh"
#include "lcx/trace.cuh"

namespace lcx {
namespace {

constexpr int kTraceBlock = 128;
// Resident 128-thread blocks per SM the register budget is cut for (measured
// on GB300, terrain workload: quantised nodes peak at 7 -- 8 spills and drops
// 1.77 -> 1.65 Grays/s -- and FP32 nodes at 7, 1.61 -> 1.62 over 6).
#ifndef LCX_TRACE_MIN_BLOCKS_Q
#define LCX_TRACE_MIN_BLOCKS_Q 7
#endif
#ifndef LCX_PER_THREAD_MIN_BLOCKS
// loop mode 3 (one ray per thread): terrain workload closest / any Grays/s 1.004 / 2.45 at 7 blocks per
// SM (72 registers, 188 bytes spilled), 1.004 / 2.48 at 6, 1.001 / 2.32 at 5 (96 registers), 0.87 at 4
#define LCX_PER_THREAD_MIN_BLOCKS 7
#endif
#ifndef LCX_TRACE_MIN_BLOCKS_F
#define LCX_TRACE_MIN_BLOCKS_F 7
#endif
// The curve kernels carry the curve test and the motion interpolation: 5 blocks
// per SM (96 registers) keeps the quantised-node ones from spilling; measured
// on the hair workload (Catmull-Rom, camera rays): 5 blocks 0.902, 6 blocks
// (8 bytes spilled) 0.911, 7 blocks 0.893 Grays/s; 4 blocks were 11 % slower.
#ifndef LCX_TRACE_MIN_BLOCKS_EXT
#define LCX_TRACE_MIN_BLOCKS_EXT 5
#endif
// Stack entries kept in shared memory per thread (the rest of the kStackSize
// entries go to local memory): a launch-time choice among 8, 16 (default) and
// 24 for the single-job closest / any kernels; 16 for the others.
constexpr int kDefaultShortStack = 16;

// Loop mode 0 with the triangle tests spread over the warp (coop_triangles):
// results identical, but measured slower on GB300 (terrain workload, closest
// hit 1.78 -> 1.56 Grays/s): with ~4 pending triangles per warp-step, the
// prefix scan, owner search and shuffles cost what the one or two divergent
// iterations they replace cost.  Off.
#ifndef LCX_COOP_TRIS
#define LCX_COOP_TRIS 0
#endif
// Measured without effect on the terrain workload, so off: loading an instance record's rows before
// its mask test (one round trip instead of two: 1.975 -> 1.965 Grays/s) and the triangle-queue
// prefix from one ballot per bit instead of a shuffle scan (1.975 -> 1.961).
#ifndef LCX_INST_LOADS_FIRST
#define LCX_INST_LOADS_FIRST 0
#endif
#ifndef LCX_QUEUE_BALLOT
#define LCX_QUEUE_BALLOT 0
#endif
// Deferred kernel: ray ids a warp takes from the global counter at a time (0 = just its idle lanes'
// count), the chunk's rays prefetched into L2 when it is taken.  Measured on the terrain workload
// (closest / any Grays/s): 0: 1.975 / 3.34; 32: 2.023 / 3.45; 64: 2.025 / 3.47; 128: 1.996 / 3.45
// (the end of the launch waits on the larger chunks).
// Deferred kernel: an instance entry records the object-space ray and the flush sets up the
// watertight test per queued entry (1), or the entry sets it up and records it (0).  The entry runs
// with a few lanes in nearly every step, the flush with all of them: 2.035 -> 2.12 Grays/s on the
// terrain workload (any hit 3.48 -> 3.55), same records.
#ifndef LCX_WT_AT_FLUSH
#define LCX_WT_AT_FLUSH 1
#endif
#ifndef LCX_RAY_CHUNK
#define LCX_RAY_CHUNK 64
#endif
#ifndef LCX_PREFETCH
#define LCX_PREFETCH 0  // 1: prefetch the next node into L1 (measured: 1.77 -> 1.66 Grays/s, so off)
#endif

// Per-lane traversal state and the operations both loop structures share.
// kMulti: the launch serves several jobs (scenes); each lane takes its job's
// TLAS, instance table, mask and buffers when it takes a ray.
// kExt: the extended kernels.  1: accels with motion instances or vertex-motion
// meshes (each ray has a time); 2: also curves (curve segments get the curve test,
// with a larger register budget).
// kNoWt: the caller tests triangles from its own ray records (the deferred kernel): an instance
// entry keeps the object-space direction instead of setting up the watertight test.
template <int kLayout, bool kAny, bool kCount, bool kMulti, int kShort, int kExt = 0, bool kNoWt = false>
struct Walker {
    static constexpr int kShortStack = kShort < kStackSize ? kShort : kStackSize;
    static constexpr int kDeep = kStackSize - kShortStack;    // entries in local memory
    static constexpr int kDeepSlots = kDeep > 0 ? kDeep : 1;  // array size (1 when unused)

    const TraceParams &P;
    uint2 *stk;
    const void *tlas_nodes;
    const InstRec *insts;
    const Ray *rays;
    void *out;
    uint32_t mask;
    uint32_t slot = 0;  // ray index within its job
    // world ray
    float wox = 0, woy = 0, woz = 0, wdx = 0, wdy = 0, wdz = 1;
    float tmin = 0, best_t = 0, best_u = 0, best_v = 0;
    float time = 0;  // motion launches: the ray's time
    uint32_t best_inst = kInvalid, best_prim = kInvalid;
    // current-space ray (world at the TLAS level, object inside a BLAS)
    float ox = 0, oy = 0, oz = 0, ix = 1, iy = 1, iz = 1;
    float rdx = 0, rdy = 0, rdz = 1;  // current-space direction (read by the curve test only)
    uint32_t octinv = 0;
    WtRay wt{};
    uint2 G = make_uint2(0, 0);
    int sp = 0, blas_sp = 0;
    bool in_blas = false, occluded = false;
    uint32_t cur_inst = 0;
    const void *blas_nodes = nullptr;
    const TriRec *blas_tris = nullptr;
    uint32_t c_nodes = 0, c_tris = 0, c_insts = 0;

    __device__ Walker(const TraceParams &p, uint2 *s, uint2 *d)
        : P(p), stk(s), deep(d),
          tlas_nodes(kLayout == LCX_NODES_QUANT8 ? static_cast<const void *>(p.tlas_q)
                                                 : static_cast<const void *>(p.tlas_f)),
          insts(p.insts), rays(p.rays),
          out(kAny ? static_cast<void *>(p.occluded) : static_cast<void *>(p.hits)), mask(p.mask) {}

    uint2 *deep;  // local-memory overflow (an array of the kernel, not of this struct,
                  // so that the struct itself stays in registers)

    // Every index below is clamped into its array as well as branched on, so a
    // load the compiler hoists out of the untaken branch stays in bounds.
    __device__ __forceinline__ void push(uint2 v) {
        if (sp < kShortStack) {
            stk[min(sp, kShortStack - 1) * kTraceBlock] = v;
            sp++;
        } else if (kDeep > 0 && sp < kStackSize) {
            deep[min(max(sp - kShortStack, 0), kDeepSlots - 1)] = v;
            sp++;
        } else {
            atomicOr(P.pool + 1, 1u);  // cannot happen within the host's depth check
        }
    }
    __device__ __forceinline__ uint2 pop() {
        sp--;
        if (kDeep == 0 || sp < kShortStack) return stk[min(max(sp, 0), kShortStack - 1) * kTraceBlock];
        return deep[min(max(sp - kShortStack, 0), kDeepSlots - 1)];
    }

    __device__ __forceinline__ void start(uint32_t rid) {
        slot = rid;
        const float *times = P.times;
        if (kMulti) {  // job of global ray rid: last job whose first ray is <= rid
            uint32_t lo = 0, hi = P.job_count - 1;
            while (lo < hi) {
                const uint32_t mid = (lo + hi + 1) >> 1;
                if (__ldg(&P.jobs[mid].first) <= rid)
                    lo = mid;
                else
                    hi = mid - 1;
            }
            const DevJob &j = P.jobs[lo];
            tlas_nodes = kLayout == LCX_NODES_QUANT8 ? static_cast<const void *>(j.tlas_q)
                                                     : static_cast<const void *>(j.tlas_f);
            insts = j.insts;
            rays = j.rays;
            out = j.out;
            mask = j.mask;
            times = j.times;
            slot = rid - j.first;
        }
        else if (P.order != nullptr) {
            slot = __ldg(P.order + rid);
        }
        const float4 *rp = reinterpret_cast<const float4 *>((kMulti ? rays : P.rays) + slot);
        const float4 r0 = __ldcs(rp), r1 = __ldcs(rp + 1);
        wox = r0.x;
        woy = r0.y;
        woz = r0.z;
        tmin = r0.w;
        wdx = r1.x;
        wdy = r1.y;
        wdz = r1.z;
        best_t = r1.w;
        if (kExt) time = times != nullptr ? __ldg(times + slot) : 0.0f;
        best_u = best_v = 0.0f;
        best_inst = best_prim = kInvalid;
        to_world();
        // a zero direction meets nothing; skip the walk
        G = (wdx == 0.0f && wdy == 0.0f && wdz == 0.0f) ? make_uint2(0, 0) : root_group(octinv);
        sp = 0;
        in_blas = false;
        occluded = false;
        if (kCount) c_nodes = c_tris = c_insts = 0;
    }

    __device__ __forceinline__ void to_world() {
        ox = wox;
        oy = woy;
        oz = woz;
        ix = slab_rcp(wdx);
        iy = slab_rcp(wdy);
        iz = slab_rcp(wdz);
        octinv = octant_inv(wdx, wdy, wdz);
        if (kExt >= 2) {
            rdx = wdx;
            rdy = wdy;
            rdz = wdz;
        }
    }

    // Take the front child of node group G, push the rest, intersect it.
    __device__ __forceinline__ void visit(uint2 &Gt) {
        const uint32_t key = __ffs(G.y >> 24) - 1u;
        G.y &= ~(1u << (24 + key));
        const uint32_t slot = key ^ octinv;
        const uint32_t child = G.x + __popc(G.y & 0xffu & ((1u << slot) - 1u));
        if (G.y >= 0x01000000u) push(G);
        const void *nodes = in_blas ? blas_nodes : tlas_nodes;
        if (kLayout == LCX_NODES_QUANT8)
            intersect_q(static_cast<const Node8Q *>(nodes), child, ox, oy, oz, ix, iy, iz, octinv, tmin, best_t, G,
                        Gt);
        else
            intersect_f(static_cast<const Node8F *>(nodes), child, ox, oy, oz, ix, iy, iz, octinv, tmin, best_t, G,
                        Gt);
        if (kCount) c_nodes++;
#if LCX_PREFETCH
        if (G.y >= 0x01000000u) {  // the node the next step visits: the front child of G
            const uint32_t nkey = __ffs(G.y >> 24) - 1u;
            const uint32_t nslot = nkey ^ octinv;
            const uint32_t next = G.x + __popc(G.y & 0xffu & ((1u << nslot) - 1u));
            const char *np = kLayout == LCX_NODES_QUANT8
                                 ? reinterpret_cast<const char *>(static_cast<const Node8Q *>(nodes) + next)
                                 : reinterpret_cast<const char *>(static_cast<const Node8F *>(nodes) + next);
            asm volatile("prefetch.global.L1 [%0];" ::"l"(np));
            asm volatile("prefetch.global.L1 [%0];" ::"l"(np + (kLayout == LCX_NODES_QUANT8 ? 79 : 207)));
        }
#endif
    }

    // Test the triangles of Gt (inside a BLAS).  Returns true if trace_any is done.
    __device__ __forceinline__ bool triangles(uint2 Gt) {
        while (Gt.y) {
            const uint32_t k = __ffs(Gt.y) - 1u;
            Gt.y &= Gt.y - 1u;
            const float4 *tp = reinterpret_cast<const float4 *>(blas_tris + Gt.x + k);
            float4 a = bvh_ld(tp), b = bvh_ld(tp + 1), c = bvh_ld(tp + 2);
            if constexpr (kExt >= 2) {
                const uint32_t marker = __float_as_uint(b.w);
                if (marker == kTriCurve || marker == kTriCurveMotion) {  // a cone of a curve segment
                    if (kCount) c_tris++;
                    float4 c0 = make_float4(a.x, a.y, a.z, c.x), c1 = make_float4(b.x, b.y, b.z, c.y);
                    if (marker == kTriCurveMotion && !curve_motion_cone(a, b, c, time, c0, c1)) continue;
                    const uint32_t kn = __float_as_uint(c.z);
                    float t, u;
                    if (curve_piece_entry(make_float3(ox, oy, oz), make_float3(rdx, rdy, rdz), c0, c1, kn & 0xffffu,
                                          kn >> 16, __float_as_uint(c.w), tmin, best_t, t, u)) {
                        if (kAny) {
                            occluded = true;
                            return true;
                        }
                        const uint32_t prim = __float_as_uint(a.w);
                        if (t < best_t || cur_inst < best_inst || (cur_inst == best_inst && prim < best_prim)) {
                            best_t = t;
                            best_u = u;
                            best_v = -1.0f;
                            best_inst = cur_inst;
                            best_prim = prim;
                        }
                    }
                    continue;
                }
            }
            if constexpr (kExt >= 1) {
                if (__float_as_uint(b.w) == kTriMotion) {  // a vertex-motion mesh: its triangle at the ray's time
                    const MeshMotion *mm = reinterpret_cast<const MeshMotion *>(
                        (unsigned long long)__float_as_uint(c.x) | ((unsigned long long)__float_as_uint(c.y) << 32));
                    if (!motion_triangle(*mm, __float_as_uint(a.w), time, a, b, c)) continue;
                }
            }
            if (kCount) c_tris++;
            float t, u, v;
            if (wt_intersect(wt, tmin, best_t, a, b, c, t, u, v)) {
                if (kAny) {
                    occluded = true;
                    return true;
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
        }
        return false;
    }

    // Triangle tests spread over the whole warp.  Every lane of the warp calls
    // this together; a lane with `has` owns the triangles of its group Gt.
    // Task j (in lane order of the owners) goes to lane j mod 32, which takes
    // the owner's ray, interval and triangle pointer by shuffles.  Each owner's
    // hits are reduced in shared memory by one 64-bit atomicMin over
    // (ordered t, prim): all of an owner's triangles belong to its current
    // instance, so this minimum followed by the usual update rule gives the
    // same record as testing them one by one.  Returns true for an owner whose
    // any-hit query found a hit.
    __device__ __forceinline__ bool coop_triangles(uint2 Gt, bool has, uint32_t lane, unsigned long long *keys,
                                                   float2 *uvs) {
        const uint32_t cnt = has ? __popc(Gt.y) : 0u;
        const uint32_t owners = __ballot_sync(~0u, cnt != 0u);
        if (owners == 0u) return false;
        if (kCount) c_tris += cnt;
        uint32_t incl = cnt;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t v = __shfl_up_sync(~0u, incl, o);
            if (lane >= uint32_t(o)) incl += v;
        }
        const uint32_t total = __shfl_sync(~0u, incl, 31);
        const uint32_t excl = incl - cnt;
        const uint32_t wbase = threadIdx.x & ~31u;
        if (cnt) keys[threadIdx.x] = ~0ull;
        __syncwarp();
        for (uint32_t r0 = 0; r0 < total; r0 += 32) {
            const uint32_t j = r0 + lane;
            uint32_t own = 0, k = 0;
            bool work = false;
            for (uint32_t rem = owners; rem; rem &= rem - 1u) {
                const uint32_t o = __ffs(rem) - 1u;
                const uint32_t oe = __shfl_sync(~0u, excl, o), oc = __shfl_sync(~0u, cnt, o);
                if (j >= oe && j < oe + oc) {
                    own = o;
                    k = j - oe;
                    work = true;
                }
            }
            WtRay r;
            r.ox = __shfl_sync(~0u, wt.ox, own);
            r.oy = __shfl_sync(~0u, wt.oy, own);
            r.oz = __shfl_sync(~0u, wt.oz, own);
            r.Sx = __shfl_sync(~0u, wt.Sx, own);
            r.Sy = __shfl_sync(~0u, wt.Sy, own);
            r.Sz = __shfl_sync(~0u, wt.Sz, own);
            r.perm = __shfl_sync(~0u, wt.perm, own);
            const float lo = __shfl_sync(~0u, tmin, own), hi = __shfl_sync(~0u, best_t, own);
            const uint32_t gx = __shfl_sync(~0u, Gt.x, own), gy = __shfl_sync(~0u, Gt.y, own);
            const unsigned long long tp =
                __shfl_sync(~0u, static_cast<unsigned long long>(reinterpret_cast<uintptr_t>(blas_tris)), own);
            unsigned long long key = ~0ull;
            float t = 0.0f, u = 0.0f, v = 0.0f;
            if (work) {
                const uint32_t bit = __fns(gy, 0u, int(k) + 1);  // k-th set bit of the owner's group
                const float4 *q = reinterpret_cast<const float4 *>(reinterpret_cast<const TriRec *>(tp) + gx + bit);
                const float4 a = bvh_ld(q), b = bvh_ld(q + 1), c = bvh_ld(q + 2);
                if (wt_intersect(r, lo, hi, a, b, c, t, u, v)) {
                    key = kAny ? 0ull
                               : (static_cast<unsigned long long>(float_to_ordered(t)) << 32) | __float_as_uint(a.w);
                    atomicMin(&keys[wbase + own], key);
                }
            }
            if (!kAny) {
                __syncwarp();
                if (key != ~0ull && key == keys[wbase + own]) uvs[wbase + own] = make_float2(u, v);
                __syncwarp();
            }
        }
        __syncwarp();
        if (!cnt) return false;
        const unsigned long long best = keys[threadIdx.x];
        if (best == ~0ull) return false;
        if (kAny) {
            occluded = true;
            return true;
        }
        const float bt = ordered_to_float(uint32_t(best >> 32));
        const uint32_t prim = uint32_t(best);
        if (bt < best_t || cur_inst < best_inst || (cur_inst == best_inst && prim < best_prim)) {
            const float2 uv = uvs[threadIdx.x];
            best_t = bt;
            best_u = uv.x;
            best_v = uv.y;
            best_inst = cur_inst;
            best_prim = prim;
        }
        return false;
    }

    // Enter the first eligible instance of Gt (TLAS level); pushes the rest.
    __device__ __forceinline__ void instances(uint2 Gt) {
        while (Gt.y) {
            const uint32_t k = __ffs(Gt.y) - 1u;
            Gt.y &= Gt.y - 1u;
            const uint4 *ip = reinterpret_cast<const uint4 *>((kMulti ? insts : P.insts) + Gt.x + k);
            const uint4 m4 = bvh_ld(ip + 4);  // fnodes (x,y), inst_id (z), mask (w)
            float w[12];
            if constexpr (!kExt) {
#if LCX_INST_LOADS_FIRST
                // the whole record in one round trip, before the mask test (a masked-out instance wastes it)
                const float4 r0 = bvh_ld(reinterpret_cast<const float4 *>(ip));
                const float4 r1 = bvh_ld(reinterpret_cast<const float4 *>(ip + 1));
                const float4 r2 = bvh_ld(reinterpret_cast<const float4 *>(ip + 2));
                if ((m4.w & (kMulti ? mask : P.mask)) == 0u) continue;
#else
                if ((m4.w & (kMulti ? mask : P.mask)) == 0u) continue;
                const float4 r0 = bvh_ld(reinterpret_cast<const float4 *>(ip));
                const float4 r1 = bvh_ld(reinterpret_cast<const float4 *>(ip + 1));
                const float4 r2 = bvh_ld(reinterpret_cast<const float4 *>(ip + 2));
#endif
                w[0] = r0.x, w[1] = r0.y, w[2] = r0.z, w[3] = r0.w;
                w[4] = r1.x, w[5] = r1.y, w[6] = r1.z, w[7] = r1.w;
                w[8] = r2.x, w[9] = r2.y, w[10] = r2.z, w[11] = r2.w;
            } else {  // a motion instance: the matrix at the ray's time, inverted as a static one is
                uint32_t vis = m4.w;
                // motion and curve instances hold their mask in bits 8..15; procedural ones stay
                // unreachable (bit 31 and a shifted mask)
                const bool shifted = (vis & kInstProcedural) == 0u && (vis & (kInstMotion | kInstCurve)) != 0u;
                const bool moving = shifted && (vis & kInstMotion) != 0u;
                if (shifted) vis = (vis >> 8) & 0xffu;
                if ((vis & (kMulti ? mask : P.mask)) == 0u) continue;
                const float4 r0 = bvh_ld(reinterpret_cast<const float4 *>(ip));
                const float4 r1 = bvh_ld(reinterpret_cast<const float4 *>(ip + 1));
                const float4 r2 = bvh_ld(reinterpret_cast<const float4 *>(ip + 2));
                w[0] = r0.x, w[1] = r0.y, w[2] = r0.z, w[3] = r0.w;
                w[4] = r1.x, w[5] = r1.y, w[6] = r1.z, w[7] = r1.w;
                w[8] = r2.x, w[9] = r2.y, w[10] = r2.z, w[11] = r2.w;
                if (moving) {
                    const MotionDesc *md = reinterpret_cast<const MotionDesc *>(
                        (unsigned long long)__float_as_uint(r0.x) |
                        ((unsigned long long)__float_as_uint(r0.y) << 32));
                    float m[12];
                    if (!motion_matrix(*md, time, m)) continue;  // vanished at this time
                    affine_inverse(m, w);
                }
            }
            const uint4 pp = bvh_ld(ip + 3);  // qnodes (x,y), tris (z,w)
            if (Gt.y) push(Gt);
            if (G.y) push(G);
            float dx, dy, dz;
            transform_point(w, wox, woy, woz, ox, oy, oz);
            transform_dir(w, wdx, wdy, wdz, dx, dy, dz);
            ix = slab_rcp(dx);
            iy = slab_rcp(dy);
            iz = slab_rcp(dz);
            octinv = octant_inv(dx, dy, dz);
            if constexpr (!kNoWt) wt = wt_setup(ox, oy, oz, dx, dy, dz);
            if (kExt >= 2 || kNoWt) {
                rdx = dx;
                rdy = dy;
                rdz = dz;
            }
            const unsigned long long qptr = (unsigned long long)pp.x | ((unsigned long long)pp.y << 32);
            const unsigned long long fptr = (unsigned long long)m4.x | ((unsigned long long)m4.y << 32);
            const unsigned long long tptr = (unsigned long long)pp.z | ((unsigned long long)pp.w << 32);
            blas_nodes = reinterpret_cast<const void *>(kLayout == LCX_NODES_QUANT8 ? qptr : fptr);
            blas_tris = reinterpret_cast<const TriRec *>(tptr);
            cur_inst = m4.z;
            in_blas = true;
            blas_sp = sp;
            G = root_group(octinv);
            if (kCount) c_insts++;
            return;
        }
    }

    // With no node group left: leave a finished BLAS, pop, or report done.
    __device__ __forceinline__ bool pop_or_done() {
        if (in_blas && sp == blas_sp) {
            in_blas = false;
            to_world();
        }
        if (sp == 0) return true;
        G = pop();
        return false;
    }

    __device__ __forceinline__ void finish() {
        const uint32_t rid = slot;
        if (kAny) {
            (kMulti ? static_cast<uint8_t *>(out) : P.occluded)[rid] = occluded ? 1 : 0;
        } else {
            uint2 *hp = reinterpret_cast<uint2 *>((kMulti ? static_cast<Hit *>(out) : P.hits) + rid);
            __stcs(hp, make_uint2(best_inst, best_prim));
            __stcs(hp + 1, make_uint2(__float_as_uint(best_u), __float_as_uint(best_v)));
            __stcs(hp + 2, make_uint2(__float_as_uint(best_t), 0u));
        }
        store_counts();
    }

    // Visit counters of the counting build (per ray: nodes, triangles tested, instances entered).
    __device__ __forceinline__ void store_counts() {
        if (kCount) {
            P.counts[3ull * slot + 0] = c_nodes;
            P.counts[3ull * slot + 1] = c_tris;
            P.counts[3ull * slot + 2] = c_insts;
        }
    }
};

// kMode 0: each step visits one node and handles its items at once.
// kMode 1: speculative while-while (Aila & Laine 2009): lanes walk nodes
// together; a lane that finds items keeps walking (holding them in Gp) while
// any lane of the warp is still searching, then all lanes handle items.
template <int kLayout, bool kAny, bool kCount, int kMode, bool kMulti, int kShort, int kExt = 0>
__global__ void __launch_bounds__(kTraceBlock, kExt >= 2                     ? LCX_TRACE_MIN_BLOCKS_EXT
                                               : kLayout == LCX_NODES_QUANT8 ? LCX_TRACE_MIN_BLOCKS_Q
                                                                             : LCX_TRACE_MIN_BLOCKS_F)
    k_trace(TraceParams P) {
    using W_t = Walker<kLayout, kAny, kCount, kMulti, kShort, kExt>;
    __shared__ uint2 stack_mem[W_t::kShortStack * kTraceBlock];
#if LCX_COOP_TRIS
    __shared__ unsigned long long coop_keys[kTraceBlock];  // per owner lane: min (ordered t, prim)
    __shared__ float2 coop_uv[kTraceBlock];                 // per owner lane: barycentrics of that minimum
#endif
    uint2 deep_stack[W_t::kDeepSlots];
    const uint32_t lane = threadIdx.x & 31u;
    W_t W(P, stack_mem + threadIdx.x, deep_stack);
    const int refill = int(P.refill);
    const int postpone = int(P.postpone);
    const int postpone_sp = P.postpone_sp;

    bool active = false, exhausted = false;
    uint32_t rid = 0, ray_steps = 0;

    for (;;) {
        // warp-synchronous refill: idle lanes take new rays once enough of them are idle
        const uint32_t idle = __ballot_sync(~0u, !active);
        const int n_idle = __popc(idle);
        if (!exhausted && n_idle >= refill) {
            uint32_t base = 0;
            if (lane == 0) base = atomicAdd(P.pool, uint32_t(n_idle));
            base = __shfl_sync(~0u, base, 0);
            if (uint64_t(base) + uint64_t(n_idle) >= P.ray_count) exhausted = true;
            if (!active) {
                const uint32_t my = base + __popc(idle & ((1u << lane) - 1u));
                if (my < P.ray_count) {
                    rid = my;
                    active = true;
                    ray_steps = 0;
                    W.start(rid);
                }
            }
        }
        if (__ballot_sync(~0u, active) == 0u) {
            if (exhausted) break;
            continue;
        }

        bool done = false;
        if (kMode == 0) {
#if LCX_COOP_TRIS
            // every lane stays in the step: the triangle phase is warp-wide
            uint2 Gt = make_uint2(0, 0);
            bool tri = false;
            if (active) {
                if (++ray_steps > P.max_steps) {
                    atomicOr(P.pool + 1, 2u);
                    done = true;
                } else {
                    if (W.G.y >= 0x01000000u) {
                        W.visit(Gt);
                    } else {
                        Gt = W.G;
                        W.G = make_uint2(0, 0);
                    }
                    if (W.in_blas)
                        tri = Gt.y != 0u;
                    else
                        W.instances(Gt);
                }
            }
            if (W.coop_triangles(Gt, tri, lane, coop_keys, coop_uv)) done = true;
            if (active && !done && W.G.y == 0u) done = W.pop_or_done();
#else
            if (!active) continue;
            if (++ray_steps > P.max_steps) {
                atomicOr(P.pool + 1, 2u);
                done = true;
            } else {
                uint2 Gt;
                if (W.G.y >= 0x01000000u) {
                    W.visit(Gt);
                } else {
                    Gt = W.G;
                    W.G = make_uint2(0, 0);
                }
                if (W.in_blas) {
                    if (postpone > 0 && Gt.y && W.G.y >= 0x01000000u && W.sp < postpone_sp &&
                        int(__popc(__activemask())) < postpone) {
                        W.push(Gt);  // postpone: a lane nearly alone walks on
                    } else if (W.triangles(Gt)) {
                        done = true;
                    }
                } else {
                    W.instances(Gt);
                }
                if (!done && W.G.y == 0u) done = W.pop_or_done();
            }
#endif
        } else {
            // phase A: walk nodes together, postponing found item groups while others search
            uint2 Gt = make_uint2(0, 0), Gp = make_uint2(0, 0);
            if (active && W.G.y < 0x01000000u) {  // a popped item group
                Gt = W.G;
                W.G = make_uint2(0, 0);
            }
            for (;;) {
                const bool has_node = active && W.G.y >= 0x01000000u;
                const bool searching = has_node && Gt.y == 0u;
                if (!__any_sync(~0u, searching)) break;
                if (has_node && (Gt.y == 0u || Gp.y == 0u)) {
                    if (++ray_steps > P.max_steps) {
                        atomicOr(P.pool + 1, 2u);
                        W.G = make_uint2(0, 0);
                        Gt = Gp = make_uint2(0, 0);
                        W.sp = 0;
                        W.blas_sp = 0;
                        continue;
                    }
                    if (Gt.y) {
                        Gp = Gt;
                        Gt = make_uint2(0, 0);
                    }
                    W.visit(Gt);
                }
            }
            if (!active) continue;
            // phase B: items
            if (W.in_blas) {
                if (W.triangles(Gt) || W.triangles(Gp)) done = true;
            } else {
                if (Gp.y) W.push(Gp);  // instance groups: enter one now, the rest later
                W.instances(Gt);
            }
            // phase C: pop
            if (!done && W.G.y == 0u) done = W.pop_or_done();
        }
        if (active && done) {
            W.finish();
            active = false;
        }
    }
}

// ---------------------------------------------------------------------------
// Loop mode 2: deferred triangle batches.
//
// In modes 0 and 1 a lane tests the triangles of a visited node at once.  A
// ray meets about 2 triangles in about 19 steps, so those tests run with a
// couple of the warp's lanes active, and on the incoherent terrain workload
// they take about half of the kernel's time (measured by running every
// triangle test twice: 4.73 -> 6.98 ms; every node test twice: 4.73 -> 4.76).
// Here a lane only queues its triangles: each warp keeps a shared-memory queue
// of (triangle record, ray record) entries and tests them one per lane, 32 at
// a time, once P.postpone of them have gathered (default 32), when the queue
// is full, when a finished ray has no place to wait for its entries, or when
// the warp runs out of rays.
//
// Ray records: each lane has two in shared memory -- its ray in the object
// space of an instance (the watertight-test setup), tmin and the instance id
// -- written when the lane enters an instance, alternating, so that entries of
// the previous instance stay valid.  Entering an instance whose record still
// has queued entries flushes the queue first.
// A ray whose walk ends with entries queued retires into the lane's retire
// slot (its best hit so far) and the lane takes a new ray; the retired ray's
// record is written after the next flush.  A lane whose retire slot is taken
// waits for that flush.
// Results: per ray record, the minimum (ordered t, prim) by a 64-bit
// atomicMin and the barycentrics of that minimum.  The owner merges each
// record's minimum into its ray's best with the closest-hit rule, so the
// result does not depend on the order of the tests.  Entries are tested
// against the ray's best t at the flush, never below the best t an immediate
// test would have used, so every triangle that can hold or tie the closest
// hit is still tested: the records equal modes 0 and 1 bit for bit (any hit:
// the same flags).  Closest / any launches (single or multi-job) with quantised
// nodes and without counting; 1.77 -> 1.90 Grays/s on the terrain workload (visits per
// ray 16.95 -> 17.76 nodes, 2.17 -> 2.42 triangle tests: the lagging best t
// culls less; 31.7 tests per flush on average).
#ifndef LCX_TRI_PREFETCH
// 1: prefetch each queued triangle record into L1 at queue time (terrain workload: 2.619 against
// 2.606 Grays/s, within noise, so off)
#define LCX_TRI_PREFETCH 0
#endif
#ifndef LCX_DEFER_CAP
// queued triangle tests per warp: a step in which many lanes reach leaves queues more than the
// flush size at once, and a full queue flushes in mid-step.  Terrain workload, closest / any
// Grays/s: 48: 2.639 / 4.38; 64: 2.658-2.664 / 4.37; 80: 2.696 / 4.39; 96: 2.691-2.695 / 4.47;
// 112: 2.700 / 4.39; 128: 2.694 / 4.47 (same records)
#define LCX_DEFER_CAP 96
#endif
#ifndef LCX_DEFER_MIN_BLOCKS
#define LCX_DEFER_MIN_BLOCKS 7
#endif
#ifndef LCX_DEFER_MIN_BLOCKS_EXT
// motion launches (kExt 1): terrain workload with moving spheres 1.45 / 1.60 / 1.33 / 1.04 Grays/s
// at 4 / 5 / 6 / 7 blocks per SM (6 and 7 spill)
#define LCX_DEFER_MIN_BLOCKS_EXT 5
#endif
#ifndef LCX_DEFER_MIN_BLOCKS_CURVE
// curve launches (kExt 2): hair workload, Catmull-Rom camera / incoherent Grays/s 1.125 / 1.113
// at 4 blocks per SM (127 registers, no spills), 1.072 / 0.986 at 5 (76 bytes spilled), 0.828 /
// 0.786 at 6
#define LCX_DEFER_MIN_BLOCKS_CURVE 4
#endif
#ifndef LCX_DEFER_STACK
#define LCX_DEFER_STACK 8
#endif
// Node visits per step while a visit finds no items: 2 and 3 measured slower (1.975 -> 1.765 /
// 1.531 Grays/s; 1.898 at 6 blocks per SM): the extra visits run with few lanes and cost registers.
#ifndef LCX_DEFER_VISITS
#define LCX_DEFER_VISITS 1
#endif
constexpr int kDeferCap = LCX_DEFER_CAP;  // queued triangle tests per warp

template <bool kMulti, int kExt = 0, int kCap = kDeferCap>
struct DeferQueue {
    const TriRec *tri[kCap];
    uint32_t rec[kCap];            // ray record: lane | slot << 5
    float rr[9][64];               // per record: ox oy oz Sx Sy Sz perm tmin inst (perm, inst as bits)
    float rtime[kExt ? 64 : 1];    // motion launches: per record, its ray's time
    unsigned long long key[64];    // per record: min (ordered t << 32 | prim)
    float2 uv[64];                 // per record: barycentrics of that minimum
    float tmax[64];                // per record: the owner's best t at the flush
    float ret_t[32], ret_u[32], ret_v[32];
    uint32_t ret_inst[32], ret_prim[32], ret_rid[32];
    void *ret_out[kMulti ? 32 : 1];  // multi-job launches: the retired ray's output buffer
    uint32_t stage_ready;            // streamed launches: copy chunks [0, stage_ready) known in place
};

// Streamed launches: a copy chunk's flag, read with acquire semantics.
__device__ __forceinline__ uint32_t ld_acquire_gpu(const uint32_t *p) {
    uint32_t v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
// Polls of a copy chunk's flag before a streamed launch gives up on it (flags
// LCX_ERR_TIMEOUT): 2^20 polls with a 256 ns sleep each, one to a few seconds (a poll with
// its sleep measured about 1.5 us on GB300), where a chunk normally lands within microseconds
// of the traversal reaching it.
constexpr uint32_t kStageSpin = 1u << 20;

// kCount: the counting build (single-job closest hit), for the algorithmic bytes of this loop's own
// visits: nodes visited, triangles queued (each is tested once), instances entered.
// kExt 1: accels with motion instances or vertex-motion meshes (each ray has a time; an instance
// entry takes the instance's matrix at that time, and the flush interpolates a moving triangle at
// its ray's time); kExt 2: also curves (the flush runs the cone test of a curve segment's piece on
// the record's object-space ray, keyframed cones at the ray's time).
// kStream: a streamed host-buffer launch (TraceParams::stage_flag): a warp takes a window of rays
// only once the window's copy chunk is in place, and publishes how far its results are stored.
template <int kLayout, bool kAny, int kShort, bool kMulti, bool kCount = false, int kExt = 0, bool kStream = false>
__global__ void __launch_bounds__(kTraceBlock, kExt >= 2 ? LCX_DEFER_MIN_BLOCKS_CURVE
                                               : (kExt ? LCX_DEFER_MIN_BLOCKS_EXT : LCX_DEFER_MIN_BLOCKS))
    k_trace_deferred(TraceParams P) {
    static_assert(kExt <= 1 || LCX_WT_AT_FLUSH, "a curve test reads the record's object-space direction");
    static_assert(!kStream || (!kMulti && !kCount && kExt == 0 && LCX_RAY_CHUNK > 0),
                  "streamed launches are single-job, ray-window launches");
    using W_t = Walker<kLayout, kAny, kCount, kMulti, kShort, kExt, LCX_WT_AT_FLUSH != 0>;
    __shared__ uint2 stack_mem[W_t::kShortStack * kTraceBlock];
    // streamed launches keep the 64-entry queue: with 96 their host-buffer calls measured 2.20
    // against 2.26 Grays/s (the copies beside the kernel seem to want the L1 that the larger
    // queue's shared memory takes)
    constexpr int kCap = kStream ? 64 : kDeferCap;
    __shared__ DeferQueue<kMulti, kExt, kCap> queues[kTraceBlock / 32];
    uint2 deep_stack[W_t::kDeepSlots];
    const uint32_t lane = threadIdx.x & 31u;
    DeferQueue<kMulti, kExt, kCap> &Q = queues[threadIdx.x >> 5];
    W_t W(P, stack_mem + threadIdx.x, deep_stack);
    const int refill = int(P.refill);
    // queue size that starts a flush: P.postpone, or 24 for closest / 16 for any hit (measured on the
    // terrain workload: closest 1.860 / 1.896 / 1.886 / 1.869 Grays/s at 32 / 24 / 16 / 12; any hit
    // 3.10 / 3.20 / 3.25 / 3.26)
    const uint32_t flush_at = P.postpone >= 1 && P.postpone <= uint32_t(kCap) ? P.postpone : (kAny ? 16u : 24u);

    bool active = false, exhausted = false;
    uint32_t rid = 0, ray_steps = 0;
#if LCX_RAY_CHUNK
    uint32_t chunk_next = 0, chunk_end = 0;  // warp-uniform: ray ids this warp has taken and not yet started
#endif
    uint32_t qn = 0;        // queued entries (warp-uniform)
    uint32_t pend = 0;      // bit s: a queued entry uses this lane's record s
    uint32_t mine = 0;      // bit s: record s belongs to the lane's current ray (else to the retired one)
    uint32_t cur = 1;       // record of the current instance
    bool retired = false;   // the retire slot holds a ray waiting for queued results
    bool ret_occ = false;
    if constexpr (kStream) {
        if (lane == 0) Q.stage_ready = 0u;
        __syncwarp();
    }

    // Streamed launches (warp-uniform calls).  stage_wait: the copy chunk of ray `first` is in
    // place (chunks arrive in order; false once the wait ran out).  stage_publish: every ray this
    // warp took below `m` has its result stored; the fence orders each lane's result stores before
    // the mark, which the host reads to start the chunk's copy out.
    auto stage_wait = [&](uint32_t first) -> bool {
        const uint32_t c = first >> P.stage_shift;
        if (c < Q.stage_ready) return true;
        uint32_t ok = 1u;
        if (lane == 0) {
            for (uint32_t it = 0; ld_acquire_gpu(P.stage_flag + c) != P.stage_gen; it++) {
                if (it >= kStageSpin) {
                    ok = 0u;
                    atomicOr(P.pool + 1, kTraceErrStage);
                    break;
                }
                __nanosleep(256);
            }
            if (ok) Q.stage_ready = c + 1u;
        }
        ok = __shfl_sync(~0u, ok, 0);
        __syncwarp();
        return ok != 0u;
    };
    auto stage_publish = [&](uint32_t m) {
        __threadfence_system();
        __syncwarp();
        if (lane == 0) {
            uint32_t *dst = P.stage_mark + (blockIdx.x * (kTraceBlock / 32) + (threadIdx.x >> 5));
            asm volatile("st.relaxed.sys.global.u32 [%0], %1;" ::"l"(dst), "r"(m) : "memory");
        }
    };

    // Test every queued entry (all lanes call it together), merge the results
    // into their rays and write out the retired rays.
    auto flush = [&]() {
#pragma unroll
        for (uint32_t s = 0; s < 2; s++) {
            if ((pend >> s) & 1u) {
                const uint32_t r = lane + 32u * s;
                Q.tmax[r] = ((mine >> s) & 1u) ? W.best_t : Q.ret_t[lane];
                Q.key[r] = ~0ull;
            }
        }
        __syncwarp();
        for (uint32_t base = 0; base < qn; base += 32u) {
            const uint32_t j = base + lane;
            bool hit = false;
            unsigned long long key = ~0ull;
            uint32_t r = 0;
            float t = 0.0f, u = 0.0f, v = 0.0f;
            if (j < qn) {
                r = Q.rec[j];
                WtRay ray;
#if LCX_WT_AT_FLUSH
                // the record holds the object-space ray; the test's setup is the same function of it
                // that an entry would have computed, so the bits are the same
                ray = wt_setup(Q.rr[0][r], Q.rr[1][r], Q.rr[2][r], Q.rr[3][r], Q.rr[4][r], Q.rr[5][r]);
#else
                ray.ox = Q.rr[0][r];
                ray.oy = Q.rr[1][r];
                ray.oz = Q.rr[2][r];
                ray.Sx = Q.rr[3][r];
                ray.Sy = Q.rr[4][r];
                ray.Sz = Q.rr[5][r];
                ray.perm = __float_as_uint(Q.rr[6][r]);
#endif
                const float lo = Q.rr[7][r], hi = Q.tmax[r];
                const float4 *tp = reinterpret_cast<const float4 *>(Q.tri[j]);
                float4 a = bvh_ld(tp), b = bvh_ld(tp + 1), c = bvh_ld(tp + 2);
                bool live = true, cone = false;
                if constexpr (kExt >= 2) {
                    const uint32_t marker = __float_as_uint(b.w);
                    if (marker == kTriCurve || marker == kTriCurveMotion) {  // a cone of a curve segment
                        cone = true;
                        float4 c0 = make_float4(a.x, a.y, a.z, c.x), c1 = make_float4(b.x, b.y, b.z, c.y);
                        live = marker != kTriCurveMotion || curve_motion_cone(a, b, c, Q.rtime[r], c0, c1);
                        const uint32_t kn = __float_as_uint(c.z);
                        // the curve test on the record's object-space ray (origin, direction); v = -1
                        // marks a curve hit as in the immediate loop
                        live = live && curve_piece_entry(make_float3(Q.rr[0][r], Q.rr[1][r], Q.rr[2][r]),
                                                         make_float3(Q.rr[3][r], Q.rr[4][r], Q.rr[5][r]), c0, c1,
                                                         kn & 0xffffu, kn >> 16, __float_as_uint(c.w), lo, hi, t, u);
                        v = -1.0f;
                    }
                }
                if constexpr (kExt >= 1) {
                    if (__float_as_uint(b.w) == kTriMotion) {  // a vertex-motion mesh: its triangle at the ray's time
                        const MeshMotion *mm = reinterpret_cast<const MeshMotion *>(
                            (unsigned long long)__float_as_uint(c.x) |
                            ((unsigned long long)__float_as_uint(c.y) << 32));
                        live = motion_triangle(*mm, __float_as_uint(a.w), Q.rtime[r], a, b, c);
                    }
                }
                if (live && (cone || wt_intersect(ray, lo, hi, a, b, c, t, u, v))) {
                    hit = true;
                    key = kAny ? 0ull
                               : (static_cast<unsigned long long>(float_to_ordered(t)) << 32) | __float_as_uint(a.w);
                    atomicMin(&Q.key[r], key);
                }
            }
            if (!kAny) {
                __syncwarp();
                if (hit && key == Q.key[r]) Q.uv[r] = make_float2(u, v);
            }
            __syncwarp();
        }
#pragma unroll
        for (uint32_t s = 0; s < 2; s++) {
            if (!((pend >> s) & 1u)) continue;
            const uint32_t r = lane + 32u * s;
            const unsigned long long k = Q.key[r];
            if (k == ~0ull) continue;
            const bool cur_ray = (mine >> s) & 1u;
            if (kAny) {
                if (cur_ray)
                    W.occluded = true;
                else
                    ret_occ = true;
                continue;
            }
            const float t = ordered_to_float(uint32_t(k >> 32));
            const uint32_t prim = uint32_t(k);
            const uint32_t inst = __float_as_uint(Q.rr[8][r]);
            const float2 uv = Q.uv[r];
            // lexicographic (t, inst, prim): the other record's minimum may already
            // have lowered the best t of this flush
            if (cur_ray) {
                if (t < W.best_t || (t == W.best_t && (inst < W.best_inst || (inst == W.best_inst && prim < W.best_prim)))) {
                    W.best_t = t;
                    W.best_u = uv.x;
                    W.best_v = uv.y;
                    W.best_inst = inst;
                    W.best_prim = prim;
                }
            } else {
                const float bt = Q.ret_t[lane];
                const uint32_t bi = Q.ret_inst[lane], bp = Q.ret_prim[lane];
                if (t < bt || (t == bt && (inst < bi || (inst == bi && prim < bp)))) {
                    Q.ret_t[lane] = t;
                    Q.ret_u[lane] = uv.x;
                    Q.ret_v[lane] = uv.y;
                    Q.ret_inst[lane] = inst;
                    Q.ret_prim[lane] = prim;
                }
            }
        }
        if (retired) {  // its last queued tests are done
            const uint32_t ro = Q.ret_rid[lane];
            if (kAny) {
                (kMulti ? static_cast<uint8_t *>(Q.ret_out[lane]) : P.occluded)[ro] = ret_occ ? 1 : 0;
            } else {
                uint2 *hp = reinterpret_cast<uint2 *>((kMulti ? static_cast<Hit *>(Q.ret_out[lane]) : P.hits) + ro);
                __stcs(hp, make_uint2(Q.ret_inst[lane], Q.ret_prim[lane]));
                __stcs(hp + 1, make_uint2(__float_as_uint(Q.ret_u[lane]), __float_as_uint(Q.ret_v[lane])));
                __stcs(hp + 2, make_uint2(__float_as_uint(Q.ret_t[lane]), 0u));
            }
            retired = false;
        }
        pend = 0;
        qn = 0;
        __syncwarp();
    };

    for (;;) {
        // refill: idle lanes take new rays once enough of them are idle
        const uint32_t idle = __ballot_sync(~0u, !active);
        const int n_idle = __popc(idle);
        if (!exhausted && n_idle >= refill) {
#if LCX_RAY_CHUNK
            // the warp takes LCX_RAY_CHUNK ids at a time from the global counter and serves its idle
            // lanes from them: one atomic per chunk, and the chunk's rays prefetched into L2 at once
            if (chunk_next >= chunk_end) {
                uint32_t base = 0;
                if (lane == 0) base = atomicAdd(P.pool, uint32_t(LCX_RAY_CHUNK));
                base = __shfl_sync(~0u, base, 0);
                chunk_next = base;
                chunk_end = uint32_t(min(uint64_t(base) + LCX_RAY_CHUNK, uint64_t(P.ray_count)));
                if (chunk_next > chunk_end) chunk_next = chunk_end;
                if constexpr (kStream) {
                    // a window lies in one copy chunk (chunks are multiples of the window)
                    if (chunk_next < chunk_end && !stage_wait(chunk_next)) {
                        chunk_next = chunk_end;  // the rays did not arrive: take no more
                        exhausted = true;
                    }
                    // in flight: the lanes' rays, the retired ones, the window's untaken ones
                    uint32_t m = active ? rid : 0xffffffffu;
                    if (retired) m = min(m, Q.ret_rid[lane]);
                    m = min(__reduce_min_sync(~0u, m), chunk_next);
                    stage_publish(m);
                }
                if (!kMulti && P.order == nullptr) {
                    for (uint32_t r = base + lane; r < chunk_end; r += 32u)
                        asm volatile("prefetch.global.L2 [%0];" ::"l"(P.rays + r));
                }
            }
            const uint32_t base = chunk_next;
            const uint32_t take = min(uint32_t(n_idle), chunk_end - chunk_next);
            chunk_next += take;
            if (chunk_next >= chunk_end && chunk_end >= P.ray_count) exhausted = true;
            if (!active) {
                const uint32_t k = __popc(idle & ((1u << lane) - 1u));
                if (k < take) {
                    rid = base + k;
                    active = true;
                    ray_steps = 0;
                    mine = 0;
                    W.start(rid);
                }
            }
#else
            uint32_t base = 0;
            if (lane == 0) base = atomicAdd(P.pool, uint32_t(n_idle));
            base = __shfl_sync(~0u, base, 0);
            if (uint64_t(base) + uint64_t(n_idle) >= P.ray_count) exhausted = true;
            if (!active) {
                const uint32_t my = base + __popc(idle & ((1u << lane) - 1u));
                if (my < P.ray_count) {
                    rid = my;
                    active = true;
                    ray_steps = 0;
                    mine = 0;
                    W.start(rid);
                }
            }
#endif
        }
        if (__ballot_sync(~0u, active) == 0u) {
            if (qn != 0u || __any_sync(~0u, retired)) flush();
            if (exhausted) break;
            continue;
        }

        // 1. visit a node (or take a popped item group)
        uint2 Gt = make_uint2(0, 0);
        if (active) {
            if (kAny && W.occluded) {  // a flush found a hit: end the walk
                W.G = make_uint2(0, 0);
                W.sp = 0;
                W.blas_sp = 0;
            } else if (++ray_steps > P.max_steps) {
                atomicOr(P.pool + 1, 2u);
                W.G = make_uint2(0, 0);
                W.sp = 0;
                W.blas_sp = 0;
            } else if (W.G.y >= 0x01000000u) {
                W.visit(Gt);
#if LCX_DEFER_VISITS > 1
                // while a visit finds only internal children, take the next one in the same step
                for (int v = 1; v < LCX_DEFER_VISITS && Gt.y == 0u && W.G.y >= 0x01000000u; v++) {
                    if (++ray_steps > P.max_steps) {
                        atomicOr(P.pool + 1, 2u);
                        W.G = make_uint2(0, 0);
                        W.sp = 0;
                        W.blas_sp = 0;
                        break;
                    }
                    W.visit(Gt);
                }
#endif
            } else {
                Gt = W.G;
                W.G = make_uint2(0, 0);
            }
        }

        // 2. queue the triangles found inside a BLAS (warp-wide prefix over the lanes' counts)
        const bool has_tris = active && W.in_blas && Gt.y != 0u;
        if (kCount && has_tris) W.c_tris += __popc(Gt.y);
        if (__any_sync(~0u, has_tris)) {
            uint32_t bits = has_tris ? Gt.y : 0u;
            const TriRec *tbase = has_tris ? W.blas_tris + Gt.x : nullptr;
            for (;;) {
                const uint32_t cnt = __popc(bits);
#if LCX_QUEUE_BALLOT
                // exclusive prefix and total of the lanes' counts (< 32) from one ballot per bit:
                // independent votes instead of a chain of dependent shuffles
                uint32_t excl = 0u, total = 0u;
                const uint32_t below = (1u << lane) - 1u;
#pragma unroll
                for (int b = 0; b < 5; b++) {
                    const uint32_t m = __ballot_sync(~0u, (cnt >> b) & 1u);
                    excl += uint32_t(__popc(m & below)) << b;
                    total += uint32_t(__popc(m)) << b;
                }
                if (total == 0u) break;
                const uint32_t space = uint32_t(kCap) - qn;
                uint32_t pos = qn + excl;
#else
                uint32_t incl = cnt;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const uint32_t x = __shfl_up_sync(~0u, incl, o);
                    if (lane >= uint32_t(o)) incl += x;
                }
                const uint32_t total = __shfl_sync(~0u, incl, 31);
                if (total == 0u) break;
                const uint32_t space = uint32_t(kCap) - qn;
                uint32_t pos = qn + incl - cnt;
#endif
                while (bits != 0u && pos < uint32_t(kCap)) {
                    const uint32_t k = __ffs(bits) - 1u;
                    bits &= bits - 1u;
#if LCX_TRI_PREFETCH
                    {  // the record's two 128-byte lines into L1 now, for the flush's loads
                        const char *tp = reinterpret_cast<const char *>(tbase + k);
                        asm volatile("prefetch.global.L1 [%0];" ::"l"(tp));
                        asm volatile("prefetch.global.L1 [%0];" ::"l"(tp + 47));
                    }
#endif
                    Q.tri[pos] = tbase + k;
                    Q.rec[pos] = lane | (cur << 5);
                    pend |= 1u << cur;
                    pos++;
                }
                if (total <= space) {
                    qn += total;
                    break;
                }
                qn = uint32_t(kCap);
                flush();
            }
        }

        // 3. enter instances (TLAS items); the record to be written must be free
        const bool enter = active && !W.in_blas && Gt.y != 0u;
        if (__any_sync(~0u, enter && ((pend >> (cur ^ 1u)) & 1u))) flush();
        if (enter) {
            W.instances(Gt);
            if (W.in_blas) {
                cur ^= 1u;
                const uint32_t r = lane + 32u * cur;
#if LCX_WT_AT_FLUSH
                Q.rr[0][r] = W.ox;
                Q.rr[1][r] = W.oy;
                Q.rr[2][r] = W.oz;
                Q.rr[3][r] = W.rdx;
                Q.rr[4][r] = W.rdy;
                Q.rr[5][r] = W.rdz;
#else
                Q.rr[0][r] = W.wt.ox;
                Q.rr[1][r] = W.wt.oy;
                Q.rr[2][r] = W.wt.oz;
                Q.rr[3][r] = W.wt.Sx;
                Q.rr[4][r] = W.wt.Sy;
                Q.rr[5][r] = W.wt.Sz;
                Q.rr[6][r] = __uint_as_float(W.wt.perm);
#endif
                Q.rr[7][r] = W.tmin;
                Q.rr[8][r] = __uint_as_float(W.cur_inst);
                if constexpr (kExt >= 1) Q.rtime[r] = W.time;
                mine |= 1u << cur;
            }
        }

        // 4. pop; a finished ray with queued tests retires (or waits while the retire slot is taken)
        bool blocked = false;
        if (active && W.G.y == 0u) {
            if (W.pop_or_done()) {
                if (pend & mine) {
                    if (retired) {
                        blocked = true;
                    } else {
                        Q.ret_t[lane] = W.best_t;
                        Q.ret_u[lane] = W.best_u;
                        Q.ret_v[lane] = W.best_v;
                        Q.ret_inst[lane] = W.best_inst;
                        Q.ret_prim[lane] = W.best_prim;
                        Q.ret_rid[lane] = W.slot;
                        if (kMulti) Q.ret_out[lane] = W.out;
                        W.store_counts();  // complete: its triangles were counted when queued
                        ret_occ = W.occluded;
                        retired = true;
                        mine = 0;
                        active = false;
                    }
                } else {
                    W.finish();
                    mine = 0;
                    active = false;
                }
            }
        }

        // 5. test the queue once it is full enough, or a finished ray is waiting on it
        if (qn >= flush_at || __any_sync(~0u, blocked)) flush();
    }
    if constexpr (kStream) stage_publish(0xffffffffu);
}

// ---------------------------------------------------------------------------
// Loop mode 3: one ray per thread, each thread calling lcx::trace_closest /
// lcx::trace_any (include/lcx/trace.cuh) with a 16-entry shared short stack --
// exactly what a user megakernel's per-ray calls run, as a launch form of the
// plain entry points (so the per-ray device functions are measured and
// parity-tested through the C ABI).  No persistent warps: a warp holds its
// lanes until its slowest ray ends.  Motion accels are traced by the same walk
// (at each ray's time).
template <bool kAny>
__global__ void __launch_bounds__(kTraceBlock, LCX_PER_THREAD_MIN_BLOCKS) k_trace_per_thread(TraceParams P) {
    constexpr int kShort = 16;
    __shared__ uint2 sstack[kShort * kTraceBlock];
    const uint32_t k = blockIdx.x * kTraceBlock + threadIdx.x;
    if (k >= P.ray_count) return;
    const uint32_t i = P.order != nullptr ? __ldg(P.order + k) : k;  // reordered calls: the k-th ray taken
    LcxAccelView view;
    view.tlas_nodes = P.tlas_q;
    view.instances = P.insts;
    view.stack_need = 0u;
    view.motion = P.motion ? 1u : 0u;
    const float4 *rp = reinterpret_cast<const float4 *>(P.rays + i);
    const float4 r0 = __ldcs(rp), r1 = __ldcs(rp + 1);
    LcxRay ray;
    ray.origin[0] = r0.x;
    ray.origin[1] = r0.y;
    ray.origin[2] = r0.z;
    ray.t_min = r0.w;
    ray.direction[0] = r1.x;
    ray.direction[1] = r1.y;
    ray.direction[2] = r1.z;
    ray.t_max = r1.w;
    const float time = P.times != nullptr ? __ldg(P.times + i) : 0.0f;
    LcxTriangleHit h;
    bool occ;
    detail::trace_walk<kAny, kShort>(view, ray, time, P.mask, ShortStack{sstack + threadIdx.x, kTraceBlock}, h, occ,
                                     P.max_steps, P.pool + 1);
    if (kAny) {
        P.occluded[i] = occ ? 1 : 0;
    } else {
        uint2 *hp = reinterpret_cast<uint2 *>(P.hits + i);
        __stcs(hp, make_uint2(h.inst, h.prim));
        __stcs(hp + 1, make_uint2(__float_as_uint(h.bary[0]), __float_as_uint(h.bary[1])));
        __stcs(hp + 2, make_uint2(__float_as_uint(h.committed_ray_t), 0u));
    }
}

template <bool A>
cudaError_t launch_per_thread(const TraceParams &p, cudaStream_t st) {
    const uint64_t grid = (uint64_t(p.ray_count) + kTraceBlock - 1) / kTraceBlock;
    k_trace_per_thread<A><<<unsigned(grid), kTraceBlock, 0, st>>>(p);
    return cudaGetLastError();
}

template <int L, bool A, bool C, int M, bool X, int S, int Mo = 0>
int blocks_per_sm() {
    static int v = 0;
    if (v == 0) {
        int b = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_trace<L, A, C, M, X, S, Mo>, kTraceBlock, 0);
        v = b > 0 ? b : 1;
    }
    return v;
}

int sm_count() {
    static int v = 0;
    if (v == 0) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
        if (v <= 0) v = 1;
    }
    return v;
}

template <int L, bool A, bool C, int M, bool X = false, int S = kDefaultShortStack, int Mo = 0>
cudaError_t launch_one(const TraceParams &p, cudaStream_t st) {
    const uint64_t warps_needed = (uint64_t(p.ray_count) + 31) / 32;
    uint64_t grid = uint64_t(sm_count()) * blocks_per_sm<L, A, C, M, X, S, Mo>();
    const uint64_t grid_need = (warps_needed + (kTraceBlock / 32) - 1) / (kTraceBlock / 32);
    if (grid_need < grid) grid = grid_need;
    if (grid == 0) grid = 1;
    k_trace<L, A, C, M, X, S, Mo><<<unsigned(grid), kTraceBlock, 0, st>>>(p);
    return cudaGetLastError();
}

// Single-job, loop mode 0 closest / any kernels: short stack of 8, 16 or 24 entries.
template <int L, bool A>
cudaError_t launch_stack(const TraceParams &p, cudaStream_t st) {
    if (p.short_stack == 8) return launch_one<L, A, false, 0, false, 8>(p, st);
    if (p.short_stack == 24) return launch_one<L, A, false, 0, false, 24>(p, st);
    return launch_one<L, A, false, 0, false, kDefaultShortStack>(p, st);
}

template <int L, bool A, int S, bool X = false, bool C = false, int E = 0, bool St = false>
uint64_t deferred_grid(uint32_t ray_count) {
    static int per_sm = 0;
    if (per_sm == 0) {
        int b = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_trace_deferred<L, A, S, X, C, E, St>, kTraceBlock, 0);
        per_sm = b > 0 ? b : 1;
    }
    const uint64_t warps_needed = (uint64_t(ray_count) + 31) / 32;
    uint64_t grid = uint64_t(sm_count()) * uint64_t(per_sm);
    const uint64_t grid_need = (warps_needed + (kTraceBlock / 32) - 1) / (kTraceBlock / 32);
    if (grid_need < grid) grid = grid_need;
    return grid == 0 ? 1 : grid;
}

template <int L, bool A, int S, bool X = false, bool C = false, int E = 0, bool St = false>
cudaError_t launch_deferred(const TraceParams &p, cudaStream_t st) {
    const uint64_t grid = deferred_grid<L, A, S, X, C, E, St>(p.ray_count);
    k_trace_deferred<L, A, S, X, C, E, St><<<unsigned(grid), kTraceBlock, 0, st>>>(p);
    return cudaGetLastError();
}

template <int M>
cudaError_t launch_mode(const TraceParams &p, int layout, bool any, bool counting, cudaStream_t st) {
    if (layout == LCX_NODES_QUANT8) {
        if (counting) return launch_one<LCX_NODES_QUANT8, false, true, M>(p, st);
        if (M == 0) return any ? launch_stack<LCX_NODES_QUANT8, true>(p, st) : launch_stack<LCX_NODES_QUANT8, false>(p, st);
        if (any) return launch_one<LCX_NODES_QUANT8, true, false, M>(p, st);
        return launch_one<LCX_NODES_QUANT8, false, false, M>(p, st);
    }
    if (counting) return launch_one<LCX_NODES_FP32, false, true, M>(p, st);
    if (M == 0) return any ? launch_stack<LCX_NODES_FP32, true>(p, st) : launch_stack<LCX_NODES_FP32, false>(p, st);
    if (any) return launch_one<LCX_NODES_FP32, true, false, M>(p, st);
    return launch_one<LCX_NODES_FP32, false, false, M>(p, st);
}

// The extended kernels (kExt 1: motion; 2: motion and curves), loop mode 0 with per-ray times.
template <int E>
cudaError_t launch_ext(const TraceParams &p, int layout, bool any, bool counting, cudaStream_t st) {
    if (p.jobs != nullptr) {  // multi-job launches with motion or curves (each job's times, or time 0)
        if (layout == LCX_NODES_QUANT8)
            return any ? launch_one<LCX_NODES_QUANT8, true, false, 0, true, kDefaultShortStack, E>(p, st)
                       : launch_one<LCX_NODES_QUANT8, false, false, 0, true, kDefaultShortStack, E>(p, st);
        return any ? launch_one<LCX_NODES_FP32, true, false, 0, true, kDefaultShortStack, E>(p, st)
                   : launch_one<LCX_NODES_FP32, false, false, 0, true, kDefaultShortStack, E>(p, st);
    }
    if (layout == LCX_NODES_QUANT8) {
        if (counting) return launch_one<LCX_NODES_QUANT8, false, true, 0, false, kDefaultShortStack, E>(p, st);
        return any ? launch_one<LCX_NODES_QUANT8, true, false, 0, false, kDefaultShortStack, E>(p, st)
                   : launch_one<LCX_NODES_QUANT8, false, false, 0, false, kDefaultShortStack, E>(p, st);
    }
    if (counting) return launch_one<LCX_NODES_FP32, false, true, 0, false, kDefaultShortStack, E>(p, st);
    return any ? launch_one<LCX_NODES_FP32, true, false, 0, false, kDefaultShortStack, E>(p, st)
               : launch_one<LCX_NODES_FP32, false, false, 0, false, kDefaultShortStack, E>(p, st);
}

}  // namespace

uint32_t stream_launch_warps(uint32_t ray_count, bool any) {
    const uint64_t grid = any ? deferred_grid<LCX_NODES_QUANT8, true, LCX_DEFER_STACK, false, false, 0, true>(ray_count)
                              : deferred_grid<LCX_NODES_QUANT8, false, LCX_DEFER_STACK, false, false, 0, true>(ray_count);
    return uint32_t(grid * (kTraceBlock / 32));
}

cudaError_t launch_trace(const TraceParams &p, int layout, bool any, bool counting, cudaStream_t st) {
    if (p.stage_flag != nullptr) {  // streamed host-buffer launches (the host checked the form)
        if (p.jobs != nullptr || p.motion || counting || p.order != nullptr || layout != LCX_NODES_QUANT8)
            return cudaErrorInvalidValue;
        return any ? launch_deferred<LCX_NODES_QUANT8, true, LCX_DEFER_STACK, false, false, 0, true>(p, st)
                   : launch_deferred<LCX_NODES_QUANT8, false, LCX_DEFER_STACK, false, false, 0, true>(p, st);
    }
    // loop mode 3 (one ray per thread through the device-side trace functions): single-job,
    // quantised-node, non-counting calls, static or moving; the others run mode 0
    if (p.mode == 3 && p.jobs == nullptr && !counting && layout == LCX_NODES_QUANT8)
        return any ? launch_per_thread<true>(p, st) : launch_per_thread<false>(p, st);
    if (p.motion) {
        // accels with motion instances, vertex-motion meshes or curves: loop mode 2 (deferred
        // triangle and cone batches at each ray's time) with quantised nodes; FP32 nodes, the
        // counting build and the other loop modes: the extended kernels of loop mode 0
        if (p.mode == 2 && layout == LCX_NODES_QUANT8 && !counting) {
            if (p.curves) {  // kExt 2: curve cones tested at the flush as well
                if (p.jobs != nullptr)
                    return any ? launch_deferred<LCX_NODES_QUANT8, true, LCX_DEFER_STACK, true, false, 2>(p, st)
                               : launch_deferred<LCX_NODES_QUANT8, false, LCX_DEFER_STACK, true, false, 2>(p, st);
                return any ? launch_deferred<LCX_NODES_QUANT8, true, LCX_DEFER_STACK, false, false, 2>(p, st)
                           : launch_deferred<LCX_NODES_QUANT8, false, LCX_DEFER_STACK, false, false, 2>(p, st);
            }
            if (p.jobs != nullptr)
                return any ? launch_deferred<LCX_NODES_QUANT8, true, LCX_DEFER_STACK, true, false, 1>(p, st)
                           : launch_deferred<LCX_NODES_QUANT8, false, LCX_DEFER_STACK, true, false, 1>(p, st);
            return any ? launch_deferred<LCX_NODES_QUANT8, true, LCX_DEFER_STACK, false, false, 1>(p, st)
                       : launch_deferred<LCX_NODES_QUANT8, false, LCX_DEFER_STACK, false, false, 1>(p, st);
        }
        return p.curves ? launch_ext<2>(p, layout, any, counting, st) : launch_ext<1>(p, layout, any, counting, st);
    }
    if (p.jobs != nullptr) {  // multi-job launches: no counting; mode 2 with quantised nodes, else mode 0
        if (p.mode == 2 && layout == LCX_NODES_QUANT8)
            return any ? launch_deferred<LCX_NODES_QUANT8, true, LCX_DEFER_STACK, true>(p, st)
                       : launch_deferred<LCX_NODES_QUANT8, false, LCX_DEFER_STACK, true>(p, st);
        if (layout == LCX_NODES_QUANT8)
            return any ? launch_one<LCX_NODES_QUANT8, true, false, 0, true>(p, st)
                       : launch_one<LCX_NODES_QUANT8, false, false, 0, true>(p, st);
        return any ? launch_one<LCX_NODES_FP32, true, false, 0, true>(p, st)
                   : launch_one<LCX_NODES_FP32, false, false, 0, true>(p, st);
    }
    // deferred triangle batches: single-job quantised-node launches (with FP32 nodes mode 2
    // measured slower than mode 0, 1.06-1.10 vs 1.62 Grays/s, so those run mode 0); the counting
    // build of mode 2 counts this loop's own visits
    if (p.mode == 2 && layout == LCX_NODES_QUANT8) {
        if (counting) return launch_deferred<LCX_NODES_QUANT8, false, LCX_DEFER_STACK, false, true>(p, st);
        return any ? launch_deferred<LCX_NODES_QUANT8, true, LCX_DEFER_STACK>(p, st)
                   : launch_deferred<LCX_NODES_QUANT8, false, LCX_DEFER_STACK>(p, st);
    }
    if (p.mode >= 2) return launch_mode<0>(p, layout, any, counting, st);
    return p.mode == 1 ? launch_mode<1>(p, layout, any, counting, st) : launch_mode<0>(p, layout, any, counting, st);
}

}  // namespace lcx
