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
//     stack in shared memory (kStackSize x 8 B per thread);
//   * two levels: a TLAS leaf item is an instance; the ray is moved to object
//     space with the exact FP32 sequence of lcx_device.cuh and the same loop
//     runs over the BLAS; when the stack unwinds to the entry depth the world
//     ray is restored;
//   * 128-bit read-only loads of nodes (5 for Node8Q, 13 for Node8F) and
//     triangles (3 per triangle);
//   * closest hit keeps (t, inst, prim) minimal, so the answer is independent
//     of traversal order; any hit stops at the first accepted triangle.
#include "lcx_internal.h"

namespace lcx {
namespace {

constexpr int kTraceBlock = 128;
constexpr uint32_t kMaxRaySteps = 1u << 22;  // per-ray bound: a corrupt tree ends the ray, never hangs

__device__ __forceinline__ uint2 root_group(uint32_t octinv) {
    // visit node 0 (slot 0 internal, imask = 1); key of slot 0 is 0 ^ octinv
    return make_uint2(0u, (1u << (24 + octinv)) | 1u);
}

__device__ __forceinline__ uint32_t octant_inv(float dx, float dy, float dz) {
    return ((dx < 0.0f ? 1u : 0u) | (dy < 0.0f ? 2u : 0u) | (dz < 0.0f ? 4u : 0u)) ^ 7u;
}

__device__ __forceinline__ float byte_to_float(uint32_t w, uint32_t k) {
    // byte k of w as an exact float: 0x4B0000bb - 2^23
    return __uint_as_float(__byte_perm(w, 0x4B000000u, 0x7540u | k)) - 8388608.0f;
}

__device__ __forceinline__ void intersect_q(const Node8Q *nodes, uint32_t idx, float ox, float oy, float oz,
                                            float ix, float iy, float iz, uint32_t octinv, float tmin, float tmax,
                                            uint2 &G, uint2 &Gt) {
    const uint4 *p = reinterpret_cast<const uint4 *>(nodes + idx);
    const uint4 n0 = __ldg(p), n1 = __ldg(p + 1), n2 = __ldg(p + 2), n3 = __ldg(p + 3), n4 = __ldg(p + 4);
    const float sx = __uint_as_float((n0.w & 0xffu) << 23);
    const float sy = __uint_as_float(((n0.w >> 8) & 0xffu) << 23);
    const float sz = __uint_as_float(((n0.w >> 16) & 0xffu) << 23);
    const float adx = sx * ix, ady = sy * iy, adz = sz * iz;
    // plane offset (p - o) / d, widened by 2^-20 of itself on each side: its two
    // roundings can flip the sign of a face the ray lies in when d ~ 0 (1/d ~ 1e30)
    const float aox = (__uint_as_float(n0.x) - ox) * ix;
    const float aoy = (__uint_as_float(n0.y) - oy) * iy;
    const float aoz = (__uint_as_float(n0.z) - oz) * iz;
    const float slx = fabsf(aox) * 0x1p-20f, sly = fabsf(aoy) * 0x1p-20f, slz = fabsf(aoz) * 0x1p-20f;
    const float aoxn = aox - slx, aoxf = aox + slx;
    const float aoyn = aoy - sly, aoyf = aoy + sly;
    const float aozn = aoz - slz, aozf = aoz + slz;
    // near/far planes by ray direction sign (swap whole byte words)
    const bool nx = ix < 0.0f, ny = iy < 0.0f, nz = iz < 0.0f;
    const uint32_t nx0 = nx ? n3.z : n2.x, nx1 = nx ? n3.w : n2.y, fx0 = nx ? n2.x : n3.z, fx1 = nx ? n2.y : n3.w;
    const uint32_t ny0 = ny ? n4.x : n2.z, ny1 = ny ? n4.y : n2.w, fy0 = ny ? n2.z : n4.x, fy1 = ny ? n2.w : n4.y;
    const uint32_t nz0 = nz ? n4.z : n3.x, nz1 = nz ? n4.w : n3.y, fz0 = nz ? n3.x : n4.z, fz1 = nz ? n3.y : n4.w;
    uint32_t hits = 0, items = 0;
#pragma unroll
    for (int s = 0; s < 8; s++) {
        const uint32_t k = s & 3;
        const bool hw = s >= 4;
        const float tnx = __fmaf_rn(byte_to_float(hw ? nx1 : nx0, k), adx, aoxn);
        const float tfx = __fmaf_rn(byte_to_float(hw ? fx1 : fx0, k), adx, aoxf);
        const float tny = __fmaf_rn(byte_to_float(hw ? ny1 : ny0, k), ady, aoyn);
        const float tfy = __fmaf_rn(byte_to_float(hw ? fy1 : fy0, k), ady, aoyf);
        const float tnz = __fmaf_rn(byte_to_float(hw ? nz1 : nz0, k), adz, aozn);
        const float tfz = __fmaf_rn(byte_to_float(hw ? fz1 : fz0, k), adz, aozf);
        const float tn = fmaxf(fmaxf(tnx, tny), fmaxf(tnz, tmin));
        const float tf = fminf(fminf(tfx, tfy), fminf(tfz, tmax));
        const uint32_t meta = ((hw ? n1.w : n1.z) >> (8 * k)) & 0xffu;
        if (meta != 0u && slab_accept(tn, tf)) {
            if (meta & kMetaInternal)
                hits |= 1u << (s ^ octinv);
            else
                items |= ((1u << (meta >> 5)) - 1u) << (meta & 31u);
        }
    }
    G = make_uint2(n1.x, hits ? ((hits << 24) | (n0.w >> 24)) : 0u);
    Gt = make_uint2(n1.y, items);
}

__device__ __forceinline__ void intersect_f(const Node8F *nodes, uint32_t idx, float ox, float oy, float oz,
                                            float ix, float iy, float iz, uint32_t octinv, float tmin, float tmax,
                                            uint2 &G, uint2 &Gt) {
    const float4 *p = reinterpret_cast<const float4 *>(nodes + idx);
    const uint4 hdr = __ldg(reinterpret_cast<const uint4 *>(p + 12));
    const bool nx = ix < 0.0f, ny = iy < 0.0f, nz = iz < 0.0f;
    // lo_x: p[0..1], hi_x: p[2..3], lo_y: p[4..5], hi_y: p[6..7], lo_z: p[8..9], hi_z: p[10..11]
    uint32_t hits = 0, items = 0, imask = 0;
#pragma unroll
    for (int half = 0; half < 2; half++) {
        const float4 lx = __ldg(p + 0 + half), hx = __ldg(p + 2 + half);
        const float4 ly = __ldg(p + 4 + half), hy = __ldg(p + 6 + half);
        const float4 lz = __ldg(p + 8 + half), hz = __ldg(p + 10 + half);
        const float LX[4] = {lx.x, lx.y, lx.z, lx.w}, HX[4] = {hx.x, hx.y, hx.z, hx.w};
        const float LY[4] = {ly.x, ly.y, ly.z, ly.w}, HY[4] = {hy.x, hy.y, hy.z, hy.w};
        const float LZ[4] = {lz.x, lz.y, lz.z, lz.w}, HZ[4] = {hz.x, hz.y, hz.z, hz.w};
        const uint32_t mw = half ? hdr.w : hdr.z;
#pragma unroll
        for (int k = 0; k < 4; k++) {
            const int s = half * 4 + k;
            const float tnx = (nx ? HX[k] : LX[k]) - ox, tfx = (nx ? LX[k] : HX[k]) - ox;
            const float tny = (ny ? HY[k] : LY[k]) - oy, tfy = (ny ? LY[k] : HY[k]) - oy;
            const float tnz = (nz ? HZ[k] : LZ[k]) - oz, tfz = (nz ? LZ[k] : HZ[k]) - oz;
            const float tn = fmaxf(fmaxf(tnx * ix, tny * iy), fmaxf(tnz * iz, tmin));
            const float tf = fminf(fminf(tfx * ix, tfy * iy), fminf(tfz * iz, tmax));
            const uint32_t meta = (mw >> (8 * k)) & 0xffu;
            if (meta & kMetaInternal) imask |= 1u << s;
            if (meta != 0u && slab_accept(tn, tf)) {
                if (meta & kMetaInternal)
                    hits |= 1u << (s ^ octinv);
                else
                    items |= ((1u << (meta >> 5)) - 1u) << (meta & 31u);
            }
        }
    }
    G = make_uint2(hdr.x, hits ? ((hits << 24) | imask) : 0u);
    Gt = make_uint2(hdr.y, items);
}

template <int kLayout, bool kAny, bool kCount>
__global__ void __launch_bounds__(kTraceBlock, 4) k_trace(TraceParams P) {
    __shared__ uint2 stack_mem[kStackSize * kTraceBlock];
    uint2 *const stk = stack_mem + threadIdx.x;
    const uint32_t lane = threadIdx.x & 31u;
    const void *const tlas_nodes = kLayout == LCX_NODES_QUANT8 ? static_cast<const void *>(P.tlas_q)
                                                                : static_cast<const void *>(P.tlas_f);
    const int refill = int(P.refill);
    const int postpone = int(P.postpone);
    const int postpone_sp = P.postpone_sp;

    bool active = false, exhausted = false;
    uint32_t rid = 0;
    // world ray
    float wox = 0, woy = 0, woz = 0, wdx = 0, wdy = 0, wdz = 1;
    float tmin = 0, best_t = 0, best_u = 0, best_v = 0;
    uint32_t best_inst = kInvalid, best_prim = kInvalid;
    // current-space ray (world at the TLAS level, object inside a BLAS)
    float ox = 0, oy = 0, oz = 0, ix = 1, iy = 1, iz = 1;
    uint32_t octinv = 0;
    WtRay wt{};
    uint2 G = make_uint2(0, 0);
    int sp = 0, blas_sp = 0;
    bool in_blas = false, occluded = false;
    uint32_t cur_inst = 0;
    const void *blas_nodes = nullptr;
    const TriRec *blas_tris = nullptr;
    uint32_t c_nodes = 0, c_tris = 0, c_insts = 0;
    uint32_t ray_steps = 0;

    auto push = [&](uint2 v) {
        if (sp < kStackSize) {
            stk[sp * kTraceBlock] = v;
            sp++;
        } else {
            atomicOr(P.pool + 1, 1u);  // cannot happen within the host's depth check
        }
    };

    for (;;) {
        // warp-synchronous refill: idle lanes take new rays as soon as enough of them are idle
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
                    const float4 *rp = reinterpret_cast<const float4 *>(P.rays + rid);
                    const float4 r0 = __ldcs(rp), r1 = __ldcs(rp + 1);
                    wox = r0.x;
                    woy = r0.y;
                    woz = r0.z;
                    tmin = r0.w;
                    wdx = r1.x;
                    wdy = r1.y;
                    wdz = r1.z;
                    best_t = r1.w;
                    best_u = best_v = 0.0f;
                    best_inst = best_prim = kInvalid;
                    ox = wox;
                    oy = woy;
                    oz = woz;
                    ix = slab_rcp(wdx);
                    iy = slab_rcp(wdy);
                    iz = slab_rcp(wdz);
                    octinv = octant_inv(wdx, wdy, wdz);
                    // a zero direction meets nothing; skip the walk
                    G = (wdx == 0.0f && wdy == 0.0f && wdz == 0.0f) ? make_uint2(0, 0) : root_group(octinv);
                    sp = 0;
                    in_blas = false;
                    occluded = false;
                    ray_steps = 0;
                    if (kCount) c_nodes = c_tris = c_insts = 0;
                }
            }
        }
        if (__ballot_sync(~0u, active) == 0u) {
            if (exhausted) break;
            continue;
        }
        if (!active) continue;

        // ---- one traversal step: visit one node (or take a popped item group), then its items
        bool done = false;
        if (++ray_steps > kMaxRaySteps) {
            atomicOr(P.pool + 1, 2u);
            done = true;
        } else {
            uint2 Gt;
            if (G.y >= 0x01000000u) {
                const uint32_t key = __ffs(G.y >> 24) - 1u;
                G.y &= ~(1u << (24 + key));
                const uint32_t slot = key ^ octinv;
                const uint32_t child = G.x + __popc(G.y & 0xffu & ((1u << slot) - 1u));
                if (G.y >= 0x01000000u) push(G);
                const void *nodes = in_blas ? blas_nodes : tlas_nodes;
                if (kLayout == LCX_NODES_QUANT8)
                    intersect_q(static_cast<const Node8Q *>(nodes), child, ox, oy, oz, ix, iy, iz, octinv, tmin,
                                best_t, G, Gt);
                else
                    intersect_f(static_cast<const Node8F *>(nodes), child, ox, oy, oz, ix, iy, iz, octinv, tmin,
                                best_t, G, Gt);
                if (kCount) c_nodes++;
            } else {
                Gt = G;
                G = make_uint2(0, 0);
            }

            if (in_blas) {
                while (Gt.y) {
                    // postpone the triangles of a lane that would test them nearly alone,
                    // while it still has nodes to walk in the meantime
                    if (postpone > 0 && G.y >= 0x01000000u && sp < postpone_sp &&
                        int(__popc(__activemask())) < postpone) {
                        push(Gt);
                        break;
                    }
                    const uint32_t k = __ffs(Gt.y) - 1u;
                    Gt.y &= Gt.y - 1u;
                    const float4 *tp = reinterpret_cast<const float4 *>(blas_tris + Gt.x + k);
                    const float4 a = __ldg(tp), b = __ldg(tp + 1), c = __ldg(tp + 2);
                    if (kCount) c_tris++;
                    float t, u, v;
                    if (wt_intersect(wt, tmin, best_t, a, b, c, t, u, v)) {
                        if (kAny) {
                            occluded = true;
                            break;
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
                if (kAny && occluded) done = true;
            } else {
                while (Gt.y) {
                    const uint32_t k = __ffs(Gt.y) - 1u;
                    Gt.y &= Gt.y - 1u;
                    const uint4 *ip = reinterpret_cast<const uint4 *>(P.insts + Gt.x + k);
                    const uint4 m4 = __ldg(ip + 4);  // fnodes (x,y), inst_id (z), mask (w)
                    if ((m4.w & P.mask) == 0u) continue;
                    const float4 r0 = __ldg(reinterpret_cast<const float4 *>(ip));
                    const float4 r1 = __ldg(reinterpret_cast<const float4 *>(ip + 1));
                    const float4 r2 = __ldg(reinterpret_cast<const float4 *>(ip + 2));
                    const uint4 pp = __ldg(ip + 3);  // qnodes (x,y), tris (z,w)
                    if (Gt.y) push(Gt);
                    if (G.y) push(G);
                    const float w[12] = {r0.x, r0.y, r0.z, r0.w, r1.x, r1.y, r1.z, r1.w, r2.x, r2.y, r2.z, r2.w};
                    float dx, dy, dz;
                    transform_point(w, wox, woy, woz, ox, oy, oz);
                    transform_dir(w, wdx, wdy, wdz, dx, dy, dz);
                    ix = slab_rcp(dx);
                    iy = slab_rcp(dy);
                    iz = slab_rcp(dz);
                    octinv = octant_inv(dx, dy, dz);
                    wt = wt_setup(ox, oy, oz, dx, dy, dz);
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
                    break;
                }
            }

            if (!done && G.y == 0u) {
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
                if (sp == 0) {
                    done = true;
                } else {
                    sp--;
                    G = stk[sp * kTraceBlock];
                }
            }
        }
        if (done) {
            if (kAny) {
                P.occluded[rid] = occluded ? 1 : 0;
            } else {
                uint2 *hp = reinterpret_cast<uint2 *>(P.hits + rid);
                __stcs(hp, make_uint2(best_inst, best_prim));
                __stcs(hp + 1, make_uint2(__float_as_uint(best_u), __float_as_uint(best_v)));
                __stcs(hp + 2, make_uint2(__float_as_uint(best_t), 0u));
            }
            if (kCount) {
                P.counts[3ull * rid + 0] = c_nodes;
                P.counts[3ull * rid + 1] = c_tris;
                P.counts[3ull * rid + 2] = c_insts;
            }
            active = false;
        }
    }
}

template <int L, bool A, bool C>
int blocks_per_sm() {
    static int v = 0;
    if (v == 0) {
        int b = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_trace<L, A, C>, kTraceBlock, 0);
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

template <int L, bool A, bool C>
cudaError_t launch_one(const TraceParams &p, cudaStream_t st) {
    const uint64_t warps_needed = (uint64_t(p.ray_count) + 31) / 32;
    uint64_t grid = uint64_t(sm_count()) * blocks_per_sm<L, A, C>();
    const uint64_t grid_need = (warps_needed + (kTraceBlock / 32) - 1) / (kTraceBlock / 32);
    if (grid_need < grid) grid = grid_need;
    if (grid == 0) grid = 1;
    k_trace<L, A, C><<<unsigned(grid), kTraceBlock, 0, st>>>(p);
    return cudaGetLastError();
}

}  // namespace

cudaError_t launch_trace(const TraceParams &p, int layout, bool any, bool counting, cudaStream_t st) {
    if (layout == LCX_NODES_QUANT8) {
        if (any) return launch_one<LCX_NODES_QUANT8, true, false>(p, st);
        if (counting) return launch_one<LCX_NODES_QUANT8, false, true>(p, st);
        return launch_one<LCX_NODES_QUANT8, false, false>(p, st);
    }
    if (any) return launch_one<LCX_NODES_FP32, true, false>(p, st);
    if (counting) return launch_one<LCX_NODES_FP32, false, true>(p, st);
    return launch_one<LCX_NODES_FP32, false, false>(p, st);
}

int trace_grid_blocks(int layout, bool any, bool counting) {
    if (layout == LCX_NODES_QUANT8) {
        if (any) return sm_count() * blocks_per_sm<LCX_NODES_QUANT8, true, false>();
        if (counting) return sm_count() * blocks_per_sm<LCX_NODES_QUANT8, false, true>();
        return sm_count() * blocks_per_sm<LCX_NODES_QUANT8, false, false>();
    }
    if (any) return sm_count() * blocks_per_sm<LCX_NODES_FP32, true, false>();
    if (counting) return sm_count() * blocks_per_sm<LCX_NODES_FP32, false, true>();
    return sm_count() * blocks_per_sm<LCX_NODES_FP32, false, false>();
}

}  // namespace lcx
