// bvh_device.cuh — device-side layouts and arithmetic of the sm_103a
// acceleration-structure path.
//
// HBM layout of one BVH (BLAS over triangles, TLAS over instances):
//   * wide nodes, 8 children each, stored twice:
//       Node8Q  80 B  child boxes quantised to 8 bits relative to the node box,
//                     rounded outward (5 x 16 B vector loads);
//       Node8F 208 B  child boxes in FP32 (13 x 16 B vector loads);
//     internal children of a node are contiguous from `child_base`, leaf
//     items of a node are contiguous from `item_base`, so a node names its
//     whole subtree frontier with two integers and eight meta bytes.
//   * leaf items in traversal order: TriRec (48 B, the three vertices as
//     float4, prim id in v0.w) for a BLAS, InstRec (80 B) for a TLAS.
// Child slots are assigned by octant (the child whose centroid lies toward
// octant s goes to slot s), so a ray visits slots in order s ^ (octant ^ 7),
// an approximately front-to-back order without sorting.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace lcx {

constexpr uint32_t kInvalid = 0xffffffffu;
constexpr int kWide = 8;
constexpr int kMaxLeafItems = 3;    // items per leaf slot (meta holds a 2-bit count)
constexpr int kStackSize = 32;      // traversal stack entries per thread
constexpr int kMaxLevels = 64;      // wide-tree depth limit of the collapse
constexpr uint32_t kMaxRaySteps = 1u << 22;  // default per-ray step bound: a corrupt tree ends the ray, never hangs

#ifndef LCX_L2_KEEP
#define LCX_L2_KEEP 0
#endif

// Loads of BVH data (nodes, leaf items, instance records) by the traversal:
// the read-only path.  LCX_L2_KEEP=1 adds an L2 evict-last policy, so that the
// rays and hits streaming through L2 (loaded and stored evict-first, .cs)
// would be evicted first; measured 2 % slower on the incoherent terrain
// workload (1.730 vs 1.770 Grays/s), so it is off.
__device__ __forceinline__ uint4 bvh_ld(const uint4 *p) {
#if LCX_L2_KEEP
    uint64_t pol;
    asm("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(pol));
    uint4 v;
    asm("ld.global.nc.L2::cache_hint.v4.u32 {%0, %1, %2, %3}, [%4], %5;"
        : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w)
        : "l"(p), "l"(pol));
    return v;
#else
    return __ldg(p);
#endif
}
__device__ __forceinline__ float4 bvh_ld(const float4 *p) {
    const uint4 v = bvh_ld(reinterpret_cast<const uint4 *>(p));
    return make_float4(__uint_as_float(v.x), __uint_as_float(v.y), __uint_as_float(v.z), __uint_as_float(v.w));
}

// Meta byte of a child slot: (bits << 5) | index.  A hit child contributes
// `bits << index` to a 32-bit hit word: internal children have bits = 1 and
// index 24 + slot (so their hits land in bits 24..31, reordered front to back
// by XOR with the ray's octant), leaves have bits = 2^count - 1 (count 1..3)
// and index = offset of their items (0..23).  0 = empty or unreachable.
constexpr uint32_t kMetaInternalBase = 0x38;  // (1 << 5) | 24
__host__ __device__ __forceinline__ bool meta_internal(uint32_t m) { return m != 0u && (m & 0x18u) == 0x18u; }
__host__ __device__ __forceinline__ uint32_t meta_leaf(uint32_t count, uint32_t offset) {
    return (((1u << count) - 1u) << 5) | offset;
}
__device__ __forceinline__ uint32_t meta_count(uint32_t m) { return __popc(m >> 5); }
// Quantised boxes: exponents give (hi - lo) / e <= kQuantRange and the stored
// origin is one step below the node box, so every stored plane can be moved
// one step outward; the traversal's folded decode is then conservative.
constexpr float kQuantRange = 252.0f;

struct __align__(16) Node8Q {
    float px, py, pz;   // quantisation origin (node box lower corner)
    uint32_t exps;      // ex | ey << 8 | ez << 16 | imask << 24
    uint32_t child_base;
    uint32_t item_base;
    uint32_t meta_lo, meta_hi;
    uint32_t qlo_x[2], qlo_y[2], qlo_z[2], qhi_x[2], qhi_y[2], qhi_z[2];
};
static_assert(sizeof(Node8Q) == 80, "Node8Q is 80 B");

struct __align__(16) Node8F {
    float lo_x[8], hi_x[8], lo_y[8], hi_y[8], lo_z[8], hi_z[8];
    uint32_t child_base;
    uint32_t item_base;
    uint32_t meta_lo, meta_hi;
};
static_assert(sizeof(Node8F) == 208, "Node8F is 208 B");

struct __align__(16) TriRec {
    float4 v0;  // xyz, w = prim id bits (procedural BLAS: v0 = AABB min + prim id, v1 = AABB max)
    float4 v1;
    float4 v2;
};
static_assert(sizeof(TriRec) == 48, "TriRec is 48 B");

// Vertex motion of a mesh built with a motion option (the reference's
// keyframed vertices: the vertex buffer holds `keys` copies of the
// `vcount` vertices back to back, include/luisa/runtime/rtx/mesh.h:137-139).
// Keyframes span [t0, t1] evenly; vertices are interpolated linearly per
// component at the ray's time (flags as MotionDesc: bit 0 / 1 vanish before
// t0 / after t1).
struct __align__(16) MeshMotion {
    const unsigned char *vbase;
    const unsigned char *tbase;
    uint64_t vstride;
    uint32_t vcount;  // vertices per keyframe
    uint32_t keys;
    float t0, t1;
    uint32_t flags;
    uint32_t _pad;
};
static_assert(sizeof(MeshMotion) == 48, "MeshMotion is 48 B");

// TriRec of a vertex-motion mesh: v0.w = prim id, v1.w = this marker, v2.xy =
// the mesh's MeshMotion address; the motion kernels interpolate its vertices.
constexpr uint32_t kTriMotion = 0xffffffffu;

// Device descriptor of a built BLAS (one per mesh handle, fixed address).
struct __align__(16) BlasDesc {
    const Node8Q *qnodes;
    const Node8F *fnodes;
    const TriRec *tris;
    uint32_t node_count;
    uint32_t tri_count;
    float lo[3];
    uint32_t depth;
    float hi[3];
    uint32_t valid;  // bit 0: built with at least one item; bit 1: procedural (AABB items); bit 2: curve
    const MeshMotion *motion;  // vertex motion (null: static vertices)
    // Bounding sphere around the centre of [lo, hi]: every item lies within bs_r of it.  0 or not
    // finite: none (a refit, or a descriptor not written by a build), the box alone bounds the BLAS.
    float bs_r;
    uint32_t _pad;
};
static_assert(sizeof(BlasDesc) == 80, "BlasDesc is 80 B");
// InstRec.mask of a procedural instance: its visibility mask in bits 8..15 and
// bit 31 set, so the trace kernels' test (ray mask & mask), ray masks being
// 8 bits, never enters it; lcx::ray_query decodes it.
constexpr uint32_t kInstProcedural = 0x80000000u;

// Instance as stored in TLAS leaf order.
struct __align__(16) InstRec {
    float w2o[12];            // world-to-object, row-major 3x4
    const Node8Q *qnodes;
    const TriRec *tris;
    const Node8F *fnodes;
    uint32_t inst_id;
    uint32_t mask;
};
static_assert(sizeof(InstRec) == 80, "InstRec is 80 B");

// Motion of a motion instance (AccelOption::Motion,
// include/luisa/runtime/rhi/resource.h:101-118): `count` keyframes spaced
// evenly over [t0, t1].  Matrix mode: row-major 3x4 object-to-world matrices
// (12 floats each), interpolated linearly per element.  SRT mode (flags bit
// 2): the reference's MotionInstanceTransformSRT (16 floats: pivot xyz,
// quaternion xyzw, scale xyz, shear xyz, translation xyz), every component
// interpolated linearly and the quaternion normalised, composed as
// M = T R S with S = [[sx, sh0, sh1, px], [0, sy, sh2, py], [0, 0, sz, pz]].
// flags bit 0: the instance vanishes before t0 (else the time is clamped),
// bit 1: after t1.
struct __align__(16) MotionDesc {
    const float *keys;
    uint32_t count;
    float t0, t1;
    uint32_t flags;
    uint32_t _pad[2];
};
static_assert(sizeof(MotionDesc) == 32, "MotionDesc is 32 B");

// Instance state by instance index (what Modifications edit).
struct __align__(16) InstState {
    float o2w[12];
    const BlasDesc *blas;     // null = no mesh
    uint32_t mask;
    uint32_t user_id;
    uint32_t opaque;
    uint32_t _pad0;
    const MotionDesc *motion;  // null = a static instance (o2w)
};
static_assert(sizeof(InstState) == 80, "InstState is 80 B");

// TLAS leaf records of motion instances carry this bit with the visibility mask
// shifted up by 8 (like procedural ones), so the kernels without motion support
// never enter them; the MotionDesc address sits in the first 8 bytes of w2o.
constexpr uint32_t kInstMotion = 0x40000000u;
// TLAS leaf records of curve instances carry this bit, with the visibility mask
// shifted up by 8 as well (and kInstMotion too for a motion instance of a curve):
// only the extended (motion and curve) kernels enter them.
constexpr uint32_t kInstCurve = 0x20000000u;

struct __align__(16) ModRec {  // == LcxModification with primitive translated
    uint32_t index, user_id, flags, vis_mask;
    float affine[12];
    uint64_t primitive;  // BlasDesc device address (0 = none)
    uint64_t motion;     // with a primitive: MotionDesc device address of a motion instance (0 = static)
};
static_assert(sizeof(ModRec) == 80, "ModRec is 80 B");

struct __align__(16) Ray {
    float ox, oy, oz, tmin;
    float dx, dy, dz, tmax;
};

struct __align__(8) Hit {
    uint32_t inst, prim;
    float u, v;
    float t;
    uint32_t pad;
};

// ------------------------------------------------------------------------
// The FP32 operation sequences below are reproduced bit for bit by the
// oracle (explicit fma, every other operation separately rounded).

// Affine inverse of a row-major 3x4 object-to-world matrix
// (include/luisa/runtime/rhi/command.h:557-571 layout).
__device__ __forceinline__ void affine_inverse(const float *m, float *w) {
    const float a = m[0], b = m[1], c = m[2];
    const float d = m[4], e = m[5], f = m[6];
    const float g = m[8], h = m[9], i = m[10];
    const float c00 = __fmaf_rn(e, i, -__fmul_rn(f, h));
    const float c01 = __fmaf_rn(f, g, -__fmul_rn(d, i));
    const float c02 = __fmaf_rn(d, h, -__fmul_rn(e, g));
    const float det = __fmaf_rn(a, c00, __fmaf_rn(b, c01, __fmul_rn(c, c02)));
    const float r = __frcp_rn(det);  // the correctly rounded 1 / det
    float R[9];
    R[0] = __fmul_rn(c00, r);
    R[1] = __fmul_rn(__fmaf_rn(c, h, -__fmul_rn(b, i)), r);
    R[2] = __fmul_rn(__fmaf_rn(b, f, -__fmul_rn(c, e)), r);
    R[3] = __fmul_rn(c01, r);
    R[4] = __fmul_rn(__fmaf_rn(a, i, -__fmul_rn(c, g)), r);
    R[5] = __fmul_rn(__fmaf_rn(c, d, -__fmul_rn(a, f)), r);
    R[6] = __fmul_rn(c02, r);
    R[7] = __fmul_rn(__fmaf_rn(b, g, -__fmul_rn(a, h)), r);
    R[8] = __fmul_rn(__fmaf_rn(a, e, -__fmul_rn(b, d)), r);
    const float tx = m[3], ty = m[7], tz = m[11];
#pragma unroll
    for (int k = 0; k < 3; k++) {
        w[4 * k + 0] = R[3 * k + 0];
        w[4 * k + 1] = R[3 * k + 1];
        w[4 * k + 2] = R[3 * k + 2];
        w[4 * k + 3] = -__fmaf_rn(R[3 * k + 0], tx, __fmaf_rn(R[3 * k + 1], ty, __fmul_rn(R[3 * k + 2], tz)));
    }
}

// Object-to-world matrix of a motion instance at `time`; false when the
// instance has vanished at that time.  Segment and fraction:
// u = (time - t0) / (t1 - t0) clamped to [0, 1] (NaN -> 0), x = u (count - 1),
// i = min(floor(x), count - 2), f = x - i; element k = fma(f, K1[k] - K0[k], K0[k]).
// SRT mode: M = T R S from an interpolated SRT record (16 floats).  The
// quaternion is normalised by 1 / sqrt(|q|^2); a zero quaternion gives NaN
// (the instance is then missed), as an invalid rotation would anywhere.
__device__ __forceinline__ void srt_matrix(const float *v, float m[12]) {
    const float px = v[0], py = v[1], pz = v[2];
    float qx = v[3], qy = v[4], qz = v[5], qw = v[6];
    const float sx = v[7], sy = v[8], sz = v[9], a = v[10], b = v[11], c = v[12];
    const float tx = v[13], ty = v[14], tz = v[15];
    const float n2 = __fmaf_rn(qx, qx, __fmaf_rn(qy, qy, __fmaf_rn(qz, qz, __fmul_rn(qw, qw))));
    const float rn = __frcp_rn(__fsqrt_rn(n2));
    qx = __fmul_rn(qx, rn);
    qy = __fmul_rn(qy, rn);
    qz = __fmul_rn(qz, rn);
    qw = __fmul_rn(qw, rn);
    const float xx = __fmul_rn(qx, qx), yy = __fmul_rn(qy, qy), zz = __fmul_rn(qz, qz);
    const float xy = __fmul_rn(qx, qy), xz = __fmul_rn(qx, qz), yz = __fmul_rn(qy, qz);
    const float wx = __fmul_rn(qw, qx), wy = __fmul_rn(qw, qy), wz = __fmul_rn(qw, qz);
    const float R[9] = {
        __fsub_rn(1.0f, __fmul_rn(2.0f, __fadd_rn(yy, zz))), __fmul_rn(2.0f, __fsub_rn(xy, wz)),
        __fmul_rn(2.0f, __fadd_rn(xz, wy)),
        __fmul_rn(2.0f, __fadd_rn(xy, wz)), __fsub_rn(1.0f, __fmul_rn(2.0f, __fadd_rn(xx, zz))),
        __fmul_rn(2.0f, __fsub_rn(yz, wx)),
        __fmul_rn(2.0f, __fsub_rn(xz, wy)), __fmul_rn(2.0f, __fadd_rn(yz, wx)),
        __fsub_rn(1.0f, __fmul_rn(2.0f, __fadd_rn(xx, yy)))};
    // S columns: (sx, 0, 0), (a, sy, 0), (b, c, sz), (px, py, pz)
#pragma unroll
    for (int r = 0; r < 3; r++) {
        const float r0 = R[3 * r], r1 = R[3 * r + 1], r2 = R[3 * r + 2];
        m[4 * r + 0] = __fmul_rn(r0, sx);
        m[4 * r + 1] = __fmaf_rn(r0, a, __fmul_rn(r1, sy));
        m[4 * r + 2] = __fmaf_rn(r0, b, __fmaf_rn(r1, c, __fmul_rn(r2, sz)));
        m[4 * r + 3] = __fadd_rn(__fmaf_rn(r0, px, __fmaf_rn(r1, py, __fmul_rn(r2, pz))), r == 0 ? tx : (r == 1 ? ty : tz));
    }
}

// Keyframe segment i and fraction f of `time` over `count` keyframes on
// [t0, t1]; false when the motion has vanished at that time.
__device__ __forceinline__ bool motion_segment(float t0, float t1, uint32_t count, uint32_t flags, float time,
                                               uint32_t &i, float &f) {
    if ((flags & 1u) && time < t0) return false;
    if ((flags & 2u) && time > t1) return false;
    float u = __fdiv_rn(__fsub_rn(time, t0), __fsub_rn(t1, t0));
    u = u >= 0.0f ? (u <= 1.0f ? u : 1.0f) : 0.0f;
    const float x = __fmul_rn(u, float(count - 1u));
    i = min(uint32_t(floorf(x)), count - 2u);
    f = __fsub_rn(x, float(i));
    return true;
}

// Vertices of triangle `prim` of a vertex-motion mesh at `time` (w = prim id
// bits in a, 0 in b and c, as a TriRec); false when vanished.  Each component
// is fma(f, K1 - K0, K0).
__device__ __forceinline__ bool motion_triangle(const MeshMotion &mm, uint32_t prim, float time, float4 &a, float4 &b,
                                                float4 &c) {
    uint32_t i;
    float f;
    if (!motion_segment(mm.t0, mm.t1, mm.keys, mm.flags, time, i, f)) return false;
    const uint32_t *t = reinterpret_cast<const uint32_t *>(mm.tbase + 12ull * prim);
    float4 *out[3] = {&a, &b, &c};
#pragma unroll
    for (int k = 0; k < 3; k++) {
        const uint64_t v = t[k];
        const float4 p0 = __ldg(reinterpret_cast<const float4 *>(mm.vbase + mm.vstride * (uint64_t(i) * mm.vcount + v)));
        const float4 p1 =
            __ldg(reinterpret_cast<const float4 *>(mm.vbase + mm.vstride * (uint64_t(i + 1u) * mm.vcount + v)));
        *out[k] = make_float4(__fmaf_rn(f, __fsub_rn(p1.x, p0.x), p0.x), __fmaf_rn(f, __fsub_rn(p1.y, p0.y), p0.y),
                              __fmaf_rn(f, __fsub_rn(p1.z, p0.z), p0.z), 0.0f);
    }
    a.w = __uint_as_float(prim);
    return true;
}

__device__ __forceinline__ bool motion_matrix(const MotionDesc &md, float time, float m[12]) {
    uint32_t i;
    float f;
    if (!motion_segment(md.t0, md.t1, md.count, md.flags, time, i, f)) return false;
    if (md.flags & 4u) {  // SRT keyframes
        const float *k0 = md.keys + 16ull * i, *k1 = k0 + 16;
        float v[16];
#pragma unroll
        for (int k = 0; k < 16; k++) v[k] = __fmaf_rn(f, __fsub_rn(k1[k], k0[k]), k0[k]);
        srt_matrix(v, m);
        return true;
    }
    const float *k0 = md.keys + 12ull * i, *k1 = k0 + 12;
#pragma unroll
    for (int k = 0; k < 12; k++) m[k] = __fmaf_rn(f, __fsub_rn(k1[k], k0[k]), k0[k]);
    return true;
}

// World ray -> object ray.
__device__ __forceinline__ void transform_point(const float *w, float x, float y, float z, float &ox, float &oy,
                                                float &oz) {
    ox = __fmaf_rn(w[0], x, __fmaf_rn(w[1], y, __fmaf_rn(w[2], z, w[3])));
    oy = __fmaf_rn(w[4], x, __fmaf_rn(w[5], y, __fmaf_rn(w[6], z, w[7])));
    oz = __fmaf_rn(w[8], x, __fmaf_rn(w[9], y, __fmaf_rn(w[10], z, w[11])));
}
__device__ __forceinline__ void transform_dir(const float *w, float x, float y, float z, float &ox, float &oy,
                                              float &oz) {
    ox = __fmaf_rn(w[0], x, __fmaf_rn(w[1], y, __fmul_rn(w[2], z)));
    oy = __fmaf_rn(w[4], x, __fmaf_rn(w[5], y, __fmul_rn(w[6], z)));
    oz = __fmaf_rn(w[8], x, __fmaf_rn(w[9], y, __fmul_rn(w[10], z)));
}

// Watertight ray/triangle test (Woop, Benthin, Wald, JCGT 2013), per-ray part.
struct WtRay {
    float ox, oy, oz;
    float Sx, Sy, Sz;
    uint32_t perm;  // kx | ky << 2 | kz << 4
};

__device__ __forceinline__ float pick3(uint32_t k, float a, float b, float c) {
    return k == 0 ? a : (k == 1 ? b : c);
}

__device__ __forceinline__ WtRay wt_setup(float ox, float oy, float oz, float dx, float dy, float dz) {
    WtRay r;
    r.ox = ox;
    r.oy = oy;
    r.oz = oz;
    const float ax = fabsf(dx), ay = fabsf(dy), az = fabsf(dz);
    const uint32_t kz = (ax >= ay) ? ((ax >= az) ? 0u : 2u) : ((ay >= az) ? 1u : 2u);
    uint32_t kx = kz + 1 == 3 ? 0 : kz + 1;
    uint32_t ky = kx + 1 == 3 ? 0 : kx + 1;
    const float dkz = pick3(kz, dx, dy, dz);
    if (dkz < 0.0f) {
        const uint32_t t = kx;
        kx = ky;
        ky = t;
    }
    const float dkx = pick3(kx, dx, dy, dz), dky = pick3(ky, dx, dy, dz);
    r.Sz = __frcp_rn(dkz);  // the correctly rounded 1 / dkz (IEEE reciprocal)
    r.Sx = __fmul_rn(dkx, r.Sz);
    r.Sy = __fmul_rn(dky, r.Sz);
    r.perm = kx | (ky << 2) | (kz << 4);
    return r;
}

// Per-triangle part: returns true for a hit with t in [tmin, tmax].
__device__ __forceinline__ bool wt_intersect(const WtRay &r, float tmin, float tmax, const float4 &v0,
                                             const float4 &v1, const float4 &v2, float &t_out, float &u_out,
                                             float &v_out) {
    const uint32_t kx = r.perm & 3u, ky = (r.perm >> 2) & 3u, kz = (r.perm >> 4) & 3u;
    const float a0 = __fsub_rn(v0.x, r.ox), a1 = __fsub_rn(v0.y, r.oy), a2 = __fsub_rn(v0.z, r.oz);
    const float b0 = __fsub_rn(v1.x, r.ox), b1 = __fsub_rn(v1.y, r.oy), b2 = __fsub_rn(v1.z, r.oz);
    const float c0 = __fsub_rn(v2.x, r.ox), c1 = __fsub_rn(v2.y, r.oy), c2 = __fsub_rn(v2.z, r.oz);
    const float Akx = pick3(kx, a0, a1, a2), Aky = pick3(ky, a0, a1, a2), Akz = pick3(kz, a0, a1, a2);
    const float Bkx = pick3(kx, b0, b1, b2), Bky = pick3(ky, b0, b1, b2), Bkz = pick3(kz, b0, b1, b2);
    const float Ckx = pick3(kx, c0, c1, c2), Cky = pick3(ky, c0, c1, c2), Ckz = pick3(kz, c0, c1, c2);
    const float Ax = __fmaf_rn(-r.Sx, Akz, Akx);
    const float Ay = __fmaf_rn(-r.Sy, Akz, Aky);
    const float Bx = __fmaf_rn(-r.Sx, Bkz, Bkx);
    const float By = __fmaf_rn(-r.Sy, Bkz, Bky);
    const float Cx = __fmaf_rn(-r.Sx, Ckz, Ckx);
    const float Cy = __fmaf_rn(-r.Sy, Ckz, Cky);
    // edge functions with separately rounded products: swapping two vertices
    // negates them exactly, which keeps shared edges watertight
    const float U = __fsub_rn(__fmul_rn(Cx, By), __fmul_rn(Cy, Bx));
    const float V = __fsub_rn(__fmul_rn(Ax, Cy), __fmul_rn(Ay, Cx));
    const float W = __fsub_rn(__fmul_rn(Bx, Ay), __fmul_rn(By, Ax));
    if ((U < 0.0f || V < 0.0f || W < 0.0f) && (U > 0.0f || V > 0.0f || W > 0.0f)) return false;
    const float det = __fadd_rn(__fadd_rn(U, V), W);
    if (det == 0.0f) return false;
    const float Az = __fmul_rn(r.Sz, Akz);
    const float Bz = __fmul_rn(r.Sz, Bkz);
    const float Cz = __fmul_rn(r.Sz, Ckz);
    const float T = __fmaf_rn(U, Az, __fmaf_rn(V, Bz, __fmul_rn(W, Cz)));
    const float t = __fdiv_rn(T, det);
    if (!(t >= tmin && t <= tmax)) return false;
    t_out = t;
    u_out = __fdiv_rn(V, det);
    v_out = __fdiv_rn(W, det);
    return true;
}

// Reciprocal for slab tests: IEEE, so a zero component gives +-inf.  A ray
// lying in a slab plane then yields 0 * inf = NaN for that plane, which
// fminf/fmaxf ignore: the slab does not constrain the ray, as it must not.
// (Clamping 1/0 to a large finite value instead lets rounding decide the
// sign of a ray that lies exactly in a box face, and culls it.)
// The approximate MUFU reciprocal (rcp.approx: 1 ulp, +-0 -> +-inf) is enough:
// the slab acceptance carries a 2^-18 relative slack.
__device__ __forceinline__ float slab_rcp(float x) {
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// Conservative slab acceptance: exit distance widened by 2^-18 relative.
__device__ __forceinline__ bool slab_accept(float tn, float tf) { return tn <= __fmaf_rn(fabsf(tf), 0x1p-18f, tf); }

// Ordered-int encoding of floats for atomicMin/atomicMax.
__device__ __forceinline__ uint32_t float_to_ordered(float f) {
    const uint32_t u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__host__ __device__ __forceinline__ float ordered_to_float(uint32_t u) {
#ifdef __CUDA_ARCH__
    return __uint_as_float((u & 0x80000000u) ? (u & 0x7fffffffu) : ~u);
#else
    union {
        uint32_t u;
        float f;
    } x;
    x.u = (u & 0x80000000u) ? (u & 0x7fffffffu) : ~u;
    return x.f;
#endif
}

// ---------------------------------------------------------------------------
// Curves (the reference's Curve, include/luisa/runtime/rtx/curve.h, with the
// bases of include/luisa/runtime/rhi/curve_basis.h:11-24).  A segment of a
// curve is the union of the balls centred on its curve c(u), u in [0, 1],
// with radius r(u); position and radius (x, y, z and w of the control points)
// follow the segment's basis.  The build converts every segment to cubic
// Bezier form (4 control points, 64 B, in a build-time array); piecewise-linear
// segments keep their two points in slots 0 and 3 (slots 1 and 2 repeat them).
//
// A cubic segment is traced as `pieces` round cones, piece k being the convex
// hull of the balls at u = k/pieces and (k+1)/pieces.  The build picks the
// count so that the chords stay within 5 % of the curve's radius: with D the
// larger of the two 4-D second differences of the Bezier points, a chord of
// parameter length h deviates from the curve by at most 0.75 D h^2 (the
// interpolation bound h^2/8 max|c''|, and |c''| <= 6 D), so
// pieces = ceil(sqrt(0.75 D / eps)) with eps = 0.05 max(r_max, 1e-3 |P3 - P0|),
// at most kCurveMaxPieces.
//
// Ends: piecewise-linear segments have spherical end caps (curve_basis.h:12-13).
// Cubic segments are open (curve_basis.h:14-22) at an end where no segment of
// the same curve goes on (the next segment of the buffer does not start where
// this one ends): a ray whose entry point lies on that end's ball, behind the
// end's tangent circle, enters the open tube and does not hit it.  Joints
// between segments keep their balls, which close the small gaps that chords of
// different directions leave.  Hits are entries only: a ray starting inside a
// segment's volume does not hit that segment.  The hit record holds the curve
// parameter u of the ball that touches the hit point, and bary.y = -1 (the
// reference's curve-hit convention, include/luisa/runtime/rtx/hit.h:29-30 and
// cpu/accel.rs:491-494).
constexpr uint32_t kTriCurve = 0xfffffffeu;        // TriRec v1.w of a cone of a curve
constexpr uint32_t kTriCurveMotion = 0xfffffffdu;  // ... of a curve with keyframed control points
enum : uint32_t { kCurveLinear = 0, kCurveBSpline = 1, kCurveCatmullRom = 2, kCurveBezier = 3 };
constexpr uint32_t kCurveMaxPieces = 32;
// Leaf record of cone k of a curve segment (each cone is its own BVH item, so
// traversal culls cones with their own tight boxes): v0 = (start ball centre,
// segment id), v1 = (end ball centre, kTriCurve), v2 = (start radius, end
// radius, k | pieces << 16, flags: bit 0 open start, bit 1 open end).
// A curve with keyframed control points (the reference's curve motion,
// include/luisa/runtime/rtx/curve.h:10): its Bezier points interpolate linearly
// between keyframes, and so do the balls (they are linear in the points), so a
// cone keeps per keyframe its two balls and is interpolated at the ray's time.
// Its record: v0 = (t0, t1, vanish flags, segment id), v1 = (keyframes, 0, 0,
// kTriCurveMotion), v2 = (address of the keyframes' balls (2 float4 each),
// k | pieces << 16, open-end flags).  The cone count of a segment is the
// largest over its keyframes.

__device__ __forceinline__ float4 f4_axpy(float a, float4 x, float4 y) {  // a x + y
    return make_float4(__fmaf_rn(a, x.x, y.x), __fmaf_rn(a, x.y, y.y), __fmaf_rn(a, x.z, y.z), __fmaf_rn(a, x.w, y.w));
}
__device__ __forceinline__ float4 f4_scale(float a, float4 x) {
    return make_float4(__fmul_rn(a, x.x), __fmul_rn(a, x.y), __fmul_rn(a, x.z), __fmul_rn(a, x.w));
}
__device__ __forceinline__ float4 f4_add(float4 x, float4 y) {
    return make_float4(__fadd_rn(x.x, y.x), __fadd_rn(x.y, y.y), __fadd_rn(x.z, y.z), __fadd_rn(x.w, y.w));
}
__device__ __forceinline__ float4 f4_sub(float4 x, float4 y) {
    return make_float4(__fsub_rn(x.x, y.x), __fsub_rn(x.y, y.y), __fsub_rn(x.z, y.z), __fsub_rn(x.w, y.w));
}

// Control points q (2 for linear, else 4) of one segment to Bezier form p[4]
// (the uniform cubic B-spline and Catmull-Rom (tension 1/2) basis changes).
__device__ __forceinline__ void curve_to_bezier(uint32_t basis, const float4 *q, float4 p[4]) {
    if (basis == kCurveLinear) {
        p[0] = p[1] = q[0];
        p[2] = p[3] = q[1];
    } else if (basis == kCurveBSpline) {  // (q0 + 4 q1 + q2)/6, (2 q1 + q2)/3, (q1 + 2 q2)/3, (q1 + 4 q2 + q3)/6
        p[0] = f4_scale(1.0f / 6.0f, f4_add(f4_axpy(4.0f, q[1], q[0]), q[2]));
        p[1] = f4_scale(1.0f / 3.0f, f4_axpy(2.0f, q[1], q[2]));
        p[2] = f4_scale(1.0f / 3.0f, f4_axpy(2.0f, q[2], q[1]));
        p[3] = f4_scale(1.0f / 6.0f, f4_add(f4_axpy(4.0f, q[2], q[1]), q[3]));
    } else if (basis == kCurveCatmullRom) {  // q1, q1 + (q2 - q0)/6, q2 - (q3 - q1)/6, q2
        p[0] = q[1];
        p[1] = f4_axpy(1.0f / 6.0f, f4_sub(q[2], q[0]), q[1]);
        p[2] = f4_axpy(-1.0f / 6.0f, f4_sub(q[3], q[1]), q[2]);
        p[3] = q[2];
    } else {
        p[0] = q[0];
        p[1] = q[1];
        p[2] = q[2];
        p[3] = q[3];
    }
}

__device__ __forceinline__ float f4_norm2(float4 x) {
    return __fadd_rn(__fadd_rn(__fmul_rn(x.x, x.x), __fmul_rn(x.y, x.y)),
                     __fadd_rn(__fmul_rn(x.z, x.z), __fmul_rn(x.w, x.w)));
}

// Round cones a segment is traced as (see above).  Every operation is
// separately rounded so that a CPU restatement gets the same count.
__device__ __forceinline__ uint32_t curve_pieces(uint32_t basis, const float4 p[4]) {
    if (basis == kCurveLinear) return 1u;
    const float4 d0 = make_float4(__fadd_rn(__fsub_rn(p[0].x, __fmul_rn(2.0f, p[1].x)), p[2].x),
                                  __fadd_rn(__fsub_rn(p[0].y, __fmul_rn(2.0f, p[1].y)), p[2].y),
                                  __fadd_rn(__fsub_rn(p[0].z, __fmul_rn(2.0f, p[1].z)), p[2].z),
                                  __fadd_rn(__fsub_rn(p[0].w, __fmul_rn(2.0f, p[1].w)), p[2].w));
    const float4 d1 = make_float4(__fadd_rn(__fsub_rn(p[1].x, __fmul_rn(2.0f, p[2].x)), p[3].x),
                                  __fadd_rn(__fsub_rn(p[1].y, __fmul_rn(2.0f, p[2].y)), p[3].y),
                                  __fadd_rn(__fsub_rn(p[1].z, __fmul_rn(2.0f, p[2].z)), p[3].z),
                                  __fadd_rn(__fsub_rn(p[1].w, __fmul_rn(2.0f, p[2].w)), p[3].w));
    const float D = __fsqrt_rn(fmaxf(f4_norm2(d0), f4_norm2(d1)));
    const float rmax = fmaxf(fmaxf(p[0].w, p[1].w), fmaxf(p[2].w, p[3].w));
    const float4 ch = make_float4(__fsub_rn(p[3].x, p[0].x), __fsub_rn(p[3].y, p[0].y), __fsub_rn(p[3].z, p[0].z), 0.0f);
    const float len = __fsqrt_rn(f4_norm2(ch));
    const float eps = __fmul_rn(0.05f, fmaxf(rmax, __fmul_rn(1e-3f, len)));
    if (!(D > 0.0f)) return 1u;  // a straight segment (or NaN input)
    if (!(eps > 0.0f)) return kCurveMaxPieces;
    const float n = ceilf(__fsqrt_rn(__fdiv_rn(__fmul_rn(0.75f, D), eps)));
    if (!(n < float(kCurveMaxPieces))) return kCurveMaxPieces;
    return n < 1.0f ? 1u : uint32_t(n);
}

// Point and radius of a Bezier segment at u (Bernstein form; exact at 0 and 1).
// The curve arithmetic below rounds every operation explicitly (no contraction),
// so every kernel that inlines it -- the trace kernels and lcx::ray_query in a
// user's kernel -- computes the same bits.
__device__ __forceinline__ float4 bezier_at(const float4 p[4], float u) {
    const float s = __fsub_rn(1.0f, u);
    const float b0 = __fmul_rn(__fmul_rn(s, s), s), b1 = __fmul_rn(__fmul_rn(__fmul_rn(3.0f, u), s), s);
    const float b2 = __fmul_rn(__fmul_rn(__fmul_rn(3.0f, u), u), s), b3 = __fmul_rn(__fmul_rn(u, u), u);
    const float4 q = make_float4(__fmul_rn(b0, p[0].x), __fmul_rn(b0, p[0].y), __fmul_rn(b0, p[0].z),
                                 __fmul_rn(b0, p[0].w));
    return f4_axpy(b3, p[3], f4_axpy(b2, p[2], f4_axpy(b1, p[1], q)));
}

// Reciprocal and square root from the MUFU approximations (about 1 ulp): the
// curve test needs neither correctly rounded, only the same bits in every
// kernel, which one fixed instruction gives.
__device__ __forceinline__ float rcp_fast(float x) {
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}
__device__ __forceinline__ float sqrt_fast(float x) {
    float r;
    asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

__device__ __forceinline__ float dot3_rn(float ax, float ay, float az, float bx, float by, float bz) {
    return __fadd_rn(__fadd_rn(__fmul_rn(ax, bx), __fmul_rn(ay, by)), __fmul_rn(az, bz));
}

// Entry of the ray o + t d into the round cone of balls (a.xyz, a.w) and
// (b.xyz, b.w) (radii >= 0): the convex hull of the two balls, the union of
// the balls along the segment with linearly interpolated radius.  A convex
// body meets a line in one interval, whose start is the smallest start among
// its parts (the two balls and the truncated cone between the circles where
// the hull touches them).  Returns true if that start lies in [tmin, tmax],
// with the ball parameter u in [0, 1] of the hit point and `part` 0 (start
// ball, behind its tangent circle), 1 (the cone) or 2 (end ball).  The ray is
// re-based at its point closest to the cone's middle, which keeps the
// quadratics well conditioned for far-away origins.
__device__ __forceinline__ bool round_cone_entry(float3 o, float3 d, float4 a, float4 b, float tmin, float tmax,
                                                 float &t_out, float &u_out, int &part) {
    const float kInf = __int_as_float(0x7f800000);
    const float dd = dot3_rn(d.x, d.y, d.z, d.x, d.y, d.z);
    const float mx = __fmul_rn(0.5f, __fadd_rn(a.x, b.x)), my = __fmul_rn(0.5f, __fadd_rn(a.y, b.y)),
                mz = __fmul_rn(0.5f, __fadd_rn(a.z, b.z));
    const float idd = rcp_fast(dd);
    const float tc = __fmul_rn(dot3_rn(__fsub_rn(mx, o.x), __fsub_rn(my, o.y), __fsub_rn(mz, o.z), d.x, d.y, d.z), idd);
    const float3 os = make_float3(__fmaf_rn(tc, d.x, o.x), __fmaf_rn(tc, d.y, o.y), __fmaf_rn(tc, d.z, o.z));
    const float3 ba = make_float3(__fsub_rn(b.x, a.x), __fsub_rn(b.y, a.y), __fsub_rn(b.z, a.z));
    const float L = sqrt_fast(dot3_rn(ba.x, ba.y, ba.z, ba.x, ba.y, ba.z));
    const float dr = __fsub_rn(a.w, b.w);
    float best = kInf;
    int bp = -1;
    // balls: smaller root of |os + t d - c|^2 = r^2
    auto ball = [&](float4 c, int which) {
        const float ocx = __fsub_rn(os.x, c.x), ocy = __fsub_rn(os.y, c.y), ocz = __fsub_rn(os.z, c.z);
        const float hb = dot3_rn(ocx, ocy, ocz, d.x, d.y, d.z);
        const float cc = __fsub_rn(dot3_rn(ocx, ocy, ocz, ocx, ocy, ocz), __fmul_rn(c.w, c.w));
        const float disc = __fsub_rn(__fmul_rn(hb, hb), __fmul_rn(dd, cc));
        if (disc < 0.0f) return;
        const float t = __fmul_rn(__fsub_rn(-hb, sqrt_fast(disc)), idd);
        if (t < best) {
            best = t;
            bp = which;
        }
    };
    float sn = 0.0f, cs = 1.0f;
    if (!(L > fabsf(dr))) {  // one ball holds the other: the larger ball alone
        ball(a.w >= b.w ? a : b, 3);
    } else {
        ball(a, 0);
        ball(b, 2);
        // the truncated cone: s = axial coordinate from a, rho = distance from the axis;
        // its side is rho cos + s sin = ra for s in [ra sin, L + rb sin]
        const float iL = rcp_fast(L);
        const float wx = __fmul_rn(ba.x, iL), wy = __fmul_rn(ba.y, iL), wz = __fmul_rn(ba.z, iL);
        sn = __fmul_rn(dr, iL);
        const float c2 = fmaxf(__fmul_rn(__fsub_rn(1.0f, sn), __fadd_rn(1.0f, sn)), 0.0f);
        cs = sqrt_fast(c2);
        const float q0x = __fsub_rn(os.x, a.x), q0y = __fsub_rn(os.y, a.y), q0z = __fsub_rn(os.z, a.z);
        const float s0 = dot3_rn(q0x, q0y, q0z, wx, wy, wz);
        const float sd = dot3_rn(d.x, d.y, d.z, wx, wy, wz);
        const float qd = dot3_rn(q0x, q0y, q0z, d.x, d.y, d.z);
        const float qq = dot3_rn(q0x, q0y, q0z, q0x, q0y, q0z);
        const float ras = __fmul_rn(a.w, sn);
        const float s_lo = ras, s_hi = __fadd_rn(L, __fmul_rn(b.w, sn));
        float lo = -kInf, hi = kInf;
        if (sd != 0.0f) {
            const float isd = rcp_fast(sd);
            const float t1 = __fmul_rn(__fsub_rn(s_lo, s0), isd), t2 = __fmul_rn(__fsub_rn(s_hi, s0), isd);
            lo = fminf(t1, t2);
            hi = fmaxf(t1, t2);
        } else if (!(s0 >= s_lo && s0 <= s_hi)) {
            lo = kInf;
        }
        // f(t) = c2 |q|^2 - s^2 + 2 ra sn s - ra^2 <= 0 inside the (one-sheeted, within the slab) cone
        const float A = __fsub_rn(__fmul_rn(c2, dd), __fmul_rn(sd, sd));
        const float hB = __fadd_rn(__fsub_rn(__fmul_rn(c2, qd), __fmul_rn(s0, sd)), __fmul_rn(ras, sd));
        const float C = __fsub_rn(__fadd_rn(__fsub_rn(__fmul_rn(c2, qq), __fmul_rn(s0, s0)),
                                            __fmul_rn(__fmul_rn(2.0f, ras), s0)),
                                  __fmul_rn(a.w, a.w));
        if (lo <= hi) {
            if (A != 0.0f) {
                const float disc = __fsub_rn(__fmul_rn(hB, hB), __fmul_rn(A, C));
                if (disc >= 0.0f) {
                    const float sq = sqrt_fast(disc);
                    const float qv = -__fadd_rn(hB, copysignf(sq, hB));
                    float r1 = __fmul_rn(qv, rcp_fast(A)), r2 = (qv != 0.0f) ? __fmul_rn(C, rcp_fast(qv)) : r1;
                    if (r1 > r2) {
                        const float tt = r1;
                        r1 = r2;
                        r2 = tt;
                    }
                    if (A > 0.0f) {
                        lo = fmaxf(lo, r1);
                        hi = fminf(hi, r2);
                    } else if (lo <= fminf(hi, r1)) {  // f <= 0 outside [r1, r2]: one side lies in the slab
                        hi = fminf(hi, r1);
                    } else {
                        lo = fmaxf(lo, r2);
                    }
                } else if (A > 0.0f) {
                    lo = kInf;
                }
            } else if (hB != 0.0f) {
                const float tr = __fmul_rn(-C, rcp_fast(__fmul_rn(2.0f, hB)));
                if (hB > 0.0f)
                    hi = fminf(hi, tr);
                else
                    lo = fmaxf(lo, tr);
            } else if (C > 0.0f) {
                lo = kInf;
            }
            if (lo <= hi && lo < best) {
                best = lo;
                bp = 1;
            }
        }
    }
    if (bp < 0) return false;
    const float t = __fadd_rn(tc, best);
    if (!(t >= tmin && t <= tmax)) return false;
    // the ball touching the hit point: on the cone side its centre sits rho tan below the point's s
    float u;
    if (bp == 0)
        u = 0.0f;
    else if (bp == 2)
        u = 1.0f;
    else if (bp == 3)
        u = a.w >= b.w ? 0.0f : 1.0f;
    else {
        const float xx = __fsub_rn(__fmaf_rn(best, d.x, os.x), a.x), xy = __fsub_rn(__fmaf_rn(best, d.y, os.y), a.y),
                    xz = __fsub_rn(__fmaf_rn(best, d.z, os.z), a.z);
        const float iL = rcp_fast(L);
        const float s = __fmul_rn(dot3_rn(xx, xy, xz, ba.x, ba.y, ba.z), iL);
        const float rho = sqrt_fast(fmaxf(__fsub_rn(dot3_rn(xx, xy, xz, xx, xy, xz), __fmul_rn(s, s)), 0.0f));
        u = fminf(fmaxf(__fmul_rn(__fsub_rn(s, __fmul_rn(__fmul_rn(rho, sn), rcp_fast(cs))), iL), 0.0f), 1.0f);
    }
    t_out = t;
    u_out = u;
    part = bp == 3 ? 1 : bp;  // a lone ball is never an open end's cap
    return true;
}

// Ball k of `pieces` along a Bezier segment: centre and radius (>= 0) at u = k / pieces.
__device__ __forceinline__ float4 curve_piece_point(const float4 p[4], uint32_t k, uint32_t pieces) {
    float4 c = k == 0 ? p[0] : k >= pieces ? p[3] : bezier_at(p, __fdiv_rn(float(k), float(pieces)));
    c.w = fmaxf(c.w, 0.0f);
    return c;
}

// The two balls of a keyframed cone at `time` (one FMA per component, as
// motion_triangle); false when the curve has vanished at that time.
__device__ __forceinline__ bool curve_motion_cone(const float4 &a, const float4 &b, const float4 &c, float time,
                                                  float4 &c0, float4 &c1) {
    uint32_t i;
    float f;
    if (!motion_segment(a.x, a.y, __float_as_uint(b.x), __float_as_uint(a.z), time, i, f)) return false;
    const float4 *kd = reinterpret_cast<const float4 *>(
                           (unsigned long long)__float_as_uint(c.x) | ((unsigned long long)__float_as_uint(c.y) << 32)) +
                       2ull * i;
    const float4 p0 = bvh_ld(kd), p1 = bvh_ld(kd + 1), q0 = bvh_ld(kd + 2), q1 = bvh_ld(kd + 3);
    c0 = make_float4(__fmaf_rn(f, __fsub_rn(q0.x, p0.x), p0.x), __fmaf_rn(f, __fsub_rn(q0.y, p0.y), p0.y),
                     __fmaf_rn(f, __fsub_rn(q0.z, p0.z), p0.z), __fmaf_rn(f, __fsub_rn(q0.w, p0.w), p0.w));
    c1 = make_float4(__fmaf_rn(f, __fsub_rn(q1.x, p1.x), p1.x), __fmaf_rn(f, __fsub_rn(q1.y, p1.y), p1.y),
                     __fmaf_rn(f, __fsub_rn(q1.z, p1.z), p1.z), __fmaf_rn(f, __fsub_rn(q1.w, p1.w), p1.w));
    return true;
}

// Entry into cone k of a curve segment's `pieces` (balls c0, c1; `flags` as in
// the leaf record) with t in [tmin, tmax]; u = the curve parameter of the hit.
__device__ __forceinline__ bool curve_piece_entry(float3 o, float3 d, float4 c0, float4 c1, uint32_t k,
                                                  uint32_t pieces, uint32_t flags, float tmin, float tmax,
                                                  float &t_out, float &u_out) {
    if (!(c0.w > 0.0f || c1.w > 0.0f)) return false;
    float t, u;
    int part;
    if (!round_cone_entry(o, d, c0, c1, tmin, tmax, t, u, part)) return false;
    if ((part == 0 && k == 0 && (flags & 1u)) || (part == 2 && k + 1 >= pieces && (flags & 2u)))
        return false;  // the open end of a cubic curve
    t_out = t;
    u_out = fminf(__fdiv_rn(__fadd_rn(float(k), u), float(pieces)), 1.0f);
    return true;
}

}  // namespace lcx
