// node_test.cuh — the ray / wide-node test of the traversal (both node
// layouts), shared by the persistent trace kernels and by lcx::ray_query in
// user kernels.
//
// A node test takes the ray in the current space (origin, IEEE reciprocal of
// the direction, octant) and its interval, and returns the node group (the
// hit internal children, as bits 24..31 of a hit word in front-to-back order,
// with the child base and the internal-child mask) and the item group (the
// hit leaf items, bits 0..23 with the item base).
#pragma once

#include "lcx/bvh_device.cuh"

namespace lcx {

__device__ __forceinline__ uint2 root_group(uint32_t octinv) {
    // visit node 0 (slot 0 internal, imask = 1); key of slot 0 is 0 ^ octinv
    return make_uint2(0u, (1u << (24 + octinv)) | 1u);
}

__device__ __forceinline__ uint32_t octant_inv(float dx, float dy, float dz) {
    return ((dx < 0.0f ? 1u : 0u) | (dy < 0.0f ? 2u : 0u) | (dz < 0.0f ? 4u : 0u)) ^ 7u;
}

// byte k of w as the float 2^23 + byte (exact): one PRMT
__device__ __forceinline__ float byte_magic(uint32_t w, uint32_t k) {
    return __uint_as_float(__byte_perm(w, 0x4B000000u, 0x7540u | k));
}

// Hit word contribution of a slot: (bits << index), index of internal slots
// reordered by the ray octant.
__device__ __forceinline__ uint32_t slot_bits(uint32_t meta, uint32_t octinv) {
    uint32_t idx = meta & 31u;
    idx ^= ((meta & 0x18u) == 0x18u) ? octinv : 0u;
    return (meta >> 5) << idx;
}

// Measured on GB300 (terrain workload, 8.4M incoherent rays): the word-wide
// meta decode raised closest hit 1.664 -> 1.771 Grays/s and any hit 3.03 ->
// 3.23; the three-input min/max made no difference, so it stays off.
#ifndef LCX_META_BYTEPAR
#define LCX_META_BYTEPAR 1  // decode the meta bytes of four slots with word operations
#endif
#ifndef LCX_MINMAX3
#define LCX_MINMAX3 0  // three-input float min/max for the slab distances
#endif

// The meta bytes of four slots at once (the compressed-wide-BVH decode of
// Ylitie, Karras & Laine 2017): per byte, the hit-word index (internal slots
// 24 + (slot ^ octant), leaves their item offset) and the bits to set there.
// A byte is internal iff its bits 3 and 4 are both set; the flag, moved to
// bit 0 of its byte, times 0xff fills the byte (no carry between bytes).
__device__ __forceinline__ uint32_t meta4(uint32_t m, uint32_t oct4, uint32_t &idx4, uint32_t &bits4) {
    const uint32_t inner = (m & (m << 1)) & 0x10101010u;
    const uint32_t inner_mask = (inner >> 4) * 0xffu;
    idx4 = (m ^ (oct4 & inner_mask)) & 0x1f1f1f1fu;
    bits4 = (m >> 5) & 0x07070707u;
    // the four internal flags as bits 0..3: flag i sits at bit 8i, and the
    // product's term for i lands at bit 21 + i with no carry from lower terms
    return (((inner >> 4) * 0x00204081u) >> 21) & 0xfu;
}

// Entry and exit distances of a slab test: max / min of the three planes and
// the ray interval.  IEEE min/max ignore a NaN operand (a ray lying in a box
// face gives 0 * inf); the three-input forms behave the same way.
__device__ __forceinline__ float entry4(float a, float b, float c, float tmin) {
#if LCX_MINMAX3
    float d;
    asm("max.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(fmaxf(c, tmin)));
    return d;
#else
    return fmaxf(fmaxf(a, b), fmaxf(c, tmin));
#endif
}
__device__ __forceinline__ float exit4(float a, float b, float c, float tmax) {
#if LCX_MINMAX3
    float d;
    asm("min.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(fminf(c, tmax)));
    return d;
#else
    return fminf(fminf(a, b), fminf(c, tmax));
#endif
}

// Quantised node: planes are p + e*q; with M = 2^23 + q (one PRMT) the
// decode t = (p - o)/d + q*e/d becomes fma(M, e/d, (p - o)/d - 2^23 e/d).
// The folded constant loses up to half a step, which the build-side one-step
// outward dilation absorbs; the 2^-20 widening of (p - o)/d covers its own
// rounding (and 1/d ~ 1e30 when d ~ 0).
__device__ __forceinline__ void intersect_q(const Node8Q *nodes, uint32_t idx, float ox, float oy, float oz,
                                            float ix, float iy, float iz, uint32_t octinv, float tmin, float tmax,
                                            uint2 &G, uint2 &Gt) {
    const uint4 *p = reinterpret_cast<const uint4 *>(nodes + idx);
    const uint4 n0 = bvh_ld(p), n1 = bvh_ld(p + 1), n2 = bvh_ld(p + 2), n3 = bvh_ld(p + 3), n4 = bvh_ld(p + 4);
    const float adx = __uint_as_float((n0.w & 0xffu) << 23) * ix;
    const float ady = __uint_as_float(((n0.w >> 8) & 0xffu) << 23) * iy;
    const float adz = __uint_as_float(((n0.w >> 16) & 0xffu) << 23) * iz;
    const float aox = (__uint_as_float(n0.x) - ox) * ix;
    const float aoy = (__uint_as_float(n0.y) - oy) * iy;
    const float aoz = (__uint_as_float(n0.z) - oz) * iz;
    const float fx = __fmaf_rn(-8388608.0f, adx, aox), fy = __fmaf_rn(-8388608.0f, ady, aoy),
                fz = __fmaf_rn(-8388608.0f, adz, aoz);
    const float slx = fabsf(aox) * 0x1p-20f, sly = fabsf(aoy) * 0x1p-20f, slz = fabsf(aoz) * 0x1p-20f;
    const float cxn = fx - slx, cxf = fx + slx, cyn = fy - sly, cyf = fy + sly, czn = fz - slz, czf = fz + slz;
    // near/far planes by ray direction sign (swap whole byte words)
    const bool nx = ix < 0.0f, ny = iy < 0.0f, nz = iz < 0.0f;
    const uint32_t nx0 = nx ? n3.z : n2.x, nx1 = nx ? n3.w : n2.y, fx0 = nx ? n2.x : n3.z, fx1 = nx ? n2.y : n3.w;
    const uint32_t ny0 = ny ? n4.x : n2.z, ny1 = ny ? n4.y : n2.w, fy0 = ny ? n2.z : n4.x, fy1 = ny ? n2.w : n4.y;
    const uint32_t nz0 = nz ? n4.z : n3.x, nz1 = nz ? n4.w : n3.y, fz0 = nz ? n3.x : n4.z, fz1 = nz ? n3.y : n4.w;
    uint32_t bits = 0;
#if LCX_META_BYTEPAR
    uint32_t idx_lo, idx_hi, cb_lo, cb_hi;
    meta4(n1.z, octinv * 0x01010101u, idx_lo, cb_lo);
    meta4(n1.w, octinv * 0x01010101u, idx_hi, cb_hi);
#endif
#pragma unroll
    for (int s = 0; s < 8; s++) {
        const uint32_t k = s & 3;
        const bool hw = s >= 4;
        const float tnx = __fmaf_rn(byte_magic(hw ? nx1 : nx0, k), adx, cxn);
        const float tfx = __fmaf_rn(byte_magic(hw ? fx1 : fx0, k), adx, cxf);
        const float tny = __fmaf_rn(byte_magic(hw ? ny1 : ny0, k), ady, cyn);
        const float tfy = __fmaf_rn(byte_magic(hw ? fy1 : fy0, k), ady, cyf);
        const float tnz = __fmaf_rn(byte_magic(hw ? nz1 : nz0, k), adz, czn);
        const float tfz = __fmaf_rn(byte_magic(hw ? fz1 : fz0, k), adz, czf);
        const float tn = entry4(tnx, tny, tnz, tmin);
        const float tf = exit4(tfx, tfy, tfz, tmax);
#if LCX_META_BYTEPAR
        const uint32_t idx = ((hw ? idx_hi : idx_lo) >> (8 * k)) & 0xffu;
        const uint32_t cb = ((hw ? cb_hi : cb_lo) >> (8 * k)) & 0xffu;
        if (slab_accept(tn, tf)) bits |= cb << idx;
#else
        const uint32_t meta = ((hw ? n1.w : n1.z) >> (8 * k)) & 0xffu;
        if (slab_accept(tn, tf)) bits |= slot_bits(meta, octinv);
#endif
    }
    G = make_uint2(n1.x, (bits >> 24) ? ((bits & 0xff000000u) | (n0.w >> 24)) : 0u);
    Gt = make_uint2(n1.y, bits & 0x00ffffffu);
}

__device__ __forceinline__ void intersect_f(const Node8F *nodes, uint32_t idx, float ox, float oy, float oz,
                                            float ix, float iy, float iz, uint32_t octinv, float tmin, float tmax,
                                            uint2 &G, uint2 &Gt) {
    const float4 *p = reinterpret_cast<const float4 *>(nodes + idx);
    const uint4 hdr = bvh_ld(reinterpret_cast<const uint4 *>(p + 12));
    const bool nx = ix < 0.0f, ny = iy < 0.0f, nz = iz < 0.0f;
    // lo_x: p[0..1], hi_x: p[2..3], lo_y: p[4..5], hi_y: p[6..7], lo_z: p[8..9], hi_z: p[10..11]
    uint32_t bits = 0, imask = 0;
#if LCX_META_BYTEPAR
    uint32_t idx_w[2], cb_w[2];
    imask = meta4(hdr.z, octinv * 0x01010101u, idx_w[0], cb_w[0]) |
            (meta4(hdr.w, octinv * 0x01010101u, idx_w[1], cb_w[1]) << 4);
#endif
#pragma unroll
    for (int half = 0; half < 2; half++) {
        const float4 lx = bvh_ld(p + 0 + half), hx = bvh_ld(p + 2 + half);
        const float4 ly = bvh_ld(p + 4 + half), hy = bvh_ld(p + 6 + half);
        const float4 lz = bvh_ld(p + 8 + half), hz = bvh_ld(p + 10 + half);
        const float LX[4] = {lx.x, lx.y, lx.z, lx.w}, HX[4] = {hx.x, hx.y, hx.z, hx.w};
        const float LY[4] = {ly.x, ly.y, ly.z, ly.w}, HY[4] = {hy.x, hy.y, hy.z, hy.w};
        const float LZ[4] = {lz.x, lz.y, lz.z, lz.w}, HZ[4] = {hz.x, hz.y, hz.z, hz.w};
#if !LCX_META_BYTEPAR
        const uint32_t mw = half ? hdr.w : hdr.z;
#endif
#pragma unroll
        for (int k = 0; k < 4; k++) {
            const float tnx = (nx ? HX[k] : LX[k]) - ox, tfx = (nx ? LX[k] : HX[k]) - ox;
            const float tny = (ny ? HY[k] : LY[k]) - oy, tfy = (ny ? LY[k] : HY[k]) - oy;
            const float tnz = (nz ? HZ[k] : LZ[k]) - oz, tfz = (nz ? LZ[k] : HZ[k]) - oz;
            const float tn = entry4(tnx * ix, tny * iy, tnz * iz, tmin);
            const float tf = exit4(tfx * ix, tfy * iy, tfz * iz, tmax);
#if LCX_META_BYTEPAR
            const uint32_t idx = (idx_w[half] >> (8 * k)) & 0xffu, cb = (cb_w[half] >> (8 * k)) & 0xffu;
            if (slab_accept(tn, tf)) bits |= cb << idx;
#else
            const uint32_t meta = (mw >> (8 * k)) & 0xffu;
            if (meta_internal(meta)) imask |= 1u << (half * 4 + k);
            if (slab_accept(tn, tf)) bits |= slot_bits(meta, octinv);
#endif
        }
    }
    G = make_uint2(hdr.x, (bits >> 24) ? ((bits & 0xff000000u) | imask) : 0u);
    Gt = make_uint2(hdr.y, bits & 0x00ffffffu);
}

}  // namespace lcx
