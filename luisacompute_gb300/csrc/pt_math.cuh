// pt_math.cuh — sampling arithmetic of the wavefront path tracer, with a fixed
// FP32 operation sequence (explicit fma, every other operation separately
// rounded) so a CPU restatement reproduces it bit for bit.
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>

#ifndef __CUDACC__
#define __host__
#define __device__
#define __forceinline__ inline
#endif

namespace lcx {
namespace pt {

// PCG RXS-M-XS output permutation (O'Neill 2014) of a 32-bit state.
__host__ __device__ __forceinline__ uint32_t hash32(uint32_t x) {
    x = x * 747796405u + 2891336453u;
    const uint32_t w = ((x >> ((x >> 28u) + 4u)) ^ x) * 277803737u;
    return (w >> 22u) ^ w;
}

// Uniform in [0, 1) with 24 random bits, keyed by (path, bounce, dimension).
__host__ __device__ __forceinline__ float uniform(uint32_t seed, uint32_t path, uint32_t bounce, uint32_t dim) {
    const uint32_t h = hash32(hash32(hash32(path ^ seed) + bounce * 0x9E3779B9u) + dim * 0x85EBCA6Bu);
    return float(h >> 8) * 0x1p-24f;
}

#ifdef __CUDA_ARCH__
#define LCX_FMA(a, b, c) __fmaf_rn(a, b, c)
#define LCX_MUL(a, b) __fmul_rn(a, b)
#define LCX_ADD(a, b) __fadd_rn(a, b)
#define LCX_SUB(a, b) __fsub_rn(a, b)
#define LCX_DIV(a, b) __fdiv_rn(a, b)
#define LCX_SQRT(a) __fsqrt_rn(a)
#else
#define LCX_FMA(a, b, c) std::fma(a, b, c)
#define LCX_MUL(a, b) ((a) * (b))
#define LCX_ADD(a, b) ((a) + (b))
#define LCX_SUB(a, b) ((a) - (b))
#define LCX_DIV(a, b) ((a) / (b))
#define LCX_SQRT(a) std::sqrt(a)
#endif

// cos and sin of 2*pi*u for u in [0, 1): quadrant reduction, then Taylor
// polynomials of degree 10 / 11 on [0, pi/2) (error < 5e-7).
__host__ __device__ __forceinline__ void cos_sin_turn(float u, float &c, float &s) {
    const float x = LCX_MUL(u, 4.0f);
    const int q = int(x);  // 0..3
    const float a = LCX_MUL(LCX_SUB(x, float(q)), 1.57079632679f);
    const float a2 = LCX_MUL(a, a);
    // cos a = 1 - a^2/2! + a^4/4! - ... + a^10/10!
    float pc = -2.75573192e-7f;
    pc = LCX_FMA(pc, a2, 2.48015873e-5f);
    pc = LCX_FMA(pc, a2, -1.38888889e-3f);
    pc = LCX_FMA(pc, a2, 4.16666667e-2f);
    pc = LCX_FMA(pc, a2, -0.5f);
    pc = LCX_FMA(pc, a2, 1.0f);
    // sin a = a (1 - a^2/3! + ... - a^10/11!)
    float ps = -2.50521084e-8f;
    ps = LCX_FMA(ps, a2, 2.75573192e-6f);
    ps = LCX_FMA(ps, a2, -1.98412698e-4f);
    ps = LCX_FMA(ps, a2, 8.33333333e-3f);
    ps = LCX_FMA(ps, a2, -1.66666667e-1f);
    ps = LCX_FMA(ps, a2, 1.0f);
    ps = LCX_MUL(ps, a);
    switch (q & 3) {
        case 0: c = pc; s = ps; break;
        case 1: c = -ps; s = pc; break;
        case 2: c = -pc; s = -ps; break;
        default: c = ps; s = -pc; break;
    }
}

// Cosine-weighted direction around unit normal n (Malley's method with an
// orthonormal basis from Duff et al. 2017).
__host__ __device__ __forceinline__ void cosine_dir(const float n[3], float u1, float u2, float out[3]) {
    const float r = LCX_SQRT(u1);
    float c, s;
    cos_sin_turn(u2, c, s);
    const float lx = LCX_MUL(r, c), ly = LCX_MUL(r, s);
    const float lz = LCX_SQRT(fmaxf(0.0f, LCX_SUB(1.0f, u1)));
    const float sign = n[2] >= 0.0f ? 1.0f : -1.0f;
    const float a = LCX_DIV(-1.0f, LCX_ADD(sign, n[2]));
    const float b = LCX_MUL(LCX_MUL(n[0], n[1]), a);
    const float t[3] = {LCX_FMA(LCX_MUL(sign, LCX_MUL(n[0], n[0])), a, 1.0f), LCX_MUL(sign, b), LCX_MUL(-sign, n[0])};
    const float bb[3] = {b, LCX_FMA(LCX_MUL(n[1], n[1]), a, sign), -n[1]};
    for (int k = 0; k < 3; k++) out[k] = LCX_FMA(lx, t[k], LCX_FMA(ly, bb[k], LCX_MUL(lz, n[k])));
}

__host__ __device__ __forceinline__ void normalize3(float v[3]) {
    const float l2 = LCX_FMA(v[0], v[0], LCX_FMA(v[1], v[1], LCX_MUL(v[2], v[2])));
    const float inv = LCX_DIV(1.0f, LCX_SQRT(l2));
    v[0] = LCX_MUL(v[0], inv);
    v[1] = LCX_MUL(v[1], inv);
    v[2] = LCX_MUL(v[2], inv);
}

// Offset of a surface point along its normal against self-intersection: the
// integer-ULP method of Waechter & Binder (Ray Tracing Gems, ch. 6), the
// behaviour of LuisaCompute's offset_ray_origin (src/dsl/rtx/ray.cpp:16-27).
__host__ __device__ __forceinline__ float offset_coord(float p, float n) {
    const float origin = 1.0f / 32.0f, float_scale = 1.0f / 65536.0f, int_scale = 256.0f;
    const int of = int(LCX_MUL(int_scale, n));
    int bits;
#ifdef __CUDA_ARCH__
    bits = __float_as_int(p);
#else
    std::memcpy(&bits, &p, 4);
#endif
    bits += (p < 0.0f) ? -of : of;
    float pi;
#ifdef __CUDA_ARCH__
    pi = __int_as_float(bits);
#else
    std::memcpy(&pi, &bits, 4);
#endif
    return fabsf(p) < origin ? LCX_FMA(float_scale, n, p) : pi;
}

}  // namespace pt
}  // namespace lcx
