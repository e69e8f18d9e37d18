// accel_instances.cuh — read and write an accel's instances from device code.
//
// The reference lets kernels edit a TLAS's instances in place and rebuild or
// update the accel afterwards (DSL Accel::set_instance_transform /
// set_instance_visibility / set_instance_opacity / set_instance_user_id and
// their getters; CUDA backend cuda_device_resource.h:1450-1512, which write
// the OptiX instance buffer that the next AccelBuildCommand builds from).
// Here the instances of an accel are InstState records (bvh_device.cuh) in
// device memory, handed out by lcx_accel_instance_buffer.  A kernel edits
// them with the functions below; the edits take effect at the next
// lcx_accel_build of that accel -- a refit (PREFER_UPDATE on an accel created
// with allow_update: kernels only, so a frame "kernel edits instances, TLAS
// refit, trace" can be captured in one CUDA graph) or a rebuild.  Traces
// before that build see the old instances.
//
// Every function checks the index against the buffer's count and does
// nothing (getters: return the default instance) for an index out of range.
#pragma once

#include "lcx/bvh_device.cuh"

namespace lcx {

// Matches LcxInstanceBuffer of lcx_accel.h.
struct InstanceBuffer {
    InstState *states;
    uint32_t count;
    uint32_t _pad;
};

// Row-major 3x4 object-to-world transform (the layout of
// Modification::set_transform, include/luisa/runtime/rhi/command.h:557-571).
__device__ __forceinline__ void instance_transform(const InstanceBuffer &b, uint32_t i, float m[12]) {
    for (int k = 0; k < 12; k++) m[k] = (k % 4 == k / 4) ? 1.0f : 0.0f;
    if (i >= b.count) return;
    for (int k = 0; k < 12; k++) m[k] = b.states[i].o2w[k];
}

__device__ __forceinline__ void set_instance_transform(const InstanceBuffer &b, uint32_t i, const float m[12]) {
    if (i >= b.count) return;
    for (int k = 0; k < 12; k++) b.states[i].o2w[k] = m[k];
}

// The DSL's float4x4 is column-major (m[column][row]); its last row is dropped.
__device__ __forceinline__ void set_instance_transform_cols(const InstanceBuffer &b, uint32_t i,
                                                            const float cols[4][4]) {
    float m[12];
    for (int r = 0; r < 3; r++)
        for (int c = 0; c < 4; c++) m[4 * r + c] = cols[c][r];
    set_instance_transform(b, i, m);
}

__device__ __forceinline__ uint32_t instance_visibility(const InstanceBuffer &b, uint32_t i) {
    return i < b.count ? b.states[i].mask : 0xffu;
}

__device__ __forceinline__ void set_instance_visibility(const InstanceBuffer &b, uint32_t i, uint32_t mask) {
    if (i < b.count) b.states[i].mask = mask & 0xffu;
}

__device__ __forceinline__ uint32_t instance_user_id(const InstanceBuffer &b, uint32_t i) {
    return i < b.count ? b.states[i].user_id : 0u;
}

__device__ __forceinline__ void set_instance_user_id(const InstanceBuffer &b, uint32_t i, uint32_t user_id) {
    if (i < b.count) b.states[i].user_id = user_id;
}

__device__ __forceinline__ bool instance_opaque(const InstanceBuffer &b, uint32_t i) {
    return i < b.count ? b.states[i].opaque != 0u : true;
}

// As the reference, procedural instances ignore the opacity flag.
__device__ __forceinline__ void set_instance_opacity(const InstanceBuffer &b, uint32_t i, bool opaque) {
    if (i >= b.count) return;
    const BlasDesc *d = b.states[i].blas;
    if (d != nullptr && (d->valid & 2u)) return;
    b.states[i].opaque = opaque ? 1u : 0u;
}

// Keyframes of a motion instance (the reference's instance_motion_matrix /
// set_instance_motion_matrix / instance_motion_srt / set_instance_motion_srt,
// include/luisa/dsl/rtx/accel.h:69-110).  Matrix keyframes are row-major 3x4
// (12 floats); SRT keyframes the 16-float MotionInstanceTransformSRT records
// (pivot, quaternion, scale, shear, translation).  The getters return false and
// leave `out` alone, and the setters do nothing, when instance i is out of range,
// is not a motion instance, holds the other kind of keyframe, or `key` is past
// its keyframe count.  As with the other edits, the next lcx_accel_build of the
// accel (a refit or a rebuild) takes the new keyframes into its bounds; traces
// before it see new keyframes inside old bounds.  The keyframes belong to the
// motion instance: every instance of it, in any accel, moves with them, and a
// later lcx_motion_instance_build uploads the host's keyframes over them.
__device__ __forceinline__ const MotionDesc *instance_motion(const InstanceBuffer &b, uint32_t i, bool srt,
                                                             uint32_t key) {
    if (i >= b.count) return nullptr;
    const MotionDesc *md = b.states[i].motion;
    if (md == nullptr || key >= md->count || ((md->flags & 4u) != 0u) != srt) return nullptr;
    return md;
}

__device__ __forceinline__ bool instance_motion_matrix(const InstanceBuffer &b, uint32_t i, uint32_t key,
                                                       float out[12]) {
    const MotionDesc *md = instance_motion(b, i, false, key);
    if (md == nullptr) return false;
    for (int k = 0; k < 12; k++) out[k] = md->keys[12ull * key + k];
    return true;
}

__device__ __forceinline__ void set_instance_motion_matrix(const InstanceBuffer &b, uint32_t i, uint32_t key,
                                                           const float m[12]) {
    const MotionDesc *md = instance_motion(b, i, false, key);
    if (md == nullptr) return;
    float *k0 = const_cast<float *>(md->keys) + 12ull * key;  // device memory of the motion instance
    for (int k = 0; k < 12; k++) k0[k] = m[k];
}

__device__ __forceinline__ bool instance_motion_srt(const InstanceBuffer &b, uint32_t i, uint32_t key,
                                                    float out[16]) {
    const MotionDesc *md = instance_motion(b, i, true, key);
    if (md == nullptr) return false;
    for (int k = 0; k < 16; k++) out[k] = md->keys[16ull * key + k];
    return true;
}

__device__ __forceinline__ void set_instance_motion_srt(const InstanceBuffer &b, uint32_t i, uint32_t key,
                                                        const float v[16]) {
    const MotionDesc *md = instance_motion(b, i, true, key);
    if (md == nullptr) return;
    float *k0 = const_cast<float *>(md->keys) + 16ull * key;
    for (int k = 0; k < 16; k++) k0[k] = v[k];
}

}  // namespace lcx
