// User kernels that edit and read an accel's instances in place through
// include/lcx/accel_instances.cuh (compiled by tests/test_instances_gpu.py as
// a user would compile them).
#include <cuda_runtime.h>

#include "lcx/accel_instances.cuh"
#include "lcx_accel.h"

namespace {

// Instance i: new row-major affine (or, for odd i, the same matrix given
// column-major as the DSL's float4x4), new mask, user id 1000 + i, opacity i % 2.
__global__ void k_edit(lcx::InstanceBuffer b, const float *affines, const uint32_t *masks, uint32_t n) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float *m = affines + 12ull * i;
    if (i & 1u) {
        float cols[4][4];
        for (int c = 0; c < 4; c++) {
            for (int r = 0; r < 3; r++) cols[c][r] = m[4 * r + c];
            cols[c][3] = c == 3 ? 1.0f : 0.0f;
        }
        lcx::set_instance_transform_cols(b, i, cols);
    } else {
        lcx::set_instance_transform(b, i, m);
    }
    lcx::set_instance_visibility(b, i, masks[i]);
    lcx::set_instance_user_id(b, i, 1000u + i);
    lcx::set_instance_opacity(b, i, (i & 1u) != 0u);
}

// Reads n records back (indices >= the buffer's count give the defaults).
__global__ void k_read(lcx::InstanceBuffer b, uint32_t n, float *affines, uint32_t *masks, uint32_t *user_ids,
                       uint32_t *opaque) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    lcx::instance_transform(b, i, affines + 12ull * i);
    masks[i] = lcx::instance_visibility(b, i);
    user_ids[i] = lcx::instance_user_id(b, i);
    opaque[i] = lcx::instance_opaque(b, i) ? 1u : 0u;
}

// Motion keyframe `key` of instances 0..n-1: read the old one into `old` (12 floats; untouched when
// the instance has no such keyframe), write `m` + 12 i, and report which reads succeeded.
__global__ void k_motion_key(lcx::InstanceBuffer b, uint32_t n, uint32_t key, const float *m, float *old,
                             uint32_t *found) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    found[i] = lcx::instance_motion_matrix(b, i, key, old + 12ull * i) ? 1u : 0u;
    lcx::set_instance_motion_matrix(b, i, key, m + 12ull * i);
}

lcx::InstanceBuffer as_buffer(const LcxInstanceBuffer *b) {
    return lcx::InstanceBuffer{static_cast<lcx::InstState *>(b->states), b->count, 0u};
}

}  // namespace

extern "C" __attribute__((visibility("default"))) int inst_edit(const LcxInstanceBuffer *b, const float *affines,
                                                                const uint32_t *masks, uint32_t n, void *stream) {
    if (!b || !affines || !masks || n > b->count) return -1;
    if (n == 0) return 0;
    k_edit<<<(n + 127) / 128, 128, 0, static_cast<cudaStream_t>(stream)>>>(as_buffer(b), affines, masks, n);
    return cudaGetLastError() == cudaSuccess ? 0 : -5;
}

extern "C" __attribute__((visibility("default"))) int inst_read(const LcxInstanceBuffer *b, uint32_t n, float *affines,
                                                                uint32_t *masks, uint32_t *user_ids, uint32_t *opaque) {
    if (!b || !affines || !masks || !user_ids || !opaque) return -1;
    if (n == 0) return 0;
    k_read<<<(n + 127) / 128, 128>>>(as_buffer(b), n, affines, masks, user_ids, opaque);
    return cudaGetLastError() == cudaSuccess ? 0 : -5;
}

extern "C" __attribute__((visibility("default"))) int inst_motion_key(const LcxInstanceBuffer *b, uint32_t n,
                                                                      uint32_t key, const float *m, float *old,
                                                                      uint32_t *found) {
    if (!b || !m || !old || !found) return -1;
    if (n == 0) return 0;
    k_motion_key<<<(n + 127) / 128, 128>>>(as_buffer(b), n, key, m, old, found);
    return cudaGetLastError() == cudaSuccess ? 0 : -5;
}
