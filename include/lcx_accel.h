/*
 * lcx_accel.h — C ABI of the GB300 (sm_103a) acceleration-structure path.
 *
 * This library replaces, on one GPU, the two implementations LuisaCompute has
 * for its Mesh/Accel path:
 *   - the CPU backend's Embree calls
 *     (src/rust/luisa_compute_backend_impl/src/cpu/accel.rs:205-535), and
 *   - the CUDA backend's OptiX calls
 *     (src/backends/cuda/cuda_mesh.cpp:31-69, cuda_accel.cpp:26-318,
 *      cuda_builtin/cuda_device_resource.h:1742-1829).
 *
 * Every entry point is `extern "C"`, takes plain pointers and sizes, and
 * returns an int status (LCX_OK == 0, negative on error).  Nothing aborts:
 * where the reference asserts (LUISA_ASSERT / panic_abort!), this library
 * returns LCX_ERR_INVALID_ARG and records a message readable through
 * lcx_last_error_string().
 *
 * Memory contract (same as the reference, include/luisa/runtime/rtx/mesh.h:41):
 * vertex and triangle buffers passed to lcx_mesh_build are *borrowed* device
 * memory; they are read during the build only (the BVH keeps its own copy of
 * the triangles in traversal order), and a mesh must be rebuilt after they
 * change.  Ray and hit buffers are device pointers owned by the caller.
 *
 * Streams are `cudaStream_t` passed as `void *` (NULL = legacy default stream).
 * All work is stream-ordered; no entry point synchronises the host except
 * where its comment says so.
 */
#ifndef LCX_ACCEL_H
#define LCX_ACCEL_H

#include <stdbool.h>
#include <stddef.h>
#include <stdint.h>

#if defined(__GNUC__)
#define LCX_API __attribute__((visibility("default")))
#else
#define LCX_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- status */
enum {
    LCX_OK = 0,
    LCX_ERR_INVALID_ARG = -1,  /* bad handle, size, stride, alignment or index */
    LCX_ERR_OOM = -2,          /* device allocation failed or budget exceeded */
    LCX_ERR_NOT_BUILT = -3,    /* mesh/accel used before a successful build */
    LCX_ERR_TIMEOUT = -4,      /* a bounded device-side wait gave up */
    LCX_ERR_CUDA = -5,         /* a CUDA runtime call failed */
    LCX_ERR_DEPTH = -6,        /* BVH deeper than the traversal stack */
};

/* --------------------------------------------------------- shared records */

/* Ray: include/luisa/runtime/rtx/ray.h:10-16 (32 B, align 16).  Also the CPU
 * kernel ABI `defs::Ray` (luisa_compute_cpu_kernel_defs/src/lib.rs:42-53). */
typedef struct __attribute__((aligned(16))) LcxRay {
    float origin[3];
    float t_min;
    float direction[3];
    float t_max;
} LcxRay;

/* TriangleHit (== SurfaceHit): include/luisa/runtime/rtx/hit.h:30-46
 * (24 B, align 8).  A miss is {~0u, ~0u, (0,0), ray.t_max}, the CPU
 * backend's record (accel.rs:501-507); `inst == ~0u` is the miss test
 * (include/luisa/dsl/rtx/hit.h:67).  bary = (u, v) with
 * p = (1-u-v)*v0 + u*v1 + v*v2 (src/dsl/rtx/hit.cpp:7-20). */
typedef struct __attribute__((aligned(8))) LcxTriangleHit {
    uint32_t inst;
    uint32_t prim;
    float bary[2];
    float committed_ray_t;
    uint32_t _pad;
} LcxTriangleHit;

/* Triangle: include/luisa/runtime/rtx/triangle.h:7-11. */
typedef struct LcxTriangle {
    uint32_t i0, i1, i2;
} LcxTriangle;

/* AccelOption: include/luisa/runtime/rhi/resource.h:94-125.  Its motion part
 * is LcxMotionOption, taken by lcx_mesh_create_motion, lcx_curve_create_motion
 * and lcx_motion_instance_create. */
enum { LCX_HINT_FAST_TRACE = 0, LCX_HINT_FAST_BUILD = 1 };
typedef struct LcxAccelOption {
    uint32_t hint;            /* LCX_HINT_FAST_TRACE | LCX_HINT_FAST_BUILD */
    uint8_t allow_compaction; /* accepted for ABI parity; BVHs are always exact-size */
    uint8_t allow_update;     /* keep what a refit needs (see lcx_mesh_build, lcx_accel_build) */
    uint8_t _pad[2];
} LcxAccelOption;

/* AccelBuildRequest: include/luisa/runtime/rhi/command.h:401-404. */
enum { LCX_REQUEST_PREFER_UPDATE = 0, LCX_REQUEST_FORCE_BUILD = 1 };

/* MeshBuildCommand: include/luisa/runtime/rhi/command.h:407-444.  The buffer
 * fields are device addresses (the CUDA backend stores CUDABuffer device
 * addresses, cuda_mesh.cpp:56-61).  Checks follow src/runtime/rtx/mesh.cpp:
 * vertex_stride % 16 == 0, vertex offset/size multiples of the stride,
 * triangle offset % 4 == 0, triangle size % 12 == 0. */
typedef struct LcxMeshBuildCommand {
    uint32_t request;
    uint32_t _pad;
    uint64_t vertex_buffer;
    size_t vertex_buffer_offset;
    size_t vertex_buffer_size;
    size_t vertex_stride;
    uint64_t triangle_buffer;
    size_t triangle_buffer_offset;
    size_t triangle_buffer_size;
} LcxMeshBuildCommand;

/* AccelBuildCommand::Modification: include/luisa/runtime/rhi/command.h:534-592
 * (80 B, align 16, byte-identical).  affine is the row-major 3x4
 * object-to-world matrix (command.h:557-571).  `primitive` is a mesh handle
 * returned by lcx_mesh_create. */
enum {
    LCX_MOD_PRIMITIVE = 1u << 0,
    LCX_MOD_TRANSFORM = 1u << 1,
    LCX_MOD_OPAQUE_ON = 1u << 2,
    LCX_MOD_OPAQUE_OFF = 1u << 3,
    LCX_MOD_VISIBILITY = 1u << 4,
    LCX_MOD_USER_ID = 1u << 5,
};
typedef struct __attribute__((aligned(16))) LcxModification {
    uint32_t index;
    uint32_t user_id;
    uint32_t flags;
    uint32_t vis_mask;
    float affine[12];
    uint64_t primitive;
} LcxModification;

/* Node layout used by a trace call. */
enum {
    LCX_NODES_FP32 = 0,  /* plain: 8-wide nodes with FP32 child boxes (208 B) */
    LCX_NODES_QUANT8 = 1 /* 8-wide nodes, child boxes quantised to 8 bits
                            relative to the parent, rounded outward (80 B) */
};

typedef struct LcxAccelStats {
    uint64_t node_count;     /* wide nodes */
    uint64_t leaf_prim_count;/* triangles (BLAS) or instances (TLAS) stored */
    uint64_t device_bytes;   /* device memory owned by the handle */
    uint32_t depth;          /* wide-tree depth (root = 1) */
    uint32_t max_blas_depth; /* TLAS only: deepest referenced BLAS */
    double sah_cost;         /* SAH cost of the binary tree (C_node=1, C_tri=1,
                                normalised by the root surface area) */
    double wide_sah_cost;    /* same for the 8-wide tree (as built; a refit keeps it) */
    uint64_t refits;         /* refits since the last full build (SAH figures: that build's) */
} LcxAccelStats;

/* ------------------------------------------------------------ device setup */

/* Select the CUDA device used by later calls made from this thread and
 * create the library's per-device state.  Optional: the first call of any
 * other entry point initialises the current device. */
LCX_API int lcx_device_init(int device);

/* Message describing the last error on the calling thread ("" if none). */
LCX_API const char *lcx_last_error_string(void);

/* Library version as 0xMMmmpp. */
LCX_API uint32_t lcx_version(void);

/* ------------------------------------------------------------------- mesh */

/* DeviceInterface::create_mesh / destroy_mesh:
 * include/luisa/runtime/rhi/device_interface.h:171-172. */
LCX_API int lcx_mesh_create(const LcxAccelOption *option, uint64_t *out_handle);
LCX_API int lcx_mesh_destroy(uint64_t mesh);


/* MeshBuildCommand visit (CPU: accel.rs:205-260; CUDA: cuda_mesh.cpp:31-69).
 * Builds the BLAS on `stream`: Morton-code LBVH, collapsed to 8-wide nodes in
 * both node layouts.  Returns after enqueueing; the mesh may be used by
 * lcx_accel_build on the same stream immediately.  Synchronises the host once
 * to learn the tree size.
 * PREFER_UPDATE (the OptiX update of cuda_mesh.cpp:42-67): a mesh created with
 * allow_update and already built is refit in place -- same topology, triangle
 * records and boxes recomputed from the buffers of the command -- when its
 * triangle count is unchanged and the call covers every mesh built together
 * with it (for lcx_mesh_build_batch: the same set of meshes); otherwise it is
 * rebuilt.  Either way the accels over it must be built again.  A refit
 * synchronises the host once, to report bad indices.  Hit records are the same
 * as after a full build of the new geometry (they do not depend on topology). */
LCX_API int lcx_mesh_build(uint64_t mesh, const LcxMeshBuildCommand *command, void *stream);

/* Many MeshBuildCommands at once (no single counterpart in the reference,
 * whose backends build one Mesh per command: CPU accel.rs:205-260, CUDA
 * cuda_mesh.cpp:31-69 with one host sync each at cuda_primitive.cpp:74).
 * All meshes' triangles go through one sort, one LBVH pass, one cooperative
 * collapse and one emit into one shared device block; the host synchronises
 * once.  Results equal `count` separate lcx_mesh_build calls on the same
 * commands.  A mesh may appear once; all or none are rebuilt. */
LCX_API int lcx_mesh_build_batch(const uint64_t *meshes, const LcxMeshBuildCommand *commands, uint32_t count,
                                 void *stream);

LCX_API int lcx_mesh_stats(uint64_t mesh, LcxAccelStats *out);

/* ------------------------------------------------------ procedural primitive */

/* ProceduralPrimitiveBuildCommand: include/luisa/runtime/rhi/command.h:488-512
 * (CPU backend: accel.rs:84-141, Embree user geometry).  aabb_buffer: device
 * address of `Aabb` records {float min[3]; float max[3];} (24 B,
 * src/rust/luisa_compute_cpu_kernel_defs/src/lib.rs:56-59); size in bytes. */
typedef struct LcxProceduralBuildCommand {
    uint32_t request;          /* LCX_REQUEST_* */
    uint32_t _pad;
    uint64_t aabb_buffer;
    size_t aabb_buffer_offset;
    size_t aabb_buffer_size;
} LcxProceduralBuildCommand;

/* DeviceInterface::create_procedural_primitive / destroy_procedural_primitive:
 * device_interface.h:174-175.  A procedural primitive is a BLAS over AABBs; an
 * accel instances it like a mesh (Modification.primitive = its handle).  The
 * trace calls (lcx_trace_*) do not see procedural instances, as the
 * reference's trace_closest / trace_any do not; lcx::ray_query
 * (include/lcx/ray_query.cuh) offers their AABB candidates to a callback that
 * commits its own distance. */
LCX_API int lcx_procedural_create(const LcxAccelOption *option, uint64_t *out_handle);
LCX_API int lcx_procedural_destroy(uint64_t handle);
/* Builds a batch like lcx_mesh_build_batch and reserves it for rebuilds
 * captured in CUDA graphs: the batch's block gets room for any tree over the
 * same triangles (wide nodes <= triangles + meshes) and keeps its segment
 * table on the device.  A later lcx_mesh_build_batch (or a single-mesh batch's
 * lcx_mesh_build) of the same meshes, in the same order, over the same
 * buffers, sizes and strides -- the vertices may have moved -- rebuilds the
 * BVHs in place with kernels only: no host synchronisation, no allocation
 * outside stream-ordered scratch, so it can be captured.  Such rebuilds
 * report errors through lcx_check_trace_errors, and lcx_mesh_stats keeps the
 * reserving build's figures.  Splitting is off for reserved batches; meshes
 * with allow_update or vertex motion are refused.  Synchronises the host
 * once (as a batch build).  No counterpart in the reference, whose builds
 * synchronise per mesh (cuda_primitive.cpp:74). */
LCX_API int lcx_mesh_build_batch_reserve(const uint64_t *meshes, const LcxMeshBuildCommand *cmds,
                                         uint32_t count, void *stream);
/* Reserves a batch without building it: the same block lcx_mesh_build_batch_reserve keeps (room
 * for any tree over the batch's triangles: triangles + meshes wide nodes, the segment table and
 * the initial control words on the device), allocated and uploaded with one synchronisation, and
 * no build.  The batch's first build is then the next lcx_mesh_build_batch of the same meshes, in
 * the same order, over the same buffers: it runs the reserved-rebuild kernels only, with no host
 * synchronisation and no allocation of its own (stream-ordered scratch), so it can be captured in
 * a CUDA graph together with what follows it.  Until that build has run on the stream the meshes
 * are empty to a TLAS build.  Their statistics stay zero (node count, depth, SAH) until a
 * synchronising build; a tree deeper than the traversal stack is reported by
 * lcx_check_trace_errors.  Errors of the in-graph build (bad indices) go to the same asynchronous
 * error word.  Triangle meshes without allow_update or motion.  Replaces the reference's per-mesh
 * build with a host sync each (cuda_primitive.cpp:20-113, sync at :74). */
LCX_API int lcx_mesh_reserve_batch(const uint64_t *meshes, const LcxMeshBuildCommand *cmds, uint32_t count,
                                   void *stream);

/* Builds (PREFER_UPDATE with allow_update: refits) on `stream`, like
 * lcx_mesh_build.  Empty boxes (min > max on an axis) are never reported. */
LCX_API int lcx_procedural_build(uint64_t handle, const LcxProceduralBuildCommand *command, void *stream);

/* ------------------------------------------------------------------ curve */

/* CurveBasis (include/luisa/runtime/rhi/curve_basis.h:11-24): 2 control points
 * per segment for PIECEWISE_LINEAR, 4 for the others. */
#define LCX_CURVE_PIECEWISE_LINEAR 0u
#define LCX_CURVE_CUBIC_BSPLINE 1u
#define LCX_CURVE_CATMULL_ROM 2u
#define LCX_CURVE_BEZIER 3u

/* CurveBuildCommand (include/luisa/runtime/rhi/command.h:446-486; C ABI
 * src/rust/luisa_compute_api_types/src/lib.rs:620-631).  Control points are
 * float4 {x, y, z, radius} records `cp_stride` bytes apart (>= 16 and a multiple of 4, as the reference's
 * Embree path requires, cpu/accel.rs:160); the segment buffer holds one u32 per
 * segment, the index of its first control point. */
typedef struct LcxCurveBuildCommand {
    uint32_t request;  /* LCX_REQUEST_* */
    uint32_t basis;    /* LCX_CURVE_* */
    uint64_t cp_buffer;
    size_t cp_buffer_offset;
    size_t cp_stride;
    size_t cp_count;
    uint64_t seg_buffer;
    size_t seg_buffer_offset;
    size_t seg_count;
} LcxCurveBuildCommand;

/* DeviceInterface::create_curve / destroy_curve (device_interface.h:177-178).  A curve
 * is a BLAS over its segments; an accel instances it like a mesh
 * (Modification.primitive = its handle), with a transform, a mask and motion
 * instances (lcx_motion_instance_create) as for meshes.  Segment i is the
 * union of balls along its curve (position and radius from the basis); hits
 * report prim = i, bary = (u, -1) with u the curve parameter of the hit, and
 * the ray's t (hit.h:29-30).  Linear segments have spherical end caps; cubic
 * segments are open where the next segment of the buffer does not continue
 * them.  Cubic segments are traced as up to 32 round cones whose chords stay
 * within 5 % of the radius of the exact curve (the BLAS items are the cones:
 * lcx_mesh_stats counts them); hits are entries only (a ray starting inside a
 * segment does not hit it).  Accels holding curves trace with
 * the extended kernels (those of motion), through lcx_trace_* and the
 * *_motion / *_host / *_ex entry points and lcx_trace_jobs (a group with a
 * curve job runs the curve kernel); lcx::ray_query offers curve segments as
 * surface candidates with bary_v = -1. */
LCX_API int lcx_curve_create(const LcxAccelOption *option, uint64_t *out_handle);
LCX_API int lcx_curve_destroy(uint64_t handle);
/* Builds on `stream` (every request rebuilds: the reference's PREFER_UPDATE
 * refit of the control points gives the same hits as a rebuild).  Errors: a
 * segment whose control points run past cp_count (LCX_ERR_INVALID_ARG); a
 * build inside a CUDA graph capture. */
LCX_API int lcx_curve_build(uint64_t handle, const LcxCurveBuildCommand *command, void *stream);

/* ------------------------------------------------------------------ accel */

/* DeviceInterface::create_accel / destroy_accel: device_interface.h:183-184. */
LCX_API int lcx_accel_create(const LcxAccelOption *option, uint64_t *out_handle);
LCX_API int lcx_accel_destroy(uint64_t accel);

/* AccelBuildCommand visit (CPU: accel.rs:324-447; CUDA: cuda_accel.cpp:152-318
 * with the update_accel kernel, cuda_builtin_kernels.cu:52-111).
 * `mods` is host memory (the command's vector).  Instance i keeps its mesh,
 * transform, mask (default 0xff), opacity and user id until modified.
 * instance_count == 0 is an error, as in src/runtime/rtx/accel.cpp:72-73.
 * update_instance_buffer_only != 0 stores the modifications without
 * rebuilding the TLAS.  PREFER_UPDATE on an accel created with allow_update,
 * built before with the same instance_count: the TLAS is refit in place (same
 * topology; new instance boxes, transforms, masks and BLAS references from
 * the current meshes, rebuilt or refit) with kernels only -- no host
 * synchronisation, no allocation, so it can be captured in a CUDA graph.
 * Otherwise the TLAS is rebuilt (the OptiX update of cuda_accel.cpp). */
LCX_API int lcx_accel_build(uint64_t accel, uint32_t instance_count, uint32_t request,
                    const LcxModification *mods, size_t mod_count,
                    int update_instance_buffer_only, void *stream);

LCX_API int lcx_accel_stats(uint64_t accel, LcxAccelStats *out);

/* ------------------------------------------------------ motion instances */

/* AccelOption::Motion (include/luisa/runtime/rhi/resource.h:101-118) for a
 * motion instance (MotionInstance, include/luisa/runtime/rtx/motion_instance.h):
 * keyframe_count >= 2 keyframes spaced evenly over [time_start, time_end]
 * (time_end > time_start); a ray time before time_start (after time_end)
 * makes the instance vanish if vanish_start (vanish_end) is set, else it is
 * clamped.  LCX_MOTION_MATRIX keyframes are row-major 3x4 object-to-world
 * matrices (12 floats), interpolated per element; LCX_MOTION_SRT keyframes
 * are the reference's MotionInstanceTransformSRT (16 floats: pivot xyz,
 * quaternion xyzw, scale xyz, shear xyz, translation xyz;
 * include/luisa/runtime/rtx/motion_transform.h:13-19), every component
 * interpolated linearly and the quaternion normalised, composed as
 * T * R * S with S = [[sx, shear0, shear1, px], [0, sy, shear2, py],
 * [0, 0, sz, pz]]. */
enum { LCX_MOTION_MATRIX = 0, LCX_MOTION_SRT = 1 };
typedef struct LcxMotionOption {
    uint32_t keyframe_count;
    float time_start;
    float time_end;
    uint8_t vanish_start;
    uint8_t vanish_end;
    uint8_t mode;        /* LCX_MOTION_MATRIX or LCX_MOTION_SRT */
    uint8_t _pad;
} LcxMotionOption;

/* A motion instance of a built triangle mesh (Device::create_motion_instance).
 * Its keyframes start as identities.  An accel instances it by passing its
 * handle as a Modification's primitive; the TLAS then bounds the mesh over
 * all keyframes, and traces move it by the keyframe matrices interpolated
 * linearly per element at each ray's time (OptiX's matrix motion transform,
 * the CUDA backend's path).  Accels that instance it keep its memory alive;
 * destroying it, or building it again with new keyframes, makes their traces
 * fail until they are built again.  No CPU-backend counterpart. */
LCX_API int lcx_motion_instance_create(uint64_t mesh, const LcxMotionOption *option, uint64_t *out_handle);
LCX_API int lcx_motion_instance_destroy(uint64_t motion_instance);
/* `count` (== keyframe_count) keyframes in host memory: 12 floats each
 * (LCX_MOTION_MATRIX: the reference's float4x4 matrices packed as
 * Modification::set_transform packs them) or 16 (LCX_MOTION_SRT)
 * (MotionInstance::set_keyframes). */
LCX_API int lcx_motion_instance_set_keyframes(uint64_t motion_instance, const float *matrices, uint32_t count);
/* Uploads the keyframes on `stream` (MotionInstance::build). */
LCX_API int lcx_motion_instance_build(uint64_t motion_instance, void *stream);

/* A mesh with keyframed vertices (AccelOption::Motion on a mesh,
 * include/luisa/runtime/rtx/mesh.h:85-86, 127-139; the CUDA backend's motion
 * GAS, cuda_mesh.cpp:20-22): its build commands' vertex buffers hold
 * motion->keyframe_count copies of the vertices back to back (the vertex
 * count must be a whole multiple), indexed by the same triangles.  Traces
 * interpolate the three vertices of a triangle linearly at the ray's time
 * (lcx_trace_closest_motion / lcx_trace_any_motion; other calls use time 0);
 * vanish_start / vanish_end and the time range behave as for motion
 * instances; motion->mode is ignored.  The vertex buffer is borrowed and read
 * by every later trace.  allow_update is rejected (no refit). */
LCX_API int lcx_mesh_create_motion(const LcxAccelOption *option, const LcxMotionOption *motion,
                                   uint64_t *out_handle);
/* A curve with keyframed control points (the reference's curve motion,
 * AccelOption::motion with Curve, include/luisa/runtime/rtx/curve.h:10-11):
 * the build command's control point buffer holds keyframe_count copies of
 * cp_count / keyframe_count points back to back, and segment indices address
 * one copy.  The points interpolate linearly between keyframes spaced evenly over
 * [time_start, time_end] (clamped, or vanishing with vanish_start / vanish_end);
 * traces take the ray's time through the *_motion entry points, as for
 * lcx_mesh_create_motion. */
LCX_API int lcx_curve_create_motion(const LcxAccelOption *option, const LcxMotionOption *motion,
                                    uint64_t *out_handle);

/* ----------------------------------------------------------------- queries */

/* Device view of a built accel, for lcx::ray_query in user CUDA kernels
 * (include/lcx/ray_query.cuh: RayQuery with per-candidate callbacks,
 * include/luisa/dsl/rtx/ray_query.h:17-240).  The reference hands the accel
 * to kernels through its DSL binding; this is that handle as plain pointers.
 * Valid until the accel is rebuilt (a refit keeps it valid) or destroyed, or
 * a mesh it instances is rebuilt or refit without the accel being built
 * again.  Fails like a trace call on an accel that is not ready
 * (LCX_ERR_NOT_BUILT, LCX_ERR_DEPTH).  `motion` = 1: the accel has motion
 * instances or keyframed meshes or curves, which lcx::ray_query_motion traces
 * and the plain lcx::ray_query passes over. */
typedef struct LcxAccelView {
    const void *tlas_nodes;  /* the TLAS's 8-bit quantised nodes (device) */
    const void *instances;   /* its leaf instance records (device) */
    uint32_t stack_need;     /* stack entries a query needs (<= 32) */
    uint32_t motion;         /* 1: motion instances or keyframed meshes / curves (lcx::ray_query_motion) */
} LcxAccelView;
LCX_API int lcx_accel_device_view(uint64_t accel, LcxAccelView *out);

/* The accel's instance records in device memory, for kernels that read or
 * edit instances in place (include/lcx/accel_instances.cuh: the reference's
 * device-side Accel::set_instance_transform / visibility / opacity / user_id
 * and getters, src/backends/cuda/cuda_builtin/cuda_device_resource.h:1450-1512).
 * Edits take effect at the next lcx_accel_build (PREFER_UPDATE refits an
 * accel created with allow_update).  Valid until an lcx_accel_build grows the
 * instance count past its capacity, or the accel is destroyed.  Fails with
 * LCX_ERR_NOT_BUILT while the accel has no instances. */
typedef struct LcxInstanceBuffer {
    void *states;    /* `count` 80-byte InstState records (include/lcx/bvh_device.cuh) */
    uint32_t count;  /* instance count of the last lcx_accel_build */
    uint32_t _pad;
} LcxInstanceBuffer;
LCX_API int lcx_accel_instance_buffer(uint64_t accel, LcxInstanceBuffer *out);

/* trace_closest over a batch: CPU accel.rs:449-509, CUDA
 * cuda_device_resource.h:1784-1807.  d_rays / d_hits are device arrays of
 * `ray_count` records.  An instance is eligible when (vis_mask & mask) != 0
 * (accel.rs:414, cuda_device_resource.h:1776).  Back faces are not culled
 * (cuda_mesh.cpp:15-16).  Ties in t are broken by the smaller (inst, prim),
 * so the result does not depend on BVH topology.  ray_count <= 2^31. */
LCX_API int lcx_trace_closest(uint64_t accel, const LcxRay *d_rays, uint32_t ray_count,
                      uint32_t mask, LcxTriangleHit *d_hits, void *stream);

/* trace_any over a batch: CPU accel.rs:511-535 (occluded <=> any hit with
 * t in [t_min, t_max]), CUDA cuda_device_resource.h:1809-1829.
 * d_occluded[i] is 1 if occluded, else 0. */
LCX_API int lcx_trace_any(uint64_t accel, const LcxRay *d_rays, uint32_t ray_count,
                  uint32_t mask, uint8_t *d_occluded, void *stream);

/* One ray batch of a multi-job launch: `ray_count` rays against `accel`,
 * written to `out` (LcxTriangleHit[] when any == 0, uint8_t[] when any != 0). */
typedef struct LcxTraceJob {
    uint64_t accel;
    const LcxRay *rays;
    void *out;
    uint32_t ray_count;
    uint32_t mask;
    uint32_t any;
    uint32_t _pad;
} LcxTraceJob;

/* Many ray batches against many accels in one launch per query kind
 * (continuous batching; no counterpart in the reference, whose queries run
 * inside one user kernel per dispatch).  Persistent warps take global ray
 * indices and each lane serves its ray's job, so jobs of any size and scene
 * share the GPU.  Results equal one lcx_trace_closest / lcx_trace_any call
 * per job.  At most 2^31 rays per kind. */
LCX_API int lcx_trace_jobs(const LcxTraceJob *jobs, uint32_t count, uint32_t node_layout, void *stream);
/* The same with a time per ray for accels with motion (times[i]: job i's
 * ray_count floats, device-accessible, or null for time 0; `times` null: all
 * time 0, as lcx_trace_jobs).  Results equal one lcx_trace_closest_motion /
 * lcx_trace_any_motion call per job. */
LCX_API int lcx_trace_jobs_motion(const LcxTraceJob *jobs, const float *const *times, uint32_t count,
                                  uint32_t node_layout, void *stream);

/* Same queries with an explicit node layout (LCX_NODES_FP32 or
 * LCX_NODES_QUANT8); lcx_trace_closest/any use LCX_NODES_QUANT8. */
LCX_API int lcx_trace_closest_ex(uint64_t accel, const LcxRay *d_rays, uint32_t ray_count,
                         uint32_t mask, LcxTriangleHit *d_hits, uint32_t node_layout,
                         void *stream);
LCX_API int lcx_trace_any_ex(uint64_t accel, const LcxRay *d_rays, uint32_t ray_count,
                     uint32_t mask, uint8_t *d_occluded, uint32_t node_layout,
                     void *stream);

/* Queries with a time per ray (DSL Accel::intersect_motion /
 * intersect_any_motion, include/luisa/dsl/rtx/accel.h:47-48): d_times holds
 * ray_count floats (null: time 0).  Static instances ignore the time.  Any
 * trace of an accel that instances a motion instance runs the motion kernels
 * (time 0 for the calls without times; lcx_trace_jobs_motion takes a time
 * per ray of each job), and user kernels trace them with
 * lcx::ray_query_motion. */
LCX_API int lcx_trace_closest_motion(uint64_t accel, const LcxRay *d_rays, const float *d_times,
                                     uint32_t ray_count, uint32_t mask, LcxTriangleHit *d_hits,
                                     uint32_t node_layout, void *stream);
LCX_API int lcx_trace_any_motion(uint64_t accel, const LcxRay *d_rays, const float *d_times,
                                 uint32_t ray_count, uint32_t mask, uint8_t *d_occluded,
                                 uint32_t node_layout, void *stream);

/* The same queries over HOST buffers, for callers whose rays and results live
 * in host memory -- the form of the reference's CPU backend, whose
 * trace_closest / trace_any read and write host arrays
 * (src/rust/luisa_compute_backend_impl/src/cpu/accel.rs:449-535).  Two
 * paths (lcx_set_host_access):
 *   - direct: when both buffers are pinned (page-locked, each one allocation)
 *     and the device reads host memory through a coherent link (NVLink-C2C on
 *     Grace systems; the default there for calls of at most 2^18 rays), the
 *     traversal kernel itself reads the rays from and writes the results to
 *     host memory, with no staging and no copies;
 *   - staged: otherwise the rays stream through device staging in chunks
 *     (lcx_set_host_chunk, default 2^22 rays; a ring of 4 chunks of staging,
 *     56 B per ray, kept in a memory pool): the copy in of one chunk, the
 *     traversal of the previous one and the copy out of the one before run at
 *     once.  Stream-ordered like the device
 * forms: the work starts after `stream`'s earlier work and `stream` waits for
 * the last result copy, so h_hits / h_occluded are complete once `stream` is
 * synchronised.  Results equal the device forms'.  Pinned host memory
 * (cudaHostAlloc / cudaHostRegister) overlaps the copies with the traversal;
 * pageable memory works but serialises them.  Cannot be captured in a CUDA
 * graph. */
LCX_API int lcx_trace_closest_host(uint64_t accel, const LcxRay *h_rays, uint32_t ray_count,
                                   uint32_t mask, LcxTriangleHit *h_hits, uint32_t node_layout,
                                   void *stream);
LCX_API int lcx_trace_any_host(uint64_t accel, const LcxRay *h_rays, uint32_t ray_count,
                               uint32_t mask, uint8_t *h_occluded, uint32_t node_layout,
                               void *stream);
/* Rays per chunk of the host-buffer traces (2^14..2^26).  A tuning knob with
 * no reference counterpart. */
LCX_API int lcx_set_host_chunk(uint32_t rays);
/* Host-buffer trace path: LCX_HOST_AUTO (direct when the device has a
 * coherent host link, the buffers are pinned and the call has at most 2^18
 * rays, else streamed where the call allows it, else staged), LCX_HOST_STAGED
 * (chunks through a ring of device slots, one traversal launch per chunk),
 * LCX_HOST_DIRECT (direct whenever the buffers are pinned: on a device without
 * a coherent link the kernel's host accesses cross PCIe one by one),
 * LCX_HOST_STREAMED (one traversal launch over the whole call that takes each
 * copy chunk of rays as it arrives, while finished chunks are copied out; for
 * pinned buffers, accels without motion or curves, quantised nodes and loop
 * mode 2, else staged; staged too while launches are serialised, under
 * CUDA_LAUNCH_BLOCKING=1 or an Nsight tool; one such call at a time per
 * device, others staged).
 * lcx_get_host_access reports the mode and whether the current device has the
 * coherent link.  Tuning knobs with no reference counterpart. */
enum { LCX_HOST_AUTO = 0, LCX_HOST_STAGED = 1, LCX_HOST_DIRECT = 2, LCX_HOST_STREAMED = 3 };
LCX_API int lcx_set_host_access(uint32_t mode);
LCX_API int lcx_get_host_access(uint32_t *mode, uint32_t *coherent_link);

/* Builds, refits and traces take their scratch from a stream-ordered pool of the
 * current device that keeps freed memory for the next call (a build of n items
 * uses a few hundred bytes per item; 135M triangles: ~34 GB).  This hands the
 * unused part back to the driver, after synchronising the device; a BVH
 * allocation that finds the device out of memory does the same once before it
 * fails.  No reference counterpart (OptiX and Embree manage their own build
 * memory). */
LCX_API int lcx_release_scratch(void);

/* Counting build of the closest-hit traversal: per-ray visit counts
 * d_counts[3*i + {0,1,2}] = {wide nodes fetched, triangles tested, instances
 * entered}.  Used to compute algorithmic bytes per ray.  The counts are those
 * of the loop structure the plain call would run (lcx_set_trace_tuning's
 * mode: loop mode 2 for quantised nodes by default). */
LCX_API int lcx_trace_closest_counts(uint64_t accel, const LcxRay *d_rays, uint32_t ray_count,
                             uint32_t mask, LcxTriangleHit *d_hits, uint32_t *d_counts,
                             uint32_t node_layout, void *stream);

/* trace_closest that allocates nothing, for callers that cannot allocate
 * device memory (an application that reserves its HBM at start-up and forbids
 * later allocations, a plugin whose host framework owns every device
 * allocation, a latency-bound loop that must not hit cudaMalloc's implicit
 * device synchronisation).  No counterpart in the reference.  Same results as
 * lcx_trace_closest (8-bit quantised nodes); the caller passes the built
 * accel, the rays and the hit buffer.  Its scratch is a 256-byte static
 * device array held by every GPU that loads the library until exit; the first
 * call on a device looks up that array's device address, so make that first
 * call before any stream capture.  All calls share the array (it is cleared at
 * the start of each call): calls that overlap on the GPU race and must be
 * ordered by the caller.  ray_count <= 2^31; larger counts return
 * LCX_ERR_INVALID_ARG.  Kernel-side bounds (stack overflow, step bound) are
 * reported by lcx_check_trace_errors like those of the other trace calls.  The
 * array's device address is kept for the life of the process: do not call this
 * entry point again after a cudaDeviceReset. */
LCX_API int lcx_trace_closest_noalloc(uint64_t accel, const LcxRay *d_rays, uint32_t ray_count, uint32_t mask,
                                      LcxTriangleHit *d_hits, void *stream);

/* ------------------------------------------- the CPU backend's per-ray table */

/* The accel table that kernels of the reference's CPU backend call per ray
 * (defs::Accel, src/rust/luisa_compute_cpu_kernel_defs/src/lib.rs:111-125,
 * filled per binding in src/rust/luisa_compute_backend_impl/src/cpu/stream.rs:546-560
 * and called by the generated code, src/rust/luisa_compute_backend_impl/src/cpu/codegen/cpp.rs:1334-1350),
 * with the same layout, field order and calling convention. */
typedef struct __attribute__((aligned(16))) LcxMat4 {
    float m[16]; /* column-major: m[4 * column + row] */
} LcxMat4;
typedef struct __attribute__((aligned(8))) LcxCpuCommittedHit {
    uint32_t inst, prim;
    float bary[2];
    uint32_t hit_type; /* 0 miss, 1 triangle, 2 procedural */
    float committed_ray_t;
} LcxCpuCommittedHit;
typedef struct LcxCpuProceduralHit {
    uint32_t inst, prim;
} LcxCpuProceduralHit;
struct LcxCpuAccel;
/* defs::RayQuery (lib.rs:127-141), 128 B. */
typedef struct __attribute__((aligned(16))) LcxCpuRayQuery {
    LcxCpuCommittedHit hit;
    LcxRay ray;
    uint32_t mask;
    float cur_committed_ray_t;
    LcxTriangleHit cur_triangle_hit;
    LcxCpuProceduralHit cur_procedural_hit;
    bool cur_commited;
    bool terminate_on_first;
    bool terminated;
    void *user_data;
    const struct LcxCpuAccel *accel;
} LcxCpuRayQuery;
typedef void (*LcxCpuHitCallback)(LcxCpuRayQuery *);
typedef struct LcxCpuAccel {
    const void *handle;
    LcxTriangleHit (*trace_closest)(const void *handle, const LcxRay *ray, uint32_t mask);
    bool (*trace_any)(const void *handle, const LcxRay *ray, uint32_t mask);
    void (*set_instance_visibility)(const void *handle, uint32_t instance, uint32_t mask);
    void (*set_instance_transform)(const void *handle, uint32_t instance, const LcxMat4 *transform);
    void (*set_instance_user_id)(const void *handle, uint32_t instance, uint32_t user_id);
    LcxMat4 (*instance_transform)(const void *handle, uint32_t instance);
    uint32_t (*instance_user_id)(const void *handle, uint32_t instance);
    uint32_t (*instance_visibility_mask)(const void *handle, uint32_t instance);
    void (*ray_query)(const void *handle, LcxCpuRayQuery *rq, LcxCpuHitCallback on_triangle,
                      LcxCpuHitCallback on_procedural);
} LcxCpuAccel;
/* Fills `out` for a built accel (its handle field is `accel`).  Each function
 * is one host round trip to the GPU (tens of microseconds per ray): a
 * compatibility form for generated code that keeps the per-ray calls; the
 * batched entry points are the fast form.  The functions cannot return a status: on an error trace_closest
 * returns the miss record, trace_any false, the getters their defaults, and
 * lcx_last_error_string says why.  Instance edits take effect at the next
 * lcx_accel_build (as the reference's CPU backend marks instances dirty);
 * the getters read the current instance state.  ray_query runs the host
 * callbacks on the candidates of the ray found on the GPU (at most 4096),
 * in increasing t, with the reference's commit / terminate protocol; motion
 * is traced at time 0, as the reference's CPU backend does. */
LCX_API int lcx_accel_cpu_table(uint64_t accel, LcxCpuAccel *out);

/* ------------------------------------------------------ wavefront path tracer */

/* Geometry and material of one mesh for shading (device pointers): float3-in-16-B
 * vertices, uint3 triangles, one grey Lambert albedo per triangle. */
typedef struct LcxPtMesh {
    const void *vertices;
    uint64_t vertex_stride;
    const uint32_t *triangles;
    const float *albedo;
} LcxPtMesh;

typedef struct LcxPtParams {
    uint32_t width, height, spp, max_bounces;
    uint32_t rr_start;   /* Russian roulette from this bounce on */
    uint32_t seed;
    float eye[3], target[3], up[3];
    float tan_half_fov;  /* tan(vertical field of view / 2) */
    float light_pos[3], light_intensity[3];
    float env[3];        /* constant environment radiance */
} LcxPtParams;

typedef struct LcxPtStats {
    uint64_t closest_rays, any_rays;
    uint32_t bounces;
    float ms;            /* device time of the frame */
    uint32_t launches;   /* kernels of this library launched for the frame */
    uint32_t _pad;
} LcxPtStats;

/* Renders one frame of diffuse path tracing over `accel` (the shape of the
 * reference's src/tests/test_path_tracing.cpp, as a wavefront): per bounce one
 * lcx_trace_closest over the live paths, shading, one lcx_trace_any over the
 * shadow rays; the surviving paths are compacted between bounces.
 * inst_mesh / inst_o2w (host arrays) give each TLAS instance's mesh and
 * object-to-world transform.  d_image: width*height*3 floats (linear RGB,
 * the mean over spp).  d_first_hits (optional): the first bounce's hit of every
 * path, path = pixel * spp + sample.  Synchronises the host once per bounce. */
LCX_API int lcx_pt_render(uint64_t accel, const LcxPtMesh *meshes, uint32_t mesh_count, const uint32_t *inst_mesh,
                          const float *inst_o2w, uint32_t instance_count, const LcxPtParams *params, float *d_image,
                          LcxTriangleHit *d_first_hits, LcxPtStats *stats, void *stream);

/* Synchronises the current device and reports whether any trace call since
 * the last check hit a kernel-side bound: LCX_ERR_TIMEOUT when a ray exceeded
 * the per-ray step bound (only a corrupt BVH can cause it), LCX_ERR_DEPTH when
 * a push found the stack full.  Also reports refits run without host
 * synchronisation (lcx_set_refit_sync(0)) that met a triangle index out of
 * range or unquantisable coordinates (LCX_ERR_INVALID_ARG).  Clears the flags.
 * (No counterpart in the reference, whose kernels cannot report errors.) */
LCX_API int lcx_check_trace_errors(void);

/* Refit mode for later PREFER_UPDATE mesh builds (lcx_mesh_build and
 * lcx_mesh_build_batch on meshes created with allow_update): 1 (default)
 * synchronises the host once to report bad indices from the call itself; 0
 * only enqueues kernels (no host synchronisation, no allocation, so a refit
 * can be captured in a CUDA graph) and leaves errors for
 * lcx_check_trace_errors.  TLAS refits (lcx_accel_build with PREFER_UPDATE on
 * an accel created with allow_update, same instance count, meshes built)
 * never synchronise.  No counterpart in the reference. */
LCX_API int lcx_set_refit_sync(uint32_t sync);

/* Build knobs, process-wide, for builds that start after the call (no
 * counterpart in the reference).  leaf_max: triangles per leaf slot, 1..3, or
 * 0 to follow AccelOption.hint (FAST_TRACE 2, FAST_BUILD 3); width: children
 * per wide node, 2..8 (default 8).  Results of queries do not depend on them. */
LCX_API int lcx_set_build_tuning(uint32_t leaf_max, uint32_t width);
LCX_API int lcx_get_build_tuning(uint32_t *leaf_max, uint32_t *width);
/* Morton-code options for later builds: blas_cube / tlas_cube = 1 normalise
 * centroids by the largest extent on all axes (0: each axis by its own);
 * tlas_size_bits = size-class bits above the TLAS Morton code (extended Morton
 * codes; 0 = off).  Defaults 1, 0, 0. */
LCX_API int lcx_set_build_morton(uint32_t blas_cube, uint32_t tlas_cube, uint32_t tlas_size_bits);
LCX_API int lcx_get_build_morton(uint32_t *blas_cube, uint32_t *tlas_cube, uint32_t *tlas_size_bits);
/* Triangle splitting for later builds of FAST_TRACE meshes created without
 * allow_update (the spatial splits of the high-quality builder the reference
 * asks Embree for, cpu/accel.rs:58-61): triangles whose box is much larger
 * than the triangle get extra references with tighter boxes, at most
 * fraction x (triangles of the mesh) of them (0 = off; 0..4, default 0).
 * Every reference stores the whole triangle, so hit records do not change; a
 * RayQuery triangle callback may see a triangle more than once (as with the
 * reference's OptiX and Embree builders). */
LCX_API int lcx_set_build_split(float fraction);
LCX_API int lcx_get_build_split(float *fraction);
/* Leaf-slot filling for later BLAS builds (0 or 1): once no child of a wide
 * node can become a wide node itself, its free slots are filled by splitting
 * leaf slots (largest area first) into slots of fewer triangles.  The node
 * count and the cost of a node test stay the same; a ray tests fewer
 * triangles.  Default 1.  Results do not depend on it. */
LCX_API int lcx_set_build_fill(uint32_t fill);
LCX_API int lcx_get_build_fill(uint32_t *fill);
/* TLAS builds (0 or 1): 1 builds the binary tree by binned SAH (16 bins per
 * axis, top-down, on the GPU) instead of the Morton LBVH, before the same
 * collapse to wide nodes.  Instance sets mixing a few large objects with many
 * small ones trace faster through it.  Default 1.  Results do not depend on it. */
LCX_API int lcx_set_build_tlas_sah(uint32_t sah);
LCX_API int lcx_get_build_tlas_sah(uint32_t *sah);
/* BLAS builds of FAST_TRACE meshes (0 or 1): 1 builds the binary tree by the
 * same binned SAH instead of the Morton LBVH (the reference's FAST_TRACE builds
 * are SAH builds too: Embree's high-quality builder, OptiX's PREFER_FAST_TRACE).
 * The build synchronises the stream once per level of node ranges above 1024
 * triangles, so it takes longer than the LBVH; FAST_BUILD meshes, reserved
 * batches (lcx_mesh_build_batch_reserve, lcx_mesh_reserve_batch) and their
 * rebuilds keep the LBVH.  Default 1.  Results do not depend on it. */
/* The collapse of FAST_TRACE BLASes and TLASes to wide nodes (0 or 1): 0
 * opens the largest-area children greedily (then fills free slots by
 * splitting leaf slots); 1 follows a dynamic program over the binary tree that
 * minimises the wide tree's cost (Ylitie, Karras and Laine 2017).  Default 1.
 * FAST_BUILD meshes and reserved batches keep the greedy collapse.  Results do
 * not depend on it. */
LCX_API int lcx_set_build_collapse(uint32_t mode);
LCX_API int lcx_get_build_collapse(uint32_t *mode);
LCX_API int lcx_set_build_blas_sah(uint32_t sah);
LCX_API int lcx_get_build_blas_sah(uint32_t *sah);
/* Kernels of this library launched by builds, refits and instance updates
 * since it was loaded (a host-side counter for launch accounting; the CUB
 * sort and scan kernels a build also runs are library kernels and are not
 * counted).  No counterpart in the reference. */
LCX_API int lcx_get_build_kernel_launches(uint64_t *count);

/* Traversal knobs, process-wide (no counterpart in the reference: OptiX and
 * Embree pick theirs internally).  refill: a warp takes new rays once at
 * least this many of its 32 lanes are idle (1..32, default 4).  mode: loop
 * structure -- 2 (default) = deferred triangle batches: each warp queues the
 * triangles its lanes find and tests them 32 at a time (quantised-node,
 * single-job, non-counting calls; the others run mode 0); 0 = each step
 * visits one node and tests its triangles; 1 = speculative while-while;
 * 3 = one ray per thread through lcx::trace_closest / lcx::trace_any
 * (include/lcx/trace.cuh), the form a user kernel's per-ray calls take
 * (quantised-node single-job calls; the others run mode 0).
 * postpone: in mode 2, the queue size that starts a batch (1..32; 0 = 24 for
 * closest, 16 for any hit); in modes 0 and 1, a lane defers its triangle tests
 * while fewer than this many lanes would run them (0 = never).  Results do
 * not depend on any of them. */
LCX_API int lcx_set_trace_tuning(uint32_t refill, uint32_t postpone, uint32_t mode);
LCX_API int lcx_get_trace_tuning(uint32_t *refill, uint32_t *postpone, uint32_t *mode);
/* Ray reordering for later lcx_trace_closest / lcx_trace_any calls (and their
 * _ex / _counts forms): the rays of a call are sorted by direction octant and
 * the Morton code of the origin's cell in the scene box (`bits` per axis,
 * 1..9; 0 = off) and traversed in that order; calls with fewer than min_rays
 * rays are not reordered.  The results are the same bit for bit.  A tuning
 * knob with no reference counterpart. */
LCX_API int lcx_set_trace_reorder(uint32_t bits, uint32_t min_rays);
/* Traversal stack entries per thread kept in shared memory (8, 16 or 24; the
 * rest of the 32-entry stack lives in local memory) for later single-job
 * closest / any calls in loop mode 0.  Default 16.  Results do not depend on
 * it.  A tuning knob with no reference counterpart. */
LCX_API int lcx_set_trace_stack(uint32_t short_entries);
LCX_API int lcx_get_trace_stack(uint32_t *short_entries);
LCX_API int lcx_get_trace_reorder(uint32_t *bits, uint32_t *min_rays);
/* Per-ray step bound of later trace calls (every form): a ray that takes more
 * traversal steps ends with the record it has and flags LCX_ERR_TIMEOUT for
 * lcx_check_trace_errors.  0 restores the default, 2^22 steps, which no valid
 * BVH reaches; a small bound lets a caller (or a test) check the timeout path
 * on a valid scene without a hang.  A guard with no reference counterpart:
 * the reference's OptiX and Embree traversals have no step bound. */
LCX_API int lcx_set_trace_step_bound(uint32_t steps);
LCX_API int lcx_get_trace_step_bound(uint32_t *steps);

#ifdef __cplusplus
}
#endif

#endif /* LCX_ACCEL_H */
