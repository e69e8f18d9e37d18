// accel_ext.hpp — C++ host side of the GB300 Mesh/Accel path, shaped like
// LuisaCompute's own interfaces so that a backend can hand it out from
// DeviceInterface::extension("AccelGpuExt").
//
//   AccelGpuExt        a DeviceExtension (include/luisa/runtime/rhi/device_interface.h:90-93)
//                      with `static constexpr std::string_view name`, like the reference's
//                      extensions (include/luisa/backends/ext/pinned_memory_ext.hpp:17-22);
//                      its methods are the accel part of DeviceInterface
//                      (device_interface.h:171-184) plus the visits of MeshBuildCommand and
//                      AccelBuildCommand (cuda_command_encoder.cpp:235-243).
//   MeshBuildCommand   fields of include/luisa/runtime/rhi/command.h:407-444.
//   AccelBuildCommand  fields of command.h:594-616, Modification of command.h:534-592.
//   Mesh / Accel       RAII host objects with the reference's staging API
//                      (include/luisa/runtime/rtx/accel.h:21-134, src/runtime/rtx/accel.cpp:68-249).
//
// Header-only over the C ABI of lcx_accel.h; errors are status codes wrapped
// in lcx::Error exceptions by the RAII layer, never aborts.
#pragma once

#include <array>
#include <cstdint>
#include <cstring>
#include <map>
#include <stdexcept>
#include <string>
#include <string_view>
#include <vector>

#include "../lcx_accel.h"

namespace lcx {

class Error : public std::runtime_error {
public:
    Error(int code, const std::string &where)
        : std::runtime_error(where + ": " + lcx_last_error_string()), code_(code) {}
    [[nodiscard]] int code() const noexcept { return code_; }

private:
    int code_;
};

inline void check(int code, const char *where) {
    if (code != LCX_OK) throw Error(code, where);
}

// include/luisa/runtime/rhi/resource.h:94-125
struct AccelOption {
    enum struct UsageHint : uint32_t { FAST_TRACE = LCX_HINT_FAST_TRACE, FAST_BUILD = LCX_HINT_FAST_BUILD };
    UsageHint hint{UsageHint::FAST_TRACE};
    bool allow_compaction{true};
    bool allow_update{false};
    [[nodiscard]] LcxAccelOption c() const noexcept {
        LcxAccelOption o{};
        o.hint = static_cast<uint32_t>(hint);
        o.allow_compaction = allow_compaction;
        o.allow_update = allow_update;
        return o;
    }
};

// include/luisa/runtime/rhi/command.h:401-404
enum struct AccelBuildRequest : uint32_t {
    PREFER_UPDATE = LCX_REQUEST_PREFER_UPDATE,
    FORCE_BUILD = LCX_REQUEST_FORCE_BUILD,
};

// include/luisa/runtime/rhi/resource.h ResourceCreationInfo: handle + native handle
struct ResourceCreationInfo {
    uint64_t handle{0};
    void *native_handle{nullptr};
};

using Ray = LcxRay;
using TriangleHit = LcxTriangleHit;
using Modification = LcxModification;

struct MeshBuildCommand {
    uint64_t handle;
    AccelBuildRequest request;
    uint64_t vertex_buffer;
    size_t vertex_buffer_offset;
    size_t vertex_buffer_size;
    size_t vertex_stride;
    uint64_t triangle_buffer;
    size_t triangle_buffer_offset;
    size_t triangle_buffer_size;
};

// include/luisa/runtime/rhi/command.h:488-512; aabb_buffer: device address of
// 24-byte {float min[3], max[3]} records.
struct ProceduralPrimitiveBuildCommand {
    uint64_t handle;
    AccelBuildRequest request;
    uint64_t aabb_buffer;
    size_t aabb_buffer_offset;
    size_t aabb_buffer_size;
};

// include/luisa/runtime/rhi/command.h:446-486; control points are float4
// {x, y, z, radius} records cp_stride bytes apart, segments u32 first-point indices.
enum class CurveBasis : uint32_t { PIECEWISE_LINEAR = 0, CUBIC_BSPLINE = 1, CATMULL_ROM = 2, BEZIER = 3 };
struct CurveBuildCommand {
    uint64_t handle;
    AccelBuildRequest request;
    CurveBasis basis;
    size_t cp_count;
    size_t seg_count;
    uint64_t cp_buffer;
    size_t cp_buffer_offset;
    size_t cp_stride;
    uint64_t seg_buffer;
    size_t seg_buffer_offset;
};

struct AccelBuildCommand {
    uint64_t handle;
    uint32_t instance_count;
    AccelBuildRequest request;
    std::vector<Modification> modifications;
    bool update_instance_buffer_only;
};

// The device extension a backend returns from extension("AccelGpuExt").
class AccelGpuExt {
public:
    static constexpr std::string_view name = "AccelGpuExt";

    explicit AccelGpuExt(int device = 0) { check(lcx_device_init(device), "lcx_device_init"); }

    [[nodiscard]] ResourceCreationInfo create_mesh(const AccelOption &option) const {
        const LcxAccelOption o = option.c();
        ResourceCreationInfo info;
        check(lcx_mesh_create(&o, &info.handle), "create_mesh");
        return info;
    }
    void destroy_mesh(uint64_t handle) const { check(lcx_mesh_destroy(handle), "destroy_mesh"); }

    // device_interface.h:174-175: a BLAS over AABBs, instanced like a mesh
    [[nodiscard]] ResourceCreationInfo create_procedural_primitive(const AccelOption &option) const {
        const LcxAccelOption o = option.c();
        ResourceCreationInfo info;
        check(lcx_procedural_create(&o, &info.handle), "create_procedural_primitive");
        return info;
    }
    void destroy_procedural_primitive(uint64_t handle) const {
        check(lcx_procedural_destroy(handle), "destroy_procedural_primitive");
    }

    // device_interface.h:177-178: a BLAS over curve segments, instanced like a mesh
    [[nodiscard]] ResourceCreationInfo create_curve(const AccelOption &option) const {
        const LcxAccelOption o = option.c();
        ResourceCreationInfo info;
        check(lcx_curve_create(&o, &info.handle), "create_curve");
        return info;
    }
    // AccelOption::motion with >= 2 keyframes: the control-point buffer holds the keyframes back to back
    [[nodiscard]] ResourceCreationInfo create_curve(const AccelOption &option, const LcxMotionOption &motion) const {
        const LcxAccelOption o = option.c();
        ResourceCreationInfo info;
        check(lcx_curve_create_motion(&o, &motion, &info.handle), "create_curve");
        return info;
    }
    void destroy_curve(uint64_t handle) const { check(lcx_curve_destroy(handle), "destroy_curve"); }

    // device_interface.h create_motion_instance: a mesh moved by matrix keyframes (row-major 3x4 each)
    [[nodiscard]] ResourceCreationInfo create_motion_instance(uint64_t mesh, const LcxMotionOption &option,
                                                              const std::vector<std::array<float, 12>> &keyframes,
                                                              void *stream) const {
        ResourceCreationInfo info;
        check(lcx_motion_instance_create(mesh, &option, &info.handle), "create_motion_instance");
        check(lcx_motion_instance_set_keyframes(info.handle, keyframes.empty() ? nullptr : keyframes[0].data(),
                                                uint32_t(keyframes.size())),
              "MotionInstance::set_keyframes");
        check(lcx_motion_instance_build(info.handle, stream), "MotionInstance::build");
        return info;
    }
    void destroy_motion_instance(uint64_t handle) const {
        check(lcx_motion_instance_destroy(handle), "destroy_motion_instance");
    }

    [[nodiscard]] ResourceCreationInfo create_accel(const AccelOption &option) const {
        const LcxAccelOption o = option.c();
        ResourceCreationInfo info;
        check(lcx_accel_create(&o, &info.handle), "create_accel");
        return info;
    }
    void destroy_accel(uint64_t handle) const { check(lcx_accel_destroy(handle), "destroy_accel"); }

    // Command visits, stream-ordered on `stream` (a cudaStream_t).
    void dispatch(const MeshBuildCommand &cmd, void *stream) const {
        LcxMeshBuildCommand c{};
        c.request = static_cast<uint32_t>(cmd.request);
        c.vertex_buffer = cmd.vertex_buffer;
        c.vertex_buffer_offset = cmd.vertex_buffer_offset;
        c.vertex_buffer_size = cmd.vertex_buffer_size;
        c.vertex_stride = cmd.vertex_stride;
        c.triangle_buffer = cmd.triangle_buffer;
        c.triangle_buffer_offset = cmd.triangle_buffer_offset;
        c.triangle_buffer_size = cmd.triangle_buffer_size;
        check(lcx_mesh_build(cmd.handle, &c, stream), "MeshBuildCommand");
    }
    // A command list's MeshBuildCommands at once: one segmented build, one host sync
    // (PREFER_UPDATE of meshes built together with allow_update: one refit).
    void dispatch(const std::vector<MeshBuildCommand> &cmds, void *stream) const {
        std::vector<uint64_t> handles(cmds.size());
        std::vector<LcxMeshBuildCommand> cs(cmds.size());
        for (size_t i = 0; i < cmds.size(); i++) {
            handles[i] = cmds[i].handle;
            cs[i] = LcxMeshBuildCommand{static_cast<uint32_t>(cmds[i].request), 0u, cmds[i].vertex_buffer,
                                        cmds[i].vertex_buffer_offset, cmds[i].vertex_buffer_size,
                                        cmds[i].vertex_stride, cmds[i].triangle_buffer,
                                        cmds[i].triangle_buffer_offset, cmds[i].triangle_buffer_size};
        }
        check(lcx_mesh_build_batch(handles.data(), cs.data(), uint32_t(cmds.size()), stream), "MeshBuildCommand batch");
    }
    void dispatch(const ProceduralPrimitiveBuildCommand &cmd, void *stream) const {
        const LcxProceduralBuildCommand c{static_cast<uint32_t>(cmd.request), 0u, cmd.aabb_buffer,
                                          cmd.aabb_buffer_offset, cmd.aabb_buffer_size};
        check(lcx_procedural_build(cmd.handle, &c, stream), "ProceduralPrimitiveBuildCommand");
    }
    void dispatch(const CurveBuildCommand &cmd, void *stream) const {
        const LcxCurveBuildCommand c{static_cast<uint32_t>(cmd.request), static_cast<uint32_t>(cmd.basis),
                                     cmd.cp_buffer, cmd.cp_buffer_offset, cmd.cp_stride, cmd.cp_count,
                                     cmd.seg_buffer, cmd.seg_buffer_offset, cmd.seg_count};
        check(lcx_curve_build(cmd.handle, &c, stream), "CurveBuildCommand");
    }
    void dispatch(const AccelBuildCommand &cmd, void *stream) const {
        check(lcx_accel_build(cmd.handle, cmd.instance_count, static_cast<uint32_t>(cmd.request),
                              cmd.modifications.data(), cmd.modifications.size(), cmd.update_instance_buffer_only,
                              stream),
              "AccelBuildCommand");
    }

    // Batched ray queries (device buffers).
    void trace_closest(uint64_t accel, const Ray *rays, uint32_t n, uint32_t mask, TriangleHit *hits,
                       void *stream) const {
        check(lcx_trace_closest(accel, rays, n, mask, hits, stream), "trace_closest");
    }
    void trace_any(uint64_t accel, const Ray *rays, uint32_t n, uint32_t mask, uint8_t *occluded,
                   void *stream) const {
        check(lcx_trace_any(accel, rays, n, mask, occluded, stream), "trace_any");
    }
    // The same queries over host buffers (the CPU backend's form), copies overlapped with the traversal.
    void trace_closest_host(uint64_t accel, const Ray *rays, uint32_t n, uint32_t mask, TriangleHit *hits,
                            void *stream, uint32_t layout = LCX_NODES_QUANT8) const {
        check(lcx_trace_closest_host(accel, rays, n, mask, hits, layout, stream), "trace_closest_host");
    }
    void trace_any_host(uint64_t accel, const Ray *rays, uint32_t n, uint32_t mask, uint8_t *occluded, void *stream,
                        uint32_t layout = LCX_NODES_QUANT8) const {
        check(lcx_trace_any_host(accel, rays, n, mask, occluded, layout, stream), "trace_any_host");
    }
    // Accel::intersect_motion / intersect_any_motion: a time per ray (device array, null = 0).
    void trace_closest_motion(uint64_t accel, const Ray *rays, const float *times, uint32_t n, uint32_t mask,
                              TriangleHit *hits, void *stream, uint32_t layout = LCX_NODES_QUANT8) const {
        check(lcx_trace_closest_motion(accel, rays, times, n, mask, hits, layout, stream), "trace_closest_motion");
    }
    void trace_any_motion(uint64_t accel, const Ray *rays, const float *times, uint32_t n, uint32_t mask,
                          uint8_t *occluded, void *stream, uint32_t layout = LCX_NODES_QUANT8) const {
        check(lcx_trace_any_motion(accel, rays, times, n, mask, occluded, layout, stream), "trace_any_motion");
    }
    // Ray batches of many jobs (accels, closest or any) in one launch per kind.
    void trace_jobs(const std::vector<LcxTraceJob> &jobs, void *stream, uint32_t layout = LCX_NODES_QUANT8) const {
        check(lcx_trace_jobs(jobs.data(), uint32_t(jobs.size()), layout, stream), "trace_jobs");
    }
    // times[i]: job i's per-ray times (device-accessible) or null for time 0
    void trace_jobs_motion(const std::vector<LcxTraceJob> &jobs, const std::vector<const float *> &times,
                           void *stream, uint32_t layout = LCX_NODES_QUANT8) const {
        if (times.size() != jobs.size()) throw Error(LCX_ERR_INVALID_ARG, "trace_jobs_motion: one time array per job");
        check(lcx_trace_jobs_motion(jobs.data(), times.data(), uint32_t(jobs.size()), layout, stream),
              "trace_jobs_motion");
    }
    // The accel for lcx::ray_query in the backend's own kernels (include/lcx/ray_query.cuh).
    [[nodiscard]] LcxAccelView device_view(uint64_t accel) const {
        LcxAccelView v{};
        check(lcx_accel_device_view(accel, &v), "device_view");
        return v;
    }
    // The accel's instances for device-side edits (include/lcx/accel_instances.cuh).
    [[nodiscard]] LcxInstanceBuffer instance_buffer(uint64_t accel) const {
        LcxInstanceBuffer b{};
        check(lcx_accel_instance_buffer(accel, &b), "instance_buffer");
        return b;
    }
    [[nodiscard]] LcxAccelStats mesh_stats(uint64_t mesh) const {
        LcxAccelStats s{};
        check(lcx_mesh_stats(mesh, &s), "mesh_stats");
        return s;
    }
};

// ---------------------------------------------------------------- RAII layer

class Mesh {
public:
    // vertices: device float3-in-16-byte records (stride multiple of 16); triangles: device uint3
    Mesh(const AccelGpuExt &ext, uint64_t vertex_buffer, size_t vertex_count, size_t vertex_stride,
         uint64_t triangle_buffer, size_t triangle_count, const AccelOption &option = {})
        : ext_(&ext), v_(vertex_buffer), v_stride_(vertex_stride), v_size_(vertex_count * vertex_stride),
          t_(triangle_buffer), t_size_(triangle_count * sizeof(LcxTriangle)) {
        handle_ = ext.create_mesh(option).handle;
    }
    Mesh(const Mesh &) = delete;
    Mesh &operator=(const Mesh &) = delete;
    ~Mesh() {
        if (handle_) lcx_mesh_destroy(handle_);
    }
    // src/runtime/rtx/mesh.cpp:6-12
    [[nodiscard]] MeshBuildCommand build(AccelBuildRequest request = AccelBuildRequest::FORCE_BUILD) const {
        return MeshBuildCommand{handle_, request, v_, 0, v_size_, v_stride_, t_, 0, t_size_};
    }
    [[nodiscard]] uint64_t handle() const noexcept { return handle_; }

private:
    const AccelGpuExt *ext_;
    uint64_t handle_{0};
    uint64_t v_;
    size_t v_stride_, v_size_;
    uint64_t t_;
    size_t t_size_;
};

class ProceduralPrimitive {
public:
    // aabbs: device array of `count` 24-byte {float min[3], max[3]} records
    ProceduralPrimitive(const AccelGpuExt &ext, uint64_t aabbs, size_t count, const AccelOption &option = {})
        : ext_(&ext), aabbs_(aabbs), size_(count * 24) {
        handle_ = ext.create_procedural_primitive(option).handle;
    }
    ProceduralPrimitive(const ProceduralPrimitive &) = delete;
    ProceduralPrimitive &operator=(const ProceduralPrimitive &) = delete;
    ~ProceduralPrimitive() {
        if (handle_) lcx_procedural_destroy(handle_);
    }
    [[nodiscard]] ProceduralPrimitiveBuildCommand build(
        AccelBuildRequest request = AccelBuildRequest::FORCE_BUILD) const {
        return ProceduralPrimitiveBuildCommand{handle_, request, aabbs_, 0, size_};
    }
    [[nodiscard]] uint64_t handle() const noexcept { return handle_; }

private:
    const AccelGpuExt *ext_;
    uint64_t handle_{0};
    uint64_t aabbs_;
    size_t size_;
};

class Curve {
public:
    // control_points: device array of `cp_count` float4 {x, y, z, radius}; segments: `seg_count` u32
    Curve(const AccelGpuExt &ext, CurveBasis basis, uint64_t control_points, size_t cp_count, uint64_t segments,
          size_t seg_count, const AccelOption &option = {})
        : ext_(&ext), basis_(basis), cps_(control_points), cp_count_(cp_count), segs_(segments),
          seg_count_(seg_count) {
        handle_ = ext.create_curve(option).handle;
    }
    Curve(const Curve &) = delete;
    Curve &operator=(const Curve &) = delete;
    ~Curve() {
        if (handle_) lcx_curve_destroy(handle_);
    }
    [[nodiscard]] CurveBuildCommand build(AccelBuildRequest request = AccelBuildRequest::FORCE_BUILD) const {
        return CurveBuildCommand{handle_, request, basis_, cp_count_, seg_count_, cps_, 0, 16, segs_, 0};
    }
    [[nodiscard]] uint64_t handle() const noexcept { return handle_; }

private:
    const AccelGpuExt *ext_;
    uint64_t handle_{0};
    CurveBasis basis_;
    uint64_t cps_;
    size_t cp_count_;
    uint64_t segs_;
    size_t seg_count_;
};

// include/luisa/runtime/rtx/motion_instance.h: a built mesh (or curve) moved by keyframes.
class MotionInstance {
public:
    MotionInstance(const AccelGpuExt &ext, uint64_t child, const LcxMotionOption &option,
                   const std::vector<std::array<float, 12>> &keyframes, void *stream = nullptr) {
        handle_ = ext.create_motion_instance(child, option, keyframes, stream).handle;
    }
    MotionInstance(const MotionInstance &) = delete;
    MotionInstance &operator=(const MotionInstance &) = delete;
    ~MotionInstance() {
        if (handle_) lcx_motion_instance_destroy(handle_);
    }
    [[nodiscard]] uint64_t handle() const noexcept { return handle_; }

private:
    uint64_t handle_{0};
};

class Accel {
public:
    explicit Accel(const AccelGpuExt &ext, const AccelOption &option = {}) : ext_(&ext) {
        handle_ = ext.create_accel(option).handle;
    }
    Accel(const Accel &) = delete;
    Accel &operator=(const Accel &) = delete;
    ~Accel() {
        if (handle_) lcx_accel_destroy(handle_);
    }

    // src/runtime/rtx/accel.cpp:88-100; transform is row-major 3x4 (command.h:557-571)
    void emplace_back(const Mesh &mesh, const std::array<float, 12> &affine, uint8_t visibility_mask = 0xffu,
                      bool opaque = true, uint32_t user_id = 0) {
        emplace_handle(mesh.handle(), affine, visibility_mask, opaque, user_id);
    }
    void emplace_back(const ProceduralPrimitive &prim, const std::array<float, 12> &affine,
                      uint8_t visibility_mask = 0xffu, bool opaque = true, uint32_t user_id = 0) {
        emplace_handle(prim.handle(), affine, visibility_mask, opaque, user_id);
    }
    void emplace_back(const Curve &curve, const std::array<float, 12> &affine, uint8_t visibility_mask = 0xffu,
                      bool opaque = true, uint32_t user_id = 0) {
        emplace_handle(curve.handle(), affine, visibility_mask, opaque, user_id);
    }
    // a motion instance moves by its own keyframes, so it takes no transform here
    void emplace_back(const MotionInstance &instance, uint8_t visibility_mask = 0xffu, bool opaque = true,
                      uint32_t user_id = 0) {
        emplace_handle(instance.handle(), {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0}, visibility_mask, opaque, user_id);
    }
    // src/runtime/rtx/accel.cpp:114-131, 163-193: replace instance `index` (primitive, transform, mask,
    // opacity, user id), or only its primitive
    void set(uint32_t index, const Mesh &mesh, const std::array<float, 12> &affine, uint8_t visibility_mask = 0xffu,
             bool opaque = true, uint32_t user_id = 0) {
        set_handle(index, mesh.handle(), affine, visibility_mask, opaque, user_id);
    }
    void set(uint32_t index, const Curve &curve, const std::array<float, 12> &affine, uint8_t visibility_mask = 0xffu,
             bool opaque = true, uint32_t user_id = 0) {
        set_handle(index, curve.handle(), affine, visibility_mask, opaque, user_id);
    }
    void set(uint32_t index, const ProceduralPrimitive &prim, const std::array<float, 12> &affine,
             uint8_t visibility_mask = 0xffu, bool opaque = true, uint32_t user_id = 0) {
        set_handle(index, prim.handle(), affine, visibility_mask, opaque, user_id);
    }
    void set(uint32_t index, const MotionInstance &instance, uint8_t visibility_mask = 0xffu, bool opaque = true,
             uint32_t user_id = 0) {
        set_handle(index, instance.handle(), {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0}, visibility_mask, opaque, user_id);
    }
    // set_mesh / set_curve / set_procedural_primitive / set_motion_instance: the primitive only
    void set_mesh(uint32_t index, const Mesh &mesh) { set_prim_handle(index, mesh.handle()); }
    void set_curve(uint32_t index, const Curve &curve) { set_prim_handle(index, curve.handle()); }
    void set_procedural_primitive(uint32_t index, const ProceduralPrimitive &prim) {
        set_prim_handle(index, prim.handle());
    }
    void set_motion_instance(uint32_t index, const MotionInstance &instance) {
        set_prim_handle(index, instance.handle());
    }
    void set_prim_handle(uint32_t index, uint64_t primitive) {
        Modification &m = checked_mod(index);
        m.primitive = primitive;
        m.flags |= LCX_MOD_PRIMITIVE;
    }
    void set_handle(uint32_t index, uint64_t primitive, const std::array<float, 12> &affine, uint8_t visibility_mask,
                    bool opaque, uint32_t user_id) {
        Modification &m = checked_mod(index);
        m.primitive = primitive;
        std::memcpy(m.affine, affine.data(), sizeof(m.affine));
        m.vis_mask = visibility_mask;
        m.user_id = user_id;
        m.flags = LCX_MOD_PRIMITIVE | LCX_MOD_TRANSFORM | LCX_MOD_VISIBILITY | LCX_MOD_USER_ID |
                  (opaque ? LCX_MOD_OPAQUE_ON : LCX_MOD_OPAQUE_OFF);
    }
    void emplace_handle(uint64_t primitive, const std::array<float, 12> &affine, uint8_t visibility_mask,
                        bool opaque, uint32_t user_id) {
        const auto index = static_cast<uint32_t>(count_);
        Modification &m = mod(index);
        m.primitive = primitive;
        std::memcpy(m.affine, affine.data(), sizeof(m.affine));
        m.vis_mask = visibility_mask;
        m.user_id = user_id;
        m.flags = LCX_MOD_PRIMITIVE | LCX_MOD_TRANSFORM | LCX_MOD_VISIBILITY | LCX_MOD_USER_ID |
                  (opaque ? LCX_MOD_OPAQUE_ON : LCX_MOD_OPAQUE_OFF);
        count_++;
    }
    void pop_back() {
        if (count_ == 0) return;
        count_--;
        mods_.erase(static_cast<uint32_t>(count_));
    }
    void set_transform_on_update(uint32_t index, const std::array<float, 12> &affine) {
        Modification &m = checked_mod(index);
        std::memcpy(m.affine, affine.data(), sizeof(m.affine));
        m.flags |= LCX_MOD_TRANSFORM;
    }
    void set_visibility_on_update(uint32_t index, uint8_t mask) {
        Modification &m = checked_mod(index);
        m.vis_mask = mask;
        m.flags |= LCX_MOD_VISIBILITY;
    }
    void set_opaque_on_update(uint32_t index, bool opaque) {
        Modification &m = checked_mod(index);
        m.flags = (m.flags & ~uint32_t(LCX_MOD_OPAQUE_ON | LCX_MOD_OPAQUE_OFF)) |
                  (opaque ? LCX_MOD_OPAQUE_ON : LCX_MOD_OPAQUE_OFF);
    }
    void set_user_id_on_update(uint32_t index, uint32_t user_id) {
        Modification &m = checked_mod(index);
        m.user_id = user_id;
        m.flags |= LCX_MOD_USER_ID;
    }
    // src/runtime/rtx/accel.cpp:68-86 (the staged modifications are consumed)
    [[nodiscard]] AccelBuildCommand build(AccelBuildRequest request = AccelBuildRequest::FORCE_BUILD,
                                          bool update_instance_buffer_only = false) {
        AccelBuildCommand cmd{handle_, static_cast<uint32_t>(count_), request, {}, update_instance_buffer_only};
        cmd.modifications.reserve(mods_.size());
        for (auto &kv : mods_) cmd.modifications.push_back(kv.second);
        mods_.clear();
        return cmd;
    }
    [[nodiscard]] uint64_t handle() const noexcept { return handle_; }
    [[nodiscard]] size_t size() const noexcept { return count_; }

private:
    Modification &mod(uint32_t index) {
        auto it = mods_.find(index);
        if (it == mods_.end()) {
            Modification m{};
            m.index = index;
            it = mods_.emplace(index, m).first;
        }
        return it->second;
    }
    Modification &checked_mod(uint32_t index) {
        if (index >= count_) throw std::out_of_range("instance index out of range");
        return mod(index);
    }
    const AccelGpuExt *ext_;
    uint64_t handle_{0};
    size_t count_{0};
    std::map<uint32_t, Modification> mods_;
};

// `stream << mesh.build() << accel.build()` in the reference becomes
// CommandStream{ext, stream} << mesh.build() << accel.build().
class CommandStream {
public:
    CommandStream(const AccelGpuExt &ext, void *stream) : ext_(&ext), stream_(stream) {}
    CommandStream &operator<<(const MeshBuildCommand &c) {
        ext_->dispatch(c, stream_);
        return *this;
    }
    CommandStream &operator<<(const AccelBuildCommand &c) {
        ext_->dispatch(c, stream_);
        return *this;
    }
    CommandStream &operator<<(const std::vector<MeshBuildCommand> &c) {
        ext_->dispatch(c, stream_);
        return *this;
    }
    CommandStream &operator<<(const ProceduralPrimitiveBuildCommand &c) {
        ext_->dispatch(c, stream_);
        return *this;
    }
    CommandStream &operator<<(const CurveBuildCommand &c) {
        ext_->dispatch(c, stream_);
        return *this;
    }

private:
    const AccelGpuExt *ext_;
    void *stream_;
};

}  // namespace lcx
