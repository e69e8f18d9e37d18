// C++ host API test: builds a mesh + accel through lcx::AccelGpuExt with the
// reference-shaped command flow and checks analytic hits.  Exit code 0 = pass.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "lcx/accel_ext.hpp"

#define REQUIRE(c)                                                      \
    do {                                                                \
        if (!(c)) {                                                     \
            std::fprintf(stderr, "FAILED %s at line %d\n", #c, __LINE__); \
            return 1;                                                   \
        }                                                               \
    } while (0)

int main() {
    try {
        lcx::AccelGpuExt ext{0};
        REQUIRE(lcx::AccelGpuExt::name == "AccelGpuExt");
        // unit quad in z = 0 made of two triangles
        const float verts[4][4] = {{0, 0, 0, 0}, {1, 0, 0, 0}, {0, 1, 0, 0}, {1, 1, 0, 0}};
        const uint32_t tris[2][3] = {{0, 1, 2}, {1, 3, 2}};
        void *dv = nullptr, *dt = nullptr, *dr = nullptr, *dh = nullptr, *docc = nullptr;
        REQUIRE(cudaMalloc(&dv, sizeof(verts)) == cudaSuccess);
        REQUIRE(cudaMalloc(&dt, sizeof(tris)) == cudaSuccess);
        cudaMemcpy(dv, verts, sizeof(verts), cudaMemcpyHostToDevice);
        cudaMemcpy(dt, tris, sizeof(tris), cudaMemcpyHostToDevice);
        lcx::Mesh mesh{ext, reinterpret_cast<uint64_t>(dv), 4, 16, reinterpret_cast<uint64_t>(dt), 2};
        lcx::Accel accel{ext};
        accel.emplace_back(mesh, {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0}, 0x01u);          // identity, mask 1
        accel.emplace_back(mesh, {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, -2}, 0x02u, true, 7);  // z = -2, mask 2
        lcx::CommandStream stream{ext, nullptr};
        stream << mesh.build() << accel.build();

        std::vector<lcx::Ray> rays(4);
        auto set = [&](int i, float x, float y) {
            rays[i] = lcx::Ray{{x, y, 5.0f}, 0.0f, {0.0f, 0.0f, -1.0f}, 1e30f};
        };
        set(0, 0.25f, 0.25f);  // triangle 0 of instance 0
        set(1, 0.75f, 0.75f);  // triangle 1 of instance 0
        set(2, 2.0f, 2.0f);    // miss
        set(3, 0.25f, 0.75f);  // triangle 0 (u = 0.25, v = 0.75 ... on edge 1-2 side)
        REQUIRE(cudaMalloc(&dr, sizeof(lcx::Ray) * rays.size()) == cudaSuccess);
        REQUIRE(cudaMalloc(&dh, sizeof(lcx::TriangleHit) * rays.size()) == cudaSuccess);
        REQUIRE(cudaMalloc(&docc, rays.size()) == cudaSuccess);
        cudaMemcpy(dr, rays.data(), sizeof(lcx::Ray) * rays.size(), cudaMemcpyHostToDevice);
        ext.trace_closest(accel.handle(), static_cast<lcx::Ray *>(dr), 4, 0xffu, static_cast<lcx::TriangleHit *>(dh),
                          nullptr);
        std::vector<lcx::TriangleHit> hits(4);
        cudaMemcpy(hits.data(), dh, sizeof(lcx::TriangleHit) * 4, cudaMemcpyDeviceToHost);
        REQUIRE(hits[0].inst == 0 && hits[0].prim == 0 && hits[0].committed_ray_t == 5.0f);
        REQUIRE(hits[0].bary[0] == 0.25f && hits[0].bary[1] == 0.25f);
        REQUIRE(hits[1].inst == 0 && hits[1].prim == 1);
        REQUIRE(hits[2].inst == 0xffffffffu && hits[2].committed_ray_t == 1e30f);
        REQUIRE(hits[3].inst == 0);
        // mask 2 sees only the lower instance (t = 7)
        ext.trace_closest(accel.handle(), static_cast<lcx::Ray *>(dr), 4, 0x02u, static_cast<lcx::TriangleHit *>(dh),
                          nullptr);
        cudaMemcpy(hits.data(), dh, sizeof(lcx::TriangleHit) * 4, cudaMemcpyDeviceToHost);
        REQUIRE(hits[0].inst == 1 && hits[0].committed_ray_t == 7.0f);
        ext.trace_any(accel.handle(), static_cast<lcx::Ray *>(dr), 4, 0xffu, static_cast<uint8_t *>(docc), nullptr);
        uint8_t occ[4];
        cudaMemcpy(occ, docc, 4, cudaMemcpyDeviceToHost);
        REQUIRE(occ[0] == 1 && occ[1] == 1 && occ[2] == 0 && occ[3] == 1);
        // updates: hide instance 0, move instance 1
        accel.set_visibility_on_update(0, 0);
        accel.set_transform_on_update(1, {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, -1});
        stream << accel.build();
        ext.trace_closest(accel.handle(), static_cast<lcx::Ray *>(dr), 4, 0xffu, static_cast<lcx::TriangleHit *>(dh),
                          nullptr);
        cudaMemcpy(hits.data(), dh, sizeof(lcx::TriangleHit) * 4, cudaMemcpyDeviceToHost);
        REQUIRE(hits[0].inst == 1 && hits[0].committed_ray_t == 6.0f);
        // batched builds and refit: two meshes built together with allow_update, refit together
        lcx::AccelOption upd;
        upd.allow_update = true;
        lcx::Mesh ma{ext, reinterpret_cast<uint64_t>(dv), 4, 16, reinterpret_cast<uint64_t>(dt), 2, upd};
        lcx::Mesh mb{ext, reinterpret_cast<uint64_t>(dv), 4, 16, reinterpret_cast<uint64_t>(dt), 2, upd};
        stream << std::vector<lcx::MeshBuildCommand>{ma.build(), mb.build()};
        REQUIRE(ext.mesh_stats(ma.handle()).refits == 0);
        stream << std::vector<lcx::MeshBuildCommand>{ma.build(lcx::AccelBuildRequest::PREFER_UPDATE),
                                                     mb.build(lcx::AccelBuildRequest::PREFER_UPDATE)};
        REQUIRE(ext.mesh_stats(ma.handle()).refits == 1 && ext.mesh_stats(mb.handle()).refits == 1);
        // a procedural primitive (one AABB above the quad): instanced, invisible to trace calls
        const float box[6] = {0.0f, 0.0f, 1.0f, 1.0f, 1.0f, 2.0f};
        void *dbox = nullptr;
        REQUIRE(cudaMalloc(&dbox, sizeof(box)) == cudaSuccess);
        cudaMemcpy(dbox, box, sizeof(box), cudaMemcpyHostToDevice);
        lcx::ProceduralPrimitive prim{ext, reinterpret_cast<uint64_t>(dbox), 1};
        lcx::Accel mixed{ext};
        mixed.emplace_back(ma, {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0});
        mixed.emplace_back(prim, {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0});
        stream << prim.build() << mixed.build();
        ext.trace_closest(mixed.handle(), static_cast<lcx::Ray *>(dr), 4, 0xffu, static_cast<lcx::TriangleHit *>(dh),
                          nullptr);
        cudaMemcpy(hits.data(), dh, sizeof(lcx::TriangleHit) * 4, cudaMemcpyDeviceToHost);
        REQUIRE(hits[0].inst == 0 && hits[0].committed_ray_t == 5.0f);  // the box at z in [1, 2] is not hit
        const LcxAccelView view = ext.device_view(mixed.handle());
        REQUIRE(view.tlas_nodes != nullptr && view.instances != nullptr && view.stack_need <= 32);
        // the same rays as one job of a multi-job launch
        std::vector<LcxTraceJob> jobs{
            LcxTraceJob{mixed.handle(), static_cast<const LcxRay *>(dr), dh, 4u, 0xffu, 0u, 0u}};
        ext.trace_jobs(jobs, nullptr);
        std::vector<lcx::TriangleHit> hits2(4);
        cudaMemcpy(hits2.data(), dh, sizeof(lcx::TriangleHit) * 4, cudaMemcpyDeviceToHost);
        REQUIRE(std::memcmp(hits2.data(), hits.data(), sizeof(lcx::TriangleHit) * 4) == 0);
        cudaFree(dbox);
        // a curve: one linear strand of radius 0.1 along x at y = 0.25, z = 1, above the quad
        const float cps[2][4] = {{0.0f, 0.25f, 1.0f, 0.1f}, {1.0f, 0.25f, 1.0f, 0.1f}};
        const uint32_t seg0 = 0;
        void *dcp = nullptr, *dseg = nullptr;
        REQUIRE(cudaMalloc(&dcp, sizeof(cps)) == cudaSuccess && cudaMalloc(&dseg, sizeof(seg0)) == cudaSuccess);
        cudaMemcpy(dcp, cps, sizeof(cps), cudaMemcpyHostToDevice);
        cudaMemcpy(dseg, &seg0, sizeof(seg0), cudaMemcpyHostToDevice);
        {
            lcx::Curve strand{ext, lcx::CurveBasis::PIECEWISE_LINEAR, reinterpret_cast<uint64_t>(dcp), 2,
                              reinterpret_cast<uint64_t>(dseg), 1};
            lcx::Accel hair{ext};
            hair.emplace_back(ma, {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0});
            hair.emplace_back(strand, {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0});
            stream << strand.build() << hair.build();
            ext.trace_closest(hair.handle(), static_cast<lcx::Ray *>(dr), 4, 0xffu,
                              static_cast<lcx::TriangleHit *>(dh), nullptr);
            cudaMemcpy(hits.data(), dh, sizeof(lcx::TriangleHit) * 4, cudaMemcpyDeviceToHost);
            // ray 0 meets the strand's top at z = 1.1 (t = 3.9, u = 0.25); ray 1 passes it by
            REQUIRE(hits[0].inst == 1 && hits[0].prim == 0 && hits[0].bary[1] == -1.0f);
            REQUIRE(std::fabs(hits[0].committed_ray_t - 3.9f) < 1e-5f && std::fabs(hits[0].bary[0] - 0.25f) < 1e-5f);
            REQUIRE(hits[1].inst == 0 && hits[1].committed_ray_t == 5.0f);
        }
        cudaFree(dcp);
        cudaFree(dseg);
        // set / set_mesh replace an instance; a motion instance moves the quad from z = 0 to z = -1
        {
            lcx::Accel swap{ext};
            swap.emplace_back(ma, {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0});
            stream << swap.build();
            swap.set(0, mb, {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, -3});
            stream << swap.build();
            ext.trace_closest(swap.handle(), static_cast<lcx::Ray *>(dr), 4, 0xffu,
                              static_cast<lcx::TriangleHit *>(dh), nullptr);
            cudaMemcpy(hits.data(), dh, sizeof(lcx::TriangleHit) * 4, cudaMemcpyDeviceToHost);
            REQUIRE(hits[0].inst == 0 && hits[0].committed_ray_t == 8.0f);
            swap.set_mesh(0, ma);
            stream << swap.build();
            LcxMotionOption mo{2, 0.0f, 1.0f, 0, 0, LCX_MOTION_MATRIX, 0};
            lcx::MotionInstance moving{ext, ma.handle(), mo,
                                       {{1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0}, {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, -1}}};
            lcx::Accel blur{ext};
            blur.emplace_back(moving);
            stream << blur.build();
            std::vector<float> times{1.0f, 0.5f, 0.0f, 0.0f};
            void *dtimes = nullptr;
            REQUIRE(cudaMalloc(&dtimes, sizeof(float) * 4) == cudaSuccess);
            cudaMemcpy(dtimes, times.data(), sizeof(float) * 4, cudaMemcpyHostToDevice);
            ext.trace_closest_motion(blur.handle(), static_cast<lcx::Ray *>(dr), static_cast<const float *>(dtimes), 4,
                                     0xffu, static_cast<lcx::TriangleHit *>(dh), nullptr);
            cudaMemcpy(hits.data(), dh, sizeof(lcx::TriangleHit) * 4, cudaMemcpyDeviceToHost);
            REQUIRE(hits[0].committed_ray_t == 6.0f && hits[1].committed_ray_t == 5.5f);
            cudaFree(dtimes);
        }
        // errors surface as exceptions with the library's status code
        bool threw = false;
        try {
            lcx::Accel empty{ext};
            stream << empty.build();
        } catch (const lcx::Error &e) {
            threw = e.code() == LCX_ERR_INVALID_ARG;
        }
        REQUIRE(threw);
        REQUIRE(lcx_check_trace_errors() == LCX_OK);
        cudaFree(dv);
        cudaFree(dt);
        cudaFree(dr);
        cudaFree(dh);
        cudaFree(docc);
    } catch (const std::exception &e) {
        std::fprintf(stderr, "exception: %s\n", e.what());
        return 1;
    }
    std::puts("accel_ext ok");
    return 0;
}
