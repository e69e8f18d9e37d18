// pathtrace.cu — wavefront diffuse path tracing over the Mesh/Accel path.
//
// A caller of the hot path, in the shape of the reference's path-tracing
// tests (src/tests/test_path_tracing.cpp) but as a wavefront: every bounce is
// one batched trace_closest over the live paths, one shading kernel (Lambert
// with a point light, constant environment, Russian roulette from
// `rr_start`), one trace_any over the shadow rays and a kernel that adds the
// unoccluded light.  Shading compacts the surviving paths into the next
// bounce's ray queue.  Random numbers are keyed by (path, bounce, dimension)
// and radiance is summed per path in bounce order, then per pixel in sample
// order, so the image does not depend on scheduling.
#include <cstring>
#include <mutex>
#include <vector>

#include "lcx_internal.h"
#include "pt_math.cuh"

namespace lcx {
namespace {

struct PtMeshDev {
    const unsigned char *vertices;
    uint64_t vstride;
    const uint32_t *triangles;
    const float *albedo;
};

struct PtInstDev {
    float w2o[12];
    uint32_t mesh;
    uint32_t _pad[3];
};

struct PtBuffers {
    Ray *rays[2];
    Hit *hits;
    uint32_t *path[2];  // path id of each queued ray
    float *thr;         // 3 per path
    float *rad;         // 3 per path
    Ray *srays;
    uint8_t *occ;
    uint32_t *spath;
    float *pending;     // 3 per shadow ray
    uint32_t *counts;   // [0] next queue length, [1] shadow rays
};

__global__ void k_pt_prep_insts(const float *o2w, const uint32_t *mesh_of, uint32_t n, PtInstDev *out) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float m[12], w[12];
    for (int k = 0; k < 12; k++) m[k] = o2w[12 * i + k];
    affine_inverse(m, w);
    for (int k = 0; k < 12; k++) out[i].w2o[k] = w[k];
    out[i].mesh = mesh_of[i];
}

__global__ void k_pt_generate(LcxPtParams P, Ray *rays, uint32_t *path, float *thr, float *rad) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t n = P.width * P.height * P.spp;
    if (i >= n) return;
    const uint32_t pixel = i / P.spp;
    const uint32_t px = pixel % P.width, py = pixel / P.width;
    // camera basis (identical arithmetic on the CPU)
    float fwd[3] = {LCX_SUB(P.target[0], P.eye[0]), LCX_SUB(P.target[1], P.eye[1]), LCX_SUB(P.target[2], P.eye[2])};
    pt::normalize3(fwd);
    float right[3] = {LCX_SUB(LCX_MUL(fwd[1], P.up[2]), LCX_MUL(fwd[2], P.up[1])),
                      LCX_SUB(LCX_MUL(fwd[2], P.up[0]), LCX_MUL(fwd[0], P.up[2])),
                      LCX_SUB(LCX_MUL(fwd[0], P.up[1]), LCX_MUL(fwd[1], P.up[0]))};
    pt::normalize3(right);
    const float up[3] = {LCX_SUB(LCX_MUL(right[1], fwd[2]), LCX_MUL(right[2], fwd[1])),
                         LCX_SUB(LCX_MUL(right[2], fwd[0]), LCX_MUL(right[0], fwd[2])),
                         LCX_SUB(LCX_MUL(right[0], fwd[1]), LCX_MUL(right[1], fwd[0]))};
    const float jx = pt::uniform(P.seed, i, 0, 0), jy = pt::uniform(P.seed, i, 0, 1);
    const float sx = LCX_MUL(LCX_MUL(LCX_SUB(LCX_MUL(LCX_DIV(LCX_ADD(float(px), jx), float(P.width)), 2.0f), 1.0f),
                                     P.tan_half_fov),
                             LCX_DIV(float(P.width), float(P.height)));
    const float sy = LCX_MUL(LCX_SUB(1.0f, LCX_MUL(LCX_DIV(LCX_ADD(float(py), jy), float(P.height)), 2.0f)),
                             P.tan_half_fov);
    float d[3];
    for (int k = 0; k < 3; k++) d[k] = LCX_FMA(sx, right[k], LCX_FMA(sy, up[k], fwd[k]));
    pt::normalize3(d);
    Ray r;
    r.ox = P.eye[0];
    r.oy = P.eye[1];
    r.oz = P.eye[2];
    r.tmin = 0.0f;
    r.dx = d[0];
    r.dy = d[1];
    r.dz = d[2];
    r.tmax = 1e30f;
    rays[i] = r;
    path[i] = i;
    for (int k = 0; k < 3; k++) {
        thr[3 * i + k] = 1.0f;
        rad[3 * i + k] = 0.0f;
    }
}

// Shading of queue entry j at bounce b: environment on a miss; otherwise a
// shadow ray toward the light and, if the path survives, a cosine-weighted
// continuation appended to the next queue.
__global__ void k_pt_shade(LcxPtParams P, uint32_t bounce, uint32_t n, const Ray *rays, const Hit *hits,
                           const uint32_t *path, const PtMeshDev *meshes, const PtInstDev *insts, float *thr,
                           float *rad, Ray *next_rays, uint32_t *next_path, Ray *srays, uint32_t *spath,
                           float *pending, uint32_t *counts) {
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    const uint32_t id = path[j];
    const Hit h = hits[j];
    const Ray r = rays[j];
    float T[3] = {thr[3 * id], thr[3 * id + 1], thr[3 * id + 2]};
    if (h.inst == kInvalid) {
        for (int k = 0; k < 3; k++) rad[3 * id + k] = LCX_FMA(T[k], P.env[k], rad[3 * id + k]);
        return;
    }
    const PtInstDev &I = insts[h.inst];
    const PtMeshDev &M = meshes[I.mesh];
    const uint32_t *tri = M.triangles + 3ull * h.prim;
    const float4 v0 = *reinterpret_cast<const float4 *>(M.vertices + M.vstride * tri[0]);
    const float4 v1 = *reinterpret_cast<const float4 *>(M.vertices + M.vstride * tri[1]);
    const float4 v2 = *reinterpret_cast<const float4 *>(M.vertices + M.vstride * tri[2]);
    const float e1[3] = {LCX_SUB(v1.x, v0.x), LCX_SUB(v1.y, v0.y), LCX_SUB(v1.z, v0.z)};
    const float e2[3] = {LCX_SUB(v2.x, v0.x), LCX_SUB(v2.y, v0.y), LCX_SUB(v2.z, v0.z)};
    const float no[3] = {LCX_SUB(LCX_MUL(e1[1], e2[2]), LCX_MUL(e1[2], e2[1])),
                         LCX_SUB(LCX_MUL(e1[2], e2[0]), LCX_MUL(e1[0], e2[2])),
                         LCX_SUB(LCX_MUL(e1[0], e2[1]), LCX_MUL(e1[1], e2[0]))};
    // world normal = transpose(world-to-object) * object normal
    float N[3];
    for (int k = 0; k < 3; k++) N[k] = LCX_FMA(I.w2o[k], no[0], LCX_FMA(I.w2o[4 + k], no[1], LCX_MUL(I.w2o[8 + k], no[2])));
    pt::normalize3(N);
    const float d[3] = {r.dx, r.dy, r.dz};
    if (LCX_FMA(N[0], d[0], LCX_FMA(N[1], d[1], LCX_MUL(N[2], d[2]))) > 0.0f) {
        N[0] = -N[0];
        N[1] = -N[1];
        N[2] = -N[2];
    }
    const float p[3] = {LCX_FMA(h.t, d[0], r.ox), LCX_FMA(h.t, d[1], r.oy), LCX_FMA(h.t, d[2], r.oz)};
    const float po[3] = {pt::offset_coord(p[0], N[0]), pt::offset_coord(p[1], N[1]), pt::offset_coord(p[2], N[2])};
    const float albedo = M.albedo[h.prim];
    // direct light through a shadow ray
    float wl[3] = {LCX_SUB(P.light_pos[0], po[0]), LCX_SUB(P.light_pos[1], po[1]), LCX_SUB(P.light_pos[2], po[2])};
    const float dist2 = LCX_FMA(wl[0], wl[0], LCX_FMA(wl[1], wl[1], LCX_MUL(wl[2], wl[2])));
    const float dist = LCX_SQRT(dist2);
    for (int k = 0; k < 3; k++) wl[k] = LCX_DIV(wl[k], dist);
    const float cosl = LCX_FMA(N[0], wl[0], LCX_FMA(N[1], wl[1], LCX_MUL(N[2], wl[2])));
    if (cosl > 0.0f) {
        const uint32_t s = atomicAdd(&counts[1], 1u);
        Ray sr;
        sr.ox = po[0];
        sr.oy = po[1];
        sr.oz = po[2];
        sr.tmin = 0.0f;
        sr.dx = wl[0];
        sr.dy = wl[1];
        sr.dz = wl[2];
        sr.tmax = dist;
        srays[s] = sr;
        spath[s] = id;
        const float f = LCX_DIV(LCX_MUL(LCX_MUL(albedo, 0.318309886f), cosl), dist2);
        for (int k = 0; k < 3; k++) pending[3 * s + k] = LCX_MUL(LCX_MUL(T[k], f), P.light_intensity[k]);
    }
    // continuation
    if (bounce + 1 >= P.max_bounces) return;
    for (int k = 0; k < 3; k++) T[k] = LCX_MUL(T[k], albedo);
    if (bounce + 1 >= P.rr_start) {
        const float q = fminf(0.95f, fmaxf(T[0], fmaxf(T[1], T[2])));
        if (pt::uniform(P.seed, id, bounce + 1, 2) >= q) return;
        for (int k = 0; k < 3; k++) T[k] = LCX_DIV(T[k], q);
    }
    float nd[3];
    pt::cosine_dir(N, pt::uniform(P.seed, id, bounce + 1, 0), pt::uniform(P.seed, id, bounce + 1, 1), nd);
    for (int k = 0; k < 3; k++) thr[3 * id + k] = T[k];
    const uint32_t q = atomicAdd(&counts[0], 1u);
    Ray nr;
    nr.ox = po[0];
    nr.oy = po[1];
    nr.oz = po[2];
    nr.tmin = 0.0f;
    nr.dx = nd[0];
    nr.dy = nd[1];
    nr.dz = nd[2];
    nr.tmax = 1e30f;
    next_rays[q] = nr;
    next_path[q] = id;
}

__global__ void k_pt_shadow(uint32_t n, const uint8_t *occ, const uint32_t *spath, const float *pending, float *rad) {
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n || occ[s]) return;
    const uint32_t id = spath[s];
    for (int k = 0; k < 3; k++) rad[3 * id + k] = LCX_ADD(rad[3 * id + k], pending[3 * s + k]);
}

__global__ void k_pt_resolve(LcxPtParams P, const float *rad, float *image) {
    const uint32_t pix = blockIdx.x * blockDim.x + threadIdx.x;
    if (pix >= P.width * P.height) return;
    const float inv = LCX_DIV(1.0f, float(P.spp));
    for (int k = 0; k < 3; k++) {
        float acc = 0.0f;
        for (uint32_t s = 0; s < P.spp; s++) acc = LCX_ADD(acc, rad[3 * (pix * P.spp + s) + k]);
        image[3 * pix + k] = LCX_MUL(acc, inv);
    }
}

inline unsigned blocks(uint64_t n, unsigned b) { return unsigned((n + b - 1) / b); }

// Per-frame buffers from the device's scratch pool (kept between frames);
// freed on scope exit, stream-ordered.
struct PtScratch {
    cudaStream_t st;
    cudaMemPool_t pool = nullptr;
    std::vector<void *> ptrs;
    explicit PtScratch(cudaStream_t s) : st(s) {}
    template <class T>
    cudaError_t alloc(T **p, size_t count) {
        if (!pool && scratch_pool(&pool) != LCX_OK) return cudaErrorMemoryAllocation;
        cudaError_t e = cudaMallocFromPoolAsync(reinterpret_cast<void **>(p), sizeof(T) * (count ? count : 1), pool, st);
        if (e == cudaSuccess) ptrs.push_back(*p);
        return e;
    }
    ~PtScratch() {
        for (void *p : ptrs) cudaFreeAsync(p, st);
    }
};

}  // namespace
}  // namespace lcx

using namespace lcx;

// The side stream of the shadow rays, one per device (created once).
static cudaStream_t side_stream() {
    static std::mutex mtx;
    static cudaStream_t streams[64] = {};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return nullptr;
    std::lock_guard<std::mutex> lk(mtx);
    if (streams[dev] == nullptr && cudaStreamCreateWithFlags(&streams[dev], cudaStreamNonBlocking) != cudaSuccess) {
        cudaGetLastError();
        streams[dev] = nullptr;
    }
    return streams[dev];
}

struct PtEvent {
    cudaEvent_t e = nullptr;
    cudaError_t create() { return cudaEventCreateWithFlags(&e, cudaEventDisableTiming); }
    ~PtEvent() {
        if (e) cudaEventDestroy(e);
    }
};

extern "C" int lcx_pt_render(uint64_t accel, const LcxPtMesh *meshes, uint32_t mesh_count, const uint32_t *inst_mesh,
                             const float *inst_o2w, uint32_t instance_count, const LcxPtParams *params,
                             float *d_image, LcxTriangleHit *d_first_hits, LcxPtStats *stats, void *stream) {
    if (!params || !meshes || !inst_mesh || !inst_o2w || !d_image || mesh_count == 0 || instance_count == 0)
        return record_error(LCX_ERR_INVALID_ARG, "lcx_pt_render: null or empty arguments");
    const LcxPtParams P = *params;
    const uint64_t n64 = uint64_t(P.width) * P.height * P.spp;
    if (n64 == 0 || n64 > (1ull << 31) || P.max_bounces == 0 || P.max_bounces > 64)
        return record_error(LCX_ERR_INVALID_ARG, "lcx_pt_render: image size, spp or bounces out of range");
    for (uint32_t i = 0; i < instance_count; i++)
        if (inst_mesh[i] >= mesh_count) return record_error(LCX_ERR_INVALID_ARG, "instance mesh index out of range");
    const uint32_t n = uint32_t(n64);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    PtScratch sc(st);
    PtBuffers B{};
    PtMeshDev *d_meshes = nullptr;
    PtInstDev *d_insts = nullptr;
    float *d_o2w = nullptr;
    uint32_t *d_mesh_of = nullptr;
    cudaError_t e = cudaSuccess;
#define PT_TRY(x)                                                              \
    do {                                                                       \
        e = (x);                                                               \
        if (e != cudaSuccess) {                                                \
            cudaGetLastError();                                                \
            return record_error(LCX_ERR_CUDA, cudaGetErrorString(e));          \
        }                                                                      \
    } while (0)
    PT_TRY(sc.alloc(&B.rays[0], n));
    PT_TRY(sc.alloc(&B.rays[1], n));
    PT_TRY(sc.alloc(&B.hits, n));
    PT_TRY(sc.alloc(&B.path[0], n));
    PT_TRY(sc.alloc(&B.path[1], n));
    PT_TRY(sc.alloc(&B.thr, 3ull * n));
    PT_TRY(sc.alloc(&B.rad, 3ull * n));
    PT_TRY(sc.alloc(&B.srays, n));
    PT_TRY(sc.alloc(&B.occ, n));
    PT_TRY(sc.alloc(&B.spath, n));
    PT_TRY(sc.alloc(&B.pending, 3ull * n));
    PT_TRY(sc.alloc(&B.counts, 4));
    PT_TRY(sc.alloc(&d_meshes, mesh_count));
    PT_TRY(sc.alloc(&d_insts, instance_count));
    PT_TRY(sc.alloc(&d_o2w, 12ull * instance_count));
    PT_TRY(sc.alloc(&d_mesh_of, instance_count));
    std::vector<PtMeshDev> hm(mesh_count);
    for (uint32_t i = 0; i < mesh_count; i++)
        hm[i] = PtMeshDev{static_cast<const unsigned char *>(meshes[i].vertices), meshes[i].vertex_stride,
                          meshes[i].triangles, meshes[i].albedo};
    PT_TRY(cudaMemcpyAsync(d_meshes, hm.data(), sizeof(PtMeshDev) * mesh_count, cudaMemcpyHostToDevice, st));
    PT_TRY(cudaMemcpyAsync(d_o2w, inst_o2w, sizeof(float) * 12 * instance_count, cudaMemcpyHostToDevice, st));
    PT_TRY(cudaMemcpyAsync(d_mesh_of, inst_mesh, sizeof(uint32_t) * instance_count, cudaMemcpyHostToDevice, st));
    k_pt_prep_insts<<<blocks(instance_count, 128), 128, 0, st>>>(d_o2w, d_mesh_of, instance_count, d_insts);

    cudaEvent_t t_begin, t_end;
    cudaEventCreate(&t_begin);
    cudaEventCreate(&t_end);
    cudaEventRecord(t_begin, st);
    k_pt_generate<<<blocks(n, 256), 256, 0, st>>>(P, B.rays[0], B.path[0], B.thr, B.rad);
    uint32_t live = n;
    uint64_t closest_rays = 0, any_rays = 0;
    uint32_t bounces = 0, launches = 2;  // k_pt_prep_insts, k_pt_generate
    int cur = 0;
    // Bounce b's shadow rays (trace_any, then their radiance) run on a side stream beside bounce
    // b+1's closest-hit trace, which fills the other launch's ramp and tail; the shading of bounce
    // b+1 waits for them, since both add to the same paths' radiance (in bounce order) and it
    // rewrites the shadow buffers.
    cudaStream_t side = side_stream();
    if (side == nullptr) return record_error(LCX_ERR_CUDA, "lcx_pt_render: side stream");
    // on every return the caller's stream (whose order frees the scratch) waits for the side stream
    struct SideJoin {
        cudaStream_t st, side;
        ~SideJoin() {
            cudaEvent_t e = nullptr;
            if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) == cudaSuccess) {
                cudaEventRecord(e, side);
                cudaStreamWaitEvent(st, e, 0);
                cudaEventDestroy(e);
            }
        }
    } join{st, side};
    PtEvent ev_shaded, ev_shadowed;
    PT_TRY(ev_shaded.create());
    PT_TRY(ev_shadowed.create());
    bool shadow_pending = false;
    for (uint32_t b = 0; b < P.max_bounces && live > 0; b++) {
        PT_TRY(cudaMemsetAsync(B.counts, 0, 4 * sizeof(uint32_t), st));
        int r = lcx_trace_closest(accel, reinterpret_cast<const LcxRay *>(B.rays[cur]), live, 0xffu,
                                  reinterpret_cast<LcxTriangleHit *>(B.hits), stream);
        if (r != LCX_OK) return r;
        if (b == 0 && d_first_hits)
            PT_TRY(cudaMemcpyAsync(d_first_hits, B.hits, sizeof(Hit) * n, cudaMemcpyDeviceToDevice, st));
        closest_rays += live;
        launches += 2;  // k_trace, k_pt_shade
        if (shadow_pending) PT_TRY(cudaStreamWaitEvent(st, ev_shadowed.e, 0));
        shadow_pending = false;
        k_pt_shade<<<blocks(live, 128), 128, 0, st>>>(P, b, live, B.rays[cur], B.hits, B.path[cur], d_meshes, d_insts,
                                                       B.thr, B.rad, B.rays[cur ^ 1], B.path[cur ^ 1], B.srays,
                                                       B.spath, B.pending, B.counts);
        PT_TRY(cudaGetLastError());
        uint32_t h_counts[2] = {0, 0};
        PT_TRY(cudaMemcpyAsync(h_counts, B.counts, sizeof(h_counts), cudaMemcpyDeviceToHost, st));
        PT_TRY(cudaStreamSynchronize(st));
        if (h_counts[1]) {
            PT_TRY(cudaEventRecord(ev_shaded.e, st));
            PT_TRY(cudaStreamWaitEvent(side, ev_shaded.e, 0));
            r = lcx_trace_any(accel, reinterpret_cast<const LcxRay *>(B.srays), h_counts[1], 0xffu, B.occ, side);
            if (r != LCX_OK) return r;
            any_rays += h_counts[1];
            launches += 2;  // k_trace, k_pt_shadow
            k_pt_shadow<<<blocks(h_counts[1], 256), 256, 0, side>>>(h_counts[1], B.occ, B.spath, B.pending, B.rad);
            PT_TRY(cudaGetLastError());
            PT_TRY(cudaEventRecord(ev_shadowed.e, side));
            shadow_pending = true;
        }
        live = h_counts[0];
        cur ^= 1;
        bounces = b + 1;
    }
    if (shadow_pending) PT_TRY(cudaStreamWaitEvent(st, ev_shadowed.e, 0));
    k_pt_resolve<<<blocks(uint64_t(P.width) * P.height, 256), 256, 0, st>>>(P, B.rad, d_image);
    PT_TRY(cudaGetLastError());
    cudaEventRecord(t_end, st);
    PT_TRY(cudaEventSynchronize(t_end));
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, t_begin, t_end);
    cudaEventDestroy(t_begin);
    cudaEventDestroy(t_end);
    if (stats) {
        stats->closest_rays = closest_rays;
        stats->any_rays = any_rays;
        stats->bounces = bounces;
        stats->ms = ms;
        stats->launches = launches + 1;  // + k_pt_resolve
    }
    return LCX_OK;
#undef PT_TRY
}
