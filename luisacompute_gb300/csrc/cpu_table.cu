// cpu_table.cu — the CPU backend's kernel-side accel table over the GPU path.
//
// Kernels of the reference's CPU backend reach an accel through a table of
// per-ray functions (defs::Accel, src/rust/luisa_compute_cpu_kernel_defs/src/lib.rs:111-125),
// filled per binding in src/rust/luisa_compute_backend_impl/src/cpu/stream.rs:546-560
// and called from the generated code (src/rust/luisa_compute_backend_impl/src/cpu/codegen/cpp.rs:1334-1350).
// lcx_accel_cpu_table fills a table of the same shape whose functions run on
// the GPU path: each call is one host round trip through the C ABI (the ray
// and its record in per-thread pinned memory that the kernel reads and writes
// directly, one stream per calling thread).  It is a compatibility form --
// tens of microseconds per ray -- for code that must keep the per-ray calls;
// the batched entry points are the fast form.
//
// ray_query with host callbacks: the device cannot call host function
// pointers, so one kernel enumerates every candidate of the ray in
// [t_min, t_max] (triangles and curve segments with their hit, procedural
// boxes with their entry distance), and the host presents them to the
// callbacks in increasing t (then inst, prim), with the reference's protocol
// (src/rust/luisa_compute_backend_impl/src/cpu/accel.rs:582-800): a commit
// shortens the ray to the committed distance, candidates beyond it are not
// presented, terminate ends the query, and a terminate_on_first query ends at
// its first commit.  Committing every candidate gives lcx_trace_closest's
// record.
#include <algorithm>
#include <cstring>
#include <vector>

#include "lcx/ray_query.cuh"
#include "lcx_internal.h"

namespace {

static_assert(sizeof(LcxCpuRayQuery) == 128, "RayQuery is 128 B");
static_assert(offsetof(LcxCpuRayQuery, ray) == 32 && offsetof(LcxCpuRayQuery, mask) == 64 &&
                  offsetof(LcxCpuRayQuery, cur_triangle_hit) == 72 && offsetof(LcxCpuRayQuery, cur_procedural_hit) == 96 &&
                  offsetof(LcxCpuRayQuery, cur_commited) == 104 && offsetof(LcxCpuRayQuery, user_data) == 112 &&
                  offsetof(LcxCpuRayQuery, accel) == 120,
              "RayQuery layout of cpu_kernel_defs/src/lib.rs:127-141");

constexpr uint32_t kMaxCandidates = 4096;  // per ray_query call

struct Candidate {
    uint32_t kind;  // 1 triangle (or curve segment), 2 procedural box
    uint32_t inst, prim;
    float u, v, t;  // triangle: its hit; box: its entry distance
};

// Per calling thread: pinned memory the kernels read and write, and a stream.
struct ThreadCtx {
    int device = -1;
    cudaStream_t stream = nullptr;
    unsigned char *host = nullptr;  // ray | hit | count | candidates
    LcxRay *ray() { return reinterpret_cast<LcxRay *>(host); }
    LcxTriangleHit *hit() { return reinterpret_cast<LcxTriangleHit *>(host + 32); }
    uint8_t *occ() { return host + 56; }
    uint32_t *count() { return reinterpret_cast<uint32_t *>(host + 60); }
    Candidate *cands() { return reinterpret_cast<Candidate *>(host + 64); }
    ~ThreadCtx() {
        if (host) cudaFreeHost(host);
        if (stream) cudaStreamDestroy(stream);
    }
};
thread_local ThreadCtx t_ctx;

ThreadCtx *thread_ctx() {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return nullptr;
    if (t_ctx.device != dev) {
        if (t_ctx.host) cudaFreeHost(t_ctx.host);
        if (t_ctx.stream) cudaStreamDestroy(t_ctx.stream);
        t_ctx.host = nullptr;
        t_ctx.stream = nullptr;
        if (cudaStreamCreateWithFlags(&t_ctx.stream, cudaStreamNonBlocking) != cudaSuccess ||
            cudaHostAlloc(reinterpret_cast<void **>(&t_ctx.host), 64 + sizeof(Candidate) * kMaxCandidates,
                          cudaHostAllocDefault) != cudaSuccess) {
            cudaGetLastError();
            t_ctx.device = -1;
            return nullptr;
        }
        t_ctx.device = dev;
    }
    return &t_ctx;
}

uint64_t accel_of(const void *handle) { return static_cast<uint64_t>(reinterpret_cast<uintptr_t>(handle)); }

LcxTriangleHit miss_for(const LcxRay *ray) {
    LcxTriangleHit h{};
    h.inst = h.prim = 0xffffffffu;
    if (ray) std::memcpy(&h.committed_ray_t, reinterpret_cast<const unsigned char *>(static_cast<const void *>(ray)) + 28, 4);
    return h;
}

// The caller's ray, copied bytewise (no alignment assumed of the caller's storage).
void copy_ray(ThreadCtx *c, const LcxRay *ray) {
    std::memcpy(c->host, reinterpret_cast<const unsigned char *>(static_cast<const void *>(ray)), sizeof(LcxRay));
}

LcxTriangleHit table_trace_closest(const void *handle, const LcxRay *ray, uint32_t mask) {
    ThreadCtx *c = thread_ctx();
    if (!c || !ray) return miss_for(ray);  // no status in this signature: the error string says why
    copy_ray(c, ray);
    if (lcx_trace_closest_host(accel_of(handle), c->ray(), 1, mask, c->hit(), LCX_NODES_QUANT8, c->stream) != LCX_OK)
        return miss_for(ray);
    if (cudaStreamSynchronize(c->stream) != cudaSuccess) {
        lcx::record_error(LCX_ERR_CUDA, "per-ray trace: stream synchronisation failed");
        return miss_for(ray);
    }
    return *c->hit();
}

bool table_trace_any(const void *handle, const LcxRay *ray, uint32_t mask) {
    ThreadCtx *c = thread_ctx();
    if (!c || !ray) return false;
    copy_ray(c, ray);
    if (lcx_trace_any_host(accel_of(handle), c->ray(), 1, mask, c->occ(), LCX_NODES_QUANT8, c->stream) != LCX_OK)
        return false;
    if (cudaStreamSynchronize(c->stream) != cudaSuccess) return false;
    return *c->occ() != 0;
}

// The instance state record of instance `i` (device), or null.
lcx::InstState *instance_state(const void *handle, uint32_t i) {
    LcxInstanceBuffer b{};
    if (lcx_accel_instance_buffer(accel_of(handle), &b) != LCX_OK) return nullptr;
    if (i >= b.count) {
        lcx::record_error(LCX_ERR_INVALID_ARG, "instance index out of range");
        return nullptr;
    }
    return static_cast<lcx::InstState *>(b.states) + i;
}

template <class T>
void write_field(lcx::InstState *s, size_t offset, const T &v) {
    if (s && cudaMemcpy(reinterpret_cast<char *>(s) + offset, &v, sizeof(T), cudaMemcpyHostToDevice) != cudaSuccess)
        lcx::record_error(LCX_ERR_CUDA, "instance write failed");
}
template <class T>
T read_field(lcx::InstState *s, size_t offset, T dflt) {
    T v = dflt;
    if (s && cudaMemcpy(&v, reinterpret_cast<const char *>(s) + offset, sizeof(T), cudaMemcpyDeviceToHost) != cudaSuccess)
        lcx::record_error(LCX_ERR_CUDA, "instance read failed");
    return v;
}

// Edits take effect at the next lcx_accel_build, as device-side edits do
// (the reference's CPU backend marks the instance dirty, accel.rs:560-579).
void table_set_instance_visibility(const void *handle, uint32_t i, uint32_t mask) {
    write_field(instance_state(handle, i), offsetof(lcx::InstState, mask), mask & 0xffu);
}
void table_set_instance_user_id(const void *handle, uint32_t i, uint32_t user_id) {
    write_field(instance_state(handle, i), offsetof(lcx::InstState, user_id), user_id);
}
// Mat4 is column-major (m[4 * column + row]); the affine rows are its first three
// rows (stream.rs:597-625).
void table_set_instance_transform(const void *handle, uint32_t i, const LcxMat4 *m) {
    if (!m) return;
    struct Rows {
        float v[12];
    } rows;
    for (int r = 0; r < 3; r++)
        for (int c = 0; c < 4; c++) rows.v[4 * r + c] = m->m[4 * c + r];
    write_field(instance_state(handle, i), offsetof(lcx::InstState, o2w), rows);
}
LcxMat4 table_instance_transform(const void *handle, uint32_t i) {
    struct Rows {
        float v[12];
    } rows = {{1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0}};
    rows = read_field(instance_state(handle, i), offsetof(lcx::InstState, o2w), rows);
    LcxMat4 m{};
    for (int r = 0; r < 3; r++)
        for (int c = 0; c < 4; c++) m.m[4 * c + r] = rows.v[4 * r + c];
    m.m[15] = 1.0f;
    return m;
}
uint32_t table_instance_user_id(const void *handle, uint32_t i) {
    return read_field(instance_state(handle, i), offsetof(lcx::InstState, user_id), 0u);
}
uint32_t table_instance_visibility_mask(const void *handle, uint32_t i) {
    return read_field(instance_state(handle, i), offsetof(lcx::InstState, mask), 0xffu);
}

// Every candidate of one ray, in traversal order (all callbacks skip, so the
// interval never shrinks).  Procedural boxes report their entry distance.
__global__ void k_candidates(LcxAccelView view, LcxRay ray, uint32_t mask, Candidate *out, uint32_t cap,
                             uint32_t *count) {
    uint32_t n = 0;
    auto on_tri = [&](const lcx::TriangleCandidate &c) {
        if (n < cap) out[n] = Candidate{1u, c.inst, c.prim, c.bary_u, c.bary_v, c.t};
        n++;
        return int(lcx::kSkip);
    };
    auto on_proc = [&](const lcx::ProceduralCandidate &c) {
        float tn = ray.t_min;
        for (int k = 0; k < 3; k++) {
            const float inv = 1.0f / c.obj_dir[k];
            const float a = (c.aabb_min[k] - c.obj_origin[k]) * inv, b = (c.aabb_max[k] - c.obj_origin[k]) * inv;
            tn = fmaxf(tn, fminf(a, b));
        }
        if (n < cap) out[n] = Candidate{2u, c.inst, c.prim, 0.0f, 0.0f, tn};
        n++;
        return lcx::ProceduralDecision{lcx::kSkip, 0.0f};
    };
    if (view.motion)
        lcx::ray_query_motion(view, ray, 0.0f, mask, on_tri, on_proc);
    else
        lcx::ray_query(view, ray, mask, on_tri, on_proc);
    *count = n;
}

void table_ray_query(const void *handle, LcxCpuRayQuery *rq, LcxCpuHitCallback on_triangle,
                     LcxCpuHitCallback on_procedural) {
    if (!rq) return;
    ThreadCtx *c = thread_ctx();
    LcxAccelView view{};
    if (!c || lcx_accel_device_view(accel_of(handle), &view) != LCX_OK) {
        rq->terminated = true;  // the error string says why
        return;
    }
    *c->count() = 0u;
    k_candidates<<<1, 1, 0, c->stream>>>(view, rq->ray, rq->mask, c->cands(), kMaxCandidates, c->count());
    if (cudaGetLastError() != cudaSuccess || cudaStreamSynchronize(c->stream) != cudaSuccess) {
        lcx::record_error(LCX_ERR_CUDA, "ray_query: candidate kernel failed");
        rq->terminated = true;
        return;
    }
    const uint32_t total = *c->count();
    if (total > kMaxCandidates)
        lcx::record_error(LCX_ERR_INVALID_ARG, "ray_query: more than 4096 candidates; the nearest 4096 were presented");
    std::vector<Candidate> cand(c->cands(), c->cands() + std::min(total, kMaxCandidates));
    std::sort(cand.begin(), cand.end(), [](const Candidate &a, const Candidate &b) {
        if (a.t != b.t) return a.t < b.t;
        if (a.inst != b.inst) return a.inst < b.inst;
        return a.prim < b.prim;
    });
    const float t_near = rq->ray.t_min;
    float t_far = rq->ray.t_max;
    bool committed = false;
    for (const Candidate &k : cand) {
        // [t_min, t_far]; after a commit only candidates strictly before it
        if (k.t < t_near || k.t > t_far || (committed && !(k.t < t_far))) continue;
        rq->ray.t_max = t_far;
        rq->cur_commited = false;
        rq->terminated = false;
        if (k.kind == 1u) {
            rq->cur_triangle_hit.inst = k.inst;
            rq->cur_triangle_hit.prim = k.prim;
            rq->cur_triangle_hit.bary[0] = k.u;
            rq->cur_triangle_hit.bary[1] = k.v;
            rq->cur_triangle_hit.committed_ray_t = k.t;
            rq->cur_triangle_hit._pad = 0u;
            if (on_triangle) on_triangle(rq);
            if (rq->cur_commited) {
                rq->hit.inst = k.inst;
                rq->hit.prim = k.prim;
                rq->hit.bary[0] = k.u;
                rq->hit.bary[1] = k.v;
                rq->hit.hit_type = 1u;
                rq->hit.committed_ray_t = k.t;
                t_far = k.t;
                committed = true;
            }
        } else {
            rq->cur_procedural_hit.inst = k.inst;
            rq->cur_procedural_hit.prim = k.prim;
            if (on_procedural) on_procedural(rq);
            if (rq->cur_commited) {
                const float t = rq->cur_committed_ray_t;
                if (t < t_far && t >= t_near) {
                    rq->hit.inst = k.inst;
                    rq->hit.prim = k.prim;
                    rq->hit.hit_type = 2u;
                    rq->hit.committed_ray_t = t;
                    t_far = t;
                    committed = true;
                } else {
                    rq->cur_commited = false;
                }
            }
        }
        if (rq->terminated || (rq->terminate_on_first && rq->cur_commited)) break;
    }
    rq->ray.t_max = t_far;
}

}  // namespace

extern "C" int lcx_accel_cpu_table(uint64_t accel, LcxCpuAccel *out) {
    if (!out) return lcx::record_error(LCX_ERR_INVALID_ARG, "lcx_accel_cpu_table: out is null");
    LcxAccelView v{};
    if (int r = lcx_accel_device_view(accel, &v)) return r;  // built, current, within the stack
    out->handle = reinterpret_cast<const void *>(static_cast<uintptr_t>(accel));
    out->trace_closest = table_trace_closest;
    out->trace_any = table_trace_any;
    out->set_instance_visibility = table_set_instance_visibility;
    out->set_instance_transform = table_set_instance_transform;
    out->set_instance_user_id = table_set_instance_user_id;
    out->instance_transform = table_instance_transform;
    out->instance_user_id = table_instance_user_id;
    out->instance_visibility_mask = table_instance_visibility_mask;
    out->ray_query = table_ray_query;
    return LCX_OK;
}
