// capi.cu — the C ABI (include/lcx_accel.h): handle registry, argument
// validation, device memory ownership and orchestration of the build and
// trace kernels.  Mirrors the reference's DeviceInterface accel entry points
// (include/luisa/runtime/rhi/device_interface.h:171-184) and the command
// visits of its backends (CUDA: src/backends/cuda/cuda_command_encoder.cpp:235-243;
// CPU: src/rust/luisa_compute_backend_impl/src/cpu/stream.rs:410-428), with
// status codes in place of the reference's aborts.
#include <algorithm>
#include <chrono>
#include <cstddef>
#include <cmath>
#include <unordered_set>
#include <atomic>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <memory>
#include <mutex>
#include <shared_mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include <cuda.h>  // the types of cuStreamWriteValue32 (taken through the runtime's entry-point query)

#include "lcx_internal.h"

using namespace lcx;

namespace {

thread_local std::string g_last_error;

int fail(int code, const char *fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_last_error = buf;
    return code;
}

int cuda_fail(cudaError_t e, const char *what) {
    cudaGetLastError();  // clear sticky-free errors
    return fail(e == cudaErrorMemoryAllocation ? LCX_ERR_OOM : LCX_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

#define LCX_CUDA(call, what)                               \
    do {                                                   \
        cudaError_t e_ = (call);                           \
        if (e_ != cudaSuccess) return cuda_fail(e_, what); \
    } while (0)

constexpr uint32_t kPoolSlots = 4096;  // trace-call counters (16 B each)
// the last kGraphSlots slots go to calls captured into CUDA graphs, whose slot is
// fixed at capture, so a replay never shares a counter with a live call
constexpr uint32_t kGraphSlots = 512;
// warps overshoot the ray counter by at most 32 each, so 2^31 keeps it from wrapping
constexpr uint32_t kMaxTraceRays = 1u << 31;

struct DeviceState {
    int device = -1;
    uint32_t *pool = nullptr;  // kPoolSlots x 4 words
    uint32_t *refit_ctl = nullptr;  // kCtlWords words: errors of refits that do not synchronise
    std::atomic<uint32_t> next_slot{0};
    std::atomic<uint32_t> next_graph_slot{0};
    // host-buffer traces: copy-in, copy-out and two traversal streams
    cudaStream_t io_in = nullptr, io_out = nullptr, io_trace[2] = {nullptr, nullptr};
    // streamed host-buffer traces (one at a time per device): the copy chunks' flags (device
    // memory, one more word for the support probe), the warps' marks (mapped pinned memory),
    // the generation of the last call, and whether the stream memory write is available
    std::mutex stage_mtx;
    // its own copy-in, copy-out and traversal streams: the traversal waits on what the copy-in
    // stream carries, so no other call may queue work there (a staged call's waits would sit
    // between the chunks' copies)
    cudaStream_t stage_in = nullptr, stage_out = nullptr, stage_trace = nullptr;
    uint32_t *stage_flags = nullptr;
    uint32_t *stage_marks = nullptr, *stage_marks_dev = nullptr;
    uint32_t stage_gen = 0;
    int stage_state = 0;  // 0: not set up yet, 1: ready, 2: unavailable
};

std::mutex g_dev_mtx;
DeviceState g_dev[16];

int current_device_state(DeviceState **out) {
    int dev = 0;
    LCX_CUDA(cudaGetDevice(&dev), "cudaGetDevice");
    if (dev < 0 || dev >= 16) return fail(LCX_ERR_INVALID_ARG, "device index %d out of range", dev);
    std::lock_guard<std::mutex> lk(g_dev_mtx);
    DeviceState &s = g_dev[dev];
    if (s.pool == nullptr) {
        LCX_CUDA(cudaMalloc(&s.pool, kPoolSlots * 4 * sizeof(uint32_t)), "cudaMalloc(trace pool)");
        LCX_CUDA(cudaMemset(s.pool, 0, kPoolSlots * 4 * sizeof(uint32_t)), "cudaMemset(trace pool)");
        LCX_CUDA(cudaMalloc(&s.refit_ctl, kCtlWords * sizeof(uint32_t)), "cudaMalloc(refit errors)");
        LCX_CUDA(cudaMemset(s.refit_ctl, 0, kCtlWords * sizeof(uint32_t)), "cudaMemset(refit errors)");
        LCX_CUDA(cudaStreamCreateWithFlags(&s.io_in, cudaStreamNonBlocking), "cudaStreamCreate");
        LCX_CUDA(cudaStreamCreateWithFlags(&s.io_out, cudaStreamNonBlocking), "cudaStreamCreate");
        for (auto &t : s.io_trace) LCX_CUDA(cudaStreamCreateWithFlags(&t, cudaStreamNonBlocking), "cudaStreamCreate");
        s.device = dev;
    }
    *out = &s;
    return LCX_OK;
}

// Device memory that holds built BVHs; a batch build shares one block
// between its meshes, which keep it alive by reference.
struct DevBlock {
    void *ptr = nullptr;
    size_t bytes = 0;
    // blocks built with allow_update: the layout, the parent table and the
    // scratch a refit needs (all in this allocation, so a refit allocates nothing)
    unsigned long long *rtab = nullptr;
    uint32_t wide = 0, nseg = 0;
    Node8Q *qn = nullptr;
    Node8F *fn = nullptr;
    TriRec *tris = nullptr;           // BLAS
    uint32_t *counters = nullptr;     // wide words
    SegInput *d_segs = nullptr;       // BLAS: the segment table of the last build or refit
    std::vector<SegInput> h_segs;     // its host copy
    float4 *ilo = nullptr, *ihi = nullptr;  // TLAS: instance boxes
    float *w2o = nullptr;             // TLAS: instance inverses
    uint32_t *segctl = nullptr;       // TLAS: kSegWords words
    // reserved batches (lcx_mesh_build_batch_reserve): room for any tree over the
    // same items (cap_wide nodes), the segment table (d_segs / h_segs) and the
    // initial control words on the device, so a rebuild needs no host sync
    bool reserved = false;
    uint32_t items = 0, cap_wide = 0;
    uint32_t *d_segctl_init = nullptr;
    double *wsah = nullptr;
    ~DevBlock() {
        // cudaFree waits for work still using it, without stopping the host.  (BVH blocks from
        // the stream-ordered scratch pool rebuilt a 4096-mesh batch 10 ms faster, with no
        // unmapping, but a cudaFree of pool memory synchronises the device: a serving loop that
        // builds scenes while other requests trace went from 0.45 / 4.3 ms to 8.2 / 150 ms at
        // p50 / p99.)
        if (ptr) cudaFree(ptr);
    }
};

// BVH lifetime.  Trace calls hold g_life_mtx shared from the accel lookup
// until their kernel is enqueued.  Releasing BVH memory (destroy, rebuild)
// takes it exclusively once, as a barrier: a destroy unregisters the object
// under it (no later trace can find it), a rebuild's replaced blocks are
// already unreachable; once the lock has been held, every trace that read the
// old pointers has enqueued its kernel, whichever thread launched it.  The
// device synchronisation that waits for those kernels and the frees then run
// outside the lock, so traces on other objects are not held up while the
// device drains (a serving loop evicting scenes keeps dispatching).  The
// exclusive lock is never requested while a mesh or accel mutex is held (a
// build hands its replaced blocks to a Retired declared before its mutex
// guard), so a trace holding the shared lock and waiting for such a mutex
// cannot deadlock with it.  Order: g_life_mtx, registry, object mutexes.
std::shared_mutex g_life_mtx;

struct Retired {
    std::vector<std::shared_ptr<DevBlock>> blocks;
    std::vector<std::shared_ptr<void>> others;  // motion instances an accel let go of
    ~Retired() {
        if (blocks.empty() && others.empty()) return;
        // a barrier, not a critical section: once the exclusive lock has been held, every
        // trace that looked up these blocks has enqueued its kernel; the frees (cudaFree,
        // which the driver completes after the work queued before it) run outside it.  No
        // explicit device synchronisation: it would stop the host from preparing the next
        // build while this one runs (batched builds 93.7 -> 141.5 ms with it)
        { std::unique_lock<std::shared_mutex> lk(g_life_mtx); }
        blocks.clear();
        others.clear();
    }
};

struct MeshObj {
    LcxAccelOption opt{};
    int device = 0;
    BlasDesc *d_desc = nullptr;
    std::shared_ptr<DevBlock> block;  // nodes + triangles (possibly shared by a batch)
    double *wide_sah = nullptr;       // in `block`: 2 doubles of this mesh's segment
    size_t mem_bytes = 0;             // this mesh's share of the block
    uint32_t node_count = 0, tri_count = 0, depth = 0;
    uint32_t ref_count = 0;  // leaf items: tri_count, or more with triangle splitting
    uint32_t kind = kSegTriangles;  // or kSegAabbs: a procedural primitive (lcx_procedural_*),
                                    // kSegCurves: a curve (lcx_curve_*; items are its cones)
    std::shared_ptr<DevBlock> curve_keys;  // keyframed curves: the cones' balls per keyframe
    LcxMotionOption motion{};       // keyframe_count >= 2: vertex motion (lcx_mesh_create_motion)
    MeshMotion *d_motion = nullptr;  // after the BlasDesc in d_desc's allocation
    uint32_t seg = 0;  // segment (position in its build) within `block`
    uint64_t refits = 0;  // refits since the last full build
    bool built = false;
    uint64_t generation = 0;
    double sah = 0.0;
    std::mutex mtx;
};

// A motion instance (MotionInstance, include/luisa/runtime/rtx/motion_instance.h):
// a child mesh moved by matrix keyframes; device memory holds the keyframes
// and the MotionDesc that TLAS records point to.  Accels that instance it hold
// a reference, so the memory outlives them; `alive` and `generation` make
// their traces fail once it is destroyed or its keyframes are rebuilt.
struct MotionObj {
    uint64_t child = 0;  // mesh handle
    LcxMotionOption opt{};
    std::vector<float> keys;  // keyframe_count x 12 (row-major 3x4 object-to-world)
    void *mem = nullptr;      // MotionDesc (32 B) + keys
    MotionDesc *d_md = nullptr;
    bool built = false;
    std::atomic<bool> alive{true};
    uint64_t generation = 0;
    std::mutex mtx;
    ~MotionObj() {
        if (mem) cudaFree(mem);
    }
};

struct AccelObj {
    LcxAccelOption opt{};
    int device = 0;
    InstState *d_inst = nullptr;
    uint32_t inst_cap = 0, inst_count = 0;
    std::vector<uint64_t> inst_mesh;  // mesh handle per instance (0 = none)
    std::vector<std::shared_ptr<MotionObj>> inst_motion;  // motion instance per instance (null = static)
    std::vector<std::pair<std::shared_ptr<MotionObj>, uint64_t>> motion_gens;  // at the TLAS build
    bool has_motion = false;
    bool has_curves = false;  // an instanced BLAS is a curve: traced by the extended kernels
    std::vector<uint64_t> uniq_mesh;  // the distinct nonzero handles of inst_mesh
    bool uniq_dirty = true;           // inst_mesh changed since uniq_mesh was made
    std::shared_ptr<DevBlock> block;
    double *wide_sah = nullptr;
    Node8Q *qn = nullptr;
    Node8F *fn = nullptr;
    InstRec *recs = nullptr;
    uint32_t node_count = 0, depth = 0, max_blas_depth = 0, built_instances = 0;
    bool built = false;
    bool pending_rebuild = false;  // an instance's primitive changed since the last full build
    uint64_t refits = 0;           // TLAS refits since the last full build
    double sah = 0.0;
    std::vector<std::pair<uint64_t, uint64_t>> mesh_gens;  // (mesh handle, generation) at TLAS build
    uint64_t checked_epoch = 0;  // g_mesh_epoch when mesh_gens was last found current
    std::mutex mtx;
};

std::mutex g_reg_mtx;
std::unordered_map<uint64_t, std::shared_ptr<MeshObj>> g_meshes;
std::unordered_map<uint64_t, std::shared_ptr<AccelObj>> g_accels;
std::atomic<uint64_t> g_next_handle{1};

std::shared_ptr<MeshObj> find_mesh(uint64_t h) {
    std::lock_guard<std::mutex> lk(g_reg_mtx);
    auto it = g_meshes.find(h);
    return it == g_meshes.end() ? nullptr : it->second;
}
std::shared_ptr<AccelObj> find_accel(uint64_t h) {
    std::lock_guard<std::mutex> lk(g_reg_mtx);
    auto it = g_accels.find(h);
    return it == g_accels.end() ? nullptr : it->second;
}
std::unordered_map<uint64_t, std::shared_ptr<MotionObj>> g_motions;
std::shared_ptr<MotionObj> find_motion(uint64_t h) {
    std::lock_guard<std::mutex> lk(g_reg_mtx);
    auto it = g_motions.find(h);
    return it == g_motions.end() ? nullptr : it->second;
}

// Bumped (after the change) by every mesh build, refit and destroy, so a trace
// over an accel whose meshes did not change skips the per-mesh lookups.
std::atomic<uint64_t> g_mesh_epoch{1};
void bump_mesh_epoch() { g_mesh_epoch.fetch_add(1, std::memory_order_acq_rel); }

// Whether every mesh the accel's TLAS references still exists with the
// generation it was built against; else the first stale handle and whether it
// was destroyed.  The caller holds a->mtx.
bool meshes_current(AccelObj *a, uint64_t *stale = nullptr, bool *destroyed = nullptr) {
    const uint64_t epoch = g_mesh_epoch.load(std::memory_order_acquire);
    if (a->checked_epoch == epoch) return true;
    for (const auto &mg : a->mesh_gens) {
        auto m = find_mesh(mg.first);
        if (!m || m->generation != mg.second) {
            if (stale) *stale = mg.first;
            if (destroyed) *destroyed = !m;
            return false;
        }
    }
    for (const auto &mg : a->motion_gens)
        if (!mg.first->alive.load() || mg.first->generation != mg.second) {
            if (stale) *stale = 0;
            if (destroyed) *destroyed = !mg.first->alive.load();
            return false;
        }
    a->checked_epoch = epoch;
    return true;
}

// cudaMalloc for a BVH block; when the device is out of memory, the scratch pool's unused memory
// (which it keeps for the next build) goes back to the driver and the allocation runs once more.
cudaError_t block_malloc(void **p, size_t bytes) {
    cudaError_t e = cudaMalloc(p, bytes);
    if (e != cudaErrorMemoryAllocation) return e;
    cudaGetLastError();
    cudaMemPool_t pool;
    if (scratch_pool(&pool) != LCX_OK) return e;
    if (cudaDeviceSynchronize() != cudaSuccess || cudaMemPoolTrimTo(pool, 0) != cudaSuccess) return e;
    return cudaMalloc(p, bytes);
}

// Build scratch from the stream-ordered allocator, freed on the same stream.  Outside a graph
// capture it comes from the library's scratch pool (reorder.cu), which keeps freed memory for the
// next build (lcx_release_scratch hands it back): the device's default pool returns it to the
// driver at each synchronisation, so every build mapped its scratch again -- 23 ms of the 150 ms
// a 4096-mesh, 135M-triangle batch took on the host, against 88 ms from the scratch pool.
struct ScratchHolder {
    cudaStream_t st;
    std::vector<void *> ptrs;
    cudaMemPool_t pool = nullptr;  // null: the default pool (under capture)
    explicit ScratchHolder(cudaStream_t s) : st(s) {
        cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
        if (cudaStreamIsCapturing(st, &cs) != cudaSuccess) {
            cudaGetLastError();
            return;
        }
        if (cs == cudaStreamCaptureStatusNone && scratch_pool(&pool) != LCX_OK) pool = nullptr;
    }
    cudaError_t alloc(void **p, size_t bytes) {
        cudaError_t e = pool != nullptr ? cudaMallocFromPoolAsync(p, bytes ? bytes : 16, pool, st)
                                        : cudaMallocAsync(p, bytes ? bytes : 16, st);
        if (e == cudaSuccess) ptrs.push_back(*p);
        return e;
    }
    ~ScratchHolder() {
        for (void *p : ptrs) cudaFreeAsync(p, st);
    }
};

// Allocates the scratch of a build over n items in the given segments and
// uploads the segment table and initial control words.
int alloc_scratch(ScratchHolder &h, BuildScratch &s, const std::vector<SegInput> &segs, uint32_t n, bool tlas,
                  const SegInput *d_segs_src = nullptr, const uint32_t *d_segctl_src = nullptr, bool dp = false) {
    const size_t nn = std::max<uint32_t>(n, 1);
    s.n = n;
    s.nseg = uint32_t(segs.size());
    s.axis_bits = morton_axis_bits(s.nseg, &s.seg_bits);
    s.queue_len = n + s.nseg + 1;
    SegInput *d_segs = nullptr;
    LCX_CUDA(h.alloc((void **)&d_segs, sizeof(SegInput) * s.nseg), "scratch");
    s.segs = d_segs;
    LCX_CUDA(h.alloc((void **)&s.segctl, sizeof(uint32_t) * kSegWords * s.nseg), "scratch");
    LCX_CUDA(h.alloc((void **)&s.bin_sah, sizeof(double) * 2 * s.nseg), "scratch");
    LCX_CUDA(h.alloc((void **)&s.box_lo, sizeof(float4) * nn), "scratch");
    LCX_CUDA(h.alloc((void **)&s.box_hi, sizeof(float4) * nn), "scratch");
    LCX_CUDA(h.alloc((void **)&s.keys, sizeof(unsigned long long) * nn), "scratch");
    LCX_CUDA(h.alloc((void **)&s.keys_sorted, sizeof(unsigned long long) * nn), "scratch");
    LCX_CUDA(h.alloc((void **)&s.vals, sizeof(uint32_t) * nn), "scratch");
    LCX_CUDA(h.alloc((void **)&s.vals_sorted, sizeof(uint32_t) * nn), "scratch");
    LCX_CUDA(h.alloc((void **)&s.bin_child, sizeof(uint32_t) * 2 * nn), "scratch");
    LCX_CUDA(h.alloc((void **)&s.bin_lo, sizeof(float4) * nn), "scratch");
    LCX_CUDA(h.alloc((void **)&s.bin_hi, sizeof(float4) * nn), "scratch");
    LCX_CUDA(h.alloc((void **)&s.other, sizeof(int32_t) * nn), "scratch");
    LCX_CUDA(h.alloc((void **)&s.desc, sizeof(uint32_t) * 12 * s.queue_len), "scratch");
    LCX_CUDA(h.alloc((void **)&s.queue, sizeof(uint2) * 2 * s.queue_len), "scratch");
    if (tlas) LCX_CUDA(h.alloc((void **)&s.w2o, sizeof(float) * 12 * nn), "scratch");
    if (dp) LCX_CUDA(h.alloc((void **)&s.dp_cost, sizeof(float) * 8 * nn), "scratch");
    LCX_CUDA(h.alloc((void **)&s.ctl, sizeof(uint32_t) * kCtlWords), "scratch");
    s.sort_tmp_bytes = std::max(sort_temp_bytes(uint32_t(nn)), sah_scan_temp_bytes(uint32_t(nn)));
    LCX_CUDA(h.alloc(&s.sort_tmp, s.sort_tmp_bytes), "scratch");
    // uploads: segment table, control words (centroid minima start at the largest ordered value);
    // a reserved rebuild copies both from the device (no host data: capturable)
    if (d_segs_src != nullptr) {
        LCX_CUDA(cudaMemcpyAsync(d_segs, d_segs_src, sizeof(SegInput) * s.nseg, cudaMemcpyDeviceToDevice, h.st),
                 "segment copy");
        LCX_CUDA(cudaMemcpyAsync(s.segctl, d_segctl_src, sizeof(uint32_t) * kSegWords * s.nseg,
                                 cudaMemcpyDeviceToDevice, h.st),
                 "segment copy");
    } else {
        std::vector<uint32_t> segctl(size_t(kSegWords) * s.nseg, 0u);
        for (uint32_t i = 0; i < s.nseg; i++)
            for (int k = 0; k < 3; k++) segctl[size_t(kSegWords) * i + kSegCenLo + k] = 0xffffffffu;
        LCX_CUDA(cudaMemcpyAsync(d_segs, segs.data(), sizeof(SegInput) * s.nseg, cudaMemcpyHostToDevice, h.st),
                 "segment upload");
        LCX_CUDA(cudaMemcpyAsync(s.segctl, segctl.data(), sizeof(uint32_t) * segctl.size(), cudaMemcpyHostToDevice,
                                 h.st),
                 "segment upload");
    }
    LCX_CUDA(cudaMemsetAsync(s.bin_sah, 0, sizeof(double) * 2 * s.nseg, h.st), "scratch init");
    LCX_CUDA(cudaMemsetAsync(s.ctl, 0, sizeof(uint32_t) * kCtlWords, h.st), "scratch init");
    // (copies from pageable memory return once the source has been staged)
    return LCX_OK;
}

struct BuildReadback {
    std::vector<uint32_t> ctl, segctl;
    std::vector<double> bin_sah;
};

int read_back(const BuildScratch &s, cudaStream_t st, BuildReadback &out) {
    out.ctl.resize(kCtlWords);
    out.segctl.resize(size_t(kSegWords) * s.nseg);
    out.bin_sah.resize(2 * size_t(s.nseg));
    LCX_CUDA(cudaMemcpyAsync(out.ctl.data(), s.ctl, sizeof(uint32_t) * kCtlWords, cudaMemcpyDeviceToHost, st),
             "readback");
    LCX_CUDA(cudaMemcpyAsync(out.segctl.data(), s.segctl, sizeof(uint32_t) * out.segctl.size(), cudaMemcpyDeviceToHost,
                             st),
             "readback");
    LCX_CUDA(cudaMemcpyAsync(out.bin_sah.data(), s.bin_sah, sizeof(double) * out.bin_sah.size(),
                             cudaMemcpyDeviceToHost, st),
             "readback");
    LCX_CUDA(cudaStreamSynchronize(st), "build sync");
    return LCX_OK;
}

int check_option(const LcxAccelOption *o) {
    if (o && o->hint > LCX_HINT_FAST_BUILD) return fail(LCX_ERR_INVALID_ARG, "invalid AccelOption.hint %u", o->hint);
    return LCX_OK;
}

// Triangles per leaf slot by hint.  Measured on GB300 (terrain workload, 8.4M
// incoherent rays, quantised nodes): 1 -> 1.66, 2 -> 1.58, 3 -> 1.49 Grays/s,
// with 741k / 343k / 306k wide nodes; FAST_BUILD takes the smallest tree.
// Items per leaf slot by hint.  FAST_TRACE 2: with the deferred triangle batches
// (traversal mode 2) two per leaf traced fastest on the terrain workload
// (closest 1.895 / 1.955 / 1.933 Grays/s at 1 / 2 / 3; any hit 3.26 / 3.37 / 3.36).
int leaf_items_for(const LcxAccelOption &o) { return o.hint == LCX_HINT_FAST_BUILD ? 3 : 2; }

#ifndef LCX_DP_PRIM
// the collapse's dynamic program: an item test against a node test of 1 (terrain workload, closest hit:
// 2.660 / 2.659 / 2.666 / 2.664 Grays/s at 0.2 / 0.3 / 0.5 / 0.8)
#define LCX_DP_PRIM 0.5f
#endif

// Build knobs (see lcx_set_build_tuning); 0 = derive from the AccelOption hint.
struct BuildTuning {
    int leaf_max = 0;
    int width = 8;
    // Measured on the terrain workload (8.4M rays): cube-normalised BLAS codes
    // cut node visits per ray 17.7 -> 16.5; cube or size-class TLAS codes raised
    // the TLAS SAH 22.9 -> 30.7+ and slowed traversal, so both stay off.
    uint32_t blas_cube = 1, tlas_cube = 0, tlas_size_bits = 0;
    // triangle splitting of FAST_TRACE meshes without allow_update (lcx_set_build_split):
    // extra references as a fraction of the triangles.  Off by default: on the terrain
    // workload it makes no splits at 0.3 (axis-aligned right triangles weigh 0) and costs
    // traversal at 1 and 3 (1.525 -> 1.467 / 1.364 Grays/s); on a displaced 1M-triangle mesh
    // it takes 0.61 -> 0.68 / 1.00 Grays/s (nodes per ray 27.7 -> 13.0 at 3).  The
    // autotuner and callers with such meshes turn it on.
    float split = 0.0f;
    // leaf-slot filling (lcx_set_build_fill), on: on the terrain workload triangle tests per ray fall
    // 3.00 -> 2.64 with the same 343k wide nodes (closest 2.020 -> 2.030 Grays/s in loop mode 2,
    // 1.660 -> 1.716 in mode 0)
    uint32_t fill = 1;
    // binned-SAH TLAS (lcx_set_build_tlas_sah), on: on the terrain workload (a heightfield and 256
    // small spheres) TLAS SAH 20.0 -> 15.2, node visits per ray 15.19 -> 13.99, closest 2.358 ->
    // 2.492 Grays/s, any hit 3.89 -> 4.12
    uint32_t tlas_sah = 1;
    // binned-SAH BLAS of FAST_TRACE meshes (lcx_set_build_blas_sah), on
    uint32_t blas_sah = 1;
    // collapse by dynamic program (lcx_set_build_collapse), on for FAST_TRACE BLASes and TLASes: on the
    // terrain workload terrain wide nodes 306,743 -> 211,762, node visits per ray 13.35 -> 12.96 (triangle
    // tests 2.42 -> 2.68), closest 2.613 -> 2.666 Grays/s, any hit 4.29 -> 4.37; the terrain BLAS build
    // 6.0 -> 6.7 ms
    uint32_t dp = 1;
};
BuildTuning g_build_tune;

BuildParams build_params_for(const LcxAccelOption &o) {
    BuildParams bp;
    bp.leaf_max = g_build_tune.leaf_max > 0 ? g_build_tune.leaf_max : leaf_items_for(o);
    bp.width = g_build_tune.width;
    bp.cube = g_build_tune.blas_cube;
    bp.split = (o.hint == LCX_HINT_FAST_TRACE && !o.allow_update) ? g_build_tune.split : 0.0f;
    bp.fill = g_build_tune.fill;
    bp.blas_sah = o.hint == LCX_HINT_FAST_TRACE ? g_build_tune.blas_sah : 0u;
    bp.dp = o.hint == LCX_HINT_FAST_TRACE ? g_build_tune.dp : 0u;
    bp.dp_prim = LCX_DP_PRIM;
    return bp;
}

int validate_mesh_command(const LcxMeshBuildCommand *cmd, uint64_t &tri64, uint64_t &vcount64) {
    if (!cmd) return fail(LCX_ERR_INVALID_ARG, "mesh build command is null");
    // src/runtime/rtx/mesh.cpp:41-50 and :33-39
    if (cmd->request > LCX_REQUEST_FORCE_BUILD) return fail(LCX_ERR_INVALID_ARG, "invalid build request %u", cmd->request);
    if (cmd->vertex_stride == 0 || cmd->vertex_stride % 16 != 0)
        return fail(LCX_ERR_INVALID_ARG, "Vertex stride must be aligned to 16 bytes (got %zu).", cmd->vertex_stride);
    if (cmd->vertex_buffer_offset % cmd->vertex_stride != 0 || cmd->vertex_buffer_size % cmd->vertex_stride != 0)
        return fail(LCX_ERR_INVALID_ARG, "vertex buffer offset %zu / size %zu not aligned to vertex stride %zu",
                    cmd->vertex_buffer_offset, cmd->vertex_buffer_size, cmd->vertex_stride);
    if (cmd->triangle_buffer_offset % 4 != 0 || cmd->triangle_buffer_size % 12 != 0)
        return fail(LCX_ERR_INVALID_ARG, "triangle buffer offset %zu / size %zu not aligned (4 / 12 bytes)",
                    cmd->triangle_buffer_offset, cmd->triangle_buffer_size);
    tri64 = cmd->triangle_buffer_size / 12;
    vcount64 = cmd->vertex_buffer_size / cmd->vertex_stride;
    if (tri64 >= (1ull << 31) || vcount64 >= (1ull << 32))
        return fail(LCX_ERR_INVALID_ARG, "mesh too large (%llu triangles, %llu vertices)", (unsigned long long)tri64,
                    (unsigned long long)vcount64);
    if (tri64 && (cmd->vertex_buffer == 0 || cmd->triangle_buffer == 0))
        return fail(LCX_ERR_INVALID_ARG, "null vertex or triangle buffer");
    if ((cmd->vertex_buffer + cmd->vertex_buffer_offset) % 16 != 0 || (cmd->triangle_buffer % 4) != 0)
        return fail(LCX_ERR_INVALID_ARG, "vertex buffer must be 16-byte aligned, triangle buffer 4-byte aligned");
    return LCX_OK;
}

// Builds the BLASes of `meshes` (locked by the caller) from `cmds` in one
// segmented pipeline: one sort, one LBVH pass, one cooperative collapse and
// one emit for all of them, into one shared device block.  Synchronises the
// host once to size the block.
// Whether `st` is being captured into a CUDA graph: host-to-device copies from
// pageable memory cannot be captured, so the calls that would make one fail.
bool capturing(cudaStream_t st) {
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(st, &cs) != cudaSuccess) {
        (void)cudaGetLastError();
        return false;
    }
    return cs == cudaStreamCaptureStatusActive;
}

constexpr int kNoRefit = 1;  // try_refit: the call is not a refit; build instead
bool g_refit_sync = true;    // lcx_set_refit_sync

// PREFER_UPDATE on meshes created with allow_update: when the call covers every
// mesh of one BVH block (as built together) and no triangle count changed,
// the block is refit in place (same topology, new triangle records and boxes)
// instead of rebuilt.  One host synchronisation, to report bad indices.
// `segs`: the call's validated segments in call order.  Otherwise kNoRefit.
int try_refit(const std::vector<MeshObj *> &meshes, const std::vector<uint32_t> &requests,
              const std::vector<SegInput> &segs, cudaStream_t st) {
    const size_t count = meshes.size();
    DevBlock *blk = meshes[0]->block.get();
    if (!blk || !blk->rtab || blk->nseg != count) return kNoRefit;
    std::vector<SegInput> ordered(count);
    std::vector<bool> seen(count, false);
    for (size_t i = 0; i < count; i++) {
        const MeshObj *m = meshes[i];
        if (requests[i] != LCX_REQUEST_PREFER_UPDATE || !m->opt.allow_update || !m->built ||
            m->block.get() != blk || m->seg >= count || seen[m->seg] || segs[i].item_count != m->tri_count ||
            segs[i].item_count == 0)
            return kNoRefit;
        seen[m->seg] = true;
        ordered[m->seg] = segs[i];
    }
    uint32_t off = 0;
    for (size_t k = 0; k < count; k++) {  // the build's item offsets: prefix sums in segment order
        ordered[k].item_offset = off;
        off += ordered[k].item_count;
    }
    // the segment table stays on the device: buffers that did not move need no upload,
    // so such a refit only enqueues a memset and three kernels (capturable in a CUDA graph)
    if (blk->h_segs.size() != count || std::memcmp(blk->h_segs.data(), ordered.data(), sizeof(SegInput) * count)) {
        if (capturing(st))
            return fail(LCX_ERR_INVALID_ARG,
                        "refit in a CUDA graph capture: the mesh buffers moved since the last refit; refit once "
                        "outside the capture first");
        LCX_CUDA(cudaMemcpyAsync(blk->d_segs, ordered.data(), sizeof(SegInput) * count, cudaMemcpyHostToDevice, st),
                 "refit segment upload");
        blk->h_segs = ordered;
    }
    DeviceState *ds = nullptr;
    if (int r = current_device_state(&ds)) return r;
    if (!g_refit_sync) {  // errors go to the device's refit error word (lcx_check_trace_errors)
        LCX_CUDA(refit_blas(blk->d_segs, uint32_t(count), blk->wide, blk->rtab, blk->qn, blk->fn, blk->tris,
                            blk->counters, ds->refit_ctl, st),
                 "BLAS refit");
    } else {
        if (capturing(st))
            return fail(LCX_ERR_INVALID_ARG, "refit in a CUDA graph capture needs lcx_set_refit_sync(0)");
        ScratchHolder hold(st);
        uint32_t *ctl = nullptr;
        LCX_CUDA(hold.alloc((void **)&ctl, sizeof(uint32_t) * kCtlWords), "refit scratch");
        LCX_CUDA(cudaMemsetAsync(ctl, 0, sizeof(uint32_t) * kCtlWords, st), "refit scratch init");
        LCX_CUDA(refit_blas(blk->d_segs, uint32_t(count), blk->wide, blk->rtab, blk->qn, blk->fn, blk->tris,
                            blk->counters, ctl, st),
                 "BLAS refit");
        uint32_t err = 0;
        LCX_CUDA(cudaMemcpyAsync(&err, ctl + kCtlErr, sizeof(uint32_t), cudaMemcpyDeviceToHost, st), "refit readback");
        LCX_CUDA(cudaStreamSynchronize(st), "refit sync");
        if (err & kErrBadIndex) return fail(LCX_ERR_INVALID_ARG, "refit: triangle index out of range");
        if (err & kErrTooDeep) return fail(LCX_ERR_DEPTH, "refit: BVH deeper than %d levels", kMaxLevels);
        if (err & kErrQuant) return fail(LCX_ERR_INVALID_ARG, "refit: vertex coordinates too large to quantise");
    }
    for (MeshObj *m : meshes) {
        m->generation++;  // accels over these meshes must be built again
        m->refits++;
    }
    bump_mesh_epoch();
    return LCX_OK;
}

// Segments of mesh build commands (validated), item offsets in call order.
int mesh_segments(const std::vector<MeshObj *> &meshes, const LcxMeshBuildCommand *cmds, std::vector<SegInput> &segs,
                  std::vector<uint32_t> &requests) {
    const size_t count = meshes.size();
    segs.assign(count, SegInput{});
    requests.assign(count, 0u);
    uint64_t total = 0;
    for (size_t i = 0; i < count; i++) {
        if (meshes[i]->kind != kSegTriangles)
            return fail(LCX_ERR_INVALID_ARG, "entry %zu: a procedural primitive takes lcx_procedural_build", i);
        uint64_t tri64 = 0, v64 = 0;
        if (int r = validate_mesh_command(&cmds[i], tri64, v64)) return r;
        const uint32_t keys = meshes[i]->motion.keyframe_count;
        if (keys >= 2) {  // mesh.cpp check_mesh_vert_buffer_motion_keyframe_count: whole keyframes
            if (v64 % keys != 0)
                return fail(LCX_ERR_INVALID_ARG, "entry %zu: %llu vertices are not %u whole keyframes", i,
                            (unsigned long long)v64, keys);
            v64 /= keys;
        }
        SegInput &g = segs[i];
        g.vbase = reinterpret_cast<const unsigned char *>(cmds[i].vertex_buffer) + cmds[i].vertex_buffer_offset;
        g.vstride = cmds[i].vertex_stride;
        g.tbase = reinterpret_cast<const unsigned char *>(cmds[i].triangle_buffer) + cmds[i].triangle_buffer_offset;
        g.vcount = uint32_t(v64);
        g.item_offset = uint32_t(total);
        g.item_count = uint32_t(tri64);
        g.kind = kSegTriangles | (keys >= 2 ? keys << 8 : 0u);
        g.desc = meshes[i]->d_desc;
        requests[i] = cmds[i].request;
        total += tri64;
        if (total >= (1ull << 31)) return fail(LCX_ERR_INVALID_ARG, "batch too large (%llu triangles)",
                                               (unsigned long long)total);
    }
    return LCX_OK;
}

// Builds (or refits) the BVHs of `meshes` from their segments in one pass.
// A reserved batch rebuilt in place (the same meshes in the same order over the
// same buffers): the build's kernels only, no host synchronisation and no
// allocation outside the stream-ordered scratch, so it can be captured in a
// CUDA graph.  Errors go to the device's asynchronous error word; the meshes'
// statistics (node count, depth) keep the reserving build's values.
// Otherwise kNoRefit.
int try_reserved_rebuild(const std::vector<MeshObj *> &meshes, const std::vector<SegInput> &segs, cudaStream_t st) {
    const size_t count = meshes.size();
    DevBlock *blk = meshes[0]->block.get();
    if (!blk || !blk->reserved || blk->nseg != count || blk->h_segs.size() != count) return kNoRefit;
    for (size_t i = 0; i < count; i++)
        if (meshes[i]->block.get() != blk || meshes[i]->seg != i) return kNoRefit;
    if (std::memcmp(blk->h_segs.data(), segs.data(), sizeof(SegInput) * count) != 0) return kNoRefit;
    DeviceState *ds = nullptr;
    if (int r = current_device_state(&ds)) return r;
    BuildParams bp = build_params_for(meshes[0]->opt);
    bp.split = 0.0f;
    bp.blas_sah = 0u;  // capturable: no host synchronisation
    bp.dp = 0u;        // as the reserving build
    ScratchHolder hold(st);
    BuildScratch s;
    if (int r = alloc_scratch(hold, s, blk->h_segs, blk->items, false, blk->d_segs, blk->d_segctl_init)) return r;
    {
        NvtxRange nr("reserved rebuild: boxes, tree, collapse");
        LCX_CUDA(build_tree_tris(s, bp, st), "BLAS rebuild");
    }
    LCX_CUDA(cudaMemsetAsync(blk->wsah, 0, 2 * sizeof(double) * count, st), "cudaMemset");
    LCX_CUDA(emit_blas(s, bp, blk->cap_wide, blk->qn, blk->fn, blk->tris, blk->wsah, nullptr, st, true),
             "BLAS rebuild emit");
    LCX_CUDA(report_build_errors(s.ctl, ds->refit_ctl, st), "BLAS rebuild errors");
    for (MeshObj *m : meshes) m->generation++;  // accels over these meshes must be built (or refit) again
    bump_mesh_epoch();
    return LCX_OK;
}

// Reserves a batch without building it: the block a reserved batch has (room for any tree over the
// items, the segment table and the initial control words on the device) and nothing else, so the
// batch's first build -- the next lcx_mesh_build_batch of the same meshes over the same buffers,
// which takes the reserved-rebuild path -- needs no host synchronisation and can be captured in a
// CUDA graph.  The meshes count as built (their descriptors are zero, i.e. empty, until that build
// runs); their statistics stay zero until a synchronising build.
int reserve_only(const std::vector<MeshObj *> &meshes, const std::vector<SegInput> &segs, cudaStream_t st,
                 Retired &retired) {
    const size_t count = meshes.size();
    uint64_t total = 0;
    for (const SegInput &g : segs) total += g.item_count;
    if (total == 0) return fail(LCX_ERR_INVALID_ARG, "a reserved batch needs triangles");
    if (total + count >= (1ull << 31)) return fail(LCX_ERR_INVALID_ARG, "too many triangles in one batch");
    const uint32_t n_items = uint32_t(total);
    // every wide node opens a binary node or is a segment root: at most items + segments of them
    const uint32_t W_alloc = uint32_t(uint64_t(n_items) + count);
    const size_t q_bytes = size_t(W_alloc) * sizeof(Node8Q), f_bytes = size_t(W_alloc) * sizeof(Node8F);
    const size_t t_bytes = size_t(n_items) * sizeof(TriRec), sah_bytes = 2 * sizeof(double) * count;
    const size_t res_bytes = sizeof(SegInput) * count + sizeof(uint32_t) * kSegWords * count;
    auto block = std::make_shared<DevBlock>();
    block->bytes = q_bytes + f_bytes + t_bytes + sah_bytes + res_bytes;
    LCX_CUDA(block_malloc(&block->ptr, block->bytes), "cudaMalloc(reserved BLAS block)");
    char *base = static_cast<char *>(block->ptr);
    block->qn = reinterpret_cast<Node8Q *>(base);
    block->fn = reinterpret_cast<Node8F *>(base + q_bytes);
    block->tris = reinterpret_cast<TriRec *>(base + q_bytes + f_bytes);
    block->wsah = reinterpret_cast<double *>(base + q_bytes + f_bytes + t_bytes);
    char *rp = base + q_bytes + f_bytes + t_bytes + sah_bytes;
    block->d_segs = reinterpret_cast<SegInput *>(rp);
    block->d_segctl_init = reinterpret_cast<uint32_t *>(rp + sizeof(SegInput) * count);
    block->h_segs = segs;
    block->reserved = true;
    block->items = n_items;
    block->cap_wide = W_alloc;
    block->wide = 0;
    block->nseg = uint32_t(count);
    std::vector<uint32_t> init(size_t(kSegWords) * count, 0u);
    for (size_t i = 0; i < count; i++)
        for (int k = 0; k < 3; k++) init[size_t(kSegWords) * i + kSegCenLo + k] = 0xffffffffu;
    LCX_CUDA(cudaMemcpyAsync(block->d_segs, segs.data(), sizeof(SegInput) * count, cudaMemcpyHostToDevice, st),
             "reserve segment table");
    LCX_CUDA(cudaMemcpyAsync(block->d_segctl_init, init.data(), sizeof(uint32_t) * init.size(), cudaMemcpyHostToDevice,
                             st),
             "reserve control words");
    LCX_CUDA(cudaMemsetAsync(block->wsah, 0, sah_bytes, st), "cudaMemset");
    // the host vectors above are read by the copies: wait for them (one sync at reservation, none later)
    LCX_CUDA(cudaStreamSynchronize(st), "reserve sync");
    for (size_t i = 0; i < count; i++) {
        MeshObj *m = meshes[i];
        LCX_CUDA(cudaMemset(m->d_desc, 0, sizeof(BlasDesc)), "cudaMemset(BlasDesc)");
        if (m->block) retired.blocks.push_back(std::move(m->block));
        m->block = block;
        m->seg = uint32_t(i);
        m->wide_sah = block->wsah + 2 * i;
        m->refits = 0;
        m->node_count = 0;
        m->depth = 0;  // unknown until a synchronising build; the traversal flags a stack overflow
        m->tri_count = m->ref_count = segs[i].item_count;
        m->mem_bytes = size_t(m->tri_count) * sizeof(TriRec);
        m->sah = 0.0;
        m->built = true;
        m->generation++;
    }
    bump_mesh_epoch();
    return LCX_OK;
}

int build_meshes(const std::vector<MeshObj *> &meshes, const std::vector<SegInput> &segs,
                 const std::vector<uint32_t> &requests, cudaStream_t st, Retired &retired, bool reserve = false) {
    const size_t count = meshes.size();
    uint64_t total = 0;
    for (const SegInput &g : segs) total += g.item_count;
    if (!reserve) {
        int r = try_refit(meshes, requests, segs, st);
        if (r != kNoRefit) return r;
        r = try_reserved_rebuild(meshes, segs, st);
        if (r != kNoRefit) return r;
    }
    if (capturing(st))  // a build sizes its block on the host
        return fail(LCX_ERR_INVALID_ARG,
                    "mesh build in a CUDA graph capture: only refits (PREFER_UPDATE, allow_update, every mesh of the "
                    "block, same triangle counts, asynchronous refit mode) and rebuilds of a reserved batch "
                    "(lcx_mesh_build_batch_reserve, same meshes and buffers) can be captured");
    BuildParams bp = build_params_for(meshes[0]->opt);
    if (reserve) bp.blas_sah = bp.dp = 0u;  // its rebuilds are capturable LBVH builds: keep the first one alike
    if (total == 0) {
        LCX_CUDA(cudaStreamSynchronize(st), "sync");
        for (MeshObj *m : meshes) {
            LCX_CUDA(cudaMemset(m->d_desc, 0, sizeof(BlasDesc)), "cudaMemset(BlasDesc)");
            if (m->block) retired.blocks.push_back(std::move(m->block));
            m->block.reset();
            m->wide_sah = nullptr;
            m->mem_bytes = 0;
            m->node_count = m->tri_count = m->ref_count = m->depth = 0;
            m->sah = 0.0;
            m->built = true;
            m->generation++;
        }
        bump_mesh_epoch();
        return LCX_OK;
    }
    const uint32_t n = uint32_t(total);
    BuildReadback rb;
    std::shared_ptr<DevBlock> block;
    bool want_rtab = false;
    for (MeshObj *m : meshes) want_rtab = want_rtab || m->opt.allow_update;
    {
        ScratchHolder hold(st);
        BuildScratch s;
        // triangle splitting: FAST_TRACE triangle meshes, none of them kept for refits
        bool split = bp.split > 0.0f && !want_rtab && !reserve;
        for (const SegInput &g : segs) split = split && g.kind == kSegTriangles;
        std::vector<SegInput> rsegs;  // the segments in reference space
        uint32_t n_items = n;
        SegInput *d_tsegs = nullptr;
        uint32_t *d_refs = nullptr, *d_ref_off = nullptr;
        if (split) {
            const uint32_t nseg = uint32_t(count);
            float *wts = nullptr;
            unsigned long long *wsum = nullptr;  // per segment: weight sums, then the largest weights
            uint32_t *seg_refs = nullptr, *ctl1 = nullptr, *segctl1 = nullptr;
            LCX_CUDA(hold.alloc((void **)&d_tsegs, sizeof(SegInput) * nseg), "split scratch");
            LCX_CUDA(hold.alloc((void **)&wts, sizeof(float) * n), "split scratch");
            LCX_CUDA(hold.alloc((void **)&wsum, (sizeof(unsigned long long) + sizeof(uint32_t)) * nseg),
                     "split scratch");
            LCX_CUDA(hold.alloc((void **)&d_refs, sizeof(uint32_t) * n), "split scratch");
            LCX_CUDA(hold.alloc((void **)&d_ref_off, sizeof(uint32_t) * n), "split scratch");
            LCX_CUDA(hold.alloc((void **)&seg_refs, sizeof(uint32_t) * nseg), "split scratch");
            LCX_CUDA(hold.alloc((void **)&segctl1, sizeof(uint32_t) * kSegWords * nseg), "split scratch");
            LCX_CUDA(hold.alloc((void **)&ctl1, sizeof(uint32_t) * kCtlWords), "split scratch");
            LCX_CUDA(cudaMemcpyAsync(d_tsegs, segs.data(), sizeof(SegInput) * nseg, cudaMemcpyHostToDevice, st),
                     "segment upload");
            LCX_CUDA(cudaMemsetAsync(segctl1, 0, sizeof(uint32_t) * kSegWords * nseg, st), "split scratch init");
            LCX_CUDA(cudaMemsetAsync(ctl1, 0, sizeof(uint32_t) * kCtlWords, st), "split scratch init");
            LCX_CUDA(split_count(d_tsegs, nseg, n, bp.split, wts, wsum, d_refs, seg_refs, segctl1, ctl1, st),
                     "split counts");
            size_t scan_bytes = 0;
            LCX_CUDA(exclusive_sum(nullptr, &scan_bytes, d_refs, d_ref_off, n, st), "scan size");
            void *scan_tmp = nullptr;
            LCX_CUDA(hold.alloc(&scan_tmp, scan_bytes), "split scratch");
            LCX_CUDA(exclusive_sum(scan_tmp, &scan_bytes, d_refs, d_ref_off, n, st), "reference offsets");
            std::vector<uint32_t> h_refs(nseg), h_err(nseg * size_t(kSegWords)), h_ctl(kCtlWords);
            LCX_CUDA(cudaMemcpyAsync(h_refs.data(), seg_refs, sizeof(uint32_t) * nseg, cudaMemcpyDeviceToHost, st),
                     "split readback");
            LCX_CUDA(cudaMemcpyAsync(h_err.data(), segctl1, sizeof(uint32_t) * h_err.size(), cudaMemcpyDeviceToHost, st),
                     "split readback");
            LCX_CUDA(cudaMemcpyAsync(h_ctl.data(), ctl1, sizeof(uint32_t) * kCtlWords, cudaMemcpyDeviceToHost, st),
                     "split readback");
            LCX_CUDA(cudaStreamSynchronize(st), "split sync");
            if (h_ctl[kCtlErr] & kErrBadIndex) {
                for (size_t i = 0; i < count; i++)
                    if (h_err[kSegWords * i + kSegErr] & kErrBadIndex)
                        return fail(LCX_ERR_INVALID_ARG,
                                    "mesh %zu of the build: triangle index out of range (vertex count %u)", i,
                                    segs[i].vcount);
                return fail(LCX_ERR_INVALID_ARG, "triangle index out of range");
            }
            rsegs = segs;
            uint64_t off = 0;
            for (size_t i = 0; i < count; i++) {
                rsegs[i].item_offset = uint32_t(off);
                rsegs[i].item_count = h_refs[i];
                off += h_refs[i];
            }
            if (off >= (1ull << 31)) return fail(LCX_ERR_INVALID_ARG, "too many triangle references (%llu)",
                                                 (unsigned long long)off);
            n_items = uint32_t(off);
        }
        const std::vector<SegInput> &isegs = split ? rsegs : segs;  // the build's items
        if (int r = alloc_scratch(hold, s, isegs, n_items, false, nullptr, nullptr, bp.dp != 0)) return r;
        if (split) {
            uint32_t *ref_prim = nullptr;
            LCX_CUDA(hold.alloc((void **)&ref_prim, sizeof(uint32_t) * n_items), "split scratch");
            LCX_CUDA(split_emit(d_tsegs, uint32_t(count), n, d_refs, d_ref_off, s, ref_prim, st), "triangle split");
        }
        {
            NvtxRange nr("BLAS build: boxes, tree, collapse");
            LCX_CUDA(build_tree_tris(s, bp, st), "BLAS build");
        }
        if (int r = read_back(s, st, rb)) return r;
        if (rb.ctl[kCtlErr] & kErrBadIndex) {
            for (size_t i = 0; i < count; i++)
                if (rb.segctl[kSegWords * i + kSegErr] & kErrBadIndex)
                    return fail(LCX_ERR_INVALID_ARG, "mesh %zu of the build: triangle index out of range (vertex count %u)",
                                i, segs[i].vcount);
            return fail(LCX_ERR_INVALID_ARG, "triangle index out of range");
        }
        if (rb.ctl[kCtlErr] & kErrTooDeep) return fail(LCX_ERR_DEPTH, "BVH deeper than %d levels", kMaxLevels);
        for (size_t i = 0; i < count; i++)
            if (rb.segctl[kSegWords * i + kSegItems] != isegs[i].item_count)
                return fail(LCX_ERR_CUDA, "BLAS build placed %u of %u items of mesh %zu",
                            rb.segctl[kSegWords * i + kSegItems], isegs[i].item_count, i);
        const uint32_t W = rb.ctl[kCtlWideCount];
        // a reserved batch has room for any tree over its items: every wide node opens a
        // binary node or is a segment root, so there are at most items + segments of them
        const uint32_t W_alloc = reserve ? uint32_t(std::max<uint64_t>(W, uint64_t(n_items) + count)) : W;
        const size_t q_bytes = size_t(W_alloc) * sizeof(Node8Q), f_bytes = size_t(W_alloc) * sizeof(Node8F);
        const size_t t_bytes = size_t(n_items) * sizeof(TriRec), sah_bytes = 2 * sizeof(double) * count;
        const size_t res_bytes = reserve ? sizeof(SegInput) * count + sizeof(uint32_t) * kSegWords * count : 0;
        // refit data: parent table, counters, segment table (16-byte aligned)
        const size_t r_bytes =
            want_rtab ? ((size_t(W) * (sizeof(unsigned long long) + sizeof(uint32_t)) + 15) & ~size_t(15)) +
                            sizeof(SegInput) * count
                      : 0;
        block = std::make_shared<DevBlock>();
        block->bytes = q_bytes + f_bytes + t_bytes + sah_bytes + r_bytes + res_bytes;
        LCX_CUDA(block_malloc(&block->ptr, block->bytes), "cudaMalloc(BLAS)");
        Node8Q *qn = static_cast<Node8Q *>(block->ptr);
        Node8F *fn = reinterpret_cast<Node8F *>(reinterpret_cast<char *>(block->ptr) + q_bytes);
        TriRec *tr = reinterpret_cast<TriRec *>(reinterpret_cast<char *>(block->ptr) + q_bytes + f_bytes);
        double *wsah = reinterpret_cast<double *>(reinterpret_cast<char *>(block->ptr) + q_bytes + f_bytes + t_bytes);
        unsigned long long *rtab =
            want_rtab ? reinterpret_cast<unsigned long long *>(reinterpret_cast<char *>(wsah) + sah_bytes) : nullptr;
        block->rtab = rtab;
        block->wide = W;
        block->nseg = uint32_t(count);
        block->qn = qn;
        block->fn = fn;
        block->tris = tr;
        if (rtab) {
            block->counters = reinterpret_cast<uint32_t *>(rtab + W);
            block->d_segs = reinterpret_cast<SegInput *>(
                reinterpret_cast<char *>(rtab) + ((size_t(W) * (sizeof(unsigned long long) + sizeof(uint32_t)) + 15) &
                                                  ~size_t(15)));
            LCX_CUDA(cudaMemcpyAsync(block->d_segs, segs.data(), sizeof(SegInput) * count, cudaMemcpyHostToDevice, st),
                     "refit segment table");
            block->h_segs = segs;
        }
        if (reserve) {  // segment table and initial control words for the rebuilds
            char *rp = reinterpret_cast<char *>(block->ptr) + q_bytes + f_bytes + t_bytes + sah_bytes + r_bytes;
            block->reserved = true;
            block->items = n_items;
            block->cap_wide = W_alloc;
            block->wsah = wsah;
            block->d_segs = reinterpret_cast<SegInput *>(rp);
            block->d_segctl_init = reinterpret_cast<uint32_t *>(rp + sizeof(SegInput) * count);
            block->h_segs = segs;
            std::vector<uint32_t> init(size_t(kSegWords) * count, 0u);
            for (size_t i = 0; i < count; i++)
                for (int k = 0; k < 3; k++) init[size_t(kSegWords) * i + kSegCenLo + k] = 0xffffffffu;
            LCX_CUDA(cudaMemcpyAsync(block->d_segs, segs.data(), sizeof(SegInput) * count, cudaMemcpyHostToDevice, st),
                     "reserve segment table");
            LCX_CUDA(cudaMemcpyAsync(block->d_segctl_init, init.data(), sizeof(uint32_t) * init.size(),
                                     cudaMemcpyHostToDevice, st),
                     "reserve control words");
        }
        LCX_CUDA(cudaMemsetAsync(wsah, 0, sah_bytes, st), "cudaMemset");
        // vertex-motion meshes: their MeshMotion (this build's buffers) before the emit reads it
        for (size_t i = 0; i < count; i++) {
            MeshObj *m = meshes[i];
            if (m->motion.keyframe_count < 2) continue;
            MeshMotion mm{};
            mm.vbase = segs[i].vbase;
            mm.tbase = segs[i].tbase;
            mm.vstride = segs[i].vstride;
            mm.vcount = segs[i].vcount;
            mm.keys = m->motion.keyframe_count;
            mm.t0 = m->motion.time_start;
            mm.t1 = m->motion.time_end;
            mm.flags = (m->motion.vanish_start ? 1u : 0u) | (m->motion.vanish_end ? 2u : 0u);
            LCX_CUDA(cudaMemcpyAsync(m->d_motion, &mm, sizeof(mm), cudaMemcpyHostToDevice, st), "motion upload");
        }
        {
            NvtxRange nr("BLAS build: emit nodes and triangles");
            LCX_CUDA(emit_blas(s, bp, W, qn, fn, tr, wsah, rtab, st), "BLAS emit");
        }
        for (size_t i = 0; i < count; i++) {
            MeshObj *m = meshes[i];
            const uint32_t *sc = &rb.segctl[kSegWords * i];
            m->wide_sah = wsah + 2 * i;
            m->seg = uint32_t(i);
            m->refits = 0;
            m->node_count = segs[i].item_count ? sc[kSegNodes] : 0u;
            m->tri_count = segs[i].item_count;
            m->ref_count = isegs[i].item_count;
            m->depth = segs[i].item_count ? sc[kSegDepth] : 0u;
            m->mem_bytes = size_t(m->node_count) * (sizeof(Node8Q) + sizeof(Node8F) + (rtab ? 8 : 0)) +
                           size_t(m->ref_count) * sizeof(TriRec);
            const double ra = rb.bin_sah[2 * i + 1];
            m->sah = ra > 0.0 ? rb.bin_sah[2 * i] / ra : 0.0;
        }
    }
    // the old blocks are released only after the new BLASes are enqueued; a
    // block shared with other meshes lives on until they are rebuilt too
    for (MeshObj *m : meshes) {
        if (m->block) retired.blocks.push_back(std::move(m->block));
        m->block = block;
        m->built = true;
        m->generation++;
    }
    bump_mesh_epoch();
    if (rb.ctl[kCtlErr] & kErrQuant) return fail(LCX_ERR_INVALID_ARG, "vertex coordinates too large to quantise");
    return LCX_OK;
}

// Traversal knobs (see lcx_set_trace_tuning).
struct TraceTuning {
    uint32_t refill = 4;    // measured best on the terrain workload (refill sweep 1..32)
    uint32_t postpone = 0;  // modes 0 / 1: postponing did not pay (sweep 0..24); mode 2: 0 = per-kind flush size
    uint32_t mode = 2;      // traversal loop structure: deferred triangle batches (quantised nodes; FP32 runs mode 0)
    uint32_t short_stack = 16;  // shared-memory stack entries per thread (8, 16, 24)
    uint32_t max_steps = kMaxRaySteps;  // per-ray step bound (lcx_set_trace_step_bound)
};
TraceTuning g_tune;

// Ray reordering (see lcx_set_trace_reorder): origin Morton bits per axis, 0 = off.
struct ReorderTuning {
    uint32_t bits = 0;
    uint32_t min_rays = 1u << 16;
};
ReorderTuning g_reorder;

}  // namespace

namespace lcx {

// Validates a trace_closest call and fills everything of TraceParams except
// `pool`, without touching device memory (no per-device state is created).
int trace_params_for(uint64_t accel, const LcxRay *d_rays, uint32_t ray_count, uint32_t mask, LcxTriangleHit *d_hits,
                     uint32_t max_rays, TraceParams &p) {
    auto a = find_accel(accel);
    if (!a) return fail(LCX_ERR_INVALID_ARG, "unknown accel handle %llu", (unsigned long long)accel);
    if (ray_count > max_rays)
        return fail(LCX_ERR_INVALID_ARG, "ray_count %u exceeds the maximum of %u for this entry point", ray_count,
                    max_rays);
    if (ray_count && (!d_rays || !d_hits)) return fail(LCX_ERR_INVALID_ARG, "null ray or hit buffer");
    if (reinterpret_cast<uintptr_t>(d_rays) % 16 != 0 || reinterpret_cast<uintptr_t>(d_hits) % 8 != 0)
        return fail(LCX_ERR_INVALID_ARG, "rays must be 16-byte and hits 8-byte aligned");
    std::lock_guard<std::mutex> lk(a->mtx);
    if (!a->built) return fail(LCX_ERR_NOT_BUILT, "accel not built");
    {
        uint64_t h = 0;
        bool gone = false;
        if (!meshes_current(a.get(), &h, &gone))
            return fail(LCX_ERR_NOT_BUILT, gone ? "mesh %llu was destroyed; rebuild the accel"
                                                : "mesh %llu was rebuilt after the accel build; rebuild the accel",
                        (unsigned long long)h);
    }
    const uint32_t depth_need = a->depth + a->max_blas_depth + 3;
    if (int(depth_need) > kStackSize)
        return fail(LCX_ERR_DEPTH, "TLAS depth %u + BLAS depth %u exceeds the traversal stack (%d)", a->depth,
                    a->max_blas_depth, kStackSize);
    p = TraceParams{};
    p.tlas_q = a->qn;
    p.tlas_f = a->fn;
    p.insts = a->recs;
    p.motion = a->has_motion || a->has_curves;
    p.curves = a->has_curves;
    p.rays = reinterpret_cast<const Ray *>(d_rays);
    p.hits = reinterpret_cast<Hit *>(d_hits);
    p.ray_count = ray_count;
    p.mask = mask & 0xffu;
    p.refill = g_tune.refill;
    p.postpone = g_tune.postpone;
    p.mode = g_tune.mode;
    p.short_stack = g_tune.short_stack;
    p.max_steps = g_tune.max_steps;
    p.postpone_sp = kStackSize - int(depth_need);
    return LCX_OK;
}

int record_error(int code, const char *msg) { return fail(code, "%s", msg); }

std::shared_mutex &lifetime_mutex() { return g_life_mtx; }

}  // namespace lcx

extern "C" {

uint32_t lcx_version(void) { return 0x000100u; }

const char *lcx_last_error_string(void) { return g_last_error.c_str(); }

int lcx_device_init(int device) {
    LCX_CUDA(cudaSetDevice(device), "cudaSetDevice");
    DeviceState *ds = nullptr;
    return current_device_state(&ds);
}

// ------------------------------------------------------------------- mesh
int lcx_mesh_create(const LcxAccelOption *option, uint64_t *out_handle) {
    if (!out_handle) return fail(LCX_ERR_INVALID_ARG, "lcx_mesh_create: out_handle is null");
    if (int r = check_option(option)) return r;
    DeviceState *ds = nullptr;
    if (int r = current_device_state(&ds)) return r;
    auto m = std::make_shared<MeshObj>();
    if (option) m->opt = *option;
    m->device = ds->device;
    LCX_CUDA(cudaMalloc(&m->d_desc, sizeof(BlasDesc)), "cudaMalloc(BlasDesc)");
    LCX_CUDA(cudaMemset(m->d_desc, 0, sizeof(BlasDesc)), "cudaMemset(BlasDesc)");
    const uint64_t h = g_next_handle.fetch_add(1);
    {
        std::lock_guard<std::mutex> lk(g_reg_mtx);
        g_meshes[h] = m;
    }
    *out_handle = h;
    return LCX_OK;
}

int lcx_mesh_create_motion(const LcxAccelOption *option, const LcxMotionOption *motion, uint64_t *out_handle) {
    if (!out_handle || !motion) return fail(LCX_ERR_INVALID_ARG, "lcx_mesh_create_motion: null argument");
    if (int r = check_option(option)) return r;
    const LcxMotionOption &o = *motion;
    if (o.keyframe_count < 2 || o.keyframe_count > (1u << 16))
        return fail(LCX_ERR_INVALID_ARG, "a motion mesh needs 2..65536 keyframes");
    if (!(o.time_end > o.time_start) || !std::isfinite(o.time_start) || !std::isfinite(o.time_end))
        return fail(LCX_ERR_INVALID_ARG, "motion time range must be finite with time_end > time_start");
    if (option && option->allow_update)
        return fail(LCX_ERR_INVALID_ARG, "motion meshes cannot be refit (allow_update)");
    DeviceState *ds = nullptr;
    if (int r = current_device_state(&ds)) return r;
    auto m = std::make_shared<MeshObj>();
    if (option) m->opt = *option;
    m->device = ds->device;
    m->motion = o;
    LCX_CUDA(cudaMalloc(&m->d_desc, sizeof(BlasDesc) + sizeof(MeshMotion)), "cudaMalloc(BlasDesc)");
    LCX_CUDA(cudaMemset(m->d_desc, 0, sizeof(BlasDesc) + sizeof(MeshMotion)), "cudaMemset(BlasDesc)");
    m->d_motion = reinterpret_cast<MeshMotion *>(m->d_desc + 1);
    const MeshMotion *mp = m->d_motion;
    LCX_CUDA(cudaMemcpy(reinterpret_cast<char *>(m->d_desc) + offsetof(BlasDesc, motion), &mp, sizeof(mp),
                        cudaMemcpyHostToDevice),
             "BlasDesc motion");
    const uint64_t h = g_next_handle.fetch_add(1);
    {
        std::lock_guard<std::mutex> lk(g_reg_mtx);
        g_meshes[h] = m;
    }
    *out_handle = h;
    return LCX_OK;
}

int lcx_mesh_destroy(uint64_t mesh) {
    std::shared_ptr<MeshObj> m;
    {
        // under the exclusive lifetime lock: every trace that found this mesh has enqueued
        // its kernel, and no later one can find it (or an accel still referencing it)
        std::unique_lock<std::shared_mutex> life(g_life_mtx);
        std::lock_guard<std::mutex> lk(g_reg_mtx);
        auto it = g_meshes.find(mesh);
        if (it == g_meshes.end()) return fail(LCX_ERR_INVALID_ARG, "lcx_mesh_destroy: unknown mesh handle %llu",
                                              (unsigned long long)mesh);
        m = it->second;
        g_meshes.erase(it);
        bump_mesh_epoch();
    }
    // outside it: traces on other objects go on while queued work that may read this BVH drains
    std::lock_guard<std::mutex> lk(m->mtx);
    cudaDeviceSynchronize();
    m->block.reset();
    m->curve_keys.reset();
    if (m->d_desc) cudaFree(m->d_desc);
    m->d_desc = nullptr;
    return LCX_OK;
}

int lcx_procedural_create(const LcxAccelOption *option, uint64_t *out_handle) {
    if (int r = lcx_mesh_create(option, out_handle)) return r;
    auto m = find_mesh(*out_handle);
    m->kind = kSegAabbs;
    return LCX_OK;
}

int lcx_procedural_destroy(uint64_t handle) {
    auto m = find_mesh(handle);
    if (m && m->kind != kSegAabbs) return fail(LCX_ERR_INVALID_ARG, "lcx_procedural_destroy: handle is a mesh");
    return lcx_mesh_destroy(handle);
}

int lcx_procedural_build(uint64_t handle, const LcxProceduralBuildCommand *cmd, void *stream) {
    auto m = find_mesh(handle);
    if (!m || m->kind != kSegAabbs)
        return fail(LCX_ERR_INVALID_ARG, "lcx_procedural_build: unknown procedural primitive handle %llu",
                    (unsigned long long)handle);
    if (!cmd) return fail(LCX_ERR_INVALID_ARG, "lcx_procedural_build: command is null");
    if (cmd->request > LCX_REQUEST_FORCE_BUILD) return fail(LCX_ERR_INVALID_ARG, "invalid build request %u", cmd->request);
    if (cmd->aabb_buffer_size % 24 != 0)
        return fail(LCX_ERR_INVALID_ARG, "AABB buffer size %zu is not a multiple of 24 bytes", cmd->aabb_buffer_size);
    const uint64_t count = cmd->aabb_buffer_size / 24;
    if (count >= (1ull << 31)) return fail(LCX_ERR_INVALID_ARG, "too many AABBs (%llu)", (unsigned long long)count);
    if (count && !cmd->aabb_buffer) return fail(LCX_ERR_INVALID_ARG, "AABB buffer is null");
    if ((cmd->aabb_buffer + cmd->aabb_buffer_offset) % 4 != 0)
        return fail(LCX_ERR_INVALID_ARG, "AABB buffer address must be 4-byte aligned");
    Retired retired;  // released after the mutex below
    std::lock_guard<std::mutex> lk(m->mtx);
    std::vector<MeshObj *> ms{m.get()};
    SegInput g{};
    g.vbase = reinterpret_cast<const unsigned char *>(cmd->aabb_buffer) + cmd->aabb_buffer_offset;
    g.vstride = 24;
    g.tbase = nullptr;
    g.vcount = uint32_t(count);
    g.item_offset = 0;
    g.item_count = uint32_t(count);
    g.kind = kSegAabbs;
    g.desc = m->d_desc;
    std::vector<SegInput> segs{g};
    std::vector<uint32_t> req{cmd->request};
    return build_meshes(ms, segs, req, static_cast<cudaStream_t>(stream), retired);
}

int lcx_curve_create(const LcxAccelOption *option, uint64_t *out_handle) {
    if (int r = lcx_mesh_create(option, out_handle)) return r;
    auto m = find_mesh(*out_handle);
    m->kind = kSegCurves;
    return LCX_OK;
}

int lcx_curve_create_motion(const LcxAccelOption *option, const LcxMotionOption *motion, uint64_t *out_handle) {
    if (motion && motion->keyframe_count >= (1u << 16))
        return fail(LCX_ERR_INVALID_ARG, "a motion curve takes at most 65535 keyframes");
    if (int r = lcx_mesh_create_motion(option, motion, out_handle)) return r;
    auto m = find_mesh(*out_handle);
    m->kind = kSegCurves;
    return LCX_OK;
}

int lcx_curve_destroy(uint64_t handle) {
    auto m = find_mesh(handle);
    if (m && m->kind != kSegCurves) return fail(LCX_ERR_INVALID_ARG, "lcx_curve_destroy: handle is not a curve");
    return lcx_mesh_destroy(handle);
}

// Curve builds (the reference's CurveBuildCommand visit, cpu/accel.rs:142-204;
// CUDA: cuda_curve.cpp:37-70).  The segments go to Bezier form and are cut into
// cones (one host read-back for the cone count), and the BLAS is built over the
// cones; their leaf records hold everything a trace needs, so the build-time
// arrays are released with the build.
int lcx_curve_build(uint64_t handle, const LcxCurveBuildCommand *cmd, void *stream) {
    auto m = find_mesh(handle);
    if (!m || m->kind != kSegCurves)
        return fail(LCX_ERR_INVALID_ARG, "lcx_curve_build: unknown curve handle %llu", (unsigned long long)handle);
    if (!cmd) return fail(LCX_ERR_INVALID_ARG, "lcx_curve_build: command is null");
    if (cmd->request > LCX_REQUEST_FORCE_BUILD) return fail(LCX_ERR_INVALID_ARG, "invalid build request %u", cmd->request);
    if (cmd->basis > LCX_CURVE_BEZIER) return fail(LCX_ERR_INVALID_ARG, "invalid curve basis %u", cmd->basis);
    if (cmd->cp_stride < 16 || cmd->cp_stride % 4 != 0)
        return fail(LCX_ERR_INVALID_ARG, "control point stride %zu must be >= 16 and a multiple of 4", cmd->cp_stride);
    if (cmd->seg_count >= (1ull << 26) || cmd->cp_count >= (1ull << 32))
        return fail(LCX_ERR_INVALID_ARG, "too many curve segments (%zu) or control points (%zu)", cmd->seg_count,
                    cmd->cp_count);
    if (cmd->seg_count && (!cmd->cp_buffer || !cmd->seg_buffer))
        return fail(LCX_ERR_INVALID_ARG, "null control point or segment buffer");
    if ((cmd->cp_buffer + cmd->cp_buffer_offset) % 4 != 0 || (cmd->seg_buffer + cmd->seg_buffer_offset) % 4 != 0)
        return fail(LCX_ERR_INVALID_ARG, "control point and segment buffers must be 4-byte aligned");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (capturing(st)) return fail(LCX_ERR_INVALID_ARG, "curve build in a CUDA graph capture");
    Retired retired;  // released after the mutex below (the build-time arrays go with it)
    std::lock_guard<std::mutex> lk(m->mtx);
    const uint32_t nseg = uint32_t(cmd->seg_count);
    const uint32_t keys = m->motion.keyframe_count >= 2 ? m->motion.keyframe_count : 1u;
    if (cmd->cp_count % keys != 0)
        return fail(LCX_ERR_INVALID_ARG, "control point count %zu is not a multiple of the %u keyframes", cmd->cp_count,
                    keys);
    const uint32_t cp_per_key = uint32_t(cmd->cp_count / keys);
    // [Bezier points 64 B per keyframe | cone offsets | metas | counts] per segment, an error word,
    // the scan's scratch
    size_t scan_bytes = 0;
    LCX_CUDA(exclusive_sum(nullptr, &scan_bytes, nullptr, nullptr, std::max(nseg, 1u), st), "scan size");
    const size_t nbytes = size_t(std::max(nseg, 1u));
    const size_t scan_at = (nbytes * (64 * size_t(keys) + 12) + 4 + 255) / 256 * 256;
    auto cblock = std::make_shared<DevBlock>();
    cblock->bytes = scan_at + scan_bytes;
    LCX_CUDA(cudaMalloc(&cblock->ptr, cblock->bytes), "cudaMalloc(curve build)");
    retired.blocks.push_back(cblock);
    char *base = static_cast<char *>(cblock->ptr);
    float4 *bez = reinterpret_cast<float4 *>(base);
    uint32_t *off = reinterpret_cast<uint32_t *>(base + 64 * size_t(keys) * nbytes);
    uint32_t *meta = off + nbytes;
    uint32_t *count = meta + nbytes;
    uint32_t *err = count + nbytes;
    const auto *cps = reinterpret_cast<const unsigned char *>(cmd->cp_buffer) + cmd->cp_buffer_offset;
    const auto *seg = reinterpret_cast<const uint32_t *>(reinterpret_cast<const unsigned char *>(cmd->seg_buffer) +
                                                         cmd->seg_buffer_offset);
    uint32_t cones = 0;
    uint32_t *cone_seg = nullptr;
    if (nseg) {
        LCX_CUDA(cudaMemsetAsync(err, 0, sizeof(uint32_t), st), "curve error word");
        LCX_CUDA(curve_prepare(cps, cmd->cp_stride, cp_per_key, keys, seg, nseg, cmd->basis, bez, count, meta, err,
                               st),
                 "curve prepare");
        LCX_CUDA(exclusive_sum(base + scan_at, &scan_bytes, count, off, nseg, st), "curve cone scan");
        uint32_t h[3] = {0, 0, 0};  // last offset, last count, error
        LCX_CUDA(cudaMemcpyAsync(&h[0], off + nseg - 1, 4, cudaMemcpyDeviceToHost, st), "cone count");
        LCX_CUDA(cudaMemcpyAsync(&h[1], count + nseg - 1, 4, cudaMemcpyDeviceToHost, st), "cone count");
        LCX_CUDA(cudaMemcpyAsync(&h[2], err, 4, cudaMemcpyDeviceToHost, st), "curve errors");
        LCX_CUDA(cudaStreamSynchronize(st), "sync");
        if (h[2]) return fail(LCX_ERR_INVALID_ARG, "curve segment control points run past the %u given", cp_per_key);
        cones = h[0] + h[1];  // at most 32 per segment: below 2^31
        auto pblock = std::make_shared<DevBlock>();
        pblock->bytes = sizeof(uint32_t) * std::max(cones, 1u);
        LCX_CUDA(cudaMalloc(&pblock->ptr, pblock->bytes), "cudaMalloc(curve cones)");
        retired.blocks.push_back(pblock);
        cone_seg = static_cast<uint32_t *>(pblock->ptr);
        LCX_CUDA(curve_fill(off, count, nseg, cone_seg, st), "curve fill");
    }
    std::shared_ptr<DevBlock> kblock;  // keyframed curves: the cones' balls per keyframe, kept with the tree
    if (keys > 1) {
        kblock = std::make_shared<DevBlock>();
        kblock->bytes = 2 * sizeof(float4) * size_t(keys) * std::max(cones, 1u);
        LCX_CUDA(cudaMalloc(&kblock->ptr, kblock->bytes), "cudaMalloc(curve keyframes)");
        MeshMotion mm{};
        mm.keys = keys;
        mm.t0 = m->motion.time_start;
        mm.t1 = m->motion.time_end;
        mm.flags = (m->motion.vanish_start ? 1u : 0u) | (m->motion.vanish_end ? 2u : 0u);
        LCX_CUDA(cudaMemcpyAsync(m->d_motion, &mm, sizeof(mm), cudaMemcpyHostToDevice, st), "motion upload");
        LCX_CUDA(cudaStreamSynchronize(st), "sync");  // `mm` is a host local
    }
    std::vector<MeshObj *> ms{m.get()};
    SegInput g{};
    g.vbase = reinterpret_cast<const unsigned char *>(bez);
    g.vstride = kblock ? reinterpret_cast<uint64_t>(kblock->ptr) : 0;
    g.tbase = reinterpret_cast<const unsigned char *>(cone_seg);
    g.vcount = nseg;
    g.item_offset = 0;
    g.item_count = cones;
    g.kind = kSegCurves | (cmd->basis << 8) | (keys > 1 ? keys << 16 : 0u);
    g.desc = m->d_desc;
    std::vector<SegInput> segs{g};
    std::vector<uint32_t> req{LCX_REQUEST_FORCE_BUILD};
    const int r = build_meshes(ms, segs, req, st, retired);
    if (r != LCX_OK) return r;  // the old tree keeps its keyframe balls
    if (m->curve_keys) retired.blocks.push_back(std::move(m->curve_keys));
    m->curve_keys = std::move(kblock);
    return LCX_OK;
}

int lcx_mesh_build(uint64_t mesh, const LcxMeshBuildCommand *cmd, void *stream) {
    NvtxRange nr("lcx_mesh_build");
    auto m = find_mesh(mesh);
    if (!m) return fail(LCX_ERR_INVALID_ARG, "lcx_mesh_build: unknown mesh handle %llu", (unsigned long long)mesh);
    if (!cmd) return fail(LCX_ERR_INVALID_ARG, "lcx_mesh_build: command is null");
    Retired retired;  // released after the mutex below
    std::lock_guard<std::mutex> lk(m->mtx);
    std::vector<MeshObj *> ms{m.get()};
    std::vector<SegInput> segs;
    std::vector<uint32_t> req;
    if (int r = mesh_segments(ms, cmd, segs, req)) return r;
    return build_meshes(ms, segs, req, static_cast<cudaStream_t>(stream), retired);
}

int lcx_mesh_build_batch(const uint64_t *meshes, const LcxMeshBuildCommand *cmds, uint32_t count, void *stream) {
    NvtxRange nr("lcx_mesh_build_batch");
    if (count == 0) return LCX_OK;
    if (!meshes || !cmds) return fail(LCX_ERR_INVALID_ARG, "lcx_mesh_build_batch: null arguments");
    std::vector<std::shared_ptr<MeshObj>> objs(count);
    for (uint32_t i = 0; i < count; i++) {
        objs[i] = find_mesh(meshes[i]);
        if (!objs[i]) return fail(LCX_ERR_INVALID_ARG, "lcx_mesh_build_batch: unknown mesh handle %llu (entry %u)",
                                  (unsigned long long)meshes[i], i);
    }
    // lock in address order (no deadlock with concurrent batches); duplicates are an error
    std::vector<MeshObj *> order(count);
    for (uint32_t i = 0; i < count; i++) order[i] = objs[i].get();
    std::vector<MeshObj *> sorted = order;
    std::sort(sorted.begin(), sorted.end());
    for (uint32_t i = 1; i < count; i++)
        if (sorted[i] == sorted[i - 1]) return fail(LCX_ERR_INVALID_ARG, "lcx_mesh_build_batch: a mesh appears twice");
    Retired retired;  // released after the mutexes below
    std::vector<std::unique_lock<std::mutex>> locks;
    locks.reserve(count);
    for (MeshObj *m : sorted) locks.emplace_back(m->mtx);
    std::vector<SegInput> segs;
    std::vector<uint32_t> req;
    if (int r = mesh_segments(order, cmds, segs, req)) return r;
    return build_meshes(order, segs, req, static_cast<cudaStream_t>(stream), retired);
}

int lcx_mesh_build_batch_reserve(const uint64_t *meshes, const LcxMeshBuildCommand *cmds, uint32_t count,
                                 void *stream) {
    if (count == 0) return LCX_OK;
    if (!meshes || !cmds) return fail(LCX_ERR_INVALID_ARG, "lcx_mesh_build_batch_reserve: null arguments");
    std::vector<std::shared_ptr<MeshObj>> objs(count);
    for (uint32_t i = 0; i < count; i++) {
        objs[i] = find_mesh(meshes[i]);
        if (!objs[i]) return fail(LCX_ERR_INVALID_ARG, "lcx_mesh_build_batch_reserve: unknown mesh handle %llu",
                                  (unsigned long long)meshes[i]);
        if (objs[i]->opt.allow_update)
            return fail(LCX_ERR_INVALID_ARG, "a reserved batch is rebuilt, not refit (allow_update)");
        if (objs[i]->motion.keyframe_count >= 2)
            return fail(LCX_ERR_INVALID_ARG, "motion meshes cannot be reserved");
    }
    std::vector<MeshObj *> order(count);
    for (uint32_t i = 0; i < count; i++) order[i] = objs[i].get();
    std::vector<MeshObj *> sorted = order;
    std::sort(sorted.begin(), sorted.end());
    for (uint32_t i = 1; i < count; i++)
        if (sorted[i] == sorted[i - 1]) return fail(LCX_ERR_INVALID_ARG, "a mesh appears twice");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (capturing(st)) return fail(LCX_ERR_INVALID_ARG, "lcx_mesh_build_batch_reserve cannot be captured");
    Retired retired;
    std::vector<std::unique_lock<std::mutex>> locks;
    locks.reserve(count);
    for (MeshObj *m : sorted) locks.emplace_back(m->mtx);
    std::vector<SegInput> segs;
    std::vector<uint32_t> req;
    if (int r = mesh_segments(order, cmds, segs, req)) return r;
    uint64_t total = 0;
    for (const SegInput &g : segs) total += g.item_count;
    if (total == 0) return fail(LCX_ERR_INVALID_ARG, "a reserved batch needs triangles");
    return build_meshes(order, segs, req, st, retired, true);
}

int lcx_mesh_reserve_batch(const uint64_t *meshes, const LcxMeshBuildCommand *cmds, uint32_t count, void *stream) {
    if (count == 0) return LCX_OK;
    if (!meshes || !cmds) return fail(LCX_ERR_INVALID_ARG, "lcx_mesh_reserve_batch: null arguments");
    std::vector<std::shared_ptr<MeshObj>> objs(count);
    for (uint32_t i = 0; i < count; i++) {
        objs[i] = find_mesh(meshes[i]);
        if (!objs[i]) return fail(LCX_ERR_INVALID_ARG, "lcx_mesh_reserve_batch: unknown mesh handle %llu",
                                  (unsigned long long)meshes[i]);
        if (objs[i]->opt.allow_update)
            return fail(LCX_ERR_INVALID_ARG, "a reserved batch is rebuilt, not refit (allow_update)");
        if (objs[i]->motion.keyframe_count >= 2) return fail(LCX_ERR_INVALID_ARG, "motion meshes cannot be reserved");
    }
    std::vector<MeshObj *> order(count);
    for (uint32_t i = 0; i < count; i++) order[i] = objs[i].get();
    std::vector<MeshObj *> sorted = order;
    std::sort(sorted.begin(), sorted.end());
    for (uint32_t i = 1; i < count; i++)
        if (sorted[i] == sorted[i - 1]) return fail(LCX_ERR_INVALID_ARG, "a mesh appears twice");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (capturing(st)) return fail(LCX_ERR_INVALID_ARG, "lcx_mesh_reserve_batch cannot be captured (it allocates)");
    NvtxRange nr("lcx_mesh_reserve_batch");
    Retired retired;
    std::vector<std::unique_lock<std::mutex>> locks;
    locks.reserve(count);
    for (MeshObj *m : sorted) locks.emplace_back(m->mtx);
    std::vector<SegInput> segs;
    std::vector<uint32_t> req;
    if (int r = mesh_segments(order, cmds, segs, req)) return r;
    for (const SegInput &g : segs)
        if (g.kind != kSegTriangles) return fail(LCX_ERR_INVALID_ARG, "a reserved batch holds triangle meshes");
    return reserve_only(order, segs, st, retired);
}

int lcx_mesh_stats(uint64_t mesh, LcxAccelStats *out) {
    auto m = find_mesh(mesh);
    if (!m || !out) return fail(LCX_ERR_INVALID_ARG, "lcx_mesh_stats: bad arguments");
    std::lock_guard<std::mutex> lk(m->mtx);
    if (!m->built) return fail(LCX_ERR_NOT_BUILT, "mesh not built");
    std::memset(out, 0, sizeof(*out));
    out->node_count = m->node_count;
    out->leaf_prim_count = m->ref_count;
    out->device_bytes = m->mem_bytes + sizeof(BlasDesc);
    out->depth = m->depth;
    out->sah_cost = m->sah;
    out->refits = m->refits;
    if (m->wide_sah) {
        double h[2] = {0, 0};
        LCX_CUDA(cudaMemcpy(h, m->wide_sah, sizeof(h), cudaMemcpyDeviceToHost), "wide SAH readback");
        out->wide_sah_cost = h[1] > 0.0 ? h[0] / h[1] : 0.0;
    }
    return LCX_OK;
}

// ------------------------------------------------------------------ accel
int lcx_accel_create(const LcxAccelOption *option, uint64_t *out_handle) {
    if (!out_handle) return fail(LCX_ERR_INVALID_ARG, "lcx_accel_create: out_handle is null");
    if (int r = check_option(option)) return r;
    DeviceState *ds = nullptr;
    if (int r = current_device_state(&ds)) return r;
    auto a = std::make_shared<AccelObj>();
    if (option) a->opt = *option;
    a->device = ds->device;
    const uint64_t h = g_next_handle.fetch_add(1);
    {
        std::lock_guard<std::mutex> lk(g_reg_mtx);
        g_accels[h] = a;
    }
    *out_handle = h;
    return LCX_OK;
}

int lcx_accel_destroy(uint64_t accel) {
    std::shared_ptr<AccelObj> a;
    {
        // as lcx_mesh_destroy: the exclusive lock only orders this after traces that found the accel
        std::unique_lock<std::shared_mutex> life(g_life_mtx);
        std::lock_guard<std::mutex> lk(g_reg_mtx);
        auto it = g_accels.find(accel);
        if (it == g_accels.end()) return fail(LCX_ERR_INVALID_ARG, "lcx_accel_destroy: unknown accel handle %llu",
                                              (unsigned long long)accel);
        a = it->second;
        g_accels.erase(it);
    }
    std::lock_guard<std::mutex> lk(a->mtx);
    cudaDeviceSynchronize();
    a->block.reset();
    if (a->d_inst) cudaFree(a->d_inst);
    a->d_inst = nullptr;
    return LCX_OK;
}

int lcx_accel_build(uint64_t accel, uint32_t instance_count, uint32_t request, const LcxModification *mods,
                    size_t mod_count, int update_instance_buffer_only, void *stream) {
    NvtxRange nr("lcx_accel_build");
    auto a = find_accel(accel);
    if (!a) return fail(LCX_ERR_INVALID_ARG, "lcx_accel_build: unknown accel handle %llu", (unsigned long long)accel);
    if (request > LCX_REQUEST_FORCE_BUILD) return fail(LCX_ERR_INVALID_ARG, "invalid build request %u", request);
    // src/runtime/rtx/accel.cpp:72-73
    if (instance_count == 0) return fail(LCX_ERR_INVALID_ARG, "Building acceleration structure without instances.");
    if (mod_count && !mods) return fail(LCX_ERR_INVALID_ARG, "modifications pointer is null");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    Retired retired;  // the replaced TLAS block, released after the locks below
    // no mesh referenced below can be destroyed (its BLAS descriptor freed) before
    // the build's kernels are enqueued
    std::shared_lock<std::shared_mutex> life(g_life_mtx);
    std::lock_guard<std::mutex> lk(a->mtx);
    // in a CUDA graph capture only a TLAS refit without modifications can run
    // (modifications are host data; a build sizes its block on the host)
    if (capturing(st) &&
        (mod_count || update_instance_buffer_only || request != LCX_REQUEST_PREFER_UPDATE || !a->opt.allow_update ||
         !a->built || a->pending_rebuild || instance_count != a->built_instances || !a->block || !a->block->rtab))
        return fail(LCX_ERR_INVALID_ARG,
                    "lcx_accel_build in a CUDA graph capture: only a TLAS refit without modifications can be captured "
                    "(apply modifications with update_instance_buffer_only outside the capture)");
    // translate and validate the modifications
    std::vector<ModRec> recs(mod_count);
    std::vector<uint64_t> new_mesh(mod_count, 0);
    std::vector<std::shared_ptr<MotionObj>> new_motion(mod_count);
    for (size_t i = 0; i < mod_count; i++) {
        const LcxModification &md = mods[i];
        if (md.index >= instance_count)
            return fail(LCX_ERR_INVALID_ARG, "modification %zu: instance index %u >= instance count %u", i, md.index,
                        instance_count);
        ModRec &r = recs[i];
        r.index = md.index;
        r.user_id = md.user_id;
        r.flags = md.flags;
        r.vis_mask = md.vis_mask;
        std::memcpy(r.affine, md.affine, sizeof(r.affine));
        r.primitive = 0;
        r.motion = 0;
        if (md.flags & LCX_MOD_PRIMITIVE) {
            uint64_t mesh = md.primitive;
            auto m = find_mesh(mesh);
            if (!m) {  // a motion instance: its mesh, moved by its keyframes
                auto mo = find_motion(md.primitive);
                if (!mo) return fail(LCX_ERR_INVALID_ARG, "modification %zu: unknown mesh handle %llu", i,
                                     (unsigned long long)md.primitive);
                if (!mo->built) return fail(LCX_ERR_NOT_BUILT, "motion instance not built");
                mesh = mo->child;
                m = find_mesh(mesh);
                if (!m) return fail(LCX_ERR_INVALID_ARG, "modification %zu: the motion instance's mesh was destroyed",
                                    i);
                r.motion = reinterpret_cast<uint64_t>(mo->d_md);
                new_motion[i] = std::move(mo);
            }
            if (!m->built) return fail(LCX_ERR_NOT_BUILT, "Mesh not built");  // accel.rs:356-358
            r.primitive = reinterpret_cast<uint64_t>(m->d_desc);
            new_mesh[i] = mesh;
        }
    }
    // instance storage
    if (instance_count > a->inst_cap) {
        const uint32_t cap = std::max<uint32_t>(instance_count, a->inst_cap * 2);
        InstState *p = nullptr;
        LCX_CUDA(cudaMalloc(&p, sizeof(InstState) * cap), "cudaMalloc(instances)");
        if (a->d_inst) {
            LCX_CUDA(cudaMemcpyAsync(p, a->d_inst, sizeof(InstState) * a->inst_count, cudaMemcpyDeviceToDevice, st),
                     "instance copy");
            LCX_CUDA(cudaStreamSynchronize(st), "sync");
            cudaFree(a->d_inst);
        }
        a->d_inst = p;
        a->inst_cap = cap;
    }
    if (instance_count > a->inst_count) LCX_CUDA(init_instances(a->d_inst, a->inst_count, instance_count, st), "init");
    if (instance_count != a->inst_count) a->uniq_dirty = true;
    a->inst_mesh.resize(instance_count, 0);
    for (uint32_t i = a->inst_count; i < instance_count; i++) a->inst_mesh[i] = 0;
    for (size_t i = instance_count; i < a->inst_motion.size(); i++)  // queued traces may still read it
        if (a->inst_motion[i]) retired.others.push_back(std::move(a->inst_motion[i]));
    a->inst_motion.resize(instance_count);
    a->inst_count = instance_count;
    for (size_t i = 0; i < mod_count; i++)
        if (new_mesh[i]) {
            a->inst_mesh[recs[i].index] = new_mesh[i];
            auto &slot = a->inst_motion[recs[i].index];
            if (slot) retired.others.push_back(std::move(slot));
            slot = std::move(new_motion[i]);
            a->uniq_dirty = true;
            a->pending_rebuild = true;  // as cuda_accel.cpp:184-185: a primitive change forces a rebuild
        }
    if (mod_count) {
        ScratchHolder hold(st);
        ModRec *d_mods = nullptr;
        LCX_CUDA(hold.alloc((void **)&d_mods, sizeof(ModRec) * mod_count), "scratch");
        LCX_CUDA(cudaMemcpyAsync(d_mods, recs.data(), sizeof(ModRec) * mod_count, cudaMemcpyHostToDevice, st),
                 "modification upload");
        LCX_CUDA(apply_modifications(d_mods, uint32_t(mod_count), a->d_inst, instance_count, st), "apply mods");
    }
    if (update_instance_buffer_only) return LCX_OK;

    // every referenced mesh must exist and be built before a kernel reads its descriptor
    std::vector<std::pair<uint64_t, uint64_t>> gens;
    uint32_t max_blas_depth = 0;
    bool mesh_motion = false;  // an instanced mesh has vertex motion
    bool curves = false;       // an instanced BLAS is a curve
    {
        if (a->uniq_dirty) {
            std::vector<uint64_t> &uniq = a->uniq_mesh;
            uniq.assign(a->inst_mesh.begin(), a->inst_mesh.end());
            std::sort(uniq.begin(), uniq.end());
            uniq.erase(std::unique(uniq.begin(), uniq.end()), uniq.end());
            if (!uniq.empty() && uniq[0] == 0) uniq.erase(uniq.begin());
            a->uniq_dirty = false;
        }
        for (uint64_t h : a->uniq_mesh) {
            auto m = find_mesh(h);
            if (!m) return fail(LCX_ERR_INVALID_ARG, "instance references destroyed mesh %llu", (unsigned long long)h);
            if (!m->built) return fail(LCX_ERR_NOT_BUILT, "Mesh not built");
            gens.emplace_back(h, m->generation);
            max_blas_depth = std::max(max_blas_depth, m->depth);
            mesh_motion = mesh_motion || m->motion.keyframe_count >= 2;
            curves = curves || m->kind == kSegCurves;
        }
    }
    const uint32_t n = instance_count;
    std::vector<std::pair<std::shared_ptr<MotionObj>, uint64_t>> mgens;
    bool inst_motion = false;
    for (const auto &mo : a->inst_motion) inst_motion = inst_motion || mo != nullptr;
    a->has_motion = inst_motion || mesh_motion;
    a->has_curves = curves;
    if (inst_motion) {
        std::unordered_set<MotionObj *> seen;
        for (const auto &mo : a->inst_motion) {
            if (!mo || !seen.insert(mo.get()).second) continue;
            if (!mo->alive.load()) return fail(LCX_ERR_INVALID_ARG, "an instance references a destroyed motion instance");
            mgens.emplace_back(mo, mo->generation);
        }
    }

    // PREFER_UPDATE of an accel created with allow_update, built with the same
    // instance count and no instance primitive changed since (the rebuild rules
    // of cuda_accel.cpp:261-267): refit the TLAS (same topology, new instance
    // boxes and records); kernels only, no host synchronisation
    DevBlock *tb = a->block.get();
    if (request == LCX_REQUEST_PREFER_UPDATE && a->opt.allow_update && a->built && !a->pending_rebuild && tb &&
        tb->rtab && n == a->built_instances) {
        DeviceState *ds = nullptr;
        if (int r = current_device_state(&ds)) return r;
        LCX_CUDA(refit_tlas(a->d_inst, n, tb->ilo, tb->ihi, tb->w2o, tb->segctl, tb->wide, tb->rtab, a->qn, a->fn,
                            a->recs, tb->counters, ds->refit_ctl, st),
                 "TLAS refit");
        a->mesh_gens = gens;
        a->motion_gens = mgens;
        a->checked_epoch = 0;
        a->max_blas_depth = max_blas_depth;
        a->refits++;
        return LCX_OK;
    }

    // TLAS build: one segment of instances, one instance per leaf slot
    BuildParams bp = build_params_for(a->opt);
    bp.leaf_max = 1;
    bp.size_bits = g_build_tune.tlas_size_bits;
    bp.cube = g_build_tune.tlas_cube;
    bp.tlas_sah = g_build_tune.tlas_sah;
    BuildReadback rb;
    std::shared_ptr<DevBlock> block;
    {
        ScratchHolder hold(st);
        BuildScratch s;
        std::vector<SegInput> segs(1);
        segs[0] = SegInput{nullptr, 0, nullptr, 0, 0, n, 0, nullptr};
        if (int r = alloc_scratch(hold, s, segs, n, true, nullptr, nullptr, bp.dp != 0)) return r;
        {
            NvtxRange nr("TLAS build: boxes, tree, collapse");
            LCX_CUDA(build_tree_insts(a->d_inst, s, bp, st), "TLAS build");
        }
        if (int r = read_back(s, st, rb)) return r;
        if (rb.ctl[kCtlErr] & kErrTooDeep) return fail(LCX_ERR_DEPTH, "TLAS deeper than %d levels", kMaxLevels);
        if (rb.segctl[kSegItems] != n)
            return fail(LCX_ERR_CUDA, "TLAS build placed %u of %u instances", rb.segctl[kSegItems], n);
        const uint32_t W = rb.ctl[kCtlWideCount];
        const size_t q_bytes = size_t(W) * sizeof(Node8Q), f_bytes = size_t(W) * sizeof(Node8F);
        const size_t r_bytes = size_t(n) * sizeof(InstRec);
        // refit data (allow_update): parent table + counters, instance boxes and inverses, segment words
        const size_t tab_bytes = (size_t(W) * (sizeof(unsigned long long) + sizeof(uint32_t)) + 15) & ~size_t(15);
        const size_t u_bytes =
            a->opt.allow_update ? tab_bytes + size_t(n) * (2 * sizeof(float4) + 12 * sizeof(float)) +
                                      sizeof(uint32_t) * kSegWords
                                : 0;
        block = std::make_shared<DevBlock>();
        block->bytes = q_bytes + f_bytes + r_bytes + 2 * sizeof(double) + u_bytes;
        LCX_CUDA(block_malloc(&block->ptr, block->bytes), "cudaMalloc(TLAS)");
        Node8Q *qn = static_cast<Node8Q *>(block->ptr);
        Node8F *fn = reinterpret_cast<Node8F *>(reinterpret_cast<char *>(block->ptr) + q_bytes);
        InstRec *ir = reinterpret_cast<InstRec *>(reinterpret_cast<char *>(block->ptr) + q_bytes + f_bytes);
        double *wsah = reinterpret_cast<double *>(reinterpret_cast<char *>(block->ptr) + q_bytes + f_bytes + r_bytes);
        unsigned long long *rtab = nullptr;
        if (a->opt.allow_update) {
            char *u = reinterpret_cast<char *>(wsah) + 2 * sizeof(double);
            rtab = reinterpret_cast<unsigned long long *>(u);
            block->rtab = rtab;
            block->counters = reinterpret_cast<uint32_t *>(rtab + W);
            block->ilo = reinterpret_cast<float4 *>(u + tab_bytes);
            block->ihi = block->ilo + n;
            block->w2o = reinterpret_cast<float *>(block->ihi + n);
            block->segctl = reinterpret_cast<uint32_t *>(block->w2o + 12ull * n);
            block->wide = W;
            block->nseg = 1;
            block->qn = qn;
            block->fn = fn;
        }
        LCX_CUDA(cudaMemsetAsync(wsah, 0, 2 * sizeof(double), st), "cudaMemset");
        {
            NvtxRange nr("TLAS build: emit nodes and instances");
            LCX_CUDA(emit_tlas(a->d_inst, s, bp, W, qn, fn, ir, wsah, rtab, st), "TLAS emit");
        }
        a->qn = qn;
        a->fn = fn;
        a->recs = ir;
        a->wide_sah = wsah;
        a->node_count = W;
        a->depth = rb.segctl[kSegDepth];
        a->sah = rb.bin_sah[1] > 0.0 ? rb.bin_sah[0] / rb.bin_sah[1] : 0.0;
    }
    if (a->block) retired.blocks.push_back(std::move(a->block));
    a->block = block;
    // remember which mesh builds this TLAS references
    a->mesh_gens = gens;
    a->motion_gens = mgens;
    a->checked_epoch = 0;
    a->max_blas_depth = max_blas_depth;
    a->built_instances = n;
    a->built = true;
    a->pending_rebuild = false;
    a->refits = 0;
    return LCX_OK;
}

int lcx_accel_stats(uint64_t accel, LcxAccelStats *out) {
    auto a = find_accel(accel);
    if (!a || !out) return fail(LCX_ERR_INVALID_ARG, "lcx_accel_stats: bad arguments");
    std::lock_guard<std::mutex> lk(a->mtx);
    if (!a->built) return fail(LCX_ERR_NOT_BUILT, "accel not built");
    std::memset(out, 0, sizeof(*out));
    out->node_count = a->node_count;
    out->leaf_prim_count = a->built_instances;
    out->device_bytes = (a->block ? a->block->bytes : 0) + sizeof(InstState) * a->inst_cap;
    out->depth = a->depth;
    out->max_blas_depth = a->max_blas_depth;
    out->refits = a->refits;
    out->sah_cost = a->sah;
    if (a->wide_sah) {
        double h[2] = {0, 0};
        LCX_CUDA(cudaMemcpy(h, a->wide_sah, sizeof(h), cudaMemcpyDeviceToHost), "wide SAH readback");
        out->wide_sah_cost = h[1] > 0.0 ? h[0] / h[1] : 0.0;
    }
    return LCX_OK;
}

int lcx_set_build_tlas_sah(uint32_t sah) {
    if (sah > 1) return fail(LCX_ERR_INVALID_ARG, "lcx_set_build_tlas_sah: 0 or 1");
    g_build_tune.tlas_sah = sah;
    return LCX_OK;
}

int lcx_get_build_tlas_sah(uint32_t *sah) {
    if (!sah) return fail(LCX_ERR_INVALID_ARG, "null output");
    *sah = g_build_tune.tlas_sah;
    return LCX_OK;
}

int lcx_get_build_kernel_launches(uint64_t *count) {
    if (!count) return fail(LCX_ERR_INVALID_ARG, "null output");
    *count = build_launches();
    return LCX_OK;
}

int lcx_set_build_collapse(uint32_t mode) {
    if (mode > 1) return fail(LCX_ERR_INVALID_ARG, "lcx_set_build_collapse: 0 or 1");
    g_build_tune.dp = mode;
    return LCX_OK;
}

int lcx_get_build_collapse(uint32_t *mode) {
    if (!mode) return fail(LCX_ERR_INVALID_ARG, "null output");
    *mode = g_build_tune.dp;
    return LCX_OK;
}

int lcx_set_build_blas_sah(uint32_t sah) {
    if (sah > 1) return fail(LCX_ERR_INVALID_ARG, "lcx_set_build_blas_sah: 0 or 1");
    g_build_tune.blas_sah = sah;
    return LCX_OK;
}

int lcx_get_build_blas_sah(uint32_t *sah) {
    if (!sah) return fail(LCX_ERR_INVALID_ARG, "null output");
    *sah = g_build_tune.blas_sah;
    return LCX_OK;
}

int lcx_set_build_fill(uint32_t fill) {
    if (fill > 1) return fail(LCX_ERR_INVALID_ARG, "lcx_set_build_fill: 0 or 1");
    g_build_tune.fill = fill;
    return LCX_OK;
}

int lcx_get_build_fill(uint32_t *fill) {
    if (!fill) return fail(LCX_ERR_INVALID_ARG, "null output");
    *fill = g_build_tune.fill;
    return LCX_OK;
}

int lcx_set_build_split(float fraction) {
    if (!(fraction >= 0.0f && fraction <= 4.0f))
        return fail(LCX_ERR_INVALID_ARG, "split fraction must be in [0, 4]");
    g_build_tune.split = fraction;
    return LCX_OK;
}

int lcx_get_build_split(float *fraction) {
    if (!fraction) return fail(LCX_ERR_INVALID_ARG, "null output");
    *fraction = g_build_tune.split;
    return LCX_OK;
}

int lcx_set_build_tuning(uint32_t leaf_max, uint32_t width) {
    if (leaf_max > 3 || width < 2 || width > 8)
        return fail(LCX_ERR_INVALID_ARG, "build tuning out of range (leaf_max 0..3, width 2..8)");
    g_build_tune.leaf_max = int(leaf_max);
    g_build_tune.width = int(width);
    return LCX_OK;
}

int lcx_set_build_morton(uint32_t blas_cube, uint32_t tlas_cube, uint32_t tlas_size_bits) {
    if (blas_cube > 1 || tlas_cube > 1 || tlas_size_bits > 6)
        return fail(LCX_ERR_INVALID_ARG, "Morton options out of range (cube 0..1, size bits 0..6)");
    g_build_tune.blas_cube = blas_cube;
    g_build_tune.tlas_cube = tlas_cube;
    g_build_tune.tlas_size_bits = tlas_size_bits;
    return LCX_OK;
}

int lcx_get_build_morton(uint32_t *blas_cube, uint32_t *tlas_cube, uint32_t *tlas_size_bits) {
    if (!blas_cube || !tlas_cube || !tlas_size_bits) return fail(LCX_ERR_INVALID_ARG, "null output");
    *blas_cube = g_build_tune.blas_cube;
    *tlas_cube = g_build_tune.tlas_cube;
    *tlas_size_bits = g_build_tune.tlas_size_bits;
    return LCX_OK;
}

int lcx_get_build_tuning(uint32_t *leaf_max, uint32_t *width) {
    if (!leaf_max || !width) return fail(LCX_ERR_INVALID_ARG, "null output");
    *leaf_max = uint32_t(g_build_tune.leaf_max);
    *width = uint32_t(g_build_tune.width);
    return LCX_OK;
}

// ---------------------------------------------------------------- queries
// Counter slot of a trace call on `st`: round robin over the live slots, or
// over the graph slots while `st` is being captured.
static uint32_t trace_slot(DeviceState *ds, cudaStream_t st) {
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(st, &cs) != cudaSuccess) {
        (void)cudaGetLastError();  // the legacy stream during another stream's capture: the launch reports it
        cs = cudaStreamCaptureStatusNone;
    }
    if (cs == cudaStreamCaptureStatusActive)
        return kPoolSlots - kGraphSlots + ds->next_graph_slot.fetch_add(1) % kGraphSlots;
    return ds->next_slot.fetch_add(1) % (kPoolSlots - kGraphSlots);
}

// A streamed host-buffer launch's copy-chunk flags and warp marks (TraceParams::stage_*).
struct StageArgs {
    const uint32_t *flags = nullptr;
    uint32_t *marks = nullptr;
    uint32_t gen = 0, shift = 0;
};

static int trace_common(uint64_t accel, const LcxRay *d_rays, uint32_t ray_count, uint32_t mask, LcxTriangleHit *d_hits,
                        uint8_t *d_occ, uint32_t *d_counts, uint32_t layout, void *stream,
                        const float *d_times = nullptr, const StageArgs *stage = nullptr) {
    if (layout > LCX_NODES_QUANT8) return fail(LCX_ERR_INVALID_ARG, "invalid node layout %u", layout);
    std::shared_lock<std::shared_mutex> life(g_life_mtx);  // until the kernel is enqueued
    auto a = find_accel(accel);
    if (!a) return fail(LCX_ERR_INVALID_ARG, "unknown accel handle %llu", (unsigned long long)accel);
    if (ray_count == 0) return LCX_OK;
    if (ray_count > kMaxTraceRays)
        return fail(LCX_ERR_INVALID_ARG, "ray_count %u exceeds %u per call (32-bit ray counter)", ray_count,
                    kMaxTraceRays);
    if (!d_rays || (!d_hits && !d_occ)) return fail(LCX_ERR_INVALID_ARG, "null ray or result buffer");
    if (reinterpret_cast<uintptr_t>(d_rays) % 16 != 0) return fail(LCX_ERR_INVALID_ARG, "rays must be 16-byte aligned");
    if (d_hits && reinterpret_cast<uintptr_t>(d_hits) % 8 != 0)
        return fail(LCX_ERR_INVALID_ARG, "hits must be 8-byte aligned");
    TraceParams p{};
    uint32_t depth_need = 0;
    {
        std::lock_guard<std::mutex> lk(a->mtx);
        if (!a->built) return fail(LCX_ERR_NOT_BUILT, "accel not built");
        uint64_t h = 0;
        bool gone = false;
        if (!meshes_current(a.get(), &h, &gone))
            return fail(LCX_ERR_NOT_BUILT, gone ? "mesh %llu was destroyed; rebuild the accel"
                                                : "mesh %llu was rebuilt after the accel build; rebuild the accel",
                        (unsigned long long)h);
        depth_need = a->depth + a->max_blas_depth + 3;
        if (int(depth_need) > kStackSize)
            return fail(LCX_ERR_DEPTH, "TLAS depth %u + BLAS depth %u exceeds the traversal stack (%d)", a->depth,
                        a->max_blas_depth, kStackSize);
        p.tlas_q = a->qn;
        p.tlas_f = a->fn;
        p.insts = a->recs;
        p.motion = a->has_motion || a->has_curves;
        p.curves = a->has_curves;
    }
    p.times = d_times;
    if (d_times && reinterpret_cast<uintptr_t>(d_times) % 4 != 0)
        return fail(LCX_ERR_INVALID_ARG, "times must be 4-byte aligned");
    DeviceState *ds = nullptr;
    if (int r = current_device_state(&ds)) return r;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    p.pool = ds->pool + 4 * trace_slot(ds, st);
    p.rays = reinterpret_cast<const Ray *>(d_rays);
    p.hits = reinterpret_cast<Hit *>(d_hits);
    p.occluded = d_occ;
    p.counts = d_counts;
    p.ray_count = ray_count;
    p.mask = mask & 0xffu;
    p.refill = g_tune.refill;
    p.postpone = g_tune.postpone;
    p.mode = g_tune.mode;
    p.short_stack = g_tune.short_stack;
    p.max_steps = g_tune.max_steps;
    // regular pushes need at most tlas_depth + blas_depth + 3 entries; postponed
    // triangle groups may use what is left
    p.postpone_sp = kStackSize - int(depth_need);
    if (stage != nullptr) {
        if (p.motion || layout != LCX_NODES_QUANT8 || p.mode != 2 || d_counts != nullptr)
            return fail(LCX_ERR_INVALID_ARG, "a streamed trace needs a static accel, quantised nodes and loop mode 2");
        p.stage_flag = stage->flags;
        p.stage_mark = stage->marks;
        p.stage_gen = stage->gen;
        p.stage_shift = stage->shift;
    }
    ReorderScratch rs;
    const uint32_t rbits = stage != nullptr ? 0u : g_reorder.bits;  // a streamed launch takes the rays in order
    if (rbits != 0 && ray_count >= g_reorder.min_rays) {
        if (int r = reorder_begin(p.rays, ray_count, p.tlas_f, rbits, st, &rs)) return r;
        p.order = rs.order;
    }
    NvtxRange nr(d_occ ? "trace_any" : "trace_closest");
    cudaError_t e = cudaMemsetAsync(p.pool, 0, 4 * sizeof(uint32_t), st);
    if (e == cudaSuccess) e = launch_trace(p, int(layout), d_occ != nullptr, d_counts != nullptr, st);
    const int released = reorder_end(&rs, st);
    if (e != cudaSuccess) return cuda_fail(e, "trace launch");
    return released;
}

int lcx_accel_instance_buffer(uint64_t accel, LcxInstanceBuffer *out) {
    if (!out) return fail(LCX_ERR_INVALID_ARG, "lcx_accel_instance_buffer: out is null");
    auto a = find_accel(accel);
    if (!a) return fail(LCX_ERR_INVALID_ARG, "unknown accel handle %llu", (unsigned long long)accel);
    std::lock_guard<std::mutex> lk(a->mtx);
    if (!a->d_inst || a->inst_count == 0) return fail(LCX_ERR_NOT_BUILT, "accel has no instances");
    out->states = a->d_inst;
    out->count = a->inst_count;
    out->_pad = 0;
    return LCX_OK;
}

int lcx_accel_device_view(uint64_t accel, LcxAccelView *out) {
    if (!out) return fail(LCX_ERR_INVALID_ARG, "lcx_accel_device_view: out is null");
    auto a = find_accel(accel);
    if (!a) return fail(LCX_ERR_INVALID_ARG, "unknown accel handle %llu", (unsigned long long)accel);
    std::lock_guard<std::mutex> lk(a->mtx);
    if (!a->built) return fail(LCX_ERR_NOT_BUILT, "accel not built");
    if (!meshes_current(a.get()))
        return fail(LCX_ERR_NOT_BUILT, "a mesh of the accel was destroyed, rebuilt or refit; rebuild the accel");
    const uint32_t need = a->depth + a->max_blas_depth + 3;
    if (int(need) > kStackSize)
        return fail(LCX_ERR_DEPTH, "TLAS depth %u + BLAS depth %u exceeds the query stack (%d)", a->depth,
                    a->max_blas_depth, kStackSize);
    out->tlas_nodes = a->qn;
    out->instances = a->recs;
    out->stack_need = need;
    out->motion = a->has_motion ? 1u : 0u;
    return LCX_OK;
}

static int trace_jobs(const LcxTraceJob *jobs, const float *const *times, uint32_t count, uint32_t node_layout,
                      void *stream) {
    if (count == 0) return LCX_OK;
    if (!jobs) return fail(LCX_ERR_INVALID_ARG, "lcx_trace_jobs: jobs is null");
    if (node_layout > LCX_NODES_QUANT8) return fail(LCX_ERR_INVALID_ARG, "invalid node layout %u", node_layout);
    std::shared_lock<std::shared_mutex> life(g_life_mtx);  // until the kernels are enqueued
    std::vector<DevJob> groups[2];  // [0] closest, [1] any
    bool curves[2] = {false, false};  // a job of the group traces curves: the curve kernel runs the group
    bool motion[2] = {false, false};  // ... motion: the motion kernel (or the curve kernel) runs it
    uint64_t totals[2] = {0, 0};
    uint32_t depth_need = 0;
    for (uint32_t i = 0; i < count; i++) {
        const LcxTraceJob &j = jobs[i];
        if (j.ray_count == 0) continue;
        if (!j.rays || !j.out) return fail(LCX_ERR_INVALID_ARG, "job %u: null ray or result buffer", i);
        if (reinterpret_cast<uintptr_t>(j.rays) % 16 != 0 || (!j.any && reinterpret_cast<uintptr_t>(j.out) % 8 != 0))
            return fail(LCX_ERR_INVALID_ARG, "job %u: rays must be 16-byte and hits 8-byte aligned", i);
        auto a = find_accel(j.accel);
        if (!a) return fail(LCX_ERR_INVALID_ARG, "job %u: unknown accel handle %llu", i, (unsigned long long)j.accel);
        std::lock_guard<std::mutex> lk(a->mtx);
        if (!a->built) return fail(LCX_ERR_NOT_BUILT, "job %u: accel not built", i);
        if (!meshes_current(a.get()))
            return fail(LCX_ERR_NOT_BUILT, "job %u: a mesh of the accel was destroyed or rebuilt; rebuild the accel",
                        i);
        const float *jt = times ? times[i] : nullptr;
        if (jt && reinterpret_cast<uintptr_t>(jt) % 4 != 0)
            return fail(LCX_ERR_INVALID_ARG, "job %u: times must be 4-byte aligned", i);
        const uint32_t need = a->depth + a->max_blas_depth + 3;
        if (int(need) > kStackSize) return fail(LCX_ERR_DEPTH, "job %u: BVH too deep for the traversal stack", i);
        depth_need = std::max(depth_need, need);
        const int g = j.any ? 1 : 0;
        curves[g] = curves[g] || a->has_curves;
        motion[g] = motion[g] || a->has_motion;
        DevJob d{};
        d.tlas_q = a->qn;
        d.tlas_f = a->fn;
        d.insts = a->recs;
        d.rays = reinterpret_cast<const Ray *>(j.rays);
        d.out = j.out;
        d.first = uint32_t(totals[g]);
        d.count = j.ray_count;
        d.mask = j.mask & 0xffu;
        d.times = jt;
        totals[g] += j.ray_count;
        if (totals[g] > kMaxTraceRays) return fail(LCX_ERR_INVALID_ARG, "lcx_trace_jobs: more than 2^31 rays");
        groups[g].push_back(d);
    }
    DeviceState *ds = nullptr;
    if (int r = current_device_state(&ds)) return r;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    NvtxRange nr("trace_jobs");
    for (int g = 0; g < 2; g++) {
        if (groups[g].empty()) continue;
        ScratchHolder hold(st);
        DevJob *d_jobs = nullptr;
        LCX_CUDA(hold.alloc((void **)&d_jobs, sizeof(DevJob) * groups[g].size()), "job table");
        LCX_CUDA(cudaMemcpyAsync(d_jobs, groups[g].data(), sizeof(DevJob) * groups[g].size(), cudaMemcpyHostToDevice,
                                 st),
                 "job table upload");
        TraceParams p{};
        p.pool = ds->pool + 4 * trace_slot(ds, st);
        p.ray_count = uint32_t(totals[g]);
        p.refill = g_tune.refill;
        p.mode = g_tune.mode == 2 ? 2u : 0u;  // multi-job kernels: mode 2 (quantised nodes) or 0
        p.postpone = p.mode == 2 ? g_tune.postpone : 0u;
        p.max_steps = g_tune.max_steps;
        p.postpone_sp = kStackSize - int(depth_need);
        p.jobs = d_jobs;
        p.job_count = uint32_t(groups[g].size());
        p.motion = curves[g] || motion[g];
        p.curves = curves[g];
        LCX_CUDA(cudaMemsetAsync(p.pool, 0, 4 * sizeof(uint32_t), st), "trace counter reset");
        LCX_CUDA(launch_trace(p, int(node_layout), g == 1, false, st), "multi-job trace launch");
    }
    return LCX_OK;
}

int lcx_trace_jobs(const LcxTraceJob *jobs, uint32_t count, uint32_t node_layout, void *stream) {
    return trace_jobs(jobs, nullptr, count, node_layout, stream);
}

int lcx_trace_jobs_motion(const LcxTraceJob *jobs, const float *const *times, uint32_t count, uint32_t node_layout,
                          void *stream) {
    return trace_jobs(jobs, times, count, node_layout, stream);
}

int lcx_check_trace_errors(void) {
    DeviceState *ds = nullptr;
    if (int r = current_device_state(&ds)) return r;
    LCX_CUDA(cudaDeviceSynchronize(), "cudaDeviceSynchronize");
    std::vector<uint32_t> h(kPoolSlots * 4);
    LCX_CUDA(cudaMemcpy(h.data(), ds->pool, h.size() * sizeof(uint32_t), cudaMemcpyDeviceToHost), "pool readback");
    uint32_t flags = 0;
    if (int r = noalloc_take_errors(&flags)) return r;  // lcx_trace_closest_noalloc's own error word
    for (uint32_t i = 0; i < kPoolSlots; i++) flags |= h[4 * i + 1];
    if (flags) {
        for (uint32_t i = 0; i < kPoolSlots; i++) h[4 * i + 1] = 0;
        LCX_CUDA(cudaMemcpy(ds->pool, h.data(), h.size() * sizeof(uint32_t), cudaMemcpyHostToDevice), "pool reset");
    }
    uint32_t rerr = 0;  // errors of refits that did not synchronise
    LCX_CUDA(cudaMemcpy(&rerr, ds->refit_ctl + kCtlErr, sizeof(uint32_t), cudaMemcpyDeviceToHost), "refit readback");
    if (rerr) {
        LCX_CUDA(cudaMemset(ds->refit_ctl, 0, kCtlWords * sizeof(uint32_t)), "refit error reset");
        if (rerr & kErrTooDeep) return fail(LCX_ERR_DEPTH, "an asynchronous refit met a BVH deeper than expected");
        return fail(LCX_ERR_INVALID_ARG,
                    "an asynchronous refit or reserved rebuild failed (bad index or unquantisable coordinates)");
    }
    if (flags & kTraceErrSteps)
        return fail(LCX_ERR_TIMEOUT, "a ray exceeded the traversal step bound (lcx_set_trace_step_bound; the "
                                     "default bound is reached only on a corrupt BVH)");
    if (flags & kTraceErrStage)
        return fail(LCX_ERR_TIMEOUT, "a streamed host-buffer trace gave up waiting for a copy of its rays");
    if (flags & kTraceErrStack) return fail(LCX_ERR_DEPTH, "a ray overflowed the traversal stack");
    return LCX_OK;
}

int lcx_set_trace_tuning(uint32_t refill, uint32_t postpone, uint32_t mode) {
    if (refill < 1 || refill > 32 || postpone > 32 || mode > 3)
        return fail(LCX_ERR_INVALID_ARG, "tuning out of range (refill 1..32, postpone 0..32, mode 0..3)");
    g_tune.refill = refill;
    g_tune.postpone = postpone;
    g_tune.mode = mode;
    return LCX_OK;
}

int lcx_set_trace_step_bound(uint32_t steps) {
    if (steps > kMaxRaySteps)
        return fail(LCX_ERR_INVALID_ARG, "step bound %u out of range (0 = default %u, 1..%u)", steps, kMaxRaySteps,
                    kMaxRaySteps);
    g_tune.max_steps = steps == 0 ? kMaxRaySteps : steps;
    return LCX_OK;
}

int lcx_get_trace_step_bound(uint32_t *steps) {
    if (!steps) return fail(LCX_ERR_INVALID_ARG, "null output");
    *steps = g_tune.max_steps;
    return LCX_OK;
}

int lcx_set_refit_sync(uint32_t sync) {
    if (sync > 1) return fail(LCX_ERR_INVALID_ARG, "lcx_set_refit_sync: 0 or 1");
    g_refit_sync = sync != 0;
    return LCX_OK;
}

int lcx_set_trace_stack(uint32_t short_entries) {
    if (short_entries != 8 && short_entries != 16 && short_entries != 24)
        return fail(LCX_ERR_INVALID_ARG, "short stack entries must be 8, 16 or 24");
    g_tune.short_stack = short_entries;
    return LCX_OK;
}

int lcx_get_trace_stack(uint32_t *short_entries) {
    if (!short_entries) return fail(LCX_ERR_INVALID_ARG, "null output");
    *short_entries = g_tune.short_stack;
    return LCX_OK;
}

int lcx_set_trace_reorder(uint32_t bits, uint32_t min_rays) {
    if (bits > 9) return fail(LCX_ERR_INVALID_ARG, "reorder bits out of range (0 = off, 1..9)");
    g_reorder.bits = bits;
    g_reorder.min_rays = min_rays;
    return LCX_OK;
}

int lcx_get_trace_reorder(uint32_t *bits, uint32_t *min_rays) {
    if (!bits || !min_rays) return fail(LCX_ERR_INVALID_ARG, "null output");
    *bits = g_reorder.bits;
    *min_rays = g_reorder.min_rays;
    return LCX_OK;
}

int lcx_get_trace_tuning(uint32_t *refill, uint32_t *postpone, uint32_t *mode) {
    if (!refill || !postpone || !mode) return fail(LCX_ERR_INVALID_ARG, "null output");
    *refill = g_tune.refill;
    *postpone = g_tune.postpone;
    *mode = g_tune.mode;
    return LCX_OK;
}

int lcx_trace_closest(uint64_t accel, const LcxRay *d_rays, uint32_t ray_count, uint32_t mask, LcxTriangleHit *d_hits,
                      void *stream) {
    if (!d_hits && ray_count) return fail(LCX_ERR_INVALID_ARG, "hits buffer is null");
    return trace_common(accel, d_rays, ray_count, mask, d_hits, nullptr, nullptr, LCX_NODES_QUANT8, stream);
}

int lcx_trace_any(uint64_t accel, const LcxRay *d_rays, uint32_t ray_count, uint32_t mask, uint8_t *d_occluded,
                  void *stream) {
    if (!d_occluded && ray_count) return fail(LCX_ERR_INVALID_ARG, "occluded buffer is null");
    return trace_common(accel, d_rays, ray_count, mask, nullptr, d_occluded, nullptr, LCX_NODES_QUANT8, stream);
}

// Host-buffer traces: the caller's rays and results live in host memory (the
// reference's CPU backend traces host arrays, accel.rs:449-535).  They stream
// through a ring of device staging slots in chunks; the copy in of chunk i+1,
// the traversal of chunk i and the copy out of chunk i-1 run at once on the
// device's copy-in, trace and copy-out streams.  Everything stays ordered
// after `stream`'s earlier work, and `stream` waits for the last copy out.
#ifndef LCX_HOST_RAMP_SHIFT
#define LCX_HOST_RAMP_SHIFT 3  // the first and last chunks: chunk >> this, doubling up to the chunk
#endif
#ifndef LCX_HOST_RING
#define LCX_HOST_RING 4  // staging slots
#endif
// lcx_set_host_chunk: 8.4M rays at 2.00 / 2.13 / 2.17 / 2.17 Grays/s with 2^20 / 2^21 / 2^22 / 2^23
// (4M rays: 1.80 / 1.85 / 1.97 / 1.93)
uint32_t g_host_chunk = 1u << 22;
std::atomic<uint32_t> g_host_access{LCX_HOST_AUTO};  // lcx_set_host_access

// Whether the device reads host memory through the host's page tables: a
// coherent CPU-GPU link (NVLink-C2C on Grace systems), where a kernel's own
// loads and stores of host memory run at link speed.
bool host_link_coherent(int device) {
    static std::atomic<int> cached[64];  // 0: not asked yet, 1: no, 2: yes
    if (device < 0 || device >= 64) return false;
    int c = cached[device].load(std::memory_order_relaxed);
    if (c == 0) {
        int v = 0;
        if (cudaDeviceGetAttribute(&v, cudaDevAttrPageableMemoryAccessUsesHostPageTables, device) != cudaSuccess) {
            cudaGetLastError();
            v = 0;
        }
        c = v ? 2 : 1;
        cached[device].store(c, std::memory_order_relaxed);
    }
    return c == 2;
}

// The device address of `bytes` bytes of pinned host memory at `p` (both ends
// inside page-locked host allocations), else null.
const void *pinned_device_address(const void *p, size_t bytes) {
    cudaPointerAttributes a{}, b{};
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess || a.type != cudaMemoryTypeHost || !a.devicePointer) {
        cudaGetLastError();
        return nullptr;
    }
    const void *last = static_cast<const char *>(p) + (bytes ? bytes - 1 : 0);
    if (cudaPointerGetAttributes(&b, last) != cudaSuccess || b.type != cudaMemoryTypeHost) {
        cudaGetLastError();
        return nullptr;
    }
    return a.devicePointer;
}
constexpr uint32_t kHostRing = LCX_HOST_RING;

// ---- streamed host-buffer traces: one traversal launch over all the rays of the call.  The rays
// go to device memory in copy chunks of 2^shift rays on the copy-in stream, each followed by a
// stream memory write of the call's generation to the chunk's flag; the kernel takes a window of
// rays once its chunk's flag holds the generation (a bounded wait: LCX_ERR_TIMEOUT past it).
// Each warp publishes, in mapped pinned memory, a ray id below which all the rays it took have
// their results stored; this thread watches the minimum over the warps and starts each chunk's
// copy out once it has passed the chunk.  Nothing on the device waits for anything the kernel
// produces, and the copy-in stream has no kernel on it, so the traversal's wait for a chunk
// ends as soon as the copy engine has moved it.  Against the chunked launches of the staged
// path (a persistent launch per chunk, each with its own ramp and tail), the traversal runs
// as one launch.
using StreamWriteValueFn = CUresult(CUDAAPI *)(CUstream, CUdeviceptr, cuuint32_t, unsigned int);
StreamWriteValueFn g_write_value = nullptr;
constexpr uint32_t kStageMarkCap = 16384;  // warps of a streamed launch (persistent grid)

// Sets up the device's streamed-trace state once (under ds->stage_mtx); false: not available.
bool stage_setup(DeviceState *ds) {
    if (ds->stage_state != 0) return ds->stage_state == 1;
    ds->stage_state = 2;
    if (g_write_value == nullptr) {
        void *fn = nullptr;
        cudaDriverEntryPointQueryResult q{};
        if (cudaGetDriverEntryPointByVersion("cuStreamWriteValue32", &fn, 12000, cudaEnableDefault, &q) !=
                cudaSuccess ||
            q != cudaDriverEntryPointSuccess || fn == nullptr) {
            cudaGetLastError();
            return false;
        }
        g_write_value = reinterpret_cast<StreamWriteValueFn>(fn);
    }
    if (cudaStreamCreateWithFlags(&ds->stage_in, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&ds->stage_out, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&ds->stage_trace, cudaStreamNonBlocking) != cudaSuccess ||
        cudaMalloc(&ds->stage_flags, sizeof(uint32_t) * (kStageMaxChunks + 1)) != cudaSuccess ||
        cudaMemset(ds->stage_flags, 0, sizeof(uint32_t) * (kStageMaxChunks + 1)) != cudaSuccess ||
        cudaHostAlloc(&ds->stage_marks, sizeof(uint32_t) * kStageMarkCap, cudaHostAllocMapped) != cudaSuccess ||
        cudaHostGetDevicePointer(reinterpret_cast<void **>(&ds->stage_marks_dev), ds->stage_marks, 0) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    // the stream memory write, once on the spare flag word
    if (g_write_value(reinterpret_cast<CUstream>(ds->stage_in),
                      reinterpret_cast<CUdeviceptr>(ds->stage_flags + kStageMaxChunks), 1u, 0) != CUDA_SUCCESS ||
        cudaStreamSynchronize(ds->stage_in) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    ds->stage_state = 1;
    return true;
}

// Whether launches run one at a time to completion (CUDA_LAUNCH_BLOCKING, or an Nsight tool in
// the process -- Nsight Compute sets NV_NSIGHT_INJECTION_* and NV_COMPUTE_PROFILER_PERFWORKS_DIR
// in its target, other tools CUDA_INJECTION64_PATH -- which serialise them): a streamed launch
// would then wait for copies that are enqueued only after its launch returns, until its bound
// ran out.
bool launches_serialized() {
    const char *b = getenv("CUDA_LAUNCH_BLOCKING");
    if (b != nullptr && b[0] == '1') return true;
    for (const char *v : {"CUDA_INJECTION64_PATH", "NV_NSIGHT_INJECTION_TRANSPORT_TYPE", "NV_COMPUTE_PROFILER_PERFWORKS_DIR"}) {
        const char *e = getenv(v);
        if (e != nullptr && e[0] != 0) return true;
    }
    return false;
}

// Whether a host-buffer trace of this accel can run streamed (a static accel, quantised nodes,
// loop mode 2, pinned buffers, launches not serialised); the launch checks the accel again.
bool stream_eligible(uint64_t accel, uint32_t layout, const void *h_rays, size_t ray_bytes, const void *h_out,
                     size_t out_bytes) {
    if (layout != LCX_NODES_QUANT8 || g_tune.mode != 2 || launches_serialized()) return false;
    {
        auto a = find_accel(accel);
        if (!a) return false;
        std::lock_guard<std::mutex> lk(a->mtx);
        if (!a->built || a->has_motion || a->has_curves) return false;
    }
    return pinned_device_address(h_rays, ray_bytes) != nullptr && pinned_device_address(h_out, out_bytes) != nullptr;
}

constexpr int kStreamFallback = -1000;  // not taken: the caller runs the staged path

static int trace_host_streamed(DeviceState *ds, uint64_t accel, const LcxRay *h_rays, uint32_t ray_count,
                               uint32_t mask, LcxTriangleHit *h_hits, uint8_t *h_occ, uint32_t layout,
                               cudaStream_t st) {
    std::unique_lock<std::mutex> lk(ds->stage_mtx, std::try_to_lock);
    if (!lk.owns_lock() || !stage_setup(ds)) return kStreamFallback;
    const uint32_t warps = stream_launch_warps(ray_count, h_occ != nullptr);
    if (warps == 0 || warps > kStageMarkCap) return kStreamFallback;
    uint32_t shift = 17;  // chunks of 2^17 rays (4 MiB), at most kStageMaxChunks of them
    while (((uint64_t(ray_count) + (1ull << shift) - 1) >> shift) > kStageMaxChunks) shift++;
    const uint32_t chunks = uint32_t((uint64_t(ray_count) + (1ull << shift) - 1) >> shift);
    const size_t rec = h_hits ? sizeof(LcxTriangleHit) : 1;
    const size_t in_bytes = (size_t(ray_count) * sizeof(LcxRay) + 255) & ~size_t(255);
    cudaMemPool_t pool;
    if (int r = scratch_pool(&pool)) return r;
    void *mem = nullptr;
    LCX_CUDA(cudaMallocFromPoolAsync(&mem, in_bytes + size_t(ray_count) * rec, pool, st), "streamed trace buffers");
    char *d_in = static_cast<char *>(mem), *d_out = d_in + in_bytes;
    if (++ds->stage_gen == 0) ds->stage_gen = 1;
    const uint32_t gen = ds->stage_gen;
    for (uint32_t w = 0; w < warps; w++) ds->stage_marks[w] = 0u;  // the last call's kernel has exited
    std::atomic_thread_fence(std::memory_order_seq_cst);
    cudaEvent_t ev0 = nullptr, ev_done = nullptr;
    cudaError_t e = cudaEventCreateWithFlags(&ev0, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ev_done, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventRecord(ev0, st);
    cudaStream_t ts = ds->stage_trace;
    for (cudaStream_t x : {ds->stage_in, ds->stage_out, ts})
        if (e == cudaSuccess) e = cudaStreamWaitEvent(x, ev0, 0);
    auto chunk_rays = [&](uint32_t c) {
        return std::min<uint64_t>(1ull << shift, uint64_t(ray_count) - (uint64_t(c) << shift));
    };
    auto copy_in = [&](uint32_t c) {
        const uint64_t off = uint64_t(c) << shift;
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(d_in + off * sizeof(LcxRay), h_rays + off, chunk_rays(c) * sizeof(LcxRay),
                                cudaMemcpyHostToDevice, ds->stage_in);
        if (e == cudaSuccess &&
            g_write_value(reinterpret_cast<CUstream>(ds->stage_in), reinterpret_cast<CUdeviceptr>(ds->stage_flags + c),
                          gen, 0) != CUDA_SUCCESS)
            e = cudaErrorUnknown;
    };
    copy_in(0);
    int status = LCX_OK;
    bool launched = false;
    if (e == cudaSuccess) {
        StageArgs sa;
        sa.flags = ds->stage_flags;
        sa.marks = ds->stage_marks_dev;
        sa.gen = gen;
        sa.shift = shift;
        status = trace_common(accel, reinterpret_cast<const LcxRay *>(d_in), ray_count, mask,
                              h_hits ? reinterpret_cast<LcxTriangleHit *>(d_out) : nullptr,
                              h_hits ? nullptr : reinterpret_cast<uint8_t *>(d_out), nullptr, layout, ts, nullptr,
                              &sa);
        launched = status == LCX_OK;
        if (launched) e = cudaEventRecord(ev_done, ts);
    }
    // the other chunks' copies in; the kernel takes each chunk once its flag is written
    for (uint32_t c = 1; c < chunks && launched; c++) copy_in(c);
    if (launched && e == cudaSuccess) {
        // copies out as the warps' marks pass the chunks (a kernel that ended has marked every
        // warp done, its error aside)
        uint32_t next = 0;
        const auto t0 = std::chrono::steady_clock::now();
        while (next < chunks && e == cudaSuccess) {
            uint32_t m = 0xffffffffu;
            for (uint32_t w = 0; w < warps; w++) {
                const uint32_t v = reinterpret_cast<volatile const uint32_t *>(ds->stage_marks)[w];
                m = std::min(m, v);
            }
            std::atomic_thread_fence(std::memory_order_acquire);
            bool moved = false;
            while (next < chunks && uint64_t(m) >= (uint64_t(next) << shift) + chunk_rays(next)) {
                const uint64_t off = uint64_t(next) << shift;
                char *dst = h_hits ? reinterpret_cast<char *>(h_hits) : reinterpret_cast<char *>(h_occ);
                e = cudaMemcpyAsync(dst + off * rec, d_out + off * rec, chunk_rays(next) * rec, cudaMemcpyDeviceToHost,
                                    ds->stage_out);
                next++;
                moved = true;
                if (e != cudaSuccess) break;
            }
            if (next >= chunks || moved) continue;
            const cudaError_t q = cudaEventQuery(ev_done);
            if (q != cudaSuccess && q != cudaErrorNotReady) {
                e = q;  // a failed launch: its marks may never come
                break;
            }
            if (q == cudaSuccess) {
                // ended: re-read the marks once (the last stores are visible now)
                bool all = true;
                for (uint32_t w = 0; w < warps; w++)
                    all = all && reinterpret_cast<volatile const uint32_t *>(ds->stage_marks)[w] == 0xffffffffu;
                if (!all) {
                    e = cudaErrorUnknown;
                    break;
                }
                continue;
            }
            if (std::chrono::steady_clock::now() - t0 > std::chrono::seconds(60)) {
                e = cudaErrorLaunchTimeout;  // the kernel's own waits end long before this
                break;
            }
            std::this_thread::yield();
        }
    }
    // the kernel has exited before the next streamed call resets the marks
    if (launched) cudaEventSynchronize(ev_done);
    // `stream` waits for everything enqueued above; the buffers return to the pool in its order
    const cudaError_t first = e;
    for (cudaStream_t x : {ds->stage_in, ds->stage_out, ts}) {
        cudaEvent_t tail = nullptr;
        if (cudaEventCreateWithFlags(&tail, cudaEventDisableTiming) == cudaSuccess) {
            cudaEventRecord(tail, x);
            cudaStreamWaitEvent(st, tail, 0);
            cudaEventDestroy(tail);
        }
    }
    cudaFreeAsync(mem, st);
    if (ev0) cudaEventDestroy(ev0);
    if (ev_done) cudaEventDestroy(ev_done);
    if (status != LCX_OK) return status;
    if (first != cudaSuccess) return cuda_fail(first, "streamed host-buffer trace");
    return LCX_OK;
}

static int trace_host(uint64_t accel, const LcxRay *h_rays, uint32_t ray_count, uint32_t mask, LcxTriangleHit *h_hits,
                      uint8_t *h_occ, uint32_t layout, void *stream) {
    if (ray_count == 0 || !h_rays || (!h_hits && !h_occ))  // validation (and the empty call) as the device form
        return trace_common(accel, reinterpret_cast<const LcxRay *>(h_rays), ray_count, mask, h_hits, h_occ, nullptr,
                            layout, stream);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (capturing(st)) return fail(LCX_ERR_INVALID_ARG, "host-buffer traces cannot be captured in a CUDA graph");
    NvtxRange nr(h_occ ? "trace_any_host" : "trace_closest_host");
    DeviceState *ds = nullptr;
    if (int r = current_device_state(&ds)) return r;
    // direct access: the traversal reads the rays from and writes the results to the pinned host
    // buffers itself, with no staging and no copies.  On GB300 over NVLink-C2C it traced 8.4M rays
    // at 1.11-1.84 Grays/s from box to box, against 2.13-2.18 through staged 2^21..2^22-ray chunks
    // (2.62 on device buffers; 4M rays: 1.11-1.78 against 1.85-1.98; 1M rays: 1.05-1.46 against
    // 1.29-1.30), so the automatic choice takes it only for calls of at most kDirectAutoRays rays,
    // where the staging's fixed costs weigh most.
    constexpr uint32_t kDirectAutoRays = 1u << 18;
    const uint32_t access = g_host_access.load();
    if (access == LCX_HOST_DIRECT ||
        (access == LCX_HOST_AUTO && ray_count <= kDirectAutoRays && host_link_coherent(ds->device))) {
        const size_t out_bytes = size_t(ray_count) * (h_hits ? sizeof(LcxTriangleHit) : 1);
        const void *dr = pinned_device_address(h_rays, size_t(ray_count) * sizeof(LcxRay));
        const void *dout = pinned_device_address(h_hits ? static_cast<const void *>(h_hits) : h_occ, out_bytes);
        const bool aligned = reinterpret_cast<uintptr_t>(dr) % 16 == 0 &&
                             (!h_hits || reinterpret_cast<uintptr_t>(dout) % 8 == 0);  // else staged, which takes any
        if (dr && dout && aligned)
            return trace_common(accel, static_cast<const LcxRay *>(dr), ray_count, mask,
                                h_hits ? static_cast<LcxTriangleHit *>(const_cast<void *>(dout)) : nullptr,
                                h_hits ? nullptr : static_cast<uint8_t *>(const_cast<void *>(dout)), nullptr, layout,
                                stream);
    }
    // streamed (explicitly, or automatically above the direct path's size) where the call allows it
    if (access == LCX_HOST_STREAMED || access == LCX_HOST_AUTO) {
        const size_t out_bytes = size_t(ray_count) * (h_hits ? sizeof(LcxTriangleHit) : 1);
        if (stream_eligible(accel, layout, h_rays, size_t(ray_count) * sizeof(LcxRay),
                            h_hits ? static_cast<const void *>(h_hits) : h_occ, out_bytes)) {
            const int r = trace_host_streamed(ds, accel, h_rays, ray_count, mask, h_hits, h_occ, layout, st);
            if (r != kStreamFallback) return r;
        }
    }
    // staged: chunk sizes: a short ramp up (the first copy in is not overlapped), full
    // chunks, and a ramp down (nor is the last copy out)
    const uint32_t chunk = g_host_chunk;
    std::vector<uint64_t> offs, cnts;
    {
        uint64_t left = ray_count, off = 0;
        auto take = [&](uint64_t c) {
            c = std::min(c, left);
            if (!c) return;
            offs.push_back(off);
            cnts.push_back(c);
            off += c;
            left -= c;
        };
        const uint64_t ramp0 = std::max<uint64_t>(chunk >> LCX_HOST_RAMP_SHIFT, 1u << 14);
        for (uint64_t c = ramp0; c < chunk && left; c <<= 1) take(c);
        uint64_t down = 0;
        for (uint64_t c = chunk >> 1; c >= ramp0; c >>= 1) down += c;
        while (left > chunk + down) take(chunk);
        if (left > down) take(left - down);
        for (uint64_t c = chunk >> 1; c >= ramp0 && left; c >>= 1) take(c);
        take(left);
    }
    const uint32_t nchunks = uint32_t(cnts.size());
    const uint32_t ring = std::min(kHostRing, nchunks);
    const size_t out_rec = h_hits ? sizeof(LcxTriangleHit) : 1;
    const size_t in_bytes = (size_t(chunk) * sizeof(LcxRay) + 255) & ~size_t(255);
    const size_t out_bytes = (size_t(chunk) * out_rec + 255) & ~size_t(255);
    cudaMemPool_t pool;
    if (int r = scratch_pool(&pool)) return r;
    void *mem = nullptr;
    LCX_CUDA(cudaMallocFromPoolAsync(&mem, ring * (in_bytes + out_bytes), pool, st), "host trace staging");
    char *in_base = static_cast<char *>(mem), *out_base = in_base + ring * in_bytes;
    std::vector<cudaEvent_t> ev(3 * size_t(nchunks) + 1, nullptr);  // [start, in_i, traced_i, out_i]
    cudaError_t e = cudaSuccess;
    for (auto &x : ev)
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&x, cudaEventDisableTiming);
    auto ev_in = [&](uint32_t i) { return ev[1 + 3 * size_t(i)]; };
    auto ev_traced = [&](uint32_t i) { return ev[2 + 3 * size_t(i)]; };
    auto ev_out = [&](uint32_t i) { return ev[3 + 3 * size_t(i)]; };
    auto count_of = [&](uint32_t i) { return cnts[i]; };
    auto copy_in = [&](uint32_t i) {
        if (i >= ring) e = cudaStreamWaitEvent(ds->io_in, ev_out(i - ring), 0);  // the slot's last copy out is done
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(in_base + (i % ring) * in_bytes, h_rays + offs[i], count_of(i) * sizeof(LcxRay),
                                cudaMemcpyHostToDevice, ds->io_in);
        if (e == cudaSuccess) e = cudaEventRecord(ev_in(i), ds->io_in);
    };
    if (e == cudaSuccess) e = cudaEventRecord(ev[0], st);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(ds->io_in, ev[0], 0);
    if (e == cudaSuccess) copy_in(0);
    int status = LCX_OK;
    for (uint32_t i = 0; i < nchunks && e == cudaSuccess && status == LCX_OK; i++) {
        if (i + 1 < nchunks) copy_in(i + 1);
        if (e != cudaSuccess) break;
        cudaStream_t ts = ds->io_trace[i & 1];
        e = cudaStreamWaitEvent(ts, ev_in(i), 0);
        if (e != cudaSuccess) break;
        char *out = out_base + (i % ring) * out_bytes;
        status = trace_common(accel, reinterpret_cast<const LcxRay *>(in_base + (i % ring) * in_bytes),
                              uint32_t(count_of(i)), mask, h_hits ? reinterpret_cast<LcxTriangleHit *>(out) : nullptr,
                              h_hits ? nullptr : reinterpret_cast<uint8_t *>(out), nullptr, layout, ts);
        if (status != LCX_OK) break;
        e = cudaEventRecord(ev_traced(i), ts);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(ds->io_out, ev_traced(i), 0);
        char *dst = h_hits ? reinterpret_cast<char *>(h_hits) + offs[i] * sizeof(LcxTriangleHit)
                           : reinterpret_cast<char *>(h_occ) + offs[i];
        if (e == cudaSuccess) e = cudaMemcpyAsync(dst, out, count_of(i) * out_rec, cudaMemcpyDeviceToHost, ds->io_out);
        if (e == cudaSuccess) e = cudaEventRecord(ev_out(i), ds->io_out);
    }
    // `stream` waits for everything enqueued above (all of it, also after an
    // error), then the staging returns to the pool in its order
    const cudaError_t first = e;
    cudaStream_t all[4] = {ds->io_in, ds->io_out, ds->io_trace[0], ds->io_trace[1]};
    for (cudaStream_t x : all) {
        cudaEvent_t tail = nullptr;
        if (cudaEventCreateWithFlags(&tail, cudaEventDisableTiming) == cudaSuccess) {
            cudaEventRecord(tail, x);
            cudaStreamWaitEvent(st, tail, 0);
            cudaEventDestroy(tail);
        }
    }
    cudaFreeAsync(mem, st);
    for (auto &x : ev)
        if (x) cudaEventDestroy(x);  // released once completed
    if (status != LCX_OK) return status;
    if (first != cudaSuccess) return cuda_fail(first, "host-buffer trace");
    return LCX_OK;
}

int lcx_trace_closest_motion(uint64_t accel, const LcxRay *d_rays, const float *d_times, uint32_t ray_count,
                             uint32_t mask, LcxTriangleHit *d_hits, uint32_t node_layout, void *stream) {
    if (!d_hits && ray_count) return fail(LCX_ERR_INVALID_ARG, "hits buffer is null");
    return trace_common(accel, d_rays, ray_count, mask, d_hits, nullptr, nullptr, node_layout, stream, d_times);
}

int lcx_trace_any_motion(uint64_t accel, const LcxRay *d_rays, const float *d_times, uint32_t ray_count, uint32_t mask,
                         uint8_t *d_occluded, uint32_t node_layout, void *stream) {
    if (!d_occluded && ray_count) return fail(LCX_ERR_INVALID_ARG, "occluded buffer is null");
    return trace_common(accel, d_rays, ray_count, mask, nullptr, d_occluded, nullptr, node_layout, stream, d_times);
}

int lcx_motion_instance_create(uint64_t mesh, const LcxMotionOption *option, uint64_t *out_handle) {
    if (!option || !out_handle) return fail(LCX_ERR_INVALID_ARG, "lcx_motion_instance_create: null argument");
    const LcxMotionOption &o = *option;
    if (o.keyframe_count < 2) return fail(LCX_ERR_INVALID_ARG, "a motion instance needs at least 2 keyframes");
    if (o.keyframe_count > (1u << 16)) return fail(LCX_ERR_INVALID_ARG, "too many keyframes (%u)", o.keyframe_count);
    if (!(o.time_end > o.time_start) || !std::isfinite(o.time_start) || !std::isfinite(o.time_end))
        return fail(LCX_ERR_INVALID_ARG, "motion time range must be finite with time_end > time_start");
    if (o.mode != LCX_MOTION_MATRIX && o.mode != LCX_MOTION_SRT)
        return fail(LCX_ERR_INVALID_ARG, "motion mode must be LCX_MOTION_MATRIX or LCX_MOTION_SRT");
    auto m = find_mesh(mesh);
    if (!m) return fail(LCX_ERR_INVALID_ARG, "lcx_motion_instance_create: unknown mesh handle %llu",
                        (unsigned long long)mesh);
    if (m->kind == kSegAabbs) return fail(LCX_ERR_INVALID_ARG, "motion instances of procedural primitives are not supported");
    auto mo = std::make_shared<MotionObj>();
    mo->child = mesh;
    mo->opt = o;
    const size_t per = o.mode == LCX_MOTION_SRT ? 16 : 12;
    mo->keys.assign(size_t(o.keyframe_count) * per, 0.0f);
    for (uint32_t k = 0; k < o.keyframe_count; k++) {  // identity keyframes
        float *v = &mo->keys[per * k];
        if (per == 16) {  // pivot 0, quaternion (0,0,0,1), scale 1, shear 0, translation 0
            v[6] = 1.0f;
            v[7] = v[8] = v[9] = 1.0f;
        } else {
            v[0] = v[5] = v[10] = 1.0f;
        }
    }
    LCX_CUDA(cudaMalloc(&mo->mem, sizeof(MotionDesc) + sizeof(float) * mo->keys.size()), "cudaMalloc(motion)");
    mo->d_md = static_cast<MotionDesc *>(mo->mem);
    const uint64_t h = g_next_handle.fetch_add(1);
    {
        std::lock_guard<std::mutex> lk(g_reg_mtx);
        g_motions.emplace(h, std::move(mo));
    }
    *out_handle = h;
    return LCX_OK;
}

int lcx_motion_instance_destroy(uint64_t handle) {
    std::shared_ptr<MotionObj> mo;
    {
        std::unique_lock<std::shared_mutex> life(g_life_mtx);  // traces that found it have enqueued
        std::lock_guard<std::mutex> lk(g_reg_mtx);
        auto it = g_motions.find(handle);
        if (it == g_motions.end()) return fail(LCX_ERR_INVALID_ARG, "lcx_motion_instance_destroy: unknown handle %llu",
                                               (unsigned long long)handle);
        mo = it->second;
        g_motions.erase(it);
        mo->alive.store(false);
        bump_mesh_epoch();
    }
    // accels that instance it keep its memory until they let go of it
    cudaDeviceSynchronize();
    mo.reset();
    return LCX_OK;
}

int lcx_motion_instance_set_keyframes(uint64_t handle, const float *matrices, uint32_t count) {
    auto mo = find_motion(handle);
    if (!mo) return fail(LCX_ERR_INVALID_ARG, "unknown motion instance handle %llu", (unsigned long long)handle);
    if (!matrices || count != mo->opt.keyframe_count)
        return fail(LCX_ERR_INVALID_ARG, "expected %u keyframes", mo->opt.keyframe_count);
    std::lock_guard<std::mutex> lk(mo->mtx);
    mo->keys.assign(matrices, matrices + size_t(count) * (mo->opt.mode == LCX_MOTION_SRT ? 16 : 12));
    return LCX_OK;
}

int lcx_motion_instance_build(uint64_t handle, void *stream) {
    auto mo = find_motion(handle);
    if (!mo) return fail(LCX_ERR_INVALID_ARG, "unknown motion instance handle %llu", (unsigned long long)handle);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (capturing(st)) return fail(LCX_ERR_INVALID_ARG, "a motion instance build cannot be captured (host keyframes)");
    std::lock_guard<std::mutex> lk(mo->mtx);
    MotionDesc md{};
    md.keys = reinterpret_cast<const float *>(reinterpret_cast<char *>(mo->mem) + sizeof(MotionDesc));
    md.count = mo->opt.keyframe_count;
    md.t0 = mo->opt.time_start;
    md.t1 = mo->opt.time_end;
    md.flags = (mo->opt.vanish_start ? 1u : 0u) | (mo->opt.vanish_end ? 2u : 0u) |
               (mo->opt.mode == LCX_MOTION_SRT ? 4u : 0u);
    // pageable sources: the calls return once the data has been staged
    LCX_CUDA(cudaMemcpyAsync(mo->mem, &md, sizeof(md), cudaMemcpyHostToDevice, st), "motion upload");
    LCX_CUDA(cudaMemcpyAsync(const_cast<float *>(md.keys), mo->keys.data(), sizeof(float) * mo->keys.size(),
                             cudaMemcpyHostToDevice, st),
             "motion upload");
    mo->built = true;
    mo->generation++;  // accels over it must be built again (their boxes bound the keyframes)
    bump_mesh_epoch();
    return LCX_OK;
}

int lcx_trace_closest_host(uint64_t accel, const LcxRay *h_rays, uint32_t ray_count, uint32_t mask,
                           LcxTriangleHit *h_hits, uint32_t node_layout, void *stream) {
    if (!h_hits && ray_count) return fail(LCX_ERR_INVALID_ARG, "hits buffer is null");
    return trace_host(accel, h_rays, ray_count, mask, h_hits, nullptr, node_layout, stream);
}

int lcx_trace_any_host(uint64_t accel, const LcxRay *h_rays, uint32_t ray_count, uint32_t mask, uint8_t *h_occluded,
                       uint32_t node_layout, void *stream) {
    if (!h_occluded && ray_count) return fail(LCX_ERR_INVALID_ARG, "occluded buffer is null");
    return trace_host(accel, h_rays, ray_count, mask, nullptr, h_occluded, node_layout, stream);
}

int lcx_release_scratch(void) {
    cudaMemPool_t pool;
    if (int r = scratch_pool(&pool)) return r;
    LCX_CUDA(cudaDeviceSynchronize(), "cudaDeviceSynchronize");
    LCX_CUDA(cudaMemPoolTrimTo(pool, 0), "cudaMemPoolTrimTo");
    return LCX_OK;
}

int lcx_set_host_access(uint32_t mode) {
    if (mode > LCX_HOST_STREAMED) return fail(LCX_ERR_INVALID_ARG, "invalid host access mode %u", mode);
    g_host_access = mode;
    return LCX_OK;
}

int lcx_get_host_access(uint32_t *mode, uint32_t *coherent_link) {
    DeviceState *ds = nullptr;
    if (int r = current_device_state(&ds)) return r;
    if (mode) *mode = g_host_access;
    if (coherent_link) *coherent_link = host_link_coherent(ds->device) ? 1u : 0u;
    return LCX_OK;
}

int lcx_set_host_chunk(uint32_t rays) {
    if (rays < (1u << 14) || rays > (1u << 26))
        return fail(LCX_ERR_INVALID_ARG, "host trace chunk must be 2^14..2^26 rays");
    g_host_chunk = rays;
    return LCX_OK;
}

int lcx_trace_closest_ex(uint64_t accel, const LcxRay *d_rays, uint32_t ray_count, uint32_t mask,
                         LcxTriangleHit *d_hits, uint32_t node_layout, void *stream) {
    if (!d_hits && ray_count) return fail(LCX_ERR_INVALID_ARG, "hits buffer is null");
    return trace_common(accel, d_rays, ray_count, mask, d_hits, nullptr, nullptr, node_layout, stream);
}

int lcx_trace_any_ex(uint64_t accel, const LcxRay *d_rays, uint32_t ray_count, uint32_t mask, uint8_t *d_occluded,
                     uint32_t node_layout, void *stream) {
    if (!d_occluded && ray_count) return fail(LCX_ERR_INVALID_ARG, "occluded buffer is null");
    return trace_common(accel, d_rays, ray_count, mask, nullptr, d_occluded, nullptr, node_layout, stream);
}

int lcx_trace_closest_counts(uint64_t accel, const LcxRay *d_rays, uint32_t ray_count, uint32_t mask,
                             LcxTriangleHit *d_hits, uint32_t *d_counts, uint32_t node_layout, void *stream) {
    if ((!d_hits || !d_counts) && ray_count) return fail(LCX_ERR_INVALID_ARG, "hits or counts buffer is null");
    return trace_common(accel, d_rays, ray_count, mask, d_hits, nullptr, d_counts, node_layout, stream);
}

}  // extern "C"
