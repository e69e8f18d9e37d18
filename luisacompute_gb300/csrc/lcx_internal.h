// lcx_internal.h — host-side interface between the C ABI layer (capi.cu) and
// the kernel translation units (build.cu, traverse.cu, sort.cu).
#pragma once

#include <shared_mutex>
#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

#include <nvtx3/nvToolsExt.h>

#include "lcx_accel.h"
#include "lcx/bvh_device.cuh"  // device-side layouts and arithmetic, shared with user kernels

namespace lcx {

// NVTX range over a build phase or a trace call, in the library's own domain
// "lcx_accel" (header-only NVTX v3: without a profiler attached a push / pop
// costs a function-pointer check).  The names are the entry points and phases:
// nsys / ncu --nvtx show where a build's or a frame's time goes, as the
// reference's named OptiX builds do (src/backends/cuda/cuda_accel.cpp:28,68).
struct NvtxRange {
    explicit NvtxRange(const char *name) {
        nvtxEventAttributes_t a{};
        a.version = NVTX_VERSION;
        a.size = NVTX_EVENT_ATTRIB_STRUCT_SIZE;
        a.messageType = NVTX_MESSAGE_TYPE_ASCII;
        a.message.ascii = name;
        nvtxDomainRangePushEx(domain(), &a);
    }
    ~NvtxRange() { nvtxDomainRangePop(domain()); }
    NvtxRange(const NvtxRange &) = delete;
    NvtxRange &operator=(const NvtxRange &) = delete;
    static nvtxDomainHandle_t domain() {
        static nvtxDomainHandle_t d = nvtxDomainCreateA("lcx_accel");
        return d;
    }
};

// One BVH of a build: a mesh's triangles (BLAS) or a TLAS's instances.
struct SegInput {
    const unsigned char *vbase;  // vertex buffer + offset (BLAS)
    uint64_t vstride;
    const unsigned char *tbase;  // triangle buffer + offset (BLAS)
    uint32_t vcount;
    uint32_t item_offset;        // first item of this segment among all items of the build
    uint32_t item_count;
    uint32_t kind;               // low byte: kSegTriangles (vbase, tbase) or kSegAabbs (vbase: 24-byte AABBs)
                                 // or kSegCurves (vbase: Bezier points, cone offsets and metas of vcount
                                 // segments; tbase: u32 segment per cone; bits 16+: keyframes; vstride:
                                 // keyframed cones' balls; see build.cu);
                                 // bits 8+: triangles: vertex-motion keyframes (vbase holds them back to back,
                                 // vcount each); curves: the basis (kCurve*)
    BlasDesc *desc;              // BLAS descriptor the emit fills in (null for a TLAS)
};
enum : uint32_t { kSegTriangles = 0, kSegAabbs = 1, kSegCurves = 2 };
static_assert(sizeof(SegInput) == 48, "SegInput is 48 B");

// Per-segment control words.
enum : int {
    kSegCenLo = 0,  // 3 ordered-uint words
    kSegCenHi = 3,  // 3 ordered-uint words
    kSegRoot = 6,
    kSegItems = 7,
    kSegNodes = 8,
    kSegDepth = 9,
    kSegErr = 10,
    kSegRad2 = 11,  // max squared distance of an item box corner from the root box centre (float bits)
    kSegWords = 12,
};

// Global control words.
enum : int {
    kCtlWideCount = 0,
    kCtlDepth = 1,
    kCtlErr = 2,
    kCtlLevel = 4,  // kMaxLevels + 1 words
    kCtlWords = 4 + kMaxLevels + 4,
};

enum : uint32_t {
    kErrBadIndex = 1u,
    kErrTooDeep = 2u,
    kErrQuant = 4u,
};

struct BuildParams {
    int leaf_max = 2;        // items per leaf slot, 1..3
    int width = 8;           // children per wide node, 2..8
    uint32_t size_bits = 0;  // extended-Morton size-class bits (TLAS builds)
    uint32_t cube = 1;       // normalise centroids by the largest extent on every axis (else per axis)
    float split = 0.0f;      // triangle splitting: extra references, as a fraction of the triangles (0 = off)
    uint32_t fill = 0;       // BLAS collapse: split leaf slots into finer ones while slots are free
    uint32_t tlas_sah = 0;   // TLAS: a binned-SAH binary tree instead of the LBVH
    uint32_t blas_sah = 0;   // BLAS: a binned-SAH binary tree instead of the LBVH (never in a capturable rebuild)
    uint32_t dp = 0;         // collapse by the dynamic program over the binary tree (else greedy)
    float dp_prim = 0.3f;    // the dynamic program's cost of an item test against a node test of 1
};

// Per-build device scratch, sized for n items in nseg segments.
struct BuildScratch {
    uint32_t n = 0, nseg = 0;
    uint32_t axis_bits = 21, seg_bits = 0;  // Morton bits per axis, segment-id bits above them
    uint32_t queue_len = 0;
    const SegInput *segs = nullptr;  // nseg
    uint32_t *segctl = nullptr;      // nseg * kSegWords
    double *bin_sah = nullptr;       // 2 nseg: binary-tree SAH sums and root areas
    float4 *box_lo = nullptr;        // n item boxes
    float4 *box_hi = nullptr;
    unsigned long long *keys = nullptr;  // n keys
    unsigned long long *keys_sorted = nullptr;
    uint32_t *vals = nullptr;  // n item ids
    uint32_t *vals_sorted = nullptr;
    uint32_t *bin_child = nullptr;  // 2 n
    float4 *bin_lo = nullptr;       // n (w = count bits)
    float4 *bin_hi = nullptr;       // n (w = first bits)
    int32_t *other = nullptr;       // n
    uint32_t *desc = nullptr;       // queue_len * 12 words
    uint2 *queue = nullptr;         // 2 queue_len
    float *w2o = nullptr;           // TLAS: 12 n
    uint32_t *ctl = nullptr;        // kCtlWords
    void *sort_tmp = nullptr;
    size_t sort_tmp_bytes = 0;
    const uint32_t *ref_prim = nullptr;  // split builds: triangle (local index) of each item (reference)
    float *dp_cost = nullptr;            // collapse by dynamic program: 8 costs per binary node (else null)
};

size_t sort_temp_bytes(uint32_t n);
cudaError_t sort_pairs(void *tmp, size_t tmp_bytes, const unsigned long long *kin, unsigned long long *kout,
                       const uint32_t *vin, uint32_t *vout, uint32_t n, uint32_t end_bit, cudaStream_t s);

// Morton bits per axis for nseg segments; *seg_bits receives the bits of the segment id.
uint32_t morton_axis_bits(uint32_t nseg, uint32_t *seg_bits);

// Phase 1: item boxes + keys + sort + LBVH + collapse of every segment.  The
// caller reads ctl (wide node count, errors) and segctl back.
cudaError_t build_tree_tris(BuildScratch &s, const BuildParams &bp, cudaStream_t st);
cudaError_t build_tree_insts(const InstState *inst, BuildScratch &s, const BuildParams &bp, cudaStream_t st);
// The pieces after the item boxes: Morton codes + sort + LBVH (then the rest); the binned-SAH
// binary tree (sah.cu; synchronises the stream once per level of ranges above 1024 items, and
// falls back to the LBVH under stream capture); the rest = binary SAH, bounding spheres, collapse.
cudaError_t build_tree_lbvh(BuildScratch &s, const BuildParams &bp, cudaStream_t st);
cudaError_t build_tree_sah(BuildScratch &s, const BuildParams &bp, cudaStream_t st);
cudaError_t build_tree_rest(BuildScratch &s, const BuildParams &bp, cudaStream_t st);
// Temporary bytes of the SAH build's scan over n items (it shares the sort's scratch).
size_t sah_scan_temp_bytes(uint32_t n);
// Kernels of this library launched by builds, refits and instance updates: a host counter
// (library kernels, CUB's sort and scan, are not counted).
void note_build_launches(uint32_t k);
uint64_t build_launches();

// Triangle splitting (split builds).  split_count: per triangle 1 + its extra
// references (refs; at most fraction x the segment's triangles extra per
// segment) and per segment their sum (seg_refs; wts: n words, sums: 12 nseg
// bytes of scratch), from the
// triangle-space segments tsegs; bad indices are flagged in segctl / ctl as by
// a build.  exclusive_sum: CUB exclusive scan (tmp null: size query).
// split_emit: the reference boxes into s (reference-space scratch) at ref_off,
// the triangle of each reference into ref_prim, and the centroid bounds.
cudaError_t split_count(const SegInput *tsegs, uint32_t nseg, uint32_t n, float fraction, float *wts,
                        unsigned long long *sums, uint32_t *refs, uint32_t *seg_refs, uint32_t *segctl, uint32_t *ctl,
                        cudaStream_t st);
cudaError_t exclusive_sum(void *tmp, size_t *tmp_bytes, const uint32_t *in, uint32_t *out, uint32_t n,
                          cudaStream_t st);
// Curve builds (see build.cu): per-segment Bezier form, cone counts and metas,
// then the segment of every cone once the counts are scanned.
cudaError_t curve_prepare(const unsigned char *cps, uint64_t stride, uint32_t cp_count, uint32_t keys,
                          const uint32_t *seg, uint32_t nseg, uint32_t basis, float4 *bez, uint32_t *count,
                          uint32_t *meta, uint32_t *err, cudaStream_t st);
cudaError_t curve_fill(const uint32_t *off, const uint32_t *count, uint32_t nseg, uint32_t *cone_seg,
                       cudaStream_t st);
cudaError_t split_emit(const SegInput *tsegs, uint32_t nseg, uint32_t n, const uint32_t *refs, const uint32_t *ref_off,
                       BuildScratch &s, uint32_t *ref_prim, cudaStream_t st);

// Phase 2: write both node layouts and the leaf items; wide_sah (2 nseg
// doubles, zeroed by the caller, may be null) receives the per-segment wide SAH.
// count_on_device: wide_count is the output's capacity and the collapse's own
// count (in s.ctl) bounds the nodes written -- a build with no host readback.
cudaError_t emit_blas(const BuildScratch &s, const BuildParams &bp, uint32_t wide_count, Node8Q *qn, Node8F *fn,
                      TriRec *tris, double *wide_sah, unsigned long long *rtab, cudaStream_t st,
                      bool count_on_device = false);
// ORs a build's error bits into another control block (the asynchronous error word).
cudaError_t report_build_errors(const uint32_t *ctl, uint32_t *into, cudaStream_t st);
// Refit (build.cu): new triangle records and boxes for a BLAS block whose
// topology is kept (rtab written by its build), from the segments' current
// buffers; bottom-up over the W wide nodes, then both node layouts re-encoded.
// Every segment must hold triangles (an empty segment's root is not written).
// counters: W words of scratch; ctl: kCtlWords zeroed words (errors).
cudaError_t refit_blas(const SegInput *segs, uint32_t nseg, uint32_t W, const unsigned long long *rtab, Node8Q *qn,
                       Node8F *fn, TriRec *tris, uint32_t *counters, uint32_t *ctl, cudaStream_t st);
// TLAS refit (same topology): instance boxes and inverses from the current
// instance states, then the bottom-up refit rewriting the instance records.
// ilo/ihi/w2o: n-sized scratch; segctl: kSegWords words of scratch.
cudaError_t refit_tlas(const InstState *inst, uint32_t n, float4 *ilo, float4 *ihi, float *w2o, uint32_t *segctl,
                       uint32_t W, const unsigned long long *rtab, Node8Q *qn, Node8F *fn, InstRec *recs,
                       uint32_t *counters, uint32_t *ctl, cudaStream_t st);
cudaError_t emit_tlas(const InstState *inst, const BuildScratch &s, const BuildParams &bp, uint32_t wide_count,
                      Node8Q *qn, Node8F *fn, InstRec *recs, double *wide_sah, unsigned long long *rtab,
                      cudaStream_t st);

cudaError_t apply_modifications(const ModRec *mods, uint32_t count, InstState *inst, uint32_t instance_count,
                                cudaStream_t st);
cudaError_t init_instances(InstState *inst, uint32_t begin, uint32_t end, cudaStream_t st);

// Traversal.
// One job of a multi-job trace launch: a ray batch against one TLAS.
struct __align__(16) DevJob {
    const Node8Q *tlas_q;
    const Node8F *tlas_f;
    const InstRec *insts;
    const Ray *rays;
    void *out;       // Hit[] (closest) or uint8_t[] (any)
    uint32_t first;  // global index of the job's first ray in the launch
    uint32_t count;
    uint32_t mask;
    uint32_t _pad;
    const float *times;  // per-ray times of the extended kernels (null: time 0)
};
static_assert(sizeof(DevJob) == 64, "DevJob size");

constexpr uint32_t kStageMaxChunks = 64;  // copy chunks of one streamed host-buffer trace (at most)
// trace error bits (TraceParams::pool[1]): stack overflow, step bound, a streamed launch's copy
// chunk that did not arrive in time
constexpr uint32_t kTraceErrStack = 1u, kTraceErrSteps = 2u, kTraceErrStage = 4u;

struct TraceParams {
    const Node8Q *tlas_q;
    const Node8F *tlas_f;
    const InstRec *insts;
    const Ray *rays;
    Hit *hits;
    uint8_t *occluded;
    uint32_t *counts;
    uint32_t *pool;  // [0] ray counter, [1] error flags
    uint32_t ray_count;
    uint32_t mask;
    uint32_t refill;      // refill a warp when at least this many lanes are idle (1..32)
    uint32_t postpone;    // postpone triangle tests when fewer lanes than this would run them (0 = off)
    int32_t postpone_sp;  // postpone only while the stack depth is below this
    uint32_t mode;        // loop structure: 0 = node + its items per step, 1 = speculative while-while
    const DevJob *jobs;   // non-null: a multi-job launch over job_count jobs (ray_count = their sum)
    uint32_t job_count;
    const uint32_t *order;  // non-null: the k-th ray taken is rays[order[k]] (single-job launches)
    uint32_t short_stack;   // shared-memory stack entries per thread: 8, 16 or 24 (single-job, mode 0)
    bool motion;            // the accel has motion or curves: the extended kernels (mode 0) run the call
    bool curves;            // with `motion`: the accel has curves (the extended kernels with the curve test)
    const float *times;     // motion launches: per-ray times (null: time 0)
    uint32_t max_steps = kMaxRaySteps;  // per-ray step bound; a ray that exceeds it ends and flags LCX_ERR_TIMEOUT
    // Streamed host-buffer launches (stage_flag non-null; single-job closest / any, quantised
    // nodes, loop mode 2): the rays arrive by copy chunks while the kernel runs.  Chunk c holds
    // rays [c << stage_shift, (c + 1) << stage_shift) and is in place once stage_flag[c] ==
    // stage_gen; each warp publishes to stage_mark[its index] a ray id below which every ray it
    // took has its result stored (0xffffffff once it has exited).
    const uint32_t *stage_flag = nullptr;
    uint32_t *stage_mark = nullptr;
    uint32_t stage_gen = 0, stage_shift = 0;
};
cudaError_t launch_trace(const TraceParams &p, int layout, bool any, bool counting, cudaStream_t st);
// Warps of a streamed launch over ray_count rays (the stage_mark entries it writes).
uint32_t stream_launch_warps(uint32_t ray_count, bool any);

// Ray reordering (reorder.cu): sorts the rays of a call by (direction octant,
// origin Morton cell of the TLAS root box, `bits` per axis) into a
// permutation held in stream-ordered scratch until reorder_end.
struct ReorderScratch {
    void *mem = nullptr;
    const uint32_t *order = nullptr;
};
int reorder_begin(const Ray *rays, uint32_t n, const Node8F *tlas_root, uint32_t bits, cudaStream_t st,
                  ReorderScratch *rs);
int reorder_end(ReorderScratch *rs, cudaStream_t st);

// The current device's stream-ordered memory pool for per-call scratch
// (reorder.cu): freed blocks stay in the pool for the next call instead of
// being returned to the driver at every synchronisation.
int scratch_pool(cudaMemPool_t *out);

// Validation + parameters of a trace_closest call with no device allocation
// (defined in capi.cu; `pool` is left for the caller to set).
int trace_params_for(uint64_t accel, const LcxRay *d_rays, uint32_t ray_count, uint32_t mask, LcxTriangleHit *d_hits,
                     uint32_t max_rays, TraceParams &p);
int record_error(int code, const char *msg);
// Error flags of lcx_trace_closest_noalloc on the current device (noalloc.cu), read and cleared.
int noalloc_take_errors(uint32_t *flags);

// BVH lifetime lock (capi.cu): a trace holds it shared from validating its
// accel until its kernel is enqueued; freeing BVH memory holds it exclusively.
std::shared_mutex &lifetime_mutex();

}  // namespace lcx
