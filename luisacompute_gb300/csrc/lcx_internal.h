// lcx_internal.h — host-side interface between the C ABI layer (capi.cu) and
// the kernel translation units (build.cu, traverse.cu, sort.cu).
#pragma once

#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

#include "lcx_accel.h"
#include "lcx_device.cuh"

namespace lcx {

// Per-build device scratch, sized for `n` items.
struct BuildScratch {
    float4 *box_lo = nullptr;        // n   item boxes
    float4 *box_hi = nullptr;        // n
    unsigned long long *keys = nullptr;  // n   Morton keys
    unsigned long long *keys_sorted = nullptr;
    uint32_t *vals = nullptr;        // n   item ids
    uint32_t *vals_sorted = nullptr;
    uint32_t *bin_child = nullptr;   // 2(n-1)
    float4 *bin_lo = nullptr;        // n-1 (w = count bits)
    float4 *bin_hi = nullptr;        // n-1 (w = first bits)
    int32_t *other = nullptr;        // n-1
    uint32_t *desc = nullptr;        // (n+1) * 12 words
    uint2 *queue = nullptr;          // 2 (n+1)
    float *w2o = nullptr;            // TLAS: 12 n
    uint32_t *ctl = nullptr;         // control words (see build.cu)
    void *sort_tmp = nullptr;
    size_t sort_tmp_bytes = 0;
};

// Control block layout (uint32 words).
enum : int {
    kCtlWideCount = 0,
    kCtlItemCount = 1,
    kCtlDepth = 2,
    kCtlErr = 3,
    kCtlRoot = 4,
    kCtlCenLo = 8,    // 3 ordered-uint words
    kCtlCenHi = 12,   // 3 ordered-uint words
    kCtlLevel = 16,   // kMaxLevels + 1 words
    kCtlWords = 16 + kMaxLevels + 2,
};

enum : uint32_t {
    kErrBadIndex = 1u,
    kErrTooDeep = 2u,
    kErrQuant = 4u,
};

size_t sort_temp_bytes(uint32_t n);
cudaError_t sort_pairs(void *tmp, size_t tmp_bytes, const unsigned long long *kin, unsigned long long *kout,
                       const uint32_t *vin, uint32_t *vout, uint32_t n, cudaStream_t s);

struct TriInput {
    const unsigned char *vbase;  // vertex buffer + offset
    size_t vstride;
    uint32_t vcount;
    const unsigned char *tbase;  // triangle buffer + offset
};

// Phase 1: item boxes + Morton keys + sort + LBVH + collapse.  Leaves
// ctl words on the device; the caller reads wide/item counts back.
cudaError_t build_tree_tris(const TriInput &in, uint32_t n, int leaf_max, BuildScratch &s, cudaStream_t st);
cudaError_t build_tree_insts(const InstState *inst, uint32_t n, int leaf_max, BuildScratch &s, cudaStream_t st);

// Phase 2: write both node layouts and the leaf items.
cudaError_t emit_blas(const TriInput &in, uint32_t n, int leaf_max, uint32_t wide_count, const BuildScratch &s,
                      Node8Q *qn, Node8F *fn, TriRec *tris, BlasDesc *desc, cudaStream_t st);
cudaError_t emit_tlas(const InstState *inst, uint32_t n, int leaf_max, uint32_t wide_count, const BuildScratch &s,
                      Node8Q *qn, Node8F *fn, InstRec *recs, cudaStream_t st);

cudaError_t apply_modifications(const ModRec *mods, uint32_t count, InstState *inst, uint32_t instance_count,
                                cudaStream_t st);
cudaError_t init_instances(InstState *inst, uint32_t begin, uint32_t end, cudaStream_t st);

// SAH of the binary tree of the last build_tree_* call (written after the
// control words; read back with them).
cudaError_t binary_sah(const BuildScratch &s, uint32_t n, cudaStream_t st);

// Wide-tree SAH (C_node = 1, C_item = 1, normalised by the root area).
cudaError_t wide_sah(const Node8F *fn, uint32_t wide_count, double *d_out, cudaStream_t st);

// Traversal.
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
};
cudaError_t launch_trace(const TraceParams &p, int layout, bool any, bool counting, cudaStream_t st);

// Validation + parameters of a trace_closest call with no device allocation
// (defined in capi.cu; `pool` is left for the caller to set).
int trace_params_for(uint64_t accel, const LcxRay *d_rays, uint32_t ray_count, uint32_t mask, LcxTriangleHit *d_hits,
                     uint32_t max_rays, TraceParams &p);
int record_error(int code, const char *msg);

}  // namespace lcx
