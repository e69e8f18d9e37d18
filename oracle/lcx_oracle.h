/*
 * lcx_oracle.h — CPU oracle for the Mesh/Accel path.  TEST INFRASTRUCTURE.
 *
 * This is the checker and the timed CPU baseline, never the product: only
 * tests/, __graft_entry__.smoke() and bench.py (cpu_baseline leg and the
 * `--impl reference` arm) load it.  It restates, on the CPU, the semantics of
 * LuisaCompute's CPU backend for this path:
 *   - trace_closest  src/rust/luisa_compute_backend_impl/src/cpu/accel.rs:449-509
 *     (hit record, miss record {~0u,~0u,(0,0),t_max}, instance id = TLAS slot)
 *   - trace_any      accel.rs:511-535 (occluded <=> a hit with t in [t_min,t_max])
 *   - instance mask  accel.rs:289,414 ((ray mask & instance mask) != 0, default 0xff)
 *   - affine layout  include/luisa/runtime/rhi/command.h:557-571 (row-major 3x4)
 *   - barycentrics   src/dsl/rtx/hit.cpp:7-20 (p = (1-u-v) v0 + u v1 + v v2)
 *   - no face culling src/backends/cuda/cuda_mesh.cpp:15-16
 * Embree's own triangle arithmetic is third-party (embree_sys 0.1.11,
 * src/rust/Cargo.lock:267-270) and not vendored in the reference, so the
 * oracle does not restate it.  It uses the published watertight test of
 * Woop, Benthin and Wald (JCGT 2(1), 2013) with a fixed FP32 operation
 * sequence (explicit fma, no contraction), and an FP64 evaluator that
 * adjudicates disagreements.  Parity against the reference's own outputs is
 * UNPINNED: the reference holds no golden vectors for this path
 * (src/tests/test_rtx.cpp only writes images) and its CPU backend cannot be
 * built here (Rust + Embree absent).
 */
#ifndef LCX_ORACLE_H
#define LCX_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct LcxoRay {
    float o[3];
    float tmin;
    float d[3];
    float tmax;
} LcxoRay;

typedef struct LcxoHit {
    uint32_t inst;
    uint32_t prim;
    float u, v;
    float t;
    uint32_t pad;
} LcxoHit;

/* FP64 evaluation of one ray against one triangle of one instance. */
typedef struct LcxoF64Hit {
    int32_t hit;       /* 1 if the FP64 ray meets the triangle with t in [tmin,tmax] */
    int32_t pad;
    double t, u, v;
    double min_bary;   /* min(1-u-v, u, v): < 0 when the FP64 ray misses the triangle */
} LcxoF64Hit;

/* Mesh: `verts` holds vertex i at verts + i*stride_floats (xyz used). */
void *lcxo_mesh_create(const float *verts, size_t stride_floats, size_t vertex_count,
                       const uint32_t *tris, size_t tri_count, int leaf_size, int bins);
void lcxo_mesh_destroy(void *mesh);
/* SAH cost with C_node = 1, C_tri = 1, normalised by the root area. */
double lcxo_mesh_sah(const void *mesh);
uint32_t lcxo_mesh_depth(const void *mesh);

/* Accel over instances: o2w is row-major 3x4 per instance (12 floats),
 * masks are the visibility masks.  meshes[i] may repeat. */
void *lcxo_accel_create(size_t instance_count, void *const *meshes, const float *o2w,
                        const uint32_t *masks);
void lcxo_accel_destroy(void *accel);

/* Batched queries with `threads` host threads (0 = all hardware threads). */
void lcxo_trace_closest(const void *accel, const LcxoRay *rays, size_t n, uint32_t mask,
                        LcxoHit *hits, int threads);
void lcxo_trace_any(const void *accel, const LcxoRay *rays, size_t n, uint32_t mask,
                    uint8_t *occluded, int threads);
/* Same results by testing every triangle of every instance (no BVH). */
void lcxo_brute_closest(const void *accel, const LcxoRay *rays, size_t n, uint32_t mask,
                        LcxoHit *hits, int threads);

/* FP64 closest hit (double transform, double intersection) through the BVH. */
void lcxo_fp64_closest(const void *accel, const LcxoRay *rays, size_t n, uint32_t mask,
                       LcxoHit *hits, double *t64, int threads);
/* FP64 evaluation of ray i against (inst[i], prim[i]). */
void lcxo_fp64_eval(const void *accel, const LcxoRay *rays, size_t n, const uint32_t *inst,
                    const uint32_t *prim, LcxoF64Hit *out);

/* Path tracer parameters: byte-identical to LcxPtParams of include/lcx_accel.h. */
typedef struct LcxoPtParams {
    uint32_t width, height, spp, max_bounces, rr_start, seed;
    float eye[3], target[3], up[3];
    float tan_half_fov;
    float light_pos[3], light_intensity[3];
    float env[3];
} LcxoPtParams;

/* The wavefront tracer's algorithm, one path at a time on the CPU: albedo[i]
 * points at the per-triangle albedo of instance i's mesh.  image: width *
 * height * 3 floats; first_hits (optional): the first bounce of every path. */
void lcxo_pathtrace(const void *accel, const float *const *albedo, const LcxoPtParams *params, float *image,
                    LcxoHit *first_hits, int threads);

/* The FP32 operation sequences the GPU kernels must reproduce bit for bit. */
void lcxo_affine_inverse(const float *o2w, float *w2o);

/* Motion instances (the product's matrix keyframes): instance i moves when
 * motion[i].keys is non-null -- `count` row-major 3x4 object-to-world
 * matrices over [t0, t1] (flags bit 2: SRT records of 16 floats instead);
 * flags bit 0 / 1: vanish before t0 / after t1.  The interpolation restates
 * motion_matrix and srt_matrix of include/lcx/bvh_device.cuh with the same
 * FP32 sequence; the inverse is affine_inverse_f32.  Every instance is
 * tested (no TLAS), each through its mesh BVH.  times: one per ray. */
typedef struct LcxoMotion {
    const float *keys;
    uint32_t count;
    float t0, t1;
    uint32_t flags;
} LcxoMotion;
/* Keyframed vertices of an instance's mesh (null verts: static): `keys`
 * copies of `vcount` vertices (stride_floats apart, xyz used) over [t0, t1],
 * interpolated per component (motion_triangle of bvh_device.cuh); such
 * instances are tested triangle by triangle. */
typedef struct LcxoMeshMotion {
    const float *verts;
    size_t stride_floats;
    uint32_t vcount, keys;
    const uint32_t *tris;
    uint32_t tri_count;
    float t0, t1;
    uint32_t flags;
} LcxoMeshMotion;
void lcxo_trace_motion(const void *accel, const LcxoMotion *motion, const LcxoMeshMotion *mesh_motion,
                       const LcxoRay *rays, const float *times, size_t n, uint32_t mask, int any, LcxoHit *hits,
                       uint8_t *occluded, int threads);
/* Curves (bases 0..3 as LuisaCompute's CurveBasis): control point i at
 * control_points + i*cp_stride_floats (x, y, z, radius); one u32 per segment
 * (its first control point).  Returns null if a segment runs past cp_count.
 * lcxo_trace_curves tests every segment of every instance whose
 * inst_curve[i] is non-null (a curve from lcxo_curve_create; null instances are
 * skipped), brute force, in FP64 (see lcx_oracle.cpp for the definition). */
void *lcxo_curve_create(const float *control_points, size_t cp_stride_floats, size_t cp_count,
                        const uint32_t *segments, size_t seg_count, uint32_t basis);
void lcxo_curve_destroy(void *curve);
uint32_t lcxo_curve_pieces(const void *curve, size_t segment);
void lcxo_trace_curves(void *const *inst_curve, const float *o2w, const uint32_t *inst_mask, size_t instance_count,
                       const LcxoRay *rays, size_t n, uint32_t mask, int any, LcxoHit *hits, uint8_t *occluded,
                       int threads);
/* Keyframed control points: `keys` copies of cp_per_key points back to back
 * over [t0, t1] (flags bit 0 / 1: vanish before / after); the Bezier points
 * interpolate linearly at each ray's time (times: one per ray, null = 0). */
void *lcxo_curve_create_motion(const float *control_points, size_t cp_stride_floats, size_t cp_per_key, uint32_t keys,
                               const uint32_t *segments, size_t seg_count, uint32_t basis, float t0, float t1,
                               uint32_t flags);
void lcxo_trace_curves_t(void *const *inst_curve, const float *o2w, const uint32_t *inst_mask, size_t instance_count,
                         const LcxoRay *rays, const float *times, size_t n, uint32_t mask, int any, LcxoHit *hits,
                         uint8_t *occluded, int threads);
int lcxo_intersect_triangle(const float *o, const float *d, float tmin, float tmax,
                            const float *v0, const float *v1, const float *v2, float *t,
                            float *u, float *v);

#ifdef __cplusplus
}
#endif

#endif
