// lcx_oracle.cpp — CPU oracle for the Mesh/Accel path.  TEST INFRASTRUCTURE:
// the checker and the timed CPU baseline, never linked into the product.
// Semantics follow LuisaCompute's CPU backend (citations in lcx_oracle.h);
// the FP32 arithmetic follows Woop, Benthin & Wald, "Watertight Ray/Triangle
// Intersection", JCGT 2(1) 2013, with the operation order fixed below.
//
// Compile with -ffp-contract=off: every fused multiply-add here is an
// explicit std::fma, every other operation rounds on its own, so the results
// are reproducible bit for bit by the CUDA kernels (which use the __f*_rn
// intrinsics in the same order).
#include "lcx_oracle.h"

// the path tracer's sampling arithmetic is shared with the GPU kernels (it is
// this project's, not the reference's); the geometry and traversal are not
#include "../luisacompute_gb300/csrc/pt_math.cuh"

#include <algorithm>
#include <atomic>
#include <cfloat>
#include <cmath>
#include <cstring>
#include <thread>
#include <vector>

namespace {

constexpr uint32_t kInvalid = 0xffffffffu;

// ------------------------------------------------------------------ FP32 math
// (1) Affine inverse of the row-major 3x4 object-to-world matrix
//     (include/luisa/runtime/rhi/command.h:557-571 layout).
void affine_inverse_f32(const float *m, float *w) {
    const float a = m[0], b = m[1], c = m[2];
    const float d = m[4], e = m[5], f = m[6];
    const float g = m[8], h = m[9], i = m[10];
    const float c00 = std::fma(e, i, -(f * h));
    const float c01 = std::fma(f, g, -(d * i));
    const float c02 = std::fma(d, h, -(e * g));
    const float det = std::fma(a, c00, std::fma(b, c01, c * c02));
    const float r = 1.0f / det;
    float R[9];
    R[0] = c00 * r;
    R[1] = std::fma(c, h, -(b * i)) * r;
    R[2] = std::fma(b, f, -(c * e)) * r;
    R[3] = c01 * r;
    R[4] = std::fma(a, i, -(c * g)) * r;
    R[5] = std::fma(c, d, -(a * f)) * r;
    R[6] = c02 * r;
    R[7] = std::fma(b, g, -(a * h)) * r;
    R[8] = std::fma(a, e, -(b * d)) * r;
    const float tx = m[3], ty = m[7], tz = m[11];
    for (int k = 0; k < 3; k++) {
        w[4 * k + 0] = R[3 * k + 0];
        w[4 * k + 1] = R[3 * k + 1];
        w[4 * k + 2] = R[3 * k + 2];
        w[4 * k + 3] = -std::fma(R[3 * k + 0], tx, std::fma(R[3 * k + 1], ty, R[3 * k + 2] * tz));
    }
}

// (2) World ray -> object ray with the world-to-object matrix.
void transform_ray_f32(const float *w, const float *o, const float *d, float *oo, float *od) {
    for (int k = 0; k < 3; k++) {
        oo[k] = std::fma(w[4 * k], o[0], std::fma(w[4 * k + 1], o[1], std::fma(w[4 * k + 2], o[2], w[4 * k + 3])));
        od[k] = std::fma(w[4 * k], d[0], std::fma(w[4 * k + 1], d[1], w[4 * k + 2] * d[2]));
    }
}

// (3) Watertight test, per-ray part.
struct WtRay {
    float o[3];
    int kx, ky, kz;
    float Sx, Sy, Sz;
    float tmin, tmax;
};

void wt_setup(WtRay &r, const float *o, const float *d, float tmin, float tmax) {
    r.o[0] = o[0];
    r.o[1] = o[1];
    r.o[2] = o[2];
    const float ax = std::fabs(d[0]), ay = std::fabs(d[1]), az = std::fabs(d[2]);
    int kz = (ax >= ay) ? ((ax >= az) ? 0 : 2) : ((ay >= az) ? 1 : 2);
    int kx = kz + 1 == 3 ? 0 : kz + 1;
    int ky = kx + 1 == 3 ? 0 : kx + 1;
    if (d[kz] < 0.0f) std::swap(kx, ky);
    r.kx = kx;
    r.ky = ky;
    r.kz = kz;
    r.Sz = 1.0f / d[kz];
    r.Sx = d[kx] * r.Sz;
    r.Sy = d[ky] * r.Sz;
    r.tmin = tmin;
    r.tmax = tmax;
}

// (4) Watertight test, per-triangle part.  Returns true on a hit with
//     t in [tmin, tmax]; (u, v) weight v1 and v2.
bool wt_intersect(const WtRay &r, const float *v0, const float *v1, const float *v2, float &t_out,
                  float &u_out, float &v_out) {
    const float A[3] = {v0[0] - r.o[0], v0[1] - r.o[1], v0[2] - r.o[2]};
    const float B[3] = {v1[0] - r.o[0], v1[1] - r.o[1], v1[2] - r.o[2]};
    const float C[3] = {v2[0] - r.o[0], v2[1] - r.o[1], v2[2] - r.o[2]};
    const float Ax = std::fma(-r.Sx, A[r.kz], A[r.kx]);
    const float Ay = std::fma(-r.Sy, A[r.kz], A[r.ky]);
    const float Bx = std::fma(-r.Sx, B[r.kz], B[r.kx]);
    const float By = std::fma(-r.Sy, B[r.kz], B[r.ky]);
    const float Cx = std::fma(-r.Sx, C[r.kz], C[r.kx]);
    const float Cy = std::fma(-r.Sy, C[r.kz], C[r.ky]);
    // edge functions with separately rounded products: swapping two vertices
    // negates them exactly, which keeps shared edges watertight
    const float U = Cx * By - Cy * Bx;
    const float V = Ax * Cy - Ay * Cx;
    const float W = Bx * Ay - By * Ax;
    if ((U < 0.0f || V < 0.0f || W < 0.0f) && (U > 0.0f || V > 0.0f || W > 0.0f)) return false;
    const float det = (U + V) + W;
    if (det == 0.0f) return false;
    const float Az = r.Sz * A[r.kz];
    const float Bz = r.Sz * B[r.kz];
    const float Cz = r.Sz * C[r.kz];
    const float T = std::fma(U, Az, std::fma(V, Bz, W * Cz));
    const float t = T / det;
    if (!(t >= r.tmin && t <= r.tmax)) return false;
    t_out = t;
    u_out = V / det;
    v_out = W / det;
    return true;
}

// Candidate (t, inst, prim) beats the current best?  Ties in t go to the
// smaller (inst, prim), so the answer does not depend on traversal order.
inline bool better(float t, uint32_t inst, uint32_t prim, const LcxoHit &b) {
    if (t < b.t) return true;
    if (t > b.t) return false;
    return inst < b.inst || (inst == b.inst && prim < b.prim);
}

// ----------------------------------------------------------------- FP64 math
struct WtRay64 {
    double o[3];
    int kx, ky, kz;
    double Sx, Sy, Sz;
    double tmin, tmax;
};

void wt_setup64(WtRay64 &r, const double *o, const double *d, double tmin, double tmax) {
    for (int k = 0; k < 3; k++) r.o[k] = o[k];
    const double ax = std::fabs(d[0]), ay = std::fabs(d[1]), az = std::fabs(d[2]);
    int kz = (ax >= ay) ? ((ax >= az) ? 0 : 2) : ((ay >= az) ? 1 : 2);
    int kx = kz + 1 == 3 ? 0 : kz + 1;
    int ky = kx + 1 == 3 ? 0 : kx + 1;
    if (d[kz] < 0.0) std::swap(kx, ky);
    r.kx = kx;
    r.ky = ky;
    r.kz = kz;
    r.Sx = d[kx] / d[kz];
    r.Sy = d[ky] / d[kz];
    r.Sz = 1.0 / d[kz];
    r.tmin = tmin;
    r.tmax = tmax;
}

// FP64 evaluation: always returns (t, u, v, min_bary) of the plane hit; `hit`
// says whether the point is inside the triangle and t in range.
bool wt_eval64(const WtRay64 &r, const double *v0, const double *v1, const double *v2, double &t,
               double &u, double &v, double &min_bary) {
    const double A[3] = {v0[0] - r.o[0], v0[1] - r.o[1], v0[2] - r.o[2]};
    const double B[3] = {v1[0] - r.o[0], v1[1] - r.o[1], v1[2] - r.o[2]};
    const double C[3] = {v2[0] - r.o[0], v2[1] - r.o[1], v2[2] - r.o[2]};
    const double Ax = A[r.kx] - r.Sx * A[r.kz], Ay = A[r.ky] - r.Sy * A[r.kz];
    const double Bx = B[r.kx] - r.Sx * B[r.kz], By = B[r.ky] - r.Sy * B[r.kz];
    const double Cx = C[r.kx] - r.Sx * C[r.kz], Cy = C[r.ky] - r.Sy * C[r.kz];
    const double U = Cx * By - Cy * Bx;
    const double V = Ax * Cy - Ay * Cx;
    const double W = Bx * Ay - By * Ax;
    const double det = U + V + W;
    if (det == 0.0) {
        t = u = v = 0.0;
        min_bary = -1.0;
        return false;
    }
    const double T = U * (r.Sz * A[r.kz]) + V * (r.Sz * B[r.kz]) + W * (r.Sz * C[r.kz]);
    t = T / det;
    u = V / det;
    v = W / det;
    const double w0 = U / det;
    min_bary = std::min(w0, std::min(u, v));
    return min_bary >= 0.0 && t >= r.tmin && t <= r.tmax;
}

void affine_inverse_f64(const float *mf, double *w) {
    double m[12];
    for (int k = 0; k < 12; k++) m[k] = mf[k];
    const double a = m[0], b = m[1], c = m[2], d = m[4], e = m[5], f = m[6], g = m[8], h = m[9], i = m[10];
    const double c00 = e * i - f * h, c01 = f * g - d * i, c02 = d * h - e * g;
    const double det = a * c00 + b * c01 + c * c02;
    const double R[9] = {c00 / det,           (c * h - b * i) / det, (b * f - c * e) / det,
                         c01 / det,           (a * i - c * g) / det, (c * d - a * f) / det,
                         c02 / det,           (b * g - a * h) / det, (a * e - b * d) / det};
    for (int k = 0; k < 3; k++) {
        w[4 * k + 0] = R[3 * k];
        w[4 * k + 1] = R[3 * k + 1];
        w[4 * k + 2] = R[3 * k + 2];
        w[4 * k + 3] = -(R[3 * k] * m[3] + R[3 * k + 1] * m[7] + R[3 * k + 2] * m[11]);
    }
}

// --------------------------------------------------------------------- BVH
struct Box {
    float lo[3] = {FLT_MAX, FLT_MAX, FLT_MAX};
    float hi[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
    void grow(const float *p) {
        for (int k = 0; k < 3; k++) {
            lo[k] = std::min(lo[k], p[k]);
            hi[k] = std::max(hi[k], p[k]);
        }
    }
    void grow(const Box &b) {
        for (int k = 0; k < 3; k++) {
            lo[k] = std::min(lo[k], b.lo[k]);
            hi[k] = std::max(hi[k], b.hi[k]);
        }
    }
    bool empty() const { return !(lo[0] <= hi[0] && lo[1] <= hi[1] && lo[2] <= hi[2]); }
    double area() const {
        if (empty()) return 0.0;
        const double dx = double(hi[0]) - lo[0], dy = double(hi[1]) - lo[1], dz = double(hi[2]) - lo[2];
        return 2.0 * (dx * dy + dy * dz + dz * dx);
    }
};

struct Node {
    Box box;
    uint32_t first;  // internal: left child index (right = first + 1); leaf: first item
    uint32_t count;  // 0 = internal
};

// Top-down binned-SAH builder over item boxes (triangles or instances).
struct Bvh {
    std::vector<Node> nodes;
    std::vector<uint32_t> items;  // item ids in leaf order
    uint32_t depth = 0;

    void build(const std::vector<Box> &boxes, int leaf_size, int bins) {
        const size_t n = boxes.size();
        items.resize(n);
        for (size_t i = 0; i < n; i++) items[i] = uint32_t(i);
        nodes.clear();
        nodes.reserve(2 * n + 1);
        std::vector<float> cen(3 * n);
        for (size_t i = 0; i < n; i++)
            for (int k = 0; k < 3; k++) {
                const float c = 0.5f * (boxes[i].lo[k] + boxes[i].hi[k]);
                cen[3 * i + k] = std::isfinite(c) ? c : 0.0f;
            }
        nodes.push_back(Node{});
        if (n == 0) {
            nodes[0].first = 0;
            nodes[0].count = 0;
            depth = 0;
            return;
        }
        struct Task {
            uint32_t node, begin, end, level;
        };
        std::vector<Task> stack{{0, 0, uint32_t(n), 1}};
        std::vector<Box> bin_box(bins), left_acc(bins);
        std::vector<uint32_t> bin_cnt(bins);
        while (!stack.empty()) {
            Task tk = stack.back();
            stack.pop_back();
            depth = std::max(depth, tk.level);
            Box nb, cb;
            for (uint32_t i = tk.begin; i < tk.end; i++) {
                nb.grow(boxes[items[i]]);
                cb.grow(&cen[3 * items[i]]);
            }
            nodes[tk.node].box = nb;
            const uint32_t cnt = tk.end - tk.begin;
            auto make_leaf = [&] {
                nodes[tk.node].first = tk.begin;
                nodes[tk.node].count = cnt;
            };
            if (cnt <= uint32_t(leaf_size)) {
                make_leaf();
                continue;
            }
            // binned SAH over the three axes
            double best_cost = double(cnt) * nb.area();
            int best_axis = -1, best_split = 0;
            for (int ax = 0; ax < 3; ax++) {
                const float ext = cb.hi[ax] - cb.lo[ax];
                if (!(ext > 0.0f)) continue;
                const float scale = float(bins) / ext;
                std::fill(bin_box.begin(), bin_box.end(), Box{});
                std::fill(bin_cnt.begin(), bin_cnt.end(), 0u);
                for (uint32_t i = tk.begin; i < tk.end; i++) {
                    int b = int((cen[3 * items[i] + ax] - cb.lo[ax]) * scale);
                    b = std::min(std::max(b, 0), bins - 1);
                    bin_cnt[b]++;
                    bin_box[b].grow(boxes[items[i]]);
                }
                Box acc;
                uint32_t acc_n = 0;
                std::vector<double> left_cost(bins);
                for (int b = 0; b < bins - 1; b++) {
                    acc.grow(bin_box[b]);
                    acc_n += bin_cnt[b];
                    left_cost[b] = double(acc_n) * acc.area();
                }
                acc = Box{};
                acc_n = 0;
                for (int b = bins - 1; b > 0; b--) {
                    acc.grow(bin_box[b]);
                    acc_n += bin_cnt[b];
                    const double c = left_cost[b - 1] + double(acc_n) * acc.area() + nb.area();
                    if (c < best_cost && acc_n > 0 && acc_n < cnt) {
                        best_cost = c;
                        best_axis = ax;
                        best_split = b;
                    }
                }
            }
            uint32_t mid;
            if (best_axis < 0) {
                if (cnt <= 16u) {
                    make_leaf();
                    continue;
                }
                // all centroids equal or SAH prefers a leaf that is too big: median split
                mid = tk.begin + cnt / 2;
            } else {
                const float scale = float(bins) / (cb.hi[best_axis] - cb.lo[best_axis]);
                auto it = std::partition(items.begin() + tk.begin, items.begin() + tk.end, [&](uint32_t id) {
                    int b = int((cen[3 * id + best_axis] - cb.lo[best_axis]) * scale);
                    b = std::min(std::max(b, 0), bins - 1);
                    return b < best_split;
                });
                mid = uint32_t(it - items.begin());
                if (mid == tk.begin || mid == tk.end) mid = tk.begin + cnt / 2;
            }
            const uint32_t l = uint32_t(nodes.size());
            nodes.push_back(Node{});
            nodes.push_back(Node{});
            nodes[tk.node].first = l;
            nodes[tk.node].count = 0;
            stack.push_back({l + 1, mid, tk.end, tk.level + 1});
            stack.push_back({l, tk.begin, mid, tk.level + 1});
        }
    }

    double sah() const {
        if (nodes.empty() || nodes[0].box.empty()) return 0.0;
        const double ra = nodes[0].box.area();
        double c = 0.0;
        for (const Node &nd : nodes) c += nd.box.area() / ra * (nd.count ? double(nd.count) : 1.0);
        return c;
    }
};

// Robust slab test in FP32 with an outward slack on the exit distance.
inline bool slab(const Box &b, const float *o, const float *inv, float tmin, float tmax, float &tnear) {
    // near/far planes chosen by the sign of 1/d, so that a NaN (ray in the
    // plane) reaches fmax/fmin alone and is ignored
    float tn = tmin, tf = tmax;
    for (int k = 0; k < 3; k++) {
        const bool neg = std::signbit(inv[k]);
        const float t0 = ((neg ? b.hi[k] : b.lo[k]) - o[k]) * inv[k];
        const float t1 = ((neg ? b.lo[k] : b.hi[k]) - o[k]) * inv[k];
        tn = std::fmax(tn, t0);
        tf = std::fmin(tf, t1);
    }
    tnear = tn;
    return tn <= tf + std::fabs(tf) * 0x1p-18f;
}

inline bool slab64(const Box &b, const double *o, const double *inv, double tmin, double tmax, double &tnear) {
    double tn = tmin, tf = tmax;
    for (int k = 0; k < 3; k++) {
        const bool neg = std::signbit(inv[k]);
        const double t0 = (double(neg ? b.hi[k] : b.lo[k]) - o[k]) * inv[k];
        const double t1 = (double(neg ? b.lo[k] : b.hi[k]) - o[k]) * inv[k];
        tn = std::fmax(tn, t0);
        tf = std::fmin(tf, t1);
    }
    tnear = tn;
    return tn <= tf + std::fabs(tf) * 1e-9;
}

// IEEE reciprocals: a zero direction component gives +-inf, and a ray lying in
// a slab plane gives 0 * inf = NaN there, which std::fmin/fmax ignore, so the
// slab does not constrain that ray.
inline float safe_inv(float x) { return 1.0f / x; }
inline double safe_inv64(double x) { return 1.0 / x; }

struct Mesh {
    std::vector<float> v;  // 3 floats per vertex
    std::vector<uint32_t> t;
    Bvh bvh;
    size_t vertex_count = 0;
    const float *vert(uint32_t i) const { return &v[3 * size_t(i)]; }
    bool tri_valid(uint32_t p) const {
        return t[3 * p] < vertex_count && t[3 * p + 1] < vertex_count && t[3 * p + 2] < vertex_count;
    }
};

struct Accel {
    std::vector<const Mesh *> mesh;
    std::vector<float> o2w, w2o;  // 12 floats each
    std::vector<double> w2o64;
    std::vector<uint32_t> mask;
    Bvh bvh;
};

// -------------------------------------------------------- FP32 traversal
template <bool kAny>
bool trace_mesh(const Mesh &m, uint32_t inst, const float *o, const float *d, float tmin, LcxoHit &best) {
    if (m.bvh.nodes.empty() || m.t.empty()) return false;
    WtRay wr;
    wt_setup(wr, o, d, tmin, best.t);
    const float inv[3] = {safe_inv(d[0]), safe_inv(d[1]), safe_inv(d[2])};
    uint32_t stack[128];
    int sp = 0;
    stack[sp++] = 0;
    while (sp) {
        const Node &nd = m.bvh.nodes[stack[--sp]];
        float tn;
        if (!slab(nd.box, o, inv, tmin, best.t, tn)) continue;
        if (nd.count) {
            for (uint32_t i = 0; i < nd.count; i++) {
                const uint32_t p = m.bvh.items[nd.first + i];
                if (!m.tri_valid(p)) continue;
                float t, u, v;
                wr.tmax = best.t;
                if (wt_intersect(wr, m.vert(m.t[3 * p]), m.vert(m.t[3 * p + 1]), m.vert(m.t[3 * p + 2]), t, u, v)) {
                    if (kAny) return true;
                    if (better(t, inst, p, best)) best = LcxoHit{inst, p, u, v, t, 0};
                }
            }
        } else {
            const Node &l = m.bvh.nodes[nd.first], &r = m.bvh.nodes[nd.first + 1];
            float tl, tr;
            const bool hl = slab(l.box, o, inv, tmin, best.t, tl);
            const bool hr = slab(r.box, o, inv, tmin, best.t, tr);
            if (hl && hr) {
                if (tl <= tr) {
                    stack[sp++] = nd.first + 1;
                    stack[sp++] = nd.first;
                } else {
                    stack[sp++] = nd.first;
                    stack[sp++] = nd.first + 1;
                }
            } else if (hl) {
                stack[sp++] = nd.first;
            } else if (hr) {
                stack[sp++] = nd.first + 1;
            }
        }
    }
    return false;
}

template <bool kAny>
bool trace_accel(const Accel &a, const LcxoRay &ray, uint32_t mask, LcxoHit &best) {
    best = LcxoHit{kInvalid, kInvalid, 0.0f, 0.0f, ray.tmax, 0};
    if (a.bvh.nodes.empty()) return false;
    const float inv[3] = {safe_inv(ray.d[0]), safe_inv(ray.d[1]), safe_inv(ray.d[2])};
    uint32_t stack[128];
    int sp = 0;
    stack[sp++] = 0;
    while (sp) {
        const Node &nd = a.bvh.nodes[stack[--sp]];
        float tn;
        if (!slab(nd.box, ray.o, inv, ray.tmin, best.t, tn)) continue;
        if (nd.count) {
            for (uint32_t i = 0; i < nd.count; i++) {
                const uint32_t id = a.bvh.items[nd.first + i];
                if ((a.mask[id] & mask) == 0u || a.mesh[id] == nullptr) continue;
                float oo[3], od[3];
                transform_ray_f32(&a.w2o[12 * size_t(id)], ray.o, ray.d, oo, od);
                if (trace_mesh<kAny>(*a.mesh[id], id, oo, od, ray.tmin, best) && kAny) return true;
            }
        } else {
            stack[sp++] = nd.first + 1;
            stack[sp++] = nd.first;
        }
    }
    return false;
}

// -------------------------------------------------------- FP64 traversal
void trace_accel64(const Accel &a, const LcxoRay &ray, uint32_t mask, LcxoHit &best, double &best_t) {
    best = LcxoHit{kInvalid, kInvalid, 0.0f, 0.0f, ray.tmax, 0};
    best_t = ray.tmax;
    if (a.bvh.nodes.empty()) return;
    const double o[3] = {ray.o[0], ray.o[1], ray.o[2]};
    const double d[3] = {ray.d[0], ray.d[1], ray.d[2]};
    const double inv[3] = {safe_inv64(d[0]), safe_inv64(d[1]), safe_inv64(d[2])};
    uint32_t stack[128];
    int sp = 0;
    stack[sp++] = 0;
    while (sp) {
        const Node &nd = a.bvh.nodes[stack[--sp]];
        double tn;
        if (!slab64(nd.box, o, inv, ray.tmin, best_t, tn)) continue;
        if (!nd.count) {
            stack[sp++] = nd.first + 1;
            stack[sp++] = nd.first;
            continue;
        }
        for (uint32_t i = 0; i < nd.count; i++) {
            const uint32_t id = a.bvh.items[nd.first + i];
            if ((a.mask[id] & mask) == 0u || a.mesh[id] == nullptr) continue;
            const Mesh &m = *a.mesh[id];
            if (m.t.empty()) continue;
            const double *w = &a.w2o64[12 * size_t(id)];
            double oo[3], od[3];
            for (int k = 0; k < 3; k++) {
                oo[k] = w[4 * k] * o[0] + w[4 * k + 1] * o[1] + w[4 * k + 2] * o[2] + w[4 * k + 3];
                od[k] = w[4 * k] * d[0] + w[4 * k + 1] * d[1] + w[4 * k + 2] * d[2];
            }
            WtRay64 wr;
            wt_setup64(wr, oo, od, ray.tmin, ray.tmax);
            const double binv[3] = {safe_inv64(od[0]), safe_inv64(od[1]), safe_inv64(od[2])};
            uint32_t st2[128];
            int sp2 = 0;
            st2[sp2++] = 0;
            while (sp2) {
                const Node &bn = m.bvh.nodes[st2[--sp2]];
                double tn2;
                if (!slab64(bn.box, oo, binv, ray.tmin, best_t, tn2)) continue;
                if (!bn.count) {
                    st2[sp2++] = bn.first + 1;
                    st2[sp2++] = bn.first;
                    continue;
                }
                for (uint32_t j = 0; j < bn.count; j++) {
                    const uint32_t p = m.bvh.items[bn.first + j];
                    if (!m.tri_valid(p)) continue;
                    double v0[3], v1[3], v2[3];
                    for (int k = 0; k < 3; k++) {
                        v0[k] = m.vert(m.t[3 * p])[k];
                        v1[k] = m.vert(m.t[3 * p + 1])[k];
                        v2[k] = m.vert(m.t[3 * p + 2])[k];
                    }
                    double t, u, v, mb;
                    if (wt_eval64(wr, v0, v1, v2, t, u, v, mb)) {
                        if (t < best_t || (t == best_t && (id < best.inst || (id == best.inst && p < best.prim)))) {
                            best_t = t;
                            best = LcxoHit{id, p, float(u), float(v), float(t), 0};
                        }
                    }
                }
            }
        }
    }
}

template <class F>
void parallel_rays(size_t n, int threads, F &&f) {
    if (threads <= 0) threads = int(std::max(1u, std::thread::hardware_concurrency()));
    std::atomic<size_t> next{0};
    constexpr size_t kChunk = 256;
    auto worker = [&] {
        for (;;) {
            const size_t b = next.fetch_add(kChunk);
            if (b >= n) return;
            const size_t e = std::min(n, b + kChunk);
            for (size_t i = b; i < e; i++) f(i);
        }
    };
    if (threads == 1 || n <= kChunk) {
        worker();
        return;
    }
    std::vector<std::thread> pool;
    for (int i = 0; i < threads; i++) pool.emplace_back(worker);
    for (auto &t : pool) t.join();
}


// ------------------------------------------------------------------ curves
// Curves (the reference's Curve, include/luisa/runtime/rtx/curve.h; bases
// include/luisa/runtime/rhi/curve_basis.h:11-24).  The reference hands curves
// to Embree's round curves (cpu/accel.rs:142-204) and OptiX's round curves
// (cuda_curve.cpp:37-70), neither of which is vendored, so what is restated is
// the geometric definition the product documents (lcx_accel.h, curve section):
// a segment is the union of balls along its curve; cubic segments are traced
// as `pieces` round cones between the balls at u = k/pieces; linear segments
// have end caps, cubic ones are open at ends no segment continues; hits are
// entries only, reporting the touching ball's parameter u and bary.y = -1.
// The basis change to Bezier form and the piece count use the same FP32
// operation sequence as the kernels (so both pick the same pieces); the
// intersection itself is computed here in FP64, independently of the kernels'
// FP32 arithmetic.

// Uniform cubic B-spline and Catmull-Rom (tension 1/2) to Bezier: the standard
// basis-change matrices; linear segments keep their points in slots 0 and 3.
void curve_to_bezier_f32(uint32_t basis, const float q[4][4], float p[4][4]) {
    for (int c = 0; c < 4; c++) {
        if (basis == 0) {
            p[0][c] = p[1][c] = q[0][c];
            p[2][c] = p[3][c] = q[1][c];
        } else if (basis == 1) {
            p[0][c] = (1.0f / 6.0f) * (std::fma(4.0f, q[1][c], q[0][c]) + q[2][c]);
            p[1][c] = (1.0f / 3.0f) * std::fma(2.0f, q[1][c], q[2][c]);
            p[2][c] = (1.0f / 3.0f) * std::fma(2.0f, q[2][c], q[1][c]);
            p[3][c] = (1.0f / 6.0f) * (std::fma(4.0f, q[2][c], q[1][c]) + q[3][c]);
        } else if (basis == 2) {
            p[0][c] = q[1][c];
            p[1][c] = std::fma(1.0f / 6.0f, q[2][c] - q[0][c], q[1][c]);
            p[2][c] = std::fma(-1.0f / 6.0f, q[3][c] - q[1][c], q[2][c]);
            p[3][c] = q[2][c];
        } else {
            p[0][c] = q[0][c];
            p[1][c] = q[1][c];
            p[2][c] = q[2][c];
            p[3][c] = q[3][c];
        }
    }
}

float norm2_4(const float *x) { return (x[0] * x[0] + x[1] * x[1]) + (x[2] * x[2] + x[3] * x[3]); }

// Chord count: eps = 0.05 max(r_max, 1e-3 |P3 - P0|), D = larger 4-D second
// difference, pieces = ceil(sqrt(0.75 D / eps)) in [1, 32] (chord deviation
// bound 0.75 D h^2).
uint32_t curve_pieces_f32(uint32_t basis, const float p[4][4]) {
    if (basis == 0) return 1u;
    float d0[4], d1[4];
    for (int c = 0; c < 4; c++) {
        d0[c] = (p[0][c] - 2.0f * p[1][c]) + p[2][c];
        d1[c] = (p[1][c] - 2.0f * p[2][c]) + p[3][c];
    }
    const float D = std::sqrt(std::max(norm2_4(d0), norm2_4(d1)));
    const float rmax = std::max(std::max(p[0][3], p[1][3]), std::max(p[2][3], p[3][3]));
    const float ch[4] = {p[3][0] - p[0][0], p[3][1] - p[0][1], p[3][2] - p[0][2], 0.0f};
    const float len = std::sqrt(norm2_4(ch));
    const float eps = 0.05f * std::max(rmax, 1e-3f * len);
    if (!(D > 0.0f)) return 1u;
    if (!(eps > 0.0f)) return 32u;
    const float n = std::ceil(std::sqrt((0.75f * D) / eps));
    if (!(n < 32.0f)) return 32u;
    return n < 1.0f ? 1u : uint32_t(n);
}

struct CurveSeg {
    double p[4][4];  // Bezier points (x, y, z, radius)
    double lo[3], hi[3];
    uint32_t pieces, flags;
};

double dot3(const double *a, const double *b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }

// Interval of the line o + t d inside the convex hull of balls a and b
// (radius in [3]); false if the line misses it.  `part_in`: 0 / 1 / 2 for an
// entry on ball a, the cone between the tangent circles, ball b.
bool round_cone_interval_f64(const double *o, const double *d, const double *a, const double *b, double &t_in,
                             int &part_in) {
    double ba[3] = {b[0] - a[0], b[1] - a[1], b[2] - a[2]};
    const double L = std::sqrt(dot3(ba, ba));
    const double ra = a[3], rb = b[3];
    const double dd = dot3(d, d);
    t_in = HUGE_VAL;
    part_in = -1;
    auto ball = [&](const double *c, double r, int which) {
        const double oc[3] = {o[0] - c[0], o[1] - c[1], o[2] - c[2]};
        const double hb = dot3(oc, d), cc = dot3(oc, oc) - r * r;
        const double disc = hb * hb - dd * cc;
        if (disc < 0.0) return;
        const double t = (-hb - std::sqrt(disc)) / dd;
        if (t < t_in) {
            t_in = t;
            part_in = which;
        }
    };
    if (!(L > std::fabs(ra - rb))) {  // one ball holds the other
        if (ra >= rb)
            ball(a, ra, 3);
        else
            ball(b, rb, 3);
        return part_in >= 0;
    }
    ball(a, ra, 0);
    ball(b, rb, 2);
    const double w[3] = {ba[0] / L, ba[1] / L, ba[2] / L};
    const double sn = (ra - rb) / L, c2 = 1.0 - sn * sn;
    const double q0[3] = {o[0] - a[0], o[1] - a[1], o[2] - a[2]};
    const double s0 = dot3(q0, w), sd = dot3(d, w);
    const double s_lo = ra * sn, s_hi = L + rb * sn;
    double lo = -HUGE_VAL, hi = HUGE_VAL;
    if (sd != 0.0) {
        const double t1 = (s_lo - s0) / sd, t2 = (s_hi - s0) / sd;
        lo = std::min(t1, t2);
        hi = std::max(t1, t2);
    } else if (!(s0 >= s_lo && s0 <= s_hi)) {
        return part_in >= 0;
    }
    // inside the cone: c2 (|q|^2 - s^2) <= (ra - s sn)^2, i.e. A t^2 + 2 hB t + C <= 0
    const double A = c2 * dd - sd * sd;
    const double hB = c2 * dot3(q0, d) - s0 * sd + ra * sn * sd;
    const double C = c2 * dot3(q0, q0) - s0 * s0 + 2.0 * ra * sn * s0 - ra * ra;
    bool ok = true;
    if (A != 0.0) {
        const double disc = hB * hB - A * C;
        if (disc >= 0.0) {
            const double sq = std::sqrt(disc);
            double r1 = (-hB - sq) / A, r2 = (-hB + sq) / A;
            if (r1 > r2) std::swap(r1, r2);
            if (A > 0.0) {
                lo = std::max(lo, r1);
                hi = std::min(hi, r2);
            } else if (lo <= std::min(hi, r1)) {
                hi = std::min(hi, r1);
            } else {
                lo = std::max(lo, r2);
            }
        } else if (A > 0.0) {
            ok = false;
        }
    } else if (hB != 0.0) {
        const double tr = -C / (2.0 * hB);
        if (hB > 0.0)
            hi = std::min(hi, tr);
        else
            lo = std::max(lo, tr);
    } else if (C > 0.0) {
        ok = false;
    }
    if (ok && lo <= hi && lo < t_in) {
        t_in = lo;
        part_in = 1;
    }
    return part_in >= 0;
}

// Closest entry (t in [tmin, tmax]) into a curve segment; u = curve parameter.
bool curve_hit_f64(const CurveSeg &sg, const double *o, const double *d, double tmin, double tmax, double &t_out,
                   double &u_out) {
    bool found = false;
    const uint32_t n = sg.pieces;
    auto at = [&](uint32_t k, double *c) {
        if (k == 0) {
            for (int j = 0; j < 4; j++) c[j] = sg.p[0][j];
        } else if (k == n) {
            for (int j = 0; j < 4; j++) c[j] = sg.p[3][j];
        } else {
            const double u = double(k) / double(n), s = 1.0 - u;
            const double b0 = s * s * s, b1 = 3.0 * u * s * s, b2 = 3.0 * u * u * s, b3 = u * u * u;
            for (int j = 0; j < 4; j++) c[j] = b0 * sg.p[0][j] + b1 * sg.p[1][j] + b2 * sg.p[2][j] + b3 * sg.p[3][j];
        }
        c[3] = std::max(c[3], 0.0);
    };
    double c0[4], c1[4];
    at(0, c0);
    for (uint32_t k = 0; k < n; k++) {
        at(k + 1, c1);
        double t;
        int part;
        if ((c0[3] > 0.0 || c1[3] > 0.0) && round_cone_interval_f64(o, d, c0, c1, t, part) && t >= tmin &&
            t <= tmax) {
            const bool open_cap = (part == 0 && k == 0 && (sg.flags & 1u)) || (part == 2 && k + 1 == n && (sg.flags & 2u));
            if (!open_cap) {
                double ul;
                if (part == 0)
                    ul = 0.0;
                else if (part == 2)
                    ul = 1.0;
                else if (part == 3)
                    ul = c0[3] >= c1[3] ? 0.0 : 1.0;
                else {  // cone side: the touching ball's centre lies rho tan(theta) before the point along the axis
                    double ba[3] = {c1[0] - c0[0], c1[1] - c0[1], c1[2] - c0[2]};
                    const double L = std::sqrt(dot3(ba, ba));
                    const double x[3] = {o[0] + t * d[0] - c0[0], o[1] + t * d[1] - c0[1], o[2] + t * d[2] - c0[2]};
                    const double s = dot3(x, ba) / L;
                    const double rho = std::sqrt(std::max(dot3(x, x) - s * s, 0.0));
                    const double sn = (c0[3] - c1[3]) / L;
                    ul = std::min(std::max((s - rho * sn / std::sqrt(1.0 - sn * sn)) / L, 0.0), 1.0);
                }
                tmax = t;
                t_out = t;
                u_out = std::min((double(k) + ul) / double(n), 1.0);
                found = true;
            }
        }
        std::memcpy(c0, c1, sizeof(c0));
    }
    return found;
}

}  // namespace

extern "C" {

void *lcxo_mesh_create(const float *verts, size_t stride_floats, size_t vertex_count, const uint32_t *tris,
                       size_t tri_count, int leaf_size, int bins) {
    auto *m = new Mesh;
    m->vertex_count = vertex_count;
    m->v.resize(3 * vertex_count);
    for (size_t i = 0; i < vertex_count; i++)
        for (int k = 0; k < 3; k++) m->v[3 * i + k] = verts[i * stride_floats + k];
    m->t.assign(tris, tris + 3 * tri_count);
    std::vector<Box> boxes(tri_count);
    for (size_t p = 0; p < tri_count; p++) {
        if (!m->tri_valid(uint32_t(p))) continue;  // empty box
        for (int j = 0; j < 3; j++) boxes[p].grow(m->vert(m->t[3 * p + j]));
    }
    m->bvh.build(boxes, leaf_size > 0 ? leaf_size : 4, bins > 1 ? bins : 32);
    return m;
}

void lcxo_mesh_destroy(void *mesh) { delete static_cast<Mesh *>(mesh); }
double lcxo_mesh_sah(const void *mesh) { return static_cast<const Mesh *>(mesh)->bvh.sah(); }
uint32_t lcxo_mesh_depth(const void *mesh) { return static_cast<const Mesh *>(mesh)->bvh.depth; }

void *lcxo_accel_create(size_t n, void *const *meshes, const float *o2w, const uint32_t *masks) {
    auto *a = new Accel;
    a->mesh.resize(n);
    a->o2w.assign(o2w, o2w + 12 * n);
    a->w2o.resize(12 * n);
    a->w2o64.resize(12 * n);
    a->mask.assign(masks, masks + n);
    std::vector<Box> boxes(n);
    for (size_t i = 0; i < n; i++) {
        a->mesh[i] = static_cast<const Mesh *>(meshes[i]);
        affine_inverse_f32(&o2w[12 * i], &a->w2o[12 * i]);
        affine_inverse_f64(&o2w[12 * i], &a->w2o64[12 * i]);
        const Mesh *m = a->mesh[i];
        if (!m || m->bvh.nodes.empty() || m->bvh.nodes[0].box.empty()) continue;
        const Box &lb = m->bvh.nodes[0].box;
        // world box of the 8 transformed corners, widened by a relative ulp so
        // the FP32 corner arithmetic cannot shrink it
        for (int c = 0; c < 8; c++) {
            const double p[3] = {(c & 1) ? lb.hi[0] : lb.lo[0], (c & 2) ? lb.hi[1] : lb.lo[1],
                                 (c & 4) ? lb.hi[2] : lb.lo[2]};
            float q[3];
            for (int k = 0; k < 3; k++) {
                const float *r = &o2w[12 * i + 4 * k];
                const double w = r[0] * p[0] + r[1] * p[1] + r[2] * p[2] + r[3];
                q[k] = float(w);
            }
            boxes[i].grow(q);
        }
        for (int k = 0; k < 3; k++) {
            const float pad = 1e-6f * std::max(std::fabs(boxes[i].lo[k]), std::fabs(boxes[i].hi[k])) + 1e-30f;
            boxes[i].lo[k] -= pad;
            boxes[i].hi[k] += pad;
        }
    }
    a->bvh.build(boxes, 1, 32);
    return a;
}

void lcxo_accel_destroy(void *accel) { delete static_cast<Accel *>(accel); }

void lcxo_trace_closest(const void *accel, const LcxoRay *rays, size_t n, uint32_t mask, LcxoHit *hits,
                        int threads) {
    const Accel &a = *static_cast<const Accel *>(accel);
    parallel_rays(n, threads, [&](size_t i) {
        LcxoHit h;
        trace_accel<false>(a, rays[i], mask, h);
        if (h.inst == kInvalid) h = LcxoHit{kInvalid, kInvalid, 0.0f, 0.0f, rays[i].tmax, 0};
        hits[i] = h;
    });
}

void lcxo_trace_any(const void *accel, const LcxoRay *rays, size_t n, uint32_t mask, uint8_t *occluded,
                    int threads) {
    const Accel &a = *static_cast<const Accel *>(accel);
    parallel_rays(n, threads, [&](size_t i) {
        LcxoHit h;
        occluded[i] = trace_accel<true>(a, rays[i], mask, h) ? 1 : 0;
    });
}

void lcxo_brute_closest(const void *accel, const LcxoRay *rays, size_t n, uint32_t mask, LcxoHit *hits,
                        int threads) {
    const Accel &a = *static_cast<const Accel *>(accel);
    parallel_rays(n, threads, [&](size_t i) {
        const LcxoRay &ray = rays[i];
        LcxoHit best{kInvalid, kInvalid, 0.0f, 0.0f, ray.tmax, 0};
        for (uint32_t id = 0; id < a.mesh.size(); id++) {
            const Mesh *m = a.mesh[id];
            if (!m || (a.mask[id] & mask) == 0u) continue;
            float oo[3], od[3];
            transform_ray_f32(&a.w2o[12 * size_t(id)], ray.o, ray.d, oo, od);
            WtRay wr;
            wt_setup(wr, oo, od, ray.tmin, ray.tmax);
            for (uint32_t p = 0; p < m->t.size() / 3; p++) {
                if (!m->tri_valid(p)) continue;
                float t, u, v;
                if (wt_intersect(wr, m->vert(m->t[3 * p]), m->vert(m->t[3 * p + 1]), m->vert(m->t[3 * p + 2]), t, u,
                                 v) &&
                    better(t, id, p, best))
                    best = LcxoHit{id, p, u, v, t, 0};
            }
        }
        if (best.inst == kInvalid) best = LcxoHit{kInvalid, kInvalid, 0.0f, 0.0f, ray.tmax, 0};
        hits[i] = best;
    });
}

void lcxo_fp64_closest(const void *accel, const LcxoRay *rays, size_t n, uint32_t mask, LcxoHit *hits,
                       double *t64, int threads) {
    const Accel &a = *static_cast<const Accel *>(accel);
    parallel_rays(n, threads, [&](size_t i) {
        LcxoHit h;
        double t;
        trace_accel64(a, rays[i], mask, h, t);
        hits[i] = h;
        if (t64) t64[i] = t;
    });
}

void lcxo_fp64_eval(const void *accel, const LcxoRay *rays, size_t n, const uint32_t *inst, const uint32_t *prim,
                    LcxoF64Hit *out) {
    const Accel &a = *static_cast<const Accel *>(accel);
    for (size_t i = 0; i < n; i++) {
        out[i] = LcxoF64Hit{0, 0, 0.0, 0.0, 0.0, -1.0};
        const uint32_t id = inst[i], p = prim[i];
        if (id >= a.mesh.size() || !a.mesh[id]) continue;
        const Mesh &m = *a.mesh[id];
        if (p >= m.t.size() / 3 || !m.tri_valid(p)) continue;
        const double *w = &a.w2o64[12 * size_t(id)];
        const LcxoRay &ray = rays[i];
        double oo[3], od[3];
        for (int k = 0; k < 3; k++) {
            oo[k] = w[4 * k] * ray.o[0] + w[4 * k + 1] * ray.o[1] + w[4 * k + 2] * ray.o[2] + w[4 * k + 3];
            od[k] = w[4 * k] * ray.d[0] + w[4 * k + 1] * ray.d[1] + w[4 * k + 2] * ray.d[2];
        }
        WtRay64 wr;
        wt_setup64(wr, oo, od, ray.tmin, ray.tmax);
        double v0[3], v1[3], v2[3];
        for (int k = 0; k < 3; k++) {
            v0[k] = m.vert(m.t[3 * p])[k];
            v1[k] = m.vert(m.t[3 * p + 1])[k];
            v2[k] = m.vert(m.t[3 * p + 2])[k];
        }
        double t, u, v, mb;
        out[i].hit = wt_eval64(wr, v0, v1, v2, t, u, v, mb) ? 1 : 0;
        out[i].t = t;
        out[i].u = u;
        out[i].v = v;
        out[i].min_bary = mb;
    }
}

void lcxo_pathtrace(const void *accel, const float *const *albedo, const LcxoPtParams *params, float *image,
                    LcxoHit *first_hits, int threads) {
    const Accel &a = *static_cast<const Accel *>(accel);
    const LcxoPtParams P = *params;
    const size_t n = size_t(P.width) * P.height * P.spp;
    std::vector<float> rad(3 * n, 0.0f);
    parallel_rays(n, threads, [&](size_t idx) {
        using namespace lcx::pt;
        const uint32_t i = uint32_t(idx);
        const uint32_t pixel = i / P.spp;
        const uint32_t px = pixel % P.width, py = pixel / P.width;
        float fwd[3] = {P.target[0] - P.eye[0], P.target[1] - P.eye[1], P.target[2] - P.eye[2]};
        normalize3(fwd);
        float right[3] = {fwd[1] * P.up[2] - fwd[2] * P.up[1], fwd[2] * P.up[0] - fwd[0] * P.up[2],
                          fwd[0] * P.up[1] - fwd[1] * P.up[0]};
        normalize3(right);
        const float up[3] = {right[1] * fwd[2] - right[2] * fwd[1], right[2] * fwd[0] - right[0] * fwd[2],
                             right[0] * fwd[1] - right[1] * fwd[0]};
        const float jx = uniform(P.seed, i, 0, 0), jy = uniform(P.seed, i, 0, 1);
        const float sx = ((((float(px) + jx) / float(P.width)) * 2.0f - 1.0f) * P.tan_half_fov) *
                         (float(P.width) / float(P.height));
        const float sy = (1.0f - ((float(py) + jy) / float(P.height)) * 2.0f) * P.tan_half_fov;
        float d[3];
        for (int k = 0; k < 3; k++) d[k] = std::fma(sx, right[k], std::fma(sy, up[k], fwd[k]));
        normalize3(d);
        LcxoRay ray{{P.eye[0], P.eye[1], P.eye[2]}, 0.0f, {d[0], d[1], d[2]}, 1e30f};
        float T[3] = {1.0f, 1.0f, 1.0f}, R[3] = {0.0f, 0.0f, 0.0f};
        for (uint32_t b = 0; b < P.max_bounces; b++) {
            LcxoHit h;
            trace_accel<false>(a, ray, 0xffu, h);
            if (h.inst == kInvalid) h = LcxoHit{kInvalid, kInvalid, 0.0f, 0.0f, ray.tmax, 0};
            if (b == 0 && first_hits) first_hits[i] = h;
            if (h.inst == kInvalid) {
                for (int k = 0; k < 3; k++) R[k] = std::fma(T[k], P.env[k], R[k]);
                break;
            }
            const Mesh &m = *a.mesh[h.inst];
            const float *v0 = m.vert(m.t[3 * h.prim]), *v1 = m.vert(m.t[3 * h.prim + 1]),
                        *v2 = m.vert(m.t[3 * h.prim + 2]);
            const float e1[3] = {v1[0] - v0[0], v1[1] - v0[1], v1[2] - v0[2]};
            const float e2[3] = {v2[0] - v0[0], v2[1] - v0[1], v2[2] - v0[2]};
            const float no[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2],
                                 e1[0] * e2[1] - e1[1] * e2[0]};
            const float *w = &a.w2o[12 * size_t(h.inst)];
            float N[3];
            for (int k = 0; k < 3; k++) N[k] = std::fma(w[k], no[0], std::fma(w[4 + k], no[1], w[8 + k] * no[2]));
            normalize3(N);
            if (std::fma(N[0], ray.d[0], std::fma(N[1], ray.d[1], N[2] * ray.d[2])) > 0.0f)
                for (int k = 0; k < 3; k++) N[k] = -N[k];
            const float p[3] = {std::fma(h.t, ray.d[0], ray.o[0]), std::fma(h.t, ray.d[1], ray.o[1]),
                                std::fma(h.t, ray.d[2], ray.o[2])};
            const float po[3] = {offset_coord(p[0], N[0]), offset_coord(p[1], N[1]), offset_coord(p[2], N[2])};
            const float alb = albedo[h.inst][h.prim];
            float wl[3] = {P.light_pos[0] - po[0], P.light_pos[1] - po[1], P.light_pos[2] - po[2]};
            const float dist2 = std::fma(wl[0], wl[0], std::fma(wl[1], wl[1], wl[2] * wl[2]));
            const float dist = std::sqrt(dist2);
            for (int k = 0; k < 3; k++) wl[k] = wl[k] / dist;
            const float cosl = std::fma(N[0], wl[0], std::fma(N[1], wl[1], N[2] * wl[2]));
            if (cosl > 0.0f) {
                LcxoRay sr{{po[0], po[1], po[2]}, 0.0f, {wl[0], wl[1], wl[2]}, dist};
                LcxoHit sh;
                if (!trace_accel<true>(a, sr, 0xffu, sh)) {
                    const float f = ((alb * 0.318309886f) * cosl) / dist2;
                    for (int k = 0; k < 3; k++) R[k] = R[k] + (T[k] * f) * P.light_intensity[k];
                }
            }
            if (b + 1 >= P.max_bounces) break;
            for (int k = 0; k < 3; k++) T[k] = T[k] * alb;
            if (b + 1 >= P.rr_start) {
                const float q = std::fmin(0.95f, std::fmax(T[0], std::fmax(T[1], T[2])));
                if (uniform(P.seed, i, b + 1, 2) >= q) break;
                for (int k = 0; k < 3; k++) T[k] = T[k] / q;
            }
            float nd[3];
            cosine_dir(N, uniform(P.seed, i, b + 1, 0), uniform(P.seed, i, b + 1, 1), nd);
            ray = LcxoRay{{po[0], po[1], po[2]}, 0.0f, {nd[0], nd[1], nd[2]}, 1e30f};
        }
        for (int k = 0; k < 3; k++) rad[3 * size_t(i) + k] = R[k];
    });
    const float inv = 1.0f / float(P.spp);
    for (size_t pix = 0; pix < size_t(P.width) * P.height; pix++)
        for (int k = 0; k < 3; k++) {
            float acc = 0.0f;
            for (uint32_t s = 0; s < P.spp; s++) acc = acc + rad[3 * (pix * P.spp + s) + k];
            image[3 * pix + k] = acc * inv;
        }
}

void lcxo_affine_inverse(const float *o2w, float *w2o) { affine_inverse_f32(o2w, w2o); }

// include/lcx/bvh_device.cuh srt_matrix, operation for operation
static void srt_matrix_f32(const float *v, float m[12]) {
    const float px = v[0], py = v[1], pz = v[2];
    float qx = v[3], qy = v[4], qz = v[5], qw = v[6];
    const float sx = v[7], sy = v[8], sz = v[9], a = v[10], b = v[11], c = v[12];
    const float tx = v[13], ty = v[14], tz = v[15];
    const float n2 = std::fma(qx, qx, std::fma(qy, qy, std::fma(qz, qz, qw * qw)));
    const float rn = 1.0f / std::sqrt(n2);
    qx = qx * rn;
    qy = qy * rn;
    qz = qz * rn;
    qw = qw * rn;
    const float xx = qx * qx, yy = qy * qy, zz = qz * qz;
    const float xy = qx * qy, xz = qx * qz, yz = qy * qz;
    const float wx = qw * qx, wy = qw * qy, wz = qw * qz;
    const float R[9] = {1.0f - 2.0f * (yy + zz), 2.0f * (xy - wz), 2.0f * (xz + wy),
                        2.0f * (xy + wz), 1.0f - 2.0f * (xx + zz), 2.0f * (yz - wx),
                        2.0f * (xz - wy), 2.0f * (yz + wx), 1.0f - 2.0f * (xx + yy)};
    for (int r = 0; r < 3; r++) {
        const float r0 = R[3 * r], r1 = R[3 * r + 1], r2 = R[3 * r + 2];
        m[4 * r + 0] = r0 * sx;
        m[4 * r + 1] = std::fma(r0, a, r1 * sy);
        m[4 * r + 2] = std::fma(r0, b, std::fma(r1, c, r2 * sz));
        m[4 * r + 3] = std::fma(r0, px, std::fma(r1, py, r2 * pz)) + (r == 0 ? tx : (r == 1 ? ty : tz));
    }
}

// include/lcx/bvh_device.cuh motion_segment, operation for operation
static bool motion_segment_f32(float t0, float t1, uint32_t count, uint32_t flags, float time, uint32_t &i, float &f) {
    if ((flags & 1u) && time < t0) return false;
    if ((flags & 2u) && time > t1) return false;
    float u = (time - t0) / (t1 - t0);
    u = u >= 0.0f ? (u <= 1.0f ? u : 1.0f) : 0.0f;
    const float x = u * float(count - 1u);
    i = uint32_t(std::floor(x));
    if (i > count - 2u) i = count - 2u;
    f = x - float(i);
    return true;
}

// include/lcx/bvh_device.cuh motion_matrix, operation for operation
static bool motion_matrix_f32(const LcxoMotion &md, float time, float m[12]) {
    uint32_t i;
    float f;
    if (!motion_segment_f32(md.t0, md.t1, md.count, md.flags, time, i, f)) return false;
    if (md.flags & 4u) {  // SRT records
        const float *k0 = md.keys + 16 * size_t(i), *k1 = k0 + 16;
        float v[16];
        for (int k = 0; k < 16; k++) v[k] = std::fma(f, k1[k] - k0[k], k0[k]);
        srt_matrix_f32(v, m);
        return true;
    }
    const float *k0 = md.keys + 12 * size_t(i), *k1 = k0 + 12;
    for (int k = 0; k < 12; k++) m[k] = std::fma(f, k1[k] - k0[k], k0[k]);
    return true;
}

// Every triangle of a keyframed-vertex mesh at `time` (motion_triangle of
// include/lcx/bvh_device.cuh, operation for operation), in object space.
static bool trace_motion_mesh(bool kAny, const LcxoMeshMotion &mm, uint32_t inst, const float *o, const float *d,
                              float tmin, float time, LcxoHit &best) {
    uint32_t seg;
    float f;
    if (!motion_segment_f32(mm.t0, mm.t1, mm.keys, mm.flags, time, seg, f)) return false;
    WtRay wr;
    wt_setup(wr, o, d, tmin, best.t);
    for (uint32_t p = 0; p < mm.tri_count; p++) {
        float v[3][3];
        bool ok = true;
        for (int k = 0; k < 3 && ok; k++) {
            const uint32_t idx = mm.tris[3 * size_t(p) + k];
            if (idx >= mm.vcount) {
                ok = false;
                break;
            }
            const float *p0 = mm.verts + mm.stride_floats * (size_t(seg) * mm.vcount + idx);
            const float *p1 = mm.verts + mm.stride_floats * (size_t(seg + 1u) * mm.vcount + idx);
            for (int j = 0; j < 3; j++) v[k][j] = std::fma(f, p1[j] - p0[j], p0[j]);
        }
        if (!ok) continue;
        float t, u, w;
        wr.tmax = best.t;
        if (wt_intersect(wr, v[0], v[1], v[2], t, u, w)) {
            if (kAny) return true;
            if (better(t, inst, p, best)) best = LcxoHit{inst, p, u, w, t, 0};
        }
    }
    return false;
}

void lcxo_trace_motion(const void *accel, const LcxoMotion *motion, const LcxoMeshMotion *mesh_motion,
                       const LcxoRay *rays, const float *times, size_t n, uint32_t mask, int any, LcxoHit *hits,
                       uint8_t *occluded, int threads) {
    const Accel &a = *static_cast<const Accel *>(accel);
    parallel_rays(n, threads, [&](size_t r) {
        const LcxoRay &ray = rays[r];
        LcxoHit best{kInvalid, kInvalid, 0.0f, 0.0f, ray.tmax, 0};
        bool occ = false;
        for (uint32_t id = 0; id < a.mesh.size() && !occ; id++) {
            const Mesh *m = a.mesh[id];
            if (!m || (a.mask[id] & mask) == 0u) continue;
            float w[12];
            const float *wp = &a.w2o[12 * size_t(id)];
            if (motion[id].keys != nullptr) {
                float mm[12];
                if (!motion_matrix_f32(motion[id], times[r], mm)) continue;
                affine_inverse_f32(mm, w);
                wp = w;
            }
            float oo[3], od[3];
            transform_ray_f32(wp, ray.o, ray.d, oo, od);
            if (mesh_motion != nullptr && mesh_motion[id].verts != nullptr) {
                if (any) {
                    if (trace_motion_mesh(true, mesh_motion[id], id, oo, od, ray.tmin, times[r], best)) occ = true;
                } else {
                    trace_motion_mesh(false, mesh_motion[id], id, oo, od, ray.tmin, times[r], best);
                }
            } else if (any) {
                if (trace_mesh<true>(*m, id, oo, od, ray.tmin, best)) occ = true;
            } else {
                trace_mesh<false>(*m, id, oo, od, ray.tmin, best);
            }
        }
        if (any) {
            occluded[r] = occ ? 1 : 0;
        } else {
            if (best.inst == kInvalid) best = LcxoHit{kInvalid, kInvalid, 0.0f, 0.0f, ray.tmax, 0};
            hits[r] = best;
        }
    });
}

int lcxo_intersect_triangle(const float *o, const float *d, float tmin, float tmax, const float *v0, const float *v1,
                            const float *v2, float *t, float *u, float *v) {
    WtRay wr;
    wt_setup(wr, o, d, tmin, tmax);
    return wt_intersect(wr, v0, v1, v2, *t, *u, *v) ? 1 : 0;
}




// Curves: segs holds keys x nseg segments, keyframe-major.  The cone count of a
// segment is the largest over its keyframes (the kernels' choice).
struct CurveObj {
    uint32_t keys = 1;
    float t0 = 0.0f, t1 = 1.0f;
    uint32_t mflags = 0;
    size_t nseg = 0;
    std::vector<CurveSeg> segs;
};

void *lcxo_curve_create_motion(const float *control_points, size_t cp_stride_floats, size_t cp_per_key, uint32_t keys,
                               const uint32_t *segments, size_t seg_count, uint32_t basis, float t0, float t1,
                               uint32_t flags) {
    auto *cv = new CurveObj();
    cv->keys = keys < 1 ? 1 : keys;
    cv->t0 = t0;
    cv->t1 = t1;
    cv->mflags = flags;
    cv->nseg = seg_count;
    cv->segs.resize(size_t(cv->keys) * seg_count);
    const uint32_t need = basis == 0 ? 2u : 4u;
    for (size_t i = 0; i < seg_count; i++) {
        const uint32_t first = segments[i];
        if (first > cp_per_key || cp_per_key - first < need) {  // the product reports this as an error
            delete cv;
            return nullptr;
        }
        uint32_t pieces = 1, flags_i = 0;
        if (basis != 0) {
            const uint32_t step = basis == 3 ? 3u : 1u;
            if (!(i > 0 && segments[i - 1] + step == first)) flags_i |= 1u;
            if (!(i + 1 < seg_count && segments[i + 1] == first + step)) flags_i |= 2u;
        }
        for (uint32_t key = 0; key < cv->keys; key++) {
            CurveSeg &sg = cv->segs[size_t(key) * seg_count + i];
            float q[4][4], p[4][4];
            for (uint32_t k = 0; k < 4; k++)
                for (int c = 0; c < 4; c++)
                    q[k][c] = control_points[(size_t(key) * cp_per_key + first + std::min(k, need - 1)) *
                                                 cp_stride_floats + c];
            curve_to_bezier_f32(basis, q, p);
            pieces = std::max(pieces, curve_pieces_f32(basis, p));
            sg.flags = flags_i;
            double pad = 0.0;
            for (int k = 0; k < 4; k++) {
                for (int c = 0; c < 4; c++) sg.p[k][c] = p[k][c];
                pad = std::max(pad, sg.p[k][3]);
            }
            for (int c = 0; c < 3; c++) {
                sg.lo[c] = std::min(std::min(sg.p[0][c], sg.p[1][c]), std::min(sg.p[2][c], sg.p[3][c])) - pad;
                sg.hi[c] = std::max(std::max(sg.p[0][c], sg.p[1][c]), std::max(sg.p[2][c], sg.p[3][c])) + pad;
            }
        }
        for (uint32_t key = 0; key < cv->keys; key++) cv->segs[size_t(key) * seg_count + i].pieces = pieces;
    }
    return cv;
}

void *lcxo_curve_create(const float *control_points, size_t cp_stride_floats, size_t cp_count,
                        const uint32_t *segments, size_t seg_count, uint32_t basis) {
    return lcxo_curve_create_motion(control_points, cp_stride_floats, cp_count, 1, segments, seg_count, basis, 0.0f,
                                    1.0f, 0u);
}

void lcxo_curve_destroy(void *curve) { delete static_cast<CurveObj *>(curve); }

uint32_t lcxo_curve_pieces(const void *curve, size_t segment) {
    return static_cast<const CurveObj *>(curve)->segs[segment].pieces;
}

void lcxo_trace_curves_t(void *const *inst_curve, const float *o2w, const uint32_t *inst_mask, size_t instance_count,
                         const LcxoRay *rays, const float *times, size_t n, uint32_t mask, int any, LcxoHit *hits,
                         uint8_t *occluded, int threads) {
    std::vector<float> w2o(12 * instance_count);
    for (size_t i = 0; i < instance_count; i++) affine_inverse_f32(&o2w[12 * i], &w2o[12 * i]);
    parallel_rays(n, threads, [&](size_t r) {
        const LcxoRay &ray = rays[r];
        const float time = times != nullptr ? times[r] : 0.0f;
        LcxoHit best{kInvalid, kInvalid, 0.0f, 0.0f, ray.tmax, 0};
        double best_t = ray.tmax;
        bool occ = false;
        for (uint32_t id = 0; id < instance_count && !occ; id++) {
            const auto *cv = static_cast<const CurveObj *>(inst_curve[id]);
            if (!cv || (inst_mask[id] & mask) == 0u) continue;
            uint32_t key = 0;
            float f = 0.0f;
            if (cv->keys > 1 && !motion_segment_f32(cv->t0, cv->t1, cv->keys, cv->mflags, time, key, f)) continue;
            float oo[3], od[3];
            transform_ray_f32(&w2o[12 * size_t(id)], ray.o, ray.d, oo, od);
            const double o[3] = {oo[0], oo[1], oo[2]}, d[3] = {od[0], od[1], od[2]};
            for (uint32_t k = 0; k < cv->nseg && !occ; k++) {
                const CurveSeg &s0 = cv->segs[size_t(key) * cv->nseg + k];
                CurveSeg sg = s0;
                if (cv->keys > 1) {  // the Bezier points at the ray's time; the box covers both keyframes
                    const CurveSeg &s1 = cv->segs[size_t(key + 1) * cv->nseg + k];
                    for (int j = 0; j < 4; j++)
                        for (int c = 0; c < 4; c++) sg.p[j][c] = s0.p[j][c] + double(f) * (s1.p[j][c] - s0.p[j][c]);
                    for (int c = 0; c < 3; c++) {
                        sg.lo[c] = std::min(s0.lo[c], s1.lo[c]);
                        sg.hi[c] = std::max(s0.hi[c], s1.hi[c]);
                    }
                }
                double tn = ray.tmin, tf = best_t;  // slab test against the segment's box
                bool in = true;
                for (int c = 0; c < 3 && in; c++) {
                    if (d[c] == 0.0) {
                        in = o[c] >= sg.lo[c] && o[c] <= sg.hi[c];
                    } else {
                        double t0 = (sg.lo[c] - o[c]) / d[c], t1 = (sg.hi[c] - o[c]) / d[c];
                        if (t0 > t1) std::swap(t0, t1);
                        tn = std::max(tn, t0);
                        tf = std::min(tf, t1);
                        in = tn <= tf * (1.0 + 1e-9) + 1e-12;
                    }
                }
                if (!in) continue;
                double t, u;
                if (!curve_hit_f64(sg, o, d, ray.tmin, best_t, t, u)) continue;
                if (any) {
                    occ = true;
                    break;
                }
                // t <= best_t; equal t goes to the smaller (inst, prim)
                if (t < best_t || id < best.inst || (id == best.inst && k < best.prim)) {
                    best_t = t;
                    best = LcxoHit{id, k, float(u), -1.0f, float(t), 0};
                }
            }
        }
        if (any)
            occluded[r] = occ ? 1 : 0;
        else
            hits[r] = best;
    });
}

void lcxo_trace_curves(void *const *inst_curve, const float *o2w, const uint32_t *inst_mask, size_t instance_count,
                       const LcxoRay *rays, size_t n, uint32_t mask, int any, LcxoHit *hits, uint8_t *occluded,
                       int threads) {
    lcxo_trace_curves_t(inst_curve, o2w, inst_mask, instance_count, rays, nullptr, n, mask, any, hits, occluded,
                        threads);
}

}  // extern "C"
