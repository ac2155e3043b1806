// ORACLE — test infrastructure only.
//
// A scalar C++ restatement of rustracer's per-frame GPU hot path (the WGSL compute shaders in
// rustracer-renderer/shaders/ and the host steps of rustracer-renderer/src/lib.rs that sit between
// them).  It is the parity checker for the CUDA backend and the timed CPU baseline; nothing in the
// product links, loads or calls it.  Parity status: the reference pins only struct layouts and BVH
// invariants in its own tests (rustracer-renderer/tests/gpu_layout.rs, rustracer-core/src/bvh.rs
// tests); radiance, RNG, BSDF, photon grid and denoise are unpinned by the reference, which cannot
// run here (no Rust toolchain, no graphics stack).  Golden vectors under tests/golden/ are made from
// this restatement.
//
// Floating point: built with -ffp-contract=off; every expression keeps the WGSL evaluation order
// (left-to-right, no fused multiply-add).  Choices where WGSL leaves behaviour to the backend:
//   * min/max with a NaN operand return the other operand (IEEE minNum/maxNum, C fminf/fmaxf);
//   * float -> int/uint conversions truncate toward zero and saturate, NaN -> 0;
//   * an out-of-range array index is clamped to the last element (naga's Restrict policy);
//   * normalize(v) = v * (1 / sqrt(dot(v, v))), inverseSqrt(x) = 1 / sqrt(x), mix(a, b, t) =
//     a * (1 - t) + b * t, length(v) = sqrt(dot(v, v)), dot = (x*x' + y*y') + z*z';
//   * textureSampleLevel(level 0, linear, repeat, rgba8unorm) = fp32 bilinear of byte/255 texels,
//     array layer clamped to [0, layers - 1]; an empty role samples as 0;
//   * rgba8unorm stores round to nearest: (u8)(clamp(c, 0, 1) * 255 + 0.5).
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <thread>
#include <vector>

#include "../include/rustracer_cuda.h"

namespace {

constexpr float PI = 3.141592653589793f;  // common.wgsl:8
constexpr float INF = 1e38f;              // common.wgsl:9
constexpr float EPS = 1e-6f;              // common.wgsl:10

struct V3 {
    float x, y, z;
};
inline V3 mk(float x, float y, float z) { return V3{x, y, z}; }
inline V3 ld(const float *p) { return V3{p[0], p[1], p[2]}; }
inline V3 operator+(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V3 operator-(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 operator-(V3 a) { return {-a.x, -a.y, -a.z}; }
inline V3 operator*(V3 a, V3 b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
inline V3 operator*(V3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
inline V3 operator*(float s, V3 a) { return {s * a.x, s * a.y, s * a.z}; }
inline V3 operator/(V3 a, float s) { return {a.x / s, a.y / s, a.z / s}; }
inline V3 operator/(V3 a, V3 b) { return {a.x / b.x, a.y / b.y, a.z / b.z}; }
inline float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline V3 cross(V3 a, V3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
inline float length(V3 a) { return std::sqrt(dot(a, a)); }
inline V3 normalize(V3 a) { return a * (1.0f / std::sqrt(dot(a, a))); }
inline float fmn(float a, float b) { return std::fmin(a, b); }
inline float fmx(float a, float b) { return std::fmax(a, b); }
inline V3 vmin(V3 a, V3 b) { return {fmn(a.x, b.x), fmn(a.y, b.y), fmn(a.z, b.z)}; }
inline V3 vmax(V3 a, V3 b) { return {fmx(a.x, b.x), fmx(a.y, b.y), fmx(a.z, b.z)}; }
inline float clampf(float x, float lo, float hi) { return fmn(fmx(x, lo), hi); }
inline float max3(V3 a) { return fmx(fmx(a.x, a.y), a.z); }
inline float mixf(float a, float b, float t) { return a * (1.0f - t) + b * t; }
inline V3 mix3(V3 a, V3 b, float t) { return a * (1.0f - t) + b * t; }
inline V3 mix3v(V3 a, V3 b, V3 t) {
    return {a.x * (1.0f - t.x) + b.x * t.x, a.y * (1.0f - t.y) + b.y * t.y, a.z * (1.0f - t.z) + b.z * t.z};
}
inline float smoothstepf(float e0, float e1, float x) {
    float t = clampf((x - e0) / (e1 - e0), 0.0f, 1.0f);
    return t * t * (3.0f - 2.0f * t);
}
inline uint32_t f2u(float f) {  // WGSL u32(f32): truncate, saturate, NaN -> 0
    if (!(f > 0.0f)) return 0u;
    if (f >= 4294967296.0f) return 0xFFFFFFFFu;
    return (uint32_t)f;
}
inline int32_t f2i(float f) {  // WGSL i32(f32)
    if (f != f) return 0;
    if (f <= -2147483648.0f) return INT32_MIN;
    if (f >= 2147483648.0f) return INT32_MAX;
    return (int32_t)f;
}

// sin, cos and the integer powers pow(x, 2) / pow(x, 5).  WGSL leaves their accuracy to the backend
// (sin and cos need only 2^-11 absolute error), so the restatement fixes one sequence of IEEE
// operations for them, the one the CUDA backend uses: Cody-Waite reduction by pi/2 with the two-part
// constant 1.5703125 + 4.83826794e-4 (Cody and Waite, Software Manual for the Elementary Functions,
// 1980), then the Taylor series of sin through x^9 and of cos through x^10 on [-pi/4, pi/4], Horner
// form; pow(x, 0.5) on [0, 1] is sqrt(x), pow(x, 2) is x * x, pow(x, 5) is (x^2)^2 * x.
inline void sincos_fixed(float x, float &s, float &c) {
    const float k = std::floor(x * 0.636619772f + 0.5f);
    const float r = (x - k * 1.5703125f) - k * 4.83826794e-4f;
    const float z = r * r;
    const float sr = r + r * z * (-(1.0f / 6.0f) + z * ((1.0f / 120.0f) + z * (-(1.0f / 5040.0f) + z * (1.0f / 362880.0f))));
    const float cr = 1.0f - 0.5f * z +
                     z * z * ((1.0f / 24.0f) + z * (-(1.0f / 720.0f) + z * ((1.0f / 40320.0f) + z * -(1.0f / 3628800.0f))));
    const int q = (int)k & 3;
    s = q == 0 ? sr : (q == 1 ? cr : (q == 2 ? -sr : -cr));
    c = q == 0 ? cr : (q == 1 ? -sr : (q == 2 ? -cr : sr));
}
inline float pow5(float x) {
    const float x2 = x * x;
    return x2 * x2 * x;
}

// ---- common.wgsl:12-25 ------------------------------------------------------------------------
inline V3 reflect(V3 v, V3 n) { return v - 2.0f * dot(v, n) * n; }
inline V3 refract(V3 v, V3 n, float eta) {
    float cos_theta = fmn(dot(-v, n), 1.0f);
    V3 r_out_perp = eta * (v + cos_theta * n);
    V3 r_out_parallel = -std::sqrt(std::fabs(1.0f - dot(r_out_perp, r_out_perp))) * n;
    return r_out_perp + r_out_parallel;
}
inline V3 fresnel_schlick(float cos_theta, V3 f0) {
    float p = pow5(clampf(1.0f - cos_theta, 0.0f, 1.0f));
    return f0 + (mk(1.0f, 1.0f, 1.0f) - f0) * p;
}

// ---- common.wgsl:29-56 (PCG hash RNG) -----------------------------------------------------------
struct Rng {
    uint32_t state, inc;
};
inline Rng rng_init(uint32_t seed) {
    Rng r;
    r.state = seed;
    r.inc = 1u;
    r.state = r.state * 747796405u + 2891336453u;
    r.state = ((r.state >> ((r.state >> 28u) + 4u)) ^ r.state) * 277803737u;
    return r;
}
inline uint32_t rng_next(Rng &r) {
    uint32_t old = r.state;
    r.state = old * 747796405u + r.inc;
    uint32_t word = ((old >> ((old >> 28u) + 4u)) ^ old) * 277803737u;
    return (word >> 22u) ^ word;
}
inline float rng_f32(Rng &r) { return (float)rng_next(r) / 4294967296.0f; }

// ---- common.wgsl:60-74 ------------------------------------------------------------------------
inline V3 sample_cosine_hemisphere(Rng &r) {
    float u1 = rng_f32(r);
    float u2 = rng_f32(r);
    float phi = 2.0f * PI * u1;
    float cos_theta = std::sqrt(u2);
    float sin_theta = std::sqrt(1.0f - u2);
    float sp, cp;
    sincos_fixed(phi, sp, cp);
    return mk(cp * sin_theta, cos_theta, sp * sin_theta);
}
inline V3 to_world(V3 local, V3 normal) {
    V3 up = std::fabs(normal.y) < 0.999f ? mk(0, 1, 0) : mk(1, 0, 0);
    V3 tangent = normalize(cross(up, normal));
    V3 bitangent = cross(normal, tangent);
    return tangent * local.x + normal * local.y + bitangent * local.z;
}

// ---- common.wgsl:78-100 (Moller-Trumbore) --------------------------------------------------------
inline float intersect_triangle(V3 ro, V3 rd, V3 v0, V3 v1, V3 v2) {
    V3 edge1 = v1 - v0;
    V3 edge2 = v2 - v0;
    V3 h = cross(rd, edge2);
    float a = dot(edge1, h);
    if (std::fabs(a) < 1e-7f) return INF;
    float f = 1.0f / a;
    V3 s = ro - v0;
    float u = f * dot(s, h);
    if (u < 0.0f || u > 1.0f) return INF;
    V3 q = cross(s, edge1);
    float v = f * dot(rd, q);
    if (v < 0.0f || u + v > 1.0f) return INF;
    float t = f * dot(edge2, q);
    if (t > EPS) return t;
    return INF;
}

struct Bary {
    float uvx, uvy, u, v;
};
// common.wgsl:178-192
inline Bary barycentric(const rt_triangle &tri, V3 ro, V3 rd, float t) {
    V3 v0 = ld(tri.v0), v1 = ld(tri.v1), v2 = ld(tri.v2);
    V3 e1 = v1 - v0;
    V3 e2 = v2 - v0;
    V3 p = ro + rd * t - v0;
    float d00 = dot(e1, e1), d01 = dot(e1, e2), d11 = dot(e2, e2);
    float d20 = dot(p, e1), d21 = dot(p, e2);
    float denom = d00 * d11 - d01 * d01;
    float u = 0.0f, v = 0.0f;
    if (denom != 0.0f) {
        u = (d11 * d20 - d01 * d21) / denom;
        v = (d00 * d21 - d01 * d20) / denom;
    }
    float w = 1.0f - u - v;
    Bary b;
    b.uvx = tri.uv0[0] * w + tri.uv1[0] * u + tri.uv2[0] * v;
    b.uvy = tri.uv0[1] * w + tri.uv1[1] * u + tri.uv2[1] * v;
    b.u = u;
    b.v = v;
    return b;
}
// common.wgsl:196-201
inline V3 smooth_normal(const rt_triangle &tri, const Bary &b, V3 geometric) {
    float w = 1.0f - b.u - b.v;
    V3 n = ld(tri.n0) * w + ld(tri.n1) * b.u + ld(tri.n2) * b.v;
    if (dot(n, n) < 1e-8f) return geometric;
    return normalize(n);
}
// common.wgsl:211-230
inline void tangent_frame(const rt_triangle &tri, V3 n, V3 *t_out, V3 *b_out) {
    V3 e1 = ld(tri.v1) - ld(tri.v0);
    V3 e2 = ld(tri.v2) - ld(tri.v0);
    float d1x = tri.uv1[0] - tri.uv0[0], d1y = tri.uv1[1] - tri.uv0[1];
    float d2x = tri.uv2[0] - tri.uv0[0], d2y = tri.uv2[1] - tri.uv0[1];
    float det = d1x * d2y - d2x * d1y;
    float f = std::fabs(det) < 1e-12f ? 0.0f : 1.0f / det;
    V3 t = (e1 * d2y - e2 * d1y) * f;
    V3 b = (e2 * d1x - e1 * d2x) * f;
    V3 tt = t - n * dot(n, t);
    if (dot(tt, tt) < 1e-10f) {
        tt = cross(n, mk(1, 0, 0));
        if (dot(tt, tt) < 1e-6f) tt = cross(n, mk(0, 1, 0));
    }
    tt = normalize(tt);
    V3 c = cross(n, tt);
    *t_out = tt;
    *b_out = c * (dot(c, b) > 0.0f ? 1.0f : -1.0f);
}
// common.wgsl:247-251
inline V3 get_triangle_normal(const rt_triangle &tri) {
    V3 edge1 = ld(tri.v1) - ld(tri.v0);
    V3 edge2 = ld(tri.v2) - ld(tri.v0);
    return normalize(cross(edge1, edge2));
}

struct Rgba {
    float r, g, b, a;
};

// textureSampleLevel(t, linear/repeat sampler, uv, layer, 0.0) on an rgba8unorm 2-D array.
inline Rgba tex_sample(const rt_texture_array &t, float u, float v, int32_t layer) {
    if (!t.rgba8 || t.layers == 0 || t.width == 0 || t.height == 0) return Rgba{0, 0, 0, 0};
    int32_t L = layer < 0 ? 0 : (layer >= (int32_t)t.layers ? (int32_t)t.layers - 1 : layer);
    const uint32_t W = t.width, H = t.height;
    float fu = u - std::floor(u), fv = v - std::floor(v);
    if (!(fu >= 0.0f)) fu = 0.0f;
    if (!(fv >= 0.0f)) fv = 0.0f;
    float x = fu * (float)W - 0.5f, y = fv * (float)H - 0.5f;
    float x0f = std::floor(x), y0f = std::floor(y);
    float ax = x - x0f, ay = y - y0f;
    int32_t x0 = (int32_t)x0f, y0 = (int32_t)y0f;
    if (x0 < 0) x0 += (int32_t)W;
    if (y0 < 0) y0 += (int32_t)H;
    if (x0 >= (int32_t)W) x0 -= (int32_t)W;
    if (y0 >= (int32_t)H) y0 -= (int32_t)H;
    int32_t x1 = x0 + 1 == (int32_t)W ? 0 : x0 + 1;
    int32_t y1 = y0 + 1 == (int32_t)H ? 0 : y0 + 1;
    const uint8_t *base = t.rgba8 + (size_t)L * W * H * 4;
    auto texel = [&](int32_t xx, int32_t yy, int c) { return (float)base[((size_t)yy * W + xx) * 4 + c] / 255.0f; };
    float out[4];
    for (int c = 0; c < 4; ++c) {
        float top = texel(x0, y0, c) * (1.0f - ax) + texel(x1, y0, c) * ax;
        float bot = texel(x0, y1, c) * (1.0f - ax) + texel(x1, y1, c) * ax;
        out[c] = top * (1.0f - ay) + bot * ay;
    }
    return Rgba{out[0], out[1], out[2], out[3]};
}
inline int32_t layer_of(uint32_t tex) { return (int32_t)tex; }  // WGSL i32(u32): bit cast

struct Hit {
    float t;
    uint32_t prim_id;
};

// An empty array reads as one zero element (the index clamp then has a target).
static const rt_triangle kZeroTri = {};
static const rt_material kZeroMat = {};

struct Scene {
    const rt_scene_desc *d;
    const rt_triangle &tri(uint32_t i) const {
        uint64_t n = d->triangle_count;
        return n ? d->triangles[i < n ? i : n - 1] : kZeroTri;
    }
    const rt_material &mat(uint32_t i) const {
        uint64_t n = d->material_count;
        return n ? d->materials[i < n ? i : n - 1] : kZeroMat;
    }
    // gather.wgsl:66-88 (photon_trace.wgsl:31-81 is the same traversal)
    // nodes / tris (optional): node fetches and triangle tests, the traversal's algorithmic work.
    Hit trace_bvh(V3 ro, V3 rd, uint64_t *nodes = nullptr, uint64_t *tris = nullptr) const {
        Hit hit{INF, 0u};
        uint64_t n_nodes = 0, n_tris = 0;
        if (d->bvh_node_count == 0) return hit;
        V3 inv = mk(1.0f, 1.0f, 1.0f) / rd;
        uint32_t idx = 0;
        uint32_t stk[64];
        uint32_t sp = 0;
        for (;;) {
            const rt_bvh_node &n = d->bvh_nodes[idx < d->bvh_node_count ? idx : d->bvh_node_count - 1];
            ++n_nodes;
            V3 t0 = (ld(n.bbox_min) - ro) * inv;
            V3 t1 = (ld(n.bbox_max) - ro) * inv;
            V3 tm = vmin(t0, t1);
            V3 tx = vmax(t0, t1);
            float te = fmx(fmx(tm.x, tm.y), tm.z);
            float ta = fmn(fmn(tx.x, tx.y), tx.z);
            if (te <= ta && ta > 0.0f && te < hit.t) {
                if (n.prim_count > 0u) {
                    for (uint32_t i = 0; i < n.prim_count; ++i) {
                        uint64_t slot = (uint64_t)n.left_first + i;
                        uint32_t pi = d->bvh_prim_count
                                          ? d->bvh_prims[slot < d->bvh_prim_count ? slot : d->bvh_prim_count - 1]
                                          : 0u;
                        const rt_triangle &tr = tri(pi);
                        ++n_tris;
                        float t = intersect_triangle(ro, rd, ld(tr.v0), ld(tr.v1), ld(tr.v2));
                        if (t < hit.t) {
                            hit.t = t;
                            hit.prim_id = pi;
                        }
                    }
                    if (sp == 0u) break;
                    sp -= 1u;
                    idx = stk[sp];
                } else {
                    if (sp < 63u) {
                        stk[sp] = n.right_child;
                        sp += 1u;
                    }
                    idx = n.left_first;
                }
            } else {
                if (sp == 0u) break;
                sp -= 1u;
                idx = stk[sp];
            }
        }
        if (nodes) *nodes += n_nodes;
        if (tris) *tris += n_tris;
        return hit;
    }
};

// ================================================================================================
// gather.wgsl (the megakernel path tracer)
// ================================================================================================
struct GatherCtx {
    Scene sc;
    const rt_camera_uniform *cam;
    const rt_image_params *ip;
    const rt_grid_params *gp;
    const rt_photon *sorted_photons;
    uint64_t sorted_count;
    const uint32_t *grid_meta;
    uint32_t max_bounces;
};

// Work counters of one thread: [0] segments, [1] shadow rays, [2] node fetches, [3] triangle tests,
// [4] segments that hit.
struct Work {
    uint64_t v[5] = {0, 0, 0, 0, 0};
};

inline float luma_of(V3 c) { return dot(c, mk(0.2126f, 0.7152f, 0.0722f)); }  // gather.wgsl:31

struct Acc {
    V3 col{0, 0, 0};
    float lum_sum = 0.0f, lum2_sum = 0.0f;
    float sample_lum[8] = {0, 0, 0, 0, 0, 0, 0, 0};
};
// gather.wgsl:36-42
inline void add_radiance(uint32_t s, Acc &a, V3 c) {
    a.col = a.col + c;
    float l = luma_of(c);
    a.lum_sum += l;
    a.lum2_sum += l * l;
    if (s < 8u) a.sample_lum[s] += l;
}

// gather.wgsl:91-103
inline bool shadowed(const GatherCtx &g, V3 origin, V3 dir, float max_dist, Work &wk) {
    wk.v[1] += 1;
    Hit sh = g.sc.trace_bvh(origin, dir, &wk.v[2], &wk.v[3]);
    if (sh.t >= max_dist - 0.001f) return false;
    const rt_triangle &bt = g.sc.tri(sh.prim_id);
    const rt_material &bm = g.sc.mat(bt.material_id);
    if ((bm.flags & RT_MAT_FLAG_ALPHA_CUTOUT) != 0u && bm.tex_albedo != RT_TEX_NONE) {
        Bary b = barycentric(bt, origin, dir, sh.t);
        float alpha = tex_sample(g.sc.d->tex_albedo, b.uvx, b.uvy, layer_of(bm.tex_albedo)).a;
        if (alpha < 0.5f) return false;
    }
    return true;
}

// gather.wgsl:107-111
inline V3 sky_color(V3 dir, V3 zenith, V3 horizon, float intensity) {
    float t = clampf(dir.y * 0.5f + 0.5f, 0.0f, 1.0f);
    return mix3(horizon, zenith, std::sqrt(t)) * intensity;
}

struct MatParams {
    V3 albedo;
    float rough, metal;
};
// gather.wgsl:120-134
inline MatParams eval_material(const GatherCtx &g, const rt_material &mat, float u, float v) {
    MatParams p{ld(mat.albedo), mat.roughness, mat.metallic};
    if (mat.tex_albedo != RT_TEX_NONE) {
        Rgba t = tex_sample(g.sc.d->tex_albedo, u, v, layer_of(mat.tex_albedo));
        p.albedo = ld(mat.albedo) * mk(t.r, t.g, t.b);
    }
    if (mat.tex_mr != RT_TEX_NONE) {
        Rgba mr = tex_sample(g.sc.d->tex_mr, u, v, layer_of(mat.tex_mr));
        p.rough = clampf(mat.roughness * mr.g, 0.0f, 1.0f);
        p.metal = clampf(mat.metallic * mr.b, 0.0f, 1.0f);
    }
    return p;
}
// gather.wgsl:136-141
inline V3 emissive_at(const GatherCtx &g, const rt_material &mat, float u, float v) {
    if (mat.tex_emissive != RT_TEX_NONE) {
        Rgba t = tex_sample(g.sc.d->tex_emissive, u, v, layer_of(mat.tex_emissive));
        return ld(mat.emissive) * mk(t.r, t.g, t.b);
    }
    return ld(mat.emissive);
}

struct LightSample {
    V3 e, wi;
};
inline uint32_t pick_index(float u, uint64_t n) {  // u32(u * f32(n)), index clamped into the array
    uint32_t i = f2u(u * (float)n);
    return i < n ? i : (uint32_t)(n - 1);
}
// gather.wgsl:152-206
inline LightSample direct_light(const GatherCtx &g, V3 hp, V3 sn, Rng &rng, Work &wk) {
    uint64_t n = g.sc.d->light_count;
    if (n == 0) return LightSample{mk(0, 0, 0), sn};
    uint32_t li = pick_index(rng_f32(rng), n);
    const rt_light &l = g.sc.d->lights[li];
    const float fn = (float)n;
    if (l.kind == 0u) {
        V3 to = ld(l.data) - hp;
        float r2 = dot(to, to);
        float r = std::sqrt(r2);
        V3 ldir = to / r;
        if (dot(sn, ldir) <= 0.0f) return LightSample{mk(0, 0, 0), ldir};
        if (shadowed(g, hp + sn * 0.01f, ldir, r - 0.001f, wk)) return LightSample{mk(0, 0, 0), ldir};
        V3 pl = ld(g.ip->point_light_emission);
        return LightSample{ld(l.color) * l.intensity * pl * fmx(dot(sn, ldir), 0.0f) / (r2 + 0.01f) * fn, ldir};
    } else if (l.kind == 1u) {
        V3 ldir = normalize(ld(l.data));
        float ndl = dot(sn, ldir);
        if (ndl <= 0.0f) return LightSample{mk(0, 0, 0), ldir};
        if (shadowed(g, hp + sn * 0.01f, ldir, 1e30f, wk)) return LightSample{mk(0, 0, 0), ldir};
        return LightSample{ld(l.color) * l.intensity * ndl * fn, ldir};
    } else if (l.kind == 2u) {
        const rt_triangle &tri = g.sc.tri(f2u(l.data[0]));
        const rt_material &mat = g.sc.mat(tri.material_id);
        float u1 = rng_f32(rng);
        float u2 = rng_f32(rng);
        float su = std::sqrt(u1);
        float u = 1.0f - su;
        float v = u2 * su;
        float w = 1.0f - u - v;
        V3 lp = ld(tri.v0) * w + ld(tri.v1) * u + ld(tri.v2) * v;
        float uvx = tri.uv0[0] * w + tri.uv1[0] * u + tri.uv2[0] * v;
        float uvy = tri.uv0[1] * w + tri.uv1[1] * u + tri.uv2[1] * v;
        V3 le = ld(l.color);
        if (mat.tex_emissive != RT_TEX_NONE) {
            Rgba t = tex_sample(g.sc.d->tex_emissive, uvx, uvy, layer_of(mat.tex_emissive));
            le = le * mk(t.r, t.g, t.b);
        }
        le = le * ld(g.ip->light_emission);
        V3 to = lp - hp;
        float r2 = dot(to, to);
        float r = std::sqrt(r2);
        V3 ldir = to / r;
        float ndl = dot(sn, ldir);
        if (ndl <= 0.0f) return LightSample{mk(0, 0, 0), ldir};
        V3 ln = get_triangle_normal(tri);
        float ndl_l = dot(ln, -ldir);
        if (ndl_l <= 0.0f) return LightSample{mk(0, 0, 0), ldir};
        if (shadowed(g, hp + sn * 0.01f, ldir, r - 0.001f, wk)) return LightSample{mk(0, 0, 0), ldir};
        float area = 0.5f * length(cross(ld(tri.v1) - ld(tri.v0), ld(tri.v2) - ld(tri.v0)));
        return LightSample{le * l.intensity * ndl * ndl_l * area * fn / (r2 + 0.01f), ldir};
    }
    return LightSample{mk(0, 0, 0), sn};
}

// gather.wgsl:210-213
inline float smith_g1(float nd, float a) {
    float k = a * 0.5f;
    return nd / (nd * (1.0f - k) + k);
}
// gather.wgsl:216-227
inline V3 spec_ggx(V3 wo, V3 n, V3 wi, float a, V3 f0) {
    float ndl = dot(n, wi);
    float ndv = dot(n, wo);
    if (ndl <= 0.0f || ndv <= 0.0f) return mk(0, 0, 0);
    V3 h = normalize(wo + wi);
    float ndh = fmx(dot(n, h), 0.0f);
    float a2 = a * a;
    float dd = ndh * ndh * (a2 - 1.0f) + 1.0f;
    float D = a2 / (PI * dd * dd);
    V3 F = fresnel_schlick(fmx(dot(wo, h), 0.0f), f0);
    return F * (D * smith_g1(ndl, a) * smith_g1(ndv, a) / (4.0f * ndl * ndv));
}
// gather.wgsl:239-256 (basis_z :230-234)
inline V3 sample_spec_dir(V3 rd, V3 n, float a, Rng &rng) {
    V3 up = std::fabs(n.y) < 0.999f ? mk(0, 1, 0) : mk(1, 0, 0);
    V3 bt = normalize(cross(up, n));
    V3 bb = cross(n, bt);
    V3 mrd = -rd;
    V3 v = mk(dot(bt, mrd), dot(bb, mrd), dot(n, mrd));
    V3 vh = normalize(mk(a * v.x, a * v.y, fmx(v.z, 1e-4f)));
    float l2 = vh.x * vh.x + vh.y * vh.y;
    V3 t1 = l2 > 0.0f ? mk(-vh.y, vh.x, 0.0f) * (1.0f / std::sqrt(l2)) : mk(1, 0, 0);
    V3 t2 = cross(vh, t1);
    float r = std::sqrt(rng_f32(rng));
    float phi = 2.0f * PI * rng_f32(rng);
    float sp, cp;
    sincos_fixed(phi, sp, cp);
    float x = r * cp;
    float y = r * sp;
    float s = 0.5f * (1.0f + vh.z);
    float yy = (1.0f - s) * std::sqrt(fmx(0.0f, 1.0f - x * x)) + s * y;
    V3 hh = x * t1 + yy * t2 + std::sqrt(fmx(0.0f, 1.0f - x * x - yy * yy)) * vh;
    V3 hn = normalize(hh);
    V3 m = bt * hn.x + bb * hn.y + n * hn.z;
    V3 out = reflect(rd, m);
    return dot(out, n) > 0.0f ? out : reflect(rd, n);
}

// gather.wgsl:55-64 (i32 cell of a position, flat index of a cell)
inline void photon_cell_i(const rt_grid_params &gp, V3 pos, int32_t c[3]) {
    c[0] = f2i((pos.x - gp.room_min_x) / gp.cell_size);
    c[1] = f2i((pos.y - gp.room_min_y) / gp.cell_size);
    c[2] = f2i((pos.z - gp.room_min_z) / gp.cell_size);
}
inline int32_t clampi(int32_t x, int32_t lo, int32_t hi) { return x < lo ? lo : (x > hi ? hi : x); }
inline int32_t wrap_add(int32_t a, int32_t b) { return (int32_t)((uint32_t)a + (uint32_t)b); }

struct PixelOut {
    float frame[4], moments[4], gbuffer[4];
};

// gather.wgsl:258-594, one pixel.
void gather_pixel(const GatherCtx &g, uint32_t px, uint32_t py, PixelOut &out, Work &wk) {
    const rt_image_params &ip = *g.ip;
    const rt_camera_uniform &cam = *g.cam;
    const uint32_t debug_view = ip._pad[0];
    uint32_t base_seed = py * ip.width + px + ip.frame * 2654435761u;
    Rng rng = rng_init(base_seed * 1664525u + 1013904223u);
    Acc A;
    V3 first_normal = mk(0, 1, 0);
    float first_depth = 1e30f;
    uint32_t spp = ip.spp > 1u ? ip.spp : 1u;

    float env_intensity = 0.0f;
    V3 env_color = mk(0.55f, 0.6f, 0.75f);
    V3 env_horizon = mk(0.95f, 0.93f, 0.9f);
    for (uint64_t i = 0; i < g.sc.d->light_count; ++i) {
        const rt_light &l = g.sc.d->lights[i];
        if (l.kind == 3u) {
            env_intensity = l.intensity;
            env_color = ld(l.color);
            env_horizon = ld(l.data);
            break;
        }
    }

    for (uint32_t s = 0; s < spp; ++s) {
        float jx = rng_f32(rng) - 0.5f;
        float jy = rng_f32(rng) - 0.5f;
        float ux = ((float)px + jx) * cam.inv_half_res[0] - 1.0f;
        float uy = 1.0f - ((float)py + jy) * cam.inv_half_res[1];
        V3 ro = ld(cam.position);
        V3 rd = normalize(ld(cam.forward) + ld(cam.right) * ux + ld(cam.up) * uy);
        V3 thr = mk(1, 1, 1);

        for (uint32_t b = 0; b < g.max_bounces; ++b) {
            wk.v[0] += 1;
            Hit hit = g.sc.trace_bvh(ro, rd, &wk.v[2], &wk.v[3]);
            if (hit.t >= INF) {
                if (b > 0u) add_radiance(s, A, thr * sky_color(rd, env_color, env_horizon, env_intensity));
                break;
            }
            wk.v[4] += 1;
            const rt_triangle &tr = g.sc.tri(hit.prim_id);
            const rt_material &mat = g.sc.mat(tr.material_id);
            V3 hp = ro + rd * hit.t;
            Bary bb = barycentric(tr, ro, rd, hit.t);
            float uvx = bb.uvx, uvy = bb.uvy;

            if ((mat.flags & RT_MAT_FLAG_ALPHA_CUTOUT) != 0u && mat.tex_albedo != RT_TEX_NONE) {
                if (tex_sample(g.sc.d->tex_albedo, uvx, uvy, layer_of(mat.tex_albedo)).a < 0.5f) {
                    ro = hp + rd * 0.002f;
                    continue;
                }
            }

            V3 gn = get_triangle_normal(tr);
            bool ff = dot(rd, gn) < 0.0f;
            V3 sn_geom = smooth_normal(tr, bb, gn);
            V3 sn = ff ? sn_geom : -sn_geom;
            V3 shn = sn;
            if (mat.tex_normal != RT_TEX_NONE) {
                Rgba t = tex_sample(g.sc.d->tex_normal, uvx, uvy, layer_of(mat.tex_normal));
                V3 nm = mk(t.r, t.g, t.b) * 2.0f - mk(1, 1, 1);
                V3 ft, fb;
                tangent_frame(tr, sn, &ft, &fb);
                shn = normalize(ft * nm.x + fb * nm.y + sn * nm.z);
            }

            if (b == 0u && hit.t < first_depth) {
                first_normal = sn;
                first_depth = hit.t;
            }

            MatParams params = eval_material(g, mat, uvx, uvy);
            V3 albedo = params.albedo;
            float rough = params.rough;
            float metal = params.metal;

            add_radiance(s, A, thr * emissive_at(g, mat, uvx, uvy));

            // gather.wgsl:359-419 debug views
            if (debug_view != 0u) {
                bool stop = true;
                switch (debug_view) {
                    case 1: A.col = mk(uvx, uvy, 0.0f); break;
                    case 2: A.col = sn * 0.5f + mk(0.5f, 0.5f, 0.5f); break;
                    case 3: A.col = shn * 0.5f + mk(0.5f, 0.5f, 0.5f); break;
                    case 4: A.col = gn * 0.5f + mk(0.5f, 0.5f, 0.5f); break;
                    case 5: A.col = emissive_at(g, mat, uvx, uvy); break;
                    case 8: {
                        float pu = (float)px / (float)ip.width, pv = (float)py / (float)ip.height;
                        Rgba t = tex_sample(g.sc.d->tex_emissive, pu, pv, 0);
                        A.col = mk(t.r, t.g, t.b);
                        break;
                    }
                    case 9: {
                        float pu = (float)px / (float)ip.width, pv = (float)py / (float)ip.height;
                        Rgba t = tex_sample(g.sc.d->tex_albedo, pu, pv, 0);
                        A.col = mk(t.r, t.g, t.b);
                        break;
                    }
                    case 11: {
                        Rgba t = tex_sample(g.sc.d->tex_emissive, uvx, uvy, 0);
                        A.col = mk(t.r, t.g, t.b);
                        break;
                    }
                    case 12: A.col = ld(mat.emissive); break;
                    case 13: A.col = mk((float)mat.tex_emissive / 65535.0f, 0.0f, 0.0f); break;
                    case 17: A.col = mk(uvx - std::floor(uvx), uvy - std::floor(uvy), 0.0f); break;
                    case 18: {
                        Rgba t = tex_sample(g.sc.d->tex_albedo, uvx, uvy, layer_of(mat.tex_albedo));
                        A.col = mk(t.r, t.g, t.b);
                        break;
                    }
                    case 19: {
                        V3 ft, fb;
                        tangent_frame(tr, sn, &ft, &fb);
                        A.col = ft * 0.5f + mk(0.5f, 0.5f, 0.5f);
                        break;
                    }
                    case 20: {
                        V3 ft, fb;
                        tangent_frame(tr, sn, &ft, &fb);
                        A.col = fb * 0.5f + mk(0.5f, 0.5f, 0.5f);
                        break;
                    }
                    case 21: A.col = hp; break;
                    default: stop = false; break;
                }
                if (stop) break;
            }

            if (mat.kind == 2u) {  // gather.wgsl:421-436
                float q = (mat.ior - 1.0f) / (mat.ior + 1.0f);
                float f0s = q * q;
                float ct = std::fabs(dot(rd, shn));
                float fr = fresnel_schlick(ct, mk(f0s, f0s, f0s)).x;
                if (rng_f32(rng) < fr) {
                    rd = reflect(rd, shn);
                    ro = hp + shn * 0.001f;
                } else {
                    float eta = ff ? 1.0f / mat.ior : mat.ior;
                    rd = refract(rd, shn, eta);
                    ro = hp - shn * 0.001f;
                    thr = thr * ld(mat.albedo);
                }
                continue;
            }

            // gather.wgsl:439-470
            V3 f0 = mix3v(mk(0.04f, 0.04f, 0.04f), albedo, mk(metal, metal, metal));
            V3 wo = -rd;
            float a = fmx(rough * rough, 1e-3f);
            V3 fr = fresnel_schlick(std::fabs(dot(rd, shn)), f0);
            V3 diffuse_weight = (1.0f - metal) * albedo;
            float sp = max3(fr);
            float dp = max3(diffuse_weight);
            float ratio = sp / (sp + dp);
            float spec_prob = clampf(sp + dp <= 0.0f ? 0.5f : ratio, 0.001f, 0.999f);
            bool do_spec = rng_f32(rng) < spec_prob;
            V3 dscale = diffuse_weight / (1.0f - spec_prob);

            if (!do_spec) {
                LightSample ls = direct_light(g, hp, shn, rng, wk);
                if (env_intensity > 0.0f)
                    add_radiance(s, A, thr * dscale * sky_color(shn, env_color, env_horizon, env_intensity));
                add_radiance(s, A, thr * dscale * ls.e / PI);
                add_radiance(s, A, thr * albedo * ip.ambient);
            } else {
                LightSample ls = direct_light(g, hp, shn, rng, wk);
                add_radiance(s, A, thr * spec_ggx(wo, shn, ls.wi, a, f0) * ls.e / spec_prob);
            }

            // gather.wgsl:473-514 photon-map indirect
            if (ip.use_photons == 1u && !do_spec) {
                const rt_grid_params &gp = *g.gp;
                float r2 = ip.photon_radius * ip.photon_radius;
                V3 ph_sum = mk(0, 0, 0);
                uint32_t ph_hits = 0u;
                uint32_t budget = 384u;
                bool done = false;
                int32_t base[3];
                photon_cell_i(gp, hp, base);
                int32_t gxmax = (int32_t)gp.grid_x - 1, gymax = (int32_t)gp.grid_y - 1, gzmax = (int32_t)gp.grid_z - 1;
                for (int32_t dz = -1; dz <= 1 && !done; ++dz)
                    for (int32_t dy = -1; dy <= 1 && !done; ++dy)
                        for (int32_t dx = -1; dx <= 1 && !done; ++dx) {
                            int32_t cx = clampi(wrap_add(base[0], dx), 0, gxmax);
                            int32_t cy = clampi(wrap_add(base[1], dy), 0, gymax);
                            int32_t cz = clampi(wrap_add(base[2], dz), 0, gzmax);
                            uint32_t cell = (uint32_t)cx + (uint32_t)cy * gp.grid_x + (uint32_t)cz * gp.grid_x * gp.grid_y;
                            uint32_t start = g.grid_meta[2 * (size_t)cell];
                            uint32_t count = g.grid_meta[2 * (size_t)cell + 1];
                            for (uint32_t i = 0; i < count && !done; ++i) {
                                if (budget == 0u) {
                                    done = true;
                                    break;
                                }
                                budget -= 1u;
                                uint64_t k = (uint64_t)start + i;
                                const rt_photon &ph = g.sorted_photons[k < g.sorted_count ? k : g.sorted_count - 1];
                                V3 pp = ld(ph.position);
                                float d2 = dot(pp - hp, pp - hp);
                                if (d2 < r2) {
                                    ph_sum = ph_sum + ld(ph.power) * fmx(dot(shn, -ld(ph.incident)), 0.0f);
                                    ph_hits += 1u;
                                    if (ph_hits >= 64u) {
                                        done = true;
                                        break;
                                    }
                                }
                            }
                        }
                if (ph_hits > 0u) {
                    add_radiance(s, A,
                                 thr * dscale * ph_sum * ip.photon_scale /
                                     (PI * (float)ph_hits * ip.photon_radius * ip.photon_radius));
                }
                if (ip.photon_debug == 1u) {
                    float density = fmn((float)ph_hits / 64.0f, 1.0f);
                    A.col = mk(1.0f - density, density, 0.0f) * 2.0f;
                }
            }

            // gather.wgsl:517-537
            if (do_spec) {
                rd = sample_spec_dir(rd, shn, a, rng);
                ro = hp + shn * 0.001f;
                V3 h = normalize(wo + rd);
                float ndl = fmx(dot(shn, rd), 0.0f);
                thr = thr * fresnel_schlick(fmx(dot(wo, h), 0.0f), f0) * smith_g1(ndl, a) / spec_prob;
            } else {
                V3 local = sample_cosine_hemisphere(rng);
                rd = to_world(local, shn);
                ro = hp + shn * 0.001f;
                thr = thr * dscale;
                if (ip.use_photons == 1u) break;
            }
            float p = max3(thr);
            if (p <= 0.0f || rng_f32(rng) > p) break;
            thr = thr / p;
        }
    }

    // gather.wgsl:548-579 firefly sigma clamp
    if (spp <= 8u) {
        float *sl = A.sample_lum;
        for (uint32_t i = 1; i < spp; ++i) {
            float key = sl[i];
            uint32_t j = i;
            while (j > 0u && sl[j - 1u] > key) {
                sl[j] = sl[j - 1u];
                j -= 1u;
            }
            sl[j] = key;
        }
        float median = (sl[(spp - 1u) / 2u] + sl[spp / 2u]) * 0.5f;
        uint32_t half = std::max(spp / 2u, 1u);
        float spread = 0.0f;
        for (uint32_t i = 0; i < half; ++i) {
            float d = sl[i] - median;
            spread += d * d;
        }
        float sigma = fmx(std::sqrt(spread / (float)half), 0.25f * median + 1e-5f);
        float thresh = median + 3.0f * sigma;
        float clamped_lum = 0.0f, clamped_lum2 = 0.0f;
        for (uint32_t i = 0; i < spp; ++i) {
            float lc = fmn(sl[i], thresh);
            clamped_lum += lc;
            clamped_lum2 += lc * lc;
        }
        A.col = A.col * (clamped_lum / fmx(A.lum_sum, 1e-10f));
        A.lum_sum = clamped_lum;
        A.lum2_sum = clamped_lum2;
    }
    V3 col = A.col / (float)spp;
    col = vmin(col, mk(10.0f, 10.0f, 10.0f));
    out.frame[0] = col.x;
    out.frame[1] = col.y;
    out.frame[2] = col.z;
    out.frame[3] = 1.0f;
    out.moments[0] = fmn(A.lum_sum / (float)spp, 10.0f);
    out.moments[1] = fmn(A.lum2_sum / (float)spp, 100.0f);
    out.moments[2] = 0.0f;
    out.moments[3] = 0.0f;
    out.gbuffer[0] = first_normal.x;
    out.gbuffer[1] = first_normal.y;
    out.gbuffer[2] = first_normal.z;
    out.gbuffer[3] = first_depth;
}

template <class F>
void parallel_for(uint64_t n, int threads, F &&fn) {
    if (threads <= 1 || n < 2) {
        for (uint64_t i = 0; i < n; ++i) fn(i, 0);
        return;
    }
    std::atomic<uint64_t> next{0};
    std::vector<std::thread> pool;
    for (int t = 0; t < threads; ++t)
        pool.emplace_back([&, t] {
            for (;;) {
                uint64_t i = next.fetch_add(1);
                if (i >= n) break;
                fn(i, t);
            }
        });
    for (auto &th : pool) th.join();
}

inline int nthreads(int t) {
    if (t > 0) return t;
    unsigned h = std::thread::hardware_concurrency();
    return h ? (int)h : 1;
}

// ================================================================================================
// photon_trace.wgsl
// ================================================================================================
// photon_trace.wgsl:83-88
inline V3 surface_albedo(const Scene &sc, const rt_material &mat, float u, float v) {
    if (mat.tex_albedo != RT_TEX_NONE) {
        Rgba t = tex_sample(sc.d->tex_albedo, u, v, layer_of(mat.tex_albedo));
        return mk(t.r, t.g, t.b);
    }
    return ld(mat.albedo);
}
// photon_trace.wgsl:91-97
inline V3 bounce_dir(V3 rd, V3 n, float rough, Rng &rng) {
    V3 mirror = reflect(rd, n);
    float blur = smoothstepf(0.0f, 1.0f, rough);
    if (blur <= 0.001f) return mirror;
    V3 diff = sample_cosine_hemisphere(rng);
    return normalize(mix3(mirror, to_world(diff, n), blur));
}

// photon_trace.wgsl:101-260, one photon.
void trace_photon(const Scene &sc, const rt_grid_params &gp, uint32_t photon_index, rt_photon *photons,
                  uint64_t n_slots) {
    uint64_t num_lights = sc.d->light_count;
    if (num_lights == 0) return;
    Rng rng = rng_init(photon_index * 1103515245u + 12345u);
    uint32_t li = pick_index(rng_f32(rng), num_lights);
    const rt_light &light = sc.d->lights[li];
    V3 origin = ld(light.data), dir = mk(0, 0, 1), power = mk(0, 0, 0);
    if (light.kind == 0u) {
        float u1 = 0.0f, u2 = 0.0f;
        for (uint32_t guard = 0;; ++guard) {
            u1 = rng_f32(rng) * 2.0f - 1.0f;
            u2 = rng_f32(rng) * 2.0f - 1.0f;
            if (u1 * u1 + u2 * u2 < 1.0f) break;
            if (guard >= (1u << 20)) return;  // not reachable in practice; bounds the loop
        }
        float z = 1.0f - 2.0f * (u1 * u1 + u2 * u2);
        float r = std::sqrt(1.0f - z * z);
        dir = normalize(mk(r * 2.0f * u1, r * 2.0f * u2, z));
        power = ld(light.color) * light.intensity;
    } else if (light.kind == 1u) {
        float disk_radius = 10.0f;
        float disk_u = (rng_f32(rng) - 0.5f) * disk_radius;
        float disk_v = (rng_f32(rng) - 0.5f) * disk_radius;
        V3 d = ld(light.data);
        V3 up = std::fabs(d.y) < 0.999f ? mk(0, 1, 0) : mk(1, 0, 0);
        V3 tangent = normalize(cross(up, d));
        V3 bitangent = cross(d, tangent);
        origin = disk_u * tangent + disk_v * bitangent - d * 100.0f;
        dir = d;
        power = ld(light.color) * light.intensity;
    } else if (light.kind == 2u) {
        const rt_triangle &tri = sc.tri(f2u(light.data[0]));
        float u1 = rng_f32(rng);
        float u2 = rng_f32(rng);
        float su = std::sqrt(u1);
        float u = 1.0f - su;
        float v = u2 * su;
        float w = 1.0f - u - v;
        origin = ld(tri.v0) * u + ld(tri.v1) * v + ld(tri.v2) * w;
        V3 n = get_triangle_normal(tri);
        V3 local = sample_cosine_hemisphere(rng);
        dir = to_world(local, n);
        power = ld(light.color) * light.intensity;
    } else if (light.kind == 3u) {
        V3 local = sample_cosine_hemisphere(rng);
        V3 d = to_world(local, mk(0, 1, 0));
        V3 span = mk((float)gp.grid_x, (float)gp.grid_y, (float)gp.grid_z) * gp.cell_size;
        V3 center = mk(gp.room_min_x, gp.room_min_y, gp.room_min_z) + span * 0.5f;
        float R = fmx(fmx(span.x, span.y), span.z) * 1.2f + 0.05f;
        origin = center + d * R;
        dir = -d;
        float t = clampf(d.y * 0.5f + 0.5f, 0.0f, 1.0f);
        power = mix3(ld(light.color), ld(light.data), std::sqrt(t)) * light.intensity;
    } else {
        return;
    }

    for (uint32_t bounce = 0; bounce < RT_MAX_BOUNCES; ++bounce) {
        Hit hit = sc.trace_bvh(origin, dir);
        if (hit.t >= INF) return;
        const rt_triangle &tri = sc.tri(hit.prim_id);
        const rt_material &mat = sc.mat(tri.material_id);
        V3 hit_pos = origin + dir * hit.t;
        Bary bb = barycentric(tri, origin, dir, hit.t);
        V3 normal = get_triangle_normal(tri);
        bool front_face = dot(dir, normal) < 0.0f;
        V3 sn_geom = smooth_normal(tri, bb, normal);
        V3 face_normal = front_face ? sn_geom : -sn_geom;
        V3 shn = face_normal;
        if (mat.tex_normal != RT_TEX_NONE) {
            Rgba t = tex_sample(sc.d->tex_normal, bb.uvx, bb.uvy, layer_of(mat.tex_normal));
            V3 nm = mk(t.r, t.g, t.b) * 2.0f - mk(1, 1, 1);
            V3 ft, fb;
            tangent_frame(tri, face_normal, &ft, &fb);
            shn = normalize(ft * nm.x + fb * nm.y + face_normal * nm.z);
        }
        if ((mat.flags & RT_MAT_FLAG_ALPHA_CUTOUT) != 0u && mat.tex_albedo != RT_TEX_NONE) {
            float alpha = tex_sample(sc.d->tex_albedo, bb.uvx, bb.uvy, layer_of(mat.tex_albedo)).a;
            if (alpha < 0.5f) {
                origin = hit_pos + dir * 0.002f;
                continue;
            }
        }
        if (mat.tex_emissive != RT_TEX_NONE || length(ld(mat.emissive)) > 1e-4f || mat.kind == 3u) return;
        if (mat.kind == 2u) {
            float q = (mat.ior - 1.0f) / (mat.ior + 1.0f);
            float f0s = q * q;
            float cos_theta = std::fabs(dot(dir, face_normal));
            float fr = fresnel_schlick(cos_theta, mk(f0s, f0s, f0s)).x;
            if (rng_f32(rng) < fr) {
                dir = reflect(dir, face_normal);
                origin = hit_pos + face_normal * 0.001f;
            } else {
                float eta = front_face ? 1.0f / mat.ior : mat.ior;
                dir = refract(dir, face_normal, eta);
                origin = hit_pos - face_normal * 0.001f;
            }
            continue;
        }
        uint64_t store_idx = (uint64_t)photon_index * 6u + bounce;
        if (store_idx < n_slots) {  // the reference clamps an out-of-range index instead
            rt_photon &ph = photons[store_idx];
            V3 inc = -dir;
            ph.position[0] = hit_pos.x; ph.position[1] = hit_pos.y; ph.position[2] = hit_pos.z;
            ph.power[0] = power.x; ph.power[1] = power.y; ph.power[2] = power.z;
            ph.incident[0] = inc.x; ph.incident[1] = inc.y; ph.incident[2] = inc.z;
            ph.normal[0] = shn.x; ph.normal[1] = shn.y; ph.normal[2] = shn.z;
        }
        V3 albedo = surface_albedo(sc, mat, bb.uvx, bb.uvy);
        V3 f0 = mix3v(mk(0.04f, 0.04f, 0.04f), albedo, mk(mat.metallic, mat.metallic, mat.metallic));
        float ct = std::fabs(dot(dir, shn));
        V3 fr = fresnel_schlick(ct, f0);
        V3 diffuse_weight = (1.0f - mat.metallic) * albedo;
        float spec_prob = clampf(max3(fr), 0.0f, 0.98f);
        bool do_spec = rng_f32(rng) < spec_prob;
        if (do_spec) {
            dir = bounce_dir(dir, shn, mat.roughness, rng);
            power = power * f0;
        } else {
            V3 local = sample_cosine_hemisphere(rng);
            dir = to_world(local, shn);
            power = power * diffuse_weight;
        }
        origin = hit_pos + shn * 0.001f;
        float p = max3(power);
        if (p <= 0.0f || rng_f32(rng) > p) return;
        power = power / p;
    }
}

// photon_count.wgsl:18-23 (u32 cell key of a position)
inline uint32_t photon_key(const rt_grid_params &gp, const float *pos) {
    uint32_t gx = f2u((pos[0] - gp.room_min_x) / gp.cell_size);
    uint32_t gy = f2u((pos[1] - gp.room_min_y) / gp.cell_size);
    uint32_t gz = f2u((pos[2] - gp.room_min_z) / gp.cell_size);
    return gx + gy * gp.grid_x + gz * gp.grid_x * gp.grid_y;
}

}  // namespace

// ================================================================================================
// C ABI of the oracle (ctypes)
// ================================================================================================
extern "C" {

void oracle_sincos(const float *x, uint64_t n, float *s, float *c) {
    for (uint64_t i = 0; i < n; ++i) sincos_fixed(x[i], s[i], c[i]);
}

uint32_t oracle_rng_sequence(uint32_t seed, uint32_t n, uint32_t *out_u32, float *out_f32) {
    Rng r = rng_init(seed);
    for (uint32_t i = 0; i < n; ++i) {
        uint32_t v = rng_next(r);
        if (out_u32) out_u32[i] = v;
        if (out_f32) out_f32[i] = (float)v / 4294967296.0f;
    }
    return r.state;
}

float oracle_intersect_triangle(const float *ro, const float *rd, const float *v0, const float *v1, const float *v2) {
    return intersect_triangle(ld(ro), ld(rd), ld(v0), ld(v1), ld(v2));
}

// Closest hit of n rays (origins/dirs: n x 3).  t_out = 1e38 on a miss.
void oracle_trace_rays(const rt_scene_desc *scene, const float *origins, const float *dirs, uint64_t n, float *t_out,
                       uint32_t *prim_out, int threads) {
    Scene sc{scene};
    parallel_for(n, nthreads(threads), [&](uint64_t i, int) {
        Hit h = sc.trace_bvh(ld(origins + 3 * i), ld(dirs + 3 * i));
        t_out[i] = h.t;
        prim_out[i] = h.prim_id;
    });
}

// One gather dispatch over rows [row_begin, row_end).  frame/moments/gbuffer are full W*H*4 images;
// only the given rows are written.  counters (5 entries) accumulate segments, shadow rays, BVH node
// fetches, triangle tests and segments that hit.
int oracle_gather(const rt_scene_desc *scene, const rt_camera_uniform *cam, const rt_image_params *ip,
                  uint32_t max_bounces, const rt_grid_params *gp, const rt_photon *sorted_photons,
                  uint64_t sorted_count, const uint32_t *grid_meta, uint32_t row_begin, uint32_t row_end,
                  int threads, float *frame, float *moments, float *gbuffer, uint64_t *counters) {
    if (!scene || !cam || !ip || !frame || !moments || !gbuffer) return 1;
    if (ip->use_photons == 1u && (!gp || !sorted_photons || !grid_meta || sorted_count == 0)) return 1;
    GatherCtx g{Scene{scene}, cam, ip, gp, sorted_photons, sorted_count, grid_meta, max_bounces ? max_bounces : 6u};
    const uint32_t W = ip->width;
    if (row_end > ip->height) row_end = ip->height;
    if (row_begin >= row_end) return 0;
    int nt = nthreads(threads);
    std::vector<Work> work((size_t)nt);
    parallel_for(row_end - row_begin, nt, [&](uint64_t r, int t) {
        uint32_t y = row_begin + (uint32_t)r;
        for (uint32_t x = 0; x < W; ++x) {
            PixelOut o;
            gather_pixel(g, x, y, o, work[(size_t)t]);
            size_t idx = ((size_t)y * W + x) * 4;
            std::memcpy(frame + idx, o.frame, 16);
            std::memcpy(moments + idx, o.moments, 16);
            std::memcpy(gbuffer + idx, o.gbuffer, 16);
        }
    });
    if (counters)
        for (int t = 0; t < nt; ++t)
            for (int k = 0; k < 5; ++k) counters[k] += work[(size_t)t].v[k];
    return 0;
}

// denoise.wgsl:122-195, one pass.
void oracle_denoise_pass(const float *in, float *out, const float *gbuffer, const float *moments,
                         const rt_denoise_params *p, int threads) {
    const uint32_t W = p->width, H = p->height;
    const float k1d[3] = {0.375f, 0.25f, 0.0625f};
    parallel_for(H, nthreads(threads), [&](uint64_t yy, int) {
        uint32_t y = (uint32_t)yy;
        for (uint32_t x = 0; x < W; ++x) {
            int32_t step = (int32_t)p->step_size;
            size_t idx = (size_t)y * W + x;
            V3 center = ld(in + 4 * idx);
            V3 n_center = ld(gbuffer + 4 * idx);
            float d_center = gbuffer[4 * idx + 3];
            float lum_center = luma_of(center);
            float var_acc = 0.0f, var_cnt = 0.0f;
            for (int32_t qy = -1; qy <= 1; ++qy)
                for (int32_t qx = -1; qx <= 1; ++qx) {
                    int32_t nx = (int32_t)x + qx, ny = (int32_t)y + qy;
                    if (nx < 0 || ny < 0 || nx >= (int32_t)W || ny >= (int32_t)H) continue;
                    size_t q = (size_t)ny * W + (size_t)nx;
                    float mx_ = moments[4 * q], my_ = moments[4 * q + 1];
                    var_acc += fmx(my_ - mx_ * mx_, 0.0f);
                    var_cnt += 1.0f;
                }
            float var_frame = var_acc / fmx(var_cnt, 1.0f);
            float ema_scale = p->alpha / fmx(2.0f - p->alpha, 1e-4f);
            float var_c = var_frame * ema_scale;
            V3 sum = mk(0, 0, 0);
            float total = 0.0f;
            for (int32_t dy = -2; dy <= 2; ++dy)
                for (int32_t dx = -2; dx <= 2; ++dx) {
                    int32_t nx = (int32_t)x + dx * step, ny = (int32_t)y + dy * step;
                    if (nx < 0 || ny < 0 || nx >= (int32_t)W || ny >= (int32_t)H) continue;
                    size_t q = (size_t)ny * W + (size_t)nx;
                    V3 nb = ld(in + 4 * q);
                    V3 nn = ld(gbuffer + 4 * q);
                    float dn = gbuffer[4 * q + 3];
                    float sw = k1d[dx < 0 ? -dx : dx] * k1d[dy < 0 ? -dy : dy];
                    float nw = std::pow(fmx(dot(n_center, nn), 0.0f), p->phi_normal);
                    float dw = std::exp(-std::fabs(d_center - dn) / (p->phi_depth * fmx(d_center, 1e-4f)));
                    float dl = luma_of(nb) - lum_center;
                    float cw = std::exp(-(dl * dl) / (var_c * p->lambda + 1e-6f));
                    float w = sw * nw * dw * cw;
                    sum = sum + nb * w;
                    total += w;
                }
            V3 o = total > 1e-6f ? sum / total : center;
            out[4 * idx] = o.x;
            out[4 * idx + 1] = o.y;
            out[4 * idx + 2] = o.z;
            out[4 * idx + 3] = 1.0f;
        }
    });
}

// composite.wgsl:211-221
void oracle_composite(const float *frame, float *acc, const rt_composite_params *p) {
    size_t n = (size_t)p->width * p->height * 4;
    for (size_t i = 0; i < n; ++i) acc[i] = mixf(acc[i], frame[i], p->alpha);
}

// tonemap.wgsl:240-271 (rgba8unorm store: round to nearest)
void oracle_tonemap(const float *acc, const float *gbuffer, const rt_tonemap_params *p, uint32_t height,
                    uint8_t *out) {
    const uint32_t W = p->width;
    for (uint32_t y = 0; y < height; ++y)
        for (uint32_t x = 0; x < W; ++x) {
            size_t idx = (size_t)y * W + x;
            V3 hdr = ld(acc + 4 * idx);
            V3 exposed = hdr * p->exposure;
            V3 mapped = exposed / (exposed + mk(1, 1, 1));
            float ig = 1.0f / p->gamma;
            V3 color = mk(std::pow(mapped.x, ig), std::pow(mapped.y, ig), std::pow(mapped.z, ig));
            if (p->marker[3] > 0.0f) {
                float px = (float)x + 0.5f, py = (float)y + 0.5f;
                float ddx = px - p->marker[0], ddy = py - p->marker[1];
                float d = std::sqrt(ddx * ddx + ddy * ddy);
                float r = fmx(p->marker[2], 1.5f);
                float hit_dist = gbuffer ? gbuffer[4 * idx + 3] : 1e30f;
                if (hit_dist > p->marker[3] - 0.2f) {
                    float ball = 1.0f - smoothstepf(r * 0.75f, r, d);
                    float halo = 1.0f - smoothstepf(r, r * 3.5f, d);
                    V3 core = mk(1.0f, 0.94f, 0.80f) * std::pow(ball, 1.4f) * 0.85f;
                    V3 ring = mk(1.0f, 0.46f, 0.14f) * halo * halo * 0.8f;
                    color = color + (core + ring) * p->glow * (mk(1, 1, 1) - 0.55f * color);
                }
            }
            float c[4] = {color.x, color.y, color.z, 1.0f};
            for (int k = 0; k < 4; ++k) out[4 * idx + k] = (uint8_t)(clampf(c[k], 0.0f, 1.0f) * 255.0f + 0.5f);
        }
}

// photon_trace dispatch of rebuild_photons (lib.rs:914-938): photons [begin, end).
void oracle_photon_trace(const rt_scene_desc *scene, const rt_grid_params *gp, uint32_t begin, uint32_t end,
                         rt_photon *photons, uint64_t n_slots, int threads) {
    Scene sc{scene};
    if (end <= begin) return;
    parallel_for(end - begin, nthreads(threads),
                 [&](uint64_t i, int) { trace_photon(sc, *gp, begin + (uint32_t)i, photons, n_slots); });
}

// Cell key per slot (photon_count.wgsl:29-32): 0xFFFFFFFF for an empty slot or a key >= num_cells.
void oracle_photon_keys(const rt_photon *photons, uint64_t n_slots, const rt_grid_params *gp, uint32_t *keys) {
    for (uint64_t s = 0; s < n_slots; ++s) {
        const rt_photon &ph = photons[s];
        uint32_t k = 0xFFFFFFFFu;
        if (!(ph.power[0] <= 0.0f)) {
            uint32_t c = photon_key(*gp, ph.position);
            if (c < gp->num_cells) k = c;
        }
        keys[s] = k;
    }
}

// photon_count.wgsl:25-34 + host scan lib.rs:987-1007 + photon_scatter.wgsl:61-71 with the scatter
// taken in slot order within each cell.  Returns the number of binned photons.
uint64_t oracle_photon_grid(const rt_photon *photons, uint64_t n_slots, const rt_grid_params *gp, uint32_t *counts,
                            uint32_t *meta, rt_photon *sorted) {
    const uint32_t C = gp->num_cells;
    std::vector<uint32_t> keys(n_slots);
    oracle_photon_keys(photons, n_slots, gp, keys.data());
    std::memset(counts, 0, (size_t)C * 4);
    for (uint64_t s = 0; s < n_slots; ++s)
        if (keys[s] != 0xFFFFFFFFu) counts[keys[s]] += 1u;
    uint32_t acc = 0;
    for (uint32_t c = 0; c < C; ++c) {
        meta[2 * (size_t)c] = acc;
        meta[2 * (size_t)c + 1] = counts[c];
        acc += counts[c];
    }
    if (sorted) {
        std::memset(sorted, 0, (size_t)n_slots * sizeof(rt_photon));
        std::vector<uint32_t> cursor(C, 0u);
        for (uint64_t s = 0; s < n_slots; ++s) {
            uint32_t k = keys[s];
            if (k == 0xFFFFFFFFu) continue;
            uint64_t dst = (uint64_t)meta[2 * (size_t)k] + cursor[k]++;
            if (dst < n_slots) sorted[dst] = photons[s];
        }
    }
    return acc;
}

// Camera::to_uniform (rustracer-core/src/camera.rs:278-301).  glam's normalize is v * (1/|v|);
// tan(fov/2) is evaluated in double and rounded once.
void oracle_camera_to_uniform(const float *position, const float *look_at, const float *up, float fov_degrees,
                              float near_plane, float aperture, float focus_dist, uint32_t width, uint32_t height,
                              rt_camera_uniform *out) {
    std::memset(out, 0, sizeof(*out));
    V3 pos = ld(position);
    V3 forward = normalize(ld(look_at) - pos);
    V3 right = normalize(cross(forward, ld(up)));
    V3 u = cross(right, forward);
    float aspect = (float)width / (float)height;
    const float rads_per_deg = 3.14159265358979323846f / 180.0f;
    float fov_scale = (float)std::tan((double)(fov_degrees * rads_per_deg * 0.5f));
    V3 rs = right * aspect * fov_scale, us = u * fov_scale;
    float *dst[4] = {out->position, out->forward, out->right, out->up};
    V3 src[4] = {pos, forward, rs, us};
    for (int i = 0; i < 4; ++i) {
        dst[i][0] = src[i].x;
        dst[i][1] = src[i].y;
        dst[i][2] = src[i].z;
    }
    out->inv_half_res[0] = 2.0f / (float)width;
    out->inv_half_res[1] = 2.0f / (float)height;
    out->near_plane = near_plane;
    out->fov_scale = fov_scale;
    out->aperture = aperture;
    out->focus_dist = focus_dist;
}

// Photon grid of Renderer::new (rustracer-renderer/src/lib.rs:416-457) with the cap G on cells per
// axis (26 in the reference) and the radius rule (0: clamp(4 cell, .01, 2); 1: cell / 2).
void oracle_derive_grid(const float *bmin_in, const float *bmax_in, int has_bounds, uint32_t G, uint32_t radius_mode,
                        uint32_t photon_slots, rt_grid_params *gp, float *radius) {
    if (G == 0) G = 26;
    V3 bmin = has_bounds ? ld(bmin_in) : mk(-1.05f, -1.05f, -1.05f);
    V3 bmax = has_bounds ? ld(bmax_in) : mk(1.05f, 1.05f, 1.05f);
    V3 ext = bmax - bmin;
    float max_ext = fmx(fmx(ext.x, fmx(ext.y, ext.z)), 1e-3f);
    float cell = max_ext / ((float)G - 2.0f);
    auto dim = [&](float e) {
        uint32_t v = f2u(std::ceil(e / cell));
        return v < 1u ? 1u : (v > G ? G : v);
    };
    std::memset(gp, 0, sizeof(*gp));
    gp->grid_x = dim(ext.x);
    gp->grid_y = dim(ext.y);
    gp->grid_z = dim(ext.z);
    gp->num_cells = gp->grid_x * gp->grid_y * gp->grid_z;
    gp->room_min_x = bmin.x - cell * 0.5f;
    gp->room_min_y = bmin.y - cell * 0.5f;
    gp->room_min_z = bmin.z - cell * 0.5f;
    gp->cell_size = cell;
    gp->photon_slots = photon_slots;
    *radius = radius_mode == 1 ? cell * 0.5f : clampf(cell * 4.0f, 0.01f, 2.0f);
}

}  // extern "C"
