// Device-side building blocks of the sm_103a hot path: vector math, the PCG hash RNG, rgba8 texture
// sampling, Moller-Trumbore, BVH traversal, hit shading and the BSDF pieces.
//
// Numerics follow the WGSL sources term by term (rustracer-renderer/shaders/common.wgsl, gather.wgsl,
// photon_trace.wgsl); the library is compiled with --fmad=false and IEEE division / square root so
// a product a*b+c is rounded twice, as the shaders' separate multiply and add are.  WGSL leaves a
// few behaviours to the backend; this implementation fixes them as:
//   * min/max with one NaN operand return the other (fminf/fmaxf);
//   * float -> u32/i32 conversion truncates toward zero and saturates, NaN -> 0;
//   * an out-of-range buffer index is clamped to the last element;
//   * normalize(v) = v * (1/sqrt(dot(v,v))), inverseSqrt(x) = 1/sqrt(x), mix(a,b,t) = a(1-t) + bt;
//   * textureSampleLevel(level 0, linear, repeat, rgba8unorm) = fp32 bilinear of byte/255 texels with
//     the array layer clamped to the layer count (an empty role samples as zero).
#pragma once
#include <cstdint>

#include "../../include/rustracer_cuda.h"

namespace rtd {

constexpr float kPi = 3.141592653589793f;
constexpr float kInf = 1e38f;
constexpr float kEps = 1e-6f;
constexpr uint32_t kInvalidKey = 0xFFFFFFFFu;

struct f3 {
    float x, y, z;
};
__device__ __forceinline__ f3 mk3(float x, float y, float z) { return f3{x, y, z}; }
__device__ __forceinline__ f3 xyz(float4 a) { return f3{a.x, a.y, a.z}; }
__device__ __forceinline__ f3 operator+(f3 a, f3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ f3 operator-(f3 a, f3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ f3 operator-(f3 a) { return {-a.x, -a.y, -a.z}; }
__device__ __forceinline__ f3 operator*(f3 a, f3 b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
__device__ __forceinline__ f3 operator*(f3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
__device__ __forceinline__ f3 operator*(float s, f3 a) { return {s * a.x, s * a.y, s * a.z}; }
__device__ __forceinline__ f3 operator/(f3 a, float s) { return {a.x / s, a.y / s, a.z / s}; }
__device__ __forceinline__ f3 operator/(f3 a, f3 b) { return {a.x / b.x, a.y / b.y, a.z / b.z}; }
__device__ __forceinline__ float dot(f3 a, f3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ f3 cross(f3 a, f3 b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
__device__ __forceinline__ float len3(f3 a) { return sqrtf(dot(a, a)); }
__device__ __forceinline__ f3 normalize(f3 a) { return a * (1.0f / sqrtf(dot(a, a))); }
__device__ __forceinline__ f3 vmin(f3 a, f3 b) { return {fminf(a.x, b.x), fminf(a.y, b.y), fminf(a.z, b.z)}; }
__device__ __forceinline__ f3 vmax(f3 a, f3 b) { return {fmaxf(a.x, b.x), fmaxf(a.y, b.y), fmaxf(a.z, b.z)}; }
__device__ __forceinline__ float clampf(float x, float lo, float hi) { return fminf(fmaxf(x, lo), hi); }
__device__ __forceinline__ float max3(f3 a) { return fmaxf(fmaxf(a.x, a.y), a.z); }
// Three-input min / max (PTX min.f32 / max.f32 with three sources): the same value as two nested
// fminf / fmaxf, NaN operands ignored alike.
__device__ __forceinline__ float fmin3f(float a, float b, float c) {
    float r;
    asm("min.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
    return r;
}
__device__ __forceinline__ float fmax3f(float a, float b, float c) {
    float r;
    asm("max.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
    return r;
}
// One 32-byte read-only load (ld.global.nc.v8.f32; the address is 32-byte aligned).
__device__ __forceinline__ void ldg32(const float4 *p, float4 &a, float4 &b) {
    asm("ld.global.nc.v8.f32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
        : "=f"(a.x), "=f"(a.y), "=f"(a.z), "=f"(a.w), "=f"(b.x), "=f"(b.y), "=f"(b.z), "=f"(b.w)
        : "l"(p));
}
__device__ __forceinline__ f3 mix3(f3 a, f3 b, float t) { return a * (1.0f - t) + b * t; }
__device__ __forceinline__ float smoothstepf(float e0, float e1, float x) {
    float t = clampf((x - e0) / (e1 - e0), 0.0f, 1.0f);
    return t * t * (3.0f - 2.0f * t);
}
// sin and cos of one angle, and the integer powers the shaders write as pow(x, 2) and pow(x, 5).
// WGSL leaves the accuracy of sin, cos and pow to the backend, so each is one fixed sequence of IEEE
// operations, evaluated the same way in the oracle.  sin / cos: Cody-Waite reduction by pi/2 with a
// two-part constant (W. J. Cody and W. Waite, Software Manual for the Elementary Functions, 1980;
// 1.5703125 has 8 significant bits, so k * 1.5703125 is exact for |k| < 2^16), then the Taylor
// series of sin (through x^9) and cos (through x^10) on [-pi/4, pi/4] in Horner form, whose
// truncation error (below 3e-9) is under the float rounding; the quadrant picks the signs.
__device__ __forceinline__ void sincos_fixed(float x, float &s, float &c) {
    const float k = floorf(x * 0.636619772f + 0.5f);
    const float r = (x - k * 1.5703125f) - k * 4.83826794e-4f;
    const float z = r * r;
    const float sr = r + r * z * (-(1.0f / 6.0f) + z * ((1.0f / 120.0f) + z * (-(1.0f / 5040.0f) + z * (1.0f / 362880.0f))));
    const float cr = 1.0f - 0.5f * z +
                     z * z * ((1.0f / 24.0f) + z * (-(1.0f / 720.0f) + z * ((1.0f / 40320.0f) + z * -(1.0f / 3628800.0f))));
    const int q = (int)k & 3;
    s = q == 0 ? sr : (q == 1 ? cr : (q == 2 ? -sr : -cr));
    c = q == 0 ? cr : (q == 1 ? -sr : (q == 2 ? -cr : sr));
}
__device__ __forceinline__ float pow5(float x) {
    const float x2 = x * x;
    return x2 * x2 * x;
}
__device__ __forceinline__ uint32_t f2u_sat(float f) {
    if (!(f > 0.0f)) return 0u;
    if (f >= 4294967296.0f) return 0xFFFFFFFFu;
    return __float2uint_rz(f);
}
__device__ __forceinline__ int32_t f2i_sat(float f) {
    if (f != f) return 0;
    if (f <= -2147483648.0f) return INT32_MIN;
    if (f >= 2147483648.0f) return INT32_MAX;
    return __float2int_rz(f);
}

__device__ __forceinline__ f3 reflect(f3 v, f3 n) { return v - 2.0f * dot(v, n) * n; }
__device__ __forceinline__ f3 refract(f3 v, f3 n, float eta) {
    float cos_theta = fminf(dot(-v, n), 1.0f);
    f3 perp = eta * (v + cos_theta * n);
    f3 par = -sqrtf(fabsf(1.0f - dot(perp, perp))) * n;
    return perp + par;
}
__device__ __forceinline__ f3 fresnel_schlick(float cos_theta, f3 f0) {
    float p = pow5(clampf(1.0f - cos_theta, 0.0f, 1.0f));
    return f0 + (mk3(1.0f, 1.0f, 1.0f) - f0) * p;
}

// ---- PCG hash RNG (common.wgsl:29-52) ----------------------------------------------------------
struct Rng {
    uint32_t state;  // inc is always 1 in the reference
};
__device__ __forceinline__ Rng rng_init(uint32_t seed) {
    uint32_t s = seed * 747796405u + 2891336453u;
    s = ((s >> ((s >> 28u) + 4u)) ^ s) * 277803737u;
    return Rng{s};
}
__device__ __forceinline__ uint32_t rng_next(Rng &r) {
    uint32_t old = r.state;
    r.state = old * 747796405u + 1u;
    uint32_t word = ((old >> ((old >> 28u) + 4u)) ^ old) * 277803737u;
    return (word >> 22u) ^ word;
}
// f32(u32) rounds to nearest even; the division by 2^32 is exact.
__device__ __forceinline__ float rng_f32(Rng &r) { return __uint2float_rn(rng_next(r)) * 2.3283064365386963e-10f; }

__device__ __forceinline__ f3 sample_cosine_hemisphere(Rng &r) {
    float u1 = rng_f32(r);
    float u2 = rng_f32(r);
    float phi = 2.0f * kPi * u1;
    float ct = sqrtf(u2);
    float st = sqrtf(1.0f - u2);
    float sp, cp;
    sincos_fixed(phi, sp, cp);
    return mk3(cp * st, ct, sp * st);
}
__device__ __forceinline__ f3 to_world(f3 local, f3 n) {
    f3 up = fabsf(n.y) < 0.999f ? mk3(0.0f, 1.0f, 0.0f) : mk3(1.0f, 0.0f, 0.0f);
    f3 t = normalize(cross(up, n));
    f3 b = cross(n, t);
    return t * local.x + n * local.y + b * local.z;
}

// ---- scene views ------------------------------------------------------------------------------
struct DevTex {
    const uchar4 *texels;  // layer-major, row-major
    uint32_t width, height, layers;
};

struct DevScene {
    // Traversal layout, derived at create from the reference's BVHNode / prim-index / triangle arrays
    // (same tree): one 64-byte record per internal node holding both children's boxes
    //   q0 = (left.min, left.ref)  q1 = (left.max, left.count)  q2 = (right.min, right.ref)
    //   q3 = (right.max, right.count)
    // where count > 0 marks a leaf child (ref = first slot in the leaf-ordered triangles) and
    // count == 0 an internal child (ref = its record index); and one 48-byte record per prim slot,
    // (v0, original index), (v1 - v0), (v2 - v0): the edges Moller-Trumbore computes first.
    const float4 *cnodes;
    const float4 *tri_ord;
    uint32_t cnode_count, stack_cap;
    // The same tree with up to four children per 128-byte record (per child (min, ref), (max, count);
    // count 0xFFFFFFFF marks an empty place), when a near-first walk of it needs at most 64 stack
    // entries (wide_stack); otherwise wnodes is null and only the two-wide records are used.
    const float4 *wnodes;
    uint32_t wnode_count, wide_stack;
    uint32_t any_hit_shadows;  // 1: no alpha-cutout material, shadow rays may stop at the first hit
    const float4 *tris;      // 8 x float4 per TriangleGpu
    const float4 *mats;      // 4 x float4 per MaterialGpu
    const float4 *lights;    // 4 x float4 per LightGpu
    uint32_t tri_count, mat_count, light_count;
    DevTex tex[4];
    // The first environment light (gather.wgsl:276-289), resolved on the host.
    float env_intensity;
    float env_color[3];
    float env_horizon[3];
};

// Index clamped into [0, n) (n == 0 maps to element 0, which every scene array has).
__device__ __forceinline__ uint32_t clampi_u(uint32_t i, uint32_t n) { return i < n ? i : (n ? n - 1u : 0u); }

struct Tri {
    f3 v0, v1, v2;
};
__device__ __forceinline__ Tri load_tri_verts(const DevScene &s, uint32_t i) {
    const float4 *p = s.tris + 8ull * clampi_u(i, s.tri_count);
    float4 a = __ldg(p), b = __ldg(p + 1), c = __ldg(p + 2);
    return Tri{xyz(a), xyz(b), xyz(c)};
}
struct TriFull {
    f3 v0, v1, v2, n0, n1, n2;
    float uv0x, uv0y, uv1x, uv1y, uv2x, uv2y;
    uint32_t material_id;
};
__device__ __forceinline__ TriFull load_tri(const DevScene &s, uint32_t i) {
    const float4 *p = s.tris + 8ull * clampi_u(i, s.tri_count);
    float4 a = __ldg(p), b = __ldg(p + 1), c = __ldg(p + 2), d = __ldg(p + 3), e = __ldg(p + 4), f = __ldg(p + 5),
           g = __ldg(p + 6), h = __ldg(p + 7);
    TriFull t;
    t.v0 = xyz(a); t.v1 = xyz(b); t.v2 = xyz(c);
    t.n0 = xyz(d); t.n1 = xyz(e); t.n2 = xyz(f);
    t.uv0x = g.x; t.uv0y = g.y; t.uv1x = g.z; t.uv1y = g.w; t.uv2x = h.x; t.uv2y = h.y;
    t.material_id = __float_as_uint(h.z);
    return t;
}
struct Mat {
    f3 albedo;
    float alpha;
    f3 emissive;
    float roughness, metallic, ior;
    uint32_t kind, flags, tex_albedo, tex_mr, tex_emissive, tex_normal;
};
__device__ __forceinline__ Mat load_mat(const DevScene &s, uint32_t i) {
    const float4 *p = s.mats + 4ull * clampi_u(i, s.mat_count);
    float4 a = __ldg(p), b = __ldg(p + 1), c = __ldg(p + 2), d = __ldg(p + 3);
    Mat m;
    m.albedo = xyz(a);
    m.alpha = a.w;
    m.emissive = xyz(b);
    m.roughness = b.w;
    m.metallic = c.x;
    m.ior = c.y;
    m.kind = __float_as_uint(c.z);
    m.flags = __float_as_uint(c.w);
    m.tex_albedo = __float_as_uint(d.x);
    m.tex_mr = __float_as_uint(d.y);
    m.tex_emissive = __float_as_uint(d.z);
    m.tex_normal = __float_as_uint(d.w);
    return m;
}
struct Light {
    f3 data;
    float data_w;
    f3 color;
    float intensity;
    uint32_t kind;
};
__device__ __forceinline__ Light load_light(const DevScene &s, uint32_t i) {
    const float4 *p = s.lights + 4ull * i;
    float4 a = __ldg(p), b = __ldg(p + 1), c = __ldg(p + 2);
    return Light{xyz(a), a.w, xyz(b), b.w, __float_as_uint(c.x)};
}

// textureSampleLevel on an rgba8unorm array with a linear / repeat sampler, level 0.
// c / 255 for a byte c, rounded as the IEEE division rounds it: the product with the rounded
// reciprocal of 255, corrected once by its residual (a Markstein-style correction step).  Checked
// against the correctly rounded quotient for all 256 inputs (tests/test_oracle_pins.py); four
// instructions in place of a full division.
__device__ __forceinline__ float unorm8(uint32_t c) {
    const float a = (float)c;  // exact
    const float r = 0x1.010102p-8f;  // 1 / 255 rounded to float
    const float q0 = __fmul_rn(a, r);
    return __fmaf_rn(__fmaf_rn(-q0, 255.0f, a), r, q0);
}

__device__ __forceinline__ float4 tex_sample(const DevTex &t, float u, float v, int32_t layer) {
    if (t.texels == nullptr) return make_float4(0.f, 0.f, 0.f, 0.f);
    int32_t L = layer < 0 ? 0 : (layer >= (int32_t)t.layers ? (int32_t)t.layers - 1 : layer);
    const uint32_t W = t.width, H = t.height;
    float fu = u - floorf(u), fv = v - floorf(v);
    if (!(fu >= 0.0f)) fu = 0.0f;
    if (!(fv >= 0.0f)) fv = 0.0f;
    float x = fu * (float)W - 0.5f, y = fv * (float)H - 0.5f;
    float x0f = floorf(x), y0f = floorf(y);
    float ax = x - x0f, ay = y - y0f;
    int32_t x0 = (int32_t)x0f, y0 = (int32_t)y0f;
    if (x0 < 0) x0 += (int32_t)W;
    if (y0 < 0) y0 += (int32_t)H;
    if (x0 >= (int32_t)W) x0 -= (int32_t)W;
    if (y0 >= (int32_t)H) y0 -= (int32_t)H;
    int32_t x1 = x0 + 1 == (int32_t)W ? 0 : x0 + 1;
    int32_t y1 = y0 + 1 == (int32_t)H ? 0 : y0 + 1;
    const uchar4 *base = t.texels + (size_t)L * W * H;
    uchar4 t00 = __ldg(base + (size_t)y0 * W + x0), t10 = __ldg(base + (size_t)y0 * W + x1);
    uchar4 t01 = __ldg(base + (size_t)y1 * W + x0), t11 = __ldg(base + (size_t)y1 * W + x1);
    auto lerp2 = [&](unsigned char a, unsigned char b, unsigned char c, unsigned char d) {
        float fa = unorm8(a), fb = unorm8(b), fc = unorm8(c), fd = unorm8(d);
        float top = fa * (1.0f - ax) + fb * ax;
        float bot = fc * (1.0f - ax) + fd * ax;
        return top * (1.0f - ay) + bot * ay;
    };
    return make_float4(lerp2(t00.x, t10.x, t01.x, t11.x), lerp2(t00.y, t10.y, t01.y, t11.y),
                       lerp2(t00.z, t10.z, t01.z, t11.z), lerp2(t00.w, t10.w, t01.w, t11.w));
}

// ---- Moller-Trumbore (common.wgsl:78-100) ------------------------------------------------------
__device__ __forceinline__ float intersect_triangle(f3 ro, f3 rd, f3 v0, f3 v1, f3 v2) {
    f3 e1 = v1 - v0;
    f3 e2 = v2 - v0;
    f3 h = cross(rd, e2);
    float a = dot(e1, h);
    if (fabsf(a) < 1e-7f) return kInf;
    float f = 1.0f / a;
    f3 s = ro - v0;
    float u = f * dot(s, h);
    if (u < 0.0f || u > 1.0f) return kInf;
    f3 q = cross(s, e1);
    float v = f * dot(rd, q);
    if (v < 0.0f || u + v > 1.0f) return kInf;
    float t = f * dot(e2, q);
    if (t > kEps) return t;
    return kInf;
}

// BVH traversal over the child-pair records.  Each record fetch tests both children's boxes with the
// reference's slab test (gather.wgsl:71-75: (bmin - ro) / d, te <= ta && ta > 0 && te < t); leaf
// children are intersected on the spot, internal children are visited nearest entry first with the
// farther one pushed (a push is dropped once `stack_cap` entries are in use, as the reference drops
// pushes at 63).  The tree is the reference's, so the closest hit is the reference's.  Triangles hit at
// exactly equal t resolve to the lowest prim slot: leaves hold consecutive slot ranges with the left
// child's below the right's (bvh.rs:159-219), so the reference's left-first walk, where the first
// strictly smaller t wins, meets the lowest slot first.  During the walk st.prim holds the best prim
// slot; trav_hit_prim gives the triangle index.  The stack lives in shared memory, one
// 4-byte column per thread.  TravState makes the traversal resumable one record at a time, so
// persistent warps can refill lanes whose ray finished.
struct TravState {
    f3 ro, rd, inv;
    float t;
    uint32_t prim, node, sp;  // prim: the prim slot of the best hit so far
    const float4 *cnodes, *tri_ord;  // the traversal layout of the ray's scene
    uint32_t cap;                    // stack entries this scene may use
};

// kWide: walk the four-wide records with the lane's whole stack (stack_entries, at least
// s.wide_stack, so no push is dropped); otherwise the two-wide records with the reference's push
// limit (s.stack_cap, at most stack_entries).
template <bool kWide>
__device__ __forceinline__ TravState trav_begin(const DevScene &s, f3 ro, f3 rd, float t_limit,
                                                uint32_t stack_entries) {
    TravState st;
    st.cnodes = kWide ? s.wnodes : s.cnodes;
    st.tri_ord = s.tri_ord;
    st.cap = kWide ? stack_entries : s.stack_cap;
    st.ro = ro;
    st.rd = rd;
    st.inv = mk3(1.0f, 1.0f, 1.0f) / rd;
    st.t = t_limit;
    st.prim = 0u;
    st.node = 0u;
    st.sp = 0u;
    return st;
}

// One traversal step for every lane of a warp; all 32 lanes call it together.  `active` lanes visit
// their current record.  The triangles of the record's hit leaves are tested by the whole warp: the
// leaf work of all lanes is laid out as one list (lane order, left leaf before right leaf, triangles
// in leaf order), cut into rounds of 32 tests, one per lane, and each lane then folds the results of
// its own tests in list order (a test wins when its t is strictly below the best so far, or equal to it
// with a lower prim slot), so a lane's result is what testing its leaves one by one gives.  Testing them one by
// one in each lane instead leaves the warp waiting on the lanes with four-triangle leaves.
//
// Returns true for an active lane whose traversal has finished (st.t and the prim slot st.prim hold
// the closest hit below the starting st.t).  `any` lanes (occlusion queries) also finish at the first record whose
// leaves hold a triangle below st.t; st.t is then the smallest such t of that record.  WarpLeaves is
// per warp, and warp_leaves_set_ray must have stored a lane's ray before its first step.
struct WarpLeaves {
    float4 ray[2][32];  // per lane: (ro, low half of tri_ord), (rd, high half of tri_ord)
    uint4 leaf_ref[32];    // four-wide step: per lane the first prim slot of each hit leaf
    uint4 leaf_start[32];  // and where its tests start in the lane's run (0xFFFFFFFF: none)
    uint32_t owner[32];
    float t[32];
    uint32_t prim[32];
};

__device__ __forceinline__ void warp_leaves_set_ray(WarpLeaves &w, const TravState &st) {
    const uint32_t lane = threadIdx.x & 31u;
    const unsigned long long tp = (unsigned long long)st.tri_ord;
    w.ray[0][lane] = make_float4(st.ro.x, st.ro.y, st.ro.z, __uint_as_float((uint32_t)tp));
    w.ray[1][lane] = make_float4(st.rd.x, st.rd.y, st.rd.z, __uint_as_float((uint32_t)(tp >> 32)));
}

// The leaf tests of one traversal step for the whole warp: lane l has n_l tests (its run), laid out
// in lane order and cut into rounds of 32; tri_of(owner, j) gives the prim slot of the owner's j-th
// test (every lane calls it, with its own arguments).  Each lane folds its own results in run order
// into st.t / st.prim (a test wins when its t is strictly below the best so far, or equal to it with a
// lower prim slot) and returns whether any of them won.
template <typename TriOf>
__device__ __forceinline__ bool warp_leaf_rounds(TravState &st, uint32_t n, WarpLeaves &w, TriOf tri_of) {
    const uint32_t lane = threadIdx.x & 31u;
    if (!__any_sync(0xFFFFFFFFu, n != 0u)) return false;  // no lane reached a leaf this step
    uint32_t incl = n;
#pragma unroll
    for (uint32_t d = 1u; d < 32u; d <<= 1) {
        const uint32_t v = __shfl_up_sync(0xFFFFFFFFu, incl, d);
        if (lane >= d) incl += v;
    }
    const uint32_t total = __shfl_sync(0xFFFFFFFFu, incl, 31);
    const uint32_t excl = incl - n;
    bool found = false;
    for (uint32_t base = 0u; base < total; base += 32u) {
        // This round tests list entries [base, base + 32); a lane owning some of them marks where its
        // run starts, so every position finds its owner as the last start at or below it.
        const uint32_t lo = excl > base ? excl : base;
        const uint32_t hi = excl + n < base + 32u ? excl + n : base + 32u;
        const bool mine = lo < hi;
        if (mine) w.owner[lo - base] = lane;
        const uint32_t starts = __reduce_or_sync(0xFFFFFFFFu, mine ? 1u << (lo - base) : 0u);
        __syncwarp();
        const uint32_t start = 31u - __clz((starts | 1u) & (0xFFFFFFFFu >> (31u - lane)));
        const uint32_t o = w.owner[start];
        const uint32_t o_excl = __shfl_sync(0xFFFFFFFFu, excl, o);
        const uint32_t o_tri = tri_of(o, base + lane - o_excl);  // every lane calls: shuffles inside
        float t = kInf;
        uint32_t prim = 0u;
        if (base + lane < total) {
            const float4 r0 = w.ray[0][o], r1 = w.ray[1][o];
            const float4 *tris = reinterpret_cast<const float4 *>(
                ((unsigned long long)__float_as_uint(r1.w) << 32) | (unsigned long long)__float_as_uint(r0.w));
            const uint32_t tri = o_tri;
            const float4 *tp = tris + 3ull * tri;
            const float4 v0 = __ldg(tp), e1 = __ldg(tp + 1), e2 = __ldg(tp + 2);
            const f3 ro = xyz(r0), rd = xyz(r1);
            // Moller-Trumbore (common.wgsl:78-100) with the edges precomputed.
            const f3 h3 = cross(rd, xyz(e2));
            const float a = dot(xyz(e1), h3);
            if (!(fabsf(a) < 1e-7f)) {
                const float f = 1.0f / a;
                const f3 sv = ro - xyz(v0);
                const float u = f * dot(sv, h3);
                if (!(u < 0.0f || u > 1.0f)) {
                    const f3 q = cross(sv, xyz(e1));
                    const float v = f * dot(rd, q);
                    if (!(v < 0.0f || u + v > 1.0f)) {
                        const float tt = f * dot(xyz(e2), q);
                        if (tt > kEps) t = tt;
                    }
                }
            }
            prim = tri;
        }
        w.t[lane] = t;
        w.prim[lane] = prim;
        __syncwarp();
        if (mine) {
            for (uint32_t k = lo - base; k < hi - base; ++k) {
                const float tk = w.t[k];
                const uint32_t sk = w.prim[k];
                if (tk < st.t || (tk == st.t && sk < st.prim)) {
                    st.t = tk;
                    st.prim = sk;
                    found = true;
                }
            }
        }
        __syncwarp();
    }
    return found;
}

// tests_out (optional): the lane's leaf triangle tests of this step (the work counters of the
// profiling kernels).
__device__ __forceinline__ bool trav_step_warp(TravState &st, bool active, bool any, uint32_t *stk, uint32_t stride,
                                               WarpLeaves &w, uint32_t *tests_out = nullptr) {
    bool hl = false, hr = false;
    float le = 0.0f, re = 0.0f;
    uint32_t lref = 0u, lcnt = 0u, rref = 0u, rcnt = 0u;
    if (active) {
        const float4 *np = st.cnodes + 4ull * st.node;
        const float4 q0 = __ldg(np), q1 = __ldg(np + 1), q2 = __ldg(np + 2), q3 = __ldg(np + 3);
        const f3 ro = st.ro, inv = st.inv;
        const f3 a0 = (xyz(q0) - ro) * inv, a1 = (xyz(q1) - ro) * inv;
        const f3 b0 = (xyz(q2) - ro) * inv, b1 = (xyz(q3) - ro) * inv;
        le = fmax3f(fminf(a0.x, a1.x), fminf(a0.y, a1.y), fminf(a0.z, a1.z));
        const float lx = fmin3f(fmaxf(a0.x, a1.x), fmaxf(a0.y, a1.y), fmaxf(a0.z, a1.z));
        re = fmax3f(fminf(b0.x, b1.x), fminf(b0.y, b1.y), fminf(b0.z, b1.z));
        const float rx = fmin3f(fmaxf(b0.x, b1.x), fmaxf(b0.y, b1.y), fmaxf(b0.z, b1.z));
        hl = le <= lx && lx > 0.0f && le < st.t;
        hr = re <= rx && rx > 0.0f && re < st.t;
        lref = __float_as_uint(q0.w);
        lcnt = __float_as_uint(q1.w);
        rref = __float_as_uint(q2.w);
        rcnt = __float_as_uint(q3.w);
    }
    const uint32_t nl = (hl && lcnt != 0u) ? lcnt : 0u;
    const uint32_t n = nl + ((hr && rcnt != 0u) ? rcnt : 0u);
    if (tests_out) *tests_out = n;
    // The next record does not depend on this record's leaf results (they only lower st.t for later
    // box tests), so the lane moves on first and its next record is on the way to L1 while the warp
    // tests leaves.
    bool exhausted = false;
    if (active) {
        const bool il = hl && lcnt == 0u, ir = hr && rcnt == 0u;
        if (il && ir) {
            const bool left_first = le <= re;
            const uint32_t far = left_first ? rref : lref;
            st.node = left_first ? lref : rref;
            if (st.sp < st.cap) {
                stk[st.sp * stride] = far;
                st.sp += 1u;
            }
        } else if (il) {
            st.node = lref;
        } else if (ir) {
            st.node = rref;
        } else if (st.sp == 0u) {
            exhausted = true;
        } else {
            st.sp -= 1u;
            st.node = stk[st.sp * stride];
        }
        if (!exhausted) asm volatile("prefetch.global.L1 [%0];" ::"l"(st.cnodes + 4ull * st.node));
    }
    const bool found = warp_leaf_rounds(st, n, w, [&](uint32_t o, uint32_t j) {
        const uint32_t o_nl = __shfl_sync(0xFFFFFFFFu, nl, o);
        const uint32_t o_lref = __shfl_sync(0xFFFFFFFFu, lref, o);
        const uint32_t o_rref = __shfl_sync(0xFFFFFFFFu, rref, o);
        return j < o_nl ? o_lref + j : o_rref + (j - o_nl);
    });
    return active && (exhausted || (any && found));
}

// trav_step_warp over the four-wide records: each active lane tests the four child boxes of its
// record with the same slab test, queues the hit leaves' triangles (child order) for the warp's leaf
// rounds, and visits the hit internal children nearest entry first (the others pushed, farthest
// first; the stack holds every pending entry).  Same results as the two-wide walk: the closest hit
// below the starting st.t, ties resolved to the lowest prim slot as in the two-wide walk.
//
// tree (optional): the block's treelet, the first tree_n records of the four-wide layout of the scene
// whose records start at tree_src, staged in shared memory; a lane on that scene reads those records
// from there (the breadth-first layout puts the top levels first).
__device__ __forceinline__ bool trav_step_warp4(TravState &st, bool active, bool any, uint32_t *stk, uint32_t stride,
                                                WarpLeaves &w, uint32_t *tests_out = nullptr,
                                                const float4 *tree = nullptr, const float4 *tree_src = nullptr,
                                                uint32_t tree_n = 0u) {
    const uint32_t lane = threadIdx.x & 31u;
    uint32_t n = 0u;
    bool exhausted = false;
    if (active) {
        float4 q[8];
        if (tree != nullptr && st.cnodes == tree_src && st.node < tree_n) {
            const float4 *tp = tree + 8u * st.node;
#pragma unroll
            for (int i = 0; i < 8; ++i) q[i] = tp[i];
        } else {
            // the 128-byte record as four 32-byte loads (records are 128-byte aligned)
            const float4 *np = st.cnodes + 8ull * st.node;
#pragma unroll
            for (int i = 0; i < 4; ++i) ldg32(np + 2 * i, q[2 * i], q[2 * i + 1]);
        }
        const f3 ro = st.ro, inv = st.inv;
        float key[4];
        uint32_t ref[4];
        // The hit leaves go straight to the lane's leaf slots (first prim slot, start of its tests in
        // the lane's run); unused slots keep start 0xFFFFFFFF.  The previous step's readers are done
        // (each leaf round ends at a warp barrier).
        uint32_t *lr = &w.leaf_ref[lane].x, *ls = &w.leaf_start[lane].x;
        w.leaf_start[lane] = make_uint4(0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu);
        uint32_t n_leaf = 0u;
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            const f3 a0 = (xyz(q[2 * c]) - ro) * inv, a1 = (xyz(q[2 * c + 1]) - ro) * inv;
            const float te = fmax3f(fminf(a0.x, a1.x), fminf(a0.y, a1.y), fminf(a0.z, a1.z));
            const float tx = fmin3f(fmaxf(a0.x, a1.x), fmaxf(a0.y, a1.y), fmaxf(a0.z, a1.z));
            const uint32_t cref = __float_as_uint(q[2 * c].w), cnt = __float_as_uint(q[2 * c + 1].w);
            const bool hit = cnt != 0xFFFFFFFFu && te <= tx && tx > 0.0f && te < st.t;
            ref[c] = cref;
            key[c] = (hit && cnt == 0u) ? te : __int_as_float(0x7F800000);  // +inf: not a pending child
            if (hit && cnt != 0u) {
                lr[n_leaf] = cref;
                ls[n_leaf] = n;
                n_leaf += 1u;
                n += cnt;
            }
        }
        // Near-first order of the hit internal children (a fixed five-exchange network).
        auto cswap = [&](int i, int j) {
            if (key[j] < key[i]) {
                const float tk = key[i];
                key[i] = key[j];
                key[j] = tk;
                const uint32_t tr = ref[i];
                ref[i] = ref[j];
                ref[j] = tr;
            }
        };
        cswap(0, 1);
        cswap(2, 3);
        cswap(0, 2);
        cswap(1, 3);
        cswap(1, 2);
        const float kNone = __int_as_float(0x7F800000);
        const uint32_t m = (key[0] < kNone ? 1u : 0u) + (key[1] < kNone ? 1u : 0u) + (key[2] < kNone ? 1u : 0u) +
                           (key[3] < kNone ? 1u : 0u);
        if (m != 0u) {
            st.node = ref[0];
#pragma unroll
            for (int i = 3; i >= 1; --i)
                if ((uint32_t)i < m && st.sp < st.cap) {
                    stk[st.sp * stride] = ref[i];
                    st.sp += 1u;
                }
        } else if (st.sp == 0u) {
            exhausted = true;
        } else {
            st.sp -= 1u;
            st.node = stk[st.sp * stride];
        }
        if (!exhausted && !(tree != nullptr && st.cnodes == tree_src && st.node < tree_n))
            asm volatile("prefetch.global.L1 [%0];" ::"l"(st.cnodes + 8ull * st.node));
    }
    if (tests_out) *tests_out = n;
    const bool found = warp_leaf_rounds(st, n, w, [&](uint32_t o, uint32_t j) {
        const uint4 r = w.leaf_ref[o], b = w.leaf_start[o];
        const uint32_t i = (j >= b.y ? 1u : 0u) + (j >= b.z ? 1u : 0u) + (j >= b.w ? 1u : 0u);
        const uint32_t first = i == 0u ? r.x : (i == 1u ? r.y : (i == 2u ? r.z : r.w));
        const uint32_t at = i == 0u ? b.x : (i == 1u ? b.y : (i == 2u ? b.z : b.w));
        return first + (j - at);
    });
    return active && (exhausted || (any && found));
}

// The triangle index of a finished closest-hit traversal (st.prim holds the hit's prim slot; a miss
// gives 0).
__device__ __forceinline__ uint32_t trav_hit_prim(const TravState &st) {
    return st.t < kInf ? __float_as_uint(__ldg(st.tri_ord + 3ull * st.prim).w) : 0u;
}


struct Bary {
    float uvx, uvy, u, v;
};
__device__ __forceinline__ Bary barycentric(const TriFull &tri, f3 ro, f3 rd, float t) {
    f3 e1 = tri.v1 - tri.v0;
    f3 e2 = tri.v2 - tri.v0;
    f3 p = ro + rd * t - tri.v0;
    float d00 = dot(e1, e1), d01 = dot(e1, e2), d11 = dot(e2, e2);
    float d20 = dot(p, e1), d21 = dot(p, e2);
    float denom = d00 * d11 - d01 * d01;
    float u = 0.0f, v = 0.0f;
    if (denom != 0.0f) {
        u = (d11 * d20 - d01 * d21) / denom;
        v = (d00 * d21 - d01 * d20) / denom;
    }
    float w = 1.0f - u - v;
    return Bary{tri.uv0x * w + tri.uv1x * u + tri.uv2x * v, tri.uv0y * w + tri.uv1y * u + tri.uv2y * v, u, v};
}
__device__ __forceinline__ f3 smooth_normal(const TriFull &tri, const Bary &b, f3 geometric) {
    float w = 1.0f - b.u - b.v;
    f3 n = tri.n0 * w + tri.n1 * b.u + tri.n2 * b.v;
    if (dot(n, n) < 1e-8f) return geometric;
    return normalize(n);
}
__device__ __forceinline__ void tangent_frame(const TriFull &tri, f3 n, f3 &t_out, f3 &b_out) {
    f3 e1 = tri.v1 - tri.v0;
    f3 e2 = tri.v2 - tri.v0;
    float d1x = tri.uv1x - tri.uv0x, d1y = tri.uv1y - tri.uv0y;
    float d2x = tri.uv2x - tri.uv0x, d2y = tri.uv2y - tri.uv0y;
    float det = d1x * d2y - d2x * d1y;
    float f = fabsf(det) < 1e-12f ? 0.0f : 1.0f / det;
    f3 t = (e1 * d2y - e2 * d1y) * f;
    f3 b = (e2 * d1x - e1 * d2x) * f;
    f3 tt = t - n * dot(n, t);
    if (dot(tt, tt) < 1e-10f) {
        tt = cross(n, mk3(1.0f, 0.0f, 0.0f));
        if (dot(tt, tt) < 1e-6f) tt = cross(n, mk3(0.0f, 1.0f, 0.0f));
    }
    tt = normalize(tt);
    f3 c = cross(n, tt);
    t_out = tt;
    b_out = c * (dot(c, b) > 0.0f ? 1.0f : -1.0f);
}
__device__ __forceinline__ f3 triangle_normal(f3 v0, f3 v1, f3 v2) { return normalize(cross(v1 - v0, v2 - v0)); }

// Programmatic dependent launch.  A kernel launched with the programmatic-serialization attribute may
// start while the kernel before it in the stream finishes; grid_dependency_wait() returns once that
// kernel has completed and its writes are visible (at once for a kernel launched the ordinary way).
// grid_launch_dependents() lets the next such kernel's blocks be scheduled as this grid's blocks
// retire.
__device__ __forceinline__ void grid_dependency_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void grid_launch_dependents() { asm volatile("griddepcontrol.launch_dependents;" :::); }

// Warp helpers of the queue kernels.
__device__ __forceinline__ uint32_t lanemask_lt() {
    uint32_t m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

// Appends `item` to queue (count at *counter) for the lanes with want == true; one atomic per warp.
// Every lane of the warp must call it.
__device__ __forceinline__ void warp_append(bool want, uint32_t item, uint32_t *queue, uint32_t *counter) {
    const uint32_t mask = __ballot_sync(0xFFFFFFFFu, want);
    if (mask == 0u) return;
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t leader = __ffs(mask) - 1u;
    uint32_t base = 0;
    if (lane == leader) base = atomicAdd(counter, (uint32_t)__popc(mask));
    base = __shfl_sync(0xFFFFFFFFu, base, leader);
    if (want) queue[base + __popc(mask & lanemask_lt())] = item;
}

}  // namespace rtd
