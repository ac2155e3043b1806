// ORACLE — test infrastructure only.
//
// The scene side of the oracle: the reference's binned-SAH BVH build (rustracer-core/src/bvh.rs:120-336),
// the flattening of meshes into TriangleGpu records (rustracer-core/src/scene.rs:213-291), and the two
// seeded procedural workloads the parity tests and the CPU baseline render (the 555-unit Cornell box
// and the displaced-icosphere room).  With it the oracle renders a scene it generated and indexed
// itself; the CPU tests check that its triangles, materials, lights, textures and BVH equal the CUDA
// backend's byte for byte.  Nothing in the product links, loads or calls this file.
//
// Orders the reference leaves open, fixed the same way in the product:
//   * the SAH partition selects by (centroid on the split axis, primitive index); the reference's
//     select_nth_unstable_by leaves equal centroids in an unspecified order;
//   * a leaf lists its primitives in index order (select_nth_unstable_by leaves that order
//     unspecified too, and it decides which of two triangles hit at exactly equal t is reported).
//
// Built with -ffp-contract=off like oracle.cpp.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <new>
#include <unordered_map>
#include <vector>

#include "../include/rustracer_cuda.h"

namespace {

struct P3 {
    float x, y, z;
};
inline P3 add(P3 a, P3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline P3 sub(P3 a, P3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline P3 scale(P3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
inline float dot3(P3 a, P3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline P3 cross3(P3 a, P3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
inline P3 unit(P3 a) { return scale(a, 1.0f / std::sqrt(dot3(a, a))); }  // glam normalize: v * (1 / |v|)
inline P3 pmin(P3 a, P3 b) { return {std::fmin(a.x, b.x), std::fmin(a.y, b.y), std::fmin(a.z, b.z)}; }
inline P3 pmax(P3 a, P3 b) { return {std::fmax(a.x, b.x), std::fmax(a.y, b.y), std::fmax(a.z, b.z)}; }
inline float axis_of(const P3 &p, int a) { return a == 0 ? p.x : (a == 1 ? p.y : p.z); }
inline void put3(float *d, P3 v) {
    d[0] = v.x;
    d[1] = v.y;
    d[2] = v.z;
}

constexpr float kBig = std::numeric_limits<float>::max();

// AABB (bvh.rs:13-60): EMPTY = (+MAX, -MAX); union by per-axis min / max; surface area 2(xy + yz + zx).
struct Box {
    P3 lo{kBig, kBig, kBig}, hi{-kBig, -kBig, -kBig};
    void grow(const Box &o) {
        lo = pmin(lo, o.lo);
        hi = pmax(hi, o.hi);
    }
    float area() const {
        const P3 e = sub(hi, lo);
        return 2.0f * (e.x * e.y + e.y * e.z + e.z * e.x);
    }
};

// ---- BVHBuilder (bvh.rs:120-336) ----------------------------------------------------------------
class SahBuild {
  public:
    SahBuild(const std::vector<P3> &cen, const std::vector<Box> &box) : cen_(cen), box_(box) {
        order_.resize(cen.size());
        for (size_t i = 0; i < order_.size(); ++i) order_[i] = (uint32_t)i;
    }

    // BVHBuilder::build: children-first emission, then the array reversed so the root is node 0.
    void run(std::vector<rt_bvh_node> &nodes, std::vector<uint32_t> &prims) {
        out_.clear();
        if (!order_.empty()) emit(0, order_.size());
        const uint32_t n = (uint32_t)out_.size();
        std::reverse(out_.begin(), out_.end());
        if (n > 1)
            for (rt_bvh_node &nd : out_)
                if (nd.prim_count == 0) {
                    nd.left_first = n - 1 - nd.left_first;
                    nd.right_child = n - 1 - nd.right_child;
                }
        nodes = std::move(out_);
        prims = order_;
    }

  private:
    static constexpr size_t kLeafMax = 4;
    static constexpr int kBinCount = 12;
    const std::vector<P3> &cen_;
    const std::vector<Box> &box_;
    std::vector<uint32_t> order_;
    std::vector<rt_bvh_node> out_;

    // build_subtree (bvh.rs:152-219); returns the index of the subtree's root in out_.
    uint32_t emit(size_t first, size_t last) {
        Box bb;
        for (size_t i = first; i < last; ++i) bb.grow(box_[order_[i]]);
        rt_bvh_node nd;
        std::memset(&nd, 0, sizeof(nd));
        put3(nd.bbox_min, bb.lo);
        put3(nd.bbox_max, bb.hi);
        int axis = 0;
        size_t n_left = 0;
        const size_t n = last - first;
        if (n <= kLeafMax || !best_split(first, last, bb, axis, n_left)) {
            std::sort(order_.begin() + first, order_.begin() + last);
            nd.left_first = (uint32_t)first;
            nd.prim_count = (uint32_t)n;
            out_.push_back(nd);
            return (uint32_t)(out_.size() - 1);
        }
        const std::vector<P3> &c = cen_;
        std::nth_element(order_.begin() + first, order_.begin() + first + n_left, order_.begin() + last,
                         [&c, axis](uint32_t a, uint32_t b) {
                             const float ka = axis_of(c[a], axis), kb = axis_of(c[b], axis);
                             return ka < kb || (!(kb < ka) && a < b);
                         });
        const uint32_t l = emit(first, first + n_left);
        const uint32_t r = emit(first + n_left, last);
        nd.left_first = l;
        nd.right_child = r;
        out_.push_back(nd);
        return (uint32_t)(out_.size() - 1);
    }

    // find_best_split (bvh.rs:229-319): 12 centroid bins per axis carrying the full primitive boxes,
    // cost 1 + (A_l n_l + A_r n_r) / A; a split only when it is cheaper than n leaf tests.
    bool best_split(size_t first, size_t last, const Box &bb, int &axis_out, size_t &left_out) const {
        const float sa = bb.area();
        if (sa <= 0.0f) return false;
        const float inv_sa = 1.0f / sa;
        P3 clo{kBig, kBig, kBig}, chi{-kBig, -kBig, -kBig};
        for (size_t i = first; i < last; ++i) {
            clo = pmin(clo, cen_[order_[i]]);
            chi = pmax(chi, cen_[order_[i]]);
        }
        float best = std::numeric_limits<float>::infinity();
        bool found = false;
        for (int a = 0; a < 3; ++a) {
            const float lo = axis_of(clo, a);
            const float extent = axis_of(chi, a) - lo;
            if (extent <= 0.0f) continue;
            const float to_bin = (float)kBinCount / extent;
            Box bins[kBinCount];
            size_t counts[kBinCount] = {};
            for (size_t i = first; i < last; ++i) {
                const uint32_t p = order_[i];
                const float f = (axis_of(cen_[p], a) - lo) * to_bin;
                // `as usize`: toward zero, saturating, NaN -> 0; the top bin takes c == max
                size_t b = 0;
                if (f > 0.0f) b = f >= (float)kBinCount ? (size_t)kBinCount : (size_t)f;
                if (b > (size_t)kBinCount - 1) b = kBinCount - 1;
                counts[b] += 1;
                bins[b].grow(box_[p]);
            }
            float area_l[kBinCount], area_r[kBinCount];
            size_t cnt_l[kBinCount], cnt_r[kBinCount];
            Box run;
            size_t m = 0;
            for (int b = 0; b < kBinCount; ++b) {
                run.grow(bins[b]);
                m += counts[b];
                area_l[b] = run.area();
                cnt_l[b] = m;
            }
            run = Box();
            m = 0;
            for (int b = kBinCount - 1; b >= 0; --b) {
                run.grow(bins[b]);
                m += counts[b];
                area_r[b] = run.area();
                cnt_r[b] = m;
            }
            for (int b = 0; b + 1 < kBinCount; ++b) {
                if (cnt_l[b] == 0 || cnt_r[b + 1] == 0) continue;
                const float cost =
                    1.0f + (area_l[b] * (float)cnt_l[b] + area_r[b + 1] * (float)cnt_r[b + 1]) * inv_sa;
                if (cost < best) {
                    best = cost;
                    axis_out = a;
                    left_out = cnt_l[b];
                    found = true;
                }
            }
        }
        return found && best < (float)(last - first);
    }
};

// ---- scene model ------------------------------------------------------------------------------
struct MeshIn {
    std::vector<P3> pos, nrm;
    std::vector<float> uv;
    std::vector<uint32_t> idx;
    uint32_t material = 0;
    std::vector<uint32_t> per_tri_material;  // empty: every triangle uses `material`
};

struct Tex {
    std::vector<uint8_t> rgba8;
    uint32_t w = 0, h = 0, layers = 0;
};

struct OScene {
    std::vector<rt_triangle> tris;
    std::vector<rt_bvh_node> nodes;
    std::vector<uint32_t> prims;
    std::vector<rt_material> mats;
    std::vector<rt_light> lights;
    Tex tex[4];
    P3 lo{0, 0, 0}, hi{0, 0, 0};
    bool has_bounds = false;
    rt_camera cam;
};

void camera_defaults(rt_camera &c) {  // Camera::default (camera.rs:42-54)
    std::memset(&c, 0, sizeof(c));
    c.position[2] = 5.0f;
    c.up[1] = 1.0f;
    c.fov_degrees = 60.0f;
    c.near_plane = 0.1f;
    c.focus_dist = 5.0f;
}

// Per-primitive centroid (p0 + p1 + p2) / 3 and box (scene.rs:62-70), then the SAH build.
void index_triangles(OScene &s) {
    const size_t n = s.tris.size();
    std::vector<P3> cen(n);
    std::vector<Box> box(n);
    for (size_t i = 0; i < n; ++i) {
        const rt_triangle &t = s.tris[i];
        const P3 a{t.v0[0], t.v0[1], t.v0[2]}, b{t.v1[0], t.v1[1], t.v1[2]}, c{t.v2[0], t.v2[1], t.v2[2]};
        cen[i] = P3{(a.x + b.x + c.x) / 3.0f, (a.y + b.y + c.y) / 3.0f, (a.z + b.z + c.z) / 3.0f};
        box[i].lo = pmin(pmin(pmin(box[i].lo, a), b), c);
        box[i].hi = pmax(pmax(pmax(box[i].hi, a), b), c);
    }
    SahBuild(cen, box).run(s.nodes, s.prims);
}

// Scene::flatten (scene.rs:213-291): one TriangleGpu per index triple, mesh after mesh; bounds over
// every mesh vertex.
void flatten(OScene &s, const std::vector<MeshIn> &meshes) {
    s.tris.clear();
    P3 lo{kBig, kBig, kBig}, hi{-kBig, -kBig, -kBig};
    for (const MeshIn &m : meshes) {
        for (const P3 &p : m.pos) {
            lo = pmin(lo, p);
            hi = pmax(hi, p);
        }
        for (size_t k = 0; k + 2 < m.idx.size(); k += 3) {
            rt_triangle t;
            std::memset(&t, 0, sizeof(t));
            float *v[3] = {t.v0, t.v1, t.v2}, *nn[3] = {t.n0, t.n1, t.n2}, *uv[3] = {t.uv0, t.uv1, t.uv2};
            for (int j = 0; j < 3; ++j) {
                const uint32_t ix = m.idx[k + j];
                put3(v[j], ix < m.pos.size() ? m.pos[ix] : P3{0, 0, 0});
                put3(nn[j], ix < m.nrm.size() ? m.nrm[ix] : P3{0, 1, 0});
                if (2 * (size_t)ix + 1 < m.uv.size()) {
                    uv[j][0] = m.uv[2 * ix];
                    uv[j][1] = m.uv[2 * ix + 1];
                }
            }
            t.material_id = m.per_tri_material.empty() ? m.material : m.per_tri_material[k / 3];
            s.tris.push_back(t);
        }
    }
    s.has_bounds = !(lo.x > hi.x);
    s.lo = s.has_bounds ? lo : P3{0, 0, 0};
    s.hi = s.has_bounds ? hi : P3{0, 0, 0};
    index_triangles(s);
}

// Material constructors (material.rs:101-140) and light_to_gpu (rustracer-renderer/src/lib.rs:1231-1282).
rt_material lambert(float r, float g, float b) {
    rt_material m;
    std::memset(&m, 0, sizeof(m));
    m.albedo[0] = r;
    m.albedo[1] = g;
    m.albedo[2] = b;
    m.albedo[3] = 1.0f;
    m.roughness = 1.0f;
    m.ior = 1.5f;
    m.kind = RT_MAT_LAMBERTIAN;
    m.tex_albedo = m.tex_mr = m.tex_emissive = m.tex_normal = RT_TEX_NONE;
    return m;
}
rt_material metal(float r, float g, float b, float rough) {
    rt_material m = lambert(r, g, b);
    m.kind = RT_MAT_METAL;
    m.roughness = std::fmin(std::fmax(rough, 0.001f), 1.0f);
    m.metallic = 1.0f;
    return m;
}
rt_material glass(float ior) {
    rt_material m = lambert(1.0f, 1.0f, 1.0f);
    m.kind = RT_MAT_DIELECTRIC;
    m.roughness = 0.0f;
    m.ior = ior;
    return m;
}
rt_material emitter(float r, float g, float b, float intensity) {  // albedo = colour, roughness default
    rt_material m = lambert(r, g, b);
    m.kind = RT_MAT_EMISSIVE;
    m.roughness = 0.5f;
    m.emissive[0] = r * intensity;
    m.emissive[1] = g * intensity;
    m.emissive[2] = b * intensity;
    return m;
}
rt_light area_light(uint32_t tri, float e) {
    rt_light l;
    std::memset(&l, 0, sizeof(l));
    l.data[0] = (float)tri;
    l.color[0] = l.color[1] = l.color[2] = e;
    l.intensity = 1.0f;
    l.kind = RT_LIGHT_AREA;
    return l;
}

// create_quad (scene.rs:463-480): shared flat normal, unit-square uvs, triangles (0,1,2), (0,2,3).
MeshIn quad(P3 a, P3 b, P3 c, P3 d, uint32_t mat) {
    MeshIn m;
    m.pos = {a, b, c, d};
    const P3 n = unit(cross3(sub(b, a), sub(c, a)));
    m.nrm = {n, n, n, n};
    m.uv = {0, 0, 1, 0, 1, 1, 0, 1};
    m.idx = {0, 1, 2, 0, 2, 3};
    m.material = mat;
    return m;
}

// The six faces of a box (create_cube's face order, scene.rs:483-505) from its corners k[x + 2y + 4z].
void box_faces(std::vector<MeshIn> &out, const P3 k[8], uint32_t mat) {
    static const int f[6][4] = {{0, 2, 6, 4}, {5, 7, 3, 1}, {4, 5, 1, 0}, {2, 3, 7, 6}, {1, 3, 2, 0}, {4, 6, 7, 5}};
    for (const auto &q : f) out.push_back(quad(k[q[0]], k[q[1]], k[q[2]], k[q[3]], mat));
}

// The box [0,sx]x[0,sy]x[0,sz] turned about +y by `deg` degrees (in double), then moved by t.
void turned_box(std::vector<MeshIn> &out, double sx, double sy, double sz, double deg, P3 t, uint32_t mat) {
    const double a = deg * 3.14159265358979323846 / 180.0;
    const double ca = std::cos(a), sa = std::sin(a);
    P3 k[8];
    for (int i = 0; i < 8; ++i) {
        const double x = (i & 1) ? sx : 0.0, y = (i & 2) ? sy : 0.0, z = (i & 4) ? sz : 0.0;
        k[i] = P3{(float)(ca * x + sa * z + t.x), (float)(y + t.y), (float)(-sa * x + ca * z + t.z)};
    }
    box_faces(out, k, mat);
}

// The workloads' host generator: splitmix64, uniform = top 53 bits / 2^53, normal = Irwin-Hall
// (twelve uniforms minus 6).
struct SplitMix64 {
    uint64_t state;
    uint64_t bits() {
        state += 0x9E3779B97F4A7C15ull;
        uint64_t z = state;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    }
    double uniform() { return (double)(bits() >> 11) / 9007199254740992.0; }
    double gauss() {
        double s = 0.0;
        for (int i = 0; i < 12; ++i) s += uniform();
        return s - 6.0;
    }
};

// Periodic two-octave value noise in [0, 1]: lattices of n x n and 2n x 2n seeded values,
// smoothstep-weighted bilinear interpolation at texel centres.
std::vector<float> value_noise(uint32_t size, uint32_t n, SplitMix64 &rng) {
    std::vector<float> coarse((size_t)n * n), fine((size_t)4 * n * n);
    for (float &v : coarse) v = (float)rng.uniform();
    for (float &v : fine) v = (float)rng.uniform();
    auto lookup = [](const std::vector<float> &lat, uint32_t m, float u, float v) {
        const float x = u * (float)m, y = v * (float)m;
        const uint32_t ix = (uint32_t)x, iy = (uint32_t)y;
        float wx = x - (float)ix, wy = y - (float)iy;
        wx = wx * wx * (3.0f - 2.0f * wx);
        wy = wy * wy * (3.0f - 2.0f * wy);
        const uint32_t x0 = ix % m, y0 = iy % m, x1 = (ix + 1) % m, y1 = (iy + 1) % m;
        const float p = lat[(size_t)y0 * m + x0], q = lat[(size_t)y0 * m + x1];
        const float r = lat[(size_t)y1 * m + x0], s = lat[(size_t)y1 * m + x1];
        const float top = p + (q - p) * wx, bottom = r + (s - r) * wx;
        return top + (bottom - top) * wy;
    };
    std::vector<float> out((size_t)size * size);
    for (uint32_t y = 0; y < size; ++y)
        for (uint32_t x = 0; x < size; ++x) {
            const float u = ((float)x + 0.5f) / (float)size, v = ((float)y + 0.5f) / (float)size;
            out[(size_t)y * size + x] = 0.65f * lookup(coarse, n, u, v) + 0.35f * lookup(fine, 2 * n, u, v);
        }
    return out;
}

// create_role_array's quantisation (rustracer-renderer/src/lib.rs:1315-1326): truncating.
inline uint8_t to_u8(float c) { return (uint8_t)(std::fmin(std::fmax(c, 0.0f), 1.0f) * 255.0f); }

OScene *make_cornell() {
    OScene *s = new OScene();
    s->mats = {lambert(0.73f, 0.73f, 0.73f), lambert(0.65f, 0.05f, 0.05f), lambert(0.12f, 0.45f, 0.15f),
               emitter(15.0f, 15.0f, 15.0f, 1.0f)};
    const float L = 555.0f;
    std::vector<MeshIn> m;
    m.push_back(quad({0, 0, 0}, {0, 0, L}, {L, 0, L}, {L, 0, 0}, 0));  // floor
    m.push_back(quad({0, L, 0}, {L, L, 0}, {L, L, L}, {0, L, L}, 0));  // ceiling
    m.push_back(quad({0, 0, L}, {0, L, L}, {L, L, L}, {L, 0, L}, 0));  // back
    m.push_back(quad({L, 0, 0}, {L, 0, L}, {L, L, L}, {L, L, 0}, 1));  // x = 555, red
    m.push_back(quad({0, 0, 0}, {0, L, 0}, {0, L, L}, {0, 0, L}, 2));  // x = 0, green
    m.push_back(quad({213, 554, 227}, {343, 554, 227}, {343, 554, 332}, {213, 554, 332}, 3));  // light: tris 10, 11
    turned_box(m, 165.0, 165.0, 165.0, -18.0, {130, 0, 65}, 0);
    turned_box(m, 165.0, 330.0, 165.0, 15.0, {265, 0, 295}, 0);
    s->lights = {area_light(10, 15.0f), area_light(11, 15.0f)};
    camera_defaults(s->cam);
    s->cam.position[0] = 278.0f;
    s->cam.position[1] = 278.0f;
    s->cam.position[2] = -800.0f;
    s->cam.look_at[0] = 278.0f;
    s->cam.look_at[1] = 278.0f;
    s->cam.fov_degrees = 40.0f;
    s->cam.focus_dist = 800.0f;
    flatten(*s, m);
    return s;
}

OScene *make_icosphere_room(uint32_t level, uint64_t seed, float sigma, uint32_t tex_size) {
    OScene *s = new OScene();
    SplitMix64 rng{seed * 0x2545F4914F6CDD1Dull + 0x1234567ull};
    // Icosahedron on the unit sphere, faces turned outward, then `level` 4:1 subdivisions with the
    // edge midpoints pushed back onto the sphere (a midpoint is numbered when first met).
    const float g = 1.6180339887498949f;
    std::vector<P3> v = {{-1, g, 0}, {1, g, 0}, {-1, -g, 0}, {1, -g, 0}, {0, -1, g}, {0, 1, g},
                         {0, -1, -g}, {0, 1, -g}, {g, 0, -1}, {g, 0, 1}, {-g, 0, -1}, {-g, 0, 1}};
    for (P3 &p : v) p = unit(p);
    std::vector<uint32_t> f = {0, 11, 5, 0, 5, 1, 0, 1, 7, 0, 7, 10, 0, 10, 11, 1, 5, 9, 5, 11, 4, 11, 10, 2, 10, 7, 6,
                               7, 1, 8, 3, 9, 4, 3, 4, 2, 3, 2, 6, 3, 6, 8, 3, 8, 9, 4, 9, 5, 2, 4, 11, 6, 2, 10, 8, 6,
                               7, 9, 8, 1};
    for (size_t i = 0; i < f.size(); i += 3) {
        const P3 a = v[f[i]], b = v[f[i + 1]], c = v[f[i + 2]];
        if (dot3(cross3(sub(b, a), sub(c, a)), add(add(a, b), c)) < 0.0f) std::swap(f[i + 1], f[i + 2]);
    }
    for (uint32_t it = 0; it < level; ++it) {
        std::unordered_map<uint64_t, uint32_t> seen;
        seen.reserve(f.size() * 2);
        auto mid = [&](uint32_t a, uint32_t b) -> uint32_t {
            const uint64_t key = a < b ? ((uint64_t)a << 32) | b : ((uint64_t)b << 32) | a;
            const auto [pos, fresh] = seen.try_emplace(key, (uint32_t)v.size());
            if (fresh) v.push_back(unit(scale(add(v[a], v[b]), 0.5f)));
            return pos->second;
        };
        std::vector<uint32_t> next;
        next.reserve(f.size() * 4);
        for (size_t i = 0; i < f.size(); i += 3) {
            const uint32_t a = f[i], b = f[i + 1], c = f[i + 2];
            const uint32_t ab = mid(a, b);
            const uint32_t bc = mid(b, c);
            const uint32_t ca = mid(c, a);
            for (uint32_t x : {a, ab, ca, b, bc, ab, c, ca, bc, ab, bc, ca}) next.push_back(x);
        }
        f.swap(next);
    }
    for (P3 &p : v) p = scale(p, 1.0f + sigma * (float)rng.gauss());
    std::vector<P3> nrm(v.size(), P3{0, 0, 0});
    for (size_t i = 0; i < f.size(); i += 3) {
        const P3 fn = cross3(sub(v[f[i + 1]], v[f[i]]), sub(v[f[i + 2]], v[f[i]]));
        for (int k = 0; k < 3; ++k) nrm[f[i + k]] = add(nrm[f[i + k]], fn);
    }
    for (P3 &n : nrm) n = unit(n);
    std::vector<float> uv(2 * v.size());
    for (size_t i = 0; i < v.size(); ++i) {
        uv[2 * i] = (v[i].x + 1.0f) * 1.0f;
        uv[2 * i + 1] = (v[i].y + 1.0f) * 1.0f;
    }
    // Materials: 0 room, 1 light, then one per sphere triangle drawn from the seed.
    s->mats = {lambert(0.73f, 0.73f, 0.73f), emitter(20.0f, 20.0f, 20.0f, 1.0f)};
    const uint32_t layer = tex_size ? 0u : RT_TEX_NONE;
    const size_t nf = f.size() / 3;
    for (size_t i = 0; i < nf; ++i) {
        const double pick = rng.uniform();
        rt_material m;
        if (pick < 0.60) {
            const float r = (float)(0.2 + 0.6 * rng.uniform());
            const float gg = (float)(0.2 + 0.6 * rng.uniform());
            const float b = (float)(0.2 + 0.6 * rng.uniform());
            m = lambert(r, gg, b);
        } else if (pick < 0.85) {
            const float r = (float)(0.5 + 0.45 * rng.uniform());
            const float gg = (float)(0.5 + 0.45 * rng.uniform());
            const float b = (float)(0.5 + 0.45 * rng.uniform());
            const float rough = (float)(0.05 + 0.55 * rng.uniform());
            m = metal(r, gg, b, rough);
        } else {
            m = glass(1.5f);
        }
        if (m.kind != RT_MAT_DIELECTRIC) m.tex_albedo = m.tex_mr = layer;
        m.tex_normal = layer;
        s->mats.push_back(m);
    }
    const float R = 5.0f, ly = R - 0.01f;
    std::vector<MeshIn> m;
    m.push_back(quad({-R, -R, -R}, {-R, -R, R}, {R, -R, R}, {R, -R, -R}, 0));
    m.push_back(quad({-R, R, -R}, {R, R, -R}, {R, R, R}, {-R, R, R}, 0));
    m.push_back(quad({-R, -R, -R}, {R, -R, -R}, {R, R, -R}, {-R, R, -R}, 0));
    m.push_back(quad({-R, -R, R}, {-R, R, R}, {R, R, R}, {R, -R, R}, 0));
    m.push_back(quad({-R, -R, -R}, {-R, R, -R}, {-R, R, R}, {-R, -R, R}, 0));
    m.push_back(quad({R, -R, -R}, {R, -R, R}, {R, R, R}, {R, R, -R}, 0));
    m.push_back(quad({-0.5f, ly, -0.5f}, {0.5f, ly, -0.5f}, {0.5f, ly, 0.5f}, {-0.5f, ly, 0.5f}, 1));  // tris 12, 13
    MeshIn sphere;
    sphere.pos = v;
    sphere.nrm = nrm;
    sphere.uv = uv;
    sphere.idx = f;
    sphere.material = 2;
    sphere.per_tri_material.resize(nf);
    for (size_t i = 0; i < nf; ++i) sphere.per_tri_material[i] = (uint32_t)(2 + i);
    m.push_back(std::move(sphere));
    s->lights = {area_light(12, 20.0f), area_light(13, 20.0f)};
    for (int i = 0; i < 4; ++i) {
        const float x = (float)(-4.0 + 8.0 * rng.uniform());
        const float y = (float)(1.5 + 3.0 * rng.uniform());
        const float z = (float)(-4.0 + 8.0 * rng.uniform());
        rt_light l;
        std::memset(&l, 0, sizeof(l));
        l.data[0] = x;
        l.data[1] = y;
        l.data[2] = z;
        l.color[0] = 1.0f;
        l.color[1] = 0.95f;
        l.color[2] = 0.9f;
        l.intensity = 8.0f;
        l.kind = RT_LIGHT_POINT;
        s->lights.push_back(l);
    }
    if (tex_size) {
        const std::vector<float> a = value_noise(tex_size, 16, rng);
        const std::vector<float> b = value_noise(tex_size, 16, rng);
        const std::vector<float> c = value_noise(tex_size, 32, rng);
        const size_t n = (size_t)tex_size * tex_size;
        for (int role : {RT_TEX_ALBEDO, RT_TEX_MR, RT_TEX_NORMAL}) {
            s->tex[role].rgba8.assign(4 * n, 255);
            s->tex[role].w = s->tex[role].h = tex_size;
            s->tex[role].layers = 1;
        }
        uint8_t *alb = s->tex[RT_TEX_ALBEDO].rgba8.data(), *mr = s->tex[RT_TEX_MR].rgba8.data(),
                *nm = s->tex[RT_TEX_NORMAL].rgba8.data();
        for (size_t i = 0; i < n; ++i) {
            alb[4 * i] = to_u8(0.35f + 0.65f * a[i]);
            alb[4 * i + 1] = to_u8(0.35f + 0.65f * b[i]);
            alb[4 * i + 2] = to_u8(0.35f + 0.65f * c[i]);
            mr[4 * i + 1] = to_u8(0.5f + 0.5f * b[i]);  // roughness in G; R and B stay 255
            const float nx = (a[i] - 0.5f) * 0.6f, ny = (c[i] - 0.5f) * 0.6f;
            const float nz = std::sqrt(std::fmax(1.0f - nx * nx - ny * ny, 0.0f));
            nm[4 * i] = to_u8(0.5f + 0.5f * nx);
            nm[4 * i + 1] = to_u8(0.5f + 0.5f * ny);
            nm[4 * i + 2] = to_u8(0.5f + 0.5f * nz);
        }
    }
    camera_defaults(s->cam);
    s->cam.position[0] = 1.2f;
    s->cam.position[1] = 0.8f;
    s->cam.position[2] = 2.4f;
    flatten(*s, m);
    return s;
}

}  // namespace

extern "C" {

void *oracle_scene_cornell555(void) { return make_cornell(); }

void *oracle_scene_icosphere_room(uint32_t level, uint64_t seed, float sigma, uint32_t tex_size) {
    if (level > 10 || tex_size > 8192) return nullptr;
    return make_icosphere_room(level, seed, sigma, tex_size);
}

// A scene from flattened arrays (any scene the CUDA backend renders: glTF, test-built meshes); the
// oracle indexes it with its own BVH build.  Bounds over the triangles' vertices.
void *oracle_scene_from_arrays(const rt_triangle *tris, uint64_t n_tris, const rt_material *mats, uint64_t n_mats,
                               const rt_light *lights, uint64_t n_lights, const rt_texture_array *tex4) {
    OScene *s = new (std::nothrow) OScene();
    if (!s) return nullptr;
    s->tris.assign(tris, tris + n_tris);
    s->mats.assign(mats, mats + n_mats);
    s->lights.assign(lights, lights + n_lights);
    for (int r = 0; r < 4 && tex4; ++r) {
        const rt_texture_array &t = tex4[r];
        if (!t.layers || !t.rgba8) continue;
        s->tex[r].w = t.width;
        s->tex[r].h = t.height;
        s->tex[r].layers = t.layers;
        s->tex[r].rgba8.assign(t.rgba8, t.rgba8 + (size_t)t.width * t.height * t.layers * 4);
    }
    P3 lo{kBig, kBig, kBig}, hi{-kBig, -kBig, -kBig};
    for (const rt_triangle &t : s->tris)
        for (const float *p : {t.v0, t.v1, t.v2}) {
            lo = pmin(lo, P3{p[0], p[1], p[2]});
            hi = pmax(hi, P3{p[0], p[1], p[2]});
        }
    s->has_bounds = !(lo.x > hi.x);
    s->lo = s->has_bounds ? lo : P3{0, 0, 0};
    s->hi = s->has_bounds ? hi : P3{0, 0, 0};
    camera_defaults(s->cam);
    index_triangles(*s);
    return s;
}

void oracle_scene_describe(void *h, rt_scene_desc *d) {
    const OScene *s = (const OScene *)h;
    std::memset(d, 0, sizeof(*d));
    d->triangles = s->tris.data();
    d->triangle_count = s->tris.size();
    d->bvh_nodes = s->nodes.data();
    d->bvh_node_count = s->nodes.size();
    d->bvh_prims = s->prims.data();
    d->bvh_prim_count = s->prims.size();
    d->materials = s->mats.data();
    d->material_count = s->mats.size();
    d->lights = s->lights.data();
    d->light_count = s->lights.size();
    rt_texture_array *roles[4] = {&d->tex_albedo, &d->tex_mr, &d->tex_emissive, &d->tex_normal};
    for (int r = 0; r < 4; ++r) {
        roles[r]->rgba8 = s->tex[r].layers ? s->tex[r].rgba8.data() : nullptr;
        roles[r]->width = s->tex[r].w;
        roles[r]->height = s->tex[r].h;
        roles[r]->layers = s->tex[r].layers;
    }
    put3(d->bounds_min, s->lo);
    put3(d->bounds_max, s->hi);
    d->has_bounds = s->has_bounds ? 1u : 0u;
}

void oracle_scene_camera(void *h, rt_camera *c) { *c = ((const OScene *)h)->cam; }

void oracle_scene_destroy(void *h) { delete (OScene *)h; }

// The SAH build alone on raw primitive centroids and boxes (the reference's BVH tests drive its
// builder this way).  nodes needs room for 2n - 1 records, prims for n; returns the node count.
uint64_t oracle_bvh_build(const float *centroids, const float *bmin, const float *bmax, uint64_t n,
                          rt_bvh_node *nodes, uint32_t *prims) {
    std::vector<P3> cen(n);
    std::vector<Box> box(n);
    for (uint64_t i = 0; i < n; ++i) {
        cen[i] = P3{centroids[3 * i], centroids[3 * i + 1], centroids[3 * i + 2]};
        box[i].lo = P3{bmin[3 * i], bmin[3 * i + 1], bmin[3 * i + 2]};
        box[i].hi = P3{bmax[3 * i], bmax[3 * i + 1], bmax[3 * i + 2]};
    }
    std::vector<rt_bvh_node> nd;
    std::vector<uint32_t> pr;
    SahBuild(cen, box).run(nd, pr);
    std::memcpy(nodes, nd.data(), nd.size() * sizeof(rt_bvh_node));
    std::memcpy(prims, pr.data(), pr.size() * sizeof(uint32_t));
    return nd.size();
}

}  // extern "C"
