// Host-side scene model of the backend: the part of rustracer-core the frame path consumes.
//
//   * mesh flattening            rustracer-core/src/scene.rs:213-273  (flatten_triangles)
//   * binned-SAH BVH build       rustracer-core/src/bvh.rs:135-336    (BVHBuilder::build)
//   * scene bounds               rustracer-core/src/scene.rs:198-210
//   * camera uniform / framing   rustracer-core/src/camera.rs:278-345
//   * photon-grid derivation     rustracer-renderer/src/lib.rs:416-457
//   * RenderConfig::default      rustracer-renderer/src/lib.rs:44-65
//   * procedural scenes for the measured workloads (555-unit Cornell box, displaced icosphere room)
//
// Compiled with -ffp-contract=off so results are identical on x86-64 and AArch64 hosts; values that
// need a transcendental function are computed in double precision and rounded once.
#include <algorithm>
#include <array>
#include <cmath>
#include <cstring>
#include <limits>
#include <atomic>
#include <memory>
#include <new>
#include <thread>
#include <unordered_map>

#include "rt_internal.h"

namespace rt {

static thread_local std::string g_last_error;

void set_error(const char *fmt, ...) {
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_last_error = buf;
}
void clear_error() { g_last_error.clear(); }

Vec3 normalize(Vec3 a) {
    float inv = 1.0f / std::sqrt(dot(a, a));
    return a * inv;
}

// ------------------------------------------------------------------------------------------------
// BVH (bvh.rs:120-336).  Same algorithm: 12 centroid bins per axis, bins carry the union of the full
// primitive AABBs, split cost 1 + (A_l n_l + A_r n_r) / A, leaf when that is not below n, at most 4
// primitives per leaf, children emitted before parents and the array reversed so the root is node 0.
// The partition is a selection by (centroid[axis], primitive index) and a leaf lists its primitives
// in index order: the reference's select_nth_unstable_by leaves both orders unspecified, this one
// fixes them.
// ------------------------------------------------------------------------------------------------
namespace {

struct Aabb {
    Vec3 mn, mx;
};
constexpr float F32_MAX = std::numeric_limits<float>::max();
inline Aabb aabb_empty() { return {{F32_MAX, F32_MAX, F32_MAX}, {-F32_MAX, -F32_MAX, -F32_MAX}}; }
inline float fmin_(float a, float b) { return std::fmin(a, b); }
inline float fmax_(float a, float b) { return std::fmax(a, b); }
inline Aabb aabb_union(const Aabb &a, const Aabb &b) {
    return {{fmin_(a.mn.x, b.mn.x), fmin_(a.mn.y, b.mn.y), fmin_(a.mn.z, b.mn.z)},
            {fmax_(a.mx.x, b.mx.x), fmax_(a.mx.y, b.mx.y), fmax_(a.mx.z, b.mx.z)}};
}
inline float surface_area(const Aabb &b) {
    Vec3 e = b.mx - b.mn;
    return 2.0f * (e.x * e.y + e.y * e.z + e.z * e.x);
}
inline float comp(const Vec3 &v, int axis) { return axis == 0 ? v.x : (axis == 1 ? v.y : v.z); }

// Worker threads of the host BVH build (0: one per hardware thread).
std::atomic<unsigned> g_host_threads{0};

struct Builder {
    const std::vector<Vec3> &centroids;
    std::vector<Aabb> boxes;
    std::vector<rt_bvh_node> nodes;
    std::vector<uint32_t> prims;
    static constexpr size_t kMaxLeaf = 4;
    static constexpr int kBins = 12;
    // Subtrees with at least this many primitives near the top of the tree are built on their own
    // thread; the result is identical to the sequential build (see build()).
    static constexpr size_t kParallelMin = 8192;

    bool best_split(size_t start, size_t end, const Aabb &bb, int *axis_out, size_t *left_out) const {
        float bb_sa = surface_area(bb);
        if (!(bb_sa > 0.0f)) return false;
        float inv_bb_sa = 1.0f / bb_sa;
        Vec3 cmin{F32_MAX, F32_MAX, F32_MAX}, cmax{-F32_MAX, -F32_MAX, -F32_MAX};
        for (size_t i = start; i < end; ++i) {
            const Vec3 &c = centroids[prims[i]];
            cmin = {fmin_(cmin.x, c.x), fmin_(cmin.y, c.y), fmin_(cmin.z, c.z)};
            cmax = {fmax_(cmax.x, c.x), fmax_(cmax.y, c.y), fmax_(cmax.z, c.z)};
        }
        int best_axis = 0;
        size_t best_left = 0;
        float best_cost = std::numeric_limits<float>::infinity();
        for (int axis = 0; axis < 3; ++axis) {
            float lo = comp(cmin, axis);
            float range = comp(cmax, axis) - lo;
            if (range <= 0.0f) continue;
            float scale = (float)kBins / range;
            Aabb bin_box[kBins];
            size_t bin_cnt[kBins];
            for (int b = 0; b < kBins; ++b) {
                bin_box[b] = aabb_empty();
                bin_cnt[b] = 0;
            }
            for (size_t i = start; i < end; ++i) {
                uint32_t p = prims[i];
                float f = (comp(centroids[p], axis) - lo) * scale;
                // Rust `as usize`: truncation toward zero, saturating, NaN -> 0.
                size_t bin = (f != f || f <= 0.0f) ? 0 : (f >= 1e18f ? (size_t)kBins : (size_t)f);
                if (bin >= (size_t)kBins) bin = kBins - 1;
                bin_cnt[bin] += 1;
                bin_box[bin] = aabb_union(bin_box[bin], boxes[p]);
            }
            float left_area[kBins], right_area[kBins];
            size_t left_cnt[kBins], right_cnt[kBins];
            Aabb acc = aabb_empty();
            size_t n = 0;
            for (int b = 0; b < kBins; ++b) {
                acc = aabb_union(acc, bin_box[b]);
                n += bin_cnt[b];
                left_area[b] = surface_area(acc);
                left_cnt[b] = n;
            }
            acc = aabb_empty();
            n = 0;
            for (int b = kBins - 1; b >= 0; --b) {
                acc = aabb_union(acc, bin_box[b]);
                n += bin_cnt[b];
                right_area[b] = surface_area(acc);
                right_cnt[b] = n;
            }
            for (int b = 0; b < kBins - 1; ++b) {
                size_t lc = left_cnt[b], rc = right_cnt[b + 1];
                if (lc == 0 || rc == 0) continue;
                float cost = 1.0f + (left_area[b] * (float)lc + right_area[b + 1] * (float)rc) * inv_bb_sa;
                if (cost < best_cost) {
                    best_cost = cost;
                    best_axis = axis;
                    best_left = lc;
                }
            }
        }
        float leaf_cost = (float)(end - start);
        if (best_cost < leaf_cost) {
            *axis_out = best_axis;
            *left_out = best_left;
            return true;
        }
        return false;
    }

    // Appends the subtree over prims[start, end) to `out` in post-order (children before parent) and
    // returns its root's index in `out`.  With par_depth > 0 the left subtree is built on another
    // thread into its own vector and both are appended in the sequential order afterwards, their
    // child indices shifted: the nodes and the prim order equal those of the sequential build.
    uint32_t build(size_t start, size_t end, std::vector<rt_bvh_node> &out, int par_depth) {
        size_t count = end - start;
        if (count == 0) return 0;
        Aabb bb = aabb_empty();
        for (size_t i = start; i < end; ++i) bb = aabb_union(bb, boxes[prims[i]]);
        int axis = 0;
        size_t left_count = 0;
        bool split = count > kMaxLeaf && best_split(start, end, bb, &axis, &left_count);
        rt_bvh_node node;
        std::memset(&node, 0, sizeof(node));
        node.bbox_min[0] = bb.mn.x; node.bbox_min[1] = bb.mn.y; node.bbox_min[2] = bb.mn.z;
        node.bbox_max[0] = bb.mx.x; node.bbox_max[1] = bb.mx.y; node.bbox_max[2] = bb.mx.z;
        if (!split) {
            // A leaf's primitives in index order: the selection leaves their order unspecified, and
            // it decides which of two triangles hit at exactly equal t the traversal reports.
            std::sort(prims.begin() + start, prims.begin() + end);
            node.left_first = (uint32_t)start;
            node.right_child = 0;
            node.prim_count = (uint32_t)count;
            out.push_back(node);
            return (uint32_t)(out.size() - 1);
        }
        size_t mid = start + left_count;
        const std::vector<Vec3> &cs = centroids;
        std::nth_element(prims.begin() + start, prims.begin() + mid, prims.begin() + end,
                         [&cs, axis](uint32_t a, uint32_t b) {
                             float ca = comp(cs[a], axis), cb = comp(cs[b], axis);
                             if (ca < cb) return true;
                             if (cb < ca) return false;
                             return a < b;
                         });
        uint32_t left, right;
        if (par_depth > 0 && count >= kParallelMin) {
            std::vector<rt_bvh_node> lnodes, rnodes;
            uint32_t lroot = 0;
            std::thread t([&] { lroot = build(start, mid, lnodes, par_depth - 1); });
            const uint32_t rroot = build(mid, end, rnodes, par_depth - 1);
            t.join();
            const uint32_t lbase = (uint32_t)out.size();
            for (rt_bvh_node nd : lnodes) {
                if (nd.prim_count == 0) {
                    nd.left_first += lbase;
                    nd.right_child += lbase;
                }
                out.push_back(nd);
            }
            const uint32_t rbase = (uint32_t)out.size();
            for (rt_bvh_node nd : rnodes) {
                if (nd.prim_count == 0) {
                    nd.left_first += rbase;
                    nd.right_child += rbase;
                }
                out.push_back(nd);
            }
            left = lbase + lroot;
            right = rbase + rroot;
        } else {
            left = build(start, mid, out, 0);
            right = build(mid, end, out, 0);
        }
        node.left_first = left;
        node.right_child = right;
        node.prim_count = 0;
        out.push_back(node);
        return (uint32_t)(out.size() - 1);
    }
};

}  // namespace

BVH build_bvh(const std::vector<Vec3> &centroids, const std::vector<Vec3> &bmin, const std::vector<Vec3> &bmax) {
    Builder b{centroids, {}, {}, {}};
    size_t n = centroids.size();
    b.boxes.resize(n);
    for (size_t i = 0; i < n; ++i) b.boxes[i] = {bmin[i], bmax[i]};
    b.prims.resize(n);
    for (size_t i = 0; i < n; ++i) b.prims[i] = (uint32_t)i;
    b.nodes.reserve(n > 0 ? 2 * n / 2 + 1 : 0);
    unsigned threads = g_host_threads.load();
    if (threads == 0) threads = std::max(1u, std::thread::hardware_concurrency());
    int par_depth = 0;
    while ((1u << par_depth) < threads && par_depth < 8) ++par_depth;
    b.build(0, n, b.nodes, par_depth);
    // reverse_nodes (bvh.rs:322-335)
    size_t cnt = b.nodes.size();
    if (cnt > 1) {
        std::reverse(b.nodes.begin(), b.nodes.end());
        for (auto &nd : b.nodes) {
            if (nd.prim_count == 0) {
                nd.left_first = (uint32_t)(cnt - 1 - nd.left_first);
                nd.right_child = (uint32_t)(cnt - 1 - nd.right_child);
            }
        }
    }
    BVH out;
    out.nodes = std::move(b.nodes);
    out.prims = std::move(b.prims);
    return out;
}

// ------------------------------------------------------------------------------------------------
// Traversal layout (child-pair records over the reference's tree)
// ------------------------------------------------------------------------------------------------
static inline uint32_t f2bits(float f) {
    uint32_t u;
    std::memcpy(&u, &f, 4);
    return u;
}
static inline float bits2f(uint32_t u) {
    float f;
    std::memcpy(&f, &u, 4);
    return f;
}

bool build_traversal_layout(const rt_bvh_node *nodes, uint64_t n_nodes, const uint32_t *prims, uint64_t n_prims,
                            const rt_triangle *tris, uint64_t n_tris, TraversalLayout &out) {
    out.cnodes.clear();
    out.tri_ord.clear();
    out.max_depth = 0;
    if (n_nodes == 0) return true;
    // Leaf-ordered triangles: slot k holds triangle prims[k] with its two edges precomputed.
    out.tri_ord.resize(n_prims * 12);
    for (uint64_t k = 0; k < n_prims; ++k) {
        uint32_t id = prims[k];
        if (id >= n_tris) {
            set_error("BVH prim slot %llu references triangle %u of %llu", (unsigned long long)k, id,
                      (unsigned long long)n_tris);
            return false;
        }
        const rt_triangle &t = tris[id];
        float *o = &out.tri_ord[k * 12];
        o[0] = t.v0[0]; o[1] = t.v0[1]; o[2] = t.v0[2]; o[3] = bits2f(id);
        o[4] = t.v1[0] - t.v0[0]; o[5] = t.v1[1] - t.v0[1]; o[6] = t.v1[2] - t.v0[2]; o[7] = 0.0f;
        o[8] = t.v2[0] - t.v0[0]; o[9] = t.v2[1] - t.v0[1]; o[10] = t.v2[2] - t.v0[2]; o[11] = 0.0f;
    }
    auto leaf_ok = [&](const rt_bvh_node &n) { return (uint64_t)n.left_first + n.prim_count <= n_prims; };
    // Record index of every internal node, in node order (the root, node 0, gets record 0).
    std::vector<uint32_t> rec(n_nodes, 0xFFFFFFFFu);
    uint32_t n_int = 0;
    for (uint64_t i = 0; i < n_nodes; ++i)
        if (nodes[i].prim_count == 0) rec[i] = n_int++;
    auto child = [&](uint32_t c, float *box_lo, float *box_hi, uint32_t *ref, uint32_t *cnt) -> bool {
        if (c >= n_nodes) {
            set_error("BVH child index %u out of range (%llu nodes)", c, (unsigned long long)n_nodes);
            return false;
        }
        const rt_bvh_node &n = nodes[c];
        for (int a = 0; a < 3; ++a) {
            box_lo[a] = n.bbox_min[a];
            box_hi[a] = n.bbox_max[a];
        }
        if (n.prim_count > 0) {
            if (!leaf_ok(n)) {
                set_error("BVH leaf %u exceeds the prim-index array", c);
                return false;
            }
            *ref = n.left_first;
            *cnt = n.prim_count;
        } else {
            *ref = rec[c];
            *cnt = 0;
        }
        return true;
    };
    auto emit = [&](uint32_t l, uint32_t r) -> bool {
        float q[16];
        uint32_t lref, lcnt, rref, rcnt;
        if (!child(l, &q[0], &q[4], &lref, &lcnt) || !child(r, &q[8], &q[12], &rref, &rcnt)) return false;
        q[3] = bits2f(lref);
        q[7] = bits2f(lcnt);
        q[11] = bits2f(rref);
        q[15] = bits2f(rcnt);
        out.cnodes.insert(out.cnodes.end(), q, q + 16);
        return true;
    };
    if (nodes[0].prim_count > 0) {  // single-leaf tree: both children are the root leaf
        if (!emit(0, 0)) return false;
        out.max_depth = 0;
        return true;
    }
    out.cnodes.reserve((size_t)n_int * 16);
    for (uint64_t i = 0; i < n_nodes; ++i)
        if (nodes[i].prim_count == 0 && !emit(nodes[i].left_first, nodes[i].right_child)) return false;
    // Depth (iterative; also rejects cycles by bounding the walk to n_nodes visits).
    std::vector<std::pair<uint32_t, uint32_t>> st{{0u, 0u}};
    uint64_t visits = 0;
    while (!st.empty()) {
        auto [i, d] = st.back();
        st.pop_back();
        if (++visits > n_nodes) {
            set_error("BVH is not a tree (a node is reachable twice)");
            return false;
        }
        out.max_depth = std::max(out.max_depth, d);
        if (nodes[i].prim_count == 0) {
            st.push_back({nodes[i].left_first, d + 1});
            st.push_back({nodes[i].right_child, d + 1});
        }
    }
    (void)f2bits;
    return true;
}

void build_wide_layout(const rt_bvh_node *nodes, uint64_t n_nodes, WideLayout &out) {
    out.nodes.clear();
    out.stack_need = 0;
    if (n_nodes == 0) return;
    auto area = [&](uint32_t i) {
        const rt_bvh_node &n = nodes[i];
        const float dx = n.bbox_max[0] - n.bbox_min[0], dy = n.bbox_max[1] - n.bbox_min[1],
                    dz = n.bbox_max[2] - n.bbox_min[2];
        return dx * dy + dy * dz + dz * dx;
    };
    // Records in breadth-first order: rec_src[r] is the binary node whose subtree record r covers.
    std::vector<uint32_t> rec_src;
    std::vector<std::array<uint32_t, 4>> kids;  // binary node of each place (0xFFFFFFFF: empty)
    rec_src.push_back(0);
    for (size_t r = 0; r < rec_src.size(); ++r) {
        std::array<uint32_t, 4> k;
        k.fill(0xFFFFFFFFu);
        uint32_t cnt = 0;
        const rt_bvh_node &root = nodes[rec_src[r]];
        if (root.prim_count > 0) {  // a tree that is one leaf: one record holding that leaf
            k[cnt++] = rec_src[r];
        } else {
            k[cnt++] = root.left_first;
            k[cnt++] = root.right_child;
            while (cnt < 4u) {
                int best = -1;
                float best_a = -1.0f;
                for (uint32_t i = 0; i < cnt; ++i)
                    if (nodes[k[i]].prim_count == 0 && area(k[i]) > best_a) {
                        best = (int)i;
                        best_a = area(k[i]);
                    }
                if (best < 0) break;
                const rt_bvh_node &n = nodes[k[best]];
                for (uint32_t i = cnt; i > (uint32_t)best + 1u; --i) k[i] = k[i - 1];
                k[best] = n.left_first;
                k[best + 1] = n.right_child;
                ++cnt;
            }
        }
        kids.push_back(k);
        for (uint32_t i = 0; i < cnt; ++i)
            if (nodes[k[i]].prim_count == 0) rec_src.push_back(k[i]);
    }
    const size_t n_rec = rec_src.size();
    out.nodes.assign(n_rec * 32, 0.0f);
    std::vector<uint32_t> need(n_rec, 0);
    // Children get their record numbers in the order the breadth-first pass queued them.
    std::vector<uint32_t> first_child(n_rec, 0);
    uint32_t next = 1;
    for (size_t r = 0; r < n_rec; ++r) {
        first_child[r] = next;
        for (uint32_t i = 0; i < 4; ++i)
            if (kids[r][i] != 0xFFFFFFFFu && nodes[kids[r][i]].prim_count == 0) ++next;
    }
    for (size_t r = 0; r < n_rec; ++r) {
        float *q = &out.nodes[r * 32];
        uint32_t child_rec = first_child[r];
        for (uint32_t i = 0; i < 4; ++i) {
            float *c = q + 8 * i;
            const uint32_t b = kids[r][i];
            if (b == 0xFFFFFFFFu) {
                c[3] = bits2f(0u);
                c[7] = bits2f(0xFFFFFFFFu);
                continue;
            }
            const rt_bvh_node &n = nodes[b];
            for (int a = 0; a < 3; ++a) {
                c[a] = n.bbox_min[a];
                c[4 + a] = n.bbox_max[a];
            }
            if (n.prim_count > 0) {
                c[3] = bits2f(n.left_first);
                c[7] = bits2f(n.prim_count);
            } else {
                c[3] = bits2f(child_rec++);
                c[7] = bits2f(0u);
            }
        }
    }
    // Stack bound, children before parents (breadth-first numbers grow downwards).
    for (size_t r = n_rec; r-- > 0;) {
        uint32_t internal = 0, deepest = 0;
        const float *q = &out.nodes[r * 32];
        for (uint32_t i = 0; i < 4; ++i) {
            uint32_t cnt, ref;
            std::memcpy(&cnt, q + 8 * i + 7, 4);
            std::memcpy(&ref, q + 8 * i + 3, 4);
            if (cnt == 0u) {
                ++internal;
                deepest = std::max(deepest, need[ref]);
            }
        }
        need[r] = internal ? internal - 1u + deepest : 0u;
    }
    out.stack_need = need[0];
}

// ------------------------------------------------------------------------------------------------
// Deterministic host RNG for the procedural scenes (splitmix64; Irwin-Hall normal approximation).
// Only integer arithmetic and +,-,*,/ so both host architectures build identical scenes.
// ------------------------------------------------------------------------------------------------
struct HostRng {
    uint64_t s;
    explicit HostRng(uint64_t seed) : s(seed) {}
    uint64_t next() {
        uint64_t z = (s += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    }
    double uniform() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
    double normal() {
        double acc = 0.0;
        for (int i = 0; i < 12; ++i) acc += uniform();
        return acc - 6.0;
    }
};

}  // namespace rt

using namespace rt;

// ================================================================================================
// C ABI: errors, config defaults, camera, grid derivation
// ================================================================================================
extern "C" const char *rt_last_error(void) { return g_last_error.c_str(); }

extern "C" const char *rt_version(void) { return "rustracer-gb300 0.1.0 (sm_103a)"; }

extern "C" void rt_render_config_default(rt_render_config *c) {
    if (!c) return;
    std::memset(c, 0, sizeof(*c));
    c->width = 800;
    c->height = 600;
    c->photon_count = 1000000;
    c->spp = 1;
    c->exposure = 1.0f;
    c->gamma = 2.2f;
    for (int i = 0; i < 3; ++i) {
        c->light_emission[i] = 1.0f;
        c->point_light_emission[i] = 1.0f;
    }
    c->accumulate_frames = 0;
    c->enable_photon_map = 0;
    c->enable_denoise = 1;
    c->photon_debug = 0;
    c->debug_view = 0;
    c->photon_scale = 0.02f;
    c->photon_radius = 0.5f;
    c->ambient = 0.03f;
}

extern "C" void rt_camera_default(rt_camera *c) {
    if (!c) return;
    const float pos[3] = {0.0f, 0.0f, 5.0f};
    for (int i = 0; i < 3; ++i) {
        c->position[i] = pos[i];
        c->look_at[i] = 0.0f;
        c->up[i] = (i == 1) ? 1.0f : 0.0f;
    }
    c->fov_degrees = 60.0f;
    c->near_plane = 0.1f;
    c->aperture = 0.0f;
    c->focus_dist = 5.0f;
}

static inline Vec3 ld3(const float *p) { return Vec3{p[0], p[1], p[2]}; }
static inline void st3(float *p, Vec3 v) {
    p[0] = v.x;
    p[1] = v.y;
    p[2] = v.z;
}
// f32::to_radians is a multiply by PI/180 in f32; tan is taken in double and rounded once.
static inline float tan_half_fov(float fov_degrees) {
    const float rads_per_deg = 3.14159265358979323846f / 180.0f;
    float half = fov_degrees * rads_per_deg * 0.5f;
    return (float)std::tan((double)half);
}

extern "C" void rt_camera_to_uniform(const rt_camera *cam, uint32_t width, uint32_t height, rt_camera_uniform *out) {
    if (!cam || !out) return;
    std::memset(out, 0, sizeof(*out));
    Vec3 pos = ld3(cam->position);
    Vec3 forward = normalize(ld3(cam->look_at) - pos);
    Vec3 right = normalize(cross(forward, ld3(cam->up)));
    Vec3 up = cross(right, forward);
    float aspect = (float)width / (float)height;
    float fov_scale = tan_half_fov(cam->fov_degrees);
    st3(out->position, pos);
    st3(out->forward, forward);
    st3(out->right, right * aspect * fov_scale);
    st3(out->up, up * fov_scale);
    out->inv_half_res[0] = 2.0f / (float)width;
    out->inv_half_res[1] = 2.0f / (float)height;
    out->near_plane = cam->near_plane;
    out->fov_scale = fov_scale;
    out->aperture = cam->aperture;
    out->focus_dist = cam->focus_dist;
}

extern "C" int rt_camera_frame_scene(const rt_scene *s, rt_camera *out) {
    if (!s || !out) {
        set_error("rt_camera_frame_scene: null argument");
        return RT_ERR_INVALID_ARGUMENT;
    }
    rt_camera_default(out);
    // Scene::bounds over every mesh position (scene.rs:198-210).
    Vec3 mn{F32_MAX, F32_MAX, F32_MAX}, mx{-F32_MAX, -F32_MAX, -F32_MAX};
    for (const auto &m : s->meshes)
        for (const auto &p : m.positions) {
            mn = {std::fmin(mn.x, p.x), std::fmin(mn.y, p.y), std::fmin(mn.z, p.z)};
            mx = {std::fmax(mx.x, p.x), std::fmax(mx.y, p.y), std::fmax(mx.z, p.z)};
        }
    if (mn.x > mx.x) return RT_OK;
    Vec3 center = (mn + mx) * 0.5f;
    Vec3 d = mx - mn;
    float diag = std::fmax(std::sqrt(dot(d, d)), 1e-3f);
    float tan_half = tan_half_fov(70.0f);
    float dist = (diag * 0.5f / tan_half) * 1.3f;
    Vec3 dir = normalize(Vec3{0.55f, 0.35f, 0.75f});
    st3(out->position, center + dir * dist);
    st3(out->look_at, center);
    out->fov_degrees = 70.0f;
    return RT_OK;
}

// Rotation of v about the unit axis k by angle a (Rodrigues), in double precision.
static Vec3 rotate_axis(Vec3 v, Vec3 k, float angle) {
    double c = std::cos((double)angle), s = std::sin((double)angle);
    double vx = v.x, vy = v.y, vz = v.z, kx = k.x, ky = k.y, kz = k.z;
    double kdv = kx * vx + ky * vy + kz * vz;
    double cx = ky * vz - kz * vy, cy = kz * vx - kx * vz, cz = kx * vy - ky * vx;
    return Vec3{(float)(vx * c + cx * s + kx * kdv * (1.0 - c)), (float)(vy * c + cy * s + ky * kdv * (1.0 - c)),
                (float)(vz * c + cz * s + kz * kdv * (1.0 - c))};
}

extern "C" void rt_camera_orbit(rt_camera *cam, float delta_yaw, float delta_pitch) {
    if (!cam) return;
    Vec3 pos = ld3(cam->position), look = ld3(cam->look_at), up = ld3(cam->up);
    Vec3 forward = normalize(look - pos);
    Vec3 diff = look - pos;
    float dist = std::sqrt(dot(diff, diff));
    Vec3 new_forward = rotate_axis(forward, normalize(up), delta_yaw);
    Vec3 right = normalize(cross(new_forward, up));
    Vec3 final_forward = rotate_axis(new_forward, right, delta_pitch);
    st3(cam->position, look - final_forward * dist);
}

extern "C" void rt_camera_zoom(rt_camera *cam, float delta) {
    if (!cam) return;
    Vec3 pos = ld3(cam->position), look = ld3(cam->look_at);
    Vec3 forward = normalize(look - pos);
    Vec3 diff = look - pos;
    float dist = std::sqrt(dot(diff, diff));
    float new_dist = std::fmax(dist - delta, 0.01f);
    st3(cam->position, look - forward * new_dist);
}

extern "C" void rt_derive_grid(const float bounds_min[3], const float bounds_max[3], int has_bounds,
                               uint32_t grid_max_dim, uint32_t radius_mode, uint32_t photon_slots,
                               rt_grid_params *gp, float *photon_radius) {
    if (!gp) return;
    uint32_t G = grid_max_dim ? grid_max_dim : RT_GRID_MAX_DIM;
    if (G < 3) G = 3;
    Vec3 bmin{-1.05f, -1.05f, -1.05f}, bmax{1.05f, 1.05f, 1.05f};
    if (has_bounds && bounds_min && bounds_max) {
        bmin = ld3(bounds_min);
        bmax = ld3(bounds_max);
    }
    Vec3 ext = bmax - bmin;
    float max_ext = std::fmax(std::fmax(ext.x, std::fmax(ext.y, ext.z)), 1e-3f);
    float cell = max_ext / ((float)G - 2.0f);
    auto dim = [&](float e) -> uint32_t {
        float q = std::ceil(e / cell);
        uint32_t v = (q != q || q <= 0.0f) ? 0u : (q >= 4294967295.0f ? 0xFFFFFFFFu : (uint32_t)q);
        return std::min(std::max(v, 1u), G);
    };
    std::memset(gp, 0, sizeof(*gp));
    gp->grid_x = dim(ext.x);
    gp->grid_y = dim(ext.y);
    gp->grid_z = dim(ext.z);
    gp->num_cells = gp->grid_x * gp->grid_y * gp->grid_z;
    float half = cell * 0.5f;
    gp->room_min_x = bmin.x - half;
    gp->room_min_y = bmin.y - half;
    gp->room_min_z = bmin.z - half;
    gp->cell_size = cell;
    gp->photon_slots = photon_slots;
    if (photon_radius) {
        if (radius_mode == 1)
            *photon_radius = cell * 0.5f;
        else
            *photon_radius = std::fmin(std::fmax(cell * 4.0f, 0.01f), 2.0f);
    }
}

// ================================================================================================
// C ABI: scene model
// ================================================================================================
extern "C" int rt_scene_create(rt_scene **out) {
    if (!out) {
        set_error("rt_scene_create: null out");
        return RT_ERR_INVALID_ARGUMENT;
    }
    *out = new (std::nothrow) rt_scene();
    if (!*out) {
        set_error("rt_scene_create: out of host memory");
        return RT_ERR_OUT_OF_MEMORY;
    }
    return RT_OK;
}

extern "C" void rt_scene_destroy(rt_scene *s) { delete s; }

extern "C" int rt_scene_add_mesh(rt_scene *s, const float *positions, const float *normals, const float *uvs,
                                 uint64_t vertex_count, const uint32_t *indices, uint64_t index_count,
                                 uint32_t material_id) {
    return rt::guarded("rt_scene_add_mesh", [&]() -> int {
        if (!s || (vertex_count && !positions) || (index_count && !indices) || index_count % 3 != 0) {
            set_error("rt_scene_add_mesh: invalid arguments (index_count must be a multiple of 3)");
            return RT_ERR_INVALID_ARGUMENT;
        }
        Mesh m;
        m.positions.resize(vertex_count);
        for (uint64_t i = 0; i < vertex_count; ++i) m.positions[i] = ld3(positions + 3 * i);
        if (normals) {
            m.normals.resize(vertex_count);
            for (uint64_t i = 0; i < vertex_count; ++i) m.normals[i] = ld3(normals + 3 * i);
        }
        if (uvs) m.uvs.assign(uvs, uvs + 2 * vertex_count);
        m.indices.assign(indices, indices + index_count);
        for (uint32_t ix : m.indices)
            if (ix >= vertex_count) {
                set_error("rt_scene_add_mesh: index %u out of range (%llu vertices)", ix, (unsigned long long)vertex_count);
                return RT_ERR_INVALID_ARGUMENT;
            }
        m.material_id = material_id;
        s->meshes.push_back(std::move(m));
        s->finalized = false;
        return RT_OK;
    });
}

extern "C" int rt_scene_add_material(rt_scene *s, const rt_material *m) {
    return rt::guarded("rt_scene_add_material", [&]() -> int {
        if (!s || !m) {
            set_error("rt_scene_add_material: null argument");
            return RT_ERR_INVALID_ARGUMENT;
        }
        s->materials.push_back(*m);
        s->finalized = false;
        return RT_OK;
    });
}

extern "C" int rt_scene_add_light(rt_scene *s, const rt_light *l) {
    return rt::guarded("rt_scene_add_light", [&]() -> int {
        if (!s || !l) {
            set_error("rt_scene_add_light: null argument");
            return RT_ERR_INVALID_ARGUMENT;
        }
        s->lights.push_back(*l);
        s->finalized = false;
        return RT_OK;
    });
}

extern "C" int rt_scene_set_textures(rt_scene *s, int role, const uint8_t *rgba8, uint32_t width, uint32_t height,
                                     uint32_t layers) {
    return rt::guarded("rt_scene_set_textures", [&]() -> int {
        if (!s || role < 0 || role > 3 || (layers && (!rgba8 || !width || !height))) {
            set_error("rt_scene_set_textures: invalid arguments");
            return RT_ERR_INVALID_ARGUMENT;
        }
        Texture &t = s->tex[role];
        t.width = layers ? width : 0;
        t.height = layers ? height : 0;
        t.layers = layers;
        t.rgba8.assign(rgba8, rgba8 + (size_t)width * height * layers * 4 * (layers ? 1 : 0));
        return RT_OK;
    });
}

extern "C" int rt_scene_finalize(rt_scene *s) {
    return rt::guarded("rt_scene_finalize", [&]() -> int {
        if (!s) {
            set_error("rt_scene_finalize: null scene");
            return RT_ERR_INVALID_ARGUMENT;
        }
        if (s->finalized) return RT_OK;
        size_t ntri = 0;
        for (const auto &m : s->meshes) ntri += m.indices.size() / 3;
        if (ntri > 0xFFFFFFFFull) {
            set_error("rt_scene_finalize: too many triangles");
            return RT_ERR_INVALID_ARGUMENT;
        }
        s->triangles.clear();
        s->triangles.reserve(ntri);
        std::vector<Vec3> centroids, bmin, bmax;
        centroids.reserve(ntri);
        bmin.reserve(ntri);
        bmax.reserve(ntri);
        Vec3 mn{F32_MAX, F32_MAX, F32_MAX}, mx{-F32_MAX, -F32_MAX, -F32_MAX};
        for (const auto &m : s->meshes) {
            for (const auto &p : m.positions) {
                mn = {std::fmin(mn.x, p.x), std::fmin(mn.y, p.y), std::fmin(mn.z, p.z)};
                mx = {std::fmax(mx.x, p.x), std::fmax(mx.y, p.y), std::fmax(mx.z, p.z)};
            }
            size_t nv = m.positions.size();
            for (size_t t = 0; t + 2 < m.indices.size(); t += 3) {
                uint32_t ix[3] = {m.indices[t], m.indices[t + 1], m.indices[t + 2]};
                rt_triangle tri;
                std::memset(&tri, 0, sizeof(tri));
                float *vv[3] = {tri.v0, tri.v1, tri.v2};
                float *nn[3] = {tri.n0, tri.n1, tri.n2};
                float *uu[3] = {tri.uv0, tri.uv1, tri.uv2};
                Vec3 p[3];
                for (int k = 0; k < 3; ++k) {
                    p[k] = ix[k] < nv ? m.positions[ix[k]] : Vec3{0, 0, 0};
                    st3(vv[k], p[k]);
                    Vec3 n = ix[k] < m.normals.size() ? m.normals[ix[k]] : Vec3{0, 1, 0};
                    st3(nn[k], n);
                    if ((size_t)ix[k] * 2 + 1 < m.uvs.size()) {
                        uu[k][0] = m.uvs[2 * ix[k]];
                        uu[k][1] = m.uvs[2 * ix[k] + 1];
                    }
                }
                tri.material_id = m.tri_materials.empty() ? m.material_id : m.tri_materials[t / 3];
                s->triangles.push_back(tri);
                // Mesh::triangle_centroid / triangle_aabb (scene.rs:62-70)
                centroids.push_back((p[0] + p[1] + p[2]) / 3.0f);
                Vec3 lo{F32_MAX, F32_MAX, F32_MAX}, hi{-F32_MAX, -F32_MAX, -F32_MAX};
                for (int k = 0; k < 3; ++k) {
                    lo = {std::fmin(lo.x, p[k].x), std::fmin(lo.y, p[k].y), std::fmin(lo.z, p[k].z)};
                    hi = {std::fmax(hi.x, p[k].x), std::fmax(hi.y, p[k].y), std::fmax(hi.z, p[k].z)};
                }
                bmin.push_back(lo);
                bmax.push_back(hi);
            }
        }
        s->bvh_builder_used = RT_BVH_HOST_SAH;
        if (s->bvh_builder == RT_BVH_GPU_LBVH && ntri >= 2 && rt_device_count() > 0) {
            static_assert(sizeof(Vec3) == 12, "Vec3 arrays are read as packed floats");
            uint32_t depth = 0;
            rt::BVH b;
            // The traversal stack holds at most 63 pending nodes: deeper trees take the host build.
            if (rtd::build_lbvh(&centroids[0].x, &bmin[0].x, &bmax[0].x, (uint32_t)ntri, b, &depth) == 0 && depth <= 62) {
                s->bvh = std::move(b);
                s->bvh_builder_used = RT_BVH_GPU_LBVH;
            }
        }
        if (s->bvh_builder_used == RT_BVH_HOST_SAH) s->bvh = build_bvh(centroids, bmin, bmax);
        s->has_bounds = !(mn.x > mx.x);
        st3(s->bounds_min, s->has_bounds ? mn : Vec3{0, 0, 0});
        st3(s->bounds_max, s->has_bounds ? mx : Vec3{0, 0, 0});
        s->finalized = true;
        return RT_OK;
    });
}

extern "C" int rt_scene_describe(rt_scene *s, rt_scene_desc *d) {
    if (!s || !d) {
        set_error("rt_scene_describe: null argument");
        return RT_ERR_INVALID_ARGUMENT;
    }
    int st = rt_scene_finalize(s);
    if (st != RT_OK) return st;
    std::memset(d, 0, sizeof(*d));
    d->triangles = s->triangles.data();
    d->triangle_count = s->triangles.size();
    d->bvh_nodes = s->bvh.nodes.data();
    d->bvh_node_count = s->bvh.nodes.size();
    d->bvh_prims = s->bvh.prims.data();
    d->bvh_prim_count = s->bvh.prims.size();
    d->materials = s->materials.data();
    d->material_count = s->materials.size();
    d->lights = s->lights.data();
    d->light_count = s->lights.size();
    rt_texture_array *roles[4] = {&d->tex_albedo, &d->tex_mr, &d->tex_emissive, &d->tex_normal};
    for (int r = 0; r < 4; ++r) {
        const Texture &t = s->tex[r];
        roles[r]->rgba8 = t.layers ? t.rgba8.data() : nullptr;
        roles[r]->width = t.width;
        roles[r]->height = t.height;
        roles[r]->layers = t.layers;
    }
    for (int i = 0; i < 3; ++i) {
        d->bounds_min[i] = s->bounds_min[i];
        d->bounds_max[i] = s->bounds_max[i];
    }
    d->has_bounds = s->has_bounds ? 1u : 0u;
    return RT_OK;
}

extern "C" uint64_t rt_scene_triangle_count(const rt_scene *s) {
    if (!s) return 0;
    uint64_t n = 0;
    for (const auto &m : s->meshes) n += m.indices.size() / 3;
    return n;
}

// ================================================================================================
// C ABI: BVH build on raw primitive boxes (the reference's BVH tests drive the builder this way)
// ================================================================================================
extern "C" int rt_bvh_build(const float *centroids, const float *bbox_min, const float *bbox_max, uint64_t n,
                            rt_bvh **out) {
    return rt::guarded("rt_bvh_build", [&]() -> int {
        if (!out || (n && (!centroids || !bbox_min || !bbox_max)) || n > 0xFFFFFFFFull) {
            set_error("rt_bvh_build: invalid arguments");
            return RT_ERR_INVALID_ARGUMENT;
        }
        std::vector<Vec3> c(n), lo(n), hi(n);
        for (uint64_t i = 0; i < n; ++i) {
            c[i] = ld3(centroids + 3 * i);
            lo[i] = ld3(bbox_min + 3 * i);
            hi[i] = ld3(bbox_max + 3 * i);
        }
        std::unique_ptr<rt_bvh> b(new rt_bvh());
        b->b = build_bvh(c, lo, hi);
        *out = b.release();
        return RT_OK;
    });
}
extern "C" int rt_bvh_wide_layout(const rt_bvh_node *nodes, uint64_t n_nodes, float *out, uint64_t capacity,
                                  uint64_t *records, uint32_t *stack_need) {
    return rt::guarded("rt_bvh_wide_layout", [&]() -> int {
        rt::clear_error();
        if ((!nodes && n_nodes) || !records || !stack_need) {
            rt::set_error("rt_bvh_wide_layout: null argument");
            return RT_ERR_INVALID_ARGUMENT;
        }
        rt::WideLayout w;
        rt::build_wide_layout(nodes, n_nodes, w);
        *records = w.nodes.size() / 32;
        *stack_need = w.stack_need;
        if (out) std::memcpy(out, w.nodes.data(), sizeof(float) * std::min<uint64_t>(capacity, w.nodes.size()));
        return RT_OK;
    });
}

extern "C" const rt_bvh_node *rt_bvh_nodes(const rt_bvh *b, uint64_t *count) {
    if (count) *count = b ? b->b.nodes.size() : 0;
    return b ? b->b.nodes.data() : nullptr;
}
extern "C" const uint32_t *rt_bvh_prims(const rt_bvh *b, uint64_t *count) {
    if (count) *count = b ? b->b.prims.size() : 0;
    return b ? b->b.prims.data() : nullptr;
}
extern "C" void rt_bvh_destroy(rt_bvh *b) { delete b; }

// ================================================================================================
// Procedural scenes
// ================================================================================================
static rt_material mat_lambertian(float r, float g, float b) {  // Material::lambertian (material.rs:101-108)
    rt_material m;
    std::memset(&m, 0, sizeof(m));
    m.albedo[0] = r; m.albedo[1] = g; m.albedo[2] = b; m.albedo[3] = 1.0f;
    m.roughness = 1.0f;
    m.metallic = 0.0f;
    m.ior = 1.5f;
    m.kind = RT_MAT_LAMBERTIAN;
    m.tex_albedo = m.tex_mr = m.tex_emissive = m.tex_normal = RT_TEX_NONE;
    return m;
}
static rt_material mat_metal(float r, float g, float b, float rough) {  // Material::metal (:111-119)
    rt_material m = mat_lambertian(r, g, b);
    m.kind = RT_MAT_METAL;
    m.roughness = std::fmin(std::fmax(rough, 0.001f), 1.0f);
    m.metallic = 1.0f;
    return m;
}
static rt_material mat_dielectric(float ior, float r, float g, float b) {  // Material::dielectric (:122-130)
    rt_material m = mat_lambertian(r, g, b);
    m.kind = RT_MAT_DIELECTRIC;
    m.roughness = 0.0f;
    m.ior = ior;
    return m;
}
static rt_material mat_emissive(float r, float g, float b, float intensity) {  // Material::emissive (:133-140)
    rt_material m = mat_lambertian(r, g, b);  // albedo = colour (quirk kept)
    m.kind = RT_MAT_EMISSIVE;
    m.roughness = 0.5f;  // Material::default roughness
    m.emissive[0] = r * intensity;
    m.emissive[1] = g * intensity;
    m.emissive[2] = b * intensity;
    return m;
}
static rt_light light_area(uint32_t tri, float r, float g, float b, float intensity) {  // lib.rs:1257-1268
    rt_light l;
    std::memset(&l, 0, sizeof(l));
    l.data[0] = (float)tri;
    l.color[0] = r; l.color[1] = g; l.color[2] = b;
    l.intensity = intensity;
    l.kind = RT_LIGHT_AREA;
    return l;
}
static rt_light light_point(Vec3 p, float r, float g, float b, float intensity) {  // lib.rs:1233-1244
    rt_light l;
    std::memset(&l, 0, sizeof(l));
    st3(l.data, p);
    l.color[0] = r; l.color[1] = g; l.color[2] = b;
    l.intensity = intensity;
    l.kind = RT_LIGHT_POINT;
    return l;
}

// create_quad (scene.rs:463-480): 4 vertices, shared flat normal, unit-square uvs, (0,1,2),(0,2,3).
static void add_quad(rt_scene *s, Vec3 a, Vec3 b, Vec3 c, Vec3 d, uint32_t mat) {
    Mesh m;
    m.positions = {a, b, c, d};
    Vec3 n = normalize(cross(b - a, c - a));
    m.normals = {n, n, n, n};
    m.uvs = {0, 0, 1, 0, 1, 1, 0, 1};
    m.indices = {0, 1, 2, 0, 2, 3};
    m.material_id = mat;
    s->meshes.push_back(std::move(m));
}

// create_cube (scene.rs:483-505) on a box given by its 8 (already transformed) corners
// c[ix + 2*iy + 4*iz], ix/iy/iz in {0 = lo, 1 = hi}.
static void add_box(rt_scene *s, const Vec3 c[8], uint32_t mat) {
    auto C = [&](int x, int y, int z) { return c[x + 2 * y + 4 * z]; };
    add_quad(s, C(0, 0, 0), C(0, 1, 0), C(0, 1, 1), C(0, 0, 1), mat);  // -X
    add_quad(s, C(1, 0, 1), C(1, 1, 1), C(1, 1, 0), C(1, 0, 0), mat);  // +X
    add_quad(s, C(0, 0, 1), C(1, 0, 1), C(1, 0, 0), C(0, 0, 0), mat);  // -Y
    add_quad(s, C(0, 1, 0), C(1, 1, 0), C(1, 1, 1), C(0, 1, 1), mat);  // +Y
    add_quad(s, C(1, 0, 0), C(1, 1, 0), C(0, 1, 0), C(0, 0, 0), mat);  // -Z
    add_quad(s, C(0, 0, 1), C(0, 1, 1), C(1, 1, 1), C(1, 0, 1), mat);  // +Z
}

// Box [0,sx]x[0,sy]x[0,sz] rotated about +Y by `deg` degrees, then translated by t.
static void add_rotated_box(rt_scene *s, float sx, float sy, float sz, double deg, Vec3 t, uint32_t mat) {
    const double rad = deg * 3.14159265358979323846 / 180.0;
    const double cs = std::cos(rad), sn = std::sin(rad);
    Vec3 c[8];
    for (int i = 0; i < 8; ++i) {
        double x = (i & 1) ? sx : 0.0, y = (i & 2) ? sy : 0.0, z = (i & 4) ? sz : 0.0;
        double rx = cs * x + sn * z, rz = -sn * x + cs * z;
        c[i] = Vec3{(float)(rx + t.x), (float)(y + t.y), (float)(rz + t.z)};
    }
    add_box(s, c, mat);
}

// Creates a scene and fills it; a fill that fails (or throws) leaves *out null and nothing allocated.
template <class F>
static int generate_scene(const char *fn, rt_scene **out, F &&fill) {
    int st = rt_scene_create(out);
    if (st != RT_OK) return st;
    st = rt::guarded(fn, [&]() -> int { return fill(*out); });
    if (st != RT_OK) {
        rt_scene_destroy(*out);
        *out = nullptr;
    }
    return st;
}

static int fill_cornell555(rt_scene *s);

extern "C" int rt_scene_create_cornell555(rt_scene **out) {
    return generate_scene("rt_scene_create_cornell555", out, fill_cornell555);
}

static int fill_cornell555(rt_scene *s) {
    s->materials.push_back(mat_lambertian(0.73f, 0.73f, 0.73f));      // 0 white
    s->materials.push_back(mat_lambertian(0.65f, 0.05f, 0.05f));      // 1 red
    s->materials.push_back(mat_lambertian(0.12f, 0.45f, 0.15f));      // 2 green
    s->materials.push_back(mat_emissive(15.0f, 15.0f, 15.0f, 1.0f));  // 3 light
    const float L = 555.0f;
    // Walls face the interior.  Camera looks down +z from z < 0, so +x is image-left.
    add_quad(s, v3(0, 0, 0), v3(0, 0, L), v3(L, 0, L), v3(L, 0, 0), 0);  // floor   (y = 0,   +y)
    add_quad(s, v3(0, L, 0), v3(L, L, 0), v3(L, L, L), v3(0, L, L), 0);  // ceiling (y = 555, -y)
    add_quad(s, v3(0, 0, L), v3(0, L, L), v3(L, L, L), v3(L, 0, L), 0);  // back    (z = 555, -z)
    add_quad(s, v3(L, 0, 0), v3(L, 0, L), v3(L, L, L), v3(L, L, 0), 1);  // left    (x = 555, red, -x)
    add_quad(s, v3(0, 0, 0), v3(0, L, 0), v3(0, L, L), v3(0, 0, L), 2);  // right   (x = 0, green, +x)
    // 130 x 105 ceiling light at y = 554 facing down: triangles 10 and 11.
    add_quad(s, v3(213, 554, 227), v3(343, 554, 227), v3(343, 554, 332), v3(213, 554, 332), 3);
    add_rotated_box(s, 165.0f, 165.0f, 165.0f, -18.0, v3(130, 0, 65), 0);   // short box
    add_rotated_box(s, 165.0f, 330.0f, 165.0f, 15.0, v3(265, 0, 295), 0);   // tall box
    s->lights.push_back(light_area(10, 15.0f, 15.0f, 15.0f, 1.0f));
    s->lights.push_back(light_area(11, 15.0f, 15.0f, 15.0f, 1.0f));
    // The classic Cornell camera: 800 units in front of the open side, 40 degree field of view.
    rt_camera_default(&s->camera);
    st3(s->camera.position, v3(278.0f, 278.0f, -800.0f));
    st3(s->camera.look_at, v3(278.0f, 278.0f, 0.0f));
    s->camera.fov_degrees = 40.0f;
    s->camera.focus_dist = 800.0f;
    s->has_camera = true;
    return rt_scene_finalize(s);
}

// Value noise in [0,1]: a (cells x cells) lattice of seeded values, smoothstep-interpolated,
// periodic over the texture so the repeat sampler sees no seam; two octaves.
static void value_noise(std::vector<float> &out, uint32_t size, uint32_t cells, HostRng &rng) {
    std::vector<float> lat1((size_t)cells * cells), lat2((size_t)cells * 2 * cells * 2);
    for (auto &v : lat1) v = (float)rng.uniform();
    for (auto &v : lat2) v = (float)rng.uniform();
    out.assign((size_t)size * size, 0.0f);
    auto sample = [&](const std::vector<float> &lat, uint32_t n, float fx, float fy) {
        float x = fx * (float)n, y = fy * (float)n;
        uint32_t x0 = (uint32_t)x, y0 = (uint32_t)y;
        float tx = x - (float)x0, ty = y - (float)y0;
        tx = tx * tx * (3.0f - 2.0f * tx);
        ty = ty * ty * (3.0f - 2.0f * ty);
        uint32_t x1 = (x0 + 1) % n, y1 = (y0 + 1) % n;
        x0 %= n;
        y0 %= n;
        float a = lat[(size_t)y0 * n + x0], b = lat[(size_t)y0 * n + x1];
        float c = lat[(size_t)y1 * n + x0], d = lat[(size_t)y1 * n + x1];
        float top = a + (b - a) * tx, bot = c + (d - c) * tx;
        return top + (bot - top) * ty;
    };
    for (uint32_t y = 0; y < size; ++y)
        for (uint32_t x = 0; x < size; ++x) {
            float fx = ((float)x + 0.5f) / (float)size, fy = ((float)y + 0.5f) / (float)size;
            out[(size_t)y * size + x] = 0.65f * sample(lat1, cells, fx, fy) + 0.35f * sample(lat2, cells * 2, fx, fy);
        }
}

// create_role_array's quantisation (lib.rs:1315-1326): (clamp(c, 0, 1) * 255) as u8, truncating.
static inline uint8_t quant(float c) { return (uint8_t)(std::fmin(std::fmax(c, 0.0f), 1.0f) * 255.0f); }

static int fill_icosphere_room(rt_scene *s, uint32_t level, uint64_t seed, float sigma, uint32_t tex_size);

extern "C" int rt_scene_create_icosphere_room(uint32_t level, uint64_t seed, float sigma, uint32_t tex_size,
                                              rt_scene **out) {
    if (level > 10 || tex_size > 8192) {
        set_error("rt_scene_create_icosphere_room: level must be <= 10 and tex_size <= 8192");
        return RT_ERR_INVALID_ARGUMENT;
    }
    return generate_scene("rt_scene_create_icosphere_room", out,
                          [&](rt_scene *s) { return fill_icosphere_room(s, level, seed, sigma, tex_size); });
}

static int fill_icosphere_room(rt_scene *s, uint32_t level, uint64_t seed, float sigma, uint32_t tex_size) {
    HostRng rng(seed * 0x2545F4914F6CDD1Dull + 0x1234567ull);

    // --- icosahedron, subdivided `level` times, projected to the unit sphere -------------------
    const float phi = 1.6180339887498949f;
    std::vector<Vec3> verts = {{-1, phi, 0}, {1, phi, 0}, {-1, -phi, 0}, {1, -phi, 0}, {0, -1, phi}, {0, 1, phi},
                               {0, -1, -phi}, {0, 1, -phi}, {phi, 0, -1}, {phi, 0, 1}, {-phi, 0, -1}, {-phi, 0, 1}};
    for (auto &v : verts) v = normalize(v);
    std::vector<uint32_t> faces = {0, 11, 5, 0, 5,  1,  0,  1, 7, 0, 7,  10, 0, 10, 11, 1, 5, 9, 5, 11,
                                   4, 11, 10, 2, 10, 7, 6,  7, 1, 8, 3,  9,  4, 3,  4,  2, 3, 2, 6, 3,
                                   6, 8,  3,  8, 9,  4, 9,  5, 2, 4, 11, 6,  2, 10, 8,  6, 7, 9, 8, 1};
    // Orient every face outward.
    for (size_t f = 0; f < faces.size(); f += 3) {
        Vec3 a = verts[faces[f]], b = verts[faces[f + 1]], c = verts[faces[f + 2]];
        if (dot(cross(b - a, c - a), a + b + c) < 0.0f) std::swap(faces[f + 1], faces[f + 2]);
    }
    for (uint32_t l = 0; l < level; ++l) {
        std::unordered_map<uint64_t, uint32_t> mid;
        mid.reserve(faces.size() * 2);
        auto midpoint = [&](uint32_t a, uint32_t b) {
            uint64_t key = a < b ? ((uint64_t)a << 32 | b) : ((uint64_t)b << 32 | a);
            auto it = mid.find(key);
            if (it != mid.end()) return it->second;
            uint32_t idx = (uint32_t)verts.size();
            verts.push_back(normalize((verts[a] + verts[b]) * 0.5f));
            mid.emplace(key, idx);
            return idx;
        };
        std::vector<uint32_t> nf;
        nf.reserve(faces.size() * 4);
        for (size_t f = 0; f < faces.size(); f += 3) {
            uint32_t a = faces[f], b = faces[f + 1], c = faces[f + 2];
            uint32_t ab = midpoint(a, b), bc = midpoint(b, c), ca = midpoint(c, a);
            uint32_t tri[12] = {a, ab, ca, b, bc, ab, c, ca, bc, ab, bc, ca};
            nf.insert(nf.end(), tri, tri + 12);
        }
        faces.swap(nf);
    }
    // Per-vertex displacement along the normal, N(0, sigma) (Irwin-Hall).
    for (auto &v : verts) v = v * (1.0f + sigma * (float)rng.normal());
    // Smooth normals: area-weighted face normals.
    std::vector<Vec3> normals(verts.size(), Vec3{0, 0, 0});
    for (size_t f = 0; f < faces.size(); f += 3) {
        Vec3 a = verts[faces[f]], b = verts[faces[f + 1]], c = verts[faces[f + 2]];
        Vec3 n = cross(b - a, c - a);
        for (int k = 0; k < 3; ++k) normals[faces[f + k]] = normals[faces[f + k]] + n;
    }
    for (auto &n : normals) n = normalize(n);
    // Planar uv projection, tiled twice.
    std::vector<float> uvs(verts.size() * 2);
    for (size_t i = 0; i < verts.size(); ++i) {
        uvs[2 * i] = (verts[i].x + 1.0f) * 1.0f;
        uvs[2 * i + 1] = (verts[i].y + 1.0f) * 1.0f;
    }

    // --- materials ---------------------------------------------------------------------------------
    s->materials.push_back(mat_lambertian(0.73f, 0.73f, 0.73f));      // 0: room
    s->materials.push_back(mat_emissive(20.0f, 20.0f, 20.0f, 1.0f));  // 1: area light
    const uint32_t tex_layer = tex_size ? 0u : RT_TEX_NONE;
    size_t nfaces = faces.size() / 3;
    for (size_t f = 0; f < nfaces; ++f) {
        double u = rng.uniform();
        rt_material m;
        if (u < 0.60) {
            // one declaration per draw: the order of the draws must not depend on the compiler's
            // order of evaluating call arguments
            const float r = (float)(0.2 + 0.6 * rng.uniform());
            const float g = (float)(0.2 + 0.6 * rng.uniform());
            const float b = (float)(0.2 + 0.6 * rng.uniform());
            m = mat_lambertian(r, g, b);
        } else if (u < 0.85) {
            float r = (float)(0.5 + 0.45 * rng.uniform()), g = (float)(0.5 + 0.45 * rng.uniform()),
                  b = (float)(0.5 + 0.45 * rng.uniform());
            m = mat_metal(r, g, b, (float)(0.05 + 0.55 * rng.uniform()));
        } else {
            m = mat_dielectric(1.5f, 1.0f, 1.0f, 1.0f);
        }
        if (m.kind != RT_MAT_DIELECTRIC) {
            m.tex_albedo = tex_layer;
            m.tex_mr = tex_layer;
        }
        m.tex_normal = tex_layer;
        s->materials.push_back(m);
    }

    // --- geometry: room (12), light (2), sphere -----------------------------------------------------
    const float R = 5.0f;
    add_quad(s, v3(-R, -R, -R), v3(-R, -R, R), v3(R, -R, R), v3(R, -R, -R), 0);  // floor  +y
    add_quad(s, v3(-R, R, -R), v3(R, R, -R), v3(R, R, R), v3(-R, R, R), 0);      // ceil   -y
    add_quad(s, v3(-R, -R, -R), v3(R, -R, -R), v3(R, R, -R), v3(-R, R, -R), 0);  // back   +z
    add_quad(s, v3(-R, -R, R), v3(-R, R, R), v3(R, R, R), v3(R, -R, R), 0);      // front  -z
    add_quad(s, v3(-R, -R, -R), v3(-R, R, -R), v3(-R, R, R), v3(-R, -R, R), 0);  // left   +x
    add_quad(s, v3(R, -R, -R), v3(R, -R, R), v3(R, R, R), v3(R, R, -R), 0);      // right  -x
    const float ly = R - 0.01f;
    add_quad(s, v3(-0.5f, ly, -0.5f), v3(0.5f, ly, -0.5f), v3(0.5f, ly, 0.5f), v3(-0.5f, ly, 0.5f), 1);  // tris 12,13
    // The sphere is one mesh with per-triangle materials: triangle k uses material 2 + k.
    {
        Mesh m;
        m.positions = verts;
        m.normals = normals;
        m.uvs = uvs;
        m.indices = faces;
        m.material_id = 2;
        m.tri_materials.resize(nfaces);
        for (size_t k = 0; k < nfaces; ++k) m.tri_materials[k] = (uint32_t)(2 + k);
        s->meshes.push_back(std::move(m));
    }
    s->lights.push_back(light_area(12, 20.0f, 20.0f, 20.0f, 1.0f));
    s->lights.push_back(light_area(13, 20.0f, 20.0f, 20.0f, 1.0f));
    for (int i = 0; i < 4; ++i) {
        Vec3 p{(float)(-4.0 + 8.0 * rng.uniform()), (float)(1.5 + 3.0 * rng.uniform()),
               (float)(-4.0 + 8.0 * rng.uniform())};
        s->lights.push_back(light_point(p, 1.0f, 0.95f, 0.9f, 8.0f));
    }

    // --- textures --------------------------------------------------------------------------------
    if (tex_size) {
        size_t texels = (size_t)tex_size * tex_size;
        std::vector<float> n0, n1, n2;
        value_noise(n0, tex_size, 16, rng);
        value_noise(n1, tex_size, 16, rng);
        value_noise(n2, tex_size, 32, rng);
        std::vector<uint8_t> alb(texels * 4), mr(texels * 4), nrm(texels * 4);
        for (size_t i = 0; i < texels; ++i) {
            alb[4 * i + 0] = quant(0.35f + 0.65f * n0[i]);
            alb[4 * i + 1] = quant(0.35f + 0.65f * n1[i]);
            alb[4 * i + 2] = quant(0.35f + 0.65f * n2[i]);
            alb[4 * i + 3] = 255;
            mr[4 * i + 0] = 255;
            mr[4 * i + 1] = quant(0.5f + 0.5f * n1[i]);
            mr[4 * i + 2] = 255;
            mr[4 * i + 3] = 255;
            float nx = (n0[i] - 0.5f) * 0.6f, ny = (n2[i] - 0.5f) * 0.6f;
            float nz = std::sqrt(std::fmax(1.0f - nx * nx - ny * ny, 0.0f));
            nrm[4 * i + 0] = quant(0.5f + 0.5f * nx);
            nrm[4 * i + 1] = quant(0.5f + 0.5f * ny);
            nrm[4 * i + 2] = quant(0.5f + 0.5f * nz);
            nrm[4 * i + 3] = 255;
        }
        rt_scene_set_textures(s, RT_TEX_ALBEDO, alb.data(), tex_size, tex_size, 1);
        rt_scene_set_textures(s, RT_TEX_MR, mr.data(), tex_size, tex_size, 1);
        rt_scene_set_textures(s, RT_TEX_NORMAL, nrm.data(), tex_size, tex_size, 1);
    }
    rt_camera_default(&s->camera);
    st3(s->camera.position, v3(1.2f, 0.8f, 2.4f));
    st3(s->camera.look_at, v3(0.0f, 0.0f, 0.0f));
    s->camera.fov_degrees = 60.0f;
    s->has_camera = true;
    return rt_scene_finalize(s);
}

extern "C" int rt_scene_default_camera(const rt_scene *s, rt_camera *out) {
    if (!s || !out) {
        set_error("rt_scene_default_camera: null argument");
        return RT_ERR_INVALID_ARGUMENT;
    }
    if (s->has_camera) {
        *out = s->camera;
        return RT_OK;
    }
    return rt_camera_frame_scene(s, out);
}

// PNG scanline unfiltering (PNG specification, section 9: filter types None, Sub, Up, Average,
// Paeth), for the glTF image decoder: `rows` holds h rows of 1 + stride bytes (filter byte first),
// `out` receives h * stride bytes.  bpp = bytes per complete pixel (at least 1).
extern "C" int rt_png_unfilter(const uint8_t *rows, uint32_t h, uint32_t stride, uint32_t bpp, uint8_t *out) {
    rt::clear_error();
    if ((!rows || !out) && h && stride) {
        rt::set_error("rt_png_unfilter: null buffer");
        return RT_ERR_INVALID_ARGUMENT;
    }
    if (bpp == 0) bpp = 1;
    for (uint32_t y = 0; y < h; ++y) {
        const uint8_t f = rows[(size_t)y * (stride + 1)];
        const uint8_t *in = rows + (size_t)y * (stride + 1) + 1;
        uint8_t *o = out + (size_t)y * stride;
        const uint8_t *up = y ? out + (size_t)(y - 1) * stride : nullptr;
        for (uint32_t x = 0; x < stride; ++x) {
            const int a = x >= bpp ? o[x - bpp] : 0;
            const int b = up ? up[x] : 0;
            const int c = (up && x >= bpp) ? up[x - bpp] : 0;
            int pred = 0;
            switch (f) {
                case 0: pred = 0; break;
                case 1: pred = a; break;
                case 2: pred = b; break;
                case 3: pred = (a + b) >> 1; break;
                case 4: {
                    const int p = a + b - c;
                    const int pa = p > a ? p - a : a - p, pb = p > b ? p - b : b - p, pc = p > c ? p - c : c - p;
                    pred = (pa <= pb && pa <= pc) ? a : (pb <= pc ? b : c);
                    break;
                }
                default:
                    rt::set_error("rt_png_unfilter: unknown filter type %u in row %u", (unsigned)f, y);
                    return RT_ERR_INVALID_ARGUMENT;
            }
            o[x] = (uint8_t)((in[x] + pred) & 0xFF);
        }
    }
    return RT_OK;
}

extern "C" void rt_set_host_threads(uint32_t n) { g_host_threads.store(n); }

namespace {
std::atomic<uint32_t> g_traversal_width{4u};
}
uint32_t rt::traversal_width() { return g_traversal_width.load(); }

extern "C" int rt_set_traversal_width(uint32_t width) {
    rt::clear_error();
    if (width != 2u && width != 4u) {
        rt::set_error("rt_set_traversal_width: width must be 2 or 4, got %u", width);
        return RT_ERR_INVALID_ARGUMENT;
    }
    g_traversal_width.store(width);
    return RT_OK;
}
extern "C" uint32_t rt_get_traversal_width(void) { return g_traversal_width.load(); }

extern "C" int rt_scene_set_bvh_builder(rt_scene *s, uint32_t builder) {
    if (!s || builder > RT_BVH_GPU_LBVH) {
        set_error("rt_scene_set_bvh_builder: need a scene and RT_BVH_HOST_SAH or RT_BVH_GPU_LBVH");
        return RT_ERR_INVALID_ARGUMENT;
    }
    if (s->finalized && s->bvh_builder != builder) s->finalized = false;  // rebuilt at the next describe
    s->bvh_builder = builder;
    return RT_OK;
}

extern "C" uint32_t rt_scene_bvh_builder_used(const rt_scene *s) { return s ? s->bvh_builder_used : 0u; }

extern "C" int rt_bvh_build_gpu(const float *centroids, const float *bbox_min, const float *bbox_max, uint64_t n,
                                rt_bvh **out, uint32_t *max_depth) {
    return rt::guarded("rt_bvh_build_gpu", [&]() -> int {
        rt::clear_error();
        if (!out || n < 2 || n > 0x7FFFFFFFull || !centroids || !bbox_min || !bbox_max) {
            set_error("rt_bvh_build_gpu: need 2 .. 2^31 - 1 primitives and their centroids and boxes");
            return RT_ERR_INVALID_ARGUMENT;
        }
        std::unique_ptr<rt_bvh> b(new rt_bvh());
        if (rtd::build_lbvh(centroids, bbox_min, bbox_max, (uint32_t)n, b->b, max_depth) != 0) {
            set_error("rt_bvh_build_gpu: a CUDA call failed");
            return RT_ERR_CUDA;
        }
        *out = b.release();
        return RT_OK;
    });
}
