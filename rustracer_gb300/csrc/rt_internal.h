// Internal host-side helpers shared by the translation units of librustracer_cuda.
#pragma once
#include <cstdarg>
#include <cstdint>
#include <cstdio>
#include <exception>
#include <new>
#include <string>
#include <vector>

#include "../../include/rustracer_cuda.h"
#include "rt_layout_check.h"

namespace rt {

// Thread-local error message returned by rt_last_error().
void set_error(const char *fmt, ...)
#if defined(__GNUC__)
    __attribute__((format(printf, 1, 2)))
#endif
    ;
void clear_error();

// Runs the body of a C entry point so that no C++ exception crosses the C ABI: an allocation
// failure becomes RT_ERR_OUT_OF_MEMORY, any other exception RT_ERR_STATE, each with a message.
template <class F>
int guarded(const char *fn, F &&body) {
    try {
        return body();
    } catch (const std::bad_alloc &) {
        set_error("%s: out of host memory", fn);
        return RT_ERR_OUT_OF_MEMORY;
    } catch (const std::exception &e) {
        set_error("%s: %s", fn, e.what());
        return RT_ERR_STATE;
    }
}

struct Vec3 {
    float x, y, z;
};
inline Vec3 v3(float x, float y, float z) { return Vec3{x, y, z}; }
inline Vec3 operator+(Vec3 a, Vec3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline Vec3 operator-(Vec3 a, Vec3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline Vec3 operator*(Vec3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
inline Vec3 operator/(Vec3 a, float s) { return {a.x / s, a.y / s, a.z / s}; }
inline float dot(Vec3 a, Vec3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline Vec3 cross(Vec3 a, Vec3 b) { return {a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y}; }
Vec3 normalize(Vec3 a);  // a * (1 / |a|), glam's Vec3::normalize

struct Mesh {
    std::vector<Vec3> positions, normals;
    std::vector<float> uvs;  // 2 per vertex
    std::vector<uint32_t> indices;
    uint32_t material_id = 0;
    // Optional per-triangle material ids (overrides material_id when non-empty).
    std::vector<uint32_t> tri_materials;
};

struct Texture {
    uint32_t width = 0, height = 0, layers = 0;
    std::vector<uint8_t> rgba8;
};

struct BVH {
    std::vector<rt_bvh_node> nodes;
    std::vector<uint32_t> prims;
};

// BVHBuilder::build (rustracer-core/src/bvh.rs:135-336).
BVH build_bvh(const std::vector<Vec3> &centroids, const std::vector<Vec3> &bmin, const std::vector<Vec3> &bmax);

// The traversal layout of the device kernels, derived from the reference's arrays (same tree):
// 16 floats per internal node (both children's boxes, refs and leaf counts) and 12 floats per prim
// slot ((v0, original index), v1 - v0, v2 - v0).  A tree that is a single leaf gets one record whose
// two children are that leaf.  Returns false (with the error set) on an inconsistent input.
struct TraversalLayout {
    std::vector<float> cnodes;   // 16 per record
    std::vector<float> tri_ord;  // 12 per prim slot
    uint32_t max_depth = 0;      // root-to-leaf edges of the deepest leaf
};
bool build_traversal_layout(const rt_bvh_node *nodes, uint64_t n_nodes, const uint32_t *prims, uint64_t n_prims,
                            const rt_triangle *tris, uint64_t n_tris, TraversalLayout &out);

// The same tree with every record holding up to four children: each record of the two-wide layout
// absorbs the children of its largest (surface area) internal child until it has four (leaves stay
// the reference's leaves, with the same prim slots).  32 floats per record: per child (min, ref) and
// (max, count), count > 0 a leaf of `count` prim slots from `ref`, count 0 an internal child whose
// record is `ref`, count 0xFFFFFFFF an empty place.  `stack_need` bounds the entries a near-first
// walk holds at once (the internal children of a record minus one, summed along a root-to-leaf path).
struct WideLayout {
    std::vector<float> nodes;  // 32 per record
    uint32_t stack_need = 0;
};
void build_wide_layout(const rt_bvh_node *nodes, uint64_t n_nodes, WideLayout &out);
// rt_set_traversal_width: 4 (the default) or 2; read when a scene is uploaded.
uint32_t traversal_width();

}  // namespace rt

struct rt_scene {
    std::vector<rt::Mesh> meshes;
    std::vector<rt_material> materials;
    std::vector<rt_light> lights;
    rt::Texture tex[4];
    // BVH builder of rt_scene_finalize: RT_BVH_HOST_SAH or RT_BVH_GPU_LBVH (and the one used).
    uint32_t bvh_builder = 0, bvh_builder_used = 0;
    // Flattened state (rt_scene_finalize).
    bool finalized = false;
    std::vector<rt_triangle> triangles;
    rt::BVH bvh;
    float bounds_min[3] = {0, 0, 0}, bounds_max[3] = {0, 0, 0};
    bool has_bounds = false;
    // Preferred camera of a procedural scene (rt_scene_default_camera).
    bool has_camera = false;
    rt_camera camera{};
};

struct rt_bvh {
    rt::BVH b;
};

namespace rtd {
// Linear BVH of n >= 2 primitives built on the GPU (k_bvh.cu), in the reference's node layout; 0 on
// success (with the tree's depth), < 0 when n < 2 or a CUDA call failed.
int build_lbvh(const float *centroids, const float *bmin, const float *bmax, uint32_t n, rt::BVH &out,
               uint32_t *max_depth);
}  // namespace rtd
