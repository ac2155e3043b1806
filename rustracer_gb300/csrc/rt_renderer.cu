// The renderer behind the C ABI: device-resident scene and frame buffers, one CUDA stream, and the
// frame schedule of rustracer-renderer's Renderer (rustracer-renderer/src/lib.rs:227-1042).
//
// HBM layout per renderer (allocated at create from the device's renderer pool in the renderer's
// stream order, freed at destroy without synchronising the device; the path state and the job table
// come with the first solo frame):
//   scene:  triangles 128 B, materials 64 B, lights 64 B (AoS, the reference layouts); role textures
//           as rgba8 arrays (layer-major); the traversal layout derived from the reference's BVH:
//           one 64 B record per internal node, one 48 B leaf-ordered triangle record per prim slot.
//   path:   per pixel, origin / direction / throughput (16 B each), hit 8 B, accumulators 64 B,
//           first normal 16 B, two queue entries 4 B, one deferred shadow ray 48 B, one photon-lookup
//           request 48 B (240 B / pixel).
//   frame:  frame, denoise ping-pong, moments, gbuffer, accumulation (float4 per pixel each) and the
//           rgba8 output image.
//   photon: photon slots (64 B, 6 per photon), u32 key per slot, slot order, sorted photons (64 B),
//           counts / cursor / (start, count) per cell, scan partials.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <new>
#include <vector>

#include "rt_renderer_impl.h"

using rt::DevBuf;
using rt::set_error;
using namespace rt;  // EV_* event slots

namespace {

void resolve_env(rt_renderer *r) {
    rtd::DevScene &s = r->scene;
    s.env_intensity = 0.0f;
    const float zen[3] = {0.55f, 0.6f, 0.75f}, hor[3] = {0.95f, 0.93f, 0.9f};
    for (int i = 0; i < 3; ++i) {
        s.env_color[i] = zen[i];
        s.env_horizon[i] = hor[i];
    }
    for (const auto &l : r->lights_host)
        if (l.kind == RT_LIGHT_ENVIRONMENT) {
            s.env_intensity = l.intensity;
            for (int i = 0; i < 3; ++i) {
                s.env_color[i] = l.color[i];
                s.env_horizon[i] = l.data[i];
            }
            break;
        }
}

// Every scene array gets at least one (zeroed) element, so a clamped index is always in bounds.
template <class T>
int upload(DevBuf &b, const T *src, uint64_t n, cudaStream_t st) {
    const size_t bytes = sizeof(T) * (n ? n : 1);
    RT_CK(b.alloc(bytes));
    if (n) RT_CK(cudaMemcpyAsync(b.p, src, sizeof(T) * n, cudaMemcpyHostToDevice, st));
    else RT_CK(cudaMemsetAsync(b.p, 0, bytes, st));
    return RT_OK;
}

uint32_t denoise_passes(const rt_render_config &c) { return c.denoise_passes ? c.denoise_passes : 2u; }
uint32_t max_bounces(const rt_render_config &c) { return c.max_bounces ? c.max_bounces : RT_MAX_BOUNCES; }

rt_image_params image_params(const rt_renderer *r, float alpha) {
    const rt_render_config &c = r->cfg;
    rt_image_params ip;
    std::memset(&ip, 0, sizeof(ip));
    ip.width = c.width;
    ip.height = c.height;
    ip.spp = c.spp;
    ip.frame = r->sample_counter;
    for (int i = 0; i < 3; ++i) {
        ip.light_emission[i] = c.light_emission[i];
        ip.point_light_emission[i] = c.point_light_emission[i];
    }
    ip.ambient = c.ambient;
    ip.accumulate_alpha = alpha;
    ip.use_photons = c.enable_photon_map ? 1u : 0u;
    ip.photon_count = c.photon_count;
    ip.photon_radius = c.photon_radius;
    ip.photon_scale = c.photon_scale;
    ip.photon_debug = c.photon_debug ? 1u : 0u;
    ip._pad[0] = c.debug_view;
    return ip;
}

int check_renderer(const rt_renderer *r, const char *fn) {
    if (!r) {
        set_error("%s: null renderer", fn);
        return RT_ERR_INVALID_ARGUMENT;
    }
    return RT_OK;
}

}  // namespace

extern "C" int rt_device_count(void) {
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return n;
}

namespace {

int check_scene_desc(const rt_scene_desc *sd, const char *fn) {
    if ((sd->triangle_count && !sd->triangles) || (sd->bvh_node_count && !sd->bvh_nodes) ||
        (sd->bvh_prim_count && !sd->bvh_prims) || (sd->material_count && !sd->materials) ||
        (sd->light_count && !sd->lights)) {
        set_error("%s: scene array pointer is null with a non-zero count", fn);
        return RT_ERR_INVALID_ARGUMENT;
    }
    if (sd->bvh_node_count && (sd->triangle_count == 0 || sd->material_count == 0 || sd->bvh_prim_count == 0)) {
        set_error("%s: a BVH needs triangles, prim indices and at least one material", fn);
        return RT_ERR_INVALID_ARGUMENT;
    }
    if (sd->triangle_count > 0xFFFFFFFFull || sd->bvh_node_count > 0xFFFFFFFFull || sd->bvh_prim_count > 0xFFFFFFFFull ||
        sd->material_count > 0xFFFFFFFFull || sd->light_count > 0xFFFFFFFFull) {
        set_error("%s: scene arrays are limited to 2^32 - 1 elements", fn);
        return RT_ERR_INVALID_ARGUMENT;
    }
    if (rt_device_count() <= 0) {
        set_error("%s: no CUDA device is visible", fn);
        return RT_ERR_CUDA;
    }
    return RT_OK;
}

int check_config(const rt_render_config *cfg, const char *fn) {
    if (cfg->width == 0 || cfg->height == 0 || (uint64_t)cfg->width * cfg->height > (1ull << 28)) {
        set_error("%s: width/height must be non-zero and width*height <= 2^28", fn);
        return RT_ERR_INVALID_ARGUMENT;
    }
    if (cfg->enable_photon_map && (uint64_t)cfg->photon_count * RT_MAX_BOUNCES > 0xFFFFFFFFull) {
        set_error("%s: photon_count * 6 must fit in 32 bits", fn);
        return RT_ERR_INVALID_ARGUMENT;
    }
    return RT_OK;
}

uint64_t photon_slots_of(const rt_render_config &c) {
    return c.enable_photon_map ? std::max<uint64_t>((uint64_t)c.photon_count * RT_MAX_BOUNCES, 1) : 1;
}

// The renderer's own buffers on a resident scene (Renderer::new after the scene upload).
int create_on(rt_resident_scene *res, const rt_render_config *cfg, rt_renderer **out) {
    rt_renderer *r = new (std::nothrow) rt_renderer();
    if (!r) {
        set_error("rt_renderer_create: out of host memory");
        return RT_ERR_OUT_OF_MEMORY;
    }
    auto fail = [&](int st) {
        delete r;
        return st;
    };
    cudaGetDevice(&r->device);
    if (r->device != res->device) {
        set_error("rt_renderer_create: the resident scene lives on device %d, the current device is %d",
                  res->device, r->device);
        return fail(RT_ERR_INVALID_ARGUMENT);
    }
    res->refs.fetch_add(1);
    r->res = res;
    if (cudaStreamCreateWithFlags(&r->stream, cudaStreamNonBlocking) != cudaSuccess) {
        set_error("rt_renderer_create: cudaStreamCreate failed");
        return fail(RT_ERR_CUDA);
    }
    if (r->events.create() != cudaSuccess) {
        set_error("rt_renderer_create: cudaEventCreate failed");
        return fail(RT_ERR_CUDA);
    }
    if (cudaMemPool_t pool = rt::renderer_pool_acquire(r->device)) r->bind_buffers(pool);
    r->cfg = *cfg;
    cudaStream_t s = r->stream;
    int st;
    // Lights are per renderer (update_lights changes them); the rest of the scene is shared.
    r->lights_host = res->lights;
    if ((st = upload(r->d_lights, res->lights.data(), res->lights.size(), s)) != RT_OK) return fail(st);
    r->scene = res->scene;
    r->scene.lights = r->d_lights.as<float4>();
    r->scene.light_count = (uint32_t)res->lights.size();
    resolve_env(r);

    // Camera::default().to_uniform (lib.rs:267-271).
    rt_camera c0;
    rt_camera_default(&c0);
    rt_camera_to_uniform(&c0, cfg->width, cfg->height, &r->cam);

    // Frame buffers (lib.rs:273-316).
    const size_t npix = (size_t)cfg->width * cfg->height;
    DevBuf *fb[5] = {&r->d_frame, &r->d_pingpong, &r->d_moments, &r->d_gbuffer, &r->d_accum};
    for (DevBuf *b : fb) {
        if (b->alloc(npix * 16) != cudaSuccess) {
            set_error("rt_renderer_create: out of device memory for frame buffers");
            return fail(RT_ERR_OUT_OF_MEMORY);
        }
        RT_CK(cudaMemsetAsync(b->p, 0, npix * 16, s));
    }
    r->num_sms = rtd::device_sm_count();
    rtd::prepare_kernels();
    RT_CK(r->d_output.alloc(npix * 4));
    RT_CK(cudaMemsetAsync(r->d_output.p, 0, npix * 4, s));
    RT_CK(r->d_counters.alloc(64));
    RT_CK(cudaMemsetAsync(r->d_counters.p, 0, 64, s));

    // Photon grid (lib.rs:276-286, 416-481).
    r->photon_buffers = cfg->enable_photon_map != 0;
    r->photon_slots = photon_slots_of(*cfg);
    float radius = cfg->photon_radius;
    rt_derive_grid(res->bmin, res->bmax, (int)res->has_bounds, cfg->grid_max_dim, cfg->photon_radius_mode,
                   (uint32_t)r->photon_slots, &r->gp, &radius);
    r->cfg.photon_radius = radius;
    const uint64_t S = r->photon_slots, C = r->gp.num_cells;
    if (r->d_photons.alloc(S * 64) != cudaSuccess || r->d_sorted.alloc(S * 64) != cudaSuccess ||
        r->d_sorted_pos.alloc(S * 16) != cudaSuccess || r->d_rank.alloc(S * 4) != cudaSuccess ||
        r->d_keys.alloc(S * 4) != cudaSuccess || r->d_order.alloc(S * 4) != cudaSuccess ||
        r->d_counts.alloc(C * 4) != cudaSuccess || r->d_cursor.alloc(C * 4) != cudaSuccess ||
        r->d_meta.alloc(C * 8) != cudaSuccess ||
        r->d_partials.alloc((size_t)rtd::grid_scan_partials((uint32_t)C) * 4) != cudaSuccess ||
        r->d_total.alloc(16) != cudaSuccess) {
        set_error("rt_renderer_create: out of device memory for photon buffers (%llu slots, %llu cells)",
                  (unsigned long long)S, (unsigned long long)C);
        return fail(RT_ERR_OUT_OF_MEMORY);
    }
    RT_CK(cudaMemsetAsync(r->d_photons.p, 0, S * 64, s));
    RT_CK(cudaMemsetAsync(r->d_sorted.p, 0, S * 64, s));
    RT_CK(cudaMemsetAsync(r->d_sorted_pos.p, 0, S * 16, s));
    RT_CK(cudaMemsetAsync(r->d_keys.p, 0xFF, S * 4, s));
    RT_CK(cudaMemsetAsync(r->d_counts.p, 0, C * 4, s));
    RT_CK(cudaMemsetAsync(r->d_meta.p, 0, C * 8, s));
    RT_CK(cudaMemsetAsync(r->d_total.p, 0, 16, s));
    RT_CK(cudaStreamSynchronize(s));
    *out = r;
    return RT_OK;
}

}  // namespace

rt_renderer::~rt_renderer() {
    if (stream) {
        // The frees are ordered after the renderer's own work, and a batch frame the renderer took
        // part in is part of it (the batch makes each member's stream wait for the frame).
        release_buffers();
        cudaStreamSynchronize(stream);
        cudaStreamDestroy(stream);
    }
    for (cudaEvent_t e : prof_ev)
        if (e) cudaEventDestroy(e);
    if (res) rt::resident_scene_release(res);
    if (pooled) rt::renderer_pool_release(device);
}

std::array<rt::DevBuf *, 32> rt_renderer::buffers() {
    return {&d_lights,   &d_frame,   &d_pingpong, &d_moments,     &d_gbuffer,     &d_accum,       &d_output,
            &d_photons,  &d_keys,    &d_rank,     &d_order,       &d_sorted,      &d_sorted_pos,  &d_counts,
            &d_meta,     &d_cursor,  &d_partials, &d_total,       &d_counters,    &d_work,        &jobs.dev,
            &path.ro,    &path.rd,   &path.thr,   &path.hit,      &path.acc,      &path.nrm,      &path.queue[0],
            &path.queue[1], &path.shadow, &path.preq, &path.counts};
}

void rt_renderer::bind_buffers(cudaMemPool_t pool) {
    for (rt::DevBuf *b : buffers()) b->bind(pool, stream);
    pooled = true;
}

void rt_renderer::release_buffers() {
    for (rt::DevBuf *b : buffers()) b->release();
}

uint64_t rt_renderer::device_bytes() const {
    uint64_t n = 0;
    for (const rt::DevBuf *b : const_cast<rt_renderer *>(this)->buffers()) n += b->bytes;
    return n;
}

namespace rt {

namespace {
struct PoolEntry {
    cudaMemPool_t pool = nullptr;
    uint32_t live = 0;
    bool tried = false;
};
std::mutex g_pool_mu;
PoolEntry g_pools[64];
}  // namespace

cudaMemPool_t renderer_pool_acquire(int device) {
    if (device < 0 || device >= 64) return nullptr;
    std::lock_guard<std::mutex> lk(g_pool_mu);
    PoolEntry &e = g_pools[device];
    if (!e.tried) {
        e.tried = true;
        int supported = 0;
        if (cudaDeviceGetAttribute(&supported, cudaDevAttrMemoryPoolsSupported, device) == cudaSuccess &&
            supported) {
            cudaMemPoolProps props;
            std::memset(&props, 0, sizeof(props));
            props.allocType = cudaMemAllocationTypePinned;
            props.location.type = cudaMemLocationTypeDevice;
            props.location.id = device;
            if (cudaMemPoolCreate(&e.pool, &props) == cudaSuccess) {
                uint64_t keep = ~0ull;  // freed blocks stay in the pool until the last renderer goes
                cudaMemPoolSetAttribute(e.pool, cudaMemPoolAttrReleaseThreshold, &keep);
            } else {
                e.pool = nullptr;
            }
        }
        cudaGetLastError();
    }
    if (e.pool) e.live += 1;
    return e.pool;
}

void renderer_pool_release(int device) {
    if (device < 0 || device >= 64) return;
    std::lock_guard<std::mutex> lk(g_pool_mu);
    PoolEntry &e = g_pools[device];
    if (e.pool && e.live > 0 && --e.live == 0) cudaMemPoolTrimTo(e.pool, 0);
}

int ensure_job_table(rt_renderer *r) {
    if (r->jobs.ready()) return RT_OK;
    if (r->jobs.init(1) != cudaSuccess) {
        set_error("rt_renderer: cannot allocate the job table");
        return RT_ERR_OUT_OF_MEMORY;
    }
    return RT_OK;
}

int resident_scene_create(const rt_scene_desc *sd, rt_resident_scene **out) {
    *out = nullptr;
    rt_resident_scene *res = new (std::nothrow) rt_resident_scene();
    if (!res) {
        set_error("rt_resident_scene_create: out of host memory");
        return RT_ERR_OUT_OF_MEMORY;
    }
    auto fail = [&](int st) {
        delete res;
        return st;
    };
    cudaGetDevice(&res->device);
    cudaStream_t s = nullptr;
    if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess) {
        set_error("rt_resident_scene_create: cudaStreamCreate failed");
        return fail(RT_ERR_CUDA);
    }
    struct StreamGuard {
        cudaStream_t s;
        ~StreamGuard() {
            cudaStreamSynchronize(s);
            cudaStreamDestroy(s);
        }
    } guard{s};
    int st;
    // Scene upload (Renderer::new, lib.rs:234-266).
    if ((st = upload(res->d_tris, sd->triangles, sd->triangle_count, s)) != RT_OK) return fail(st);
    rt::TraversalLayout lay;
    if (!rt::build_traversal_layout(sd->bvh_nodes, sd->bvh_node_count, sd->bvh_prims, sd->bvh_prim_count,
                                    sd->triangles, sd->triangle_count, lay))
        return fail(RT_ERR_INVALID_ARGUMENT);
    // Each prim slot's shade order key and material (clamped as the kernels clamp it) in its record's
    // spare word (the first edge's .w), which shade reads with the hit's prim slot: key 1 dielectric,
    // 2 Lambertian or emissive, 3 metal.
    for (uint64_t k = 0; k < sd->bvh_prim_count; ++k) {
        const uint64_t mid = std::min<uint64_t>(sd->triangles[sd->bvh_prims[k]].material_id,
                                                sd->material_count ? sd->material_count - 1 : 0);
        const uint32_t kind = sd->material_count ? sd->materials[mid].kind : 0u;
        const uint32_t key = kind == 2u ? 1u : (kind == 1u ? 3u : 2u);
        const uint32_t word = key | ((mid < rtd::kNoMat ? (uint32_t)mid : rtd::kNoMat) << 2);
        std::memcpy(&lay.tri_ord[k * 12 + 7], &word, 4);
    }
    if ((st = upload(res->d_cnodes, lay.cnodes.data(), lay.cnodes.size(), s)) != RT_OK) return fail(st);
    // The four-wide records when the library traverses four-wide and a walk of them fits the largest
    // shared-memory stack without dropping a push.
    rt::WideLayout wide;
    if (rt::traversal_width() == 4u && sd->bvh_node_count > 0) {
        rt::build_wide_layout(sd->bvh_nodes, sd->bvh_node_count, wide);
        if (wide.stack_need > 64u) wide.nodes.clear();
        if (!wide.nodes.empty() && (st = upload(res->d_wnodes, wide.nodes.data(), wide.nodes.size(), s)) != RT_OK)
            return fail(st);
    }
    if ((st = upload(res->d_tri_ord, lay.tri_ord.data(), lay.tri_ord.size(), s)) != RT_OK) return fail(st);
    if ((st = upload(res->d_mats, sd->materials, sd->material_count, s)) != RT_OK) return fail(st);
    res->lights.assign(sd->lights, sd->lights + sd->light_count);
    rtd::DevScene &ds = res->scene;
    ds.cnodes = res->d_cnodes.as<float4>();
    ds.tri_ord = res->d_tri_ord.as<float4>();
    ds.cnode_count = (uint32_t)(lay.cnodes.size() / 16);
    ds.wnodes = wide.nodes.empty() ? nullptr : res->d_wnodes.as<float4>();
    ds.wnode_count = (uint32_t)(wide.nodes.size() / 32);
    ds.wide_stack = wide.nodes.empty() ? 0u : wide.stack_need;
    // A near-first traversal holds at most one pending entry per tree level.
    ds.stack_cap = lay.max_depth < 32u ? 32u : 63u;
    ds.any_hit_shadows = 1u;
    for (uint64_t i = 0; i < sd->material_count; ++i)
        if ((sd->materials[i].flags & RT_MAT_FLAG_ALPHA_CUTOUT) && sd->materials[i].tex_albedo != RT_TEX_NONE)
            ds.any_hit_shadows = 0u;
    ds.tris = res->d_tris.as<float4>();
    ds.mats = res->d_mats.as<float4>();
    ds.tri_count = (uint32_t)sd->triangle_count;
    ds.mat_count = (uint32_t)sd->material_count;
    const rt_texture_array *roles[4] = {&sd->tex_albedo, &sd->tex_mr, &sd->tex_emissive, &sd->tex_normal};
    for (int i = 0; i < 4; ++i) {
        const rt_texture_array &t = *roles[i];
        if (t.rgba8 && t.layers && t.width && t.height) {
            size_t bytes = (size_t)t.width * t.height * t.layers * 4;
            if ((st = upload(res->d_tex[i], t.rgba8, bytes, s)) != RT_OK) return fail(st);
            ds.tex[i] = rtd::DevTex{res->d_tex[i].as<uchar4>(), t.width, t.height, t.layers};
        } else {
            ds.tex[i] = rtd::DevTex{nullptr, 0, 0, 0};
        }
    }
    // The host copies of the layout are freed when `lay` goes out of scope; wait for the copies first.
    RT_CK(cudaStreamSynchronize(s));
    for (int i = 0; i < 3; ++i) {
        res->bmin[i] = sd->bounds_min[i];
        res->bmax[i] = sd->bounds_max[i];
    }
    res->has_bounds = sd->has_bounds;
    res->bytes = res->d_cnodes.bytes + res->d_wnodes.bytes + res->d_tri_ord.bytes + res->d_tris.bytes + res->d_mats.bytes +
                 res->d_tex[0].bytes + res->d_tex[1].bytes + res->d_tex[2].bytes + res->d_tex[3].bytes;
    *out = res;
    return RT_OK;
}

void resident_scene_release(rt_resident_scene *s) {
    if (s && s->refs.fetch_sub(1) == 1u) delete s;
}

uint64_t path_state_bytes(uint64_t slots, uint32_t iters) {
    return slots * 240u + sizeof(uint32_t) * 4ull * ((uint64_t)iters + 1);
}

uint64_t renderer_create_bytes(const rt_render_config &c, uint64_t num_cells, uint64_t n_lights) {
    // The allocations of create_on: frame buffers (5 x float4 + rgba8 per pixel), photon slots, keys,
    // ranks, slot order, sorted photons and their positions, counts / cursor / meta per cell, scan partials, grid totals,
    // counters and the renderer's own light buffer (the one-entry job table comes with the first solo
    // frame or photon rebuild).
    const uint64_t npix = (uint64_t)c.width * c.height;
    const uint64_t S = photon_slots_of(c);
    return npix * (5 * 16 + 4) + S * (64 + 64 + 16 + 4 + 4 + 4) + num_cells * 16 +
           (uint64_t)rtd::grid_scan_partials((uint32_t)num_cells) * 4 + 16 + 64 +
           sizeof(rt_light) * std::max<uint64_t>(n_lights, 1);
}

}  // namespace rt

extern "C" int rt_resident_scene_create(const rt_scene_desc *sd, rt_resident_scene **out) {
    return rt::guarded("rt_resident_scene_create", [&]() -> int {
        rt::clear_error();
        if (!sd || !out) {
            set_error("rt_resident_scene_create: null argument");
            return RT_ERR_INVALID_ARGUMENT;
        }
        *out = nullptr;
        if (int st = check_scene_desc(sd, "rt_resident_scene_create")) return st;
        return rt::resident_scene_create(sd, out);
    });
}

extern "C" void rt_resident_scene_release(rt_resident_scene *s) { rt::resident_scene_release(s); }

extern "C" uint64_t rt_resident_scene_bytes(const rt_resident_scene *s) { return s ? s->bytes : 0; }

extern "C" uint32_t rt_resident_scene_refs(const rt_resident_scene *s) { return s ? s->refs.load() : 0u; }

extern "C" int rt_renderer_create_resident(rt_resident_scene *res, const rt_render_config *cfg, rt_renderer **out) {
    return rt::guarded("rt_renderer_create_resident", [&]() -> int {
        rt::clear_error();
        if (!res || !cfg || !out) {
            set_error("rt_renderer_create_resident: null argument");
            return RT_ERR_INVALID_ARGUMENT;
        }
        *out = nullptr;
        if (int st = check_config(cfg, "rt_renderer_create_resident")) return st;
        return create_on(res, cfg, out);
    });
}

extern "C" int rt_renderer_create(const rt_scene_desc *sd, const rt_render_config *cfg, rt_renderer **out) {
    return rt::guarded("rt_renderer_create", [&]() -> int {
        rt::clear_error();
        if (!sd || !cfg || !out) {
            set_error("rt_renderer_create: null argument");
            return RT_ERR_INVALID_ARGUMENT;
        }
        *out = nullptr;
        if (int st = check_config(cfg, "rt_renderer_create")) return st;
        if (int st = check_scene_desc(sd, "rt_renderer_create")) return st;
        rt_resident_scene *res = nullptr;
        if (int st = rt::resident_scene_create(sd, &res)) return st;
        const int st = create_on(res, cfg, out);
        rt::resident_scene_release(res);  // the renderer holds its own reference
        return st;
    });
}

extern "C" uint64_t rt_renderer_device_bytes(const rt_renderer *r) { return r ? r->device_bytes() : 0; }

extern "C" uint32_t rt_tma_timeouts(void) { return rtd::tma_timeouts(); }
extern "C" uint32_t rt_scan_timeouts(void) { return rtd::scan_timeouts(); }

extern "C" int rt_renderer_footprint(const rt_render_config *cfg, const rt_resident_scene *res, uint64_t *create_bytes,
                                     uint64_t *solo_path_bytes) {
    return rt::guarded("rt_renderer_footprint", [&]() -> int {
        rt::clear_error();
        if (!cfg || !res || !create_bytes) {
            set_error("rt_renderer_footprint: null argument");
            return RT_ERR_INVALID_ARGUMENT;
        }
        if (int st = check_config(cfg, "rt_renderer_footprint")) return st;
        rt_grid_params gp;
        float radius = cfg->photon_radius;
        rt_derive_grid(res->bmin, res->bmax, (int)res->has_bounds, cfg->grid_max_dim, cfg->photon_radius_mode,
                       (uint32_t)photon_slots_of(*cfg), &gp, &radius);
        *create_bytes = rt::renderer_create_bytes(*cfg, gp.num_cells, res->lights.size());
        if (solo_path_bytes) {
            const uint32_t spp = cfg->spp > 1u ? cfg->spp : 1u;
            *solo_path_bytes = rt::path_state_bytes((uint64_t)cfg->width * cfg->height, spp * max_bounces(*cfg)) +
                               sizeof(rtd::DevJob);
        }
        return RT_OK;
    });
}

extern "C" void rt_renderer_destroy(rt_renderer *r) { delete r; }

namespace rt {

float prepare_frame(rt_renderer *r) {
    const rt_render_config &c = r->cfg;
    // lib.rs:672-684
    r->sample_counter += 1u;
    if (r->frames_since_reset != 0xFFFFFFFFu) r->frames_since_reset += 1u;
    return c.accumulate_frames == 0 ? 1.0f : 1.0f / (float)std::min(r->frames_since_reset, c.accumulate_frames);
}

uint32_t frame_iterations(const rt_renderer *r) {
    const uint32_t spp = r->cfg.spp > 1u ? r->cfg.spp : 1u;
    return spp * max_bounces(r->cfg);
}

rtd::DevJob make_job(const rt_renderer *r, uint32_t base) {
    const rt_render_config &c = r->cfg;
    rtd::DevJob j;
    std::memset(&j, 0, sizeof(j));
    j.scene = r->scene;
    j.cam = r->cam;
    j.ip = image_params(r, c.accumulate_frames == 0 ? 1.0f
                                                    : 1.0f / (float)std::min(r->frames_since_reset, c.accumulate_frames));
    j.gp = r->gp;
    j.sorted_photons = r->d_sorted.as<float4>();
    j.sorted_pos = r->d_sorted_pos.as<float4>();
    j.sorted_count = r->photon_slots;
    j.grid_meta = r->d_meta.as<uint2>();
    j.max_bounces = max_bounces(c);
    j.npix = c.width * c.height;
    j.base = base;
    j.spp = c.spp > 1u ? c.spp : 1u;
    j.frame = r->d_frame.as<float4>();
    j.moments = r->d_moments.as<float4>();
    j.gbuffer = r->d_gbuffer.as<float4>();
    j.alpha = j.ip.accumulate_alpha;
    return j;
}

int enqueue_denoise(rt_renderer *r, float alpha, const float *alpha_dev, cudaStream_t s, float4 **result_out) {
    const rt_render_config &c = r->cfg;
    // lib.rs:743-776: a-trous passes, steps 1, 2, ..., ping-pong frame <-> pingpong.
    float4 *result = r->d_frame.as<float4>();
    const uint32_t passes = c.enable_denoise ? denoise_passes(c) : 0u;
    for (uint32_t it = 0; it < passes; ++it) {
        rt_denoise_params dp;
        std::memset(&dp, 0, sizeof(dp));
        dp.width = c.width;
        dp.height = c.height;
        dp.step_size = 1u << it;
        dp.lambda = 3.0f;
        dp.phi_normal = 12.0f;
        dp.phi_depth = 0.05f;
        dp.alpha = alpha;
        const float4 *in = (it % 2 == 0) ? r->d_frame.as<float4>() : r->d_pingpong.as<float4>();
        float4 *o = (it % 2 == 0) ? r->d_pingpong.as<float4>() : r->d_frame.as<float4>();
        RT_CK(rtd::launch_denoise(in, o, r->d_gbuffer.as<float4>(), r->d_moments.as<float4>(), dp, alpha_dev, s,
                                  it == 1u));
        result = o;
    }
    r->last_denoise_passes = passes;
    *result_out = result;
    return RT_OK;
}

int enqueue_resolve(rt_renderer *r, const float4 *result, float alpha, const float *alpha_dev, cudaStream_t s) {
    const rt_render_config &c = r->cfg;
    // lib.rs:778-831: composite, then tonemap.
    rt_tonemap_params tp;
    std::memset(&tp, 0, sizeof(tp));
    tp.exposure = c.exposure;
    tp.gamma = c.gamma;
    tp.width = c.width;
    tp.glow = r->glow;
    std::memcpy(tp.marker, r->marker, sizeof(tp.marker));
    RT_CK(rtd::launch_resolve(result, r->d_accum.as<float4>(), r->d_gbuffer.as<float4>(), c.width, c.height, alpha,
                              alpha_dev, tp, r->d_output.as<uchar4>(), s));
    return RT_OK;
}

int enqueue_post(rt_renderer *r, float alpha, const float *alpha_dev, cudaStream_t s) {
    float4 *result = nullptr;
    if (int st = enqueue_denoise(r, alpha, alpha_dev, s, &result)) return st;
    return enqueue_resolve(r, result, alpha, alpha_dev, s);
}

}  // namespace rt

extern "C" int rt_render_frame(rt_renderer *r) {
    return rt::guarded("rt_render_frame", [&]() -> int {
        if (int st = check_renderer(r, "rt_render_frame")) return st;
        rt::clear_error();
        cudaStream_t s = r->stream;
        const rt_render_config &c = r->cfg;
        const float alpha = rt::prepare_frame(r);
        const uint32_t iters = rt::frame_iterations(r);
        const size_t npix = (size_t)c.width * c.height;
        if (npix > r->path.slots || sizeof(uint32_t) * 4 * ((size_t)iters + 1) > r->path.counts_bytes) {
            RT_CK(cudaStreamSynchronize(s));
            RT_CK(r->path.ensure(npix, iters));
        }
        cudaEvent_t fe[4] = {nullptr, nullptr, nullptr, nullptr};
        for (auto &e : fe) RT_CK(r->ring.next(&e));
        RT_CK(cudaEventRecord(r->events.ev[EV_FRAME0], s));
        if (fe[3]) RT_CK(cudaEventRecord(fe[0], s));
        const rtd::DevJob job = rt::make_job(r, 0u);
        if (int st = rt::ensure_job_table(r)) return st;
        RT_CK(r->jobs.upload(&job, 1, s));
        const rtd::WaveParams wp = r->path.params(r->jobs.device(), 1u, r->d_counters.as<unsigned long long>());
        const rtd::JobShape shape{c.width,
                                  c.height,
                                  (uint32_t)npix,
                                  0u,
                                  r->scene.stack_cap,
                                  c.enable_photon_map ? 1u : 0u,
                                  c.debug_view != 0u ? 1u : 0u,
                                  r->scene.wnodes ? 1u : 0u,
                                  r->scene.wide_stack};
        if (r->prof_flags) {
            if (int st = rt::profiled_gather(r, wp, shape, iters)) return st;
        } else {
            RT_CK(rtd::launch_wavefront(wp, &shape, 1u, iters, r->num_sms, r->tuning, s));
        }
        RT_CK(cudaEventRecord(r->events.ev[EV_GATHER1], s));
        if (fe[3]) RT_CK(cudaEventRecord(fe[1], s));
        float4 *result = nullptr;
        if (int st = rt::enqueue_denoise(r, alpha, nullptr, s, &result)) return st;
        RT_CK(cudaEventRecord(r->events.ev[EV_DENOISE1], s));
        if (fe[3]) RT_CK(cudaEventRecord(fe[2], s));
        if (int st = rt::enqueue_resolve(r, result, alpha, nullptr, s)) return st;
        RT_CK(cudaEventRecord(r->events.ev[EV_RESOLVE1], s));
        if (fe[3]) RT_CK(cudaEventRecord(fe[3], s));
        r->frames += 1;
        r->have_frame_timing = true;
        return RT_OK;
    });
}

namespace rt {
// The gather pass of a profiled frame: launches bracketed by events, the counting traversal kernels
// when asked, then a wait for the pass and the sums added to r->prof.
int profiled_gather(rt_renderer *r, rtd::WaveParams wp, const rtd::JobShape &shape, uint32_t iters) {
    cudaStream_t s = r->stream;
    const size_t per_kind = 2 * ((size_t)iters + 1);
    const size_t need = 3 * per_kind + 2;
    while (r->prof_ev.size() < need) {
        cudaEvent_t e = nullptr;
        RT_CK(cudaEventCreate(&e));
        r->prof_ev.push_back(e);
    }
    const bool count = (r->prof_flags & RT_PROFILE_COUNT) != 0u;
    if (count) {
        if (!r->d_work.p) RT_CK(r->d_work.alloc(4 * sizeof(unsigned long long)));
        RT_CK(cudaMemsetAsync(r->d_work.p, 0, 4 * sizeof(unsigned long long), s));
        wp.work = r->d_work.as<unsigned long long>();
    }
    const bool events = (r->prof_flags & RT_PROFILE_EVENTS) != 0u;
    cudaEvent_t *ev = r->prof_ev.data();
    rtd::WaveProfile prof{events ? ev : nullptr, events ? ev + per_kind : nullptr, events ? ev + 2 * per_kind : nullptr,
                          0u, 0u, 0u};
    cudaEvent_t *pass = ev + 3 * per_kind;
    RT_CK(cudaEventRecord(pass[0], s));
    RT_CK(rtd::launch_wavefront(wp, &shape, 1u, iters, r->num_sms, r->tuning, s, &prof));
    RT_CK(cudaEventRecord(pass[1], s));
    RT_CK(cudaStreamSynchronize(s));
    auto span = [](cudaEvent_t a, cudaEvent_t b) {
        float v = 0.0f;
        return cudaEventElapsedTime(&v, a, b) == cudaSuccess ? (double)v : 0.0;
    };
    rt_trace_profile &p = r->prof;
    p.frames += 1;
    p.trace_launches += prof.trace_launches;
    p.shade_launches += prof.shade_launches;
    p.photon_launches += prof.photon_launches;
    if (events) {
        for (uint32_t i = 0; i < prof.trace_launches; ++i) p.ms_trace += span(ev[2 * i], ev[2 * i + 1]);
        for (uint32_t i = 0; i < prof.shade_launches; ++i)
            p.ms_shade += span(ev[per_kind + 2 * i], ev[per_kind + 2 * i + 1]);
        for (uint32_t i = 0; i < prof.photon_launches; ++i)
            p.ms_photon += span(ev[2 * per_kind + 2 * i], ev[2 * per_kind + 2 * i + 1]);
    }
    p.ms_gather += span(pass[0], pass[1]);
    std::vector<uint32_t> counts(4 * ((size_t)iters + 1));
    RT_CK(cudaMemcpy(counts.data(), wp.counts, counts.size() * sizeof(uint32_t), cudaMemcpyDeviceToHost));
    for (uint32_t i = 0; i < iters; ++i) {
        p.closest_rays += counts[4 * i];
        p.occlusion_rays += counts[4 * i + 1];
    }
    if (count) {
        unsigned long long w[4];
        RT_CK(cudaMemcpy(w, r->d_work.p, sizeof(w), cudaMemcpyDeviceToHost));
        p.records_closest += w[0];
        p.records_occlusion += w[1];
        p.tri_tests_closest += w[2];
        p.tri_tests_occlusion += w[3];
    }
    p.record_bytes = shape.wide ? 128u : 64u;
    p.pixels = shape.npix;
    return RT_OK;
}
}  // namespace rt

extern "C" int rt_set_profiling(rt_renderer *r, uint32_t flags) {
    return rt::guarded("rt_set_profiling", [&]() -> int {
        if (int st = check_renderer(r, "rt_set_profiling")) return st;
        if (flags & ~(RT_PROFILE_EVENTS | RT_PROFILE_COUNT)) {
            set_error("rt_set_profiling: unknown flags 0x%x", flags);
            return RT_ERR_INVALID_ARGUMENT;
        }
        r->prof_flags = flags;
        return RT_OK;
    });
}

extern "C" int rt_read_profile(rt_renderer *r, rt_trace_profile *out) {
    return rt::guarded("rt_read_profile", [&]() -> int {
        if (int st = check_renderer(r, "rt_read_profile")) return st;
        if (!out) {
            set_error("rt_read_profile: null out");
            return RT_ERR_INVALID_ARGUMENT;
        }
        RT_CK(cudaStreamSynchronize(r->stream));
        *out = r->prof;
        r->prof = rt_trace_profile{};
        return RT_OK;
    });
}

extern "C" int rt_render_frames(rt_renderer *r, uint32_t n) {
    return rt::guarded("rt_render_frames", [&]() -> int {
        if (int st = check_renderer(r, "rt_render_frames")) return st;
        for (uint32_t i = 0; i < n; ++i)
            if (int st = rt_render_frame(r)) return st;
        return RT_OK;
    });
}

extern "C" int rt_update_camera(rt_renderer *r, const rt_camera *cam) {
    return rt::guarded("rt_update_camera", [&]() -> int {
        if (int st = check_renderer(r, "rt_update_camera")) return st;
        if (!cam) {
            set_error("rt_update_camera: null camera");
            return RT_ERR_INVALID_ARGUMENT;
        }
        rt_camera_to_uniform(cam, r->cfg.width, r->cfg.height, &r->cam);
        return RT_OK;
    });
}

extern "C" int rt_update_camera_uniform(rt_renderer *r, const rt_camera_uniform *u) {
    return rt::guarded("rt_update_camera_uniform", [&]() -> int {
        if (int st = check_renderer(r, "rt_update_camera_uniform")) return st;
        if (!u) {
            set_error("rt_update_camera_uniform: null uniform");
            return RT_ERR_INVALID_ARGUMENT;
        }
        r->cam = *u;
        return RT_OK;
    });
}

extern "C" int rt_update_lights(rt_renderer *r, const rt_light *lights, uint64_t n) {
    return rt::guarded("rt_update_lights", [&]() -> int {
        if (int st = check_renderer(r, "rt_update_lights")) return st;
        if (n > r->lights_host.size() || (n && !lights)) {
            set_error("rt_update_lights: %llu lights given, the light buffer holds %llu", (unsigned long long)n,
                      (unsigned long long)r->lights_host.size());
            return RT_ERR_INVALID_ARGUMENT;
        }
        if (n == 0) return RT_OK;
        std::memcpy(r->lights_host.data(), lights, n * sizeof(rt_light));
        RT_CK(cudaMemcpyAsync(r->d_lights.p, r->lights_host.data(), n * sizeof(rt_light), cudaMemcpyHostToDevice,
                              r->stream));
        RT_CK(cudaStreamSynchronize(r->stream));
        resolve_env(r);
        return RT_OK;
    });
}

extern "C" int rt_reset_accumulation(rt_renderer *r, int hard) {
    return rt::guarded("rt_reset_accumulation", [&]() -> int {
        if (int st = check_renderer(r, "rt_reset_accumulation")) return st;
        if (hard) RT_CK(cudaMemsetAsync(r->d_accum.p, 0, (size_t)r->cfg.width * r->cfg.height * 16, r->stream));
        r->frames_since_reset = 0;
        return RT_OK;
    });
}

// Slots visited by the count/scatter dispatches of lib.rs:916,951,1026: floor(6P/256) groups of 256.
static uint64_t counted_slots(const rt_renderer *r) {
    const uint32_t P = std::max(r->cfg.photon_count, 1u);
    const uint64_t dispatched = (uint64_t)std::max((uint32_t)(P * RT_MAX_BOUNCES) / 256u, 1u) * 256u;
    return std::min<uint64_t>(dispatched, r->photon_slots);
}

static int build_grid(rt_renderer *r) {
    rtd::GridBuffers g;
    g.photons = r->d_photons.as<float4>();
    g.keys = r->d_keys.as<uint32_t>();
    g.num_cells = r->gp.num_cells;
    g.counts = r->d_counts.as<uint32_t>();
    g.meta = r->d_meta.as<uint2>();
    g.cursor = r->d_cursor.as<uint32_t>();
    g.order = r->d_order.as<uint32_t>();
    g.sorted = r->d_sorted.as<float4>();
    g.sorted_pos = r->d_sorted_pos.as<float4>();
    g.scan_partials = r->d_partials.as<uint32_t>();
    g.total = r->d_total.as<uint32_t>();
    g.rank = r->d_rank.as<uint32_t>();
    g.slot_count = counted_slots(r);
    RT_CK(rtd::launch_grid_build(g, r->stream));
    return RT_OK;
}

int rt::enqueue_photon_rebuild(rt_renderer *r) {
    if (!r->photon_buffers) {
        set_error("rt_rebuild_photons: the renderer was created with enable_photon_map = 0 (no photon buffers)");
        return RT_ERR_STATE;
    }
    cudaStream_t s = r->stream;
    // lib.rs:914-915: floor(P / 256) workgroups of 256 photons (at least one); photons past the
    // buffer are not traced.
    const uint32_t P = std::max(r->cfg.photon_count, 1u);
    const uint64_t traced = std::min<uint64_t>((uint64_t)std::max(P / 256u, 1u) * 256u, r->cfg.photon_count);
    rtd::PhotonTraceParams tp;
    std::memset(&tp, 0, sizeof(tp));
    tp.scene = r->scene;
    tp.gp = r->gp;
    tp.photon_begin = 0;
    tp.photon_end = (uint32_t)traced;
    tp.slot_count = r->photon_slots;
    tp.photons = r->d_photons.as<float4>();
    tp.keys = r->d_keys.as<uint32_t>();
    // The wavefront's state lives in the sorted-photon buffer (6 x 64 B per photon, at least the
    // 64 B per photon the state needs), which the grid build rewrites afterwards.
    if (rtd::photon_wave_bytes((uint32_t)traced) > r->d_sorted.bytes) {
        set_error("rt_rebuild_photons: photon state exceeds the sorted-photon buffer");
        return RT_ERR_STATE;
    }
    const rtd::PhotonWave w = rtd::photon_wave_at(r->d_sorted.p, (uint32_t)traced);
    const rtd::DevJob job = rt::make_job(r, 0u);
    if (int st = rt::ensure_job_table(r)) return st;
    RT_CK(r->jobs.upload(&job, 1, s));
    RT_CK(cudaEventRecord(r->events.ev[EV_TRACE0], s));
    RT_CK(rtd::launch_photon_wave(tp, w, r->jobs.device(), r->num_sms, r->tuning, s));
    RT_CK(cudaEventRecord(r->events.ev[EV_TRACE1], s));
    if (int st = build_grid(r)) return st;
    RT_CK(cudaEventRecord(r->events.ev[EV_GRID1], s));
    r->have_photon_timing = true;
    return RT_OK;
}

extern "C" int rt_rebuild_photons(rt_renderer *r) {
    return rt::guarded("rt_rebuild_photons", [&]() -> int {
        if (int st = check_renderer(r, "rt_rebuild_photons")) return st;
        if (int st = rt::enqueue_photon_rebuild(r)) return st;
        RT_CK(cudaStreamSynchronize(r->stream));
        return RT_OK;
    });
}

extern "C" int rt_load_photons_and_build_grid(rt_renderer *r, const rt_photon *photons, uint64_t n) {
    return rt::guarded("rt_load_photons_and_build_grid", [&]() -> int {
        if (int st = check_renderer(r, "rt_load_photons_and_build_grid")) return st;
        if (!r->photon_buffers || n != r->photon_slots || !photons) {
            set_error("rt_load_photons_and_build_grid: need enable_photon_map and exactly %llu photons",
                      (unsigned long long)r->photon_slots);
            return RT_ERR_INVALID_ARGUMENT;
        }
        cudaStream_t s = r->stream;
        RT_CK(cudaMemcpyAsync(r->d_photons.p, photons, n * 64, cudaMemcpyHostToDevice, s));
        RT_CK(rtd::launch_photon_keys(r->d_photons.as<float4>(), n, r->gp, r->d_keys.as<uint32_t>(), s));
        RT_CK(cudaEventRecord(r->events.ev[EV_TRACE0], s));
        RT_CK(cudaEventRecord(r->events.ev[EV_TRACE1], s));
        if (int st = build_grid(r)) return st;
        RT_CK(cudaEventRecord(r->events.ev[EV_GRID1], s));
        RT_CK(cudaStreamSynchronize(s));
        r->have_photon_timing = true;
        return RT_OK;
    });
}

extern "C" int rt_set_config(rt_renderer *r, const rt_render_config *c) {
    return rt::guarded("rt_set_config", [&]() -> int {
        if (int st = check_renderer(r, "rt_set_config")) return st;
        if (!c) {
            set_error("rt_set_config: null config");
            return RT_ERR_INVALID_ARGUMENT;
        }
        const rt_render_config &o = r->cfg;
        if (c->width != o.width || c->height != o.height || c->photon_count != o.photon_count ||
            c->grid_max_dim != o.grid_max_dim || c->photon_radius_mode != o.photon_radius_mode) {
            set_error("rt_set_config: width, height, photon_count, grid_max_dim and photon_radius_mode are fixed at create");
            return RT_ERR_INVALID_ARGUMENT;
        }
        r->cfg = *c;
        return RT_OK;
    });
}

extern "C" int rt_get_config(const rt_renderer *r, rt_render_config *c) {
    return rt::guarded("rt_get_config", [&]() -> int {
        if (int st = check_renderer(r, "rt_get_config")) return st;
        if (!c) return RT_ERR_INVALID_ARGUMENT;
        *c = r->cfg;
        return RT_OK;
    });
}

extern "C" int rt_set_light_marker(rt_renderer *r, const float marker[4], float glow) {
    return rt::guarded("rt_set_light_marker", [&]() -> int {
        if (int st = check_renderer(r, "rt_set_light_marker")) return st;
        if (marker) std::memcpy(r->marker, marker, sizeof(r->marker));
        else std::memset(r->marker, 0, sizeof(r->marker));
        r->glow = glow;
        return RT_OK;
    });
}

extern "C" uint32_t rt_sample_count(const rt_renderer *r) { return r ? r->sample_counter : 0u; }

extern "C" int rt_get_frame_state(const rt_renderer *r, uint32_t *sample_counter, uint32_t *frames_since_reset) {
    return rt::guarded("rt_get_frame_state", [&]() -> int {
        if (int st = check_renderer(r, "rt_get_frame_state")) return st;
        if (sample_counter) *sample_counter = r->sample_counter;
        if (frames_since_reset) *frames_since_reset = r->frames_since_reset;
        return RT_OK;
    });
}

extern "C" int rt_restore_accumulation(rt_renderer *r, const float *rgba, uint64_t n_floats, uint32_t sample_counter,
                                       uint32_t frames_since_reset) {
    return rt::guarded("rt_restore_accumulation", [&]() -> int {
        if (int st = check_renderer(r, "rt_restore_accumulation")) return st;
        const uint64_t n = (uint64_t)r->cfg.width * r->cfg.height * 4;
        if (!rgba || n_floats != n) {
            set_error("rt_restore_accumulation: need %llu floats (W * H * 4), got %llu", (unsigned long long)n,
                      (unsigned long long)n_floats);
            return RT_ERR_INVALID_ARGUMENT;
        }
        RT_CK(cudaMemcpyAsync(r->d_accum.p, rgba, n * sizeof(float), cudaMemcpyHostToDevice, r->stream));
        RT_CK(cudaStreamSynchronize(r->stream));  // the caller's buffer is only read during the call
        r->sample_counter = sample_counter;
        r->frames_since_reset = frames_since_reset;
        return RT_OK;
    });
}

extern "C" int rt_synchronize(rt_renderer *r) {
    return rt::guarded("rt_synchronize", [&]() -> int {
        if (int st = check_renderer(r, "rt_synchronize")) return st;
        RT_CK(cudaStreamSynchronize(r->stream));
        return RT_OK;
    });
}

extern "C" void *rt_renderer_stream(rt_renderer *r) { return r ? (void *)r->stream : nullptr; }

extern "C" int rt_get_grid_params(const rt_renderer *r, rt_grid_params *out) {
    return rt::guarded("rt_get_grid_params", [&]() -> int {
        if (int st = check_renderer(r, "rt_get_grid_params")) return st;
        if (!out) return RT_ERR_INVALID_ARGUMENT;
        *out = r->gp;
        return RT_OK;
    });
}

extern "C" int rt_get_stats(rt_renderer *r, rt_frame_stats *out) {
    return rt::guarded("rt_get_stats", [&]() -> int {
        if (int st = check_renderer(r, "rt_get_stats")) return st;
        if (!out) return RT_ERR_INVALID_ARGUMENT;
        std::memset(out, 0, sizeof(*out));
        RT_CK(cudaStreamSynchronize(r->stream));
        unsigned long long ctr[2] = {0, 0};
        RT_CK(cudaMemcpy(ctr, r->d_counters.p, 16, cudaMemcpyDeviceToHost));
        uint32_t total = 0;
        RT_CK(cudaMemcpy(&total, r->d_total.p, 4, cudaMemcpyDeviceToHost));
        out->frames = r->frames;
        out->segments = ctr[0];
        out->shadow_rays = ctr[1];
        out->photons_stored = total;
        auto ms = [&](int a, int b) {
            float v = 0.0f;
            if (cudaEventElapsedTime(&v, r->events.ev[a], r->events.ev[b]) != cudaSuccess) {
                cudaGetLastError();
                return 0.0f;
            }
            return v;
        };
        if (r->have_frame_timing) {
            out->ms_gather = ms(EV_FRAME0, EV_GATHER1);
            out->ms_denoise = ms(EV_GATHER1, EV_DENOISE1);
            out->ms_resolve = ms(EV_DENOISE1, EV_RESOLVE1);
            out->ms_frame = ms(EV_FRAME0, EV_RESOLVE1);
        }
        if (r->have_photon_timing) {
            out->ms_photon_trace = ms(EV_TRACE0, EV_TRACE1);
            out->ms_grid_build = ms(EV_TRACE1, EV_GRID1);
        }
        // Drain the per-frame ring: complete groups of four events.
        auto el = [](cudaEvent_t a, cudaEvent_t b) {
            float v = 0.0f;
            if (cudaEventElapsedTime(&v, a, b) != cudaSuccess) {
                cudaGetLastError();
                return 0.0;
            }
            return (double)v;
        };
        const size_t groups = r->ring.used / 4;
        for (size_t g = 0; g < groups; ++g) {
            cudaEvent_t *e = &r->ring.pool[4 * g];
            out->ms_gather_sum += el(e[0], e[1]);
            out->ms_denoise_sum += el(e[1], e[2]);
            out->ms_resolve_sum += el(e[2], e[3]);
            out->ms_frame_sum += el(e[0], e[3]);
        }
        out->timed_frames = groups;
        r->ring.used = 0;
        return RT_OK;
    });
}

namespace {
int read_back(rt_renderer *r, const DevBuf &b, void *dst, uint64_t bytes, uint64_t need, const char *fn) {
    if (int st = check_renderer(r, fn)) return st;
    if (!dst || bytes < need) {
        set_error("%s: destination holds %llu bytes, %llu needed", fn, (unsigned long long)bytes,
                  (unsigned long long)need);
        return RT_ERR_INVALID_ARGUMENT;
    }
    RT_CK(cudaMemcpyAsync(dst, b.p, need, cudaMemcpyDeviceToHost, r->stream));
    RT_CK(cudaStreamSynchronize(r->stream));
    return RT_OK;
}
}  // namespace

#define RT_IMG_BYTES(r) ((uint64_t)(r)->cfg.width * (r)->cfg.height * 16)
extern "C" int rt_read_accumulation(rt_renderer *r, float *rgba, uint64_t n) {
    return rt::guarded("rt_read_accumulation", [&]() -> int {
        return r ? read_back(r, r->d_accum, rgba, n * 4, RT_IMG_BYTES(r), "rt_read_accumulation")
                 : check_renderer(r, "rt_read_accumulation");
    });
}
extern "C" int rt_read_frame(rt_renderer *r, float *rgba, uint64_t n) {
    return rt::guarded("rt_read_frame", [&]() -> int {
        if (!r) return check_renderer(r, "rt_read_frame");
        // The frame as composite consumed it (after the denoise passes, if any).
        const DevBuf &b = (r->last_denoise_passes % 2 == 1) ? r->d_pingpong : r->d_frame;
        return read_back(r, b, rgba, n * 4, RT_IMG_BYTES(r), "rt_read_frame");
    });
}
extern "C" int rt_read_moments(rt_renderer *r, float *rgba, uint64_t n) {
    return rt::guarded("rt_read_moments", [&]() -> int {
        return r ? read_back(r, r->d_moments, rgba, n * 4, RT_IMG_BYTES(r), "rt_read_moments")
                 : check_renderer(r, "rt_read_moments");
    });
}
extern "C" int rt_read_gbuffer(rt_renderer *r, float *rgba, uint64_t n) {
    return rt::guarded("rt_read_gbuffer", [&]() -> int {
        return r ? read_back(r, r->d_gbuffer, rgba, n * 4, RT_IMG_BYTES(r), "rt_read_gbuffer")
                 : check_renderer(r, "rt_read_gbuffer");
    });
}
extern "C" int rt_read_tonemapped(rt_renderer *r, uint8_t *rgba8, uint64_t n) {
    return rt::guarded("rt_read_tonemapped", [&]() -> int {
        return r ? read_back(r, r->d_output, rgba8, n, RT_IMG_BYTES(r) / 4, "rt_read_tonemapped")
                 : check_renderer(r, "rt_read_tonemapped");
    });
}
extern "C" int rt_read_photons(rt_renderer *r, rt_photon *out, uint64_t n) {
    return rt::guarded("rt_read_photons", [&]() -> int {
        return r ? read_back(r, r->d_photons, out, n * 64, r->photon_slots * 64, "rt_read_photons")
                 : check_renderer(r, "rt_read_photons");
    });
}
extern "C" int rt_read_sorted_photons(rt_renderer *r, rt_photon *out, uint64_t n) {
    return rt::guarded("rt_read_sorted_photons", [&]() -> int {
        return r ? read_back(r, r->d_sorted, out, n * 64, r->photon_slots * 64, "rt_read_sorted_photons")
                 : check_renderer(r, "rt_read_sorted_photons");
    });
}
extern "C" int rt_read_photon_grid(rt_renderer *r, uint32_t *counts, uint32_t *meta, uint64_t num_cells) {
    return rt::guarded("rt_read_photon_grid", [&]() -> int {
        if (int st = check_renderer(r, "rt_read_photon_grid")) return st;
        if (num_cells < r->gp.num_cells) {
            set_error("rt_read_photon_grid: %llu cells given, the grid has %u", (unsigned long long)num_cells,
                      r->gp.num_cells);
            return RT_ERR_INVALID_ARGUMENT;
        }
        // The build turns the per-cell counts into (start, count) pairs and clears them for the next
        // build, so the counts are read from the pairs.
        const uint64_t C = r->gp.num_cells;
        std::vector<uint32_t> pairs;
        uint32_t *m = meta;
        if (!m && counts) {
            pairs.resize(2 * C);
            m = pairs.data();
        }
        if (m) {
            if (int st = read_back(r, r->d_meta, m, (meta ? num_cells : C) * 8, C * 8, "rt_read_photon_grid")) return st;
        }
        if (counts)
            for (uint64_t c = 0; c < C; ++c) counts[c] = m[2 * c + 1];
        return RT_OK;
    });
}

// ================================================================================================
// Stage entry points (host buffers in and out; the default stream; temporaries freed on return)
// ================================================================================================
extern "C" int rt_stage_denoise(const float *frame_rgba, const float *gbuffer, const float *moments, uint32_t width,
                                uint32_t height, float alpha, uint32_t passes, float *out_rgba) {
    return rt::guarded("rt_stage_denoise", [&]() -> int {
        rt::clear_error();
        if (!frame_rgba || !gbuffer || !moments || !out_rgba || !width || !height) {
            set_error("rt_stage_denoise: invalid arguments");
            return RT_ERR_INVALID_ARGUMENT;
        }
        const size_t bytes = (size_t)width * height * 16;
        DevBuf a, b, g, m;
        RT_CK(a.alloc(bytes));
        RT_CK(b.alloc(bytes));
        RT_CK(g.alloc(bytes));
        RT_CK(m.alloc(bytes));
        RT_CK(cudaMemcpy(a.p, frame_rgba, bytes, cudaMemcpyHostToDevice));
        RT_CK(cudaMemcpy(g.p, gbuffer, bytes, cudaMemcpyHostToDevice));
        RT_CK(cudaMemcpy(m.p, moments, bytes, cudaMemcpyHostToDevice));
        float4 *cur = a.as<float4>(), *nxt = b.as<float4>();
        for (uint32_t it = 0; it < passes; ++it) {
            rt_denoise_params dp;
            std::memset(&dp, 0, sizeof(dp));
            dp.width = width;
            dp.height = height;
            dp.step_size = 1u << it;
            dp.lambda = 3.0f;
            dp.phi_normal = 12.0f;
            dp.phi_depth = 0.05f;
            dp.alpha = alpha;
            RT_CK(rtd::launch_denoise(cur, nxt, g.as<float4>(), m.as<float4>(), dp, nullptr, 0));
            std::swap(cur, nxt);
        }
        RT_CK(cudaMemcpy(out_rgba, cur, bytes, cudaMemcpyDeviceToHost));
        return RT_OK;
    });
}

extern "C" int rt_stage_resolve(const float *frame_rgba, float *accum_inout, const float *gbuffer, uint32_t width,
                                uint32_t height, float alpha, const rt_tonemap_params *tp, uint8_t *out_rgba8) {
    return rt::guarded("rt_stage_resolve", [&]() -> int {
        rt::clear_error();
        if (!frame_rgba || !accum_inout || !tp || !out_rgba8 || !width || !height) {
            set_error("rt_stage_resolve: invalid arguments");
            return RT_ERR_INVALID_ARGUMENT;
        }
        const size_t bytes = (size_t)width * height * 16;
        DevBuf f, a, g, o;
        RT_CK(f.alloc(bytes));
        RT_CK(a.alloc(bytes));
        RT_CK(o.alloc(bytes / 4));
        RT_CK(cudaMemcpy(f.p, frame_rgba, bytes, cudaMemcpyHostToDevice));
        RT_CK(cudaMemcpy(a.p, accum_inout, bytes, cudaMemcpyHostToDevice));
        const float4 *gp = nullptr;
        if (gbuffer) {
            RT_CK(g.alloc(bytes));
            RT_CK(cudaMemcpy(g.p, gbuffer, bytes, cudaMemcpyHostToDevice));
            gp = g.as<float4>();
        }
        rt_tonemap_params t = *tp;
        t.width = width;
        RT_CK(rtd::launch_resolve(f.as<float4>(), a.as<float4>(), gp, width, height, alpha, nullptr, t, o.as<uchar4>(), 0));
        RT_CK(cudaMemcpy(accum_inout, a.p, bytes, cudaMemcpyDeviceToHost));
        RT_CK(cudaMemcpy(out_rgba8, o.p, bytes / 4, cudaMemcpyDeviceToHost));
        return RT_OK;
    });
}

extern "C" int rt_stage_photon_grid(const rt_photon *photons, const rt_grid_params *gpp, uint32_t *counts,
                                    uint32_t *meta, rt_photon *sorted) {
    return rt::guarded("rt_stage_photon_grid", [&]() -> int {
        rt::clear_error();
        if (!photons || !gpp || !counts || !meta || !sorted || gpp->num_cells == 0) {
            set_error("rt_stage_photon_grid: invalid arguments");
            return RT_ERR_INVALID_ARGUMENT;
        }
        const rt_grid_params gp = *gpp;
        const uint64_t S = gp.photon_slots, C = gp.num_cells;
        DevBuf ph, keys, rank, order, srt, cnt, cur, mt, part, tot;
        RT_CK(ph.alloc(S * 64));
        RT_CK(keys.alloc(S * 4));
        RT_CK(rank.alloc(S * 4));
        RT_CK(order.alloc(S * 4));
        RT_CK(srt.alloc(S * 64));
        RT_CK(cnt.alloc(C * 4));
        RT_CK(cur.alloc(C * 4));
        RT_CK(mt.alloc(C * 8));
        RT_CK(part.alloc((size_t)rtd::grid_scan_partials((uint32_t)C) * 4));
        RT_CK(tot.alloc(16));
        if (S) RT_CK(cudaMemcpy(ph.p, photons, S * 64, cudaMemcpyHostToDevice));
        RT_CK(cudaMemset(srt.p, 0, S * 64 ? S * 64 : 16));
        RT_CK(cudaMemset(tot.p, 0, 16));
        RT_CK(cudaMemset(cnt.p, 0, C * 4));  // the build expects zero counts and leaves them zero
        RT_CK(rtd::launch_photon_keys(ph.as<float4>(), S, gp, keys.as<uint32_t>(), 0));
        rtd::GridBuffers g;
        g.photons = ph.as<float4>();
        g.keys = keys.as<uint32_t>();
        g.slot_count = S;
        g.num_cells = (uint32_t)C;
        g.counts = cnt.as<uint32_t>();
        g.meta = mt.as<uint2>();
        g.cursor = cur.as<uint32_t>();
        g.order = order.as<uint32_t>();
        g.sorted = srt.as<float4>();
        g.sorted_pos = nullptr;
        g.scan_partials = part.as<uint32_t>();
        g.total = tot.as<uint32_t>();
        g.rank = rank.as<uint32_t>();
        RT_CK(rtd::launch_grid_build(g, 0));
        RT_CK(cudaMemcpy(meta, mt.p, C * 8, cudaMemcpyDeviceToHost));
        for (uint64_t c = 0; c < C; ++c) counts[c] = meta[2 * c + 1];  // the build cleared the counts
        if (S) RT_CK(cudaMemcpy(sorted, srt.p, S * 64, cudaMemcpyDeviceToHost));
        return RT_OK;
    });
}

