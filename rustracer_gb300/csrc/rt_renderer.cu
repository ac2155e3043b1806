// The renderer behind the C ABI: device-resident scene and frame buffers, one CUDA stream, and the
// frame schedule of rustracer-renderer's Renderer (rustracer-renderer/src/lib.rs:227-1042).
//
// HBM layout per renderer (all cudaMalloc'd at create, freed at destroy):
//   scene:  triangles 128 B, materials 64 B, lights 64 B (AoS, the reference layouts); role textures
//           as rgba8 arrays (layer-major); the traversal layout derived from the reference's BVH:
//           one 64 B record per internal node, one 48 B leaf-ordered triangle record per prim slot.
//   path:   per pixel, origin / direction / throughput (16 B each), hit 8 B, accumulators 64 B,
//           first normal 16 B, two queue entries 4 B, one deferred shadow ray 48 B (192 B / pixel).
//   frame:  frame, denoise ping-pong, moments, gbuffer, accumulation (float4 per pixel each) and the
//           rgba8 output image.
//   photon: photon slots (64 B, 6 per photon), u32 key per slot, slot order, sorted photons (64 B),
//           counts / cursor / (start, count) per cell, scan partials.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <new>
#include <vector>

#include "rt_internal.h"
#include "rt_kernels.h"

using rt::set_error;

namespace {

#define RT_CK(call)                                                                                    \
    do {                                                                                               \
        cudaError_t e_ = (call);                                                                       \
        if (e_ != cudaSuccess) {                                                                       \
            set_error("%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, __LINE__);     \
            return e_ == cudaErrorMemoryAllocation ? RT_ERR_OUT_OF_MEMORY : RT_ERR_CUDA;               \
        }                                                                                              \
    } while (0)

struct DevBuf {
    void *p = nullptr;
    size_t bytes = 0;
    DevBuf() = default;
    DevBuf(const DevBuf &) = delete;
    DevBuf &operator=(const DevBuf &) = delete;
    ~DevBuf() { release(); }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
    }
    cudaError_t alloc(size_t n) {
        release();
        if (n == 0) n = 16;
        cudaError_t e = cudaMalloc(&p, n);
        if (e == cudaSuccess) bytes = n;
        else p = nullptr;
        return e;
    }
    template <class T>
    T *as() const {
        return reinterpret_cast<T *>(p);
    }
};

struct Events {
    cudaEvent_t ev[8] = {};
    ~Events() {
        for (auto &e : ev)
            if (e) cudaEventDestroy(e);
    }
    cudaError_t create() {
        for (auto &e : ev) {
            cudaError_t r = cudaEventCreate(&e);
            if (r != cudaSuccess) return r;
        }
        return cudaSuccess;
    }
};
enum { EV_FRAME0 = 0, EV_GATHER1, EV_DENOISE1, EV_RESOLVE1, EV_TRACE0, EV_TRACE1, EV_GRID1 };

}  // namespace

// Four events per frame (frame start, gather end, denoise end, resolve end), pooled; drained by
// rt_get_stats.
struct FrameEventRing {
    std::vector<cudaEvent_t> pool;
    size_t used = 0;  // events handed out since the last drain
    ~FrameEventRing() {
        for (auto e : pool) cudaEventDestroy(e);
    }
    cudaError_t next(cudaEvent_t *out) {
        if (used == pool.size()) {
            if (pool.size() >= (1u << 16)) {  // bounded: oldest timings are dropped past 16k frames
                *out = nullptr;
                return cudaSuccess;
            }
            cudaEvent_t e;
            cudaError_t r = cudaEventCreate(&e);
            if (r != cudaSuccess) return r;
            pool.push_back(e);
        }
        *out = pool[used++];
        return cudaSuccess;
    }
};

struct rt_renderer {
    int device = 0;
    cudaStream_t stream = nullptr;
    rt_render_config cfg{};
    rt_grid_params gp{};
    rt_camera_uniform cam{};
    std::vector<rt_light> lights_host;
    rtd::DevScene scene{};
    DevBuf d_cnodes, d_tri_ord, d_tris, d_mats, d_lights, d_tex[4];
    DevBuf d_frame, d_pingpong, d_moments, d_gbuffer, d_accum, d_output;
    // wavefront path state (one slot per pixel)
    DevBuf w_ro, w_rd, w_thr, w_hit, w_acc, w_nrm, w_queue[2], w_shadow, w_counts;
    size_t w_counts_bytes = 0;
    int num_sms = 1;
    DevBuf d_photons, d_keys, d_order, d_sorted, d_counts, d_meta, d_cursor, d_partials, d_total, d_counters;
    uint64_t photon_slots = 1;
    bool photon_buffers = false;
    uint32_t sample_counter = 0, frames_since_reset = 0;
    float marker[4] = {0, 0, 0, 0};
    float glow = 1.0f;
    uint64_t frames = 0;
    bool have_frame_timing = false, have_photon_timing = false;
    uint32_t last_denoise_passes = 0;
    Events events;
    FrameEventRing ring;
    ~rt_renderer() {
        if (stream) {
            cudaStreamSynchronize(stream);
            cudaStreamDestroy(stream);
        }
    }
};

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

extern "C" int rt_renderer_create(const rt_scene_desc *sd, const rt_render_config *cfg, rt_renderer **out) {
    rt::clear_error();
    if (!sd || !cfg || !out) {
        set_error("rt_renderer_create: null argument");
        return RT_ERR_INVALID_ARGUMENT;
    }
    *out = nullptr;
    if (cfg->width == 0 || cfg->height == 0 || (uint64_t)cfg->width * cfg->height > (1ull << 28)) {
        set_error("rt_renderer_create: width/height must be non-zero and width*height <= 2^28");
        return RT_ERR_INVALID_ARGUMENT;
    }
    if ((sd->triangle_count && !sd->triangles) || (sd->bvh_node_count && !sd->bvh_nodes) ||
        (sd->bvh_prim_count && !sd->bvh_prims) || (sd->material_count && !sd->materials) ||
        (sd->light_count && !sd->lights)) {
        set_error("rt_renderer_create: scene array pointer is null with a non-zero count");
        return RT_ERR_INVALID_ARGUMENT;
    }
    if (sd->bvh_node_count && (sd->triangle_count == 0 || sd->material_count == 0 || sd->bvh_prim_count == 0)) {
        set_error("rt_renderer_create: a BVH needs triangles, prim indices and at least one material");
        return RT_ERR_INVALID_ARGUMENT;
    }
    if (sd->triangle_count > 0xFFFFFFFFull || sd->bvh_node_count > 0xFFFFFFFFull || sd->bvh_prim_count > 0xFFFFFFFFull ||
        sd->material_count > 0xFFFFFFFFull || sd->light_count > 0xFFFFFFFFull) {
        set_error("rt_renderer_create: scene arrays are limited to 2^32 - 1 elements");
        return RT_ERR_INVALID_ARGUMENT;
    }
    if (rt_device_count() <= 0) {
        set_error("rt_renderer_create: no CUDA device is visible");
        return RT_ERR_CUDA;
    }
    rt_renderer *r = new (std::nothrow) rt_renderer();
    if (!r) {
        set_error("rt_renderer_create: out of host memory");
        return RT_ERR_OUT_OF_MEMORY;
    }
    auto fail = [&](int st) {
        delete r;
        return st;
    };
    int st;
    cudaGetDevice(&r->device);
    if (cudaStreamCreateWithFlags(&r->stream, cudaStreamNonBlocking) != cudaSuccess) {
        set_error("rt_renderer_create: cudaStreamCreate failed");
        return fail(RT_ERR_CUDA);
    }
    if (r->events.create() != cudaSuccess) {
        set_error("rt_renderer_create: cudaEventCreate failed");
        return fail(RT_ERR_CUDA);
    }
    r->cfg = *cfg;
    cudaStream_t s = r->stream;

    // Scene upload (Renderer::new, lib.rs:234-266).
    if ((st = upload(r->d_tris, sd->triangles, sd->triangle_count, s)) != RT_OK) return fail(st);
    rt::TraversalLayout lay;
    if (!rt::build_traversal_layout(sd->bvh_nodes, sd->bvh_node_count, sd->bvh_prims, sd->bvh_prim_count,
                                    sd->triangles, sd->triangle_count, lay))
        return fail(RT_ERR_INVALID_ARGUMENT);
    if ((st = upload(r->d_cnodes, lay.cnodes.data(), lay.cnodes.size(), s)) != RT_OK) return fail(st);
    if ((st = upload(r->d_tri_ord, lay.tri_ord.data(), lay.tri_ord.size(), s)) != RT_OK) return fail(st);
    // Host copies of the layout are freed when `lay` goes out of scope; wait for the copies first.
    RT_CK(cudaStreamSynchronize(s));
    if ((st = upload(r->d_mats, sd->materials, sd->material_count, s)) != RT_OK) return fail(st);
    if ((st = upload(r->d_lights, sd->lights, sd->light_count, s)) != RT_OK) return fail(st);
    r->lights_host.assign(sd->lights, sd->lights + sd->light_count);
    rtd::DevScene &ds = r->scene;
    ds.cnodes = r->d_cnodes.as<float4>();
    ds.tri_ord = r->d_tri_ord.as<float4>();
    ds.cnode_count = (uint32_t)(lay.cnodes.size() / 16);
    // A near-first traversal holds at most one pending entry per tree level.
    ds.stack_cap = lay.max_depth < 32u ? 32u : 63u;
    ds.any_hit_shadows = 1u;
    for (uint64_t i = 0; i < sd->material_count; ++i)
        if ((sd->materials[i].flags & RT_MAT_FLAG_ALPHA_CUTOUT) && sd->materials[i].tex_albedo != RT_TEX_NONE)
            ds.any_hit_shadows = 0u;
    ds.tris = r->d_tris.as<float4>();
    ds.mats = r->d_mats.as<float4>();
    ds.lights = r->d_lights.as<float4>();
    ds.tri_count = (uint32_t)sd->triangle_count;
    ds.mat_count = (uint32_t)sd->material_count;
    ds.light_count = (uint32_t)sd->light_count;
    const rt_texture_array *roles[4] = {&sd->tex_albedo, &sd->tex_mr, &sd->tex_emissive, &sd->tex_normal};
    for (int i = 0; i < 4; ++i) {
        const rt_texture_array &t = *roles[i];
        if (t.rgba8 && t.layers && t.width && t.height) {
            size_t bytes = (size_t)t.width * t.height * t.layers * 4;
            if ((st = upload(r->d_tex[i], t.rgba8, bytes, s)) != RT_OK) return fail(st);
            ds.tex[i] = rtd::DevTex{r->d_tex[i].as<uchar4>(), t.width, t.height, t.layers};
        } else {
            ds.tex[i] = rtd::DevTex{nullptr, 0, 0, 0};
        }
    }
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
    {
        DevBuf *wb[6] = {&r->w_ro, &r->w_rd, &r->w_thr, &r->w_nrm, &r->w_hit, &r->w_acc};
        const size_t wsz[6] = {16, 16, 16, 16, 8, 64};
        for (int i = 0; i < 6; ++i)
            if (wb[i]->alloc(npix * wsz[i]) != cudaSuccess) {
                set_error("rt_renderer_create: out of device memory for path state");
                return fail(RT_ERR_OUT_OF_MEMORY);
            }
        if (r->w_queue[0].alloc(npix * 4) != cudaSuccess || r->w_queue[1].alloc(npix * 4) != cudaSuccess ||
            r->w_shadow.alloc(npix * 48) != cudaSuccess) {
            set_error("rt_renderer_create: out of device memory for ray queues");
            return fail(RT_ERR_OUT_OF_MEMORY);
        }
    }
    r->num_sms = rtd::device_sm_count();
    RT_CK(r->d_output.alloc(npix * 4));
    RT_CK(cudaMemsetAsync(r->d_output.p, 0, npix * 4, s));
    RT_CK(r->d_counters.alloc(64));
    RT_CK(cudaMemsetAsync(r->d_counters.p, 0, 64, s));

    // Photon grid (lib.rs:276-286, 416-481).
    r->photon_buffers = cfg->enable_photon_map != 0;
    r->photon_slots = r->photon_buffers ? std::max<uint64_t>((uint64_t)cfg->photon_count * RT_MAX_BOUNCES, 1) : 1;
    if (r->photon_slots > 0xFFFFFFFFull) {
        set_error("rt_renderer_create: photon_count * 6 must fit in 32 bits");
        return fail(RT_ERR_INVALID_ARGUMENT);
    }
    float radius = cfg->photon_radius;
    rt_derive_grid(sd->bounds_min, sd->bounds_max, (int)sd->has_bounds, cfg->grid_max_dim, cfg->photon_radius_mode,
                   (uint32_t)r->photon_slots, &r->gp, &radius);
    r->cfg.photon_radius = radius;
    const uint64_t S = r->photon_slots, C = r->gp.num_cells;
    if (r->d_photons.alloc(S * 64) != cudaSuccess || r->d_sorted.alloc(S * 64) != cudaSuccess ||
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
    RT_CK(cudaMemsetAsync(r->d_keys.p, 0xFF, S * 4, s));
    RT_CK(cudaMemsetAsync(r->d_counts.p, 0, C * 4, s));
    RT_CK(cudaMemsetAsync(r->d_meta.p, 0, C * 8, s));
    RT_CK(cudaMemsetAsync(r->d_total.p, 0, 16, s));
    RT_CK(cudaStreamSynchronize(s));
    *out = r;
    return RT_OK;
}

extern "C" void rt_renderer_destroy(rt_renderer *r) { delete r; }

extern "C" int rt_render_frame(rt_renderer *r) {
    if (int st = check_renderer(r, "rt_render_frame")) return st;
    rt::clear_error();
    cudaStream_t s = r->stream;
    const rt_render_config &c = r->cfg;
    // lib.rs:672-684
    r->sample_counter += 1u;
    if (r->frames_since_reset != 0xFFFFFFFFu) r->frames_since_reset += 1u;
    const float alpha =
        c.accumulate_frames == 0 ? 1.0f : 1.0f / (float)std::min(r->frames_since_reset, c.accumulate_frames);
    const size_t npix = (size_t)c.width * c.height;

    cudaEvent_t fe[4] = {nullptr, nullptr, nullptr, nullptr};
    for (auto &e : fe) RT_CK(r->ring.next(&e));
    RT_CK(cudaEventRecord(r->events.ev[EV_FRAME0], s));
    if (fe[3]) RT_CK(cudaEventRecord(fe[0], s));
    const uint32_t spp = c.spp > 1u ? c.spp : 1u;
    const uint32_t iters = spp * max_bounces(c);
    const size_t counts_bytes = sizeof(uint32_t) * 4 * ((size_t)iters + 1);
    if (counts_bytes > r->w_counts_bytes) {
        RT_CK(cudaStreamSynchronize(s));
        RT_CK(r->w_counts.alloc(counts_bytes));
        r->w_counts_bytes = counts_bytes;
    }
    rtd::WaveParams wp;
    std::memset(&wp, 0, sizeof(wp));
    wp.scene = r->scene;
    wp.cam = r->cam;
    wp.ip = image_params(r, alpha);
    wp.gp = r->gp;
    wp.sorted_photons = r->d_sorted.as<float4>();
    wp.sorted_count = r->photon_slots;
    wp.grid_meta = r->d_meta.as<uint2>();
    wp.max_bounces = max_bounces(c);
    wp.npix = (uint32_t)npix;
    wp.ro = r->w_ro.as<float4>();
    wp.rd = r->w_rd.as<float4>();
    wp.thr = r->w_thr.as<float4>();
    wp.hit = r->w_hit.as<float2>();
    wp.acc = r->w_acc.as<float4>();
    wp.nrm = r->w_nrm.as<float4>();
    wp.queue[0] = r->w_queue[0].as<uint32_t>();
    wp.queue[1] = r->w_queue[1].as<uint32_t>();
    wp.counts = r->w_counts.as<uint32_t>();
    wp.shadow = r->w_shadow.as<float4>();
    wp.frame = r->d_frame.as<float4>();
    wp.moments = r->d_moments.as<float4>();
    wp.gbuffer = r->d_gbuffer.as<float4>();
    wp.counters = r->d_counters.as<unsigned long long>();
    RT_CK(rtd::launch_wavefront(wp, iters, r->num_sms, s));
    RT_CK(cudaEventRecord(r->events.ev[EV_GATHER1], s));
    if (fe[3]) RT_CK(cudaEventRecord(fe[1], s));

    // lib.rs:743-776: a-trous passes, steps 1, 2, ..., ping-pong frame <-> pingpong.
    float4 *result = r->d_frame.as<float4>();
    uint32_t passes = c.enable_denoise ? denoise_passes(c) : 0u;
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
        RT_CK(rtd::launch_denoise(in, o, r->d_gbuffer.as<float4>(), r->d_moments.as<float4>(), dp, s));
        result = o;
    }
    r->last_denoise_passes = passes;
    RT_CK(cudaEventRecord(r->events.ev[EV_DENOISE1], s));
    if (fe[3]) RT_CK(cudaEventRecord(fe[2], s));

    // lib.rs:778-831: composite, then tonemap.
    rt_tonemap_params tp;
    std::memset(&tp, 0, sizeof(tp));
    tp.exposure = c.exposure;
    tp.gamma = c.gamma;
    tp.width = c.width;
    tp.glow = r->glow;
    std::memcpy(tp.marker, r->marker, sizeof(tp.marker));
    RT_CK(rtd::launch_resolve(result, r->d_accum.as<float4>(), r->d_gbuffer.as<float4>(), c.width, c.height, alpha, tp,
                              r->d_output.as<uchar4>(), s));
    RT_CK(cudaEventRecord(r->events.ev[EV_RESOLVE1], s));
    if (fe[3]) RT_CK(cudaEventRecord(fe[3], s));
    (void)npix;
    r->frames += 1;
    r->have_frame_timing = true;
    return RT_OK;
}

extern "C" int rt_render_frames(rt_renderer *r, uint32_t n) {
    if (int st = check_renderer(r, "rt_render_frames")) return st;
    for (uint32_t i = 0; i < n; ++i)
        if (int st = rt_render_frame(r)) return st;
    return RT_OK;
}

extern "C" int rt_update_camera(rt_renderer *r, const rt_camera *cam) {
    if (int st = check_renderer(r, "rt_update_camera")) return st;
    if (!cam) {
        set_error("rt_update_camera: null camera");
        return RT_ERR_INVALID_ARGUMENT;
    }
    rt_camera_to_uniform(cam, r->cfg.width, r->cfg.height, &r->cam);
    return RT_OK;
}

extern "C" int rt_update_camera_uniform(rt_renderer *r, const rt_camera_uniform *u) {
    if (int st = check_renderer(r, "rt_update_camera_uniform")) return st;
    if (!u) {
        set_error("rt_update_camera_uniform: null uniform");
        return RT_ERR_INVALID_ARGUMENT;
    }
    r->cam = *u;
    return RT_OK;
}

extern "C" int rt_update_lights(rt_renderer *r, const rt_light *lights, uint64_t n) {
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
}

extern "C" int rt_reset_accumulation(rt_renderer *r, int hard) {
    if (int st = check_renderer(r, "rt_reset_accumulation")) return st;
    if (hard) RT_CK(cudaMemsetAsync(r->d_accum.p, 0, (size_t)r->cfg.width * r->cfg.height * 16, r->stream));
    r->frames_since_reset = 0;
    return RT_OK;
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
    g.scan_partials = r->d_partials.as<uint32_t>();
    g.total = r->d_total.as<uint32_t>();
    // Slots visited by the count/scatter dispatches of lib.rs:916,951,1026: floor(6P/256) groups of 256.
    const uint32_t P = std::max(r->cfg.photon_count, 1u);
    uint64_t dispatched = (uint64_t)std::max((uint32_t)(P * RT_MAX_BOUNCES) / 256u, 1u) * 256u;
    g.slot_count = std::min<uint64_t>(dispatched, r->photon_slots);
    RT_CK(rtd::launch_grid_build(g, r->stream));
    return RT_OK;
}

extern "C" int rt_rebuild_photons(rt_renderer *r) {
    if (int st = check_renderer(r, "rt_rebuild_photons")) return st;
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
    RT_CK(cudaEventRecord(r->events.ev[EV_TRACE0], s));
    RT_CK(rtd::launch_photon_trace(tp, s));
    RT_CK(cudaEventRecord(r->events.ev[EV_TRACE1], s));
    if (int st = build_grid(r)) return st;
    RT_CK(cudaEventRecord(r->events.ev[EV_GRID1], s));
    RT_CK(cudaStreamSynchronize(s));
    r->have_photon_timing = true;
    return RT_OK;
}

extern "C" int rt_load_photons_and_build_grid(rt_renderer *r, const rt_photon *photons, uint64_t n) {
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
}

extern "C" int rt_set_config(rt_renderer *r, const rt_render_config *c) {
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
}

extern "C" int rt_get_config(const rt_renderer *r, rt_render_config *c) {
    if (int st = check_renderer(r, "rt_get_config")) return st;
    if (!c) return RT_ERR_INVALID_ARGUMENT;
    *c = r->cfg;
    return RT_OK;
}

extern "C" int rt_set_light_marker(rt_renderer *r, const float marker[4], float glow) {
    if (int st = check_renderer(r, "rt_set_light_marker")) return st;
    if (marker) std::memcpy(r->marker, marker, sizeof(r->marker));
    else std::memset(r->marker, 0, sizeof(r->marker));
    r->glow = glow;
    return RT_OK;
}

extern "C" uint32_t rt_sample_count(const rt_renderer *r) { return r ? r->sample_counter : 0u; }

extern "C" int rt_synchronize(rt_renderer *r) {
    if (int st = check_renderer(r, "rt_synchronize")) return st;
    RT_CK(cudaStreamSynchronize(r->stream));
    return RT_OK;
}

extern "C" void *rt_renderer_stream(rt_renderer *r) { return r ? (void *)r->stream : nullptr; }

extern "C" int rt_get_grid_params(const rt_renderer *r, rt_grid_params *out) {
    if (int st = check_renderer(r, "rt_get_grid_params")) return st;
    if (!out) return RT_ERR_INVALID_ARGUMENT;
    *out = r->gp;
    return RT_OK;
}

extern "C" int rt_get_stats(rt_renderer *r, rt_frame_stats *out) {
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
    return r ? read_back(r, r->d_accum, rgba, n * 4, RT_IMG_BYTES(r), "rt_read_accumulation")
             : check_renderer(r, "rt_read_accumulation");
}
extern "C" int rt_read_frame(rt_renderer *r, float *rgba, uint64_t n) {
    if (!r) return check_renderer(r, "rt_read_frame");
    // The frame as composite consumed it (after the denoise passes, if any).
    const DevBuf &b = (r->last_denoise_passes % 2 == 1) ? r->d_pingpong : r->d_frame;
    return read_back(r, b, rgba, n * 4, RT_IMG_BYTES(r), "rt_read_frame");
}
extern "C" int rt_read_moments(rt_renderer *r, float *rgba, uint64_t n) {
    return r ? read_back(r, r->d_moments, rgba, n * 4, RT_IMG_BYTES(r), "rt_read_moments")
             : check_renderer(r, "rt_read_moments");
}
extern "C" int rt_read_gbuffer(rt_renderer *r, float *rgba, uint64_t n) {
    return r ? read_back(r, r->d_gbuffer, rgba, n * 4, RT_IMG_BYTES(r), "rt_read_gbuffer")
             : check_renderer(r, "rt_read_gbuffer");
}
extern "C" int rt_read_tonemapped(rt_renderer *r, uint8_t *rgba8, uint64_t n) {
    return r ? read_back(r, r->d_output, rgba8, n, RT_IMG_BYTES(r) / 4, "rt_read_tonemapped")
             : check_renderer(r, "rt_read_tonemapped");
}
extern "C" int rt_read_photons(rt_renderer *r, rt_photon *out, uint64_t n) {
    return r ? read_back(r, r->d_photons, out, n * 64, r->photon_slots * 64, "rt_read_photons")
             : check_renderer(r, "rt_read_photons");
}
extern "C" int rt_read_sorted_photons(rt_renderer *r, rt_photon *out, uint64_t n) {
    return r ? read_back(r, r->d_sorted, out, n * 64, r->photon_slots * 64, "rt_read_sorted_photons")
             : check_renderer(r, "rt_read_sorted_photons");
}
extern "C" int rt_read_photon_grid(rt_renderer *r, uint32_t *counts, uint32_t *meta, uint64_t num_cells) {
    if (int st = check_renderer(r, "rt_read_photon_grid")) return st;
    if (num_cells < r->gp.num_cells) {
        set_error("rt_read_photon_grid: %llu cells given, the grid has %u", (unsigned long long)num_cells,
                  r->gp.num_cells);
        return RT_ERR_INVALID_ARGUMENT;
    }
    if (counts) {
        if (int st = read_back(r, r->d_counts, counts, num_cells * 4, (uint64_t)r->gp.num_cells * 4, "rt_read_photon_grid"))
            return st;
    }
    if (meta) {
        if (int st = read_back(r, r->d_meta, meta, num_cells * 8, (uint64_t)r->gp.num_cells * 8, "rt_read_photon_grid"))
            return st;
    }
    return RT_OK;
}

// ================================================================================================
// Stage entry points (host buffers in and out; the default stream; temporaries freed on return)
// ================================================================================================
extern "C" int rt_stage_denoise(const float *frame_rgba, const float *gbuffer, const float *moments, uint32_t width,
                                uint32_t height, float alpha, uint32_t passes, float *out_rgba) {
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
        RT_CK(rtd::launch_denoise(cur, nxt, g.as<float4>(), m.as<float4>(), dp, 0));
        std::swap(cur, nxt);
    }
    RT_CK(cudaMemcpy(out_rgba, cur, bytes, cudaMemcpyDeviceToHost));
    return RT_OK;
}

extern "C" int rt_stage_resolve(const float *frame_rgba, float *accum_inout, const float *gbuffer, uint32_t width,
                                uint32_t height, float alpha, const rt_tonemap_params *tp, uint8_t *out_rgba8) {
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
    RT_CK(rtd::launch_resolve(f.as<float4>(), a.as<float4>(), gp, width, height, alpha, t, o.as<uchar4>(), 0));
    RT_CK(cudaMemcpy(accum_inout, a.p, bytes, cudaMemcpyDeviceToHost));
    RT_CK(cudaMemcpy(out_rgba8, o.p, bytes / 4, cudaMemcpyDeviceToHost));
    return RT_OK;
}

extern "C" int rt_stage_photon_grid(const rt_photon *photons, const rt_grid_params *gpp, uint32_t *counts,
                                    uint32_t *meta, rt_photon *sorted) {
    rt::clear_error();
    if (!photons || !gpp || !counts || !meta || !sorted || gpp->num_cells == 0) {
        set_error("rt_stage_photon_grid: invalid arguments");
        return RT_ERR_INVALID_ARGUMENT;
    }
    const rt_grid_params gp = *gpp;
    const uint64_t S = gp.photon_slots, C = gp.num_cells;
    DevBuf ph, keys, order, srt, cnt, cur, mt, part, tot;
    RT_CK(ph.alloc(S * 64));
    RT_CK(keys.alloc(S * 4));
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
    g.scan_partials = part.as<uint32_t>();
    g.total = tot.as<uint32_t>();
    RT_CK(rtd::launch_grid_build(g, 0));
    RT_CK(cudaMemcpy(counts, cnt.p, C * 4, cudaMemcpyDeviceToHost));
    RT_CK(cudaMemcpy(meta, mt.p, C * 8, cudaMemcpyDeviceToHost));
    if (S) RT_CK(cudaMemcpy(sorted, srt.p, S * 64, cudaMemcpyDeviceToHost));
    return RT_OK;
}

