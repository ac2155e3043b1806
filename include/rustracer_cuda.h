/*
 * rustracer_cuda.h — C ABI of the GB300 (sm_103a) backend for rustracer's per-frame hot path.
 *
 * The ABI replaces the Rust `rustracer-renderer` frame API (rustracer-renderer/src/lib.rs) with
 * plain `extern "C"` entry points over POD structs.  Every GPU-visible struct keeps the byte layout
 * of the reference's `#[repr(C)]` type (which itself mirrors the WGSL structs in
 * rustracer-renderer/shaders/common.wgsl); the sizes and offsets are pinned by static asserts in
 * rt_layout_check.h and by the CPU test-suite.
 *
 * Conventions
 *   - Every fallible call returns an `int` status (RT_OK == 0).  On failure a thread-local message is
 *     available through rt_last_error().  No C++ exception crosses the ABI.
 *   - One rt_renderer owns every device buffer it uses and one CUDA stream.  A renderer is not
 *     thread-safe; distinct renderers may be driven from distinct host threads.
 *   - Host pointers passed in are only read during the call (the scene is copied to the device by
 *     rt_renderer_create, just as Renderer::new copies the borrowed &Scene).
 *   - Calls that enqueue GPU work return once it is enqueued; rt_synchronize() and every rt_read_*
 *     call wait for it (the reference's `device.poll(Maintain::Wait)`).
 */
#ifndef RUSTRACER_CUDA_H
#define RUSTRACER_CUDA_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------------------------------------
 * Status codes
 * ------------------------------------------------------------------------------------------- */
#define RT_OK 0
#define RT_ERR_INVALID_ARGUMENT 1 /* bad pointer, size or value                                 */
#define RT_ERR_CUDA 2             /* a CUDA runtime call failed (message says which)             */
#define RT_ERR_OUT_OF_MEMORY 3    /* a device or host allocation failed, or an admission cap hit */
#define RT_ERR_STATE 4            /* call not valid in the renderer's current state              */
#define RT_ERR_DEVICE_CHECK 5     /* a kernel's own bounds/timeout check fired (no fault raised) */

/* ---------------------------------------------------------------------------------------------
 * Constants shared with the reference (rustracer-core/src/material.rs:7-10,
 * rustracer-renderer/src/lib.rs:15-19)
 * ------------------------------------------------------------------------------------------- */
#define RT_TEX_NONE 0xFFFFFFFFu
#define RT_MAT_FLAG_ALPHA_CUTOUT 1u
#define RT_MAX_BOUNCES 6u    /* reference MAX_BOUNCES; camera and photon paths               */
#define RT_GRID_MAX_DIM 26u  /* reference GRID_MAX_DIM (photon grid cells per axis, maximum) */

enum rt_material_kind { RT_MAT_LAMBERTIAN = 0, RT_MAT_METAL = 1, RT_MAT_DIELECTRIC = 2, RT_MAT_EMISSIVE = 3 };
enum rt_light_kind { RT_LIGHT_POINT = 0, RT_LIGHT_DIRECTIONAL = 1, RT_LIGHT_AREA = 2, RT_LIGHT_ENVIRONMENT = 3 };
enum rt_texture_role { RT_TEX_ALBEDO = 0, RT_TEX_MR = 1, RT_TEX_EMISSIVE = 2, RT_TEX_NORMAL = 3 };

/* ---------------------------------------------------------------------------------------------
 * GPU layouts (little-endian, 4-byte fields)
 * ------------------------------------------------------------------------------------------- */

/* rustracer-core/src/bvh.rs:79-88 (BVHNode, 48 B).  Leaf: prim_count > 0, left_first = first slot in
 * the prim-index array.  Internal: prim_count == 0, left_first / right_child = child node indices. */
typedef struct rt_bvh_node {
    float bbox_min[3];
    uint32_t left_first;
    float bbox_max[3];
    uint32_t right_child;
    uint32_t prim_count;
    float _pad[3];
} rt_bvh_node;

/* rustracer-core/src/scene.rs:74-94 (TriangleGpu, 128 B). */
typedef struct rt_triangle {
    float v0[3]; float _pad0;
    float v1[3]; float _pad1;
    float v2[3]; float _pad2;
    float n0[3]; float _pad3;
    float n1[3]; float _pad4;
    float n2[3]; float _pad5;
    float uv0[2]; float uv1[2]; float uv2[2];
    uint32_t material_id;
    float _pad6;
} rt_triangle;

/* rustracer-core/src/material.rs:44-58 (MaterialGpu, 64 B). */
typedef struct rt_material {
    float albedo[4];
    float emissive[3];
    float roughness;
    float metallic;
    float ior;
    uint32_t kind;
    uint32_t flags;
    uint32_t tex_albedo;
    uint32_t tex_mr;
    uint32_t tex_emissive;
    uint32_t tex_normal;
} rt_material;

/* rustracer-core/src/scene.rs:141-150 (LightGpu, 64 B).  data: point = position, directional =
 * direction, area = (triangle index as f32, 0, 0, 0), environment = horizon colour. */
typedef struct rt_light {
    float data[4];
    float color[3];
    float intensity;
    uint32_t kind;
    float _pad_a[3];
    float _pad_b[4];
} rt_light;

/* rustracer-core/src/camera.rs:257-274 (CameraUniform, 96 B). */
typedef struct rt_camera_uniform {
    float position[3]; float _pad0;
    float forward[3]; float _pad1;
    float right[3]; float _pad2;
    float up[3]; float _pad3;
    float inv_half_res[2];
    float near_plane;
    float fov_scale;
    float aperture;
    float focus_dist;
    float _pad_end[2];
} rt_camera_uniform;

/* rustracer-renderer/src/lib.rs:86-97 (PhotonGpu, 64 B). */
typedef struct rt_photon {
    float position[3]; float _pad0;
    float power[3]; float _pad1;
    float incident[3]; float _pad2;
    float normal[3]; float _pad3;
} rt_photon;

/* rustracer-renderer/src/lib.rs:67-84 (ImageParams, 80 B).  _pad[0] carries debug_view. */
typedef struct rt_image_params {
    uint32_t width, height, spp, frame;
    float light_emission[3];
    float ambient;
    float accumulate_alpha;
    uint32_t use_photons;
    uint32_t photon_count;
    float photon_radius;
    float photon_scale;
    uint32_t photon_debug;
    float point_light_emission[3];
    uint32_t _pad[3];
} rt_image_params;

/* rustracer-renderer/src/lib.rs:137-150 (GridParamsUniform, 48 B). */
typedef struct rt_grid_params {
    float room_min_x, room_min_y, room_min_z;
    float cell_size;
    uint32_t grid_x, grid_y, grid_z;
    uint32_t num_cells;
    uint32_t photon_slots;
    uint32_t _pad[3];
} rt_grid_params;

/* rustracer-renderer/src/lib.rs:113-124 (DenoiseParamsUniform, 32 B). */
typedef struct rt_denoise_params {
    uint32_t width, height, step_size;
    float lambda, phi_normal, phi_depth, alpha;
    uint32_t _pad;
} rt_denoise_params;

/* rustracer-renderer/src/lib.rs:126-133 (CompositeParams, 16 B). */
typedef struct rt_composite_params {
    uint32_t width, height;
    float alpha;
    uint32_t _pad;
} rt_composite_params;

/* rustracer-renderer/src/lib.rs:99-111 (ToneMapUniform, 32 B).  marker = (x_px, y_px, r_px, dist),
 * dist == 0 hides the light gizmo. */
typedef struct rt_tonemap_params {
    float exposure, gamma;
    uint32_t width;
    float glow;
    float marker[4];
} rt_tonemap_params;

/* ---------------------------------------------------------------------------------------------
 * Host-side descriptions
 * ------------------------------------------------------------------------------------------- */

/* rustracer-core/src/camera.rs:7-16 (Camera). */
typedef struct rt_camera {
    float position[3];
    float look_at[3];
    float up[3];
    float fov_degrees;
    float near_plane;
    float aperture;
    float focus_dist;
} rt_camera;

/* rustracer-renderer/src/lib.rs:21-65 (RenderConfig) plus extensions.  Extensions default to the
 * reference's behaviour when zero. */
typedef struct rt_render_config {
    uint32_t width, height;
    uint32_t photon_count;
    uint32_t spp;
    float exposure, gamma;
    float light_emission[3];
    float point_light_emission[3];
    uint32_t accumulate_frames; /* 0 = overwrite, N = running mean over N frames            */
    uint32_t enable_photon_map;
    uint32_t enable_denoise;
    uint32_t photon_debug;
    uint32_t debug_view;
    float photon_scale;
    float photon_radius;        /* overwritten at create from the photon grid (lib.rs:431)  */
    float ambient;
    /* extensions (0 = reference behaviour) */
    uint32_t max_bounces;       /* camera path depth; 0 -> RT_MAX_BOUNCES                   */
    uint32_t grid_max_dim;      /* photon grid cells per axis cap; 0 -> RT_GRID_MAX_DIM     */
    uint32_t photon_radius_mode;/* 0: clamp(4*cell, .01, 2) (reference); 1: cell / 2         */
    uint32_t denoise_passes;    /* a-trous passes (steps 1,2,4,..); 0 -> 2 (reference)       */
} rt_render_config;

/* One role texture array: `layers` RGBA8 images of width x height, layer-major, row-major
 * (rustracer-renderer/src/lib.rs:1286-1358).  rgba8 == NULL or layers == 0 means an empty role
 * (bound as one zero texel, as the reference's 1x1x1 placeholder). */
typedef struct rt_texture_array {
    const uint8_t *rgba8;
    uint32_t width, height, layers, _pad;
} rt_texture_array;

/* Everything Renderer::new uploads (rustracer-renderer/src/lib.rs:234-266, 501-507) plus the scene
 * bounds it derives the photon grid from (lib.rs:418-420). */
typedef struct rt_scene_desc {
    const rt_triangle *triangles;  uint64_t triangle_count;
    const rt_bvh_node *bvh_nodes;  uint64_t bvh_node_count;
    const uint32_t *bvh_prims;     uint64_t bvh_prim_count;
    const rt_material *materials;  uint64_t material_count;
    const rt_light *lights;        uint64_t light_count;
    rt_texture_array tex_albedo, tex_mr, tex_emissive, tex_normal;
    float bounds_min[3];
    float bounds_max[3];
    uint32_t has_bounds;           /* 0: the reference's default (-1.05 .. 1.05)                */
    uint32_t _pad;
} rt_scene_desc;

/* Per-frame counters and device timings (CUDA events on the renderer's stream). */
typedef struct rt_frame_stats {
    uint64_t frames;             /* frames rendered since create                              */
    uint64_t segments;           /* closest-hit traces on camera/bounce paths since create    */
    uint64_t shadow_rays;        /* shadow traces (NEE) since create                          */
    uint64_t photons_stored;     /* valid photon slots after the last rebuild                  */
    float ms_gather;             /* last frame, gather kernel                                 */
    float ms_denoise;            /* last frame, all denoise passes                            */
    float ms_resolve;            /* last frame, composite + tonemap                           */
    float ms_frame;              /* last frame, whole frame                                   */
    float ms_photon_trace;       /* last rebuild                                              */
    float ms_grid_build;         /* last rebuild: keys, count, scan, scatter, order           */
    /* Sums over the frames rendered since the previous rt_get_stats call (that call resets them). */
    uint64_t timed_frames;
    double ms_gather_sum;
    double ms_denoise_sum;
    double ms_resolve_sum;
    double ms_frame_sum;
    uint64_t graph_captures;     /* batches: CUDA graphs captured so far                      */
} rt_frame_stats;

/* ---------------------------------------------------------------------------------------------
 * Errors and version
 * ------------------------------------------------------------------------------------------- */
const char *rt_last_error(void);
const char *rt_version(void);
/* Number of CUDA devices visible to the library (0 when none). */
int rt_device_count(void);

/* ---------------------------------------------------------------------------------------------
 * Renderer (rustracer-renderer/src/lib.rs:189-1042)
 * ------------------------------------------------------------------------------------------- */
typedef struct rt_renderer rt_renderer;

/* RenderConfig::default() (lib.rs:44-65). */
void rt_render_config_default(rt_render_config *cfg);

/* Renderer::new (lib.rs:227-663): uploads the scene, allocates frame buffers, derives the photon
 * grid (lib.rs:416-457) and writes the derived photon_radius back into the renderer's config. */
int rt_renderer_create(const rt_scene_desc *scene, const rt_render_config *cfg, rt_renderer **out);
/* Waits for the renderer's own stream (which every batch frame it took part in joins) and frees its
 * buffers into the device's renderer memory pool, without synchronising the device; the pool returns
 * its memory to the device when the last renderer on it is destroyed. */
void rt_renderer_destroy(rt_renderer *r);

/* Resident scenes (no counterpart in the reference, where each Renderer::new uploads its own copy):
 * a scene's geometry, traversal layout, materials and textures uploaded once and shared by every
 * renderer created on it.  Lights stay per renderer (rt_update_lights changes one renderer's copy).
 * A resident scene is reference-counted: create returns one reference, each renderer on it holds
 * one, and the device memory is freed with the last.  rt_renderer_create is create-resident +
 * create-on + release. */
typedef struct rt_resident_scene rt_resident_scene;
int rt_resident_scene_create(const rt_scene_desc *scene, rt_resident_scene **out);
void rt_resident_scene_release(rt_resident_scene *s);
uint64_t rt_resident_scene_bytes(const rt_resident_scene *s);   /* device bytes held             */
uint32_t rt_resident_scene_refs(const rt_resident_scene *s);    /* references (caller's + renderers') */
int rt_renderer_create_resident(rt_resident_scene *s, const rt_render_config *cfg, rt_renderer **out);
/* Device bytes the renderer owns now (frame, photon and path buffers; its scene not included). */
uint64_t rt_renderer_device_bytes(const rt_renderer *r);
/* Device bytes a renderer with this config on this scene allocates at create, and (optional) the
 * path state and job table its first solo frame adds (a photon rebuild adds the job table alone);
 * for admission by footprint before creating it. */
int rt_renderer_footprint(const rt_render_config *cfg, const rt_resident_scene *s, uint64_t *create_bytes,
                          uint64_t *solo_path_bytes);

/* record_frame (lib.rs:666-851) minus the swapchain blit: gather -> [denoise x passes] ->
 * composite -> tonemap into the renderer's RGBA8 output buffer. */
int rt_render_frame(rt_renderer *r);
/* n successive record_frame calls. */
int rt_render_frames(rt_renderer *r, uint32_t n);

/* update_camera (lib.rs:853-857): Camera::to_uniform at the renderer's resolution. */
int rt_update_camera(rt_renderer *r, const rt_camera *cam);
/* Writes an already-built camera uniform. */
int rt_update_camera_uniform(rt_renderer *r, const rt_camera_uniform *u);
/* update_lights (lib.rs:888-891): overwrites the first n lights; n must not exceed the light count
 * given at create (the light buffer keeps its size, as the reference's does). */
int rt_update_lights(rt_renderer *r, const rt_light *lights, uint64_t n);
/* reset_accumulation (hard != 0: zero the history, lib.rs:893-902) or
 * reset_accumulation_soft (hard == 0: next frame overwrites, lib.rs:907-909). */
int rt_reset_accumulation(rt_renderer *r, int hard);
/* rebuild_photons (lib.rs:913-1037): photon trace, then the exact u32 counting sort of the slots
 * into the uniform grid (keys, histogram, device exclusive scan, scatter in slot order). */
int rt_rebuild_photons(rt_renderer *r);
/* Mutates the renderer's config (callers mutate `renderer.config` directly in the reference,
 * rustracer-app/src/main.rs:447,505).  width, height and photon_count cannot change. */
int rt_set_config(rt_renderer *r, const rt_render_config *cfg);
int rt_get_config(const rt_renderer *r, rt_render_config *cfg);
/* The light-gizmo marker of the tonemap pass (lib.rs:704-717): x_px, y_px, r_px, camera distance. */
int rt_set_light_marker(rt_renderer *r, const float marker[4], float glow);

/* sample_count (lib.rs:1039-1041). */
uint32_t rt_sample_count(const rt_renderer *r);
/* Accumulation checkpoint and resume (no counterpart in the reference; its raw dump is
 * render_headless.rs:141-147, the accumulation as W*H*4 f32).  A checkpoint is that dump plus the two
 * frame counters of rt_get_frame_state (sample_counter = rt_sample_count, frames accumulated since
 * the last reset).  rt_restore_accumulation writes them back into a renderer of the same
 * configuration, scene and camera (and, with a photon map, after the same rebuild): the frames it
 * renders next are the frames the checkpointed renderer would have rendered. */
int rt_get_frame_state(const rt_renderer *r, uint32_t *sample_counter, uint32_t *frames_since_reset);
int rt_restore_accumulation(rt_renderer *r, const float *rgba, uint64_t n_floats, uint32_t sample_counter,
                            uint32_t frames_since_reset);
int rt_synchronize(rt_renderer *r);
/* Waits for the renderer's stream.  Per-kernel sums cover the frames since the previous call. */
int rt_get_stats(rt_renderer *r, rt_frame_stats *out);
int rt_get_grid_params(const rt_renderer *r, rt_grid_params *out);

/* Kernel-level profile of the gather pass (no counterpart in the reference, whose frame is one
 * megakernel dispatch).  With RT_PROFILE_EVENTS set, every later rt_render_frame records CUDA events
 * around each launch of the traversal, shade and photon-lookup kernels and waits for its frame; with
 * RT_PROFILE_COUNT it runs the counting variants of the traversal kernels (same rays and results),
 * which add the records each kind of ray visits and its leaf triangle tests.  Images are unchanged
 * either way.  rt_read_profile returns the sums over the profiled frames since the previous read and
 * resets them; rt_set_profiling(r, 0) stops profiling. */
#define RT_PROFILE_EVENTS 1u
#define RT_PROFILE_COUNT 2u
typedef struct rt_trace_profile {
    uint64_t frames;                 /* profiled frames summed here                               */
    uint64_t trace_launches, shade_launches, photon_launches;
    double ms_trace, ms_shade, ms_photon;   /* device time of those launches (RT_PROFILE_EVENTS) */
    double ms_gather;                /* whole gather passes of the profiled frames               */
    uint64_t closest_rays, occlusion_rays;  /* closest-hit (path segment) and occlusion rays       */
    uint64_t records_closest, records_occlusion;      /* traversal records visited (RT_PROFILE_COUNT) */
    uint64_t tri_tests_closest, tri_tests_occlusion;  /* leaf triangle tests (RT_PROFILE_COUNT)      */
    uint32_t record_bytes;           /* bytes of one traversal record: 128 four-wide, 64 two-wide */
    uint32_t pixels;                 /* pixels of one frame                                       */
} rt_trace_profile;
int rt_set_profiling(rt_renderer *r, uint32_t flags);
int rt_read_profile(rt_renderer *r, rt_trace_profile *out);
/* The renderer's CUDA stream (a cudaStream_t), for callers that time or order work on it. */
void *rt_renderer_stream(rt_renderer *r);

/* Read-backs (device -> host, synchronous).  Sizes are element counts of the destination. */
int rt_read_accumulation(rt_renderer *r, float *rgba, uint64_t n_floats);  /* W*H*4 */
int rt_read_frame(rt_renderer *r, float *rgba, uint64_t n_floats);         /* W*H*4 */
int rt_read_moments(rt_renderer *r, float *rgba, uint64_t n_floats);       /* W*H*4 */
int rt_read_gbuffer(rt_renderer *r, float *rgba, uint64_t n_floats);       /* W*H*4 */
int rt_read_tonemapped(rt_renderer *r, uint8_t *rgba8, uint64_t n_bytes);  /* W*H*4 */
int rt_read_photons(rt_renderer *r, rt_photon *out, uint64_t n);           /* photon_slots */
int rt_read_sorted_photons(rt_renderer *r, rt_photon *out, uint64_t n);    /* photon_slots */
/* counts: num_cells u32; meta: num_cells (start, count) pairs (either may be null).  The counts are
 * the pairs' second members (the device count buffer is cleared by the build once scanned). */
int rt_read_photon_grid(rt_renderer *r, uint32_t *counts, uint32_t *meta, uint64_t num_cells);
/* Replaces the traced photon slots (n == photon_slots) and rebuilds the grid from them, skipping the
 * trace: lets a caller feed an identical photon buffer to this backend and to another one. */
int rt_load_photons_and_build_grid(rt_renderer *r, const rt_photon *photons, uint64_t n);

/* ---------------------------------------------------------------------------------------------
 * Batched rendering (no counterpart in the reference, which renders one job per device): one call
 * renders the next progressive frame of several renderers at once, the rays of every job sharing the
 * same wavefront launches.  A job's image is identical alone and in a batch.  The renderers stay owned
 * by the caller and must outlive the batch; do not render them alone while a batch frame is queued
 * (read-backs on a renderer wait for the batch's work).  use_graphs != 0 captures each batch frame as
 * a CUDA graph, replayed with the per-frame values (frame counters, cameras) read from device memory
 * and captured again only when the launches' shape or baked settings change.
 * ------------------------------------------------------------------------------------------- */
typedef struct rt_batch rt_batch;
/* Launch shape of the persistent traversal kernels (closest-hit and shadow rays).  It changes only
 * speed, never a result.  Fields outside the supported set are clamped: block_threads 64 / 128 /
 * 256, blocks_per_sm up to 2048 / block_threads, chunk (queue items a warp takes per atomic, its
 * segment of the shared queue) 32 .. 1024 in steps of 32, steps (traversal records between lane
 * refills) 1 .. 64, stack_entries 32 / 48 / 64 per lane, raised to what the jobs' trees need.
 * Default: 128 threads, 8 blocks per SM, chunk 32, 3 steps, 32 entries, no treelet, shade_blocks 6,
 * refill_idle 0. */
typedef struct rt_wavefront_tuning {
    uint32_t block_threads, blocks_per_sm, chunk, steps, stack_entries;
    uint32_t treelet;       /* 1: the top records of the four-wide tree are staged in shared memory */
    uint32_t shade_blocks;  /* shade kernel's register budget: 4, 5 or 6 resident blocks per SM (other
                             * values: 6) */
    uint32_t refill_idle;   /* refill a warp's idle lanes before `steps` records once this many are idle
                             * (0: after `steps` only) */
} rt_wavefront_tuning;
int rt_batch_create(rt_renderer *const *renderers, uint32_t n, uint32_t use_graphs, rt_batch **out);
void rt_batch_destroy(rt_batch *b);
int rt_batch_render_frame(rt_batch *b);
int rt_batch_render_frames(rt_batch *b, uint32_t n);
int rt_batch_synchronize(rt_batch *b);
/* frames, segments / shadow rays of all jobs (cumulative), graph_captures; ms_frame_sum and
 * timed_frames cover the batch frames since the previous call. */
int rt_batch_get_stats(rt_batch *b, rt_frame_stats *out);
void *rt_batch_stream(rt_batch *b);
int rt_batch_set_tuning(rt_batch *b, const rt_wavefront_tuning *t);
int rt_batch_get_tuning(rt_batch *b, rt_wavefront_tuning *t);
/* The autotuner: renders trial frames of the batch under candidate launch shapes (coordinate
 * descent over block shape, blocks per SM, stack depth, chunk size and refill steps; trial_frames
 * frames per candidate, timed with CUDA events) and keeps the fastest.  The trial frames are undone
 * -- every job's image buffers and frame counters are restored -- so the frames rendered afterwards
 * are the ones that would have been rendered without tuning.  best / best_ms may be null. */
int rt_batch_autotune(rt_batch *b, uint32_t trial_frames, rt_wavefront_tuning *best, float *best_ms);
/* The same launch shape for a renderer's own frames (rt_render_frame). */
int rt_set_tuning(rt_renderer *r, const rt_wavefront_tuning *t);
int rt_get_tuning(const rt_renderer *r, rt_wavefront_tuning *t);

/* ---------------------------------------------------------------------------------------------
 * The render-request loop (no counterpart in the reference, which renders one job per process):
 * headless jobs of registered scenes are submitted as they arrive and rendered to their
 * accumulation budgets by one worker thread that owns the server's CUDA work.
 *   - RT_SERVER_BATCHED: continuous batching.  Every admitted job whose set-up is done is a member
 *     of the next batch frame (rt_batch semantics); jobs join and leave between frames.  Jobs are
 *     admitted in arrival order while max_jobs, max_slots (summed pixels) and hbm_cap_bytes allow.
 *   - RT_SERVER_PLAIN: the same loop with one job at a time, rendered frame by frame alone with the
 *     launches of rt_render_frame (max_jobs = 1, no graphs).
 * A job's scene is uploaded on first use and stays resident after its jobs finish; when the cap
 * would be exceeded, idle resident scenes (no admitted job) are freed least recently used first.
 * The device bytes charged against the cap are the resident scenes, the admitted jobs' renderer
 * buffers and the path state (max_slots x 240 B, reserved at create).  A job's image equals
 * the image of the same request rendered alone by rt_renderer_create + rt_render_frame.
 * Registered scene descriptions are borrowed: their arrays must stay valid and unchanged until
 * rt_server_destroy.  submit / status / read_result / release / stats may be called from any thread.
 * Times are milliseconds on the server's steady clock (0 at create); -1 where not reached yet.
 * ------------------------------------------------------------------------------------------- */
#define RT_SERVER_BATCHED 0u
#define RT_SERVER_PLAIN 1u
#define RT_JOB_QUEUED 0u
#define RT_JOB_RUNNING 1u
#define RT_JOB_DONE 2u
#define RT_JOB_FAILED 3u

typedef struct rt_server rt_server;
typedef struct rt_server_config {
    uint64_t hbm_cap_bytes;     /* 0: 120 GiB                                                    */
    uint32_t max_jobs;          /* jobs rendered together (batched mode), 0: 64                   */
    uint32_t max_slots;         /* summed pixels of the jobs rendered together, 0: 2^25           */
    uint32_t mode;              /* RT_SERVER_BATCHED or RT_SERVER_PLAIN                            */
    uint32_t graphs;            /* batched mode: capture a batch frame whose shape repeats        */
    uint32_t frames_in_flight;  /* frames queued on the GPU ahead of the host, 0: 2               */
    uint32_t _pad;
    rt_wavefront_tuning tuning; /* launch shape of the batch frames; all zero: the default        */
} rt_server_config;
typedef struct rt_request {
    uint32_t scene_id;          /* as registered with rt_server_add_scene                         */
    uint32_t budget_frames;     /* progressive frames to render (>= 1)                            */
    uint32_t keep_result;       /* keep the final accumulation for rt_server_read_result          */
    uint32_t _pad;
    rt_render_config config;
    rt_camera camera;
} rt_request;
typedef struct rt_job_status {
    uint64_t job_id;
    uint32_t state;             /* RT_JOB_*                                                        */
    uint32_t frames_done;
    double t_submit_ms, t_admit_ms, t_first_frame_ms, t_done_ms;
} rt_job_status;
typedef struct rt_server_stats {
    uint64_t submitted, admitted, completed, failed;
    uint64_t batch_frames;      /* frames launched (a batch frame counts once)                    */
    uint64_t job_frames;        /* frames finished, summed over jobs                              */
    uint64_t segments, shadow_rays;
    uint64_t scene_uploads, scene_evictions, graph_captures;
    uint64_t used_bytes, peak_bytes, resident_scene_bytes;
    uint32_t active, pending, resident_scenes, max_active;
} rt_server_stats;

int rt_server_create(const rt_server_config *cfg, rt_server **out);
/* Stops the worker after the frames in flight; queued jobs are dropped. */
void rt_server_destroy(rt_server *s);
int rt_server_add_scene(rt_server *s, uint32_t scene_id, const rt_scene_desc *scene);
/* Queues a job.  RT_ERR_STATE once the worker thread has stopped on a host allocation failure (it
 * then fails every job not yet done, so rt_server_wait_idle returns). */
int rt_server_submit(rt_server *s, const rt_request *req, uint64_t *job_id);
int rt_server_job_status(rt_server *s, uint64_t job_id, rt_job_status *out);
/* The final accumulation (W*H*4 floats) of a done job submitted with keep_result. */
int rt_server_read_result(rt_server *s, uint64_t job_id, float *rgba, uint64_t n_floats);
/* Forgets a done or failed job (its status and kept result). */
int rt_server_release_job(rt_server *s, uint64_t job_id);
/* Waits until every submitted job is done or failed; RT_ERR_STATE after timeout_ms. */
int rt_server_wait_idle(rt_server *s, uint32_t timeout_ms);
int rt_server_get_stats(rt_server *s, rt_server_stats *out);
double rt_server_now_ms(const rt_server *s);

/* ---------------------------------------------------------------------------------------------
 * Stage entry points on caller-provided host buffers (copy in, run on the device, copy out).
 * Used to check one stage on inputs shared with another implementation.
 * ------------------------------------------------------------------------------------------- */

/* The a-trous denoise of record_frame (lib.rs:743-776, denoise.wgsl:122-195): `passes` passes with
 * steps 1, 2, 4, ..., ping-pong; the result of the last pass lands in out_rgba. */
int rt_stage_denoise(const float *frame_rgba, const float *gbuffer, const float *moments, uint32_t width,
                     uint32_t height, float alpha, uint32_t passes, float *out_rgba);
/* composite.wgsl:211-221 then tonemap.wgsl:240-271: accum_inout = mix(accum, frame, alpha), then
 * the RGBA8 image.  gbuffer may be NULL when the marker is hidden. */
int rt_stage_resolve(const float *frame_rgba, float *accum_inout, const float *gbuffer, uint32_t width,
                     uint32_t height, float alpha, const rt_tonemap_params *tp, uint8_t *out_rgba8);
/* photon_count.wgsl + host scan (lib.rs:956-1007) + photon_scatter.wgsl, ordered by slot within a
 * cell.  counts/meta have gp->num_cells entries; sorted has gp->photon_slots entries (entries past
 * the number of binned photons are zero). */
int rt_stage_photon_grid(const rt_photon *photons, const rt_grid_params *gp, uint32_t *counts, uint32_t *meta,
                         rt_photon *sorted);

/* The photon-grid build of rt_stage_photon_grid without any device allocation.  It has no
 * counterpart in the reference.  It exists for callers that cannot allocate device memory: frame loops
 * with a no-allocation rule (cudaMalloc / cudaFree can synchronise the device), hosts whose device
 * memory all comes from their own allocator or pool, and processes near the memory limit.
 *   - d_photons (gp->photon_slots records), d_counts (gp->num_cells), d_meta (2 * gp->num_cells) and
 *     d_sorted (gp->photon_slots records) are DEVICE pointers owned by the caller (photon buffers
 *     16-byte aligned, counts / meta 4-byte aligned, as cudaMalloc returns them); entries of d_sorted
 *     past the number of binned photons are left as they were.
 *   - Scratch lives in one file-scope device array of RT_NOALLOC_SCRATCH_BYTES that every GPU loading
 *     the library holds until the process exits; sizes above RT_NOALLOC_MAX_SLOTS slots or
 *     RT_NOALLOC_MAX_CELLS cells are rejected with RT_ERR_INVALID_ARGUMENT.
 *   - Each call looks up that array's device address with the calling thread's current device, so the
 *     address stays right after cudaDeviceReset.  With CUDA's lazy module loading (the default since
 *     CUDA 12.2) the first call on a device may be what loads this library's kernels onto it, which
 *     creates the array there: that first call can allocate and synchronise, so make it outside the
 *     no-allocation region (a warm-up call at start-up) or set CUDA_MODULE_LOADING=EAGER; and make it
 *     before any stream capture.  Later calls allocate nothing.
 *   - Work is enqueued on `stream` (a cudaStream_t; NULL = the default stream) and the call returns
 *     without waiting.  All calls share the one array (its counters are cleared by each call): calls
 *     whose work overlaps on the GPU race, so order them on one stream or synchronise between them.
 *   - A CUDA error left pending by earlier, unrelated work is cleared on entry.  On RT_ERR_CUDA part
 *     of the build may already be enqueued: the contents of d_counts, d_meta and d_sorted are then
 *     undefined. */
#define RT_NOALLOC_MAX_SLOTS (1u << 20)
#define RT_NOALLOC_MAX_CELLS (1u << 18)
#define RT_NOALLOC_SCRATCH_BYTES 9438208u
int rt_stage_photon_grid_noalloc(const rt_photon *d_photons, const rt_grid_params *gp, uint32_t *d_counts,
                                 uint32_t *d_meta, rt_photon *d_sorted, void *stream);

/* ---------------------------------------------------------------------------------------------
 * Host-side scene model (rustracer-core): meshes, materials, lights, role textures, flattening and
 * the binned-SAH BVH build.  Used by the headless entry, the tests and the benchmarks; a Rust
 * caller keeps its own rustracer-core and fills rt_scene_desc directly.
 * ------------------------------------------------------------------------------------------- */
typedef struct rt_scene rt_scene;

int rt_scene_create(rt_scene **out);
void rt_scene_destroy(rt_scene *s);
/* Mesh::new (scene.rs:24-38).  normals/uvs may be NULL (reference defaults Y and (0,0)). */
int rt_scene_add_mesh(rt_scene *s, const float *positions, const float *normals, const float *uvs,
                      uint64_t vertex_count, const uint32_t *indices, uint64_t index_count, uint32_t material_id);
int rt_scene_add_material(rt_scene *s, const rt_material *m);
int rt_scene_add_light(rt_scene *s, const rt_light *l);
/* Sets one role texture array (copied; RGBA8, layer-major). */
int rt_scene_set_textures(rt_scene *s, int role, const uint8_t *rgba8, uint32_t width, uint32_t height,
                          uint32_t layers);
/* flatten_triangles + build_bvh + flatten_materials + bounds (scene.rs:198-291); idempotent. */
int rt_scene_finalize(rt_scene *s);
/* Fills desc with pointers into the scene's own arrays (valid until the scene is changed/destroyed). */
int rt_scene_describe(rt_scene *s, rt_scene_desc *desc);
uint64_t rt_scene_triangle_count(const rt_scene *s);

/* The 555-unit Cornell box: 36 triangles, 2 area lights (walls 10, ceiling light 2, boxes 24). */
int rt_scene_create_cornell555(rt_scene **out);
/* Displaced icosphere (20 * 4^level triangles, radius 1, per-vertex normal displacement N(0, sigma))
 * in a 10^3 Lambertian room, seeded per-triangle materials (60% Lambertian, 25% GGX metal, 15%
 * dielectric), value-noise RGBA8 albedo / MR / normal textures of tex_size^2, a 1x1 area light
 * (emission 20) and 4 seeded point lights. */
int rt_scene_create_icosphere_room(uint32_t level, uint64_t seed, float sigma, uint32_t tex_size, rt_scene **out);

/* Camera::to_uniform (camera.rs:278-301) and Camera::frame_scene (camera.rs:305-321). */
void rt_camera_default(rt_camera *cam);
void rt_camera_to_uniform(const rt_camera *cam, uint32_t width, uint32_t height, rt_camera_uniform *out);
int rt_camera_frame_scene(const rt_scene *s, rt_camera *out);
/* The camera a procedural scene was built with (Cornell: (278,278,-800) -> (278,278,0), 40 degrees),
 * else Camera::frame_scene. */
int rt_scene_default_camera(const rt_scene *s, rt_camera *out);
/* Camera::orbit / zoom (camera.rs:324-345). */
void rt_camera_orbit(rt_camera *cam, float delta_yaw, float delta_pitch);
void rt_camera_zoom(rt_camera *cam, float delta);

/* Photon-grid derivation of Renderer::new (lib.rs:416-457), generalised by grid_max_dim and the
 * radius mode (see rt_render_config).  photon_slots = photon_count * RT_MAX_BOUNCES (or 1). */
void rt_derive_grid(const float bounds_min[3], const float bounds_max[3], int has_bounds, uint32_t grid_max_dim,
                    uint32_t radius_mode, uint32_t photon_slots, rt_grid_params *gp, float *photon_radius);

/* BVHBuilder::build (bvh.rs:135-336): binned SAH over primitive centroids / AABBs. */
typedef struct rt_bvh rt_bvh;
int rt_bvh_build(const float *centroids, const float *bbox_min, const float *bbox_max, uint64_t n, rt_bvh **out);
const rt_bvh_node *rt_bvh_nodes(const rt_bvh *b, uint64_t *count);
const uint32_t *rt_bvh_prims(const rt_bvh *b, uint64_t *count);
void rt_bvh_destroy(rt_bvh *b);
/* The four-wide traversal records of a tree in the reference's node layout (what scene upload builds
 * under rt_set_traversal_width(4)): 32 floats per record, per child (min.xyz, ref) then
 * (max.xyz, count) as bit patterns in the .w slots (count > 0: a leaf of `count` prim slots from
 * `ref`; 0: an internal child, `ref` its record; 0xFFFFFFFF: an empty place).  Writes at most
 * `capacity` floats to `out` (may be null to ask for the size); *records gets the record count and
 * *stack_need the stack bound of a near-first walk. */
int rt_bvh_wide_layout(const rt_bvh_node *nodes, uint64_t n_nodes, float *out, uint64_t capacity, uint64_t *records,
                       uint32_t *stack_need);
/* BVH builders (no counterpart in the reference, which builds on the host only): RT_BVH_HOST_SAH is
 * BVHBuilder::build (bvh.rs:135-336, the default); RT_BVH_GPU_LBVH builds a linear BVH on the GPU
 * (Morton codes of the centroids, one primitive per leaf) in the same node layout, falling back to
 * the host build when no device is visible or the tree is deeper than 62 levels (the traversal
 * stack's bound).  The images are the same with either tree except where two triangles are hit at
 * exactly the same distance.  Changing the builder of a finalized scene flattens it again at the
 * next rt_scene_describe (descriptions taken before become invalid; renderers already created keep
 * their own copies). */
#define RT_BVH_HOST_SAH 0u
#define RT_BVH_GPU_LBVH 1u
int rt_scene_set_bvh_builder(rt_scene *s, uint32_t builder);
uint32_t rt_scene_bvh_builder_used(const rt_scene *s);
/* The GPU build on raw primitive boxes (n >= 2); *max_depth (optional) gets the tree's depth. */
int rt_bvh_build_gpu(const float *centroids, const float *bbox_min, const float *bbox_max, uint64_t n,
                     rt_bvh **out, uint32_t *max_depth);
/* Threads of the host BVH build (0, the default: one per hardware thread; 1: sequential).  The
 * tree does not depend on it. */
void rt_set_host_threads(uint32_t n);
/* Children per traversal record for scenes uploaded from now on (rt_renderer_create,
 * rt_resident_scene_create, the server's scene uploads): 4 (the default) adds a four-wide copy of
 * the scene's tree -- each record takes in the children of its largest internal children -- walked
 * whenever every job of a launch has one (a scene whose four-wide walk could need more than 64 stack
 * entries keeps only the two-wide records); 2 keeps the two-wide records only.  Either walk finds the
 * reference's closest hit; only triangles hit at exactly equal t may resolve to a different one of
 * them.  Returns RT_ERR_INVALID_ARGUMENT for other widths. */
int rt_set_traversal_width(uint32_t width);
/* Denoise blocks whose tensor-memory-accelerator tile copies did not arrive within the kernel's wait
 * bound since the library was loaded (such a block writes nothing; 0 is the only expected value,
 * 0xFFFFFFFF if the count cannot be read). */
uint32_t rt_tma_timeouts(void);
/* Photon-grid scans whose look-back for a preceding tile's sum gave up at the kernel's wait bound
 * since the library was loaded (such a grid's offsets are wrong; 0 is the only expected value,
 * 0xFFFFFFFF if the count cannot be read).  The scan replaces the host scan of
 * rustracer-renderer/src/lib.rs:956-1007. */
uint32_t rt_scan_timeouts(void);
uint32_t rt_get_traversal_width(void);

/* PNG scanline unfiltering for the glTF ingest (the reference decodes images through the `gltf` /
 * `image` crates, rustracer-core/src/loader.rs:36-100): h rows of 1 + stride bytes (filter type
 * first) in, h * stride unfiltered bytes out; bpp = bytes per pixel. */
int rt_png_unfilter(const uint8_t *rows, uint32_t h, uint32_t stride, uint32_t bpp, uint8_t *out);
/* JPEG decoding for the glTF ingest (the reference's `image` crate through gltf::import,
 * rustracer-core/src/loader.rs:36-113, 266): baseline / extended sequential and progressive Huffman
 * streams, 8-bit, grey or YCbCr (JFIF), sampling factors 1..2, restart intervals.  *w / *h receive the
 * size; out_rgba (w * h * 4 bytes, alpha 255) is written when out_bytes is large enough, so a first
 * call with out_rgba = NULL asks for the size.  RT_ERR_INVALID_ARGUMENT for any other stream. */
int rt_jpeg_decode(const uint8_t *data, uint64_t n, uint8_t *out_rgba, uint64_t out_bytes, uint32_t *w,
                   uint32_t *h);

#ifdef __cplusplus
} /* extern "C" */
#endif

#endif /* RUSTRACER_CUDA_H */
