// Internals of rt_renderer shared by the renderer (rt_renderer.cu) and the batch (rt_batch.cu).
#pragma once
#include <cuda_runtime.h>

#include <array>
#include <atomic>
#include <cstring>
#include <vector>

#include "rt_internal.h"
#include "rt_kernels.h"

#define RT_CK(call)                                                                                    \
    do {                                                                                               \
        cudaError_t e_ = (call);                                                                       \
        if (e_ != cudaSuccess) {                                                                       \
            rt::set_error("%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, __LINE__); \
            return e_ == cudaErrorMemoryAllocation ? RT_ERR_OUT_OF_MEMORY : RT_ERR_CUDA;               \
        }                                                                                              \
    } while (0)

namespace rt {

// One device buffer, freed with its owner.  Unbound it is cudaMalloc'd (cudaFree synchronises the
// device); bound to a memory pool and a stream it is allocated and freed in that stream's order
// (cudaMallocFromPoolAsync / cudaFreeAsync), so freeing it waits for nothing but the stream's own
// work.  A bound buffer must be released before its stream is destroyed.
struct DevBuf {
    void *p = nullptr;
    size_t bytes = 0;
    cudaMemPool_t pool = nullptr;
    cudaStream_t stream = nullptr;
    DevBuf() = default;
    DevBuf(const DevBuf &) = delete;
    DevBuf &operator=(const DevBuf &) = delete;
    ~DevBuf() { release(); }
    void bind(cudaMemPool_t pl, cudaStream_t st) {
        pool = pl;
        stream = st;
    }
    void release() {
        if (p) {
            if (pool) cudaFreeAsync(p, stream);
            else cudaFree(p);
        }
        p = nullptr;
        bytes = 0;
    }
    cudaError_t alloc(size_t n) {
        release();
        if (n == 0) n = 16;
        cudaError_t e = pool ? cudaMallocFromPoolAsync(&p, n, pool, stream) : cudaMalloc(&p, n);
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
            if (pool.size() >= (1u << 16)) {  // bounded: timings past 16k undrained frames are dropped
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

// Wavefront path state for `slots` pixel slots (240 B per slot) and the per-iteration counters.
struct PathState {
    DevBuf ro, rd, thr, hit, acc, nrm, queue[2], shadow, preq, counts;
    size_t slots = 0, counts_bytes = 0;
    // (Re)allocates when too small.  The caller's stream must be idle.
    cudaError_t ensure(size_t n_slots, uint32_t iters) {
        cudaError_t e;
        if (n_slots > slots) {
            DevBuf *b[10] = {&ro, &rd, &thr, &nrm, &hit, &acc, &queue[0], &queue[1], &shadow, &preq};
            const size_t sz[10] = {16, 16, 16, 16, 8, 64, 4, 4, 48, 48};
            for (int i = 0; i < 10; ++i)
                if ((e = b[i]->alloc(n_slots * sz[i])) != cudaSuccess) {
                    slots = 0;
                    return e;
                }
            slots = n_slots;
        }
        const size_t need = sizeof(uint32_t) * 4 * ((size_t)iters + 1);
        if (need > counts_bytes) {
            if ((e = counts.alloc(need)) != cudaSuccess) {
                counts_bytes = 0;
                return e;
            }
            counts_bytes = need;
        }
        return cudaSuccess;
    }
    rtd::WaveParams params(const rtd::DevJob *jobs, uint32_t n_jobs, unsigned long long *counters) const {
        rtd::WaveParams w;
        std::memset(&w, 0, sizeof(w));
        w.jobs = jobs;
        w.n_jobs = n_jobs;
        w.ro = ro.as<float4>();
        w.rd = rd.as<float4>();
        w.thr = thr.as<float4>();
        w.hit = hit.as<float2>();
        w.acc = acc.as<float4>();
        w.nrm = nrm.as<float4>();
        w.queue[0] = queue[0].as<uint32_t>();
        w.queue[1] = queue[1].as<uint32_t>();
        w.counts = counts.as<uint32_t>();
        w.shadow = shadow.as<float4>();
        w.preq = preq.as<float4>();
        w.counters = counters;
        return w;
    }
};

// The device job table and the pinned staging it is copied from.  A frame's table is written into
// the next of kSlots pinned slots (after the copy that last used that slot has run) and copied to the
// device on the frame's stream, ahead of the frame's kernels.
struct JobTable {
    static constexpr int kSlots = 4;
    rtd::DevJob *host = nullptr;
    size_t cap = 0;
    int next = 0;
    cudaEvent_t ev[kSlots] = {};
    DevBuf dev;
    ~JobTable() {
        if (host) cudaFreeHost(host);
        for (auto e : ev)
            if (e) cudaEventDestroy(e);
    }
    bool ready() const { return host != nullptr && dev.p != nullptr; }
    // Allocates the table for n_jobs; after a failure a second call completes what is missing.
    cudaError_t init(size_t n_jobs) {
        cudaError_t e;
        if (!host) {
            if ((e = cudaHostAlloc(reinterpret_cast<void **>(&host), sizeof(rtd::DevJob) * n_jobs * kSlots,
                                   cudaHostAllocDefault)) != cudaSuccess) {
                host = nullptr;
                return e;
            }
            cap = n_jobs;
        }
        for (auto &x : ev)
            if (!x && (e = cudaEventCreateWithFlags(&x, cudaEventDisableTiming)) != cudaSuccess) {
                x = nullptr;
                return e;
            }
        return dev.p ? cudaSuccess : dev.alloc(sizeof(rtd::DevJob) * cap);
    }
    cudaError_t upload(const rtd::DevJob *jobs, size_t n, cudaStream_t st) {
        cudaError_t e;
        const int slot = next;
        next = (next + 1) % kSlots;
        if ((e = cudaEventSynchronize(ev[slot])) != cudaSuccess) return e;
        std::memcpy(host + slot * cap, jobs, sizeof(rtd::DevJob) * n);
        if ((e = cudaMemcpyAsync(dev.p, host + slot * cap, sizeof(rtd::DevJob) * n, cudaMemcpyHostToDevice, st)) !=
            cudaSuccess)
            return e;
        return cudaEventRecord(ev[slot], st);
    }
    const rtd::DevJob *device() const { return dev.as<rtd::DevJob>(); }
};

}  // namespace rt

// A scene's read-only device data (geometry, traversal layout, materials, textures), shared by every
// renderer created on it and freed with the last reference.
struct rt_resident_scene {
    int device = 0;
    std::atomic<uint32_t> refs{1};
    rt::DevBuf d_cnodes, d_wnodes, d_tri_ord, d_tris, d_mats, d_tex[4];
    rtd::DevScene scene{};          // light fields are per renderer
    std::vector<rt_light> lights;   // the scene's lights, each renderer's initial copy
    float bmin[3] = {0, 0, 0}, bmax[3] = {0, 0, 0};
    uint32_t has_bounds = 0;
    uint64_t bytes = 0;             // device bytes held
};

struct rt_renderer {
    int device = 0;
    cudaStream_t stream = nullptr;
    rt_render_config cfg{};
    rt_grid_params gp{};
    rt_camera_uniform cam{};
    rt_resident_scene *res = nullptr;  // one reference held
    std::vector<rt_light> lights_host;
    rtd::DevScene scene{};
    rt::DevBuf d_lights;
    rt::DevBuf d_frame, d_pingpong, d_moments, d_gbuffer, d_accum, d_output;
    rt::PathState path;  // allocated on the first solo frame (a batch brings its own)
    rt::JobTable jobs;
    rtd::WaveTuning tuning = rtd::default_tuning();  // solo frames
    int num_sms = 1;
    rt::DevBuf d_photons, d_keys, d_rank, d_order, d_sorted, d_sorted_pos, d_counts, d_meta, d_cursor, d_partials,
        d_total, d_counters;
    uint64_t photon_slots = 1;
    bool photon_buffers = false;
    uint32_t sample_counter = 0, frames_since_reset = 0;
    float marker[4] = {0, 0, 0, 0};
    float glow = 1.0f;
    uint64_t frames = 0;
    bool have_frame_timing = false, have_photon_timing = false;
    uint32_t last_denoise_passes = 0;
    rt::Events events;
    rt::FrameEventRing ring;
    // Gather-pass profiling (rt_set_profiling): flags, events around the profiled launches (2 per
    // launch of each kind, plus the pass bounds), the counting kernels' work counters, the sums.
    uint32_t prof_flags = 0;
    std::vector<cudaEvent_t> prof_ev;
    rt::DevBuf d_work;
    rt_trace_profile prof{};
    // Every device buffer above comes from the device's renderer pool in the renderer's stream order
    // (bind_buffers at create; release_buffers before the stream goes).
    bool pooled = false;
    std::array<rt::DevBuf *, 32> buffers();  // every device buffer the renderer owns
    void bind_buffers(cudaMemPool_t pool);
    void release_buffers();
    ~rt_renderer();
    // Device bytes this renderer owns (its resident scene not included).
    uint64_t device_bytes() const;
};

namespace rt {
// The memory pool renderer buffers come from on `device` (created on first use; freed blocks stay in
// it for the next renderer), null if the device has no memory pools.  renderer_pool_acquire counts a
// live renderer; renderer_pool_release uncounts it and, with none left, returns the pool's unused
// memory to the device.
cudaMemPool_t renderer_pool_acquire(int device);
void renderer_pool_release(int device);
// The renderer's job table, allocated by the first solo frame or photon rebuild that needs it.
int ensure_job_table(rt_renderer *r);
// Uploads a scene description (validated by the caller); *out holds one reference.
int resident_scene_create(const rt_scene_desc *sd, rt_resident_scene **out);
void resident_scene_release(rt_resident_scene *s);
// Device bytes a renderer with this config allocates at create (frame and photon buffers), and the
// path state its first solo frame adds.
uint64_t renderer_create_bytes(const rt_render_config &c, uint64_t num_cells, uint64_t n_lights);
uint64_t path_state_bytes(uint64_t slots, uint32_t iters);
// rebuild_photons (lib.rs:913-1037) enqueued on the renderer's stream, without waiting for it.
int enqueue_photon_rebuild(rt_renderer *r);
// Advances the frame counters (lib.rs:672-684) and returns the frame's accumulation alpha.
float prepare_frame(rt_renderer *r);
// The job-table entry of the renderer's next frame; `base` is its first path slot.
rtd::DevJob make_job(const rt_renderer *r, uint32_t base);
// spp * max_bounces of the renderer's config.
uint32_t frame_iterations(const rt_renderer *r);
// Denoise passes of the renderer's frame (lib.rs:743-776); *result = the buffer composite reads.
// alpha_dev, when not null, points at the frame's alpha in device memory and is used in its place.
int enqueue_denoise(rt_renderer *r, float alpha, const float *alpha_dev, cudaStream_t st, float4 **result);
// Composite and tonemap (lib.rs:778-831).
int enqueue_resolve(rt_renderer *r, const float4 *result, float alpha, const float *alpha_dev, cudaStream_t st);
// Both, on stream `st`.
int enqueue_post(rt_renderer *r, float alpha, const float *alpha_dev, cudaStream_t st);
// The gather pass of a frame rendered with profiling on (rt_set_profiling); waits for it.
int profiled_gather(rt_renderer *r, rtd::WaveParams wp, const rtd::JobShape &shape, uint32_t iters);
}  // namespace rt
