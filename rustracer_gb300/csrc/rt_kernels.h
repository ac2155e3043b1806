// Kernel parameter blocks and host-side launchers of the hot-path kernels.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

#include "rt_device.cuh"

namespace rtd {

// One render job of the wavefront (a renderer's frame).  The table lives in device memory so the
// per-frame values (frame counter, camera) are read there, not baked into launch parameters.
struct DevJob {
    DevScene scene;
    rt_camera_uniform cam;
    rt_image_params ip;
    rt_grid_params gp;
    const float4 *sorted_photons;  // 4 x float4 per photon
    const float4 *sorted_pos;      // position of each sorted photon (its first float4), 16 B apart
    uint64_t sorted_count;
    const uint2 *grid_meta;        // (start, count) per cell
    uint32_t max_bounces, npix, base, spp;  // base: first path slot; spp = max(1, ip.spp)
    uint32_t tile0, tile_pad;               // first 8 x 4 tile of the job in the frame's generate launch
    float4 *frame;
    float4 *moments;
    float4 *gbuffer;
    float alpha;  // the frame's accumulation alpha, read by denoise and resolve in a replayed graph
};

// The wavefront gather pass over one or more jobs.  Path state has one slot per pixel of every job
// (slot = job.base + pixel); queues hold slots of any job.
constexpr uint32_t kNoMat = 0x3FFFFFFFu;  // a material index a prim slot's key word cannot carry
struct WaveParams {
    const DevJob *jobs;
    uint32_t n_jobs;
    float4 *ro;        // origin, .w = RNG state
    float4 *rd;        // direction, .w = sample index | segment index << 16
    float4 *thr;       // throughput, .w = job index
    float2 *hit;       // closest t, the hit's prim slot
    float4 *acc;       // 4 per slot: (col, lum_sum), (lum2_sum, first_depth, -, -), sample_lum[0..8]
    float4 *nrm;       // first-hit shading normal
    uint32_t *queue[2];
    uint32_t *counts;  // per iteration: [0] paths queued, [1] shadow rays, [2] trace cursor, [3] photon lookups
    float4 *shadow;    // 3 per deferred NEE ray: (origin, max_dist), (dir, slot), (contribution, tag)
    float4 *preq;      // 3 per photon-map lookup: (hit point, slot), (normal, sample), (throughput, job)
    unsigned long long *counters;  // [0] segments, [1] shadow rays (cumulative)
    // Work counters of the profiling traversal kernels (null otherwise): traversal records visited
    // by closest-hit / occlusion rays, then their leaf triangle tests.
    unsigned long long *work;
};
// Host-side shape of a job for the per-job launches.
struct JobShape {
    uint32_t width, height, npix, base, stack_cap;
    uint32_t photons;  // the job gathers from a photon map (rt_image_params.use_photons)
    uint32_t debug;    // the job renders a debug view (rt_image_params._pad[0] != 0)
    uint32_t wide;     // the job's scene has four-wide records (DevScene.wnodes)
    uint32_t wide_stack;  // stack entries a walk of them can need
};
// Launch shape of the persistent traversal kernels (extend, shadow); no effect on any result.
struct WaveTuning {
    uint32_t block_threads;  // 64, 128 or 256
    uint32_t blocks_per_sm;  // persistent blocks per SM (the grid is capped by the work)
    uint32_t chunk;          // queue items a warp takes per atomic: its segment of the queue
    uint32_t steps;          // traversal records between lane refills
    uint32_t stack_entries;  // shared-memory stack per lane: 32, 48 or 64 (raised to the jobs' need)
    uint32_t treelet;        // four-wide records at the top of the tree staged in shared memory per
                             // block: 0 or kTreeletRecords
    uint32_t shade_blocks;   // shade kernel compiled for 4, 5 or 6 resident blocks of 128 per SM
    uint32_t refill_idle;    // traversal warps refill before `steps` records once this many lanes are
                             // idle (0: only after `steps`)
};
// Records of the treelet: the first records of the breadth-first four-wide layout (the root, its
// children and most of their children), 2 KB, which fits beside 8 blocks of 128 traversal threads.
constexpr uint32_t kTreeletRecords = 16;
WaveTuning default_tuning();
// Clamps a tuning to supported values (stack raised to `stack_need`); false if it had to change.
bool normalize_tuning(WaveTuning &t, uint32_t stack_need);
// Optional instrumentation of one gather pass: CUDA events recorded before and after every launch of
// the traversal, shade and photon-lookup kernels (2 per launch; arrays of at least 2 * (iters + 1)),
// and the counting variants of the traversal kernels when p.work is set.
struct WaveProfile {
    cudaEvent_t *trace_ev, *shade_ev, *photon_ev;
    uint32_t trace_launches, shade_launches, photon_launches;  // written by launch_wavefront
};
// generate (per job), iters x (extend, shade, shadow) over all jobs, finalize (per job), counters.
cudaError_t launch_wavefront(const WaveParams &p, const JobShape *jobs, uint32_t n_jobs, uint32_t iters, int num_sms,
                             const WaveTuning &tune, cudaStream_t st, WaveProfile *prof = nullptr);
int device_sm_count();
// One-time kernel attributes (shared-memory opt-ins); call before capturing launches into a graph.
void prepare_kernels();
void prepare_wavefront_kernels();

struct PhotonTraceParams {
    DevScene scene;
    rt_grid_params gp;
    uint32_t photon_begin, photon_end;  // photon indices traced by this launch
    uint64_t slot_count;                // photon_slots
    float4 *photons;                    // 4 x float4 per slot
    uint32_t *keys;                     // cell key per slot (kInvalidKey when not binned)
};
// State of the photon wavefront, one entry per traced photon (index - photon_begin).
struct PhotonWave {
    float4 *ro;        // origin, .w = RNG state
    float4 *rd;        // direction, .w = photon index
    float4 *pw;        // power, .w = job index 0 (read by the shared closest-hit kernel)
    float2 *hit;       // closest t, primitive
    uint32_t *queue[2];
    uint32_t *counts;  // 4 per bounce (+1): [0] photons queued, [2] fetch cursor of the hit kernel
};
// Bytes of PhotonWave state for n photons (carved from one buffer, 16-byte aligned parts).
size_t photon_wave_bytes(uint32_t n);
PhotonWave photon_wave_at(void *base, uint32_t n);

// Launchers (stream-ordered, no synchronisation).  Each returns the launch error, if any.
// The photon pass (photon_trace.wgsl:91-260) as a wavefront: jobs_dev[0].scene must be p.scene.
cudaError_t launch_photon_wave(const PhotonTraceParams &p, const PhotonWave &w, const DevJob *jobs_dev, int num_sms,
                               const WaveTuning &tune, cudaStream_t st);
// One closest-hit pass of the persistent traversal kernel over queue[iter & 1] (count at
// counts[4 iter]); `max_items` bounds the grid.
cudaError_t launch_extend(const WaveParams &p, uint32_t iter, uint64_t max_items, const DevScene &scene, int num_sms,
                          const WaveTuning &tune, cudaStream_t st);

// Photon grid (exact u32 counting sort).  Scratch sizes come from grid_scratch_bytes.
struct GridBuffers {
    const float4 *photons;  // slot_count photons
    const uint32_t *keys;   // slot_count keys
    uint64_t slot_count;
    uint32_t num_cells;
    uint32_t *counts;       // num_cells
    uint2 *meta;            // num_cells
    uint32_t *cursor;       // num_cells
    uint32_t *order;        // slot_count: slot indices in (cell, slot) order
    float4 *sorted;         // slot_count photons
    float4 *sorted_pos;     // slot_count positions (the sorted photons' first float4), or null
    uint32_t *scan_partials;  // grid_scan_partials(num_cells) entries
    uint32_t *total;          // 4 entries: [0] binned photons, [1] listed cells
    // Optional per-slot rank within its cell (null: count and an atomic scatter, then a pass that
    // lists the multi-photon cells, a per-cell order pass and the gather).  With ranks the count pass
    // records them, the scan lists the occupied cells, the scatter needs no atomics and one pass per
    // occupied cell restores slot order and copies the records.
    uint32_t *rank;
};
uint32_t grid_scan_partials(uint32_t num_cells);
cudaError_t launch_photon_keys(const float4 *photons, uint64_t slot_count, const rt_grid_params &gp, uint32_t *keys,
                               cudaStream_t st);
// count -> scan -> scatter -> per-cell slot order -> photon gather.  counts/cursor are cleared here.
cudaError_t launch_grid_build(const GridBuffers &g, cudaStream_t st);

// Image kernels.
// alpha_dev, when not null, is read on the device in place of p.alpha (a CUDA graph replays the
// launch with the value of the frame being replayed).
// Denoise blocks whose TMA tile copies missed the wait bound since the library loaded (0 expected).
uint32_t tma_timeouts();
// Photon-grid scan chunks whose look-back gave up at the wait bound since the library loaded (0 expected).
uint32_t scan_timeouts();
cudaError_t launch_denoise(const float4 *in, float4 *out, const float4 *gbuffer, const float4 *moments,
                           const rt_denoise_params &p, const float *alpha_dev, cudaStream_t st, bool after_pass = false);
// accum = mix(accum, frame, alpha) and the tonemapped rgba8 image in one pass; alpha_dev as above.
cudaError_t launch_resolve(const float4 *frame, float4 *accum, const float4 *gbuffer, uint32_t width,
                           uint32_t height, float alpha, const float *alpha_dev, const rt_tonemap_params &tp,
                           uchar4 *out, cudaStream_t st);

}  // namespace rtd
