// The batch frame shared by rt_batch (a fixed set of renderers) and rt_server (a set that changes
// from frame to frame as jobs arrive and finish).
#pragma once
#include <cuda_runtime.h>

#include <vector>

#include "rt_renderer_impl.h"

namespace rt {

enum class GraphMode {
    Off,       // launch every frame directly
    Always,    // capture whenever the frame's shape changed, replay otherwise
    OnRepeat,  // capture only a shape seen on two frames in a row (membership that changes often
               // is launched directly instead of paying a capture per change)
};

struct BatchEngine {
    cudaStream_t stream = nullptr;
    PathState path;
    JobTable jobs;
    DevBuf counters;  // [0] segments, [1] shadow rays, summed over all frames
    int num_sms = 1;
    GraphMode graph_mode = GraphMode::Off;
    rtd::WaveTuning tuning = rtd::default_tuning();
    cudaGraphExec_t exec = nullptr;
    std::vector<unsigned char> sig, last_sig;  // shape of the captured graph; of the previous frame
    std::vector<uint32_t> base;                // first path slot of each member, this frame
    uint64_t frames = 0, captures = 0;
    cudaEvent_t done = nullptr;
    FrameEventRing ring;  // two events per frame (start, end)
    // Side streams for the members' denoise and resolve, which touch only each member's own buffers:
    // forked from and joined back to `stream` (parallel branches of a captured frame).
    static constexpr int kSide = 4;
    cudaStream_t side[kSide] = {};
    cudaEvent_t fork = nullptr, join[kSide] = {};

    ~BatchEngine();
    int init(uint32_t max_jobs, GraphMode mode);
    // Path state for `slots` pixel slots and `iters` iterations (waits for the engine's stream).
    int reserve(uint64_t slots, uint32_t iters);
    // The next progressive frame of each of the n renderers, on the engine's stream.  Waits for work
    // queued on the renderers' own streams; their streams wait for the frame.
    int frame(rt_renderer *const *rs, uint32_t n);
    int stats(rt_frame_stats *out);
    // Times launch shapes of the traversal kernels on `trial_frames` frames each (coordinate descent
    // from the current tuning) and keeps the fastest.  The trial frames are undone: each member's
    // accumulation and frame counters are restored, so the images that follow are unaffected.
    int autotune(rt_renderer *const *rs, uint32_t n, uint32_t trial_frames, float *best_ms);

  private:
    std::vector<unsigned char> signature(rt_renderer *const *rs, uint32_t n, uint32_t iters) const;
    int enqueue(rt_renderer *const *rs, uint32_t n, uint32_t iters, const float *alpha, bool dev_alpha);
};

}  // namespace rt
