// Batched rendering: one progressive frame of several renderers (render jobs) at once.  The rays of
// every job share the wavefront's queues and launches (extend / shade / shadow run over all jobs'
// paths together, each lane on its own job's scene), which keeps the GPU full when single jobs are
// too small to.  Each job's per-pixel work is the one it does alone -- same seeds, same order of
// operations -- so a job's image is the same bit for bit alone and in a batch.
//
// A batch frame can be captured as a CUDA graph and replayed: the per-frame values (frame counters,
// cameras, accumulation alpha) live in the device job table, copied from pinned memory ahead of each
// replay; the graph is captured again only when something baked into its launches changes (the
// member jobs and their buffers, the number of iterations, the jobs' shapes, tonemap or denoise
// settings).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <new>
#include <vector>

#include "rt_batch_engine.h"

using rt::set_error;

namespace rt {

namespace {

template <class T>
void put(std::vector<unsigned char> &v, const T &x) {
    const unsigned char *p = reinterpret_cast<const unsigned char *>(&x);
    v.insert(v.end(), p, p + sizeof(T));
}

}  // namespace

BatchEngine::~BatchEngine() {
    if (stream) cudaStreamSynchronize(stream);
    if (exec) cudaGraphExecDestroy(exec);
    if (done) cudaEventDestroy(done);
    if (fork) cudaEventDestroy(fork);
    for (int i = 0; i < kSide; ++i) {
        if (join[i]) cudaEventDestroy(join[i]);
        if (side[i]) cudaStreamDestroy(side[i]);
    }
    if (stream) cudaStreamDestroy(stream);
}

int BatchEngine::init(uint32_t max_jobs, GraphMode mode) {
    graph_mode = mode;
    if (cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&done, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&fork, cudaEventDisableTiming) != cudaSuccess) {
        set_error("batch: cannot create the stream");
        return RT_ERR_CUDA;
    }
    for (int i = 0; i < kSide; ++i)
        if (cudaStreamCreateWithFlags(&side[i], cudaStreamNonBlocking) != cudaSuccess ||
            cudaEventCreateWithFlags(&join[i], cudaEventDisableTiming) != cudaSuccess) {
            set_error("batch: cannot create the side streams");
            return RT_ERR_CUDA;
        }
    if (jobs.init(max_jobs) != cudaSuccess || counters.alloc(64) != cudaSuccess ||
        cudaMemset(counters.p, 0, 64) != cudaSuccess) {
        set_error("batch: out of device memory for the job table");
        return RT_ERR_OUT_OF_MEMORY;
    }
    num_sms = rtd::device_sm_count();
    rtd::prepare_kernels();
    return RT_OK;
}

int BatchEngine::reserve(uint64_t slots, uint32_t iters) {
    if (slots > path.slots || sizeof(uint32_t) * 4 * ((size_t)iters + 1) > path.counts_bytes) {
        RT_CK(cudaStreamSynchronize(stream));
        RT_CK(path.ensure(slots, iters));
    }
    return RT_OK;
}

// Everything the frame's launches take by value (the job table itself is read from device memory).
std::vector<unsigned char> BatchEngine::signature(rt_renderer *const *rs, uint32_t n, uint32_t iters) const {
    std::vector<unsigned char> s;
    put(s, iters);
    put(s, n);
    put(s, path.ro.p);
    put(s, path.counts.p);
    for (uint32_t j = 0; j < n; ++j) {
        const rt_renderer *r = rs[j];
        put(s, r);
        put(s, r->d_frame.p);
        put(s, r->d_pingpong.p);
        put(s, r->d_moments.p);
        put(s, r->d_gbuffer.p);
        put(s, r->d_accum.p);
        put(s, r->d_output.p);
        put(s, r->cfg.width);
        put(s, r->cfg.height);
        put(s, r->cfg.enable_denoise);
        put(s, r->cfg.enable_photon_map);  // picks the shade kernel's variant
        put(s, r->cfg.debug_view);
        put(s, r->cfg.denoise_passes);
        put(s, r->cfg.exposure);
        put(s, r->cfg.gamma);
        put(s, r->scene.stack_cap);
        put(s, r->scene.wnodes);  // picks the traversal kernels
        put(s, r->scene.wide_stack);
        put(s, r->glow);
        put(s, r->marker);
        put(s, base[j]);
    }
    put(s, tuning);
    return s;
}

int BatchEngine::enqueue(rt_renderer *const *rs, uint32_t n, uint32_t iters, const float *alpha, bool dev_alpha) {
    std::vector<rtd::JobShape> shapes(n);
    for (uint32_t j = 0; j < n; ++j) {
        const rt_renderer *r = rs[j];
        shapes[j] = rtd::JobShape{r->cfg.width, r->cfg.height, r->cfg.width * r->cfg.height, base[j],
                                  r->scene.stack_cap, r->cfg.enable_photon_map ? 1u : 0u,
                                  r->cfg.debug_view != 0u ? 1u : 0u, r->scene.wnodes ? 1u : 0u,
                                  r->scene.wide_stack};
    }
    const rtd::WaveParams wp = path.params(jobs.device(), n, counters.as<unsigned long long>());
    RT_CK(rtd::launch_wavefront(wp, shapes.data(), n, iters, num_sms, tuning, stream));
    // Each member's denoise and resolve on one of the side streams, joined back before the frame ends.
    const int k = n < (uint32_t)kSide ? (int)n : kSide;
    RT_CK(cudaEventRecord(fork, stream));
    for (int i = 0; i < k; ++i) RT_CK(cudaStreamWaitEvent(side[i], fork, 0));
    int st = RT_OK;
    for (uint32_t j = 0; j < n && st == RT_OK; ++j)
        st = rt::enqueue_post(rs[j], alpha[j], dev_alpha ? &jobs.device()[j].alpha : nullptr, side[j % k]);
    for (int i = 0; i < k; ++i) {  // joined even after a failure, so a capture can end
        RT_CK(cudaEventRecord(join[i], side[i]));
        RT_CK(cudaStreamWaitEvent(stream, join[i], 0));
    }
    return st;
}

int BatchEngine::frame(rt_renderer *const *rs, uint32_t n) {
    if (n == 0) return RT_OK;
    if (n > jobs.cap) {
        set_error("batch: %u jobs, the job table holds %zu", n, jobs.cap);
        return RT_ERR_INVALID_ARGUMENT;
    }
    // Work already queued on a member's own stream (set-up, photon rebuilds, solo frames) comes first.
    for (uint32_t j = 0; j < n; ++j) {
        RT_CK(cudaEventRecord(done, rs[j]->stream));
        RT_CK(cudaStreamWaitEvent(stream, done, 0));
    }
    std::vector<float> alpha(n);
    std::vector<rtd::DevJob> table(n);
    base.resize(n);
    uint32_t iters = 0;
    uint64_t slots = 0;
    for (uint32_t j = 0; j < n; ++j) {
        base[j] = (uint32_t)slots;
        slots += (uint64_t)rs[j]->cfg.width * rs[j]->cfg.height;
        iters = std::max(iters, rt::frame_iterations(rs[j]));
    }
    if (slots > 0xFFFFFFFFull) {
        set_error("batch: the jobs' pixels exceed 2^32");
        return RT_ERR_INVALID_ARGUMENT;
    }
    if (int st = reserve(slots, iters)) return st;
    uint32_t tile0 = 0;
    for (uint32_t j = 0; j < n; ++j) {
        alpha[j] = rt::prepare_frame(rs[j]);
        table[j] = rt::make_job(rs[j], base[j]);
        table[j].tile0 = tile0;  // the job's first tile in the frame's one generate launch
        tile0 += ((rs[j]->cfg.width + 7u) / 8u) * ((rs[j]->cfg.height + 3u) / 4u);
    }
    cudaEvent_t fe[2] = {nullptr, nullptr};
    for (auto &e : fe) RT_CK(ring.next(&e));
    if (fe[1]) RT_CK(cudaEventRecord(fe[0], stream));
    RT_CK(jobs.upload(table.data(), n, stream));
    bool replay = false;
    if (graph_mode != GraphMode::Off) {
        std::vector<unsigned char> sig = signature(rs, n, iters);
        if (exec && sig == this->sig) {
            replay = true;
        } else if (graph_mode == GraphMode::Always || sig == last_sig) {
            if (exec) {
                cudaGraphExecDestroy(exec);
                exec = nullptr;
            }
            cudaGraph_t g = nullptr;
            RT_CK(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
            int st = enqueue(rs, n, iters, alpha.data(), true);
            cudaError_t ce = cudaStreamEndCapture(stream, &g);
            if (st != RT_OK) {
                if (g) cudaGraphDestroy(g);
                return st;
            }
            RT_CK(ce);
            cudaError_t ie = cudaGraphInstantiate(&exec, g, 0);
            cudaGraphDestroy(g);
            RT_CK(ie);
            this->sig.swap(sig);
            captures += 1;
            replay = true;
        } else {
            last_sig.swap(sig);  // captured if the next frame has the same shape
        }
    }
    if (replay) RT_CK(cudaGraphLaunch(exec, stream));
    else if (int st = enqueue(rs, n, iters, alpha.data(), false)) return st;
    if (fe[1]) RT_CK(cudaEventRecord(fe[1], stream));
    // Later work on each member's own stream (read-backs, solo frames, destroy) waits for this frame.
    RT_CK(cudaEventRecord(done, stream));
    for (uint32_t j = 0; j < n; ++j) {
        RT_CK(cudaStreamWaitEvent(rs[j]->stream, done, 0));
        rs[j]->frames += 1;
    }
    frames += 1;
    return RT_OK;
}

int BatchEngine::stats(rt_frame_stats *out) {
    std::memset(out, 0, sizeof(*out));
    RT_CK(cudaStreamSynchronize(stream));
    unsigned long long ctr[2] = {0, 0};
    RT_CK(cudaMemcpy(ctr, counters.p, 16, cudaMemcpyDeviceToHost));
    out->frames = frames;
    out->segments = ctr[0];
    out->shadow_rays = ctr[1];
    out->graph_captures = captures;
    const size_t groups = ring.used / 2;
    for (size_t g = 0; g < groups; ++g) {
        float v = 0.0f;
        if (cudaEventElapsedTime(&v, ring.pool[2 * g], ring.pool[2 * g + 1]) == cudaSuccess)
            out->ms_frame_sum += v;
        else
            cudaGetLastError();
    }
    out->timed_frames = groups;
    ring.used = 0;
    return RT_OK;
}

int BatchEngine::autotune(rt_renderer *const *rs, uint32_t n, uint32_t trial_frames, float *best_ms) {
    if (n == 0) {
        set_error("batch autotune: no jobs");
        return RT_ERR_INVALID_ARGUMENT;
    }
    trial_frames = std::max(trial_frames, 1u);
    // Everything a frame changes: each member's image buffers and frame counters, the engine's
    // counters and frame count.  Saved here, restored after the trials.
    struct Saved {
        DevBuf buf[6];
        uint32_t sample_counter, frames_since_reset;
        uint64_t frames;
    };
    std::vector<Saved> saved(n);
    for (uint32_t j = 0; j < n; ++j) {
        rt_renderer *r = rs[j];
        const DevBuf *src[6] = {&r->d_frame, &r->d_pingpong, &r->d_moments, &r->d_gbuffer, &r->d_accum, &r->d_output};
        for (int k = 0; k < 6; ++k) {
            RT_CK(saved[j].buf[k].alloc(src[k]->bytes));
            RT_CK(cudaMemcpyAsync(saved[j].buf[k].p, src[k]->p, src[k]->bytes, cudaMemcpyDeviceToDevice, r->stream));
        }
        saved[j].sample_counter = r->sample_counter;
        saved[j].frames_since_reset = r->frames_since_reset;
        saved[j].frames = r->frames;
    }
    DevBuf saved_counters;
    RT_CK(saved_counters.alloc(counters.bytes));
    RT_CK(cudaMemcpyAsync(saved_counters.p, counters.p, counters.bytes, cudaMemcpyDeviceToDevice, stream));
    const uint64_t saved_frames = frames;
    const size_t saved_ring = ring.used;
    const GraphMode saved_mode = graph_mode;
    graph_mode = GraphMode::Off;

    // The stack the launches will need (four-wide records when every job's scene has them).
    uint32_t stack_two = 0, stack_four = 0;
    bool wide = n > 0;
    for (uint32_t j = 0; j < n; ++j) {
        stack_two = std::max(stack_two, rs[j]->scene.stack_cap);
        stack_four = std::max(stack_four, rs[j]->scene.wide_stack);
        wide = wide && rs[j]->scene.wnodes != nullptr;
    }
    const uint32_t stack_need = wide ? stack_four : stack_two;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    RT_CK(cudaEventCreate(&e0));
    RT_CK(cudaEventCreate(&e1));
    struct EvGuard {
        cudaEvent_t a, b;
        ~EvGuard() {
            cudaEventDestroy(a);
            cudaEventDestroy(b);
        }
    } evg{e0, e1};
    std::vector<std::pair<rtd::WaveTuning, float>> tried;
    auto measure = [&](rtd::WaveTuning t, float *ms) -> int {
        rtd::normalize_tuning(t, stack_need);
        for (auto &x : tried)
            if (std::memcmp(&x.first, &t, sizeof(t)) == 0) {
                *ms = x.second;
                return RT_OK;
            }
        tuning = t;
        RT_CK(cudaEventRecord(e0, stream));
        for (uint32_t f = 0; f < trial_frames; ++f)
            if (int st = frame(rs, n)) return st;
        RT_CK(cudaEventRecord(e1, stream));
        RT_CK(cudaEventSynchronize(e1));
        RT_CK(cudaEventElapsedTime(ms, e0, e1));
        tried.push_back({t, *ms});
        return RT_OK;
    };
    rtd::WaveTuning best = tuning;
    rtd::normalize_tuning(best, stack_need);
    float best_t = 0.0f;
    int st = measure(best, &best_t);
    // Coordinate descent, one pass over the launch-shape dimensions; a change is kept when it is
    // faster by more than 2% (frame-to-frame noise).
    const uint32_t blocks[] = {64u, 128u, 256u};
    const uint32_t per_sm[] = {2u, 4u, 6u, 8u, 12u, 16u, 24u, 32u};
    const uint32_t stacks[] = {32u, 48u, 64u};
    const uint32_t chunks[] = {32u, 64u, 128u, 256u};
    const uint32_t steps[] = {3u, 4u, 8u, 16u};
    const uint32_t refills[] = {0u, 8u, 12u};
    const uint32_t treelets[] = {0u, rtd::kTreeletRecords};
    const uint32_t shade_blocks[] = {4u, 5u, 6u};
    auto sweep = [&](uint32_t rtd::WaveTuning::*field, const uint32_t *vals, size_t nv) {
        for (size_t i = 0; i < nv && st == RT_OK; ++i) {
            rtd::WaveTuning t = best;
            t.*field = vals[i];
            float ms = 0.0f;
            st = measure(t, &ms);
            if (st == RT_OK && ms < best_t * 0.98f) {
                best = t;
                rtd::normalize_tuning(best, stack_need);
                best_t = ms;
            }
        }
    };
    sweep(&rtd::WaveTuning::block_threads, blocks, 3);
    sweep(&rtd::WaveTuning::blocks_per_sm, per_sm, 8);
    sweep(&rtd::WaveTuning::stack_entries, stacks, 3);
    sweep(&rtd::WaveTuning::chunk, chunks, 4);
    sweep(&rtd::WaveTuning::steps, steps, 4);
    sweep(&rtd::WaveTuning::refill_idle, refills, 3);
    sweep(&rtd::WaveTuning::treelet, treelets, 2);
    sweep(&rtd::WaveTuning::shade_blocks, shade_blocks, 3);
    tuning = best;
    graph_mode = saved_mode;

    // Undo the trial frames.
    for (uint32_t j = 0; j < n; ++j) {
        rt_renderer *r = rs[j];
        DevBuf *dst[6] = {&r->d_frame, &r->d_pingpong, &r->d_moments, &r->d_gbuffer, &r->d_accum, &r->d_output};
        for (int k = 0; k < 6; ++k)
            RT_CK(cudaMemcpyAsync(dst[k]->p, saved[j].buf[k].p, dst[k]->bytes, cudaMemcpyDeviceToDevice, r->stream));
        r->sample_counter = saved[j].sample_counter;
        r->frames_since_reset = saved[j].frames_since_reset;
        r->frames = saved[j].frames;
    }
    RT_CK(cudaMemcpyAsync(counters.p, saved_counters.p, counters.bytes, cudaMemcpyDeviceToDevice, stream));
    for (uint32_t j = 0; j < n; ++j) RT_CK(cudaStreamSynchronize(rs[j]->stream));
    RT_CK(cudaStreamSynchronize(stream));
    frames = saved_frames;
    ring.used = saved_ring;
    if (best_ms) *best_ms = best_t / (float)trial_frames;
    return st;
}

}  // namespace rt

namespace {

rtd::WaveTuning from_c(const rt_wavefront_tuning &t) {
    return rtd::WaveTuning{t.block_threads, t.blocks_per_sm, t.chunk,      t.steps,
                           t.stack_entries, t.treelet ? rtd::kTreeletRecords : 0u, t.shade_blocks,
                           t.refill_idle};
}

void to_c(const rtd::WaveTuning &t, rt_wavefront_tuning *out) {
    std::memset(out, 0, sizeof(*out));
    out->block_threads = t.block_threads;
    out->blocks_per_sm = t.blocks_per_sm;
    out->chunk = t.chunk;
    out->steps = t.steps;
    out->stack_entries = t.stack_entries;
    out->treelet = t.treelet ? 1u : 0u;
    out->shade_blocks = t.shade_blocks;
    out->refill_idle = t.refill_idle;
}

}  // namespace

struct rt_batch {
    std::vector<rt_renderer *> rs;
    rt::BatchEngine eng;
};

extern "C" int rt_batch_create(rt_renderer *const *renderers, uint32_t n, uint32_t use_graphs, rt_batch **out) {
    return rt::guarded("rt_batch_create", [&]() -> int {
        rt::clear_error();
        if (!out || !renderers || n == 0 || n > (1u << 15)) {
            set_error("rt_batch_create: need 1 .. 32768 renderers");
            return RT_ERR_INVALID_ARGUMENT;
        }
        *out = nullptr;
        rt_batch *b = new (std::nothrow) rt_batch();
        if (!b) {
            set_error("rt_batch_create: out of host memory");
            return RT_ERR_OUT_OF_MEMORY;
        }
        auto fail = [&](int st) {
            delete b;
            return st;
        };
        uint64_t slots = 0;
        for (uint32_t j = 0; j < n; ++j) {
            if (!renderers[j]) {
                set_error("rt_batch_create: renderer %u is null", j);
                return fail(RT_ERR_INVALID_ARGUMENT);
            }
            for (uint32_t k = 0; k < j; ++k)
                if (renderers[k] == renderers[j]) {
                    set_error("rt_batch_create: renderer %u appears twice", j);
                    return fail(RT_ERR_INVALID_ARGUMENT);
                }
            b->rs.push_back(renderers[j]);
            slots += (uint64_t)renderers[j]->cfg.width * renderers[j]->cfg.height;
            if (slots > 0xFFFFFFFFull) {
                set_error("rt_batch_create: the jobs' pixels exceed 2^32");
                return fail(RT_ERR_INVALID_ARGUMENT);
            }
        }
        if (int st = b->eng.init(n, use_graphs ? rt::GraphMode::Always : rt::GraphMode::Off)) return fail(st);
        *out = b;
        return RT_OK;
    });
}

extern "C" void rt_batch_destroy(rt_batch *b) { delete b; }

extern "C" int rt_batch_render_frame(rt_batch *b) {
    return rt::guarded("rt_batch_render_frame", [&]() -> int {
        if (!b) {
            set_error("rt_batch_render_frame: null batch");
            return RT_ERR_INVALID_ARGUMENT;
        }
        rt::clear_error();
        return b->eng.frame(b->rs.data(), (uint32_t)b->rs.size());
    });
}

extern "C" int rt_batch_render_frames(rt_batch *b, uint32_t n) {
    return rt::guarded("rt_batch_render_frames", [&]() -> int {
        for (uint32_t i = 0; i < n; ++i)
            if (int st = rt_batch_render_frame(b)) return st;
        return RT_OK;
    });
}

extern "C" int rt_batch_synchronize(rt_batch *b) {
    return rt::guarded("rt_batch_synchronize", [&]() -> int {
        if (!b) {
            set_error("rt_batch_synchronize: null batch");
            return RT_ERR_INVALID_ARGUMENT;
        }
        RT_CK(cudaStreamSynchronize(b->eng.stream));
        return RT_OK;
    });
}

extern "C" void *rt_batch_stream(rt_batch *b) { return b ? (void *)b->eng.stream : nullptr; }

extern "C" int rt_batch_get_stats(rt_batch *b, rt_frame_stats *out) {
    return rt::guarded("rt_batch_get_stats", [&]() -> int {
        if (!b || !out) {
            set_error("rt_batch_get_stats: null argument");
            return RT_ERR_INVALID_ARGUMENT;
        }
        return b->eng.stats(out);
    });
}

extern "C" int rt_batch_set_tuning(rt_batch *b, const rt_wavefront_tuning *t) {
    return rt::guarded("rt_batch_set_tuning", [&]() -> int {
        if (!b || !t) {
            set_error("rt_batch_set_tuning: null argument");
            return RT_ERR_INVALID_ARGUMENT;
        }
        b->eng.tuning = from_c(*t);
        rtd::normalize_tuning(b->eng.tuning, 0u);
        return RT_OK;
    });
}

extern "C" int rt_batch_get_tuning(rt_batch *b, rt_wavefront_tuning *t) {
    return rt::guarded("rt_batch_get_tuning", [&]() -> int {
        if (!b || !t) {
            set_error("rt_batch_get_tuning: null argument");
            return RT_ERR_INVALID_ARGUMENT;
        }
        to_c(b->eng.tuning, t);
        return RT_OK;
    });
}

extern "C" int rt_batch_autotune(rt_batch *b, uint32_t trial_frames, rt_wavefront_tuning *best, float *best_ms) {
    return rt::guarded("rt_batch_autotune", [&]() -> int {
        if (!b) {
            set_error("rt_batch_autotune: null batch");
            return RT_ERR_INVALID_ARGUMENT;
        }
        rt::clear_error();
        const int st = b->eng.autotune(b->rs.data(), (uint32_t)b->rs.size(), trial_frames, best_ms);
        if (best) to_c(b->eng.tuning, best);
        return st;
    });
}

extern "C" int rt_set_tuning(rt_renderer *r, const rt_wavefront_tuning *t) {
    return rt::guarded("rt_set_tuning", [&]() -> int {
        if (!r || !t) {
            set_error("rt_set_tuning: null argument");
            return RT_ERR_INVALID_ARGUMENT;
        }
        r->tuning = from_c(*t);
        rtd::normalize_tuning(r->tuning, 0u);
        return RT_OK;
    });
}

extern "C" int rt_get_tuning(const rt_renderer *r, rt_wavefront_tuning *t) {
    return rt::guarded("rt_get_tuning", [&]() -> int {
        if (!r || !t) {
            set_error("rt_get_tuning: null argument");
            return RT_ERR_INVALID_ARGUMENT;
        }
        to_c(r->tuning, t);
        return RT_OK;
    });
}
