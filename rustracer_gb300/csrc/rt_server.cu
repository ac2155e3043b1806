// The render-request loop: headless jobs of different scenes, resolutions, spp and accumulation
// budgets are admitted as they arrive and rendered together (continuous batching: the set of jobs in
// a batch frame changes from frame to frame as jobs arrive and reach their budgets).
//
// One worker thread owns every CUDA call of the server.  Each iteration it
//   1. retires finished frames (event queries): per-job frame counts, time to first frame, and jobs
//      that reached their budget give back their device memory (result copied out if asked for);
//   2. admits queued requests in arrival order while the job slots, the path slots and the HBM cap
//      allow, uploading the job's scene if it is not resident (idle scenes are evicted, least
//      recently used first, to make room) and creating the job's renderer on it;
//   3. launches the next batch frame over every admitted job whose set-up (photon map) is done and
//      whose budget is not yet enqueued, keeping up to `frames_in_flight` frames queued on the GPU.
// A job's renderer is created fresh on admission and renders its frames with the same per-pixel
// work as alone, so its image is the same alone and in any mix.  In plain mode the same loop admits
// one job at a time and renders its frames alone, with the launches of rt_render_frame: the
// one-job-at-a-time baseline.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <new>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "rt_batch_engine.h"

using rt::set_error;

namespace {

using Clock = std::chrono::steady_clock;

struct SceneEntry {
    rt_scene_desc desc{};            // borrowed until the server is destroyed
    rt_resident_scene *res = nullptr;
    uint64_t bytes = 0;              // exact while resident, else an estimate from the description
    uint32_t active = 0;             // admitted jobs rendering on it
    uint64_t last_used = 0;          // LRU tick
};

struct Job {
    uint64_t id = 0;
    rt_request req{};
    uint32_t state = RT_JOB_QUEUED;
    rt_renderer *r = nullptr;
    cudaEvent_t ready = nullptr;     // set-up (photon map) done
    bool is_ready = false;
    uint32_t enqueued = 0, done = 0; // frames launched / finished
    uint64_t bytes = 0;              // device bytes charged to the cap
    uint64_t npix = 0;
    double t_submit = 0, t_admit = -1, t_first = -1, t_done = -1;
    std::vector<float> result;
    std::string error;
};

struct Flight {
    cudaEvent_t ev = nullptr;
    std::vector<Job *> jobs;
};

uint64_t scene_estimate(const rt_scene_desc &d) {
    // two-wide records (at most one per node) and four-wide records (at most 128 B per two nodes)
    uint64_t b = d.triangle_count * 128 + d.bvh_node_count * 128 + d.bvh_prim_count * 48 + d.material_count * 64 + 64;
    const rt_texture_array *t[4] = {&d.tex_albedo, &d.tex_mr, &d.tex_emissive, &d.tex_normal};
    for (auto *x : t)
        if (x->rgba8) b += (uint64_t)x->width * x->height * x->layers * 4;
    return b;
}

}  // namespace

struct rt_server {
    rt_server_config cfg{};
    int device = 0;
    Clock::time_point t0;
    std::mutex mu;
    std::condition_variable cv;
    std::deque<Job *> pending;                               // under mu
    std::unordered_map<uint64_t, std::unique_ptr<Job>> jobs; // under mu
    std::map<uint32_t, SceneEntry> scenes;                   // entries added under mu before any submit uses them
    uint64_t next_id = 1;
    bool stop = false;
    // Set (under mu) when the worker thread ran out of host memory: later submits are refused.
    bool broken = false;
    std::string broken_msg;
    rt_server_stats st{};                                    // under mu
    // worker-only state
    std::vector<Job *> active;
    std::deque<Flight> flights;
    std::vector<cudaEvent_t> spare_events;
    rt::BatchEngine eng;
    uint64_t tick = 0;
    uint64_t path_bytes = 0;
    std::thread worker;

    double now_ms() const { return std::chrono::duration<double, std::milli>(Clock::now() - t0).count(); }
    bool plain() const { return cfg.mode == RT_SERVER_PLAIN; }
};

namespace {

cudaError_t take_event(rt_server *s, cudaEvent_t *ev) {
    if (!s->spare_events.empty()) {
        *ev = s->spare_events.back();
        s->spare_events.pop_back();
        return cudaSuccess;
    }
    return cudaEventCreateWithFlags(ev, cudaEventDisableTiming);
}

// Adds `delta` device bytes to the server's account (under mu).
void charge_locked(rt_server *s, int64_t delta) {
    s->st.used_bytes = (uint64_t)((int64_t)s->st.used_bytes + delta);
    s->st.peak_bytes = std::max(s->st.peak_bytes, s->st.used_bytes);
}

SceneEntry &scene_of(rt_server *s, uint32_t id) {
    std::lock_guard<std::mutex> lk(s->mu);  // entries are stable; the map may grow under add_scene
    return s->scenes.find(id)->second;
}

void fail_job(rt_server *s, Job *j, const char *what) {
    std::lock_guard<std::mutex> lk(s->mu);
    j->state = RT_JOB_FAILED;
    j->error = what ? what : "";
    j->t_done = s->now_ms();
    s->st.failed += 1;
}

// A job that reached its budget (or failed after admission): result out, device memory back.
void retire(rt_server *s, Job *j, bool ok) {
    if (ok && j->req.keep_result && j->r) {
        j->result.resize(j->npix * 4);
        if (rt_read_accumulation(j->r, j->result.data(), j->result.size()) != RT_OK) {
            ok = false;
            j->result.clear();
        }
    }
    if (j->r) rt_renderer_destroy(j->r);  // waits for the job's queued work
    j->r = nullptr;
    if (j->ready) s->spare_events.push_back(j->ready);
    j->ready = nullptr;
    s->active.erase(std::remove(s->active.begin(), s->active.end(), j), s->active.end());
    SceneEntry &e = scene_of(s, j->req.scene_id);
    e.active -= 1;
    e.last_used = ++s->tick;
    std::lock_guard<std::mutex> lk(s->mu);
    charge_locked(s, -(int64_t)j->bytes);
    j->bytes = 0;
    s->st.active = (uint32_t)s->active.size();
    if (ok) {
        j->state = RT_JOB_DONE;
        s->st.completed += 1;
    } else if (j->state != RT_JOB_FAILED) {
        j->state = RT_JOB_FAILED;
        j->error = rt_last_error();
        j->t_done = s->now_ms();
        s->st.failed += 1;
    }
}

// Retires the oldest frame in flight if it has finished (or after waiting for it when `block`).
bool complete_front(rt_server *s, bool block) {
    if (s->flights.empty()) return false;
    Flight &f = s->flights.front();
    const cudaError_t err = block ? cudaEventSynchronize(f.ev) : cudaEventQuery(f.ev);
    if (err == cudaErrorNotReady) return false;
    const double t = s->now_ms();
    std::vector<Job *> finished;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        for (Job *j : f.jobs) {
            j->done += 1;
            s->st.job_frames += 1;
            if (j->done == 1) j->t_first = t;
            if (j->done >= j->req.budget_frames) {
                j->t_done = t;
                finished.push_back(j);
            }
        }
    }
    s->spare_events.push_back(f.ev);
    s->flights.pop_front();
    if (err != cudaSuccess) set_error("server: a batch frame failed: %s", cudaGetErrorString(err));
    for (Job *j : finished) retire(s, j, err == cudaSuccess);
    return true;
}

// Frees idle resident scenes, least recently used first, until `need` more bytes fit under the cap.
bool make_room(rt_server *s, uint64_t need, uint32_t keep_scene) {
    for (;;) {
        uint64_t used;
        {
            std::lock_guard<std::mutex> lk(s->mu);
            used = s->st.used_bytes;
        }
        if (used + need <= s->cfg.hbm_cap_bytes) return true;
        SceneEntry *victim = nullptr;
        {
            std::lock_guard<std::mutex> lk(s->mu);
            for (auto &kv : s->scenes) {
                SceneEntry &e = kv.second;
                if (!e.res || e.active || kv.first == keep_scene) continue;
                if (!victim || e.last_used < victim->last_used) victim = &e;
            }
        }
        if (!victim) return false;
        const uint64_t b = victim->bytes;
        rt::resident_scene_release(victim->res);
        victim->res = nullptr;
        victim->bytes = scene_estimate(victim->desc);
        std::lock_guard<std::mutex> lk(s->mu);
        charge_locked(s, -(int64_t)b);
        s->st.resident_scene_bytes -= b;
        s->st.resident_scenes -= 1;
        s->st.scene_evictions += 1;
    }
}

// Admits the request at the head of the queue if it fits; true if the queue changed.
bool admit(rt_server *s) {
    Job *j = nullptr;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        if (s->pending.empty()) return false;
        j = s->pending.front();
    }
    if (s->active.size() >= s->cfg.max_jobs) return false;
    uint64_t slots = 0;
    for (Job *a : s->active) slots += a->npix;
    if (slots + j->npix > s->cfg.max_slots) {
        if (!s->active.empty()) return false;
        {
            std::lock_guard<std::mutex> lk(s->mu);
            s->pending.pop_front();
        }
        fail_job(s, j, "the job's pixels exceed the server's path slots");
        return true;
    }
    SceneEntry &e = scene_of(s, j->req.scene_id);
    // Device bytes of the job: its renderer, plus (plain mode) the path state of its solo frames.
    rt_grid_params gp;
    float radius = j->req.config.photon_radius;
    const rt_render_config &c = j->req.config;
    const uint64_t slots_ph = c.enable_photon_map ? std::max<uint64_t>((uint64_t)c.photon_count * RT_MAX_BOUNCES, 1) : 1;
    rt_derive_grid(e.desc.bounds_min, e.desc.bounds_max, (int)e.desc.has_bounds, c.grid_max_dim,
                   c.photon_radius_mode, (uint32_t)slots_ph, &gp, &radius);
    // (a photon rebuild adds the renderer's one-entry job table)
    const uint64_t job_bytes = rt::renderer_create_bytes(c, gp.num_cells, e.desc.light_count) +
                               (c.enable_photon_map ? sizeof(rtd::DevJob) : 0u);
    const uint64_t need = job_bytes + (e.res ? 0 : e.bytes);
    if (!make_room(s, need, j->req.scene_id)) {
        if (!s->active.empty() || !s->flights.empty()) return false;  // wait for running jobs to finish
        {
            std::lock_guard<std::mutex> lk(s->mu);
            s->pending.pop_front();
        }
        fail_job(s, j, "the job and its scene do not fit under the HBM cap");
        return true;
    }
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->pending.pop_front();
        j->state = RT_JOB_RUNNING;
        j->t_admit = s->now_ms();
        j->bytes = job_bytes;
        s->st.admitted += 1;
        charge_locked(s, (int64_t)job_bytes);
        s->st.pending = (uint32_t)s->pending.size();
    }
    e.active += 1;
    e.last_used = ++s->tick;
    s->active.push_back(j);
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->st.active = (uint32_t)s->active.size();
        s->st.max_active = std::max(s->st.max_active, s->st.active);
    }
    if (!e.res) {
        rt_resident_scene *res = nullptr;
        if (rt::resident_scene_create(&e.desc, &res) != RT_OK) {
            fail_job(s, j, rt_last_error());
            retire(s, j, false);
            return true;
        }
        e.res = res;
        e.bytes = res->bytes;
        std::lock_guard<std::mutex> lk(s->mu);
        charge_locked(s, (int64_t)e.bytes);
        s->st.resident_scene_bytes += e.bytes;
        s->st.resident_scenes += 1;
        s->st.scene_uploads += 1;
    }
    if (rt_renderer_create_resident(e.res, &c, &j->r) != RT_OK ||
        rt_update_camera(j->r, &j->req.camera) != RT_OK ||
        (c.enable_photon_map && rt::enqueue_photon_rebuild(j->r) != RT_OK) || take_event(s, &j->ready) != cudaSuccess ||
        cudaEventRecord(j->ready, j->r->stream) != cudaSuccess) {
        fail_job(s, j, rt_last_error());
        retire(s, j, false);
        return true;
    }
    return true;
}

// Launches the next frame over the admitted jobs that are ready; true if one was launched.
bool launch(rt_server *s) {
    if (s->flights.size() >= s->cfg.frames_in_flight) return false;
    std::vector<rt_renderer *> rs;
    std::vector<Job *> members;
    for (Job *j : s->active) {
        if (j->enqueued >= j->req.budget_frames) continue;
        if (!j->is_ready) {
            if (cudaEventQuery(j->ready) != cudaSuccess) {
                cudaGetLastError();
                continue;
            }
            j->is_ready = true;
        }
        members.push_back(j);
        rs.push_back(j->r);
    }
    if (members.empty()) return false;
    Flight f;
    if (take_event(s, &f.ev) != cudaSuccess) return false;
    const int st = s->eng.frame(rs.data(), (uint32_t)rs.size());
    if (st != RT_OK || cudaEventRecord(f.ev, s->eng.stream) != cudaSuccess) {
        s->spare_events.push_back(f.ev);
        const std::string msg = rt_last_error();
        for (Job *j : members) {
            fail_job(s, j, msg.c_str());
            retire(s, j, false);
        }
        return true;
    }
    for (Job *j : members) j->enqueued += 1;
    f.jobs = members;
    s->flights.push_back(std::move(f));
    std::lock_guard<std::mutex> lk(s->mu);
    s->st.batch_frames += 1;
    s->st.graph_captures = s->eng.captures;
    return true;
}

void worker_loop(rt_server *s) {
    for (;;) {
        {
            std::lock_guard<std::mutex> lk(s->mu);
            if (s->stop) break;
        }
        bool progress = false;
        while (complete_front(s, false)) progress = true;
        while (admit(s)) progress = true;
        if (launch(s)) progress = true;
        if (progress) continue;
        if (!s->flights.empty()) {
            complete_front(s, true);
            continue;
        }
        // Nothing in flight: wait for a job's set-up, or for a request.
        Job *setup = nullptr;
        for (Job *j : s->active)
            if (!j->is_ready) setup = j;
        if (setup) {
            cudaEventSynchronize(setup->ready);
            continue;
        }
        std::unique_lock<std::mutex> lk(s->mu);
        if (s->stop) break;
        if (s->pending.empty()) s->cv.wait_for(lk, std::chrono::milliseconds(20));
        if (s->stop) break;
    }
    while (complete_front(s, true)) {
    }
}

// After the worker loop threw: waits for the frames in flight and fails every job not yet done, so
// that rt_server_wait_idle returns and each job's status says why.
void fail_everything(rt_server *s, const char *why) {
    for (Flight &f : s->flights) cudaEventSynchronize(f.ev);
    for (Flight &f : s->flights) cudaEventDestroy(f.ev);
    s->flights.clear();
    for (Job *j : std::vector<Job *>(s->active)) {
        fail_job(s, j, why);
        retire(s, j, false);
    }
    std::lock_guard<std::mutex> lk(s->mu);
    for (Job *j : s->pending) {
        j->state = RT_JOB_FAILED;
        j->error = why;
        j->t_done = s->now_ms();
        s->st.failed += 1;
    }
    s->pending.clear();
}

void worker_main(rt_server *s) {
    cudaSetDevice(s->device);
    try {
        worker_loop(s);
        return;
    } catch (const std::exception &e) {
        std::lock_guard<std::mutex> lk(s->mu);
        s->broken = true;
        s->broken_msg = std::string("server worker stopped: ") + e.what();
    }
    try {
        fail_everything(s, s->broken_msg.c_str());
    } catch (const std::exception &) {
        // nothing more can be freed without host memory; destroy releases the rest
    }
}

}  // namespace

extern "C" int rt_server_create(const rt_server_config *cfg, rt_server **out) {
    return rt::guarded("rt_server_create", [&]() -> int {
        rt::clear_error();
        if (!out) {
            set_error("rt_server_create: null argument");
            return RT_ERR_INVALID_ARGUMENT;
        }
        *out = nullptr;
        if (rt_device_count() <= 0) {
            set_error("rt_server_create: no CUDA device is visible");
            return RT_ERR_CUDA;
        }
        rt_server *s = new (std::nothrow) rt_server();
        if (!s) {
            set_error("rt_server_create: out of host memory");
            return RT_ERR_OUT_OF_MEMORY;
        }
        if (cfg) s->cfg = *cfg;
        if (s->cfg.mode > RT_SERVER_PLAIN) {
            delete s;
            set_error("rt_server_create: mode must be RT_SERVER_BATCHED or RT_SERVER_PLAIN");
            return RT_ERR_INVALID_ARGUMENT;
        }
        if (!s->cfg.hbm_cap_bytes) s->cfg.hbm_cap_bytes = 120ull << 30;
        if (!s->cfg.max_jobs) s->cfg.max_jobs = 64;
        if (!s->cfg.max_slots) s->cfg.max_slots = 1u << 25;
        if (!s->cfg.frames_in_flight) s->cfg.frames_in_flight = 2;
        cudaGetDevice(&s->device);
        s->t0 = Clock::now();
        if (s->plain()) {
            s->cfg.max_jobs = 1;
            s->cfg.graphs = 0;
        }
        const rt::GraphMode gm = s->cfg.graphs ? rt::GraphMode::OnRepeat : rt::GraphMode::Off;
        int st = s->eng.init(s->cfg.max_jobs, gm);
        const rt_wavefront_tuning &tc = s->cfg.tuning;
        if (tc.block_threads | tc.blocks_per_sm | tc.chunk | tc.steps | tc.stack_entries) {
            s->eng.tuning = rtd::WaveTuning{tc.block_threads, tc.blocks_per_sm, tc.chunk,
                                            tc.steps,         tc.stack_entries, tc.treelet ? rtd::kTreeletRecords : 0u,
                                            tc.shade_blocks, tc.refill_idle};
            rtd::normalize_tuning(s->eng.tuning, 0u);
        }
        if (st == RT_OK) st = s->eng.reserve(s->cfg.max_slots, 64);
        if (st != RT_OK) {
            delete s;
            return st;
        }
        s->path_bytes = rt::path_state_bytes(s->cfg.max_slots, 64);
        charge_locked(s, (int64_t)s->path_bytes);
        try {
            s->worker = std::thread(worker_main, s);
        } catch (...) {
            delete s;
            throw;
        }
        *out = s;
        return RT_OK;
    });
}

extern "C" void rt_server_destroy(rt_server *s) {
    if (!s) return;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
    }
    s->cv.notify_all();
    if (s->worker.joinable()) s->worker.join();
    cudaSetDevice(s->device);
    for (Job *j : std::vector<Job *>(s->active)) retire(s, j, false);
    for (auto &kv : s->scenes)
        if (kv.second.res) rt::resident_scene_release(kv.second.res);
    for (cudaEvent_t e : s->spare_events) cudaEventDestroy(e);
    delete s;
}

extern "C" int rt_server_add_scene(rt_server *s, uint32_t scene_id, const rt_scene_desc *desc) {
    return rt::guarded("rt_server_add_scene", [&]() -> int {
        rt::clear_error();
        if (!s || !desc) {
            set_error("rt_server_add_scene: null argument");
            return RT_ERR_INVALID_ARGUMENT;
        }
        if ((desc->triangle_count && !desc->triangles) || (desc->bvh_node_count && !desc->bvh_nodes) ||
            (desc->bvh_prim_count && !desc->bvh_prims) || (desc->material_count && !desc->materials) ||
            (desc->light_count && !desc->lights)) {
            set_error("rt_server_add_scene: scene array pointer is null with a non-zero count");
            return RT_ERR_INVALID_ARGUMENT;
        }
        std::lock_guard<std::mutex> lk(s->mu);
        if (s->scenes.count(scene_id)) {
            set_error("rt_server_add_scene: scene %u is already registered", scene_id);
            return RT_ERR_INVALID_ARGUMENT;
        }
        SceneEntry &e = s->scenes[scene_id];
        e.desc = *desc;
        e.bytes = scene_estimate(*desc);
        return RT_OK;
    });
}

extern "C" int rt_server_submit(rt_server *s, const rt_request *req, uint64_t *job_id) {
    return rt::guarded("rt_server_submit", [&]() -> int {
        rt::clear_error();
        if (!s || !req) {
            set_error("rt_server_submit: null argument");
            return RT_ERR_INVALID_ARGUMENT;
        }
        const rt_render_config &c = req->config;
        if (c.width == 0 || c.height == 0 || (uint64_t)c.width * c.height > (1ull << 28) || req->budget_frames == 0) {
            set_error("rt_server_submit: width, height and budget_frames must be non-zero (width*height <= 2^28)");
            return RT_ERR_INVALID_ARGUMENT;
        }
        if (c.enable_photon_map && (uint64_t)c.photon_count * RT_MAX_BOUNCES > 0xFFFFFFFFull) {
            set_error("rt_server_submit: photon_count * 6 must fit in 32 bits");
            return RT_ERR_INVALID_ARGUMENT;
        }
        std::unique_ptr<Job> j(new (std::nothrow) Job());
        if (!j) {
            set_error("rt_server_submit: out of host memory");
            return RT_ERR_OUT_OF_MEMORY;
        }
        {
            std::lock_guard<std::mutex> lk(s->mu);
            if (s->broken) {
                set_error("rt_server_submit: %s", s->broken_msg.c_str());
                return RT_ERR_STATE;
            }
            if (!s->scenes.count(req->scene_id)) {
                set_error("rt_server_submit: scene %u is not registered", req->scene_id);
                return RT_ERR_INVALID_ARGUMENT;
            }
            Job *raw = j.get();
            raw->id = s->next_id++;
            raw->req = *req;
            raw->npix = (uint64_t)c.width * c.height;
            raw->t_submit = s->now_ms();
            s->jobs.emplace(raw->id, std::move(j));
            try {
                s->pending.push_back(raw);
            } catch (...) {
                s->jobs.erase(raw->id);
                throw;
            }
            if (job_id) *job_id = raw->id;
            s->st.submitted += 1;
            s->st.pending = (uint32_t)s->pending.size();
        }
        s->cv.notify_all();
        return RT_OK;
    });
}

extern "C" int rt_server_job_status(rt_server *s, uint64_t job_id, rt_job_status *out) {
    return rt::guarded("rt_server_job_status", [&]() -> int {
        if (!s || !out) {
            set_error("rt_server_job_status: null argument");
            return RT_ERR_INVALID_ARGUMENT;
        }
        std::lock_guard<std::mutex> lk(s->mu);
        auto it = s->jobs.find(job_id);
        if (it == s->jobs.end()) {
            set_error("rt_server_job_status: no job %llu", (unsigned long long)job_id);
            return RT_ERR_INVALID_ARGUMENT;
        }
        const Job &j = *it->second;
        std::memset(out, 0, sizeof(*out));
        out->job_id = j.id;
        out->state = j.state;
        out->frames_done = j.done;
        out->t_submit_ms = j.t_submit;
        out->t_admit_ms = j.t_admit;
        out->t_first_frame_ms = j.t_first;
        out->t_done_ms = j.t_done;
        return RT_OK;
    });
}

extern "C" int rt_server_read_result(rt_server *s, uint64_t job_id, float *rgba, uint64_t n_floats) {
    return rt::guarded("rt_server_read_result", [&]() -> int {
        if (!s || !rgba) {
            set_error("rt_server_read_result: null argument");
            return RT_ERR_INVALID_ARGUMENT;
        }
        std::lock_guard<std::mutex> lk(s->mu);
        auto it = s->jobs.find(job_id);
        if (it == s->jobs.end()) {
            set_error("rt_server_read_result: no job %llu", (unsigned long long)job_id);
            return RT_ERR_INVALID_ARGUMENT;
        }
        const Job &j = *it->second;
        if (j.state != RT_JOB_DONE || !j.req.keep_result) {
            set_error("rt_server_read_result: job %llu is not done or was submitted without keep_result",
                      (unsigned long long)job_id);
            return RT_ERR_STATE;
        }
        if (n_floats != j.result.size()) {
            set_error("rt_server_read_result: %llu floats given, the result has %llu", (unsigned long long)n_floats,
                      (unsigned long long)j.result.size());
            return RT_ERR_INVALID_ARGUMENT;
        }
        std::memcpy(rgba, j.result.data(), n_floats * sizeof(float));
        return RT_OK;
    });
}

extern "C" int rt_server_release_job(rt_server *s, uint64_t job_id) {
    return rt::guarded("rt_server_release_job", [&]() -> int {
        if (!s) {
            set_error("rt_server_release_job: null server");
            return RT_ERR_INVALID_ARGUMENT;
        }
        std::lock_guard<std::mutex> lk(s->mu);
        auto it = s->jobs.find(job_id);
        if (it == s->jobs.end()) {
            set_error("rt_server_release_job: no job %llu", (unsigned long long)job_id);
            return RT_ERR_INVALID_ARGUMENT;
        }
        if (it->second->state != RT_JOB_DONE && it->second->state != RT_JOB_FAILED) {
            set_error("rt_server_release_job: job %llu is still queued or running", (unsigned long long)job_id);
            return RT_ERR_STATE;
        }
        s->jobs.erase(it);
        return RT_OK;
    });
}

extern "C" int rt_server_wait_idle(rt_server *s, uint32_t timeout_ms) {
    return rt::guarded("rt_server_wait_idle", [&]() -> int {
        if (!s) {
            set_error("rt_server_wait_idle: null server");
            return RT_ERR_INVALID_ARGUMENT;
        }
        const auto end = Clock::now() + std::chrono::milliseconds(timeout_ms);
        for (;;) {
            {
                std::lock_guard<std::mutex> lk(s->mu);
                if (s->st.completed + s->st.failed == s->st.submitted) return RT_OK;
            }
            if (Clock::now() >= end) {
                set_error("rt_server_wait_idle: jobs still queued or running after %u ms", timeout_ms);
                return RT_ERR_STATE;
            }
            std::this_thread::sleep_for(std::chrono::microseconds(500));
        }
    });
}

extern "C" int rt_server_get_stats(rt_server *s, rt_server_stats *out) {
    return rt::guarded("rt_server_get_stats", [&]() -> int {
        if (!s || !out) {
            set_error("rt_server_get_stats: null argument");
            return RT_ERR_INVALID_ARGUMENT;
        }
        unsigned long long ctr[2] = {0, 0};
        if (s->eng.counters.p) {
            // a snapshot of the batch counters (kernels may be adding to them)
            if (cudaMemcpy(ctr, s->eng.counters.p, 16, cudaMemcpyDeviceToHost) != cudaSuccess) {
                set_error("rt_server_get_stats: reading the counters failed");
                return RT_ERR_CUDA;
            }
        }
        std::lock_guard<std::mutex> lk(s->mu);
        *out = s->st;
        out->segments = ctr[0];
        out->shadow_rays = ctr[1];
        out->pending = (uint32_t)s->pending.size();
        return RT_OK;
    });
}

extern "C" double rt_server_now_ms(const rt_server *s) { return s ? s->now_ms() : 0.0; }
