"""Benchmark of the per-frame hot path: path segments per second.

Workload (default, `icosphere1080p`): displaced icosphere, subdivision level 8 (1,310,720 triangles,
radius 1, per-vertex normal displacement N(0, 0.02)) in a 10^3 Lambertian room, seeded per-triangle
materials (60% Lambertian, 25% GGX metal, 15% dielectric), 1024^2 rgba8 albedo / MR / normal value-noise
textures, one 1x1 area light (emission 20) and 4 seeded point lights; 1920x1080, 4 spp per frame,
depth 8, NEE on, no photon map, no denoise; accumulation over 32 frames.  A step is one progressive
frame (gather, then composite + tonemap).  Synthetic, seeded inputs; the scene (~330 MB on the device)
is larger than L2, so no L2 flush is needed between steps.

Metric: segments/s, a segment being one closest-hit BVH trace on a camera or bounce path (shadow
rays are reported separately).  `value` is device-timed with CUDA events on the renderer's stream;
`e2e` is the same metric through the public API with host buffers (camera in, rgba8 frame out into
pinned memory) timed on the host clock.

`--impl reference` times the reference's CPU restatement (the oracle: the Rust/WGSL reference needs
wgpu and a graphics stack, which this machine does not have) on the host cores, on bounded samples
(row bands) of the same frames.

Launch: python bench.py [--gpus N --steps K --warmup W] ; N > 1 under torch.distributed.run, one
independent render job per GPU (weak scaling, no collective on the data path).
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

import numpy as np  # noqa: E402

WORKLOADS = {
    "icosphere1080p": dict(scene="icosphere", level=8, seed=0, sigma=0.02, tex=1024, width=1920, height=1080, spp=4,
                           max_bounces=8, accumulate_frames=32, denoise=False, photons=0),
    # the same scene at 480x270 (for profiler captures of one gather launch)
    "icosphere270p": dict(scene="icosphere", level=8, seed=0, sigma=0.02, tex=1024, width=480, height=270, spp=4,
                          max_bounces=8, accumulate_frames=32, denoise=False, photons=0),
    "cornell256": dict(scene="cornell", width=256, height=256, spp=1, max_bounces=6, accumulate_frames=16,
                       denoise=False, photons=0),
}


def measured_peaks() -> dict:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            return json.loads(p.read_text())
        except Exception:
            pass
    return {}


def hbm_peak() -> tuple[float, str]:
    pk = measured_peaks()
    if "hbm_gbs" in pk:
        return float(pk["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index: int):
        self.dev = device_index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.dev}", f"--query-gpu={self.QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.fh,
                                         stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self) -> dict | None:
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.fh.close()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in Path(self.path).read_text().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        os.unlink(self.path)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "samples": len(sm),
                "reasons": sorted(reasons)}


def job_totals(dist, elapsed: float, *counts: float, device: str = "cpu") -> tuple:
    """Whole-job figures of a weak-scaling run: the slowest rank's elapsed time and the per-rank counts
    summed over ranks (all-reduce MAX and SUM; no reduction without a process group)."""
    import torch

    t = torch.tensor([elapsed, *counts], dtype=torch.float64, device=device)
    if dist is None:
        return tuple(float(x) for x in t)
    tmax = t.clone()
    dist.all_reduce(tmax, op=dist.ReduceOp.MAX)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return (float(tmax[0]),) + tuple(float(x) for x in t[1:])


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def make_scene(w: dict):
    import rustracer_gb300 as rt

    if w["scene"] == "cornell":
        return rt.Scene.cornell555()
    return rt.Scene.icosphere_room(w["level"], w["seed"], w["sigma"], w["tex"])


def make_config(w: dict):
    import rustracer_gb300 as rt

    return rt.RenderConfig(width=w["width"], height=w["height"], spp=w["spp"], accumulate_frames=w["accumulate_frames"],
                           enable_denoise=w["denoise"], enable_photon_map=bool(w["photons"]),
                           photon_count=max(w["photons"], 1), max_bounces=w["max_bounces"])


# ------------------------------------------------------------------------------------------------
# CPU legs (oracle): bounded samples of the same frames.  They load only the oracle: the scene is
# the one the oracle generates and indexes itself (byte-identical to the backend's, checked by
# tests/test_oracle_scene.py), so no product code runs on the reference's path.
# ------------------------------------------------------------------------------------------------
def oracle_workload(w: dict):
    """(oracle scene, oracle config) of a workload."""
    import oracle

    if w["scene"] == "cornell":
        scene = oracle.OracleScene.cornell555()
    else:
        scene = oracle.OracleScene.icosphere_room(w["level"], w["seed"], w["sigma"], w["tex"])
    cfg = oracle.Config(width=w["width"], height=w["height"], spp=w["spp"], accumulate_frames=w["accumulate_frames"],
                        enable_denoise=w["denoise"], enable_photon_map=bool(w["photons"]),
                        photon_count=max(w["photons"], 1), max_bounces=w["max_bounces"])
    return scene, cfg


def cpu_sample(scene, cfg, seconds: float, threads: int, frames: int = 1):
    """Times the oracle on row bands of `frames` consecutive frames of its own scene (default
    camera), sized to ~`seconds` in total.  Returns (segments/s, sample description, per-ray work
    counters)."""
    import oracle

    c = scene.camera()
    u = oracle.camera_uniform(tuple(c.position), tuple(c.look_at), tuple(c.up), c.fov_degrees, cfg.width, cfg.height,
                              c.near_plane, c.aperture, c.focus_dist)
    o = oracle.OracleRenderer(scene, cfg, u, threads=threads)
    # calibrate on a small band
    rows = max(1, min(cfg.height, 4 * max(threads, 1)))
    t0 = time.perf_counter()
    o.sample_counter = 0
    _gather_rows(o, (cfg.height // 2 - rows // 2, cfg.height // 2 - rows // 2 + rows))
    dt = time.perf_counter() - t0
    per_row = dt / rows
    rows_total = int(max(1, min(cfg.height, seconds / max(per_row, 1e-6) / max(frames, 1))))
    # eight bands spread evenly over the frame, so that the per-ray work counts are the frame's
    n_bands = min(8, rows_total)
    band = max(1, rows_total // n_bands)
    starts = [int(round((i + 0.5) * cfg.height / n_bands - band / 2)) for i in range(n_bands)]
    starts = [min(max(0, y), cfg.height - band) for y in starts]
    o.counters[:] = 0
    t0 = time.perf_counter()
    for f in range(frames):
        for i, y in enumerate(starts):
            _gather_rows(o, (y, y + band), new_frame=i == 0)
    dt = time.perf_counter() - t0
    c = o.counters.astype(np.float64)
    seg = c[0]
    desc = (f"{n_bands} bands of {band} rows ({n_bands * band} of {cfg.height}) of {frames} frame(s) of "
            f"{cfg.width}x{cfg.height}, spp {cfg.spp}, depth {cfg.max_bounces or 6} ({int(seg)} segments in "
            f"{dt:.1f} s)")
    rays = max(c[0] + c[1], 1.0)
    work = {"nodes_per_ray": c[2] / rays, "tris_per_ray": c[3] / rays, "hit_fraction": c[4] / max(c[0], 1.0),
            "shadow_per_segment": c[1] / max(c[0], 1.0)}
    return seg / dt, desc, work


def _gather_rows(o, rows, new_frame: bool = True):
    """One gather dispatch of the oracle over a row band (the CPU cost of the frame); new_frame
    advances the frame counter first."""
    import ctypes as C

    import oracle

    if new_frame:
        o.sample_counter += 1
        o.frames_since_reset += 1
    ip = o.image_params(o.alpha())
    mb = o.cfg.max_bounces or 6
    oracle.load().oracle_gather(C.cast(C.pointer(o.desc), C.c_void_p), C.byref(o.cam), C.byref(ip), mb,
                                C.byref(o.gp), None, len(o.sorted), None, rows[0], rows[1], o.threads,
                                oracle._p(o.frame), oracle._p(o.moments), oracle._p(o.gbuffer), oracle._p(o.counters))


def run_reference(args, w):
    rank, world, local = dist_env()
    if rank != 0:
        return 0
    threads = os.cpu_count() or 1
    scene, cfg = oracle_workload(w)
    # warm-up samples, then K timed samples (one row band each)
    per_step = max(0.05, min(20.0, args.ref_seconds / max(args.steps + args.warmup, 1)))
    for _ in range(args.warmup):
        cpu_sample(scene, cfg, per_step / 4, threads)
    vals, descs = [], []
    t_all = time.perf_counter()
    for _ in range(args.steps):
        v, d, _ = cpu_sample(scene, cfg, per_step, threads)
        vals.append(v)
        descs.append(d)
    wall = time.perf_counter() - t_all
    value = float(np.mean(vals))
    line = {"impl": "reference", "metric": "segments/s", "value": value, "unit": "segments/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * wall / max(args.steps, 1),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": args.workload, **{k: v for k, v in w.items()}, "l2": "inputs larger than L2",
                       "parallelism": f"replicas{world}"},
            "cpu_baseline": {"value": value, "unit": "segments/s", "cores": threads, "kind": "port",
                             "sample": descs[0]},
            "e2e": {"value": value, "unit": "segments/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "note": "reference = the oracle's C++ restatement of the WGSL path on the host cores, on the scene the "
                    "oracle generates and indexes itself (no product library is loaded); the Rust/wgpu reference "
                    "cannot run here (no Rust toolchain, no graphics stack)"}
    print(json.dumps(line), flush=True)
    return 0


# ------------------------------------------------------------------------------------------------
# GPU arm
# ------------------------------------------------------------------------------------------------
# Bytes of per-ray state a traversal launch moves besides the tree: a closest-hit ray reads its
# queue entry (4), origin and direction (32) and the job word of its throughput (16) and writes its
# hit (8); an occlusion ray reads its 48-byte record and, when the light is visible, adds its term to
# the accumulator (16 read + 16 written, counted for every ray: an upper bound).
CLOSEST_RAY_BYTES = 4 + 32 + 16 + 8
OCCLUSION_RAY_BYTES = 48 + 32
TRI_BYTES = 48  # one leaf-ordered triangle record: v0 (+ index), v1 - v0, v2 - v0


def trace_roofline(prof_ev, prof_ct, peak: float, peak_kind: str, gather_ms: float) -> dict:
    """Roofline of wf_trace_kernel, the frame's dominant kernel (closest-hit and occlusion rays in one
    persistent launch per iteration).  Algorithmic bytes per launch = the records its rays visit x
    the record size + the leaf triangles they test x 48 B + the per-ray state bytes above, all
    counted on the device by the counting variant of the kernel over one frame; the launch duration
    is the CUDA-event time of the ordinary kernel's launches over two frames.  The records are mostly
    served by L1 / L2 (DRAM traffic is measured by ncu: profiles/), so this is the rate at which the
    kernel consumes tree bytes, set against the HBM peak."""
    f_ct = max(prof_ct.frames, 1)
    launches = prof_ev.trace_launches / max(prof_ev.frames, 1)
    ms_launch = prof_ev.ms_trace / max(prof_ev.trace_launches, 1)
    rb = prof_ct.record_bytes
    rec = (prof_ct.records_closest + prof_ct.records_occlusion) / f_ct
    tests = (prof_ct.tri_tests_closest + prof_ct.tri_tests_occlusion) / f_ct
    per_frame = (rb * rec + TRI_BYTES * tests + CLOSEST_RAY_BYTES * prof_ct.closest_rays / f_ct
                 + OCCLUSION_RAY_BYTES * prof_ct.occlusion_rays / f_ct)
    per_launch = per_frame / max(launches, 1)
    achieved = per_launch / (ms_launch / 1000.0) / 1e9
    rays_c, rays_o = max(prof_ct.closest_rays, 1), max(prof_ct.occlusion_rays, 1)
    return {"bound": "hbm", "kernel": "wf_trace_kernel", "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": achieved / peak, "traffic": None,
            "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured"
            else "fallback 6.8 TB/s",
            "algorithmic_bytes_per_launch": per_launch, "launch_ms": ms_launch, "launches_per_step": launches,
            "share_of_gather": prof_ev.ms_trace / max(prof_ev.ms_gather, 1e-9),
            "shade_share_of_gather": prof_ev.ms_shade / max(prof_ev.ms_gather, 1e-9),
            "gather_ms": gather_ms,
            "work": {"record_bytes": rb,
                     "records_per_closest_ray": prof_ct.records_closest / rays_c,
                     "records_per_occlusion_ray": prof_ct.records_occlusion / rays_o,
                     "tri_tests_per_closest_ray": prof_ct.tri_tests_closest / rays_c,
                     "tri_tests_per_occlusion_ray": prof_ct.tri_tests_occlusion / rays_o,
                     "closest_rays_per_frame": prof_ct.closest_rays / f_ct,
                     "occlusion_rays_per_frame": prof_ct.occlusion_rays / f_ct},
            "traffic_note": "DRAM bytes per launch come from an ncu capture (profiles/), not from this run"}


def photon_denoise_stages(steps: int, warmup: int, peak: float) -> dict:
    """Config 3's pipeline on the 555-unit Cornell box at 1920x1080: 1,048,576 photons traced from the
    ceiling light (depth 6), binned into the 128^3 grid (cell = extent / 128, radius = cell / 2), then
    progressive frames at 4 spp with the photon lookup and the two a-trous passes.  Device times come
    from the renderer's CUDA events."""
    import rustracer_gb300 as rt

    scene = rt.Scene.cornell555()
    cfg = rt.RenderConfig(width=1920, height=1080, spp=4, accumulate_frames=64, enable_denoise=True,
                          enable_photon_map=True, photon_count=1 << 20, grid_max_dim=130, photon_radius_mode=1,
                          photon_scale=2000.0)
    r = rt.Renderer(scene, cfg)
    r.update_camera(scene.default_camera())
    r.rebuild_photons()  # warm-up
    trace_ms, grid_ms = [], []
    for _ in range(max(steps // 4, 2)):
        r.rebuild_photons()
        st = r.stats()
        trace_ms.append(st.ms_photon_trace)
        grid_ms.append(st.ms_grid_build)
    binned = r.stats().photons_stored
    gp = r.grid_params()
    slots, cells = gp.photon_slots, gp.num_cells
    for _ in range(warmup):
        r.record_frame()
    r.stats()
    for _ in range(steps):
        r.record_frame()
    st = r.stats()
    frames = max(st.timed_frames, 1)
    den_ms = st.ms_denoise_sum / frames
    res_ms = st.ms_resolve_sum / frames
    gat_ms = st.ms_gather_sum / frames
    npix = cfg.width * cfg.height
    t_ms, g_ms = statistics.median(trace_ms), statistics.median(grid_ms)
    # Compulsory bytes of this dataflow (the photon pass emits u32 keys): keys read by the count and
    # the scatter (4 + 4 B/slot); counts read once by the single-pass scan and (start, count) written
    # (12 B/cell); per binned photon the rank written by the count and read by the scatter (4 + 4), the
    # slot order written by the scatter and read by the per-cell sort-and-copy pass (4 + 4), the 64 B
    # photon read + 64 B write of that pass and its 16 B compact position.
    grid_bytes = 8.0 * slots + 12.0 * cells + (8.0 + 8.0 + 128.0 + 16.0) * binned
    den_bytes = 2 * 64.0 * npix
    res_bytes = 52.0 * npix
    r.close()
    return {
        "workload": "cornell555 1920x1080, 2^20 photons, 128^3 grid, spp 4, denoise 2 passes",
        "photons_per_s": (1 << 20) / (t_ms / 1000.0),
        "photon_trace_ms": t_ms,
        "grid_keys_per_s": slots / (g_ms / 1000.0),
        "grid_build_ms": g_ms, "photon_slots": slots, "binned_photons": int(binned), "cells": cells,
        "grid_roofline": {"bound": "hbm", "achieved": grid_bytes / (g_ms / 1000.0) / 1e9, "peak": peak,
                          "unit": "GB/s", "frac": grid_bytes / (g_ms / 1000.0) / 1e9 / peak,
                          "algorithmic_bytes": grid_bytes},
        "denoised_mpix_per_s": npix / (den_ms / 1000.0) / 1e6,
        "denoise_ms_2pass": den_ms,
        "denoise_roofline": {"bound": "hbm", "achieved": den_bytes / (den_ms / 1000.0) / 1e9, "peak": peak,
                             "unit": "GB/s", "frac": den_bytes / (den_ms / 1000.0) / 1e9 / peak,
                             "algorithmic_bytes": den_bytes},
        "resolve_ms": res_ms,
        "resolve_roofline": {"achieved": res_bytes / (res_ms / 1000.0) / 1e9, "frac":
                             res_bytes / (res_ms / 1000.0) / 1e9 / peak},
        "gather_ms_with_photons": gat_ms,
    }


# ------------------------------------------------------------------------------------------------
# Many jobs: the batched form (64 jobs per frame) and the served form (Poisson arrivals)
# ------------------------------------------------------------------------------------------------
RESOLUTIONS = [(256, 256), (512, 512), (640, 480), (1280, 720)]
SPPS = [1, 2, 4, 8, 16]


def ico_level(tris: float) -> int:
    """Subdivision level of the displaced icosphere closest (in log) to `tris` triangles: level L has
    20 * 4^L, so the 10k - 2M range maps to levels 5 - 8 (20k, 82k, 328k, 1.3M)."""
    return int(min(8, max(5, round(math.log(tris / 20.0, 4)))))


def scene_pool(n: int, seed: int) -> list[tuple[int, object]]:
    """n seeded icosphere rooms, triangle counts log-uniform in [10k, 2M], built on all host cores."""
    from concurrent.futures import ThreadPoolExecutor

    import rustracer_gb300 as rt

    rng = np.random.default_rng(seed)
    levels = [ico_level(math.exp(rng.uniform(math.log(1e4), math.log(2e6)))) for _ in range(n)]
    keys = [(lv, 1000 + i) for i, lv in enumerate(levels)]
    with ThreadPoolExecutor(max_workers=min(n, os.cpu_count() or 1)) as ex:
        scenes = list(ex.map(lambda k: rt.Scene.icosphere_room(k[0], k[1], 0.02, 1024), keys))
    return list(zip(levels, scenes))


def job_spec(rng, pool) -> dict:
    """One render job as in the batched workload: scene drawn by triangle count (log-uniform in
    [10k, 2M]) from the pool, resolution from RESOLUTIONS, spp from SPPS, depth 5-8, photon map on
    half the jobs (2^18 - 2^20 photons), denoise on three quarters, a random camera orbit."""
    level = ico_level(math.exp(rng.uniform(math.log(1e4), math.log(2e6))))
    cands = [i for i, (lv, _) in enumerate(pool) if lv == level] or list(range(len(pool)))
    w, h = RESOLUTIONS[int(rng.integers(len(RESOLUTIONS)))]
    photons = int(2.0 ** rng.uniform(18, 20)) if rng.random() < 0.5 else 0
    return dict(scene=int(cands[int(rng.integers(len(cands)))]), width=w, height=h,
                spp=SPPS[int(rng.integers(len(SPPS)))], depth=int(rng.integers(5, 9)), photons=photons,
                denoise=bool(rng.random() < 0.75), yaw=float(rng.uniform(-0.8, 0.8)),
                pitch=float(rng.uniform(-0.3, 0.3)))


def job_objects(spec: dict, pool):
    import rustracer_gb300 as rt

    scene = pool[spec["scene"]][1]
    cfg = rt.RenderConfig(width=spec["width"], height=spec["height"], spp=spec["spp"], max_bounces=spec["depth"],
                          accumulate_frames=0, enable_denoise=spec["denoise"],
                          enable_photon_map=spec["photons"] > 0, photon_count=max(spec["photons"], 1))
    cam = scene.default_camera()
    cam.orbit(spec["yaw"], spec["pitch"])
    return scene, cfg, cam


def frame_launches(cfgs) -> int:
    """Kernel launches of one batch frame over jobs with these configs: one generate and one finalize
    launch over all jobs, per iteration one trace launch (closest-hit rays of the iteration with the
    occlusion rays of the one before), one shade and, when a job has a photon map, one photon-lookup
    launch; the closing trace launch, the counter kernel, then per job the denoise passes and the
    resolve."""
    iters = max(max(c.spp, 1) * (c.max_bounces or 6) for c in cfgs)
    per_iter = 3 if any(c.enable_photon_map for c in cfgs) else 2
    return (2 + per_iter * iters + 2 +
            sum((c.denoise_passes or 2) * int(c.enable_denoise) + 1 for c in cfgs))


def batched_leg(n_jobs: int, steps: int, warmup: int, pool, seed: int = 4) -> dict:
    """64 jobs rendered (a) one job at a time with its own per-frame launches (default launch shape)
    and (b) as one batch per progressive frame captured as a CUDA graph, `steps` frames with the
    default launch shape, then the autotuner, then `steps` frames with the tuned shape.  Both arms
    render warmup + 2 steps frames of every job from a fresh renderer; the final accumulations are
    compared bit for bit (equal per-job RMSE)."""
    import hashlib

    import torch

    import rustracer_gb300 as rt

    rng = np.random.default_rng(seed)
    specs = [job_spec(rng, pool) for _ in range(n_jobs)]
    resident = {i: rt.ResidentScene(pool[i][1]) for i in sorted({s["scene"] for s in specs})}

    def make(spec):
        scene, cfg, cam = job_objects(spec, pool)
        r = rt.Renderer(resident[spec["scene"]], cfg)
        r.update_camera(cam)
        if cfg.enable_photon_map:
            r.rebuild_photons()
        return r

    digest = lambda r: hashlib.blake2b(r.read_accumulation().tobytes(), digest_size=16).hexdigest()  # noqa

    # (a) plain: one job at a time
    plain_s, plain_seg, plain_hash = 0.0, 0, []
    for spec in specs:
        r = make(spec)
        r.render_frames(warmup)
        r.synchronize()
        s0 = r.stats()
        t0 = time.perf_counter()
        r.render_frames(2 * steps)
        r.synchronize()
        plain_s += time.perf_counter() - t0
        plain_seg += r.stats().segments - s0.segments
        plain_hash.append(digest(r))
        r.close()

    # (b) batched: every job in each frame, one CUDA graph per progressive frame
    rs = [make(spec) for spec in specs]
    b = rt.Batch(rs, use_graphs=True)
    b.render_frames(warmup)
    b.synchronize()
    stream = torch.cuda.ExternalStream(b.stream())

    def timed():
        s0 = b.stats()
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        t0 = time.perf_counter()
        ev0.record(stream)
        b.render_frames(steps)
        ev1.record(stream)
        b.synchronize()
        wall = time.perf_counter() - t0
        return b.stats().segments - s0.segments, wall, ev0.elapsed_time(ev1)

    default_shape = b.tuning
    seg_d, wall_d, _ = timed()
    t_tune = time.perf_counter()
    tuned_shape, tuned_ms = b.autotune(trial_frames=1)
    tune_s = time.perf_counter() - t_tune
    batch_seg, batch_s, batch_dev_ms = timed()
    s1 = b.stats()
    same = all(digest(r) == h for r, h in zip(rs, plain_hash))
    b.close()
    for r in rs:
        r.close()
    pixels = sum(s["width"] * s["height"] for s in specs)
    plain_v, batch_v = plain_seg / plain_s, batch_seg / batch_s
    return {
        "workload": f"{n_jobs} jobs: icosphere rooms 10k-2M triangles (levels 5-8), resolutions {RESOLUTIONS}, "
                    f"spp {SPPS}, depth 5-8, photon map on {sum(s['photons'] > 0 for s in specs)}, denoise on "
                    f"{sum(s['denoise'] for s in specs)}; {pixels} pixels per frame",
        "steps": steps, "warmup": warmup,
        "plain_segments_per_s": plain_v,
        "batched_segments_per_s": batch_v,
        "batched_device_segments_per_s": batch_seg / (batch_dev_ms / 1000.0),
        "batched_default_shape_segments_per_s": seg_d / wall_d,
        "speedup": batch_v / plain_v,
        "segments_per_frame": batch_seg / steps,
        "identical_outputs": bool(same and plain_seg == seg_d + batch_seg),
        "autotune": {"default": default_shape, "chosen": tuned_shape, "ms_per_frame": tuned_ms,
                     "seconds": tune_s},
        "graph_captures": int(s1.graph_captures),
        "gpu_launches_per_frame": frame_launches([job_objects(s, pool)[1] for s in specs]),
        "resident_scenes": len(resident),
    }


def served_trace(rate: float, seconds: float, pool, seed: int) -> list[tuple[float, dict, int]]:
    """Poisson arrivals at `rate` jobs/s for `seconds`: (arrival time, job spec, budget frames), the
    budget log-uniform in [8, 256] frames."""
    rng = np.random.default_rng(seed)
    out, t = [], 0.0
    while True:
        t += float(rng.exponential(1.0 / rate))
        if t > seconds:
            return out
        spec = job_spec(rng, pool)
        spec["scene"] = int(rng.integers(len(pool)))  # requests spread over the whole pool
        budget = int(round(math.exp(rng.uniform(math.log(8), math.log(256)))))
        out.append((t, spec, budget))


def served_arm(mode: str, trace, pool, seconds: float, tuning: dict | None) -> dict:
    import rustracer_gb300 as rt

    srv = rt.Server(mode=mode, graphs=True, hbm_cap_bytes=120 << 30, max_jobs=64, max_slots=1 << 25,
                    tuning=tuning)
    for i, (_, sc) in enumerate(pool):
        srv.add_scene(i, sc)
    ids, t_sub = [], []
    s0 = srv.stats()
    start = time.perf_counter()
    for t_arr, spec, budget in trace:
        delay = start + t_arr - time.perf_counter()
        if delay > 0:
            time.sleep(delay)
        _, cfg, cam = job_objects(spec, pool)
        t_sub.append(time.perf_counter() - start)
        ids.append(srv.submit(spec["scene"], cfg, cam, budget))
    rest = start + seconds - time.perf_counter()
    if rest > 0:
        time.sleep(rest)
    wall = time.perf_counter() - start
    st = srv.stats()
    stats = [srv.status(j) for j in ids]
    srv.close()  # finishes the frames in flight, drops the queue
    ttff = [s.t_first_frame_ms - s.t_submit_ms for s in stats if s.t_first_frame_ms >= 0]
    ttb = [s.t_done_ms - s.t_submit_ms for s in stats if s.state == rt._abi.JOB_DONE]
    pct = lambda v, q: float(np.percentile(v, q)) if v else None  # noqa
    # Over every submitted job: a job without a first frame (or not done) when the window closed is
    # censored.  "all_jobs" counts it as +inf (a percentile that lands on one is reported as null);
    # "all_jobs_lower_bound" counts it at its age when the window closed (a lower bound on its time).
    ages = [1000.0 * (wall - t) for t in t_sub]
    ttff_all = [s.t_first_frame_ms - s.t_submit_ms if s.t_first_frame_ms >= 0 else math.inf for s in stats]
    ttb_all = [s.t_done_ms - s.t_submit_ms if s.state == rt._abi.JOB_DONE else math.inf for s in stats]

    def pcts(v):
        if not v:
            return {"p50": None, "p95": None, "p99": None}
        out = {}
        for q in (50, 95, 99):
            x = float(np.percentile(np.asarray(v, np.float64), q, method="inverted_cdf"))
            out[f"p{q}"] = x if math.isfinite(x) else None
        return out

    censored = lambda v: [x if math.isfinite(x) else a for x, a in zip(v, ages)]  # noqa: E731
    return {
        "segments_per_s": (st.segments - s0.segments) / wall,
        "jobs_submitted": len(ids), "jobs_done": len(ttb), "jobs_started": len(ttff),
        "unstarted_at_window_end": len(ids) - len(ttff), "unfinished_at_window_end": len(ids) - len(ttb),
        "ttff_ms": {"p50": pct(ttff, 50), "p95": pct(ttff, 95), "p99": pct(ttff, 99)},
        "time_to_budget_ms": {"p50": pct(ttb, 50), "p95": pct(ttb, 95), "p99": pct(ttb, 99)},
        "ttff_ms_all_jobs": pcts(ttff_all), "ttff_ms_all_jobs_lower_bound": pcts(censored(ttff_all)),
        "time_to_budget_ms_all_jobs": pcts(ttb_all),
        "time_to_budget_ms_all_jobs_lower_bound": pcts(censored(ttb_all)),
        "job_frames": int(st.job_frames), "batch_frames": int(st.batch_frames), "max_active": int(st.max_active),
        "scene_uploads": int(st.scene_uploads), "scene_evictions": int(st.scene_evictions),
        "graph_captures": int(st.graph_captures), "peak_device_bytes": int(st.peak_bytes),
    }


def served_leg(rate: float, seconds: float, pool, tuning: dict | None, seed: int = 5) -> dict:
    """The request loop under Poisson arrivals, continuous batching against the one-job-at-a-time
    loop on the same arrival trace.  "ttff_ms" / "time_to_budget_ms" are over the jobs that reached
    their first frame / their budget inside the window; the "all_jobs" forms cover every submitted job
    with the ones still waiting when the window closed counted as censored (see served_arm)."""
    trace = served_trace(rate, seconds, pool, seed)
    batched = served_arm("batched", trace, pool, seconds, tuning)
    plain = served_arm("plain", trace, pool, seconds, None)
    return {
        "workload": f"Poisson arrivals at {rate} jobs/s for {seconds} s over a pool of {len(pool)} scenes "
                    f"(10k-2M triangles), budgets log-uniform in [8, 256] frames, HBM cap 120 GiB",
        "rate_jobs_per_s": rate, "seconds": seconds,
        "batched": batched, "plain": plain,
        "speedup": batched["segments_per_s"] / max(plain["segments_per_s"], 1e-9),
        "jobs_done_ratio": batched["jobs_done"] / max(plain["jobs_done"], 1),
    }


def run_ours(args, w):
    import torch

    import rustracer_gb300 as rt

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist_mod

        dist_mod.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
        dist = dist_mod

    def barrier():
        if dist is not None:
            dist.barrier()

    scene = make_scene(w)
    cfg = make_config(w)
    cam = scene.default_camera()
    if rank:
        cam.orbit(0.1 * rank, 0.0)  # an independent job per rank
    r = rt.Renderer(scene, cfg)
    r.update_camera(cam)
    stream = torch.cuda.ExternalStream(r.stream())

    for _ in range(args.warmup):
        r.record_frame()
    r.synchronize()
    s0 = r.stats()  # drains the warm-up timings

    # ---- device-timed region ----------------------------------------------------------------
    sampler = ClockSampler(local)
    barrier()
    torch.cuda.synchronize()
    sampler.start()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    for _ in range(args.steps):
        r.record_frame()
    ev1.record(stream)
    ev1.synchronize()
    torch.cuda.synchronize()
    clocks = sampler.stop()
    barrier()
    ms = ev0.elapsed_time(ev1)
    s1 = r.stats()
    segments = s1.segments - s0.segments
    shadow = s1.shadow_rays - s0.shadow_rays

    ms_max, seg_all, shd_all = job_totals(dist, ms, float(segments), float(shadow), device="cuda")
    value = seg_all / (ms_max / 1000.0)

    # ---- end-to-end through the public API with host buffers --------------------------------
    out = torch.empty((cfg.height, cfg.width, 4), dtype=torch.uint8, pin_memory=True)
    out_np = out.numpy()
    s_e0 = r.stats()
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        r.update_camera(cam)
        r.record_frame()
        r.read_tonemapped(out_np)
    t1 = time.perf_counter()
    s_e1 = r.stats()
    e2e_seg = float(s_e1.segments - s_e0.segments)
    e2e_wall, e2e_seg_all = job_totals(dist, t1 - t0, e2e_seg, device="cuda")
    e2e_value = e2e_seg_all / e2e_wall

    # ---- kernel-level profile of the dominant kernel (untimed frames after the timed region) -----
    # Two frames with CUDA events around every traversal / shade launch, then one frame of the
    # counting traversal kernels (records visited and leaf triangle tests per kind of ray).
    r.set_profiling(rt._abi.PROFILE_EVENTS)
    r.render_frames(2)
    prof_ev = r.read_profile()
    r.set_profiling(rt._abi.PROFILE_COUNT)
    r.render_frames(1)
    prof_ct = r.read_profile()
    r.set_profiling(0)

    if rank == 0:
        gather_ms = s1.ms_gather_sum / max(s1.timed_frames, 1)
        resolve_ms = s1.ms_resolve_sum / max(s1.timed_frames, 1)
        # CPU baseline (oracle on this host's cores, bounded sample) and the per-ray work it counts.
        threads = os.cpu_count() or 1
        oscene, ocfg = oracle_workload(w)
        cpu_val, cpu_desc, work = cpu_sample(oscene, ocfg, args.cpu_seconds, threads)
        del oscene
        peak, peak_kind = hbm_peak()
        roofline = trace_roofline(prof_ev, prof_ct, peak, peak_kind, gather_ms)
        stages = photon_denoise_stages(args.steps, args.warmup, peak) if args.stages else None
        pool = scene_pool(32, 7) if (args.batched or args.served) else None
        batched = batched_leg(args.batched_jobs, args.batched_steps, 2, pool) if args.batched else None
        shape = batched["autotune"]["chosen"] if batched else None
        served = None
        if args.served:
            # the main rate first (its figures stay at the top level), then the others: one below the
            # GPU's capacity (service times) and one far above it (queueing)
            rates = [args.served_rate] + [x for x in args.served_other_rates if x != args.served_rate]
            legs = [served_leg(x, args.served_seconds, pool, shape) for x in rates]
            served = dict(legs[0])
            served["by_rate"] = [{k: v for k, v in leg.items() if k != "workload"} for leg in legs]
        line = {
            "metric": "segments/s", "value": value, "unit": "segments/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": args.workload, **{k: v for k, v in w.items()}, "l2": "inputs larger than L2",
                       "parallelism": f"replicas{world}"},
            "shadow_rays_per_s": shd_all / (ms_max / 1000.0),
            "gpu_launches": int(frame_launches([cfg]) * args.steps),
            "kernel_ms": {"gather": gather_ms, "resolve": resolve_ms},
            "roofline": roofline,
            "oracle_work_per_ray": work,
            "cpu_baseline": {"value": cpu_val, "unit": "segments/s", "cores": threads, "kind": "port",
                             "sample": cpu_desc},
            "e2e": {"value": e2e_value, "unit": "segments/s", "h2d_bytes_per_step": 96 + 80,
                    "d2h_bytes_per_step": int(cfg.width * cfg.height * 4)},
            "clocks": clocks,
            "stages": stages,
            "batched": batched,
            "served": served,
        }
        print(json.dumps(line), flush=True)
    r.close()
    if dist is not None:
        dist.destroy_process_group()
    return 0


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=16)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=sorted(WORKLOADS), default="icosphere1080p")
    ap.add_argument("--cpu-seconds", type=float, default=12.0, help="size of the CPU-baseline sample")
    ap.add_argument("--ref-seconds", type=float, default=120.0,
                    help="CPU time of the whole --impl reference run (warm-up and timed samples)")
    ap.add_argument("--no-stages", dest="stages", action="store_false",
                    help="skip the photon-map / denoise stage measurements")
    ap.add_argument("--no-batched", dest="batched", action="store_false", help="skip the 64-job batch leg")
    ap.add_argument("--batched-jobs", type=int, default=64)
    ap.add_argument("--batched-steps", type=int, default=3)
    ap.add_argument("--no-served", dest="served", action="store_false", help="skip the request-loop leg")
    ap.add_argument("--served-rate", type=float, default=10.0, help="Poisson arrival rate, jobs/s")
    ap.add_argument("--served-seconds", type=float, default=20.0, help="arrival window (s) of each rate")
    ap.add_argument("--served-other-rates", type=lambda x: [float(v) for v in x.split(",") if v], default=[1.0, 200.0],
                    help="further arrival rates of the request-loop leg (comma-separated; empty for none)")
    args = ap.parse_args(argv)
    args.warmup = max(args.warmup, 3)
    w = WORKLOADS[args.workload]
    if args.impl == "reference":
        return run_reference(args, w)
    return run_ours(args, w)


if __name__ == "__main__":
    sys.exit(main())
