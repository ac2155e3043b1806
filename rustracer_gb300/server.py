"""The render-request loop (rt_server_*): jobs of registered scenes are submitted as they arrive and
rendered to their accumulation budgets by the server's native worker thread.

    srv = Server(mode="batched", hbm_cap_bytes=120 << 30)
    srv.add_scene(0, scene)                          # the Scene object is kept alive by the server
    jid = srv.submit(0, RenderConfig(width=256, height=256, spp=4), camera, budget_frames=16,
                     keep_result=True)
    srv.wait_idle()
    img = srv.result(jid)                            # (H, W, 4) float32 accumulation
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _abi as A
from .renderer import RenderConfig, tuning_c
from .scene import Camera, Scene


class Server:
    def __init__(self, mode: str = "batched", hbm_cap_bytes: int = 0, max_jobs: int = 0, max_slots: int = 0,
                 graphs: bool = True, frames_in_flight: int = 0, tuning: dict | None = None):
        self._lib = A.load()
        cfg = A.ServerConfig()
        cfg.hbm_cap_bytes = hbm_cap_bytes
        cfg.max_jobs = max_jobs
        cfg.max_slots = max_slots
        cfg.mode = {"batched": A.SERVER_BATCHED, "plain": A.SERVER_PLAIN}[mode]
        cfg.graphs = int(graphs)
        cfg.frames_in_flight = frames_in_flight
        cfg.tuning = tuning_c(tuning)
        h = C.c_void_p()
        A.check("rt_server_create", self._lib.rt_server_create(C.byref(cfg), C.byref(h)))
        self._h = h
        self._scenes: dict[int, tuple[Scene, A.SceneDesc]] = {}
        self._sizes: dict[int, tuple[int, int]] = {}

    def close(self) -> None:
        if getattr(self, "_h", None) is not None and self._h.value:
            self._lib.rt_server_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def add_scene(self, scene_id: int, scene: Scene) -> None:
        desc = scene.describe()
        A.check("rt_server_add_scene", self._lib.rt_server_add_scene(self._h, scene_id, C.byref(desc)))
        self._scenes[scene_id] = (scene, desc)  # the server borrows the scene's arrays

    def submit(self, scene_id: int, config: RenderConfig, camera: Camera, budget_frames: int,
               keep_result: bool = False) -> int:
        req = A.Request()
        req.scene_id = scene_id
        req.budget_frames = budget_frames
        req.keep_result = int(keep_result)
        req.config = config.to_c()
        req.camera = camera.to_c()
        jid = C.c_uint64()
        A.check("rt_server_submit", self._lib.rt_server_submit(self._h, C.byref(req), C.byref(jid)))
        self._sizes[jid.value] = (config.height, config.width)
        return jid.value

    def status(self, job_id: int) -> A.JobStatus:
        s = A.JobStatus()
        A.check("rt_server_job_status", self._lib.rt_server_job_status(self._h, job_id, C.byref(s)))
        return s

    def result(self, job_id: int) -> np.ndarray:
        h, w = self._sizes[job_id]
        out = np.empty((h, w, 4), np.float32)
        A.check("rt_server_read_result", self._lib.rt_server_read_result(
            self._h, job_id, out.ctypes.data_as(C.POINTER(C.c_float)), out.size))
        return out

    def release(self, job_id: int) -> None:
        A.check("rt_server_release_job", self._lib.rt_server_release_job(self._h, job_id))
        self._sizes.pop(job_id, None)

    def wait_idle(self, timeout_s: float = 600.0) -> None:
        A.check("rt_server_wait_idle", self._lib.rt_server_wait_idle(self._h, int(timeout_s * 1000)))

    def stats(self) -> A.ServerStats:
        s = A.ServerStats()
        A.check("rt_server_get_stats", self._lib.rt_server_get_stats(self._h, C.byref(s)))
        return s

    def now_ms(self) -> float:
        return float(self._lib.rt_server_now_ms(self._h))
