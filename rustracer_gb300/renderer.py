"""The frame API of rustracer-renderer (rustracer-renderer/src/lib.rs:21-1042) over the CUDA backend.

    cfg = RenderConfig(width=256, height=256, spp=1, accumulate_frames=16, enable_denoise=False)
    r = Renderer(scene, cfg)          # Renderer::new
    r.update_camera(scene.default_camera())
    for _ in range(16):
        r.record_frame()              # gather -> denoise -> composite -> tonemap
    img = r.read_accumulation()       # (H, W, 4) float32

Every method calls the native library; there is no other implementation behind it.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field, fields

import numpy as np

from . import _abi as A
from .scene import Camera, Scene


@dataclass
class RenderConfig:
    """RenderConfig (lib.rs:21-65) with its Default values, plus backend extensions (0 = reference)."""
    width: int = 800
    height: int = 600
    photon_count: int = 1_000_000
    spp: int = 1
    exposure: float = 1.0
    gamma: float = 2.2
    light_emission: tuple = (1.0, 1.0, 1.0)
    point_light_emission: tuple = (1.0, 1.0, 1.0)
    accumulate_frames: int = 0
    enable_photon_map: bool = False
    enable_denoise: bool = True
    photon_debug: bool = False
    debug_view: int = 0
    photon_scale: float = 0.02
    photon_radius: float = 0.5
    ambient: float = 0.03
    max_bounces: int = 0          # 0 -> 6 (MAX_BOUNCES)
    grid_max_dim: int = 0         # 0 -> 26 (GRID_MAX_DIM)
    photon_radius_mode: int = 0   # 0: clamp(4 cell, .01, 2); 1: cell / 2
    denoise_passes: int = 0       # 0 -> 2

    def to_c(self) -> A.RenderConfigC:
        c = A.RenderConfigC()
        for f in fields(self):
            v = getattr(self, f.name)
            if isinstance(v, tuple):
                getattr(c, f.name)[:] = tuple(float(x) for x in v)
            elif isinstance(v, bool):
                setattr(c, f.name, int(v))
            else:
                setattr(c, f.name, v)
        return c

    @staticmethod
    def from_c(c: A.RenderConfigC) -> "RenderConfig":
        kw = {}
        for f in fields(RenderConfig):
            v = getattr(c, f.name)
            if f.name in ("light_emission", "point_light_emission"):
                v = tuple(v)
            elif f.name in ("enable_photon_map", "enable_denoise", "photon_debug"):
                v = bool(v)
            kw[f.name] = v
        return RenderConfig(**kw)


class ResidentScene:
    """A scene uploaded once and shared by every renderer created on it (rt_resident_scene_*)."""

    def __init__(self, scene: Scene | A.SceneDesc):
        self._lib = A.load()
        desc = scene.describe() if isinstance(scene, Scene) else scene
        h = C.c_void_p()
        A.check("rt_resident_scene_create", self._lib.rt_resident_scene_create(C.byref(desc), C.byref(h)))
        self._h = h

    @property
    def handle(self) -> C.c_void_p:
        return self._h

    def device_bytes(self) -> int:
        return int(self._lib.rt_resident_scene_bytes(self._h))

    def refs(self) -> int:
        return int(self._lib.rt_resident_scene_refs(self._h))

    def footprint(self, config: RenderConfig) -> tuple[int, int]:
        """(bytes a renderer with `config` allocates at create, path bytes its first solo frame adds)."""
        a, b = C.c_uint64(), C.c_uint64()
        A.check("rt_renderer_footprint", self._lib.rt_renderer_footprint(C.byref(config.to_c()), self._h,
                                                                         C.byref(a), C.byref(b)))
        return a.value, b.value

    def close(self) -> None:
        if getattr(self, "_h", None) is not None and self._h.value:
            self._lib.rt_resident_scene_release(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Renderer:
    """Renderer (lib.rs:189-1042): owns every device buffer; not thread-safe.  `scene` is a Scene (or
    its description), uploaded for this renderer, or a ResidentScene shared with other renderers."""

    def __init__(self, scene: Scene | A.SceneDesc | ResidentScene, config: RenderConfig):
        self._lib = A.load()
        h = C.c_void_p()
        if isinstance(scene, ResidentScene):
            A.check("rt_renderer_create_resident",
                    self._lib.rt_renderer_create_resident(scene.handle, C.byref(config.to_c()), C.byref(h)))
        else:
            desc = scene.describe() if isinstance(scene, Scene) else scene
            A.check("rt_renderer_create",
                    self._lib.rt_renderer_create(C.byref(desc), C.byref(config.to_c()), C.byref(h)))
        self._h = h
        self._scene = scene  # keeps the borrowed arrays alive for the renderer's lifetime

    def close(self) -> None:
        if getattr(self, "_h", None) is not None and self._h.value:
            self._lib.rt_renderer_destroy(self._h)
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

    @property
    def handle(self) -> C.c_void_p:
        return self._h

    # ---- configuration ---------------------------------------------------------------------------
    @property
    def config(self) -> RenderConfig:
        c = A.RenderConfigC()
        A.check("rt_get_config", self._lib.rt_get_config(self._h, C.byref(c)))
        return RenderConfig.from_c(c)

    @config.setter
    def config(self, cfg: RenderConfig) -> None:
        A.check("rt_set_config", self._lib.rt_set_config(self._h, C.byref(cfg.to_c())))

    @property
    def width(self) -> int:
        return self.config.width

    @property
    def height(self) -> int:
        return self.config.height

    def grid_params(self) -> A.GridParams:
        gp = A.GridParams()
        A.check("rt_get_grid_params", self._lib.rt_get_grid_params(self._h, C.byref(gp)))
        return gp

    # ---- frame API -------------------------------------------------------------------------------
    def record_frame(self) -> None:
        A.check("rt_render_frame", self._lib.rt_render_frame(self._h))

    render_frame = record_frame

    def render_frames(self, n: int) -> None:
        A.check("rt_render_frames", self._lib.rt_render_frames(self._h, n))

    def update_camera(self, cam: Camera) -> None:
        A.check("rt_update_camera", self._lib.rt_update_camera(self._h, C.byref(cam.to_c())))

    def update_camera_uniform(self, u: A.CameraUniform) -> None:
        A.check("rt_update_camera_uniform", self._lib.rt_update_camera_uniform(self._h, C.byref(u)))

    def update_lights(self, lights: list[A.Light]) -> None:
        arr = (A.Light * len(lights))(*lights)
        A.check("rt_update_lights", self._lib.rt_update_lights(self._h, arr, len(lights)))

    def reset_accumulation(self) -> None:
        A.check("rt_reset_accumulation", self._lib.rt_reset_accumulation(self._h, 1))

    def reset_accumulation_soft(self) -> None:
        A.check("rt_reset_accumulation", self._lib.rt_reset_accumulation(self._h, 0))

    def rebuild_photons(self) -> None:
        A.check("rt_rebuild_photons", self._lib.rt_rebuild_photons(self._h))

    def load_photons(self, photons: np.ndarray) -> None:
        """Replaces the photon slots with `photons` (dtype of Photon) and rebuilds the grid from them."""
        p = np.ascontiguousarray(photons)
        A.check("rt_load_photons_and_build_grid", self._lib.rt_load_photons_and_build_grid(self._h, A.ptr(p), len(p)))

    def set_light_marker(self, marker=None, glow: float = 1.0) -> None:
        m = None if marker is None else (C.c_float * 4)(*map(float, marker))
        A.check("rt_set_light_marker", self._lib.rt_set_light_marker(self._h, m, glow))

    def sample_count(self) -> int:
        return int(self._lib.rt_sample_count(self._h))

    def frame_state(self) -> tuple[int, int]:
        """(sample_counter, frames accumulated since the last reset)."""
        a, b = C.c_uint32(), C.c_uint32()
        A.check("rt_get_frame_state", self._lib.rt_get_frame_state(self._h, C.byref(a), C.byref(b)))
        return a.value, b.value

    def checkpoint(self, path) -> None:
        """Writes the accumulation as raw little-endian f32 RGBA (render_headless.rs's raw dump) to
        `path` and the frame counters to `path` + ".json"."""
        import json
        from pathlib import Path

        acc = self.read_accumulation()
        sc, fr = self.frame_state()
        c = self.config
        Path(path).write_bytes(acc.astype("<f4").tobytes())
        Path(str(path) + ".json").write_text(json.dumps(
            {"width": c.width, "height": c.height, "sample_counter": sc, "frames_since_reset": fr}))

    def resume(self, path) -> None:
        """Restores a checkpoint written by checkpoint() (same configuration, scene and camera)."""
        import json
        from pathlib import Path

        meta = json.loads(Path(str(path) + ".json").read_text())
        c = self.config
        if (meta["width"], meta["height"]) != (c.width, c.height):
            raise ValueError(f"checkpoint is {meta['width']}x{meta['height']}, the renderer {c.width}x{c.height}")
        acc = np.frombuffer(Path(path).read_bytes(), dtype="<f4").astype(np.float32)
        A.check("rt_restore_accumulation", self._lib.rt_restore_accumulation(
            self._h, acc.ctypes.data_as(C.POINTER(C.c_float)), acc.size, meta["sample_counter"],
            meta["frames_since_reset"]))

    def synchronize(self) -> None:
        A.check("rt_synchronize", self._lib.rt_synchronize(self._h))

    def stats(self) -> A.FrameStats:
        s = A.FrameStats()
        A.check("rt_get_stats", self._lib.rt_get_stats(self._h, C.byref(s)))
        return s

    def set_profiling(self, flags: int) -> None:
        """A.PROFILE_EVENTS (events around each traversal / shade / photon-lookup launch) and / or
        A.PROFILE_COUNT (counting traversal kernels) for the following frames; 0 turns it off."""
        A.check("rt_set_profiling", self._lib.rt_set_profiling(self._h, flags))

    def read_profile(self) -> A.TraceProfile:
        p = A.TraceProfile()
        A.check("rt_read_profile", self._lib.rt_read_profile(self._h, C.byref(p)))
        return p

    def stream(self) -> int:
        return int(self._lib.rt_renderer_stream(self._h) or 0)

    def device_bytes(self) -> int:
        return int(self._lib.rt_renderer_device_bytes(self._h))

    @property
    def tuning(self) -> dict:
        t = A.WavefrontTuning()
        A.check("rt_get_tuning", self._lib.rt_get_tuning(self._h, C.byref(t)))
        return t.as_dict()

    @tuning.setter
    def tuning(self, values: dict) -> None:
        A.check("rt_set_tuning", self._lib.rt_set_tuning(self._h, C.byref(tuning_c(values))))

    # ---- read-backs ------------------------------------------------------------------------------
    def _img(self, fn: str) -> np.ndarray:
        c = self.config
        out = np.empty((c.height, c.width, 4), np.float32)
        A.check(fn, getattr(self._lib, fn)(self._h, A.ptr(out), out.size))
        return out

    def read_accumulation(self) -> np.ndarray:
        return self._img("rt_read_accumulation")

    def read_frame(self) -> np.ndarray:
        return self._img("rt_read_frame")

    def read_moments(self) -> np.ndarray:
        return self._img("rt_read_moments")

    def read_gbuffer(self) -> np.ndarray:
        return self._img("rt_read_gbuffer")

    def read_tonemapped(self, out: np.ndarray | None = None) -> np.ndarray:
        c = self.config
        if out is None:
            out = np.empty((c.height, c.width, 4), np.uint8)
        A.check("rt_read_tonemapped", self._lib.rt_read_tonemapped(self._h, A.ptr(out), out.size))
        return out

    def photon_slots(self) -> int:
        return int(self.grid_params().photon_slots)

    def read_photons(self) -> np.ndarray:
        out = np.empty(self.photon_slots(), A.np_dtype(A.Photon))
        A.check("rt_read_photons", self._lib.rt_read_photons(self._h, A.ptr(out), len(out)))
        return out

    def read_sorted_photons(self) -> np.ndarray:
        out = np.empty(self.photon_slots(), A.np_dtype(A.Photon))
        A.check("rt_read_sorted_photons", self._lib.rt_read_sorted_photons(self._h, A.ptr(out), len(out)))
        return out

    def read_photon_grid(self) -> tuple[np.ndarray, np.ndarray]:
        n = self.grid_params().num_cells
        counts = np.empty(n, np.uint32)
        meta = np.empty((n, 2), np.uint32)
        A.check("rt_read_photon_grid", self._lib.rt_read_photon_grid(self._h, A.ptr(counts), A.ptr(meta), n))
        return counts, meta


def tuning_c(values: dict | None) -> A.WavefrontTuning:
    t = A.WavefrontTuning()
    for k, v in (values or {}).items():
        setattr(t, k, int(v))
    return t


class Batch:
    """Renders the next frame of several renderers at once (rt_batch_*); their rays share the same
    wavefront launches.  use_graphs captures each batch frame as a CUDA graph."""

    def __init__(self, renderers: list[Renderer], use_graphs: bool = True):
        self._lib = A.load()
        self.renderers = list(renderers)  # kept alive for the batch's lifetime
        arr = (C.c_void_p * len(renderers))(*[r.handle.value for r in renderers])
        h = C.c_void_p()
        A.check("rt_batch_create", self._lib.rt_batch_create(arr, len(renderers), int(use_graphs), C.byref(h)))
        self._h = h

    def close(self) -> None:
        if getattr(self, "_h", None) is not None and self._h.value:
            self._lib.rt_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def render_frame(self) -> None:
        A.check("rt_batch_render_frame", self._lib.rt_batch_render_frame(self._h))

    def render_frames(self, n: int) -> None:
        A.check("rt_batch_render_frames", self._lib.rt_batch_render_frames(self._h, n))

    def synchronize(self) -> None:
        A.check("rt_batch_synchronize", self._lib.rt_batch_synchronize(self._h))

    def stats(self) -> A.FrameStats:
        s = A.FrameStats()
        A.check("rt_batch_get_stats", self._lib.rt_batch_get_stats(self._h, C.byref(s)))
        return s

    def stream(self) -> int:
        return int(self._lib.rt_batch_stream(self._h) or 0)

    @property
    def tuning(self) -> dict:
        t = A.WavefrontTuning()
        A.check("rt_batch_get_tuning", self._lib.rt_batch_get_tuning(self._h, C.byref(t)))
        return t.as_dict()

    @tuning.setter
    def tuning(self, values: dict) -> None:
        A.check("rt_batch_set_tuning", self._lib.rt_batch_set_tuning(self._h, C.byref(tuning_c(values))))

    def autotune(self, trial_frames: int = 1) -> tuple[dict, float]:
        """Picks the traversal launch shape by timing trial frames (undone afterwards); returns the
        chosen shape and its milliseconds per frame."""
        t, ms = A.WavefrontTuning(), C.c_float()
        A.check("rt_batch_autotune", self._lib.rt_batch_autotune(self._h, trial_frames, C.byref(t), C.byref(ms)))
        return t.as_dict(), float(ms.value)


def set_traversal_width(width: int) -> None:
    """Children per traversal record for scenes uploaded from now on: 4 (default) or 2
    (rt_set_traversal_width)."""
    lib = A.load()
    A.check("rt_set_traversal_width", lib.rt_set_traversal_width(int(width)))


def traversal_width() -> int:
    return int(A.load().rt_get_traversal_width())


def render_config_default() -> RenderConfig:
    """RenderConfig::default() as the native library defines it."""
    c = A.RenderConfigC()
    A.load().rt_render_config_default(C.byref(c))
    return RenderConfig.from_c(c)


# ---- stage entry points (host arrays in and out) ------------------------------------------------
def stage_denoise(frame: np.ndarray, gbuffer: np.ndarray, moments: np.ndarray, alpha: float = 1.0,
                  passes: int = 2) -> np.ndarray:
    h, w, _ = frame.shape
    f, g, m = (np.ascontiguousarray(x, np.float32) for x in (frame, gbuffer, moments))
    out = np.empty_like(f)
    A.check("rt_stage_denoise", A.load().rt_stage_denoise(A.ptr(f), A.ptr(g), A.ptr(m), w, h, alpha, passes, A.ptr(out)))
    return out


def stage_resolve(frame: np.ndarray, accum: np.ndarray, alpha: float, exposure: float = 1.0, gamma: float = 2.2,
                  marker=(0.0, 0.0, 0.0, 0.0), glow: float = 1.0, gbuffer: np.ndarray | None = None):
    h, w, _ = frame.shape
    f = np.ascontiguousarray(frame, np.float32)
    acc = np.array(accum, np.float32, copy=True, order="C")
    g = None if gbuffer is None else np.ascontiguousarray(gbuffer, np.float32)
    tp = A.TonemapParams()
    tp.exposure, tp.gamma, tp.width, tp.glow = exposure, gamma, w, glow
    tp.marker[:] = tuple(float(x) for x in marker)
    out = np.empty((h, w, 4), np.uint8)
    A.check("rt_stage_resolve", A.load().rt_stage_resolve(A.ptr(f), A.ptr(acc), A.ptr(g), w, h, alpha, C.byref(tp),
                                                          A.ptr(out)))
    return acc, out


def stage_photon_grid(photons: np.ndarray, gp: A.GridParams):
    p = np.ascontiguousarray(photons)
    g = A.GridParams.from_buffer_copy(gp)
    g.photon_slots = len(p)
    counts = np.empty(g.num_cells, np.uint32)
    meta = np.empty((g.num_cells, 2), np.uint32)
    srt = np.empty(len(p), A.np_dtype(A.Photon))
    A.check("rt_stage_photon_grid",
            A.load().rt_stage_photon_grid(A.ptr(p), C.byref(g), A.ptr(counts), A.ptr(meta), A.ptr(srt)))
    return counts, meta, srt
