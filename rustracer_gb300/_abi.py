"""ctypes mirror of include/rustracer_cuda.h and the loader of the in-tree librustracer_cuda.so.

The library is loaded from this package directory only; a missing library raises instead of falling
back to any other implementation.
"""
from __future__ import annotations

import ctypes as C
import os
import re
from pathlib import Path

import numpy as np

PKG = Path(__file__).resolve().parent
LIB_PATH = PKG / "librustracer_cuda.so"
HEADER = PKG.parent / "include" / "rustracer_cuda.h"

RT_OK = 0
RT_ERR_INVALID_ARGUMENT = 1
RT_ERR_CUDA = 2
RT_ERR_OUT_OF_MEMORY = 3
RT_ERR_STATE = 4
RT_ERR_DEVICE_CHECK = 5

TEX_NONE = 0xFFFFFFFF
MAT_FLAG_ALPHA_CUTOUT = 1
MAX_BOUNCES = 6
GRID_MAX_DIM = 26
MAT_LAMBERTIAN, MAT_METAL, MAT_DIELECTRIC, MAT_EMISSIVE = 0, 1, 2, 3
LIGHT_POINT, LIGHT_DIRECTIONAL, LIGHT_AREA, LIGHT_ENVIRONMENT = 0, 1, 2, 3
TEX_ALBEDO, TEX_MR, TEX_EMISSIVE, TEX_NORMAL = 0, 1, 2, 3
BVH_HOST_SAH, BVH_GPU_LBVH = 0, 1
NOALLOC_MAX_SLOTS = 1 << 20
NOALLOC_MAX_CELLS = 1 << 18
NOALLOC_SCRATCH_BYTES = 9438208

f3 = C.c_float * 3
f4 = C.c_float * 4
u32 = C.c_uint32
u64 = C.c_uint64


class BVHNode(C.Structure):
    _fields_ = [("bbox_min", f3), ("left_first", u32), ("bbox_max", f3), ("right_child", u32),
                ("prim_count", u32), ("_pad", f3)]


class Triangle(C.Structure):
    _fields_ = [("v0", f3), ("_pad0", C.c_float), ("v1", f3), ("_pad1", C.c_float), ("v2", f3), ("_pad2", C.c_float),
                ("n0", f3), ("_pad3", C.c_float), ("n1", f3), ("_pad4", C.c_float), ("n2", f3), ("_pad5", C.c_float),
                ("uv0", C.c_float * 2), ("uv1", C.c_float * 2), ("uv2", C.c_float * 2), ("material_id", u32),
                ("_pad6", C.c_float)]


class Material(C.Structure):
    _fields_ = [("albedo", f4), ("emissive", f3), ("roughness", C.c_float), ("metallic", C.c_float),
                ("ior", C.c_float), ("kind", u32), ("flags", u32), ("tex_albedo", u32), ("tex_mr", u32),
                ("tex_emissive", u32), ("tex_normal", u32)]


class Light(C.Structure):
    _fields_ = [("data", f4), ("color", f3), ("intensity", C.c_float), ("kind", u32), ("_pad_a", f3),
                ("_pad_b", f4)]


class CameraUniform(C.Structure):
    _fields_ = [("position", f3), ("_pad0", C.c_float), ("forward", f3), ("_pad1", C.c_float), ("right", f3),
                ("_pad2", C.c_float), ("up", f3), ("_pad3", C.c_float), ("inv_half_res", C.c_float * 2),
                ("near_plane", C.c_float), ("fov_scale", C.c_float), ("aperture", C.c_float),
                ("focus_dist", C.c_float), ("_pad_end", C.c_float * 2)]


class Photon(C.Structure):
    _fields_ = [("position", f3), ("_pad0", C.c_float), ("power", f3), ("_pad1", C.c_float), ("incident", f3),
                ("_pad2", C.c_float), ("normal", f3), ("_pad3", C.c_float)]


class ImageParams(C.Structure):
    _fields_ = [("width", u32), ("height", u32), ("spp", u32), ("frame", u32), ("light_emission", f3),
                ("ambient", C.c_float), ("accumulate_alpha", C.c_float), ("use_photons", u32),
                ("photon_count", u32), ("photon_radius", C.c_float), ("photon_scale", C.c_float),
                ("photon_debug", u32), ("point_light_emission", f3), ("_pad", u32 * 3)]


class GridParams(C.Structure):
    _fields_ = [("room_min_x", C.c_float), ("room_min_y", C.c_float), ("room_min_z", C.c_float),
                ("cell_size", C.c_float), ("grid_x", u32), ("grid_y", u32), ("grid_z", u32), ("num_cells", u32),
                ("photon_slots", u32), ("_pad", u32 * 3)]


class DenoiseParams(C.Structure):
    _fields_ = [("width", u32), ("height", u32), ("step_size", u32), ("lambda_", C.c_float),
                ("phi_normal", C.c_float), ("phi_depth", C.c_float), ("alpha", C.c_float), ("_pad", u32)]


class CompositeParams(C.Structure):
    _fields_ = [("width", u32), ("height", u32), ("alpha", C.c_float), ("_pad", u32)]


class TonemapParams(C.Structure):
    _fields_ = [("exposure", C.c_float), ("gamma", C.c_float), ("width", u32), ("glow", C.c_float),
                ("marker", f4)]


class Camera(C.Structure):
    _fields_ = [("position", f3), ("look_at", f3), ("up", f3), ("fov_degrees", C.c_float),
                ("near_plane", C.c_float), ("aperture", C.c_float), ("focus_dist", C.c_float)]


class RenderConfigC(C.Structure):
    _fields_ = [("width", u32), ("height", u32), ("photon_count", u32), ("spp", u32), ("exposure", C.c_float),
                ("gamma", C.c_float), ("light_emission", f3), ("point_light_emission", f3),
                ("accumulate_frames", u32), ("enable_photon_map", u32), ("enable_denoise", u32),
                ("photon_debug", u32), ("debug_view", u32), ("photon_scale", C.c_float),
                ("photon_radius", C.c_float), ("ambient", C.c_float), ("max_bounces", u32), ("grid_max_dim", u32),
                ("photon_radius_mode", u32), ("denoise_passes", u32)]


class TextureArray(C.Structure):
    _fields_ = [("rgba8", C.POINTER(C.c_uint8)), ("width", u32), ("height", u32), ("layers", u32), ("_pad", u32)]


class SceneDesc(C.Structure):
    _fields_ = [("triangles", C.POINTER(Triangle)), ("triangle_count", C.c_uint64),
                ("bvh_nodes", C.POINTER(BVHNode)), ("bvh_node_count", C.c_uint64),
                ("bvh_prims", C.POINTER(C.c_uint32)), ("bvh_prim_count", C.c_uint64),
                ("materials", C.POINTER(Material)), ("material_count", C.c_uint64),
                ("lights", C.POINTER(Light)), ("light_count", C.c_uint64),
                ("tex_albedo", TextureArray), ("tex_mr", TextureArray), ("tex_emissive", TextureArray),
                ("tex_normal", TextureArray), ("bounds_min", f3), ("bounds_max", f3), ("has_bounds", u32),
                ("_pad", u32)]


class FrameStats(C.Structure):
    _fields_ = [("frames", C.c_uint64), ("segments", C.c_uint64), ("shadow_rays", C.c_uint64),
                ("photons_stored", C.c_uint64), ("ms_gather", C.c_float), ("ms_denoise", C.c_float),
                ("ms_resolve", C.c_float), ("ms_frame", C.c_float), ("ms_photon_trace", C.c_float),
                ("ms_grid_build", C.c_float), ("timed_frames", C.c_uint64), ("ms_gather_sum", C.c_double),
                ("ms_denoise_sum", C.c_double), ("ms_resolve_sum", C.c_double), ("ms_frame_sum", C.c_double),
                ("graph_captures", C.c_uint64)]


class TraceProfile(C.Structure):
    _fields_ = [("frames", C.c_uint64), ("trace_launches", C.c_uint64), ("shade_launches", C.c_uint64),
                ("photon_launches", C.c_uint64), ("ms_trace", C.c_double), ("ms_shade", C.c_double),
                ("ms_photon", C.c_double), ("ms_gather", C.c_double), ("closest_rays", C.c_uint64),
                ("occlusion_rays", C.c_uint64), ("records_closest", C.c_uint64), ("records_occlusion", C.c_uint64),
                ("tri_tests_closest", C.c_uint64), ("tri_tests_occlusion", C.c_uint64), ("record_bytes", u32),
                ("pixels", u32)]

    def as_dict(self) -> dict:
        return {name: getattr(self, name) for name, _ in self._fields_}


PROFILE_EVENTS, PROFILE_COUNT = 1, 2

SERVER_BATCHED, SERVER_PLAIN = 0, 1
JOB_QUEUED, JOB_RUNNING, JOB_DONE, JOB_FAILED = 0, 1, 2, 3


class WavefrontTuning(C.Structure):
    _fields_ = [("block_threads", u32), ("blocks_per_sm", u32), ("chunk", u32), ("steps", u32),
                ("stack_entries", u32), ("treelet", u32), ("shade_blocks", u32), ("refill_idle", u32)]

    def as_dict(self) -> dict:
        return {f: int(getattr(self, f)) for f, _ in self._fields_ if f != "_pad"}


class ServerConfig(C.Structure):
    _fields_ = [("hbm_cap_bytes", C.c_uint64), ("max_jobs", u32), ("max_slots", u32), ("mode", u32),
                ("graphs", u32), ("frames_in_flight", u32), ("_pad", u32), ("tuning", WavefrontTuning)]


class Request(C.Structure):
    _fields_ = [("scene_id", u32), ("budget_frames", u32), ("keep_result", u32), ("_pad", u32),
                ("config", RenderConfigC), ("camera", Camera)]


class JobStatus(C.Structure):
    _fields_ = [("job_id", C.c_uint64), ("state", u32), ("frames_done", u32), ("t_submit_ms", C.c_double),
                ("t_admit_ms", C.c_double), ("t_first_frame_ms", C.c_double), ("t_done_ms", C.c_double)]


class ServerStats(C.Structure):
    _fields_ = [(n, C.c_uint64) for n in ("submitted", "admitted", "completed", "failed", "batch_frames",
                                          "job_frames", "segments", "shadow_rays", "scene_uploads",
                                          "scene_evictions", "graph_captures", "used_bytes", "peak_bytes",
                                          "resident_scene_bytes")] + \
                [(n, u32) for n in ("active", "pending", "resident_scenes", "max_active")]


def np_dtype(struct: type[C.Structure]) -> np.dtype:
    """A numpy dtype with the struct's byte layout (for bulk arrays of it)."""
    return np.dtype(struct)


vp = C.c_void_p
P = C.POINTER
_PROTOS: dict[str, tuple] = {
    "rt_last_error": (C.c_char_p, []),
    "rt_version": (C.c_char_p, []),
    "rt_device_count": (C.c_int, []),
    "rt_render_config_default": (None, [P(RenderConfigC)]),
    "rt_renderer_create": (C.c_int, [P(SceneDesc), P(RenderConfigC), P(vp)]),
    "rt_renderer_destroy": (None, [vp]),
    "rt_render_frame": (C.c_int, [vp]),
    "rt_render_frames": (C.c_int, [vp, u32]),
    "rt_update_camera": (C.c_int, [vp, P(Camera)]),
    "rt_update_camera_uniform": (C.c_int, [vp, P(CameraUniform)]),
    "rt_update_lights": (C.c_int, [vp, P(Light), C.c_uint64]),
    "rt_reset_accumulation": (C.c_int, [vp, C.c_int]),
    "rt_rebuild_photons": (C.c_int, [vp]),
    "rt_set_config": (C.c_int, [vp, P(RenderConfigC)]),
    "rt_get_config": (C.c_int, [vp, P(RenderConfigC)]),
    "rt_set_light_marker": (C.c_int, [vp, P(C.c_float), C.c_float]),
    "rt_sample_count": (u32, [vp]),
    "rt_synchronize": (C.c_int, [vp]),
    "rt_get_stats": (C.c_int, [vp, P(FrameStats)]),
    "rt_set_profiling": (C.c_int, [vp, u32]),
    "rt_read_profile": (C.c_int, [vp, P(TraceProfile)]),
    "rt_get_grid_params": (C.c_int, [vp, P(GridParams)]),
    "rt_renderer_stream": (vp, [vp]),
    "rt_read_accumulation": (C.c_int, [vp, vp, C.c_uint64]),
    "rt_read_frame": (C.c_int, [vp, vp, C.c_uint64]),
    "rt_read_moments": (C.c_int, [vp, vp, C.c_uint64]),
    "rt_read_gbuffer": (C.c_int, [vp, vp, C.c_uint64]),
    "rt_read_tonemapped": (C.c_int, [vp, vp, C.c_uint64]),
    "rt_read_photons": (C.c_int, [vp, vp, C.c_uint64]),
    "rt_read_sorted_photons": (C.c_int, [vp, vp, C.c_uint64]),
    "rt_read_photon_grid": (C.c_int, [vp, vp, vp, C.c_uint64]),
    "rt_load_photons_and_build_grid": (C.c_int, [vp, vp, C.c_uint64]),
    "rt_resident_scene_create": (C.c_int, [P(SceneDesc), P(vp)]),
    "rt_resident_scene_release": (None, [vp]),
    "rt_resident_scene_bytes": (u64, [vp]),
    "rt_resident_scene_refs": (u32, [vp]),
    "rt_renderer_create_resident": (C.c_int, [vp, P(RenderConfigC), P(vp)]),
    "rt_renderer_device_bytes": (u64, [vp]),
    "rt_renderer_footprint": (C.c_int, [P(RenderConfigC), vp, P(u64), P(u64)]),
    "rt_get_frame_state": (C.c_int, [vp, P(u32), P(u32)]),
    "rt_restore_accumulation": (C.c_int, [vp, P(C.c_float), u64, u32, u32]),
    "rt_set_host_threads": (None, [u32]),
    "rt_set_traversal_width": (C.c_int, [u32]),
    "rt_get_traversal_width": (u32, []),
    "rt_tma_timeouts": (u32, []),
    "rt_scan_timeouts": (u32, []),
    "rt_scene_set_bvh_builder": (C.c_int, [vp, u32]),
    "rt_scene_bvh_builder_used": (u32, [vp]),
    "rt_bvh_build_gpu": (C.c_int, [P(C.c_float), P(C.c_float), P(C.c_float), u64, P(vp), P(u32)]),
    "rt_png_unfilter": (C.c_int, [P(C.c_uint8), u32, u32, u32, P(C.c_uint8)]),
    "rt_jpeg_decode": (C.c_int, [vp, C.c_uint64, vp, C.c_uint64, P(u32), P(u32)]),
    "rt_batch_create": (C.c_int, [P(vp), u32, u32, P(vp)]),
    "rt_batch_destroy": (None, [vp]),
    "rt_batch_render_frame": (C.c_int, [vp]),
    "rt_batch_render_frames": (C.c_int, [vp, u32]),
    "rt_batch_synchronize": (C.c_int, [vp]),
    "rt_batch_get_stats": (C.c_int, [vp, P(FrameStats)]),
    "rt_batch_stream": (vp, [vp]),
    "rt_batch_set_tuning": (C.c_int, [vp, P(WavefrontTuning)]),
    "rt_batch_get_tuning": (C.c_int, [vp, P(WavefrontTuning)]),
    "rt_batch_autotune": (C.c_int, [vp, u32, P(WavefrontTuning), P(C.c_float)]),
    "rt_set_tuning": (C.c_int, [vp, P(WavefrontTuning)]),
    "rt_get_tuning": (C.c_int, [vp, P(WavefrontTuning)]),
    "rt_server_create": (C.c_int, [P(ServerConfig), P(vp)]),
    "rt_server_destroy": (None, [vp]),
    "rt_server_add_scene": (C.c_int, [vp, u32, P(SceneDesc)]),
    "rt_server_submit": (C.c_int, [vp, P(Request), P(u64)]),
    "rt_server_job_status": (C.c_int, [vp, u64, P(JobStatus)]),
    "rt_server_read_result": (C.c_int, [vp, u64, P(C.c_float), u64]),
    "rt_server_release_job": (C.c_int, [vp, u64]),
    "rt_server_wait_idle": (C.c_int, [vp, u32]),
    "rt_server_get_stats": (C.c_int, [vp, P(ServerStats)]),
    "rt_server_now_ms": (C.c_double, [vp]),
    "rt_stage_denoise": (C.c_int, [vp, vp, vp, u32, u32, C.c_float, u32, vp]),
    "rt_stage_resolve": (C.c_int, [vp, vp, vp, u32, u32, C.c_float, P(TonemapParams), vp]),
    "rt_stage_photon_grid": (C.c_int, [vp, P(GridParams), vp, vp, vp]),
    "rt_stage_photon_grid_noalloc": (C.c_int, [vp, P(GridParams), vp, vp, vp, vp]),
    "rt_scene_create": (C.c_int, [P(vp)]),
    "rt_scene_destroy": (None, [vp]),
    "rt_scene_add_mesh": (C.c_int, [vp, vp, vp, vp, C.c_uint64, vp, C.c_uint64, u32]),
    "rt_scene_add_material": (C.c_int, [vp, P(Material)]),
    "rt_scene_add_light": (C.c_int, [vp, P(Light)]),
    "rt_scene_set_textures": (C.c_int, [vp, C.c_int, vp, u32, u32, u32]),
    "rt_scene_finalize": (C.c_int, [vp]),
    "rt_scene_describe": (C.c_int, [vp, P(SceneDesc)]),
    "rt_scene_triangle_count": (C.c_uint64, [vp]),
    "rt_scene_create_cornell555": (C.c_int, [P(vp)]),
    "rt_scene_create_icosphere_room": (C.c_int, [u32, C.c_uint64, C.c_float, u32, P(vp)]),
    "rt_camera_default": (None, [P(Camera)]),
    "rt_camera_to_uniform": (None, [P(Camera), u32, u32, P(CameraUniform)]),
    "rt_camera_frame_scene": (C.c_int, [vp, P(Camera)]),
    "rt_scene_default_camera": (C.c_int, [vp, P(Camera)]),
    "rt_camera_orbit": (None, [P(Camera), C.c_float, C.c_float]),
    "rt_camera_zoom": (None, [P(Camera), C.c_float]),
    "rt_derive_grid": (None, [P(C.c_float), P(C.c_float), C.c_int, u32, u32, u32, P(GridParams), P(C.c_float)]),
    "rt_bvh_build": (C.c_int, [vp, vp, vp, C.c_uint64, P(vp)]),
    "rt_bvh_wide_layout": (C.c_int, [vp, C.c_uint64, vp, C.c_uint64, P(C.c_uint64), P(u32)]),
    "rt_bvh_nodes": (P(BVHNode), [vp, P(C.c_uint64)]),
    "rt_bvh_prims": (P(C.c_uint32), [vp, P(C.c_uint64)]),
    "rt_bvh_destroy": (None, [vp]),
}

_lib: C.CDLL | None = None


class RtError(RuntimeError):
    def __init__(self, fn: str, status: int, msg: str):
        super().__init__(f"{fn} failed with status {status}: {msg}")
        self.status = status


def header_functions() -> list[str]:
    """Names of every function declared in include/rustracer_cuda.h."""
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"\b(rt_[a-z0-9_]+)\s*\(", text)
    seen: list[str] = []
    for n in names:
        if n not in seen:
            seen.append(n)
    return seen


def load(path: os.PathLike | str | None = None) -> C.CDLL:
    """Loads librustracer_cuda.so from the package directory (build it with rustracer_gb300.build)."""
    global _lib
    if _lib is not None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise ImportError(f"{p} is missing: run `python -m rustracer_gb300.build` (the CUDA backend has no fallback)")
    lib = C.CDLL(str(p))
    for name, (res, args) in _PROTOS.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(fn: str, status: int) -> None:
    if status != RT_OK:
        msg = load().rt_last_error()
        raise RtError(fn, status, msg.decode() if msg else "")


def ptr(a: np.ndarray | None) -> C.c_void_p | None:
    if a is None:
        return None
    if not a.flags["C_CONTIGUOUS"]:
        raise ValueError("array must be C-contiguous")
    return C.c_void_p(a.ctypes.data)
