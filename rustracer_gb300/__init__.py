"""rustracer_gb300: the per-frame hot path of the rustracer path tracer on GB300 (sm_103a).

BVH traversal with Moller-Trumbore intersection, Lambertian / GGX-metal / dielectric sampling with
next-event estimation, the photon trace with its exact u32 counting-sort grid and radius gather, the
two-pass edge-aware a-trous denoise and the accumulate / tonemap resolve, behind the C ABI of
include/rustracer_cuda.h (librustracer_cuda.so, built in-tree by rustracer_gb300.build).
"""
from . import _abi
from .renderer import (Batch, RenderConfig, Renderer, ResidentScene, render_config_default, set_traversal_width,
                       stage_denoise, stage_photon_grid, stage_resolve, traversal_width)
from .server import Server
from .scene import (Camera, Scene, area_light, derive_grid, dielectric, directional_light, emissive,
                    environment_light, lambertian, material, metal, point_light)

__all__ = ["_abi", "Batch", "RenderConfig", "Renderer", "ResidentScene", "Server", "render_config_default",
           "set_traversal_width", "stage_denoise", "stage_photon_grid", "stage_resolve", "traversal_width", "Camera", "Scene", "area_light", "derive_grid", "dielectric", "directional_light",
           "emissive", "environment_light", "lambertian", "material", "metal", "point_light"]
