"""Host-side scene model: the part of rustracer-core the frame path consumes.

Scene mirrors rustracer_core::scene::Scene (rustracer-core/src/scene.rs:156-291): meshes, materials,
lights and role textures, flattened into the GPU layouts with the binned-SAH BVH on finalize.  The
work happens in the native library (rt_scene_* in include/rustracer_cuda.h).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import _abi as A


def material(kind: int = A.MAT_LAMBERTIAN, albedo=(0.8, 0.8, 0.8), roughness: float = 0.5, metallic: float = 0.0,
             ior: float = 1.5, emissive=(0.0, 0.0, 0.0), alpha_cutout: bool = False, tex_albedo: int = A.TEX_NONE,
             tex_mr: int = A.TEX_NONE, tex_emissive: int = A.TEX_NONE, tex_normal: int = A.TEX_NONE) -> A.Material:
    """Material::to_gpu (rustracer-core/src/material.rs:143-161); defaults of Material::default."""
    m = A.Material()
    m.albedo[:] = (float(albedo[0]), float(albedo[1]), float(albedo[2]), 1.0)
    m.emissive[:] = tuple(float(x) for x in emissive)
    m.roughness, m.metallic, m.ior = roughness, metallic, ior
    m.kind = kind
    m.flags = A.MAT_FLAG_ALPHA_CUTOUT if alpha_cutout else 0
    m.tex_albedo, m.tex_mr, m.tex_emissive, m.tex_normal = tex_albedo, tex_mr, tex_emissive, tex_normal
    return m


def lambertian(albedo) -> A.Material:  # material.rs:101-108
    return material(A.MAT_LAMBERTIAN, albedo, roughness=1.0)


def metal(albedo, roughness: float) -> A.Material:  # material.rs:111-119
    return material(A.MAT_METAL, albedo, roughness=float(np.float32(min(max(roughness, 0.001), 1.0))), metallic=1.0)


def dielectric(ior: float, albedo=(1.0, 1.0, 1.0)) -> A.Material:  # material.rs:122-130
    return material(A.MAT_DIELECTRIC, albedo, roughness=0.0, ior=ior)


def emissive(color, intensity: float) -> A.Material:  # material.rs:133-140 (albedo = colour)
    c = np.asarray(color, np.float32)
    return material(A.MAT_EMISSIVE, tuple(c), emissive=tuple(c * np.float32(intensity)))


def light(kind: int, data=(0.0, 0.0, 0.0, 0.0), color=(1.0, 1.0, 1.0), intensity: float = 1.0) -> A.Light:
    """light_to_gpu (rustracer-renderer/src/lib.rs:1231-1282)."""
    l = A.Light()
    d = list(data) + [0.0] * (4 - len(data))
    l.data[:] = tuple(float(x) for x in d[:4])
    l.color[:] = tuple(float(x) for x in color)
    l.intensity = intensity
    l.kind = kind
    return l


def point_light(position, color=(1.0, 1.0, 1.0), intensity: float = 1.0) -> A.Light:
    return light(A.LIGHT_POINT, tuple(position), color, intensity)


def directional_light(direction, color=(1.0, 1.0, 1.0), intensity: float = 1.0) -> A.Light:
    return light(A.LIGHT_DIRECTIONAL, tuple(direction), color, intensity)


def area_light(triangle_index: int, color=(1.0, 1.0, 1.0), intensity: float = 1.0) -> A.Light:
    return light(A.LIGHT_AREA, (float(triangle_index), 0.0, 0.0, 0.0), color, intensity)


def environment_light(zenith=(0.55, 0.6, 0.75), horizon=(0.95, 0.93, 0.9), intensity: float = 1.0) -> A.Light:
    return light(A.LIGHT_ENVIRONMENT, tuple(horizon), zenith, intensity)


@dataclass
class Camera:
    """rustracer_core::camera::Camera (rustracer-core/src/camera.rs:7-40)."""
    position: tuple = (0.0, 0.0, 5.0)
    look_at: tuple = (0.0, 0.0, 0.0)
    up: tuple = (0.0, 1.0, 0.0)
    fov_degrees: float = 60.0
    near: float = 0.1
    aperture: float = 0.0
    focus_dist: float = 5.0

    def to_c(self) -> A.Camera:
        c = A.Camera()
        c.position[:] = self.position
        c.look_at[:] = self.look_at
        c.up[:] = self.up
        c.fov_degrees, c.near_plane, c.aperture, c.focus_dist = self.fov_degrees, self.near, self.aperture, self.focus_dist
        return c

    @staticmethod
    def from_c(c: A.Camera) -> "Camera":
        return Camera(tuple(c.position), tuple(c.look_at), tuple(c.up), c.fov_degrees, c.near_plane, c.aperture,
                      c.focus_dist)

    def to_uniform(self, width: int, height: int) -> A.CameraUniform:
        u = A.CameraUniform()
        A.load().rt_camera_to_uniform(C.byref(self.to_c()), width, height, C.byref(u))
        return u

    def orbit(self, delta_yaw: float, delta_pitch: float) -> None:
        c = self.to_c()
        A.load().rt_camera_orbit(C.byref(c), delta_yaw, delta_pitch)
        self.position = tuple(c.position)

    def zoom(self, delta: float) -> None:
        c = self.to_c()
        A.load().rt_camera_zoom(C.byref(c), delta)
        self.position = tuple(c.position)


class Scene:
    """Owning handle of a native rt_scene."""

    def __init__(self, handle: int | None = None):
        lib = A.load()
        if handle is None:
            h = C.c_void_p()
            A.check("rt_scene_create", lib.rt_scene_create(C.byref(h)))
            handle = h.value
        self._h = C.c_void_p(handle)
        self._desc: A.SceneDesc | None = None
        self._n_materials = None

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            A.load().rt_scene_destroy(h)
            self._h = None

    @property
    def handle(self) -> C.c_void_p:
        return self._h

    # ---- procedural scenes -----------------------------------------------------------------------
    @staticmethod
    def cornell555() -> "Scene":
        h = C.c_void_p()
        A.check("rt_scene_create_cornell555", A.load().rt_scene_create_cornell555(C.byref(h)))
        return Scene(h.value)

    @staticmethod
    def icosphere_room(level: int = 8, seed: int = 0, sigma: float = 0.02, tex_size: int = 1024) -> "Scene":
        h = C.c_void_p()
        A.check("rt_scene_create_icosphere_room",
                A.load().rt_scene_create_icosphere_room(level, seed, sigma, tex_size, C.byref(h)))
        return Scene(h.value)

    # ---- building --------------------------------------------------------------------------------
    def add_mesh(self, positions, indices, material_id: int, normals=None, uvs=None) -> None:
        pos = np.ascontiguousarray(positions, np.float32).reshape(-1, 3)
        idx = np.ascontiguousarray(indices, np.uint32).reshape(-1)
        nrm = None if normals is None else np.ascontiguousarray(normals, np.float32).reshape(-1, 3)
        uv = None if uvs is None else np.ascontiguousarray(uvs, np.float32).reshape(-1, 2)
        A.check("rt_scene_add_mesh", A.load().rt_scene_add_mesh(self._h, A.ptr(pos), A.ptr(nrm), A.ptr(uv), len(pos),
                                                                 A.ptr(idx), len(idx), material_id))
        self._desc = None

    def add_material(self, m: A.Material) -> int:
        """Appends a material; returns its index."""
        if self._n_materials is None:
            self._n_materials = self.describe().material_count
        A.check("rt_scene_add_material", A.load().rt_scene_add_material(self._h, C.byref(m)))
        self._desc = None
        self._n_materials += 1
        return self._n_materials - 1

    def add_light(self, l: A.Light) -> None:
        A.check("rt_scene_add_light", A.load().rt_scene_add_light(self._h, C.byref(l)))
        self._desc = None

    def set_textures(self, role: int, rgba8: np.ndarray) -> None:
        """rgba8: uint8 array (layers, height, width, 4)."""
        t = np.ascontiguousarray(rgba8, np.uint8)
        if t.ndim == 3:
            t = t[None]
        layers, h, w, _ = t.shape
        A.check("rt_scene_set_textures", A.load().rt_scene_set_textures(self._h, role, A.ptr(t), w, h, layers))
        self._desc = None

    def describe(self) -> A.SceneDesc:
        """Flattened arrays (triangles, BVH, materials, lights, textures); valid while the scene lives."""
        if self._desc is None:
            d = A.SceneDesc()
            A.check("rt_scene_describe", A.load().rt_scene_describe(self._h, C.byref(d)))
            self._desc = d
        return self._desc

    def triangle_count(self) -> int:
        return int(A.load().rt_scene_triangle_count(self._h))

    def set_bvh_builder(self, builder: int) -> None:
        """A.BVH_HOST_SAH (the reference's builder, default) or A.BVH_GPU_LBVH; before finalizing."""
        A.check("rt_scene_set_bvh_builder", A.load().rt_scene_set_bvh_builder(self._h, builder))
        self._desc = None  # flattened again with the new tree at the next describe

    def bvh_builder_used(self) -> int:
        return int(A.load().rt_scene_bvh_builder_used(self._h))

    def default_camera(self) -> Camera:
        c = A.Camera()
        A.check("rt_scene_default_camera", A.load().rt_scene_default_camera(self._h, C.byref(c)))
        return Camera.from_c(c)

    def frame_camera(self) -> Camera:
        c = A.Camera()
        A.check("rt_camera_frame_scene", A.load().rt_camera_frame_scene(self._h, C.byref(c)))
        return Camera.from_c(c)

    # ---- numpy views of the flattened arrays -----------------------------------------------------
    def arrays(self) -> dict[str, np.ndarray]:
        """Copies of the flattened arrays (safe to keep after the scene is gone)."""
        d = self.describe()

        def view(p, n, struct):
            if n == 0:
                return np.zeros(0, dtype=A.np_dtype(struct))
            return np.ctypeslib.as_array(C.cast(p, C.POINTER(C.c_uint8)), shape=(n * C.sizeof(struct),)).view(
                A.np_dtype(struct)).copy()

        out = {
            "triangles": view(d.triangles, d.triangle_count, A.Triangle),
            "bvh_nodes": view(d.bvh_nodes, d.bvh_node_count, A.BVHNode),
            "materials": view(d.materials, d.material_count, A.Material),
            "lights": view(d.lights, d.light_count, A.Light),
        }
        out["bvh_prims"] = (np.ctypeslib.as_array(d.bvh_prims, shape=(d.bvh_prim_count,)).copy()
                            if d.bvh_prim_count else np.zeros(0, np.uint32))
        return out

    def bounds(self) -> tuple[np.ndarray, np.ndarray] | None:
        d = self.describe()
        if not d.has_bounds:
            return None
        return np.array(d.bounds_min, np.float32), np.array(d.bounds_max, np.float32)


def derive_grid(bounds, grid_max_dim: int = 0, radius_mode: int = 0, photon_slots: int = 1):
    """Renderer::new's photon-grid derivation (rustracer-renderer/src/lib.rs:416-457)."""
    gp = A.GridParams()
    r = C.c_float(0.5)
    if bounds is None:
        A.load().rt_derive_grid(None, None, 0, grid_max_dim, radius_mode, photon_slots, C.byref(gp), C.byref(r))
    else:
        bmin = (C.c_float * 3)(*map(float, bounds[0]))
        bmax = (C.c_float * 3)(*map(float, bounds[1]))
        A.load().rt_derive_grid(bmin, bmax, 1, grid_max_dim, radius_mode, photon_slots, C.byref(gp), C.byref(r))
    return gp, r.value
