"""ORACLE — test infrastructure only (parity checker and timed CPU baseline).

ctypes wrapper of oracle/oracle.cpp (a scalar, multithreaded C++ restatement of rustracer's WGSL hot
path) and a CPU driver of the reference's frame schedule (rustracer-renderer/src/lib.rs:666-851,
913-1037).  Only the tests, the smoke check and bench.py's CPU-baseline leg use it; the product never
imports, links or runs anything here.

Parity pinning: the reference's own tests pin only struct layouts and BVH invariants; radiance, RNG,
BSDF, photon grid and denoise are unpinned by the reference (it cannot run here).  The golden
vectors under tests/golden/ were generated from this restatement.
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "build" / "liboracle.so"

f3 = C.c_float * 3
u32 = C.c_uint32


# Own copies of the layouts the oracle exchanges (sizes are checked against the public header by the
# CPU tests).
class CameraUniform(C.Structure):
    _fields_ = [("position", f3), ("_pad0", C.c_float), ("forward", f3), ("_pad1", C.c_float), ("right", f3),
                ("_pad2", C.c_float), ("up", f3), ("_pad3", C.c_float), ("inv_half_res", C.c_float * 2),
                ("near_plane", C.c_float), ("fov_scale", C.c_float), ("aperture", C.c_float),
                ("focus_dist", C.c_float), ("_pad_end", C.c_float * 2)]


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
                ("marker", C.c_float * 4)]


class TextureArray(C.Structure):
    _fields_ = [("rgba8", C.c_void_p), ("width", u32), ("height", u32), ("layers", u32), ("_pad", u32)]


class SceneDesc(C.Structure):
    _fields_ = [("triangles", C.c_void_p), ("triangle_count", C.c_uint64), ("bvh_nodes", C.c_void_p),
                ("bvh_node_count", C.c_uint64), ("bvh_prims", C.c_void_p), ("bvh_prim_count", C.c_uint64),
                ("materials", C.c_void_p), ("material_count", C.c_uint64), ("lights", C.c_void_p),
                ("light_count", C.c_uint64), ("tex_albedo", TextureArray), ("tex_mr", TextureArray),
                ("tex_emissive", TextureArray), ("tex_normal", TextureArray), ("bounds_min", f3),
                ("bounds_max", f3), ("has_bounds", u32), ("_pad", u32)]


class Camera(C.Structure):
    _fields_ = [("position", f3), ("look_at", f3), ("up", f3), ("fov_degrees", C.c_float), ("near_plane", C.c_float),
                ("aperture", C.c_float), ("focus_dist", C.c_float)]


BVH_NODE_DTYPE = np.dtype([("bbox_min", "<f4", 3), ("left_first", "<u4"), ("bbox_max", "<f4", 3),
                           ("right_child", "<u4"), ("prim_count", "<u4"), ("_pad", "<f4", 3)])

PHOTON_DTYPE = np.dtype([("position", "<f4", 3), ("_pad0", "<f4"), ("power", "<f4", 3), ("_pad1", "<f4"),
                         ("incident", "<f4", 3), ("_pad2", "<f4"), ("normal", "<f4", 3), ("_pad3", "<f4")])

vp = C.c_void_p
_PROTOS = {
    "oracle_rng_sequence": (u32, [u32, u32, vp, vp]),
    "oracle_sincos": (None, [vp, C.c_uint64, vp, vp]),
    "oracle_intersect_triangle": (C.c_float, [vp, vp, vp, vp, vp]),
    "oracle_trace_rays": (None, [vp, vp, vp, C.c_uint64, vp, vp, C.c_int]),
    "oracle_gather": (C.c_int, [vp, C.POINTER(CameraUniform), C.POINTER(ImageParams), u32, C.POINTER(GridParams),
                                vp, C.c_uint64, vp, u32, u32, C.c_int, vp, vp, vp, vp]),
    "oracle_denoise_pass": (None, [vp, vp, vp, vp, C.POINTER(DenoiseParams), C.c_int]),
    "oracle_composite": (None, [vp, vp, C.POINTER(CompositeParams)]),
    "oracle_tonemap": (None, [vp, vp, C.POINTER(TonemapParams), u32, vp]),
    "oracle_photon_trace": (None, [vp, C.POINTER(GridParams), u32, u32, vp, C.c_uint64, C.c_int]),
    "oracle_photon_keys": (None, [vp, C.c_uint64, C.POINTER(GridParams), vp]),
    "oracle_photon_grid": (C.c_uint64, [vp, C.c_uint64, C.POINTER(GridParams), vp, vp, vp]),
    "oracle_camera_to_uniform": (None, [vp, vp, vp, C.c_float, C.c_float, C.c_float, C.c_float, u32, u32,
                                        C.POINTER(CameraUniform)]),
    "oracle_derive_grid": (None, [vp, vp, C.c_int, u32, u32, u32, C.POINTER(GridParams), C.POINTER(C.c_float)]),
    "oracle_scene_cornell555": (vp, []),
    "oracle_scene_icosphere_room": (vp, [u32, C.c_uint64, C.c_float, u32]),
    "oracle_scene_from_arrays": (vp, [vp, C.c_uint64, vp, C.c_uint64, vp, C.c_uint64, vp]),
    "oracle_scene_describe": (None, [vp, C.POINTER(SceneDesc)]),
    "oracle_scene_camera": (None, [vp, C.POINTER(Camera)]),
    "oracle_scene_destroy": (None, [vp]),
    "oracle_bvh_build": (C.c_uint64, [vp, vp, vp, C.c_uint64, vp, vp]),
}

_lib: C.CDLL | None = None


def build(force: bool = False) -> Path:
    """Compiles oracle/oracle.cpp with the committed Makefile (g++, -ffp-contract=off)."""
    args = ["make", "-C", str(HERE)]
    if force:
        args.insert(1, "-B")
    res = subprocess.run(args, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"building the oracle failed:\n{res.stdout}\n{res.stderr}")
    return LIB


def load() -> C.CDLL:
    global _lib
    if _lib is None:
        if not LIB.exists():
            build()
        lib = C.CDLL(str(LIB))
        for name, (res, args) in _PROTOS.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
    return _lib


def _p(a: np.ndarray | None):
    return None if a is None else C.c_void_p(a.ctypes.data)


def rng_sequence(seed: int, n: int) -> tuple[np.ndarray, np.ndarray]:
    u = np.empty(n, np.uint32)
    f = np.empty(n, np.float32)
    load().oracle_rng_sequence(seed, n, _p(u), _p(f))
    return u, f


def sincos(x: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
    """The fixed-sequence sin and cos both backends use for sampling angles."""
    a = np.ascontiguousarray(x, np.float32)
    s = np.empty_like(a)
    c = np.empty_like(a)
    load().oracle_sincos(_p(a), len(a), _p(s), _p(c))
    return s, c


def trace_rays(scene_desc, origins: np.ndarray, dirs: np.ndarray, threads: int = 0):
    o = np.ascontiguousarray(origins, np.float32)
    d = np.ascontiguousarray(dirs, np.float32)
    t = np.empty(len(o), np.float32)
    prim = np.empty(len(o), np.uint32)
    load().oracle_trace_rays(C.cast(C.pointer(scene_desc), vp), _p(o), _p(d), len(o), _p(t), _p(prim), threads)
    return t, prim


def camera_uniform(position, look_at, up, fov_degrees, width, height, near=0.1, aperture=0.0, focus_dist=5.0):
    u = CameraUniform()
    pos, la, upv = (np.asarray(x, np.float32) for x in (position, look_at, up))
    load().oracle_camera_to_uniform(_p(pos), _p(la), _p(upv), fov_degrees, near, aperture, focus_dist, width, height,
                                    C.byref(u))
    return u


def derive_grid(bounds, grid_max_dim=0, radius_mode=0, photon_slots=1):
    gp = GridParams()
    r = C.c_float(0.0)
    if bounds is None:
        load().oracle_derive_grid(None, None, 0, grid_max_dim, radius_mode, photon_slots, C.byref(gp), C.byref(r))
    else:
        bmin, bmax = (np.asarray(b, np.float32) for b in bounds)
        load().oracle_derive_grid(_p(bmin), _p(bmax), 1, grid_max_dim, radius_mode, photon_slots, C.byref(gp),
                                  C.byref(r))
    return gp, r.value


def denoise_pass(frame, gbuffer, moments, step, alpha, threads=0):
    h, w, _ = frame.shape
    dp = DenoiseParams(w, h, step, 3.0, 12.0, 0.05, alpha, 0)
    f, g, m = (np.ascontiguousarray(x, np.float32) for x in (frame, gbuffer, moments))
    out = np.empty_like(f)
    load().oracle_denoise_pass(_p(f), _p(out), _p(g), _p(m), C.byref(dp), threads)
    return out


def denoise(frame, gbuffer, moments, alpha, passes=2, threads=0):
    cur = np.ascontiguousarray(frame, np.float32)
    for it in range(passes):
        cur = denoise_pass(cur, gbuffer, moments, 1 << it, alpha, threads)
    return cur


def composite(frame, accum, alpha):
    h, w, _ = frame.shape
    cp = CompositeParams(w, h, alpha, 0)
    acc = np.array(accum, np.float32, copy=True, order="C")
    f = np.ascontiguousarray(frame, np.float32)
    load().oracle_composite(_p(f), _p(acc), C.byref(cp))
    return acc


def tonemap(accum, exposure=1.0, gamma=2.2, marker=(0.0, 0.0, 0.0, 0.0), glow=1.0, gbuffer=None):
    h, w, _ = accum.shape
    tp = TonemapParams(exposure, gamma, w, glow, (C.c_float * 4)(*map(float, marker)))
    a = np.ascontiguousarray(accum, np.float32)
    g = None if gbuffer is None else np.ascontiguousarray(gbuffer, np.float32)
    out = np.empty((h, w, 4), np.uint8)
    load().oracle_tonemap(_p(a), _p(g), C.byref(tp), h, _p(out))
    return out


def photon_keys(photons: np.ndarray, gp: GridParams) -> np.ndarray:
    p = np.ascontiguousarray(photons)
    keys = np.empty(len(p), np.uint32)
    load().oracle_photon_keys(_p(p), len(p), C.byref(gp), _p(keys))
    return keys


def photon_grid(photons: np.ndarray, gp: GridParams):
    """(counts, meta (cells x 2), sorted photons, number binned) of a photon slot buffer."""
    p = np.ascontiguousarray(photons)
    counts = np.empty(gp.num_cells, np.uint32)
    meta = np.empty((gp.num_cells, 2), np.uint32)
    srt = np.empty(len(p), p.dtype)
    n = load().oracle_photon_grid(_p(p), len(p), C.byref(gp), _p(counts), _p(meta), _p(srt))
    return counts, meta, srt, int(n)


class Config:
    """The RenderConfig fields the oracle reads (rustracer-renderer/src/lib.rs:21-65 and its defaults,
    plus the max_bounces / denoise_passes / grid extensions; 0 means the reference's value)."""

    def __init__(self, **kw):
        self.width, self.height, self.photon_count, self.spp = 800, 600, 1_000_000, 1
        self.exposure, self.gamma = 1.0, 2.2
        self.light_emission, self.point_light_emission = (1.0, 1.0, 1.0), (1.0, 1.0, 1.0)
        self.accumulate_frames, self.enable_photon_map, self.enable_denoise = 0, False, True
        self.photon_debug, self.debug_view, self.photon_scale, self.photon_radius = False, 0, 0.02, 0.5
        self.ambient = 0.03
        self.max_bounces, self.denoise_passes, self.grid_max_dim, self.photon_radius_mode = 0, 0, 0, 0
        for k, v in kw.items():
            if not hasattr(self, k):
                raise AttributeError(f"unknown config field {k}")
            setattr(self, k, v)


class OracleScene:
    """A scene generated and indexed by the oracle itself (oracle/scene.cpp): its own flattening and
    SAH BVH build, so the oracle's traversal does not depend on the CUDA backend's host code."""

    def __init__(self, handle: int, keep=None):
        if not handle:
            raise RuntimeError("the oracle rejected the scene arguments")
        self._h = C.c_void_p(handle)
        self._keep = keep
        self.desc = SceneDesc()
        load().oracle_scene_describe(self._h, C.byref(self.desc))

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            load().oracle_scene_destroy(h)
            self._h = None

    @staticmethod
    def cornell555() -> "OracleScene":
        return OracleScene(load().oracle_scene_cornell555())

    @staticmethod
    def icosphere_room(level: int = 8, seed: int = 0, sigma: float = 0.02, tex_size: int = 1024) -> "OracleScene":
        return OracleScene(load().oracle_scene_icosphere_room(level, seed, sigma, tex_size))

    @staticmethod
    def from_arrays(triangles: np.ndarray, materials: np.ndarray, lights: np.ndarray,
                    textures=None) -> "OracleScene":
        """triangles / materials / lights: arrays of the 128 / 64 / 64-byte records; textures: up to
        four (layers, h, w, 4) uint8 arrays or None per role (albedo, MR, emissive, normal)."""
        t, m, li = (np.ascontiguousarray(x) for x in (triangles, materials, lights))
        tex = (TextureArray * 4)()
        keep = [t, m, li]
        for r, arr in enumerate(textures or []):
            if arr is None or arr.size == 0:
                continue
            a = np.ascontiguousarray(arr, np.uint8)
            if a.ndim == 3:
                a = a[None]
            keep.append(a)
            tex[r].rgba8 = a.ctypes.data
            tex[r].layers, tex[r].height, tex[r].width = a.shape[0], a.shape[1], a.shape[2]
        h = load().oracle_scene_from_arrays(_p(t), len(t), _p(m), len(m), _p(li) if len(li) else None, len(li), tex)
        return OracleScene(h, keep)

    def camera(self) -> Camera:
        c = Camera()
        load().oracle_scene_camera(self._h, C.byref(c))
        return c

    def arrays(self) -> dict[str, np.ndarray]:
        """Byte copies of the flattened arrays (triangles / materials / lights as raw records)."""
        d = self.desc

        def raw(ptr, n, size):
            if n == 0:
                return np.zeros((0, size), np.uint8)
            return np.ctypeslib.as_array(C.cast(ptr, C.POINTER(C.c_uint8)), shape=(n * size,)).reshape(n, size).copy()

        out = {"triangles": raw(d.triangles, d.triangle_count, 128), "materials": raw(d.materials, d.material_count, 64),
               "lights": raw(d.lights, d.light_count, 64),
               "bvh_nodes": raw(d.bvh_nodes, d.bvh_node_count, 48).view(BVH_NODE_DTYPE).reshape(-1),
               "bvh_prims": raw(d.bvh_prims, d.bvh_prim_count, 4).view(np.uint32).reshape(-1)}
        for name in ("tex_albedo", "tex_mr", "tex_emissive", "tex_normal"):
            t = getattr(d, name)
            n = t.width * t.height * t.layers * 4
            out[name] = (np.ctypeslib.as_array(C.cast(t.rgba8, C.POINTER(C.c_uint8)), shape=(n,)).copy()
                         if t.layers and t.rgba8 else np.zeros(0, np.uint8))
        out["bounds"] = (np.array(d.bounds_min, np.float32), np.array(d.bounds_max, np.float32), int(d.has_bounds))
        return out


def bvh_build(centroids: np.ndarray, bmin: np.ndarray, bmax: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
    """The oracle's SAH build on raw primitive centroids and boxes: (nodes, prim indices)."""
    c, lo, hi = (np.ascontiguousarray(x, np.float32).reshape(-1, 3) for x in (centroids, bmin, bmax))
    n = len(c)
    nodes = np.zeros(max(2 * n, 1), BVH_NODE_DTYPE)
    prims = np.zeros(max(n, 1), np.uint32)
    k = load().oracle_bvh_build(_p(c), _p(lo), _p(hi), n, _p(nodes), _p(prims))
    return nodes[:k].copy(), prims[:n].copy()


class OracleRenderer:
    """CPU driver of the reference's frame schedule over the oracle kernels.

    scene_desc: an rt_scene_desc (ctypes) whose arrays stay alive; config: an object with the
    RenderConfig attribute names; camera_uniform: a 96-byte camera uniform.
    """

    def __init__(self, scene_desc, config, camera_uniform=None, threads: int = 0):
        if isinstance(scene_desc, OracleScene):
            self.scene = scene_desc
            scene_desc = scene_desc.desc
        self.desc = scene_desc
        self.cfg = config
        self.threads = threads
        w, h = config.width, config.height
        self.cam = camera_uniform
        self.accum = np.zeros((h, w, 4), np.float32)
        self.frame = np.zeros((h, w, 4), np.float32)
        self.moments = np.zeros((h, w, 4), np.float32)
        self.gbuffer = np.zeros((h, w, 4), np.float32)
        self.output = np.zeros((h, w, 4), np.uint8)
        self.sample_counter = 0
        self.frames_since_reset = 0
        self.counters = np.zeros(5, np.uint64)  # segments, shadow rays, node fetches, tri tests, hits
        slots = max(config.photon_count * 6, 1) if config.enable_photon_map else 1
        bounds = None
        if scene_desc.has_bounds:
            bounds = (np.array(scene_desc.bounds_min, np.float32), np.array(scene_desc.bounds_max, np.float32))
        self.gp, self.photon_radius = derive_grid(bounds, config.grid_max_dim, config.photon_radius_mode, slots)
        self.photons = np.zeros(slots, PHOTON_DTYPE)
        self.sorted = np.zeros(slots, PHOTON_DTYPE)
        self.grid_counts = np.zeros(self.gp.num_cells, np.uint32)
        self.grid_meta = np.zeros((self.gp.num_cells, 2), np.uint32)
        self.binned = 0
        self.marker = (0.0, 0.0, 0.0, 0.0)
        self.glow = 1.0

    def image_params(self, alpha: float) -> ImageParams:
        c = self.cfg
        ip = ImageParams()
        ip.width, ip.height, ip.spp, ip.frame = c.width, c.height, c.spp, self.sample_counter
        ip.light_emission[:] = tuple(c.light_emission)
        ip.point_light_emission[:] = tuple(c.point_light_emission)
        ip.ambient = c.ambient
        ip.accumulate_alpha = alpha
        ip.use_photons = 1 if c.enable_photon_map else 0
        ip.photon_count = c.photon_count
        ip.photon_radius = self.photon_radius
        ip.photon_scale = c.photon_scale
        ip.photon_debug = 1 if c.photon_debug else 0
        ip._pad[0] = c.debug_view
        return ip

    def alpha(self) -> float:
        n = self.cfg.accumulate_frames
        if n == 0:
            return 1.0
        return float(np.float32(1.0) / np.float32(min(self.frames_since_reset, n)))

    def record_frame(self, rows=None) -> None:
        """record_frame (lib.rs:666-851).  rows restricts the gather to a row range (r0, r1) or to a list
        of such ranges (sampled rows of a large frame); the other rows of frame, moments and gbuffer keep
        their contents, and the denoise / composite / tonemap stages run over the whole image."""
        c = self.cfg
        self.sample_counter = (self.sample_counter + 1) & 0xFFFFFFFF
        self.frames_since_reset = min(self.frames_since_reset + 1, 0xFFFFFFFF)
        alpha = self.alpha()
        ip = self.image_params(alpha)
        if rows is None:
            ranges = [(0, c.height)]
        elif isinstance(rows[0], (tuple, list)):
            ranges = [tuple(r) for r in rows]
        else:
            ranges = [tuple(rows)]
        mb = c.max_bounces or 6
        use = ip.use_photons == 1
        for r0, r1 in ranges:
            st = load().oracle_gather(C.cast(C.pointer(self.desc), vp), C.byref(self.cam), C.byref(ip), mb,
                                      C.byref(self.gp), _p(self.sorted) if use else None, len(self.sorted),
                                      _p(self.grid_meta) if use else None, r0, r1, self.threads, _p(self.frame),
                                      _p(self.moments), _p(self.gbuffer), _p(self.counters))
            if st != 0:
                raise RuntimeError("oracle_gather rejected its arguments")
        result = self.frame
        if c.enable_denoise:
            result = denoise(self.frame, self.gbuffer, self.moments, alpha, c.denoise_passes or 2, self.threads)
        self.result = result
        self.accum = composite(result, self.accum, alpha)
        self.output = tonemap(self.accum, c.exposure, c.gamma, self.marker, self.glow, self.gbuffer)

    def rebuild_photons(self) -> None:
        """rebuild_photons (lib.rs:913-1037) with the grid scatter in slot order."""
        P = max(self.cfg.photon_count, 1)
        traced = min(max(P // 256, 1) * 256, self.cfg.photon_count)
        load().oracle_photon_trace(C.cast(C.pointer(self.desc), vp), C.byref(self.gp), 0, traced, _p(self.photons),
                                   len(self.photons), self.threads)
        self._build_grid()

    def load_photons(self, photons: np.ndarray) -> None:
        self.photons = np.array(photons, PHOTON_DTYPE, copy=True)
        self._build_grid()

    def _build_grid(self) -> None:
        P = max(self.cfg.photon_count, 1)
        dispatched = max(((P * 6) & 0xFFFFFFFF) // 256, 1) * 256
        n = min(dispatched, len(self.photons))
        gp = GridParams.from_buffer_copy(self.gp)
        counts, meta, srt, binned = photon_grid(self.photons[:n], gp)
        self.grid_counts, self.grid_meta, self.binned = counts, meta, binned
        self.sorted = np.zeros(len(self.photons), PHOTON_DTYPE)
        self.sorted[:n] = srt
