"""glTF 2.0 scene ingest (rustracer-core/src/loader.rs:265-649) and scene.toml overrides
(rustracer-core/src/config.rs:60-164), producing the native Scene the renderer consumes.

    model = load_gltf_model("scene.gltf")          # host model: meshes, materials, lights, role textures
    apply_descriptor(model, parse_descriptor(open("scene.toml").read()))   # optional
    scene = model.to_scene()                        # flattened + BVH (rt_scene_*)

What the reference's loader does is done here the same way: the default scene's node hierarchy is
baked into world space (matrix or TRS per node, children in document order), strips and fans are
triangulated, missing normals are computed as smooth vertex normals, normals are transformed by the
inverse transpose and the winding is flipped under mirroring transforms; materials take the
metallic-roughness factors (NaN or negative roughness -> 1, metallic -> 0), alphaMode MASK becomes an
alpha cut-out and BLEND solid glass; textures go into one array per role (albedo, metallic-roughness,
emissive, normal), sRGB-decoded for albedo and emissive, normal maps with their scale baked into X/Y,
sized by the first texture used in the role (others are dropped, at most 240 layers); every triangle
of an emitting material whose emissive colour at its centroid is bright enough becomes an area light,
and a procedural sky is added when no environment light exists.  Images decoded here: PNG (8/16-bit
grey, grey+alpha, RGB, RGBA, palette; non-interlaced) and JPEG (baseline, extended and progressive
Huffman, 8-bit grey or YCbCr, through rt_jpeg_decode); other streams fall back to the reference's
solid grey texture, as an undecodable image does there.
"""
from __future__ import annotations

import base64
import json
import math
import struct
import warnings
import zlib
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np

from . import _abi as A
from .scene import Scene, area_light, environment_light, directional_light, material, point_light

MAX_ROLE_LAYERS = 240  # loader.rs:23


# ---------------------------------------------------------------------------------------------------
# Textures (loader.rs:28-124)
# ---------------------------------------------------------------------------------------------------
def srgb_to_linear(c):
    """loader.rs:28-34 (the glTF sRGB transfer function), elementwise in float32."""
    c = np.asarray(c, np.float32)
    return np.where(c <= np.float32(0.04045), c / np.float32(12.92),
                    ((c + np.float32(0.055)) / np.float32(1.055)) ** np.float32(2.4)).astype(np.float32)


@dataclass
class Texture:
    """rustracer-core Texture: width x height linear RGBA floats, row-major."""
    width: int
    height: int
    data: np.ndarray  # (height, width, 4) float32

    @staticmethod
    def solid(color) -> "Texture":
        return Texture(1, 1, np.asarray(color, np.float32).reshape(1, 1, 4).copy())


def decode_jpeg(data: bytes) -> Texture | None:
    """JPEG to linear [0, 1] RGBA floats through the native decoder (rt_jpeg_decode); None when the
    stream is not a JPEG this decoder handles."""
    if data[:2] != b"\xff\xd8":
        return None
    lib = A.load()
    buf = np.frombuffer(data, np.uint8)
    w, h = A.C.c_uint32(), A.C.c_uint32()
    if lib.rt_jpeg_decode(buf.ctypes.data, len(buf), None, 0, A.C.byref(w), A.C.byref(h)) != A.RT_OK:
        return None
    out = np.empty((h.value, w.value, 4), np.uint8)
    if lib.rt_jpeg_decode(buf.ctypes.data, len(buf), out.ctypes.data, out.nbytes, A.C.byref(w),
                          A.C.byref(h)) != A.RT_OK:
        return None
    return Texture(w.value, h.value, out.astype(np.float32) / 255.0)


def decode_image(data: bytes) -> Texture | None:
    """The image formats the ingest decodes: PNG and JPEG."""
    return decode_png(data) if data[:8] == b"\x89PNG\r\n\x1a\n" else decode_jpeg(data)


def decode_png(data: bytes) -> Texture | None:
    """PNG to linear [0, 1] RGBA floats (loader.rs:36-100 does the same for the decoded formats)."""
    if data[:8] != b"\x89PNG\r\n\x1a\n":
        return None
    pos, idat, plte, trns = 8, [], None, None
    w = h = depth = ctype = interlace = None
    while pos + 8 <= len(data):
        n, tag = struct.unpack(">I4s", data[pos:pos + 8])
        body = data[pos + 8:pos + 8 + n]
        if tag == b"IHDR":
            w, h, depth, ctype, _, _, interlace = struct.unpack(">IIBBBBB", body)
        elif tag == b"PLTE":
            plte = np.frombuffer(body, np.uint8).reshape(-1, 3)
        elif tag == b"tRNS":
            trns = np.frombuffer(body, np.uint8)
        elif tag == b"IDAT":
            idat.append(body)
        elif tag == b"IEND":
            break
        pos += 12 + n
    if w is None or interlace != 0 or depth not in (8, 16) and not (ctype == 3 and depth in (1, 2, 4, 8)):
        return None
    channels = {0: 1, 2: 3, 3: 1, 4: 2, 6: 4}.get(ctype)
    if channels is None:
        return None
    raw = zlib.decompress(b"".join(idat))
    bits = channels * depth
    stride = (w * bits + 7) // 8
    bpp = max(1, bits // 8)
    rows = np.ascontiguousarray(np.frombuffer(raw, np.uint8)[:h * (stride + 1)])
    if len(rows) < h * (stride + 1):
        return None
    out = np.empty((h, stride), np.uint8)
    lib = A.load()
    if lib.rt_png_unfilter(rows.ctypes.data_as(A.C.POINTER(A.C.c_uint8)), h, stride, bpp,
                           out.ctypes.data_as(A.C.POINTER(A.C.c_uint8))) != A.RT_OK:
        return None
    if ctype == 3:
        idx = np.unpackbits(out, axis=1)[:, :w * depth].reshape(h, w, depth) if depth < 8 else out[:, :w, None]
        if depth < 8:
            idx = (idx * (1 << np.arange(depth - 1, -1, -1))).sum(-1)
        idx = np.asarray(idx).reshape(h, w).astype(np.int64)
        rgb = plte[np.minimum(idx, len(plte) - 1)].astype(np.float32) / 255.0
        alpha = np.ones((h, w, 1), np.float32)
        if trns is not None:
            a = np.full(len(plte), 255, np.uint8)
            a[:len(trns)] = trns[:len(plte)]
            alpha = (a[np.minimum(idx, len(plte) - 1)].astype(np.float32) / 255.0)[..., None]
        return Texture(w, h, np.concatenate([rgb, alpha], -1).astype(np.float32))
    if depth == 16:
        v = out.reshape(h, -1).view(">u2").astype(np.float32) / 65535.0
    else:
        v = out.astype(np.float32) / 255.0
    v = v.reshape(h, w, channels)
    if channels == 1:
        v = np.concatenate([v, v, v, np.ones_like(v)], -1)
    elif channels == 2:
        v = np.concatenate([v[..., :1]] * 3 + [v[..., 1:2]], -1)
    elif channels == 3:
        v = np.concatenate([v, np.ones_like(v[..., :1])], -1)
    return Texture(w, h, v.astype(np.float32))


def build_role(master: list[Texture], used: list[int | None], srgb: bool, scales=None):
    """loader.rs:131-229 (build_role / build_role_scaled): every used master texture, once, into one
    role array sized by the first used texture; returns (role textures, map master index -> layer)."""
    mapping: list[int | None] = [None] * len(master)
    if not master:
        return [], mapping
    first = next((u for u in used if u is not None), 0)
    ref = (master[first].width, master[first].height)
    role: list[Texture] = []
    for m in used:
        if m is None or mapping[m] is not None:
            continue
        tex = master[m]
        if (tex.width, tex.height) != ref:
            warnings.warn(f"dropping {tex.width}x{tex.height} texture from an array of {ref[0]}x{ref[1]} textures")
            continue
        if len(role) >= MAX_ROLE_LAYERS:
            warnings.warn(f"too many textures for one role array (max {MAX_ROLE_LAYERS}); dropping the rest")
            continue
        data = tex.data.copy()
        if srgb:
            data[..., :3] = srgb_to_linear(data[..., :3])
        if scales is not None:
            s = np.float32(scales[m] if m < len(scales) else 1.0)
            if abs(float(s) - 1.0) > 1e-6:
                data[..., 0] *= s
                data[..., 1] *= s
        mapping[m] = len(role)
        role.append(Texture(tex.width, tex.height, data))
    return role, mapping


def sample_nearest(tex: Texture, u: float, v: float):
    """loader.rs:255-264."""
    if tex.width == 0 or tex.height == 0:
        return np.zeros(4, np.float32)
    u = math.fmod(u, 1.0) % 1.0
    v = math.fmod(v, 1.0) % 1.0
    x = min(int(np.float32(u) * np.float32(tex.width)), tex.width - 1)
    y = min(int(np.float32(v) * np.float32(tex.height)), tex.height - 1)
    return tex.data[y, x]


# ---------------------------------------------------------------------------------------------------
# Host model
# ---------------------------------------------------------------------------------------------------
@dataclass
class Mat:
    """Material (material.rs:60-97) with role-layer texture indices."""
    kind: int = A.MAT_LAMBERTIAN
    albedo: tuple = (0.8, 0.8, 0.8)
    roughness: float = 0.5
    metallic: float = 0.0
    ior: float = 1.5
    emissive: tuple = (0.0, 0.0, 0.0)
    albedo_texture: int | None = None
    roughness_texture: int | None = None
    emissive_texture: int | None = None
    normal_texture: int | None = None
    alpha_cutout: bool = False

    def emits_light(self) -> bool:  # material.rs:177-179
        return self.emissive_texture is not None or float(np.linalg.norm(np.float32(self.emissive))) > 1e-4

    def to_gpu(self) -> A.Material:  # material.rs:143-161
        none = lambda t: A.TEX_NONE if t is None else t  # noqa: E731
        return material(self.kind, self.albedo, self.roughness, self.metallic, self.ior, self.emissive,
                        self.alpha_cutout, none(self.albedo_texture), none(self.roughness_texture),
                        none(self.emissive_texture), none(self.normal_texture))


@dataclass
class MeshData:
    positions: np.ndarray  # (n, 3) float32, world space
    normals: np.ndarray    # (n, 3) float32
    uvs: np.ndarray        # (n, 2) float32
    indices: np.ndarray    # (3 t,) uint32
    material_id: int

    def triangle_count(self) -> int:
        return len(self.indices) // 3


@dataclass
class Model:
    meshes: list[MeshData] = field(default_factory=list)
    materials: list[Mat] = field(default_factory=list)
    lights: list[A.Light] = field(default_factory=list)
    tex_albedo: list[Texture] = field(default_factory=list)
    tex_mr: list[Texture] = field(default_factory=list)
    tex_emissive: list[Texture] = field(default_factory=list)
    tex_normal: list[Texture] = field(default_factory=list)

    def triangle_count(self) -> int:
        return sum(m.triangle_count() for m in self.meshes)

    def to_scene(self) -> Scene:
        """The native scene: role arrays quantised as the renderer uploads them
        (rustracer-renderer/src/lib.rs:1315-1326, `(c.clamp(0, 1) * 255) as u8`), then materials,
        meshes and lights in order (flattened and BVH-built by rt_scene_finalize)."""
        s = Scene()
        for role, texs in ((A.TEX_ALBEDO, self.tex_albedo), (A.TEX_MR, self.tex_mr),
                           (A.TEX_EMISSIVE, self.tex_emissive), (A.TEX_NORMAL, self.tex_normal)):
            if texs:
                arr = np.stack([t.data for t in texs])
                s.set_textures(role, (np.clip(arr, 0.0, 1.0) * np.float32(255.0)).astype(np.uint8))
        for m in self.materials:
            s.add_material(m.to_gpu())
        for mesh in self.meshes:
            s.add_mesh(mesh.positions, mesh.indices, mesh.material_id, mesh.normals, mesh.uvs)
        for l in self.lights:
            s.add_light(l)
        return s


def triangle_emits(mesh: MeshData, tri: int, mat: Mat, tex_emissive: list[Texture]) -> bool:
    """loader.rs:241-253: untextured emissives always emit; textured ones when the emissive colour
    at the triangle's centroid UV (nearest texel) is bright enough."""
    if mat.emissive_texture is None:
        return float(np.linalg.norm(np.float32(mat.emissive))) > 1e-4
    if mat.emissive_texture >= len(tex_emissive):
        return False
    i = mesh.indices[3 * tri:3 * tri + 3]
    uv = (mesh.uvs[i[0]] + mesh.uvs[i[1]] + mesh.uvs[i[2]]) / np.float32(3.0)
    c = sample_nearest(tex_emissive[mat.emissive_texture], float(uv[0]), float(uv[1]))
    e = np.float32(mat.emissive)
    return float(c[0] * e[0] + c[1] * e[1] + c[2] * e[2]) > 0.05


# ---------------------------------------------------------------------------------------------------
# glTF container, accessors
# ---------------------------------------------------------------------------------------------------
_COMPONENT = {5120: np.int8, 5121: np.uint8, 5122: np.int16, 5123: np.uint16, 5125: np.uint32, 5126: np.float32}
_NCOMP = {"SCALAR": 1, "VEC2": 2, "VEC3": 3, "VEC4": 4, "MAT4": 16}


def _read_uri(uri: str, base: Path) -> bytes:
    if uri.startswith("data:"):
        return base64.b64decode(uri.split(",", 1)[1])
    return (base / uri).read_bytes()


class _Doc:
    def __init__(self, path: Path):
        raw = path.read_bytes()
        bin_chunk = None
        if raw[:4] == b"glTF":
            _, _, length = struct.unpack("<4sII", raw[:12])
            pos, js = 12, None
            while pos < length:
                clen, ctype = struct.unpack("<I4s", raw[pos:pos + 8])
                chunk = raw[pos + 8:pos + 8 + clen]
                if ctype == b"JSON":
                    js = json.loads(chunk.decode("utf-8"))
                elif ctype == b"BIN\x00":
                    bin_chunk = chunk
                pos += 8 + clen
            self.j = js
        else:
            self.j = json.loads(raw.decode("utf-8"))
        self.base = path.parent
        self.buffers = []
        for b in self.j.get("buffers", []):
            self.buffers.append(_read_uri(b["uri"], self.base) if "uri" in b else bin_chunk)

    def view_bytes(self, index: int) -> tuple[bytes, int]:
        v = self.j["bufferViews"][index]
        off = v.get("byteOffset", 0)
        return self.buffers[v["buffer"]][off:off + v["byteLength"]], v.get("byteStride", 0)

    def accessor(self, index: int) -> np.ndarray:
        a = self.j["accessors"][index]
        dt = np.dtype(_COMPONENT[a["componentType"]]).newbyteorder("<")
        nc = _NCOMP[a["type"]]
        count = a["count"]
        if "bufferView" in a:
            data, stride = self.view_bytes(a["bufferView"])
            off = a.get("byteOffset", 0)
            elem = dt.itemsize * nc
            stride = stride or elem
            buf = np.frombuffer(data, np.uint8)
            rows = np.lib.stride_tricks.as_strided(buf[off:], shape=(count, elem), strides=(stride, 1)) if count else \
                np.zeros((0, elem), np.uint8)
            out = np.ascontiguousarray(rows).view(dt).reshape(count, nc)
        else:
            out = np.zeros((count, nc), dt)
        if a.get("normalized") and dt.kind in "iu":
            out = out.astype(np.float32) / np.float32(np.iinfo(dt).max)
            if dt.kind == "i":
                out = np.maximum(out, -1.0)
        return out

    def image_bytes(self, img: dict) -> bytes:
        if "uri" in img:
            return _read_uri(img["uri"], self.base)
        return self.view_bytes(img["bufferView"])[0]


def _node_matrix(n: dict) -> np.ndarray:
    if "matrix" in n:
        return np.asarray(n["matrix"], np.float32).reshape(4, 4).T  # column-major in the file
    t = np.asarray(n.get("translation", [0, 0, 0]), np.float32)
    q = np.asarray(n.get("rotation", [0, 0, 0, 1]), np.float32)
    s = np.asarray(n.get("scale", [1, 1, 1]), np.float32)
    x, y, z, w = q
    r = np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                  [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                  [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]], np.float32)
    m = np.eye(4, dtype=np.float32)
    m[:3, :3] = r * s[None, :]
    m[:3, 3] = t
    return m


def _triangulate(mode: int, idx: np.ndarray) -> np.ndarray:
    """loader.rs:520-546."""
    if mode == 4:
        n = len(idx) // 3 * 3
        return idx[:n].reshape(-1, 3)
    out = []
    if mode == 5:
        for i in range(max(len(idx) - 2, 0)):
            a, b, c = idx[i], idx[i + 1], idx[i + 2]
            out.append((a, b, c) if i % 2 == 0 else (a, c, b))
    elif mode == 6:
        for i in range(1, max(len(idx) - 1, 1)):
            out.append((idx[0], idx[i], idx[i + 1]))
    return np.asarray(out, np.uint32).reshape(-1, 3)


def _bake_primitive(doc: _Doc, prim: dict, world: np.ndarray, n_materials: int) -> MeshData | None:
    """loader.rs:502-649."""
    attrs = prim.get("attributes", {})
    if "POSITION" not in attrs:
        return None
    positions = doc.accessor(attrs["POSITION"]).astype(np.float32)
    if len(positions) == 0:
        return None
    n_verts = len(positions)
    idx = doc.accessor(prim["indices"]).reshape(-1).astype(np.uint32) if "indices" in prim else \
        np.arange(n_verts, dtype=np.uint32)
    mode = prim.get("mode", 4)
    if mode not in (4, 5, 6):
        warnings.warn(f"primitive mode {mode} is not supported; skipping")
        return None
    tris = _triangulate(mode, idx)
    if len(tris) == 0:
        return None
    if "NORMAL" in attrs:
        normals = doc.accessor(attrs["NORMAL"]).astype(np.float32)
    else:
        acc = np.zeros((n_verts, 3), np.float32)
        p = positions
        fn = np.cross(p[tris[:, 1]] - p[tris[:, 0]], p[tris[:, 2]] - p[tris[:, 0]]).astype(np.float32)
        for k in range(3):
            np.add.at(acc, tris[:, k], fn)
        ln2 = (acc * acc).sum(1)
        normals = np.where(ln2[:, None] > 1e-12, acc / np.sqrt(np.maximum(ln2, 1e-30))[:, None],
                           np.array([0, 1, 0], np.float32)).astype(np.float32)
    if len(normals) != n_verts:
        normals = np.tile(np.array([0, 1, 0], np.float32), (n_verts, 1))
    uvs = doc.accessor(attrs["TEXCOORD_0"]).astype(np.float32)[:, :2] if "TEXCOORD_0" in attrs else \
        np.zeros((n_verts, 2), np.float32)
    w = world.astype(np.float64)
    normal_mat = np.linalg.inv(w).T
    mirrored = np.linalg.det(w) < 0.0
    tp = (positions.astype(np.float64) @ w[:3, :3].T + w[:3, 3]).astype(np.float32)
    tn = (normals.astype(np.float64) @ normal_mat[:3, :3].T).astype(np.float32)
    ln2 = (tn * tn).sum(1)
    tn = np.where(ln2[:, None] > 1e-12, tn / np.sqrt(np.maximum(ln2, 1e-30))[:, None], normals).astype(np.float32)
    if mirrored:
        tris = tris[:, [0, 2, 1]]
    mi = prim.get("material")
    material_id = max(n_materials - 1, 0) if mi is None else min(mi, max(n_materials - 1, 0))
    return MeshData(tp, tn, uvs, np.ascontiguousarray(tris.reshape(-1), np.uint32), material_id)


def load_gltf_model(path) -> Model:
    """load_gltf (loader.rs:265-497) up to the Scene: the host model."""
    doc = _Doc(Path(path))
    j = doc.j
    model = Model()
    # textures: master list in glTF texture order
    master: list[Texture] = []
    for t in j.get("textures", []):
        tex = None
        src = t.get("source")
        if src is not None:
            try:
                tex = decode_image(doc.image_bytes(j["images"][src]))
            except Exception:  # noqa: BLE001 - an undecodable image becomes the solid fallback
                tex = None
        if tex is None:
            warnings.warn(f"texture {len(master)}: image not decodable here (PNG and JPEG only); using solid grey")
            tex = Texture.solid([0.5, 0.5, 0.5, 1.0])
        master.append(tex)
    # materials
    pending = []
    for mj in j.get("materials", []):
        pbr = mj.get("pbrMetallicRoughness", {})
        bc = pbr.get("baseColorFactor", [1, 1, 1, 1])
        rough = pbr.get("roughnessFactor", 1.0)
        metal = pbr.get("metallicFactor", 1.0)
        m = Mat(kind=A.MAT_LAMBERTIAN, albedo=tuple(np.float32(bc[:3])), roughness=float(np.float32(rough)),
                metallic=float(np.float32(metal)), ior=1.5, emissive=tuple(np.float32(mj.get("emissiveFactor", [0, 0, 0]))))
        if not (m.roughness >= 0.0):
            m.roughness = 1.0
        if not (m.metallic >= 0.0):
            m.metallic = 0.0
        mode = mj.get("alphaMode", "OPAQUE")
        if mode == "MASK":
            m.alpha_cutout = True
        elif mode == "BLEND":
            warnings.warn(f"material {mj.get('name')!r} uses alphaMode BLEND; rendering it as solid dielectric glass")
            m.kind = A.MAT_DIELECTRIC
        nt = mj.get("normalTexture")
        pending.append(dict(material=m, albedo=pbr.get("baseColorTexture", {}).get("index"),
                            mr=pbr.get("metallicRoughnessTexture", {}).get("index"),
                            emissive=mj.get("emissiveTexture", {}).get("index"),
                            normal=None if nt is None else nt.get("index"),
                            normal_scale=1.0 if nt is None else float(nt.get("scale", 1.0))))
    if not pending:
        pending.append(dict(material=Mat(kind=A.MAT_LAMBERTIAN, albedo=(0.8, 0.8, 0.8), roughness=1.0), albedo=None,
                            mr=None, emissive=None, normal=None, normal_scale=1.0))
    for p in pending:
        if p["emissive"] is not None and float(np.linalg.norm(np.float32(p["material"].emissive))) < 1e-6:
            p["material"].emissive = (1.0, 1.0, 1.0)
    role_albedo, map_albedo = build_role(master, [p["albedo"] for p in pending], True)
    role_mr, map_mr = build_role(master, [p["mr"] for p in pending], False)
    role_emissive, map_emissive = build_role(master, [p["emissive"] for p in pending], True)
    normal_scales = [1.0] * len(master)
    for p in pending:
        i = p["normal"]
        if i is not None:
            if abs(normal_scales[i] - p["normal_scale"]) > 1e-4 and normal_scales[i] != 1.0:
                warnings.warn(f"normal texture {i} reused with different scales; using the first")
            else:
                normal_scales[i] = p["normal_scale"]
    role_normal, map_normal = build_role(master, [p["normal"] for p in pending], False, scales=normal_scales)
    lookup = lambda mp, i: None if i is None or i >= len(mp) else mp[i]  # noqa: E731
    for p in pending:
        m = p["material"]
        m.albedo_texture = lookup(map_albedo, p["albedo"])
        m.roughness_texture = lookup(map_mr, p["mr"])
        m.emissive_texture = lookup(map_emissive, p["emissive"])
        m.normal_texture = lookup(map_normal, p["normal"])
    model.tex_albedo, model.tex_mr, model.tex_emissive, model.tex_normal = role_albedo, role_mr, role_emissive, \
        role_normal
    model.materials = [p["material"] for p in pending]
    # the default scene's nodes, depth first in document order
    scenes = j.get("scenes", [])
    sc = scenes[j["scene"]] if "scene" in j and scenes else (scenes[0] if scenes else None)
    stack = [(n, np.eye(4, dtype=np.float32)) for n in reversed(sc.get("nodes", []))] if sc else []
    if not stack:
        warnings.warn("glTF file has no scene nodes; nothing to render")
    while stack:
        ni, parent = stack.pop()
        node = j["nodes"][ni]
        world = (parent.astype(np.float64) @ _node_matrix(node).astype(np.float64)).astype(np.float32)
        if "mesh" in node:
            if "skin" in node:
                warnings.warn(f"node {node.get('name')!r} is skinned; rendering the bind pose")
            for prim in j["meshes"][node["mesh"]].get("primitives", []):
                if prim.get("targets"):
                    warnings.warn("primitive has morph targets; rendering the base shape")
                md = _bake_primitive(doc, prim, world, len(model.materials))
                if md is not None:
                    model.meshes.append(md)
        for c in reversed(node.get("children", [])):
            stack.append((c, world))
    # area lights from emitting triangles
    tri_offset = 0
    for mesh in model.meshes:
        mat = model.materials[mesh.material_id] if mesh.material_id < len(model.materials) else None
        if mat is not None and mat.emits_light():
            for t in range(mesh.triangle_count()):
                if triangle_emits(mesh, t, mat, model.tex_emissive):
                    model.lights.append(area_light(tri_offset + t, mat.emissive, 1.0))
        tri_offset += mesh.triangle_count()
    if not any(l.kind == A.LIGHT_ENVIRONMENT for l in model.lights):
        model.lights.append(environment_light())
    return model


def load_gltf(path) -> Scene:
    """load_gltf: the glTF file as a native Scene (with a sibling scene.toml applied when present,
    as the reference's app and headless example do)."""
    model = load_gltf_model(path)
    desc = Path(path).with_name("scene.toml")
    if desc.exists():
        apply_descriptor(model, parse_descriptor(desc.read_text()))
    return model.to_scene()


# ---------------------------------------------------------------------------------------------------
# scene.toml (config.rs)
# ---------------------------------------------------------------------------------------------------
def parse_descriptor(text: str) -> dict:
    import tomllib

    return tomllib.loads(text)


_KINDS = {"lambertian": A.MAT_LAMBERTIAN, "metal": A.MAT_METAL, "dielectric": A.MAT_DIELECTRIC,
          "emissive": A.MAT_EMISSIVE}


def _apply_override(mat: Mat, ov: dict) -> None:
    """config.rs:125-164."""
    if "kind" in ov:
        k = _KINDS.get(ov["kind"])
        if k is None:
            warnings.warn(f"unknown material kind {ov['kind']!r}")
        else:
            mat.kind = k
    if mat.kind == A.MAT_METAL and "metallic" not in ov:
        mat.metallic = 1.0
    elif mat.kind == A.MAT_DIELECTRIC:
        if "metallic" not in ov:
            mat.metallic = 0.0
        if "roughness" not in ov:
            mat.roughness = 0.0
        if "ior" not in ov:
            mat.ior = 1.5
    if "albedo" in ov:
        mat.albedo = tuple(np.float32(ov["albedo"]))
    if "roughness" in ov:
        mat.roughness = float(ov["roughness"])
    if "metallic" in ov:
        mat.metallic = float(ov["metallic"])
    if "emissive" in ov:
        mat.emissive = tuple(np.float32(ov["emissive"]))
    if "ior" in ov:
        mat.ior = float(ov["ior"])
    if mat.kind == A.MAT_EMISSIVE and "emissive" not in ov:
        mat.emissive = mat.albedo


def apply_descriptor(model: Model, desc: dict) -> None:
    """config.rs:60-123: environment replaces the existing environment light; lights are appended;
    material overrides go to one index or, without one, to every material."""
    env = desc.get("environment")
    if env is not None:
        model.lights = [l for l in model.lights if l.kind != A.LIGHT_ENVIRONMENT]
        model.lights.append(environment_light(tuple(env.get("sky_zenith", (0.55, 0.6, 0.75))),
                                              tuple(env.get("sky_horizon", (0.95, 0.93, 0.9))),
                                              float(env.get("intensity", 1.0))))
    for lc in desc.get("lights", []):
        color = tuple(lc.get("color", (1.0, 1.0, 1.0)))
        kind = lc.get("type")
        if kind == "point":
            model.lights.append(point_light(tuple(lc.get("position", (0.0, 0.0, 0.0))), color, float(lc["intensity"])))
        elif kind == "directional":
            d = np.asarray(lc.get("direction", (0.0, -1.0, 0.0)), np.float32)
            d = d / np.float32(np.sqrt(np.float32((d * d).sum())))
            model.lights.append(directional_light(tuple(d), color, float(lc["intensity"])))
        elif kind == "area":
            model.lights.append(area_light(int(lc.get("triangle_index", 0)), color, float(lc["intensity"])))
        else:
            warnings.warn(f"unknown light kind {kind!r}")
    for ov in desc.get("materials", []):
        if "index" in ov:
            i = int(ov["index"])
            if i < len(model.materials):
                _apply_override(model.materials[i], ov)
            else:
                warnings.warn(f"material override index {i} out of range ({len(model.materials)} materials)")
        else:
            for m in model.materials:
                _apply_override(m, ov)
