"""glTF ingest and scene.toml overrides (CPU only: the scene model and BVH are host code).

The first group restates the reference's own unit tests of rustracer-core/src/loader.rs:651-760 and
config.rs:166-231 against this module; the rest load synthetic glTF / GLB files written here.
"""
import base64
import json
import struct

import numpy as np
import pytest

from rustracer_gb300 import _abi as A
from rustracer_gb300 import gltf
from rustracer_gb300.headless import write_png


def tex(w, h, color):
    return gltf.Texture(w, h, np.tile(np.asarray(color, np.float32), (h, w, 1)))


# ---- the reference's loader / config unit tests -----------------------------------------------------
def test_srgb_decode_matches_gltf_spec():
    assert abs(float(gltf.srgb_to_linear(0.0)) - 0.0) < 1e-6
    assert abs(float(gltf.srgb_to_linear(0.04045)) - 0.0031308) < 1e-4
    assert abs(float(gltf.srgb_to_linear(1.0)) - 1.0) < 1e-6
    assert abs(float(gltf.srgb_to_linear(0.5)) - 0.21404114) < 1e-5


def test_build_role_compacts_dedups_and_decodes_srgb():
    master = [tex(2, 2, [0.5, 0.5, 0.5, 1.0]), tex(2, 2, [1.0, 1.0, 1.0, 1.0])]
    role, mapping = gltf.build_role(master, [0, 1, 0], True)
    assert len(role) == 2
    assert abs(float(role[0].data[0, 0, 0]) - 0.21404114) < 1e-5
    assert mapping[0] == 0 and mapping[1] == 1


def test_build_role_drops_mixed_sizes():
    master = [tex(2, 2, [0.5, 0.5, 0.5, 1.0]), tex(4, 4, [0.5, 0.5, 0.5, 1.0])]
    with pytest.warns(UserWarning):
        role, mapping = gltf.build_role(master, [0, 1], False)
    assert len(role) == 1 and mapping[0] == 0 and mapping[1] is None


def test_build_role_scaled_bakes_normal_scale():
    master = [tex(2, 2, [1.0, 0.5, 0.0, 1.0])]
    role, mapping = gltf.build_role(master, [0], False, scales=[2.0])
    assert mapping[0] == 0
    px = role[0].data[0, 0]
    assert abs(px[0] - 2.0) < 1e-6 and abs(px[1] - 1.0) < 1e-6 and abs(px[2]) < 1e-6 and px[3] == 1.0


def test_triangle_emits_samples_the_emissive_texture():
    bright = gltf.Texture(2, 2, np.array([[[1.0, 0.5, 0.2, 1.0], [0, 0, 0, 1]], [[0, 0, 0, 1], [0, 0, 0, 1]]], np.float32))
    mat = gltf.Mat(emissive=(1.0, 1.0, 1.0), emissive_texture=0)
    mesh = gltf.MeshData(np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.float32), np.tile([0, 0, 1.0], (3, 1)),
                         np.zeros((3, 2), np.float32), np.array([0, 1, 2], np.uint32), 0)
    assert gltf.triangle_emits(mesh, 0, mat, [bright])
    dark = gltf.Texture(2, 2, np.zeros((2, 2, 4), np.float32))
    assert not gltf.triangle_emits(mesh, 0, mat, [dark])


def test_environment_override_replaces_the_default_light():
    m = gltf.Model()
    m.lights.append(gltf.environment_light((0, 0, 0), (0, 0, 0), 1.0))
    gltf.apply_descriptor(m, gltf.parse_descriptor(
        '[environment]\nintensity = 2.0\nsky_zenith = [0.1, 0.2, 0.3]\nsky_horizon = [0.7, 0.8, 0.9]\n'))
    assert len(m.lights) == 1
    l = m.lights[0]
    assert l.kind == A.LIGHT_ENVIRONMENT and l.intensity == 2.0
    assert np.allclose(tuple(l.color), (0.1, 0.2, 0.3)) and np.allclose(tuple(l.data)[:3], (0.7, 0.8, 0.9))


def test_material_kind_sets_defaults_and_explicit_values_win():
    m = gltf.Model()
    m.materials.append(gltf.Mat(kind=A.MAT_LAMBERTIAN, albedo=(0.5, 0.5, 0.5), roughness=1.0))
    gltf.apply_descriptor(m, gltf.parse_descriptor('[[materials]]\nindex = 0\nkind = "dielectric"\nior = 1.3\n'))
    mat = m.materials[0]
    assert mat.kind == A.MAT_DIELECTRIC and mat.ior == 1.3 and mat.metallic == 0.0 and mat.roughness == 0.0


# ---- synthetic files ---------------------------------------------------------------------------------
def png_bytes(tmp_path, img):
    p = tmp_path / "t.png"
    write_png(p, img)
    return p.read_bytes()


def build_gltf(tmp_path, binary=False, embed=False):
    """A strip quad under a translated parent, a mirrored copy (scale x = -1), a fan, an emissive
    triangle and a MASK material with a PNG base colour."""
    quad = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [1, 1, 0]], np.float32)
    uv = np.array([[0, 0], [1, 0], [0, 1], [1, 1]], np.float32)
    strip = np.array([0, 1, 2, 3], np.uint16)
    fan_pos = np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0]], np.float32)
    tri = np.array([[0, 2, 0], [1, 2, 0], [0, 2, 1]], np.float32)
    blobs = [quad.tobytes(), uv.tobytes(), strip.tobytes() + b"\0\0" * 0, fan_pos.tobytes(), tri.tobytes()]
    offsets, buf = [], b""
    for b in blobs:
        while len(buf) % 4:
            buf += b"\0"
        offsets.append(len(buf))
        buf += b
    views = [{"buffer": 0, "byteOffset": o, "byteLength": len(b)} for o, b in zip(offsets, blobs)]
    acc = [
        {"bufferView": 0, "componentType": 5126, "count": 4, "type": "VEC3"},
        {"bufferView": 1, "componentType": 5126, "count": 4, "type": "VEC2"},
        {"bufferView": 2, "componentType": 5123, "count": 4, "type": "SCALAR"},
        {"bufferView": 3, "componentType": 5126, "count": 4, "type": "VEC3"},
        {"bufferView": 4, "componentType": 5126, "count": 3, "type": "VEC3"},
    ]
    img = np.zeros((4, 4, 4), np.uint8)
    img[..., 0] = 255
    img[..., 3] = 255
    img[0, 0, 3] = 0
    png = png_bytes(tmp_path, img)
    doc = {
        "asset": {"version": "2.0"},
        "scene": 0,
        "scenes": [{"nodes": [0, 2]}],
        "nodes": [
            {"translation": [0, 0, 5], "children": [1], "mesh": 0},
            {"scale": [-1, 1, 1], "mesh": 0},
            {"matrix": [1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 10, 0, 0, 1], "mesh": 1},
        ],
        "meshes": [
            {"primitives": [{"attributes": {"POSITION": 0, "TEXCOORD_0": 1}, "indices": 2, "mode": 5, "material": 0}]},
            {"primitives": [{"attributes": {"POSITION": 3}, "mode": 6, "material": 1},
                            {"attributes": {"POSITION": 4}, "material": 2}]},
        ],
        "materials": [
            {"pbrMetallicRoughness": {"baseColorFactor": [1, 1, 1, 1], "baseColorTexture": {"index": 0},
                                      "metallicFactor": 0.0, "roughnessFactor": 0.7}, "alphaMode": "MASK"},
            {"pbrMetallicRoughness": {"baseColorFactor": [0.2, 0.4, 0.6, 1], "metallicFactor": 1.0,
                                      "roughnessFactor": 0.3}},
            {"emissiveFactor": [4.0, 3.0, 2.0]},
        ],
        "textures": [{"source": 0}],
        "bufferViews": views,
        "accessors": acc,
    }
    if binary:
        doc["buffers"] = [{"byteLength": len(buf)}]
        img_off = len(buf) + (-len(buf)) % 4
        buf = buf + b"\0" * ((-len(buf)) % 4) + png
        doc["images"] = [{"bufferView": len(views), "mimeType": "image/png"}]
        doc["bufferViews"].append({"buffer": 0, "byteOffset": img_off, "byteLength": len(png)})
        doc["buffers"][0]["byteLength"] = len(buf)
        js = json.dumps(doc).encode()
        js += b" " * ((-len(js)) % 4)
        buf += b"\0" * ((-len(buf)) % 4)
        glb = struct.pack("<4sII", b"glTF", 2, 12 + 8 + len(js) + 8 + len(buf)) + \
            struct.pack("<I4s", len(js), b"JSON") + js + struct.pack("<I4s", len(buf), b"BIN\0") + buf
        path = tmp_path / "scene.glb"
        path.write_bytes(glb)
        return path
    if embed:
        doc["buffers"] = [{"byteLength": len(buf), "uri": "data:application/octet-stream;base64," +
                           base64.b64encode(buf).decode()}]
        doc["images"] = [{"uri": "data:image/png;base64," + base64.b64encode(png).decode()}]
    else:
        (tmp_path / "scene.bin").write_bytes(buf)
        (tmp_path / "albedo.png").write_bytes(png)
        doc["buffers"] = [{"byteLength": len(buf), "uri": "scene.bin"}]
        doc["images"] = [{"uri": "albedo.png"}]
    path = tmp_path / "scene.gltf"
    path.write_text(json.dumps(doc))
    return path


@pytest.mark.parametrize("kind", ["separate", "embedded", "glb"])
def test_synthetic_gltf(tmp_path, kind):
    path = build_gltf(tmp_path, binary=kind == "glb", embed=kind == "embedded")
    m = gltf.load_gltf_model(path)
    # node order: parent quad, its mirrored child, then the fan and the triangle of node 2
    assert [len(x.indices) // 3 for x in m.meshes] == [2, 2, 2, 1]
    parent, child, fan, tri = m.meshes
    assert np.allclose(parent.positions, [[0, 0, 5], [1, 0, 5], [0, 1, 5], [1, 1, 5]])
    assert np.allclose(child.positions[:, 0], [0, -1, 0, -1]) and np.allclose(child.positions[:, 2], 5)
    # strip: (0 1 2), (1 3 2); the mirrored copy flips the winding
    assert parent.indices.tolist() == [0, 1, 2, 1, 3, 2]
    assert child.indices.tolist() == [0, 2, 1, 1, 2, 3]
    # computed smooth normals, transformed: +z for the quad, still +z under the x mirror
    assert np.allclose(parent.normals, [0, 0, 1]) and np.allclose(child.normals, [0, 0, 1])
    assert fan.indices.tolist() == [0, 1, 2, 0, 2, 3] and np.allclose(fan.positions[:, 0], [10, 11, 11, 10])
    # materials: MASK cut-out with the sRGB-decoded albedo texture, the metal factors, the emitter
    m0, m1, m2 = m.materials
    assert m0.alpha_cutout and m0.albedo_texture == 0 and abs(m0.roughness - 0.7) < 1e-6
    assert m1.metallic == 1.0 and abs(m1.roughness - 0.3) < 1e-6 and m1.albedo_texture is None
    assert np.allclose(m2.emissive, (4, 3, 2)) and m2.roughness == 1.0 and m2.metallic == 1.0
    assert len(m.tex_albedo) == 1 and m.tex_albedo[0].data.shape == (4, 4, 4)
    assert abs(float(m.tex_albedo[0].data[1, 1, 0]) - 1.0) < 1e-6 and float(m.tex_albedo[0].data[0, 0, 3]) == 0.0
    # one area light for the emissive triangle (global triangle index 6), then the default sky
    assert [l.kind for l in m.lights] == [A.LIGHT_AREA, A.LIGHT_ENVIRONMENT]
    assert int(m.lights[0].data[0]) == 6
    s = m.to_scene()
    assert s.triangle_count() == 7
    d = s.describe()
    assert d.tex_albedo.layers == 1 and d.material_count == 3 and d.light_count == 2


def test_scene_toml_next_to_the_file_is_applied(tmp_path):
    path = build_gltf(tmp_path)
    (tmp_path / "scene.toml").write_text(
        '[environment]\nintensity = 0.5\n\n[[lights]]\ntype = "point"\nposition = [0, 3, 0]\nintensity = 7\n\n'
        '[[materials]]\nindex = 1\nkind = "metal"\nalbedo = [0.9, 0.1, 0.1]\n')
    s = gltf.load_gltf(path)
    d = s.describe()
    lights = np.ctypeslib.as_array(d.lights, shape=(d.light_count,))
    kinds = [int(l["kind"]) for l in lights]
    assert kinds == [A.LIGHT_AREA, A.LIGHT_ENVIRONMENT, A.LIGHT_POINT]
    mats = np.ctypeslib.as_array(d.materials, shape=(d.material_count,))
    assert int(mats[1]["kind"]) == A.MAT_METAL and np.allclose(mats[1]["albedo"][:3], (0.9, 0.1, 0.1))


def test_png_decoder_filters_and_formats():
    import zlib

    rng = np.random.default_rng(1)
    img = rng.integers(0, 256, (5, 6, 3), dtype=np.uint8)
    # encode with each filter type by hand (RGB, 8 bit)
    def enc(img, ftype):
        h, w, c = img.shape
        raw = b""
        prev = np.zeros(w * c, np.int32)
        for y in range(h):
            line = img[y].reshape(-1).astype(np.int32)
            left = np.concatenate([np.zeros(c, np.int32), line[:-c]])
            upleft = np.concatenate([np.zeros(c, np.int32), prev[:-c]])
            if ftype == 0:
                f = line
            elif ftype == 1:
                f = line - left
            elif ftype == 2:
                f = line - prev
            elif ftype == 3:
                f = line - (left + prev) // 2
            else:
                p = left + prev - upleft
                pa, pb, pc = abs(p - left), abs(p - prev), abs(p - upleft)
                f = line - np.where((pa <= pb) & (pa <= pc), left, np.where(pb <= pc, prev, upleft))
            raw += bytes([ftype]) + (f & 255).astype(np.uint8).tobytes()
            prev = line
        def chunk(tag, data):
            return struct.pack(">I", len(data)) + tag + data + struct.pack(">I", zlib.crc32(tag + data) & 0xFFFFFFFF)
        return b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, 8, 2, 0, 0, 0)) + \
            chunk(b"IDAT", zlib.compress(raw)) + chunk(b"IEND", b"")
    for ftype in range(5):
        t = gltf.decode_png(enc(img, ftype))
        assert t is not None and (t.width, t.height) == (6, 5)
        assert np.array_equal(np.round(t.data[..., :3] * 255).astype(np.uint8), img), ftype
        assert (t.data[..., 3] == 1.0).all()
    assert gltf.decode_png(b"\xff\xd8\xff\xe0 not a png") is None
