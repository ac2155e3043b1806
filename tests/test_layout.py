"""Layout pins: the sizes and offsets the reference's own tests assert.

  * rustracer-renderer/tests/gpu_layout.rs:10-41 — Rust size_of == WGSL span for Light (64),
    Material (64), Triangle (128), BVHNode (48), Camera (96), Photon (64);
  * rustracer-core/src/material.rs:186-221 — MaterialGpu is 64 bytes, 4-aligned, with roughness at 28,
    metallic 32, kind 40, flags 44, tex_albedo 48, tex_emissive 56, tex_normal 60; TEX_NONE = u32::MAX.
The same layouts are checked at compile time by rustracer_gb300/csrc/rt_layout_check.h.
"""
import ctypes as C
import struct

import numpy as np

from rustracer_gb300 import _abi as A


def test_shared_struct_sizes_match_wgsl():
    expected = {A.Light: 64, A.Material: 64, A.Triangle: 128, A.BVHNode: 48, A.CameraUniform: 96, A.Photon: 64}
    for t, size in expected.items():
        assert C.sizeof(t) == size, t.__name__


def test_uniform_sizes():
    assert C.sizeof(A.ImageParams) == 80
    assert C.sizeof(A.GridParams) == 48
    assert C.sizeof(A.DenoiseParams) == 32
    assert C.sizeof(A.CompositeParams) == 16
    assert C.sizeof(A.TonemapParams) == 32
    assert A.ImageParams._pad.offset == 68  # debug_view slot (lib.rs:345)
    assert A.ImageParams.point_light_emission.offset == 56
    assert A.TonemapParams.marker.offset == 16


def test_material_layout_is_64_bytes_align_4():
    assert C.sizeof(A.Material) == 64
    assert C.alignment(A.Material) == 4


def test_material_offsets_match_wgsl():
    m = A.Material()
    m.albedo[:] = (1.0, 1.0, 1.0, 1.0)
    m.emissive[:] = (2.0, 2.0, 2.0)
    m.roughness, m.metallic, m.ior = 3.0, 4.0, 5.0
    m.kind, m.flags, m.tex_albedo, m.tex_mr, m.tex_emissive, m.tex_normal = 6, 7, 8, 9, 10, 11
    b = bytes(m)
    assert struct.unpack_from("<f", b, 28)[0] == 3.0
    assert struct.unpack_from("<f", b, 32)[0] == 4.0
    assert struct.unpack_from("<I", b, 40)[0] == 6
    assert struct.unpack_from("<I", b, 44)[0] == 7
    assert struct.unpack_from("<I", b, 48)[0] == 8
    assert struct.unpack_from("<I", b, 56)[0] == 10
    assert struct.unpack_from("<I", b, 60)[0] == 11


def test_texture_none_is_max_u32():
    assert A.TEX_NONE == 0xFFFFFFFF == np.iinfo(np.uint32).max


def test_light_tail_alignment():
    # WGSL aligns Light's trailing vec3 pad to 16: kind at 32, pad at 48 (scene.rs:128-140)
    assert A.Light.kind.offset == 32
    assert A.Light._pad_b.offset == 48


def test_oracle_layouts_agree(orc):
    for mine, theirs in [(A.CameraUniform, orc.CameraUniform), (A.ImageParams, orc.ImageParams),
                         (A.GridParams, orc.GridParams), (A.DenoiseParams, orc.DenoiseParams),
                         (A.CompositeParams, orc.CompositeParams), (A.TonemapParams, orc.TonemapParams)]:
        assert C.sizeof(mine) == C.sizeof(theirs)
        assert [f[0] for f in mine._fields_] == [f[0] for f in theirs._fields_]
        for (name, _), (name2, _) in zip(mine._fields_, theirs._fields_):
            assert getattr(mine, name).offset == getattr(theirs, name2).offset
    assert orc.PHOTON_DTYPE.itemsize == C.sizeof(A.Photon)
    for mine, theirs in [(A.SceneDesc, orc.SceneDesc), (A.Camera, orc.Camera), (A.TextureArray, orc.TextureArray)]:
        assert C.sizeof(mine) == C.sizeof(theirs)
        for (name, _), (name2, _) in zip(mine._fields_, theirs._fields_):
            assert name == name2 and getattr(mine, name).offset == getattr(theirs, name2).offset
    assert orc.BVH_NODE_DTYPE.itemsize == C.sizeof(A.BVHNode)


def test_backend_struct_sizes_match_the_header():
    """The ctypes mirrors of the backend-only structs (static_assert'ed in rt_layout_check.h)."""
    assert C.sizeof(A.RenderConfigC) == 96
    assert C.sizeof(A.Camera) == 52
    assert C.sizeof(A.WavefrontTuning) == 32
    assert C.sizeof(A.ServerConfig) == 64
    assert C.sizeof(A.Request) == 164
    assert A.Request.config.offset == 16 and A.Request.camera.offset == 112
    assert C.sizeof(A.JobStatus) == 48
    assert C.sizeof(A.ServerStats) == 128
    assert C.sizeof(A.TraceProfile) == 120 and A.TraceProfile.record_bytes.offset == 112


def test_traversal_width_setting():
    """rt_set_traversal_width takes 2 or 4 and nothing else (no device needed)."""
    lib = A.load()
    assert lib.rt_get_traversal_width() == 4
    assert lib.rt_set_traversal_width(8) == A.RT_ERR_INVALID_ARGUMENT
    assert b"width must be 2 or 4" in lib.rt_last_error()
    assert lib.rt_set_traversal_width(2) == 0 and lib.rt_get_traversal_width() == 2
    assert lib.rt_set_traversal_width(4) == 0 and lib.rt_get_traversal_width() == 4
