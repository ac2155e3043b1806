"""The oracle's own scenes and BVH build against the CUDA backend's host side (CPU, byte for byte).

The oracle generates the two seeded workloads (the 555-unit Cornell box, the displaced-icosphere
room) and indexes any scene with its own restatement of the reference's binned-SAH builder
(rustracer-core/src/bvh.rs:120-336).  The parity tests render the oracle's scene on the CPU and the
backend's on the GPU, so these checks are what makes them the same input; and the BVH comparison
pins the backend's builder to an independently built tree, not only to invariants.
"""
import ctypes as C

import numpy as np
import pytest

import rustracer_gb300 as rt
from test_bvh import build as product_build


def product_bytes(scene: rt.Scene) -> dict:
    a = scene.arrays()
    d = scene.describe()
    out = {k: a[k].view(np.uint8).reshape(len(a[k]), -1) for k in ("triangles", "materials", "lights")}
    out["bvh_nodes"] = a["bvh_nodes"].view(np.uint8)
    out["bvh_prims"] = a["bvh_prims"]
    for name in ("tex_albedo", "tex_mr", "tex_emissive", "tex_normal"):
        t = getattr(d, name)
        n = t.width * t.height * t.layers * 4
        out[name] = (np.ctypeslib.as_array(C.cast(t.rgba8, C.POINTER(C.c_uint8)), shape=(n,)).copy()
                     if t.layers else np.zeros(0, np.uint8))
    out["bounds"] = (np.array(d.bounds_min, np.float32), np.array(d.bounds_max, np.float32), int(d.has_bounds))
    return out


def assert_same_scene(p: dict, o: dict) -> None:
    for k in ("triangles", "materials", "lights", "tex_albedo", "tex_mr", "tex_emissive", "tex_normal"):
        assert p[k].shape == o[k].shape, k
        assert np.array_equal(p[k], o[k]), k
    assert np.array_equal(p["bvh_nodes"], o["bvh_nodes"].view(np.uint8)), "BVH nodes differ"
    assert np.array_equal(p["bvh_prims"], o["bvh_prims"]), "BVH prim order differs"
    assert np.array_equal(p["bounds"][0], o["bounds"][0]) and np.array_equal(p["bounds"][1], o["bounds"][1])
    assert p["bounds"][2] == o["bounds"][2]


def test_cornell_scene_is_the_backends(orc):
    assert_same_scene(product_bytes(rt.Scene.cornell555()), orc.OracleScene.cornell555().arrays())


@pytest.mark.parametrize("level,seed,sigma,tex", [(3, 7, 0.02, 64), (5, 11, 0.05, 8), (6, 0, 0.02, 128)])
def test_icosphere_scene_is_the_backends(orc, level, seed, sigma, tex):
    p = product_bytes(rt.Scene.icosphere_room(level=level, seed=seed, sigma=sigma, tex_size=tex))
    assert_same_scene(p, orc.OracleScene.icosphere_room(level, seed, sigma, tex).arrays())


def test_default_cameras_agree(orc):
    for ps, os_ in ((rt.Scene.cornell555(), orc.OracleScene.cornell555()),
                    (rt.Scene.icosphere_room(level=2, seed=1, tex_size=0), orc.OracleScene.icosphere_room(2, 1, 0.02, 0))):
        c, oc = ps.default_camera(), os_.camera()
        assert tuple(np.float32(c.position)) == tuple(np.float32(oc.position))
        assert tuple(np.float32(c.look_at)) == tuple(np.float32(oc.look_at))
        assert np.float32(c.fov_degrees) == np.float32(oc.fov_degrees)
        assert np.float32(c.focus_dist) == np.float32(oc.focus_dist)


def test_bvh_of_flattened_arrays_is_the_backends(orc):
    """A scene handed over as flattened arrays (the way tests pass glTF or hand-built scenes) gets the
    same tree from the oracle's builder as from the backend's."""
    s = rt.Scene.icosphere_room(level=4, seed=2, sigma=0.03, tex_size=0)
    a = s.arrays()
    o = orc.OracleScene.from_arrays(a["triangles"], a["materials"], a["lights"]).arrays()
    assert np.array_equal(a["bvh_nodes"].view(np.uint8), o["bvh_nodes"].view(np.uint8))
    assert np.array_equal(a["bvh_prims"], o["bvh_prims"])


@pytest.mark.parametrize("n,seed,clustered", [(1, 0, False), (12, 1, False), (513, 1234, False), (4000, 5, False),
                                             (3000, 6, True)])
def test_raw_builds_agree(orc, n, seed, clustered):
    """Random primitive boxes, and boxes with many coincident centroids (the partition's tie rule)."""
    rng = np.random.default_rng(seed)
    c = rng.uniform(-10, 10, (n, 3)).astype(np.float32)
    if clustered:
        c = np.round(c / 4).astype(np.float32) * np.float32(4)
    ext = rng.uniform(0.01, 1.0, (n, 3)).astype(np.float32)
    lo, hi = c - ext, c + ext
    nodes_p, prims_p = product_build(c, lo, hi)
    nodes_o, prims_o = orc.bvh_build(c, lo, hi)
    assert np.array_equal(nodes_p.view(np.uint8), nodes_o.view(np.uint8))
    assert np.array_equal(prims_p, prims_o)
