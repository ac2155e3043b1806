"""The GPU linear-BVH builder: the reference's BVH invariants (rustracer-core/src/bvh.rs:342-459) on
its trees, and renders through it against the oracle on the same tree."""
import ctypes as C

import numpy as np
import pytest

import rustracer_gb300 as rt
from rustracer_gb300 import _abi as A

from test_gpu_parity import FRAC, match_frac, render_both

pytestmark = pytest.mark.gpu


def gpu_build(boxes_lo, boxes_hi):
    lib = A.load()
    c = np.ascontiguousarray((boxes_lo + boxes_hi) * np.float32(0.5), np.float32)
    lo, hi = np.ascontiguousarray(boxes_lo, np.float32), np.ascontiguousarray(boxes_hi, np.float32)
    h, depth = C.c_void_p(), C.c_uint32()
    f = lambda a: a.ctypes.data_as(C.POINTER(C.c_float))  # noqa: E731
    A.check("rt_bvh_build_gpu", lib.rt_bvh_build_gpu(f(c), f(lo), f(hi), len(c), C.byref(h), C.byref(depth)))
    nn, npr = C.c_uint64(), C.c_uint64()
    nodes = np.ctypeslib.as_array(lib.rt_bvh_nodes(h, C.byref(nn)), shape=(nn.value,)).copy()
    prims = np.ctypeslib.as_array(lib.rt_bvh_prims(h, C.byref(npr)), shape=(npr.value,)).copy()
    lib.rt_bvh_destroy(h)
    return nodes, prims, depth.value


@pytest.mark.parametrize("n", [2, 3, 1000, 70001])
def test_lbvh_invariants(gpu, n):
    rng = np.random.default_rng(n)
    lo = rng.uniform(-10, 10, (n, 3)).astype(np.float32)
    hi = lo + rng.uniform(0, 0.5, (n, 3)).astype(np.float32)
    lo[: n // 10] = lo[0]  # duplicate centroids: equal Morton codes must still give a tree
    hi[: n // 10] = hi[0]
    nodes, prims, depth = gpu_build(lo, hi)
    assert len(nodes) <= 2 * n - 1 and sorted(prims.tolist()) == list(range(n))
    seen = np.zeros(n, np.int64)
    under = {}  # primitives below each node

    def walk(i, d):
        nd = nodes[i]
        bmin, bmax = np.asarray(nd["bbox_min"]), np.asarray(nd["bbox_max"])
        if nd["prim_count"] > 0:
            assert 1 <= nd["prim_count"] <= 4  # the reference's leaf size limit
            for k in range(nd["left_first"], nd["left_first"] + nd["prim_count"]):
                p = prims[k]
                seen[p] += 1
                assert (bmin <= lo[p]).all() and (bmax >= hi[p]).all()
            under[i] = int(nd["prim_count"])
            return d
        deepest = d
        for ch in (nd["left_first"], nd["right_child"]):
            cmin, cmax = np.asarray(nodes[ch]["bbox_min"]), np.asarray(nodes[ch]["bbox_max"])
            assert (bmin <= cmin).all() and (bmax >= cmax).all()
            stack.append((ch, d + 1))
        return deepest

    stack, max_d = [(0, 0)], 0
    order = []
    while stack:
        i, d = stack.pop()
        order.append(i)
        max_d = max(max_d, walk(i, d))
    for i in reversed(order):  # children were visited after their parents
        nd = nodes[i]
        if nd["prim_count"] == 0:
            under[i] = under[int(nd["left_first"])] + under[int(nd["right_child"])]
            assert under[i] > 4  # a subtree of at most four primitives is one leaf
    assert (seen == 1).all()
    assert depth == max_d


def test_render_with_gpu_built_tree_matches_the_oracle(gpu, orc):
    scene = rt.Scene.icosphere_room(level=4, seed=2, sigma=0.02, tex_size=32)
    scene.set_bvh_builder(A.BVH_GPU_LBVH)
    cfg = rt.RenderConfig(width=64, height=48, spp=2, accumulate_frames=3, enable_denoise=False)
    r, o = render_both(orc, scene, cfg, 3)
    assert scene.bvh_builder_used() == A.BVH_GPU_LBVH
    assert match_frac(r.read_accumulation(), o.accum) >= FRAC


def test_gpu_and_host_trees_render_the_same_image(gpu):
    imgs = []
    for builder in (A.BVH_HOST_SAH, A.BVH_GPU_LBVH):
        scene = rt.Scene.icosphere_room(level=5, seed=4, sigma=0.02, tex_size=32)
        scene.set_bvh_builder(builder)
        cfg = rt.RenderConfig(width=80, height=60, spp=2, accumulate_frames=2, enable_denoise=False)
        r = rt.Renderer(scene, cfg)
        r.update_camera(scene.default_camera())
        r.render_frames(2)
        imgs.append(r.read_accumulation())
        assert scene.bvh_builder_used() == builder
    # the same closest hits except where two triangles lie at exactly the same distance
    assert match_frac(imgs[1], imgs[0]) >= FRAC


@pytest.fixture
def width2():
    """Scenes uploaded inside the test keep only the two-wide records."""
    rt.set_traversal_width(2)
    yield
    rt.set_traversal_width(4)


def test_two_wide_walk_matches_the_oracle(gpu, orc, width2):
    scene = rt.Scene.icosphere_room(level=4, seed=3, sigma=0.02, tex_size=32)
    cfg = rt.RenderConfig(width=64, height=48, spp=2, accumulate_frames=3, enable_denoise=False)
    r, o = render_both(orc, scene, cfg, 3)
    assert match_frac(r.read_accumulation(), o.accum) >= FRAC


def test_four_and_two_wide_walks_render_the_same_image(gpu):
    imgs, sizes = [], []
    for width in (4, 2):
        rt.set_traversal_width(width)
        try:
            scene = rt.Scene.icosphere_room(level=5, seed=6, sigma=0.02, tex_size=32)
            res = rt.ResidentScene(scene)
            sizes.append(res.device_bytes())
            cfg = rt.RenderConfig(width=80, height=60, spp=2, accumulate_frames=2, enable_denoise=False,
                                  enable_photon_map=True, photon_count=4096)
            r = rt.Renderer(res, cfg)
            r.update_camera(scene.default_camera())
            r.rebuild_photons()
            r.render_frames(2)
            imgs.append(r.read_accumulation())
            r.close()
            res.close()
        finally:
            rt.set_traversal_width(4)
    assert sizes[0] > sizes[1]  # the four-wide records ride along with the two-wide ones
    # the same closest hits except where two triangles lie at exactly the same distance
    assert match_frac(imgs[0], imgs[1]) >= FRAC

