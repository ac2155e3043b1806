"""BVH builder and traversal.

The first five tests restate the reference's BVH unit tests (rustracer-core/src/bvh.rs:342-459):
empty, single primitive, a 4x3 grid of 12 boxes, all of 513 random primitives reachable exactly once
(the reference seeds Rust's StdRng with 1234; numpy's generator with the same seed stands in), and 16
coincident centroids collapsing to one leaf.  The rest check the builder's invariants on real
scenes and the oracle's closest-hit traversal against brute force.
"""
import ctypes as C

import numpy as np
import pytest

import rustracer_gb300 as rt
from rustracer_gb300 import _abi as A


def build(centroids, bmin, bmax):
    lib = A.load()
    c, lo, hi = (np.ascontiguousarray(x, np.float32).reshape(-1, 3) for x in (centroids, bmin, bmax))
    h = C.c_void_p()
    A.check("rt_bvh_build", lib.rt_bvh_build(A.ptr(c), A.ptr(lo), A.ptr(hi), len(c), C.byref(h)))
    n = C.c_uint64()
    p = lib.rt_bvh_nodes(h, C.byref(n))
    nodes = np.ctypeslib.as_array(C.cast(p, C.POINTER(C.c_uint8)), shape=(n.value * 48,)).view(
        A.np_dtype(A.BVHNode)).copy() if n.value else np.zeros(0, A.np_dtype(A.BVHNode))
    m = C.c_uint64()
    q = lib.rt_bvh_prims(h, C.byref(m))
    prims = np.ctypeslib.as_array(q, shape=(m.value,)).copy() if m.value else np.zeros(0, np.uint32)
    lib.rt_bvh_destroy(h)
    return nodes, prims


def collect_prims(nodes, prims):
    out, stack = [], [0]
    while stack:
        i = stack.pop()
        assert i < len(nodes), f"child index out of range: {i}"
        nd = nodes[i]
        if nd["prim_count"] > 0:
            out.extend(prims[nd["left_first"]: nd["left_first"] + nd["prim_count"]].tolist())
        else:
            stack.append(int(nd["right_child"]))
            stack.append(int(nd["left_first"]))
    return out


def test_bvh_build_empty(lib):
    nodes, prims = build(np.zeros((0, 3)), np.zeros((0, 3)), np.zeros((0, 3)))
    assert len(nodes) == 0


def test_bvh_build_single(lib):
    nodes, _ = build([[0, 0, 0]], [[-0.5] * 3], [[0.5] * 3])
    assert len(nodes) == 1 and nodes[0]["prim_count"] > 0


def test_bvh_build_many(lib):
    c, lo, hi = [], [], []
    for i in range(12):
        x, y = float(i % 4), float(i // 4)
        c.append([x, y, 0.0])
        lo.append([x - 0.1, y - 0.1, -0.1])
        hi.append([x + 0.1, y + 0.1, 0.1])
    nodes, _ = build(c, lo, hi)
    assert len(nodes) > 1
    assert nodes[0]["prim_count"] == 0
    assert nodes[0]["left_first"] < len(nodes) and nodes[0]["right_child"] < len(nodes)


def test_bvh_sah_enumerates_all_primitives_once(lib):
    n = 513
    rng = np.random.default_rng(1234)
    c = rng.uniform(-10, 10, (n, 3)).astype(np.float32)
    nodes, prims = build(c, c - np.float32(0.05), c + np.float32(0.05))
    assert sorted(collect_prims(nodes, prims)) == list(range(n))


def test_bvh_sah_coincident_centroids_still_terminates(lib):
    n = 16
    nodes, _ = build(np.zeros((n, 3)), np.full((n, 3), -0.5), np.full((n, 3), 0.5))
    assert len(nodes) == 1 and nodes[0]["prim_count"] == n


def check_invariants(scene):
    a = scene.arrays()
    nodes, prims, tris = a["bvh_nodes"], a["bvh_prims"], a["triangles"]
    assert sorted(collect_prims(nodes, prims)) == list(range(len(tris)))
    mn, mx = nodes["bbox_min"], nodes["bbox_max"]
    internal = np.nonzero(nodes["prim_count"] == 0)[0]
    for ch in ("left_first", "right_child"):
        k = nodes[ch][internal]
        assert (k < len(nodes)).all()
        assert (mn[k] >= mn[internal]).all() and (mx[k] <= mx[internal]).all()
    leaves = np.nonzero(nodes["prim_count"] > 0)[0]
    for li in leaves[:: max(1, len(leaves) // 500)]:
        nd = nodes[li]
        for p in prims[nd["left_first"]: nd["left_first"] + nd["prim_count"]]:
            v = np.stack([tris[p]["v0"], tris[p]["v1"], tris[p]["v2"]])
            assert (v >= nd["bbox_min"]).all() and (v <= nd["bbox_max"]).all()
    # root first (children are emitted before parents, then the array is reversed)
    assert nodes[0]["prim_count"] == 0 or len(nodes) == 1


def test_invariants_cornell(lib):
    s = rt.Scene.cornell555()
    assert s.describe().triangle_count == 36
    check_invariants(s)


def test_invariants_icosphere(lib):
    s = rt.Scene.icosphere_room(level=3, seed=1, sigma=0.02, tex_size=0)
    assert s.describe().triangle_count == 12 + 2 + 20 * 4 ** 3
    check_invariants(s)


def brute_force(tris, o, d):
    """Moller-Trumbore over every triangle, float32, same operation order as common.wgsl:78-100."""
    f = np.float32
    v0, v1, v2 = tris["v0"].astype(f), tris["v1"].astype(f), tris["v2"].astype(f)
    e1, e2 = v1 - v0, v2 - v0

    def cross(a, b):
        return np.stack([a[..., 1] * b[..., 2] - a[..., 2] * b[..., 1], a[..., 2] * b[..., 0] - a[..., 0] * b[..., 2],
                         a[..., 0] * b[..., 1] - a[..., 1] * b[..., 0]], -1)

    def dot(a, b):
        return (a[..., 0] * b[..., 0] + a[..., 1] * b[..., 1]) + a[..., 2] * b[..., 2]

    h = cross(np.broadcast_to(d, e2.shape), e2)
    a = dot(e1, h)
    with np.errstate(all="ignore"):
        inv = f(1.0) / a
        s = o - v0
        u = inv * dot(s, h)
        q = cross(s, e1)
        v = inv * dot(np.broadcast_to(d, q.shape), q)
        t = inv * dot(e2, q)
        ok = (np.abs(a) >= f(1e-7)) & (u >= 0) & (u <= 1) & (v >= 0) & (u + v <= 1) & (t > f(1e-6))
    t = np.where(ok, t, f(1e38))
    i = int(np.argmin(t))
    return t[i], i


def test_oracle_traversal_matches_brute_force(lib, orc):
    s = rt.Scene.icosphere_room(level=2, seed=3, sigma=0.05, tex_size=0)
    tris = s.arrays()["triangles"]
    rng = np.random.default_rng(9)
    n = 400
    o = rng.uniform(-4.5, 4.5, (n, 3)).astype(np.float32)
    d = rng.normal(size=(n, 3)).astype(np.float32)
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    t, prim = orc.trace_rays(s.describe(), o, d)
    for k in range(n):
        tb, ib = brute_force(tris, o[k], d[k])
        assert t[k] == tb
        if t[k] < 1e38:
            assert prim[k] == ib or t[k] == brute_force(tris[[prim[k]]], o[k], d[k])[0]


def test_threaded_build_equals_sequential_build():
    """The host BVH build splits the top of the tree over threads; nodes and prim order are those of
    the sequential build."""
    from rustracer_gb300 import _abi as A
    import rustracer_gb300 as rt

    lib = A.load()
    out = []
    for threads in (1, 0, 3):
        lib.rt_set_host_threads(threads)
        s = rt.Scene.icosphere_room(level=5, seed=11, tex_size=8)
        a = s.arrays()
        out.append((a["bvh_nodes"].tobytes(), a["bvh_prims"].tobytes()))
    lib.rt_set_host_threads(0)
    assert out[0] == out[1] == out[2]
    assert len(out[0][1]) // 4 >= 20 * 4 ** 5  # large enough for threaded subtrees (8192 prims each)


def wide_layout(nodes):
    lib = A.load()
    buf = np.ascontiguousarray(nodes)
    recs, need = C.c_uint64(), C.c_uint32()
    A.check("rt_bvh_wide_layout", lib.rt_bvh_wide_layout(buf.ctypes.data, len(buf), None, 0, C.byref(recs),
                                                        C.byref(need)))
    out = np.zeros(recs.value * 32, np.float32)
    A.check("rt_bvh_wide_layout", lib.rt_bvh_wide_layout(buf.ctypes.data, len(buf), out.ctypes.data, out.size,
                                                        C.byref(recs), C.byref(need)))
    return out.reshape(-1, 4, 8), need.value


@pytest.mark.parametrize("make", [lambda: rt.Scene.cornell555(),
                                  lambda: rt.Scene.icosphere_room(level=4, seed=5, sigma=0.02, tex_size=0)])
def test_wide_layout_is_the_same_tree(lib, make):
    """The four-wide records hold every leaf of the reference's tree exactly once with its own box,
    every record is reached exactly once, each record's children are the nodes it absorbed, and the
    stack bound is the largest sum of (internal children - 1) along a root-to-leaf walk."""
    nodes = make().arrays()["bvh_nodes"]
    recs, need = wide_layout(nodes)
    u = recs.view(np.uint32)
    leaves = {(int(n["left_first"]), int(n["prim_count"])): n for n in nodes if n["prim_count"] > 0}
    boxes = {tuple(n["bbox_min"]) + tuple(n["bbox_max"]) for n in nodes}
    seen_rec = np.zeros(len(recs), np.int32)
    seen_leaf = {}

    def walk(r):  # the largest stack depth below record r
        seen_rec[r] += 1
        internal, deepest = 0, 0
        for c in range(4):
            ref, cnt = int(u[r, c, 3]), int(u[r, c, 7])
            if cnt == 0xFFFFFFFF:
                continue
            box = tuple(recs[r, c, 0:3]) + tuple(recs[r, c, 4:7])
            assert box in boxes  # every child box is a box of the reference's tree
            if cnt > 0:
                assert (ref, cnt) in leaves
                seen_leaf[(ref, cnt)] = seen_leaf.get((ref, cnt), 0) + 1
            else:
                assert 0 < ref < len(recs)
                internal += 1
                deepest = max(deepest, walk(ref))
        return internal - 1 + deepest if internal else 0

    assert walk(0) == need
    assert (seen_rec == 1).all()
    assert seen_leaf == {k: 1 for k in leaves}
    assert len(recs) < int((nodes["prim_count"] == 0).sum())  # fewer records than two-wide ones
