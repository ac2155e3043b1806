"""Pins of the oracle (CPU): independent restatements, known answers, domain properties and the
golden vectors in tests/golden/ (made by tests/golden/make_golden.py from the oracle).

The reference's own tests pin only layouts and BVH invariants (test_layout.py, test_bvh.py); for the
rest of the path parity is unpinned by the reference, so the checks here are:
  * the PCG hash RNG restated a second time in pure Python integer arithmetic (common.wgsl:29-52);
  * Moller-Trumbore known answers on hand-built rays;
  * composite / tonemap against numpy float32 formulas; denoise of a constant image is the identity;
  * photon-grid invariants against a numpy stable sort;
  * golden vectors: integers bit-exact, floats within 1e-5 relative (libm may differ by an ulp
    between host architectures).
Everything here runs the oracle alone, on the scenes it generates itself.
"""
from pathlib import Path

import numpy as np
import pytest


G = Path(__file__).resolve().parent / "golden"
M32 = 0xFFFFFFFF


def pcg_init(seed):
    s = (seed * 747796405 + 2891336453) & M32
    return (((s >> ((s >> 28) + 4)) ^ s) * 277803737) & M32


def pcg_next(state):
    old = state
    state = (old * 747796405 + 1) & M32
    word = (((old >> ((old >> 28) + 4)) ^ old) * 277803737) & M32
    return state, ((word >> 22) ^ word) & M32


def test_rng_matches_python_restatement(orc):
    for seed in [0, 1, 7, 12345, M32, 2654435761, 1013904223, 0x80000000]:
        st = pcg_init(seed)
        ref = []
        for _ in range(64):
            st, v = pcg_next(st)
            ref.append(v)
        u, f = orc.rng_sequence(seed, 64)
        assert u.tolist() == ref
        assert np.array_equal(f, (u.astype(np.float32) / np.float32(4294967296.0)))


def test_rng_f32_can_reach_one():
    # f32(u32) rounds to nearest: values >= 2^32 - 128 round up to 2^32, so rng_f32 == 1.0 (q1)
    assert np.float32(np.uint32(0xFFFFFFC0)) / np.float32(4294967296.0) == 1.0
    assert np.float32(np.uint32(0xFFFFFF7F)) / np.float32(4294967296.0) < 1.0


def test_unorm8_correction_equals_ieee_division():
    """The texel conversion c / 255 of the CUDA path (rt_device.cuh unorm8): q0 = c * r with r the
    float nearest 1/255, then q0 + (c - 255 q0) * r with both steps fused multiply-adds.  For every
    byte it equals the correctly rounded float32 quotient, which the reference's division gives and
    the oracle computes.  Exact rational arithmetic stands in for the GPU's fma."""
    from fractions import Fraction

    def rnd(x: Fraction) -> np.float32:  # correctly rounded, ties to even
        f = np.float32(float(x))
        best = None
        for c in (np.nextafter(f, np.float32(-np.inf)), f, np.nextafter(f, np.float32(np.inf))):
            d = abs(Fraction(float(c)) - x)
            if best is None or d < best[0] or (d == best[0] and int(np.float32(c).view(np.uint32)) % 2 == 0):
                best = (d, np.float32(c))
        return best[1]

    r = np.float32(float.fromhex("0x1.010102p-8"))
    assert r == rnd(Fraction(1, 255))
    F = lambda v: Fraction(float(v))  # noqa: E731
    for c in range(256):
        a = np.float32(c)
        q0 = rnd(F(a) * F(r))
        e = rnd(F(-q0) * 255 + F(a))
        q = rnd(F(e) * F(r) + F(q0))
        assert q == a / np.float32(255.0) == rnd(Fraction(c, 255)), c


def test_fixed_sincos_error_bound(orc):
    """The sampling angles' sin / cos (one fixed IEEE sequence on both backends) against float64.

    The angles are 2*pi*u with u = rng_f32 in [0, 1] (common.wgsl:60-74, the VNDF disk of
    gather.wgsl:230-256); WGSL itself only asks for 2^-11 absolute error.  The bound here is 2 ulp of
    1.0 (2.4e-7) absolute over every reachable angle of a dense sweep, plus the endpoints."""
    u = np.concatenate([np.linspace(0.0, 1.0, 1 << 20, dtype=np.float32),
                        np.float32([0.0, 0.25, 0.5, 0.75, 1.0, 1e-30, 0.9999999])])
    phi = np.float32(2.0) * np.float32(np.pi) * u
    s, c = orc.sincos(phi)
    x = phi.astype(np.float64)
    assert np.abs(s - np.sin(x)).max() < 2.4e-7
    assert np.abs(c - np.cos(x)).max() < 2.4e-7
    # sin^2 + cos^2 stays 1 within float rounding, and the quadrant signs are right
    assert np.abs(s.astype(np.float64) ** 2 + c.astype(np.float64) ** 2 - 1.0).max() < 5e-7
    assert (np.sign(s[(x > 1e-3) & (x < np.pi - 1e-3)]) > 0).all()
    assert (np.sign(c[(x > np.pi / 2 + 1e-3) & (x < 1.5 * np.pi - 1e-3)]) < 0).all()


def test_pixel_seed_formula(orc):
    # gather.wgsl:262-263: rng_init((y*W + x + frame*2654435761) * 1664525 + 1013904223)
    W = 256
    for x, y, frame in [(0, 0, 1), (17, 3, 1), (255, 255, 16), (3, 200, 70000)]:
        base = (y * W + x + frame * 2654435761) & M32
        seed = (base * 1664525 + 1013904223) & M32
        st, v = pcg_next(pcg_init(seed))
        assert orc.rng_sequence(seed, 1)[0][0] == v


def test_golden_rng(orc):
    d = np.load(G / "rng.npz")
    for seed, seq in zip(d["seeds"], d["u32"]):
        assert np.array_equal(orc.rng_sequence(int(seed), len(seq))[0], seq)


def mt(orc, ro, rd, v0, v1, v2):
    arrs = [np.ascontiguousarray(a, np.float32) for a in (ro, rd, v0, v1, v2)]  # kept alive for the call
    return orc.load().oracle_intersect_triangle(*(orc._p(a) for a in arrs))


def test_moller_trumbore_known_answers(orc):
    v0, v1, v2 = [0, 0, 0], [1, 0, 0], [0, 1, 0]
    assert mt(orc, [0.25, 0.25, 1], [0, 0, -1], v0, v1, v2) == 1.0           # front hit
    assert mt(orc, [0.25, 0.25, -2], [0, 0, 1], v0, v1, v2) == 2.0           # back face hits too
    assert mt(orc, [0.75, 0.75, 1], [0, 0, -1], v0, v1, v2) == np.float32(1e38)  # outside (u+v > 1)
    assert mt(orc, [0.25, 0.25, 1], [1, 0, 0], v0, v1, v2) == np.float32(1e38)   # parallel (|a| < 1e-7)
    assert mt(orc, [0.25, 0.25, -1], [0, 0, -1], v0, v1, v2) == np.float32(1e38)  # behind (t <= 1e-6)
    assert mt(orc, [0.5, 0.5, 1], [0, 0, -1], v0, v1, v2) == 1.0             # on the hypotenuse u+v == 1
    assert mt(orc, [0, 0, 3], [0, 0, -1], v0, v1, v2) == 3.0                 # at a vertex


def test_composite_formula(orc):
    rng = np.random.default_rng(0)
    f = rng.random((5, 7, 4), np.float32)
    a = rng.random((5, 7, 4), np.float32)
    assert np.array_equal(orc.composite(f, a, 1.0), f)  # alpha 1 overwrites
    al = np.float32(1.0) / np.float32(3.0)
    ref = a * (np.float32(1) - al) + f * al
    assert np.array_equal(orc.composite(f, a, float(al)), ref)


def test_tonemap_formula(orc):
    rng = np.random.default_rng(1)
    acc = (rng.random((6, 9, 4), np.float32) * 8).astype(np.float32)
    out = orc.tonemap(acc, 1.0, 2.2)
    e = acc[..., :3]
    mapped = e / (e + np.float32(1))
    col = np.power(mapped, np.float32(1) / np.float32(2.2))
    ref = np.floor(np.clip(col, 0, 1) * 255 + 0.5).astype(int)
    assert np.abs(out[..., :3].astype(int) - ref).max() <= 1
    assert (out[..., 3] == 255).all()


def test_denoise_constant_image_is_identity(orc):
    h, w = 9, 11
    frame = np.zeros((h, w, 4), np.float32)
    frame[..., :3] = [0.3, 0.5, 0.7]
    frame[..., 3] = 1
    g = np.zeros((h, w, 4), np.float32)
    g[..., 1] = 1
    g[..., 3] = 2.0
    m = np.zeros((h, w, 4), np.float32)
    out = orc.denoise(frame, g, m, 1.0, 2)
    assert np.allclose(out, frame, rtol=1e-6, atol=0)


def camera_of(orc, scene, cfg):
    c = scene.camera()
    return orc.camera_uniform(tuple(c.position), tuple(c.look_at), tuple(c.up), c.fov_degrees, cfg.width,
                              cfg.height, c.near_plane, c.aperture, c.focus_dist)


def close(a, b, rtol=1e-5, frac=0.999):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return float((np.abs(a - b) <= rtol * np.abs(b) + 1e-7).mean()) >= frac


def test_golden_cornell_render(orc):
    d = np.load(G / "cornell_32x32.npz")
    sc = orc.OracleScene.cornell555()
    cfg = orc.Config(width=32, height=32, spp=2, accumulate_frames=4, enable_denoise=True)
    o = orc.OracleRenderer(sc, cfg, camera_of(orc, sc, cfg), threads=2)
    for _ in range(4):
        o.record_frame()
    assert close(o.accum, d["accum"]) and close(o.gbuffer, d["gbuffer"]) and close(o.moments, d["moments"])
    assert (np.abs(o.output.astype(int) - d["output"].astype(int)) <= 1).mean() >= 0.999
    assert np.abs(o.counters.astype(np.int64) - d["counters"].astype(np.int64)).max() <= 0.001 * d["counters"].max()


def test_golden_icosphere_render(orc):
    d = np.load(G / "icosphere_24x16.npz")
    sc = orc.OracleScene.icosphere_room(2, 3, 0.02, 16)
    cfg = orc.Config(width=24, height=16, spp=3, accumulate_frames=2, enable_denoise=False, max_bounces=8)
    o = orc.OracleRenderer(sc, cfg, camera_of(orc, sc, cfg), threads=2)
    for _ in range(2):
        o.record_frame()
    assert close(o.accum, d["accum"])


def test_golden_photon_trace(orc):
    d = np.load(G / "photons_cornell_512.npz")
    sc = orc.OracleScene.cornell555()
    cfg = orc.Config(width=8, height=8, enable_photon_map=True, photon_count=512, spp=1)
    o = orc.OracleRenderer(sc, cfg, camera_of(orc, sc, cfg), threads=2)
    o.rebuild_photons()
    ref = d["photons"].view(orc.PHOTON_DTYPE)
    assert close(o.photons.view(np.float32), ref.view(np.float32), frac=0.995)
    # stored bounces of a photon form a prefix 0..k (no dielectric or cut-out surfaces here)
    stored = (ref["power"][:, 0] > 0).reshape(512, 6)
    for row in stored:
        k = row.sum()
        assert row[:k].all() and not row[k:].any()
    # positions lie on the box (within float tolerance)
    p = ref["position"][ref["power"][:, 0] > 0]
    assert (p >= -1e-2).all() and (p <= 555.01).all()
    assert np.array_equal(o.grid_counts, d["counts"]) or close(o.grid_counts, d["counts"], frac=0.99)


def test_golden_denoise(orc):
    d = np.load(G / "denoise.npz")
    assert close(orc.denoise(d["frame"], d["gbuffer"], d["moments"], 1.0, 2), d["out_a1"], frac=1.0)
    assert close(orc.denoise(d["frame"], d["gbuffer"], d["moments"], 0.25, 2), d["out_a025"], frac=1.0)


def test_golden_tonemap(orc):
    d = np.load(G / "tonemap.npz")
    out = orc.tonemap(d["accum"], 1.5, 2.2, (6.0, 4.0, 2.5, 2.0), 1.2, d["gbuffer"])
    assert np.abs(out.astype(int) - d["out"].astype(int)).max() <= 1


def test_golden_photon_grid_exact(orc):
    d = np.load(G / "photon_grid.npz")
    ph = d["photons"].view(orc.PHOTON_DTYPE)
    gp, _ = orc.derive_grid((np.zeros(3, np.float32), np.full(3, 555.0, np.float32)), 130, 1, len(ph))
    keys = orc.photon_keys(ph, gp)
    assert np.array_equal(keys, d["keys"])
    counts, meta, srt, n = orc.photon_grid(ph, gp)
    nz = np.nonzero(counts)[0]
    assert np.array_equal(nz, d["nonzero_cells"])
    assert np.array_equal(counts[nz], d["counts_nz"]) and np.array_equal(meta[nz], d["meta_nz"])
    assert np.array_equal(srt[:n].view(np.uint8).ravel(), d["sorted"].ravel())


def test_photon_grid_invariants(orc):
    """Counting sort = stable sort by key: offsets are the exclusive scan of the counts, and each cell
    holds its photons in slot order (numpy's stable argsort is the independent check)."""
    d = np.load(G / "photon_grid.npz")
    ph = d["photons"].view(orc.PHOTON_DTYPE)
    gp, _ = orc.derive_grid((np.zeros(3, np.float32), np.full(3, 555.0, np.float32)), 130, 1, len(ph))
    keys = orc.photon_keys(ph, gp)
    counts, meta, srt, n = orc.photon_grid(ph, gp)
    valid = keys != 0xFFFFFFFF
    assert n == valid.sum() == counts.sum()
    assert np.array_equal(meta[:, 1], counts)
    assert np.array_equal(meta[:, 0], np.concatenate([[0], np.cumsum(counts)[:-1]]).astype(np.uint32))
    order = np.argsort(np.where(valid, keys, np.uint32(0xFFFFFFFF)), kind="stable")[:n]
    assert np.array_equal(srt[:n].view(np.uint8), ph[order].view(np.uint8))
    # empty-slot rule: power.r <= 0 is empty even with g, b > 0 (photon_count.wgsl:30)
    assert not valid[ph["power"][:, 0] <= 0].any()


def test_photon_key_wraps_like_the_reference(orc):
    """u32 per-axis keys saturate at 0 below the grid and wrap into the next row at gx == grid_x
    (photon_count.wgsl:18-23); NaN positions map to cell 0 per axis."""
    gp, _ = orc.derive_grid((np.zeros(3, np.float32), np.full(3, 555.0, np.float32)), 26, 0, 4)
    ph = np.zeros(4, orc.PHOTON_DTYPE)
    ph["power"][:, 0] = 1.0
    c = np.float32(gp.cell_size)
    ph["position"][0] = [-50, -50, -50]                           # below: key 0
    ph["position"][1] = [gp.room_min_x + c * 24.5, gp.room_min_y + c * 0.5, gp.room_min_z + c * 0.5]  # gx = 24
    ph["position"][2] = [np.nan, np.nan, np.nan]
    ph["position"][3] = [1e9, 1e9, 1e9]                           # key >= num_cells: dropped
    k = orc.photon_keys(ph, gp)
    assert k[0] == 0 and k[2] == 0
    assert k[1] == 24  # gx + 0 * X: wraps to (0, 1, 0)'s flat index
    assert k[3] == 0xFFFFFFFF
