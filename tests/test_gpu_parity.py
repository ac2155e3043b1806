"""Parity of the sm_103a kernels (through the C ABI) with the oracle on the same inputs.

Tolerances (floating point, written here as the parity bar states them):
  * accumulated radiance: |gpu - oracle| <= 1e-3 |oracle| + 1e-6 on at least 99.9% of channels (the
    path's sin / cos / pow are one fixed IEEE sequence on both backends and equal-t hits resolve to
    the lowest prim slot, so paths do not diverge; the margin is for float evaluation-order
    differences);
  * stage kernels on identical inputs: 1e-5 relative (denoise: CUDA's and glibc's exp / pow per tap
    differ by an ulp or two), bit-exact where no transcendental function is involved (composite),
    +-1 on rgba8 bytes (tonemap pow);
  * integer work (cell keys, counts, offsets, slot order): bit-exact.
"""
import ctypes as C

import numpy as np
import pytest

import rustracer_gb300 as rt
from rustracer_gb300 import _abi as A

pytestmark = pytest.mark.gpu

RTOL, ATOL, FRAC = 1e-3, 1e-6, 0.999


def match_frac(a, b, rtol=RTOL, atol=ATOL):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    ok = np.abs(a - b) <= rtol * np.abs(b) + atol
    return float(ok.mean())


def oracle_scene(orc, scene):
    """The oracle's copy of a backend scene: the flattened triangles, materials, lights and textures
    handed over and indexed by the oracle's own BVH build, so the oracle never walks the backend's
    tree (the builds agree byte for byte on the CPU: test_oracle_scene.py)."""
    a = scene.arrays()
    d = scene.describe()
    tex = []
    for name in ("tex_albedo", "tex_mr", "tex_emissive", "tex_normal"):
        t = getattr(d, name)
        n = t.width * t.height * t.layers * 4
        tex.append(np.ctypeslib.as_array(C.cast(t.rgba8, C.POINTER(C.c_uint8)), shape=(n,)).reshape(
            t.layers, t.height, t.width, 4).copy() if t.layers else None)
    o = orc.OracleScene.from_arrays(a["triangles"], a["materials"], a["lights"], tex)
    lo, hi, has = o.arrays()["bounds"]
    assert has == d.has_bounds and (not has or (tuple(lo) == tuple(d.bounds_min) and tuple(hi) == tuple(d.bounds_max)))
    return o


def oracle_for(orc, scene, cfg, cam):
    u = orc.camera_uniform(cam.position, cam.look_at, cam.up, cam.fov_degrees, cfg.width, cfg.height, cam.near,
                           cam.aperture, cam.focus_dist)
    return orc.OracleRenderer(oracle_scene(orc, scene), cfg, u)


def render_both(orc, scene, cfg, frames, cam=None, photons=False):
    cam = cam or scene.default_camera()
    r = rt.Renderer(scene, cfg)
    r.update_camera(cam)
    o = oracle_for(orc, scene, cfg, cam)
    if photons:
        r.rebuild_photons()
        o.load_photons(r.read_photons())  # identical photon buffer on both sides
    r.render_frames(frames)
    for _ in range(frames):
        o.record_frame()
    return r, o


def test_cornell_config1_accumulation(gpu, orc):
    """Config 1: 555-unit Cornell box, 256x256, 1 spp x 16 frames, accumulate 16, NEE, no photons/denoise."""
    scene = rt.Scene.cornell555()
    cfg = rt.RenderConfig(width=256, height=256, spp=1, accumulate_frames=16, enable_denoise=False)
    r, o = render_both(orc, scene, cfg, 16)
    acc = r.read_accumulation()
    assert np.isfinite(acc).all()
    f = match_frac(acc, o.accum)
    assert f >= FRAC, f"only {f:.5f} of channels within 1e-3"
    st = r.stats()
    assert st.frames == 16
    seg_o, shd_o = int(o.counters[0]), int(o.counters[1])
    assert abs(st.segments - seg_o) <= 1e-3 * seg_o
    assert abs(st.shadow_rays - shd_o) <= 1e-3 * shd_o
    assert r.sample_count() == 16
    tm = r.read_tonemapped()
    assert (np.abs(tm.astype(int) - o.output.astype(int)) <= 1).mean() >= FRAC


def test_first_frame_buffers(gpu, orc):
    scene = rt.Scene.cornell555()
    cfg = rt.RenderConfig(width=128, height=96, spp=3, accumulate_frames=0, enable_denoise=False)
    r, o = render_both(orc, scene, cfg, 1)
    assert match_frac(r.read_frame(), o.frame) >= FRAC
    assert match_frac(r.read_moments(), o.moments) >= FRAC
    g = r.read_gbuffer()
    assert match_frac(g, o.gbuffer) >= FRAC
    # primary misses keep the 1e30 depth sentinel (gather.wgsl:272); the hit masks agree
    hit_g, hit_o = g[..., 3] < 1e29, o.gbuffer[..., 3] < 1e29
    assert (hit_g == hit_o).mean() >= FRAC and 0.3 < hit_g.mean() < 1.0


def test_icosphere_textured_all_materials(gpu, orc):
    """Displaced icosphere room with per-triangle Lambertian/GGX/dielectric materials, albedo/MR/normal
    textures, an area light and point lights; depth 8 (config 2's extension of the reference's 6)."""
    scene = rt.Scene.icosphere_room(level=3, seed=7, sigma=0.02, tex_size=64)
    cfg = rt.RenderConfig(width=96, height=64, spp=4, accumulate_frames=3, enable_denoise=False, max_bounces=8)
    r, o = render_both(orc, scene, cfg, 3)
    f = match_frac(r.read_accumulation(), o.accum)
    assert f >= FRAC, f
    kinds = scene.arrays()["materials"]["kind"]
    assert {0, 1, 2, 3} <= set(np.unique(kinds).tolist())


@pytest.mark.parametrize("h,w", [(61, 97), (136, 200)])  # the larger size has tiles away from every border
def test_denoise_stage(gpu, orc, h, w):
    rng = np.random.default_rng(3)
    frame = rng.random((h, w, 4), np.float32) * 2
    frame[..., 3] = 1
    n = rng.normal(size=(h, w, 3)).astype(np.float32)
    n /= np.linalg.norm(n, axis=-1, keepdims=True)
    gbuf = np.concatenate([n, rng.uniform(0.5, 10, (h, w, 1)).astype(np.float32)], -1)
    m1 = rng.random((h, w), np.float32)
    mom = np.stack([m1, m1 * m1 + rng.random((h, w), np.float32) * 0.1, np.zeros_like(m1), np.zeros_like(m1)], -1)
    for alpha in (1.0, 0.25):
        for passes in (1, 2):
            g = rt.stage_denoise(frame, gbuf, mom, alpha, passes)
            ref = orc.denoise(frame, gbuf, mom, alpha, passes)
            assert match_frac(g, ref, rtol=1e-5, atol=1e-7) == 1.0


def test_denoise_tiles_arrive(gpu):
    """Every denoise block of the tests so far received its TMA tile copies within the wait bound."""
    assert A.load().rt_tma_timeouts() == 0


def test_resolve_stage(gpu, orc):
    rng = np.random.default_rng(4)
    h, w = 33, 45
    frame = (rng.random((h, w, 4), np.float32) * 4).astype(np.float32)
    accum = (rng.random((h, w, 4), np.float32) * 4).astype(np.float32)
    for alpha in (1.0, 0.5, 1.0 / 7.0):
        acc_g, img_g = rt.stage_resolve(frame, accum, alpha, exposure=1.3, gamma=2.2)
        acc_o = orc.composite(frame, accum, alpha)
        img_o = orc.tonemap(acc_o, 1.3, 2.2)
        assert np.array_equal(acc_g, acc_o)
        d = np.abs(img_g.astype(int) - img_o.astype(int))
        assert d.max() <= 1 and (d == 0).mean() >= FRAC
    # light gizmo (tonemap.wgsl:253-268)
    gbuf = np.full((h, w, 4), 5.0, np.float32)
    acc_g, img_g = rt.stage_resolve(frame, accum, 1.0, marker=(20.0, 15.0, 4.0, 3.0), glow=1.5, gbuffer=gbuf)
    img_o = orc.tonemap(orc.composite(frame, accum, 1.0), 1.0, 2.2, (20.0, 15.0, 4.0, 3.0), 1.5, gbuf)
    assert np.abs(img_g.astype(int) - img_o.astype(int)).max() <= 1


def random_photons(rng, n, gp, frac_invalid=0.2):
    ph = np.zeros(n, rt._abi.np_dtype(rt._abi.Photon))
    lo = np.array([gp.room_min_x, gp.room_min_y, gp.room_min_z], np.float32)
    span = np.array([gp.grid_x, gp.grid_y, gp.grid_z], np.float32) * np.float32(gp.cell_size)
    ph["position"] = lo + rng.random((n, 3), np.float32) * span * np.float32(1.1) - span * np.float32(0.05)
    ph["power"] = rng.random((n, 3), np.float32)
    ph["incident"] = rng.normal(size=(n, 3)).astype(np.float32)
    ph["normal"] = rng.normal(size=(n, 3)).astype(np.float32)
    dead = rng.random(n) < frac_invalid
    ph["power"][dead, 0] = 0.0  # empty slot rule: power.r <= 0 (photon_count.wgsl:30)
    ph["position"][:7] = np.array([np.nan, 0, 0], np.float32)  # NaN -> key 0 per axis
    # clustered photons: many share a cell (exercises the per-cell slot ordering beyond 32 and 1024)
    ph["position"][100:2600] = lo + span * np.float32(0.5)
    # cells of about 40, 100, 200 and 300 photons at slots spread over the buffer (each cell-size class
    # of the per-cell sort: one, two, four and eight entries per lane, and past the register sort)
    rest = rng.permutation(np.arange(3000, n))
    at = 0
    for size, frac in ((50, 0.21), (125, 0.33), (250, 0.71), (375, 0.83)):
        ph["position"][rest[at:at + size]] = lo + span * np.float32(frac)
        at += size
    return ph


# 26: the reference's grid (one scan tile per look-back chunk); 102: 100^3 cells (two tiles per chunk
# on a 152-SM GPU); 130: 128^3 cells (four tiles per chunk)
@pytest.mark.parametrize("grid_max_dim", [26, 102, 130])
def test_photon_grid_stage_bit_exact(gpu, orc, grid_max_dim):
    gp, _ = rt.derive_grid((np.zeros(3), np.full(3, 555.0)), grid_max_dim, 1 if grid_max_dim > 26 else 0, 1)
    rng = np.random.default_rng(grid_max_dim)
    ph = random_photons(rng, 60_000, gp)
    counts, meta, srt = rt.stage_photon_grid(ph, gp)
    gpo = orc.GridParams.from_buffer_copy(gp)
    gpo.photon_slots = len(ph)
    c_o, m_o, s_o, n = orc.photon_grid(ph.view(orc.PHOTON_DTYPE), gpo)
    assert np.array_equal(counts, c_o)
    assert np.array_equal(meta, m_o)
    assert np.array_equal(srt[:n].view(np.uint8), s_o[:n].view(np.uint8))
    # every scan tile found its predecessors' sums within the look-back's wait bound
    assert A.load().rt_scan_timeouts() == 0


def test_photon_map_and_denoise_cornell(gpu, orc):
    """Config 3's pipeline at a small size: photon trace, grid, gather with photons, 2 a-trous passes."""
    scene = rt.Scene.cornell555()
    cfg = rt.RenderConfig(width=80, height=64, spp=4, accumulate_frames=4, enable_denoise=True,
                          enable_photon_map=True, photon_count=8192, photon_scale=2000.0)
    cam = scene.default_camera()
    r = rt.Renderer(scene, cfg)
    r.update_camera(cam)
    r.rebuild_photons()
    gpu_ph = r.read_photons()
    o = oracle_for(orc, scene, cfg, cam)
    o.rebuild_photons()
    # the traces agree slot by slot (float tolerance; a diverged photon path shows as a mismatch)
    assert match_frac(gpu_ph.view(np.float32), o.photons.view(np.float32), rtol=1e-4, atol=1e-4) >= FRAC
    # the grid is exact on an identical photon buffer
    o.load_photons(gpu_ph)
    counts, meta = r.read_photon_grid()
    assert np.array_equal(counts, o.grid_counts)
    assert np.array_equal(meta, o.grid_meta)
    srt = r.read_sorted_photons()
    assert np.array_equal(srt[:o.binned].view(np.uint8), o.sorted[:o.binned].view(np.uint8))
    assert r.stats().photons_stored == o.binned
    r.render_frames(4)
    for _ in range(4):
        o.record_frame()
    f = match_frac(r.read_accumulation(), o.accum)
    assert f >= FRAC, f


@pytest.mark.parametrize("grid_max_dim, radius_mode", [(26, 0), (130, 1), (130, 0)])
def test_photon_gather_grid_modes(gpu, orc, grid_max_dim, radius_mode):
    """The gather's photon lookups on an identical photon buffer, with the reference's grid (26 cells,
    radius clamp(4 cell, .01, 2)), the fine grid with radius cell / 2, and the fine grid with the
    reference's radius rule (a radius wider than the cell: every neighbour cell may hold hits)."""
    scene = rt.Scene.cornell555()
    cfg = rt.RenderConfig(width=48, height=40, spp=2, accumulate_frames=2, enable_denoise=False,
                          enable_photon_map=True, photon_count=16384, photon_scale=2000.0,
                          grid_max_dim=grid_max_dim, photon_radius_mode=radius_mode)
    r, o = render_both(orc, scene, cfg, 2, photons=True)
    assert match_frac(r.read_accumulation(), o.accum) >= FRAC


def test_second_rebuild_counts_photons_left_from_the_first(gpu, orc):
    """The histogram is taken inside the photon pass; slots the second pass does not write keep the
    first pass's photons (the reference never clears the slot buffer) and must still be counted."""
    scene = rt.Scene.cornell555()
    cfg = rt.RenderConfig(width=16, height=16, spp=1, enable_photon_map=True, photon_count=4096 + 100,
                          photon_scale=500.0)
    r = rt.Renderer(scene, cfg)
    r.rebuild_photons()
    first = r.read_photons()
    # a dimmer, moved light: different paths, so some slots of the first pass are not rewritten
    r.update_lights([rt.point_light((278.0, 500.0, 278.0), (1.0, 1.0, 1.0), 0.4)])
    r.rebuild_photons()
    ph = r.read_photons()
    stale = (first.view(np.uint8).reshape(len(first), -1) == ph.view(np.uint8).reshape(len(ph), -1)).all(1)
    assert stale.sum() > 0 and (~stale).sum() > 0
    counts, meta = r.read_photon_grid()
    o = oracle_for(orc, scene, cfg, scene.default_camera())
    o.load_photons(ph)  # the oracle's count pass over the whole slot buffer
    assert np.array_equal(counts, o.grid_counts)
    assert np.array_equal(meta, o.grid_meta)
    srt = r.read_sorted_photons()
    assert np.array_equal(srt[:o.binned].view(np.uint8), o.sorted[:o.binned].view(np.uint8))
