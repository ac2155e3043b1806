"""Edge cases and full-size properties of the CUDA path, each checked against the oracle.

Tolerances as in test_gpu_parity.py: radiance within 1e-3 relative (+1e-6) on >= 99.9% of channels,
integer grid data bit-exact.
"""
import numpy as np
import pytest

import rustracer_gb300 as rt
from rustracer_gb300 import _abi as A

from test_gpu_parity import FRAC, match_frac, oracle_for, render_both

pytestmark = pytest.mark.gpu


def feature_scene():
    """Every light kind, an emissive texture, an alpha-cutout albedo texture, metal and glass."""
    s = rt.Scene()
    rng = np.random.default_rng(0)
    tex = (rng.random((2, 16, 16, 4)) * 255).astype(np.uint8)
    tex[0, ..., 3] = np.where((np.arange(16)[:, None] + np.arange(16)[None, :]) % 4 < 2, 255, 30)  # cut-out mask
    tex[1, ..., 3] = 255
    s.set_textures(A.TEX_ALBEDO, tex)
    s.set_textures(A.TEX_EMISSIVE, tex[1:])
    s.set_textures(A.TEX_NORMAL, np.full((1, 8, 8, 4), [128, 128, 255, 255], np.uint8))
    floor = s.add_material(rt.lambertian((0.7, 0.7, 0.7)))
    cut = s.add_material(rt.material(A.MAT_LAMBERTIAN, (0.9, 0.5, 0.2), roughness=1.0, alpha_cutout=True,
                                     tex_albedo=0, tex_normal=0))
    glow = s.add_material(rt.material(A.MAT_EMISSIVE, (1, 1, 1), emissive=(3.0, 2.0, 1.0), tex_emissive=0))
    gold = s.add_material(rt.metal((0.95, 0.64, 0.54), 0.2))
    glass = s.add_material(rt.dielectric(1.5))
    quad = lambda y, sx, sz: ([[-sx, y, -sz], [sx, y, -sz], [sx, y, sz], [-sx, y, sz]], [0, 2, 1, 0, 3, 2])  # noqa
    p, i = quad(0.0, 4.0, 4.0)
    s.add_mesh(p, i, floor, uvs=[[0, 0], [4, 0], [4, 4], [0, 4]])
    s.add_mesh([[-1, 0.1, 0], [1, 0.1, 0], [1, 2, 0], [-1, 2, 0]], [0, 1, 2, 0, 2, 3], cut,
               uvs=[[0, 0], [1, 0], [1, 1], [0, 1]])
    s.add_mesh([[1.5, 0.5, -1], [2.5, 0.5, -1], [2.0, 1.5, -1]], [0, 1, 2], glow, uvs=[[0, 0], [1, 0], [0.5, 1]])
    s.add_mesh([[-2.5, 0.2, 1], [-1.5, 0.2, 1], [-2.0, 1.2, 1]], [0, 1, 2], gold)
    s.add_mesh([[0.5, 0.2, 1.5], [1.5, 0.2, 1.5], [1.0, 1.0, 1.5]], [0, 1, 2], glass)
    s.add_light(rt.environment_light(intensity=0.6))
    s.add_light(rt.directional_light((0.3, 1.0, 0.2), (1.0, 0.9, 0.8), 2.0))
    s.add_light(rt.point_light((0.0, 3.0, 2.0), (1, 1, 1), 5.0))
    s.add_light(rt.area_light(4, (3.0, 2.0, 1.0), 1.0))
    return s


FEATURE_CAM = rt.Camera((0.5, 2.5, 6.0), (0.0, 0.8, 0.0), (0, 1, 0), 50.0)


def test_feature_scene_all_light_kinds(gpu, orc):
    s = feature_scene()
    cfg = rt.RenderConfig(width=72, height=48, spp=4, accumulate_frames=3, enable_denoise=True)
    r, o = render_both(orc, s, cfg, 3, cam=FEATURE_CAM)
    assert match_frac(r.read_accumulation(), o.accum) >= FRAC


def test_empty_scene_is_black(gpu, orc):
    s = rt.Scene()
    cfg = rt.RenderConfig(width=16, height=8, spp=2, enable_denoise=True)
    r, o = render_both(orc, s, cfg, 2)
    acc = r.read_accumulation()
    assert np.array_equal(acc[..., :3], np.zeros_like(acc[..., :3]))
    assert np.array_equal(acc, o.accum)
    assert r.stats().segments == 16 * 8 * 2 * 2  # one miss segment per sample


@pytest.mark.parametrize("w,h,spp", [(1, 1, 1), (37, 23, 3), (33, 17, 9)])
def test_odd_sizes_and_spp(gpu, orc, w, h, spp):
    s = rt.Scene.cornell555()
    cfg = rt.RenderConfig(width=w, height=h, spp=spp, accumulate_frames=2, enable_denoise=True)
    r, o = render_both(orc, s, cfg, 2)
    assert match_frac(r.read_accumulation(), o.accum) >= FRAC
    assert match_frac(r.read_gbuffer(), o.gbuffer) >= FRAC


@pytest.mark.parametrize("view", [1, 2, 3, 4, 5, 8, 9, 11, 12, 13, 17, 18, 19, 20, 21])
def test_debug_views(gpu, orc, view):
    s = feature_scene()
    # spp 9: above 8 the sigma clamp is off; at <= 8 it scales a debug colour by lum / lum_sum = 0
    cfg = rt.RenderConfig(width=32, height=24, spp=9, accumulate_frames=1, enable_denoise=False, debug_view=view)
    r, o = render_both(orc, s, cfg, 1, cam=FEATURE_CAM)
    assert match_frac(r.read_accumulation(), o.accum) >= FRAC


def test_photon_debug_view(gpu, orc):
    s = rt.Scene.cornell555()
    cfg = rt.RenderConfig(width=40, height=40, spp=2, accumulate_frames=2, enable_denoise=False,
                          enable_photon_map=True, photon_count=4096, photon_debug=True)
    r, o = render_both(orc, s, cfg, 2, photons=True)
    assert match_frac(r.read_accumulation(), o.accum) >= FRAC
    assert match_frac(r.read_moments(), o.moments) >= FRAC


@pytest.mark.parametrize("debug", [False, True])
def test_photon_map_never_built(gpu, orc, debug):
    """Photon gathering on with no rebuild: every lookup walks an empty grid (the reference reads its
    zero-initialised buffers), paths still end at their first diffuse bounce."""
    s = rt.Scene.cornell555()
    cfg = rt.RenderConfig(width=32, height=24, spp=2, accumulate_frames=2, enable_denoise=False,
                          enable_photon_map=True, photon_count=4096, photon_debug=debug)
    r, o = render_both(orc, s, cfg, 2)
    assert r.stats().photons_stored == 0
    assert match_frac(r.read_accumulation(), o.accum) >= FRAC


def test_accumulation_controls(gpu, orc):
    """reset_accumulation (hard and soft), update_lights, config mutation and sample_count."""
    s = rt.Scene.cornell555()
    cfg = rt.RenderConfig(width=48, height=48, spp=1, accumulate_frames=8, enable_denoise=False)
    r, o = render_both(orc, s, cfg, 3)
    r.reset_accumulation_soft()
    o.frames_since_reset = 0
    r.record_frame()
    o.record_frame()
    assert match_frac(r.read_accumulation(), o.accum) >= FRAC
    r.reset_accumulation()
    o.frames_since_reset = 0
    o.accum[:] = 0
    lights = [rt.area_light(10, (5.0, 5.0, 5.0), 1.0), rt.area_light(11, (5.0, 5.0, 5.0), 1.0)]
    r.update_lights(lights)
    for k, l in enumerate(lights):  # the same bytes into the oracle's own light array
        C = __import__("ctypes")
        C.memmove(o.desc.lights + k * 64, C.addressof(l), 64)
    cfg2 = r.config
    cfg2.spp = 2
    cfg2.exposure = 1.7
    r.config = cfg2
    o.cfg.spp, o.cfg.exposure = 2, 1.7
    r.render_frames(2)
    for _ in range(2):
        o.record_frame()
    assert r.sample_count() == o.sample_counter == 6
    assert match_frac(r.read_accumulation(), o.accum) >= FRAC
    assert (np.abs(r.read_tonemapped().astype(int) - o.output.astype(int)) <= 1).mean() >= FRAC
    with pytest.raises(A.RtError):
        bad = r.config
        bad.width = 10
        r.config = bad
    with pytest.raises(A.RtError):
        r.update_lights(lights * 2)  # more lights than the buffer holds


def test_deterministic(gpu):
    s = rt.Scene.icosphere_room(level=4, seed=2, sigma=0.02, tex_size=64)
    cfg = rt.RenderConfig(width=96, height=64, spp=4, accumulate_frames=2, enable_denoise=True, max_bounces=8)
    outs = []
    for _ in range(2):
        r = rt.Renderer(s, cfg)
        r.update_camera(s.default_camera())
        r.render_frames(2)
        outs.append((r.read_accumulation(), r.stats().segments))
        r.close()
    assert np.array_equal(outs[0][0], outs[1][0]) and outs[0][1] == outs[1][1]


def test_config2_full_size_sampled_rows(gpu, orc):
    """Config 2 at its full size (1.31M triangles, 1920x1080, 4 spp, depth 8): the whole frame is
    finite and repeatable; rows sampled across the frame match the oracle."""
    s = rt.Scene.icosphere_room(level=8, seed=0, sigma=0.02, tex_size=1024)
    cfg = rt.RenderConfig(width=1920, height=1080, spp=4, accumulate_frames=32, enable_denoise=False, max_bounces=8)
    cam = s.default_camera()
    r = rt.Renderer(s, cfg)
    r.update_camera(cam)
    r.record_frame()
    f1 = r.read_frame()
    assert np.isfinite(f1).all()
    o = oracle_for(orc, s, cfg, cam)
    for rows in [(0, 2), (300, 302), (540, 543), (900, 902), (1078, 1080)]:
        o.sample_counter, o.frames_since_reset = 0, 0
        o.record_frame(rows=rows)
        assert match_frac(f1[rows[0]:rows[1]], o.frame[rows[0]:rows[1]]) >= 0.999
    r2 = rt.Renderer(s, cfg)
    r2.update_camera(cam)
    r2.record_frame()
    assert np.array_equal(r2.read_frame(), f1)


def test_config3_photon_grid_full_size(gpu, orc):
    """Config 3's photon map at full size: 2^20 photons, 128^3 cells.  The grid built on the device
    from the device's photon buffer equals the oracle's counting sort of that buffer bit for bit; the
    traced photons match the oracle's trace slot by slot within float tolerance."""
    s = rt.Scene.cornell555()
    cfg = rt.RenderConfig(width=64, height=64, spp=1, enable_photon_map=True, photon_count=1 << 20,
                          grid_max_dim=130, photon_radius_mode=1)
    r = rt.Renderer(s, cfg)
    r.rebuild_photons()
    gp = r.grid_params()
    assert gp.num_cells == 128 ** 3 and gp.photon_slots == 6 << 20
    ph = r.read_photons()
    counts, meta = r.read_photon_grid()
    srt = r.read_sorted_photons()
    o = oracle_for(orc, s, cfg, s.default_camera())
    o.load_photons(ph)
    assert np.array_equal(counts, o.grid_counts)
    assert np.array_equal(meta, o.grid_meta)
    assert np.array_equal(srt[:o.binned].view(np.uint8), o.sorted[:o.binned].view(np.uint8))
    assert r.stats().photons_stored == o.binned > 1_000_000
    assert rt._abi.load().rt_scan_timeouts() == 0
    o2 = oracle_for(orc, s, cfg, s.default_camera())
    o2.rebuild_photons()
    assert match_frac(ph.view(np.float32), o2.photons.view(np.float32), rtol=1e-4, atol=1e-4) >= 0.999


def test_profiled_frames_render_the_same_image(gpu):
    """Profiling (events around the launches, counting traversal kernels) leaves every image and
    count as it is; its ray counts are the frame statistics' and every ray visits a record."""
    s = rt.Scene.icosphere_room(level=4, seed=2, sigma=0.02, tex_size=32)
    cfg = rt.RenderConfig(width=96, height=64, spp=2, accumulate_frames=3, enable_denoise=False, max_bounces=6)
    imgs = []
    for flags in (0, A.PROFILE_EVENTS, A.PROFILE_COUNT, A.PROFILE_EVENTS | A.PROFILE_COUNT):
        r = rt.Renderer(s, cfg)
        r.update_camera(s.default_camera())
        r.set_profiling(flags)
        r.render_frames(3)
        imgs.append(r.read_accumulation())
        p = r.read_profile()
        st = r.stats()
        r.close()
        if not flags:
            assert p.frames == 0
            continue
        assert p.frames == 3 and p.pixels == 96 * 64 and p.record_bytes == 128
        assert p.closest_rays == st.segments and p.occlusion_rays == st.shadow_rays
        assert p.trace_launches == 3 * (2 * 6 + 1) and p.shade_launches == 3 * 2 * 6
        if flags & A.PROFILE_EVENTS:
            assert 0.0 < p.ms_trace < p.ms_gather and 0.0 < p.ms_shade < p.ms_gather
        if flags & A.PROFILE_COUNT:
            assert p.records_closest >= p.closest_rays and p.records_occlusion >= p.occlusion_rays
            assert p.tri_tests_closest > 0 and p.tri_tests_occlusion > 0
    assert all(np.array_equal(imgs[0], im) for im in imgs[1:])
