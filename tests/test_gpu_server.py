"""The render-request loop (rt_server_*): every job's image is the one it renders alone, whatever
else is in flight (continuous batching), in batched and plain mode; scenes are evicted least
recently used first under the HBM cap; a job that cannot fit fails without blocking the others.
"""
import time

import numpy as np
import pytest

import rustracer_gb300 as rt

from test_gpu_edge import FEATURE_CAM, feature_scene

pytestmark = pytest.mark.gpu


def alone(scene, cfg, cam, frames):
    r = rt.Renderer(scene, cfg)
    r.update_camera(cam)
    if cfg.enable_photon_map:
        r.rebuild_photons()
    r.render_frames(frames)
    out = r.read_accumulation()
    r.close()
    return out


@pytest.fixture(scope="module")
def scenes():
    return {0: rt.Scene.cornell555(), 1: feature_scene(), 2: rt.Scene.icosphere_room(level=2, seed=5, tex_size=32)}


def requests(scenes):
    c0, c2 = scenes[0].default_camera(), scenes[2].default_camera()
    c0b = scenes[0].default_camera()
    c0b.orbit(-0.4, 0.2)
    return [
        (0, rt.RenderConfig(width=48, height=32, spp=2, accumulate_frames=4, enable_denoise=True, max_bounces=5), c0, 4),
        (1, rt.RenderConfig(width=40, height=24, spp=3, accumulate_frames=0, enable_denoise=False), FEATURE_CAM, 2),
        (2, rt.RenderConfig(width=32, height=32, spp=1, accumulate_frames=8, enable_denoise=True,
                            enable_photon_map=True, photon_count=2048, photon_scale=50.0), c2, 5),
        (0, rt.RenderConfig(width=17, height=9, spp=9, accumulate_frames=2, enable_denoise=True), c0b, 3),
        (2, rt.RenderConfig(width=24, height=16, spp=4, accumulate_frames=3, enable_denoise=False, max_bounces=7), c2, 6),
    ]


@pytest.fixture(scope="module")
def expected(scenes):
    return [alone(scenes[sid], cfg, cam, n) for sid, cfg, cam, n in requests(scenes)]


@pytest.mark.parametrize("mode,graphs", [("batched", True), ("batched", False), ("plain", False)])
def test_each_job_matches_its_run_alone(gpu, scenes, expected, mode, graphs):
    with rt.Server(mode=mode, graphs=graphs, hbm_cap_bytes=8 << 30, max_slots=1 << 16) as srv:
        for sid, sc in scenes.items():
            srv.add_scene(sid, sc)
        ids = []
        # staggered arrivals: later jobs join a batch already in flight
        for k, (sid, cfg, cam, n) in enumerate(requests(scenes)):
            ids.append(srv.submit(sid, cfg, cam, n, keep_result=True))
            if k % 2:
                time.sleep(0.002)
        srv.wait_idle(120)
        st = srv.stats()
        assert st.completed == len(ids) and st.failed == 0
        for k, jid in enumerate(ids):
            s = srv.status(jid)
            assert s.state == rt._abi.JOB_DONE and s.frames_done == requests(scenes)[k][3]
            assert 0 <= s.t_submit_ms <= s.t_admit_ms <= s.t_first_frame_ms <= s.t_done_ms
            img = srv.result(jid)
            assert np.array_equal(img.view(np.uint32), expected[k].view(np.uint32)), f"job {k} differs ({mode})"
        if mode == "batched":
            assert st.max_active >= 2  # jobs really overlapped
        assert st.scene_uploads == 3 and st.scene_evictions == 0


def test_lru_eviction_under_a_small_cap(gpu):
    a = rt.Scene.icosphere_room(level=4, seed=1, tex_size=128)
    b = rt.Scene.icosphere_room(level=4, seed=2, tex_size=128)
    cfg = rt.RenderConfig(width=16, height=16, spp=1, accumulate_frames=2, enable_denoise=False)
    cam = a.default_camera()
    # room for the path state, one scene and a job, not two scenes
    probe = rt.Server(max_slots=1024, hbm_cap_bytes=1 << 40)
    probe.add_scene(0, a)
    j = probe.submit(0, cfg, cam, 1)
    probe.wait_idle(60)
    st = probe.stats()
    scene_bytes, path_bytes = st.resident_scene_bytes, st.used_bytes - st.resident_scene_bytes
    probe.close()
    cap = path_bytes + scene_bytes * 3 // 2 + (1 << 20)
    with rt.Server(max_slots=1024, hbm_cap_bytes=cap) as srv:
        srv.add_scene(0, a)
        srv.add_scene(1, b)
        ids = []
        for sid in (0, 1, 0):
            ids.append(srv.submit(sid, cfg, cam, 2, keep_result=True))
            srv.wait_idle(60)
        st = srv.stats()
        assert st.completed == 3
        assert st.scene_uploads == 3 and st.scene_evictions == 2
        assert st.peak_bytes <= cap
        assert np.array_equal(srv.result(ids[0]), srv.result(ids[2]))
        assert np.array_equal(srv.result(ids[1]), alone(b, cfg, cam, 2))
    del j


def test_job_that_cannot_fit_fails_alone(gpu, scenes):
    with rt.Server(max_slots=4096, hbm_cap_bytes=1 << 30) as srv:
        srv.add_scene(0, scenes[0])
        big = srv.submit(0, rt.RenderConfig(width=128, height=128, spp=1), scenes[0].default_camera(), 1)
        ok = srv.submit(0, rt.RenderConfig(width=32, height=32, spp=1), scenes[0].default_camera(), 2)
        srv.wait_idle(60)
        assert srv.status(big).state == rt._abi.JOB_FAILED
        assert srv.status(ok).state == rt._abi.JOB_DONE
        srv.release(big)
        with pytest.raises(RuntimeError):
            srv.status(big)
