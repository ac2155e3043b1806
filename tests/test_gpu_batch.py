"""Batched rendering (rt_batch_*): several jobs' rays share the wavefront launches, and each job's
image is the one it renders alone, bit for bit (same seeds, same per-pixel operations), with and
without CUDA graph replay.
"""
import numpy as np
import pytest

import rustracer_gb300 as rt

from test_gpu_edge import FEATURE_CAM, feature_scene

pytestmark = pytest.mark.gpu


def job_specs():
    """Mixed scenes, sizes, spp, depths, accumulation budgets, denoise and photon settings."""
    cornell = rt.Scene.cornell555()
    ico = rt.Scene.icosphere_room(level=2, seed=3, sigma=0.02, tex_size=32)
    feat = feature_scene()
    cam2 = cornell.default_camera()
    cam2.orbit(0.3, -0.1)
    return [
        (cornell, rt.RenderConfig(width=64, height=48, spp=2, accumulate_frames=4, enable_denoise=True,
                                  max_bounces=5), None, False),
        (feat, rt.RenderConfig(width=40, height=24, spp=3, accumulate_frames=0, enable_denoise=False),
         FEATURE_CAM, False),
        (ico, rt.RenderConfig(width=56, height=40, spp=1, accumulate_frames=8, enable_denoise=True,
                              enable_photon_map=True, photon_count=4096, photon_scale=50.0, max_bounces=8),
         None, True),
        (cornell, rt.RenderConfig(width=17, height=9, spp=9, accumulate_frames=2, enable_denoise=True), cam2, False),
    ]


def make(spec):
    scene, cfg, cam, photons = spec
    r = rt.Renderer(scene, cfg)
    r.update_camera(cam or scene.default_camera())
    if photons:
        r.rebuild_photons()
    return r


def outputs(r):
    return [r.read_accumulation(), r.read_tonemapped(), r.read_gbuffer(), r.read_frame()]


def same(a, b):
    return all(np.array_equal(x.view(np.uint8), y.view(np.uint8)) for x, y in zip(a, b))


@pytest.fixture(scope="module")
def specs():
    return job_specs()


@pytest.fixture(scope="module")
def alone(specs):
    res = []
    for sp in specs:
        r = make(sp)
        r.render_frames(5)
        res.append((outputs(r), r.stats().segments))
        r.close()
    return res


@pytest.mark.parametrize("graphs", [False, True])
def test_batch_matches_each_job_alone(gpu, specs, alone, graphs):
    rs = [make(sp) for sp in specs]
    b = rt.Batch(rs, use_graphs=graphs)
    b.render_frames(5)
    b.synchronize()
    st = b.stats()
    assert st.frames == 5
    assert st.segments == sum(seg for _, seg in alone)
    if graphs:
        assert st.graph_captures == 1  # per-frame values (alpha, frame counters) come from the job table
    for j, r in enumerate(rs):
        assert r.sample_count() == 5
        assert same(outputs(r), alone[j][0]), f"job {j} differs from its run alone"
    b.close()


def test_batch_then_solo_frames_continue_the_sequence(gpu, specs, alone):
    """Three batch frames, then two frames rendered alone: the same images as five frames alone."""
    rs = [make(sp) for sp in specs]
    b = rt.Batch(rs, use_graphs=True)
    b.render_frames(3)
    for r in rs:
        r.render_frames(2)
    for j, r in enumerate(rs):
        assert same(outputs(r), alone[j][0]), f"job {j}"
    b.close()


def test_batch_recaptures_when_settings_change(gpu, specs):
    rs = [make(sp) for sp in specs[:2]]
    b = rt.Batch(rs, use_graphs=True)
    b.render_frames(2)
    cfg = rs[0].config
    cfg.spp = 5  # 5 x 5 iterations, more than the batch's 18: the captured launches no longer fit
    rs[0].config = cfg
    b.render_frames(2)
    assert b.stats().graph_captures == 2
    # the same four frames through a batch without graphs
    rs2 = [make(sp) for sp in specs[:2]]
    b2 = rt.Batch(rs2, use_graphs=False)
    b2.render_frames(2)
    rs2[0].config = cfg
    b2.render_frames(2)
    for r, r2 in zip(rs, rs2):
        assert same(outputs(r), outputs(r2))
    b.close()
    b2.close()


def test_batch_rejects_bad_arguments(gpu, specs):
    r = make(specs[0])
    with pytest.raises(RuntimeError):
        rt.Batch([r, r])
    with pytest.raises(RuntimeError):
        rt.Batch([])


def test_resident_scene_shared_by_renderers(gpu, specs):
    scene, cfg, cam, _ = specs[2]  # textured icosphere room with a photon map
    cam = cam or scene.default_camera()
    res = rt.ResidentScene(scene)
    assert res.refs() == 1 and res.device_bytes() > 0
    create_bytes, path_bytes = res.footprint(cfg)
    a, b = rt.Renderer(res, cfg), rt.Renderer(res, cfg)
    assert res.refs() == 3
    assert a.device_bytes() == create_bytes  # the footprint predicts the allocation
    for r in (a, b):
        r.update_camera(cam)
        r.rebuild_photons()
    # lights are per renderer: dimming b's lights leaves a's image alone
    ref = make(specs[2])
    b.update_lights([rt.point_light((0.0, 4.0, 0.0), (1.0, 1.0, 1.0), 0.0)])  # replaces light 0
    for r in (a, b, ref):
        r.render_frames(3)
    assert same(outputs(a), outputs(ref))
    assert not np.array_equal(outputs(b)[0], outputs(ref)[0])
    assert a.device_bytes() == create_bytes + path_bytes  # the first solo frame added the path state
    res.close()  # the renderers keep the scene alive
    a.render_frame()
    a.close()
    b.close()


def test_autotune_leaves_images_unchanged(gpu, specs, alone):
    """Trial frames of the autotuner are undone; any launch shape renders the same images."""
    rs = [make(sp) for sp in specs]
    b = rt.Batch(rs, use_graphs=True)
    b.render_frames(2)
    best, ms = b.autotune(trial_frames=1)
    assert ms > 0 and best == b.tuning
    assert all(r.sample_count() == 2 for r in rs)
    b.render_frames(3)
    for j, r in enumerate(rs):
        assert same(outputs(r), alone[j][0]), f"job {j}"
    b.close()


@pytest.mark.parametrize("shape", [dict(block_threads=64, blocks_per_sm=16, chunk=32, steps=4, stack_entries=48),
                                   dict(block_threads=256, blocks_per_sm=4, chunk=256, steps=32, stack_entries=64),
                                   dict(block_threads=128, blocks_per_sm=8, chunk=32, steps=4, stack_entries=32,
                                        treelet=1)])
def test_launch_shape_does_not_change_images(gpu, specs, alone, shape):
    rs = [make(sp) for sp in specs]
    for r in rs:
        r.tuning = shape
        assert r.tuning["block_threads"] == shape["block_threads"]
        r.render_frames(5)
    for j, r in enumerate(rs):
        assert same(outputs(r), alone[j][0]), f"job {j}"


def test_treelet_in_a_batch_of_several_scenes(gpu, specs, alone):
    """With the treelet on, a batch stages job 0's top records; lanes on the other jobs' scenes read
    their records from global memory.  Every job's image is its image rendered alone."""
    rs = [make(sp) for sp in specs]
    b = rt.Batch(rs, use_graphs=True)
    t = dict(b.tuning)
    t["treelet"] = 1
    b.tuning = t
    assert b.tuning["treelet"] == 1
    b.render_frames(5)
    for j, r in enumerate(rs):
        assert same(outputs(r), alone[j][0]), f"job {j}"
    b.close()


def test_renderer_buffers_are_reused(gpu):
    """A renderer's buffers come from the device's renderer pool in its stream order: destroying one
    and creating another of the same shape reuses the freed blocks, so repeated create / render /
    destroy cycles leave free device memory where the first cycle left it (no growth, no leak)."""
    torch = pytest.importorskip("torch")
    scene = rt.Scene.cornell555()
    cfg = rt.RenderConfig(width=640, height=480, spp=1, accumulate_frames=4, enable_denoise=True,
                          enable_photon_map=True, photon_count=1 << 16)

    def cycle():
        r = rt.Renderer(scene, cfg)
        r.update_camera(scene.default_camera())
        r.rebuild_photons()
        r.render_frames(2)
        acc = r.read_accumulation()
        r.close()
        torch.cuda.synchronize()
        return acc

    keep = rt.Renderer(scene, cfg)  # a live renderer keeps the pool from being trimmed in between
    first = cycle()  # its freed buffers stay in the pool
    free_after_first = torch.cuda.mem_get_info()[0]
    for _ in range(3):
        assert np.array_equal(cycle(), first)  # the reused buffers start clean: same image
        assert abs(torch.cuda.mem_get_info()[0] - free_after_first) <= 8 << 20
    keep.close()
