"""The C-ABI library: exports, host-side logic, and error behaviour without a GPU."""
import ctypes as C

import numpy as np
import pytest

import rustracer_gb300 as rt
from rustracer_gb300 import _abi as A


def test_exports_every_declared_symbol(lib):
    names = A.header_functions()
    assert len(names) > 50
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    # and the ctypes prototypes cover the header
    assert set(A._PROTOS) == set(names)


def test_version_and_error_string(lib):
    assert b"sm_103a" in lib.rt_version()
    st = lib.rt_scene_add_material(None, None)
    assert st == A.RT_ERR_INVALID_ARGUMENT
    assert b"null" in lib.rt_last_error()


def test_render_config_default_matches_reference():
    d = rt.render_config_default()  # RenderConfig::default, rustracer-renderer/src/lib.rs:44-65
    assert (d.width, d.height, d.photon_count, d.spp) == (800, 600, 1_000_000, 1)
    assert (d.exposure, np.float32(d.gamma)) == (1.0, np.float32(2.2))
    assert d.light_emission == (1.0, 1.0, 1.0) and d.point_light_emission == (1.0, 1.0, 1.0)
    assert d.accumulate_frames == 0 and not d.enable_photon_map and d.enable_denoise and not d.photon_debug
    assert np.float32(d.photon_scale) == np.float32(0.02) and d.photon_radius == 0.5
    assert np.float32(d.ambient) == np.float32(0.03)
    assert bytes(rt.RenderConfig().to_c()) == bytes(d.to_c())


def test_cornell555_scene(lib):
    s = rt.Scene.cornell555()
    a = s.arrays()
    assert len(a["triangles"]) == 36
    assert len(a["lights"]) == 2 and (a["lights"]["kind"] == A.LIGHT_AREA).all()
    assert a["lights"]["data"][:, 0].tolist() == [10.0, 11.0]
    light_mat = a["materials"][a["triangles"][10]["material_id"]]
    assert light_mat["kind"] == A.MAT_EMISSIVE and light_mat["emissive"].tolist() == [15.0, 15.0, 15.0]
    # the light faces down (its geometric normal is what NEE tests against)
    t = a["triangles"][10]
    n = np.cross(t["v1"] - t["v0"], t["v2"] - t["v0"])
    assert n[1] < 0 and n[0] == 0 and n[2] == 0
    # 130 x 105 quad at y = 554
    quad = np.concatenate([a["triangles"][10][k] for k in ("v0", "v1", "v2")]).reshape(-1, 3)
    assert np.ptp(quad[:, 0]) == 130 and np.ptp(quad[:, 2]) == 105 and (quad[:, 1] == 554).all()
    lo, hi = s.bounds()
    assert lo.tolist() == [0, 0, 0] and hi.tolist() == [555, 555, 555]


def test_icosphere_room_scene(lib):
    s = rt.Scene.icosphere_room(level=2, seed=5, sigma=0.02, tex_size=32)
    a = s.arrays()
    n_sphere = 20 * 4 ** 2
    assert len(a["triangles"]) == 14 + n_sphere
    assert len(a["materials"]) == 2 + n_sphere
    # per-triangle materials, drawn 60/25/15 (at this size the counts are only roughly those)
    kinds = a["materials"]["kind"][2:]
    assert set(np.unique(kinds).tolist()) <= {0, 1, 2}
    assert (a["triangles"]["material_id"][14:] == np.arange(2, 2 + n_sphere)).all()
    d = s.describe()
    assert d.tex_albedo.layers == 1 and d.tex_albedo.width == 32 and d.tex_normal.layers == 1
    assert d.tex_emissive.layers == 0
    kinds_l = a["lights"]["kind"].tolist()
    assert kinds_l == [2, 2, 0, 0, 0, 0]
    # same seed -> identical scene
    b = rt.Scene.icosphere_room(level=2, seed=5, sigma=0.02, tex_size=32).arrays()
    assert a["triangles"].tobytes() == b["triangles"].tobytes()
    assert a["bvh_nodes"].tobytes() == b["bvh_nodes"].tobytes()


def test_icosphere_level8_counts_formula():
    assert 20 * 4 ** 8 == 1_310_720


def test_camera_uniform_matches_oracle(lib, orc):
    for cam, (w, h) in [(rt.Camera((278, 278, -800), (278, 278, 0), (0, 1, 0), 40.0), (256, 256)),
                        (rt.Camera((1.2, 0.8, 2.4), (0, 0, 0), (0, 1, 0), 60.0), (1920, 1080)),
                        (rt.Camera(), (800, 600))]:
        mine = cam.to_uniform(w, h)
        ref = orc.camera_uniform(cam.position, cam.look_at, cam.up, cam.fov_degrees, w, h, cam.near, cam.aperture,
                                 cam.focus_dist)
        assert bytes(mine) == bytes(ref)


def test_frame_scene_camera(lib):
    s = rt.Scene.cornell555()
    c = s.frame_camera()  # Camera::frame_scene (camera.rs:305-321)
    assert c.fov_degrees == 70.0 and tuple(c.look_at) == (277.5, 277.5, 277.5)
    d = np.array(c.position) - np.array(c.look_at)
    d /= np.linalg.norm(d)
    assert np.allclose(d, np.array([0.55, 0.35, 0.75]) / np.linalg.norm([0.55, 0.35, 0.75]), atol=1e-6)


def test_orbit_zoom(lib):
    c = rt.Camera((0, 0, 5), (0, 0, 0))
    c.zoom(1.0)
    assert np.allclose(c.position, (0, 0, 4), atol=1e-6)
    c.orbit(np.pi / 2, 0.0)
    assert np.allclose(np.linalg.norm(c.position), 4.0, atol=1e-5)
    assert abs(c.position[1]) < 1e-5


@pytest.mark.parametrize("bounds", [None, ((0, 0, 0), (555, 555, 555)), ((-5, -5, -5), (5, 5, 5)),
                                    ((-1, 0, -2), (3, 0.5, 2)), ((0, 0, 0), (0, 0, 0))])
@pytest.mark.parametrize("G,mode", [(0, 0), (26, 0), (130, 1), (64, 1)])
def test_grid_derivation_matches_oracle(lib, orc, bounds, G, mode):
    gp, r = rt.derive_grid(bounds, G, mode, 123)
    gpo, ro = orc.derive_grid(bounds, G, mode, 123)
    assert bytes(gp) == bytes(gpo) and np.float32(r) == np.float32(ro)
    assert gp.num_cells == gp.grid_x * gp.grid_y * gp.grid_z
    assert max(gp.grid_x, gp.grid_y, gp.grid_z) <= (G or 26)


def test_reference_grid_for_cornell():
    """lib.rs:416-457 on the 555 cube: cell = 555/24, 24^3 cells, radius clamp(4 cell) = 2."""
    gp, r = rt.derive_grid(((0, 0, 0), (555, 555, 555)))
    assert (gp.grid_x, gp.grid_y, gp.grid_z) == (24, 24, 24)
    assert np.float32(gp.cell_size) == np.float32(555.0) / np.float32(24.0)
    assert r == 2.0
    gp2, r2 = rt.derive_grid(((0, 0, 0), (555, 555, 555)), 130, 1)
    assert gp2.num_cells == 128 ** 3 == 2_097_152
    assert np.float32(r2) == np.float32(gp2.cell_size) * np.float32(0.5)


def test_renderer_create_without_gpu_fails_loudly(lib):
    if lib.rt_device_count() > 0:
        pytest.skip("a GPU is visible; covered by the gpu tests")
    s = rt.Scene.cornell555()
    with pytest.raises(A.RtError) as e:
        rt.Renderer(s, rt.RenderConfig(width=8, height=8))
    assert e.value.status == A.RT_ERR_CUDA
    assert "no CUDA device" in str(e.value)


def test_invalid_arguments(lib):
    cfg = rt.RenderConfig(width=0, height=8).to_c()
    d = rt.Scene.cornell555().describe()
    h = C.c_void_p()
    assert lib.rt_renderer_create(C.byref(d), C.byref(cfg), C.byref(h)) == A.RT_ERR_INVALID_ARGUMENT
    assert lib.rt_render_frame(None) == A.RT_ERR_INVALID_ARGUMENT
    assert lib.rt_scene_add_mesh(rt.Scene().handle, None, None, None, 3, None, 2, 0) == A.RT_ERR_INVALID_ARGUMENT
    bad = np.array([0, 1, 7], np.uint32)
    pos = np.zeros((3, 3), np.float32)
    assert lib.rt_scene_add_mesh(rt.Scene().handle, A.ptr(pos), None, None, 3, A.ptr(bad), 3, 0) == \
        A.RT_ERR_INVALID_ARGUMENT
    assert lib.rt_stage_denoise(None, None, None, 4, 4, 1.0, 2, None) == A.RT_ERR_INVALID_ARGUMENT


def test_no_exception_crosses_the_c_abi(lib):
    """A vertex count no vector can hold makes the mesh copy throw before anything is read; the entry
    point returns an error code with a message instead of unwinding into the caller."""
    s = rt.Scene()
    pos = np.zeros((3, 3), np.float32)
    idx = np.array([0, 1, 2], np.uint32)
    st = lib.rt_scene_add_mesh(s.handle, A.ptr(pos), None, None, 1 << 63, A.ptr(idx), 3, 0)
    assert st in (A.RT_ERR_STATE, A.RT_ERR_OUT_OF_MEMORY)
    assert b"rt_scene_add_mesh" in lib.rt_last_error()
    assert s.triangle_count() == 0  # the failed call added nothing
    s.add_material(rt.lambertian((0.5, 0.5, 0.5)))
    s.add_mesh(pos + np.eye(3, dtype=np.float32), idx, 0)  # the scene is still usable
    assert s.triangle_count() == 1


def test_mesh_defaults(lib):
    """flatten_triangles (scene.rs:213-273): missing normals -> +Y, missing uvs -> (0, 0)."""
    s = rt.Scene()
    s.add_material(rt.lambertian((0.5, 0.5, 0.5)))
    s.add_mesh([[0, 0, 0], [1, 0, 0], [0, 1, 0]], [0, 1, 2], 0)
    t = s.arrays()["triangles"][0]
    assert t["n0"].tolist() == [0, 1, 0] and t["uv2"].tolist() == [0, 0]
    assert t["v1"].tolist() == [1, 0, 0]


def test_static_library_links_a_c_program(lib, tmp_path):
    """librustracer_cuda.a (the archive a Rust build links with cargo:rustc-link-lib=static) links
    into a plain C program with the CUDA runtime and answers through the C ABI (no device needed)."""
    import shutil
    import subprocess

    from rustracer_gb300 import build as b

    cc = shutil.which("gcc")
    if cc is None or not b.STATIC_LIB.exists():
        pytest.skip("no C compiler or no static archive")
    src = tmp_path / "main.c"
    src.write_text(
        '#include <stdio.h>\n#include "rustracer_cuda.h"\n'
        "int main(void) {\n"
        "    rt_render_config c; rt_render_config_default(&c);\n"
        "    rt_scene *s = 0; if (rt_scene_create_cornell555(&s) != RT_OK) return 2;\n"
        "    rt_scene_desc d; if (rt_scene_describe(s, &d) != RT_OK) return 3;\n"
        '    printf("%s %u %llu %d\\n", rt_version(), c.width, (unsigned long long)d.triangle_count,'
        " rt_device_count() >= 0);\n"
        "    rt_scene_destroy(s); return 0;\n}\n")
    exe = tmp_path / "main"
    cmd = [cc, str(src), "-I", str(b.INCLUDE), str(b.STATIC_LIB), "-L", str(b.cuda_lib_dir()), "-lcudart_static",
           "-lstdc++", "-lpthread", "-ldl", "-lrt", "-lm", "-o", str(exe)]
    res = subprocess.run(cmd, capture_output=True, text=True)
    assert res.returncode == 0, res.stderr
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=60)
    assert out.returncode == 0, out.stderr
    assert out.stdout.split()[-3:] == ["800", "36", "1"]
