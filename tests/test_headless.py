"""The headless entry (render_headless.rs's positional arguments) and accumulation checkpoint / resume."""
import struct
import subprocess
import sys
import zlib
from pathlib import Path

import numpy as np
import pytest

import rustracer_gb300 as rt
from rustracer_gb300 import headless

ROOT = Path(__file__).resolve().parent.parent


def read_png(path: Path) -> np.ndarray:
    data = path.read_bytes()
    assert data[:8] == b"\x89PNG\r\n\x1a\n"
    pos, idat = 8, b""
    w = h = 0
    while pos < len(data):
        n, tag = struct.unpack(">I4s", data[pos:pos + 8])
        body = data[pos + 8:pos + 8 + n]
        assert zlib.crc32(tag + body) & 0xFFFFFFFF == struct.unpack(">I", data[pos + 8 + n:pos + 12 + n])[0]
        if tag == b"IHDR":
            w, h = struct.unpack(">II", body[:8])
        elif tag == b"IDAT":
            idat += body
        pos += 12 + n
    raw = zlib.decompress(idat)
    rows = [raw[y * (4 * w + 1):(y + 1) * (4 * w + 1)] for y in range(h)]
    assert all(r[0] == 0 for r in rows)
    return np.frombuffer(b"".join(r[1:] for r in rows), np.uint8).reshape(h, w, 4)


def test_png_writer_round_trip(tmp_path):
    rng = np.random.default_rng(0)
    img = rng.integers(0, 256, (7, 5, 4), dtype=np.uint8)
    headless.write_png(tmp_path / "a.png", img)
    assert np.array_equal(read_png(tmp_path / "a.png"), img)


def test_reinhard_matches_the_reference_formula():
    acc = np.array([[[0.0, 0.5, 1.0, 1.0], [3.0, 100.0, 1e-4, 1.0]]], np.float32)
    got = headless.reinhard_png_bytes(acc)
    for c in range(3):
        v = float(acc[0, 1, c])
        want = int(min(max(v / (1 + v), 0.0), 1.0) ** (1 / 2.2) * 255.0)
        assert abs(int(got[0, 1, c]) - want) <= 1
    assert (got[..., 3] == 255).all()


@pytest.mark.gpu
@pytest.mark.parametrize("photons,denoise", [(False, False), (True, True)])
def test_checkpoint_resume_continues_the_run(gpu, tmp_path, photons, denoise):
    scene = rt.Scene.cornell555()
    cfg = rt.RenderConfig(width=48, height=40, spp=2, accumulate_frames=6, enable_denoise=denoise,
                          enable_photon_map=photons, photon_count=2048, photon_scale=500.0)

    def fresh():
        r = rt.Renderer(scene, cfg)
        r.update_camera(scene.default_camera())
        if photons:
            r.rebuild_photons()
        return r

    straight = fresh()
    straight.render_frames(8)
    a = fresh()
    a.render_frames(5)
    a.checkpoint(tmp_path / "ck.bin")
    assert (tmp_path / "ck.bin").stat().st_size == 48 * 40 * 16
    b = fresh()
    b.resume(tmp_path / "ck.bin")
    assert b.frame_state() == a.frame_state() == (5, 5)
    b.render_frames(3)
    assert np.array_equal(b.read_accumulation().view(np.uint32), straight.read_accumulation().view(np.uint32))
    assert np.array_equal(b.read_tonemapped(), straight.read_tonemapped())


@pytest.mark.gpu
def test_headless_cli_png_raw_and_resume(gpu, tmp_path):
    base = [sys.executable, "-m", "rustracer_gb300.headless", "cornell"]
    out = tmp_path / "c.png"
    p = subprocess.run(base + ["4", str(out), "1", "0", "0", "2", "8", "40", "30"], cwd=ROOT, capture_output=True,
                       text=True, timeout=300)
    assert p.returncode == 0, p.stderr
    assert read_png(out).shape == (30, 40, 4)
    ck = tmp_path / "ck.bin"
    p = subprocess.run(base + ["4", str(tmp_path / "r"), "0", "0", "0", "1", "8", "40", "30", "0", "0", "0", "0", "1",
                               "--checkpoint", str(ck)], cwd=ROOT, capture_output=True, text=True, timeout=300)
    assert p.returncode == 0, p.stderr
    raw = np.frombuffer((tmp_path / "r.bin").read_bytes(), "<f4").reshape(30, 40, 4)
    assert np.isfinite(raw).all() and raw[..., :3].max() > 0
    # four frames + a resume of four more equal eight frames straight
    p = subprocess.run(base + ["4", str(tmp_path / "s"), "0", "0", "0", "1", "8", "40", "30", "0", "0", "0", "0", "1",
                               "--resume", str(ck)], cwd=ROOT, capture_output=True, text=True, timeout=300)
    assert p.returncode == 0, p.stderr
    p = subprocess.run(base + ["8", str(tmp_path / "t"), "0", "0", "0", "1", "8", "40", "30", "0", "0", "0", "0", "1"],
                       cwd=ROOT, capture_output=True, text=True, timeout=300)
    assert p.returncode == 0, p.stderr
    assert (tmp_path / "s.bin").read_bytes() == (tmp_path / "t.bin").read_bytes()
