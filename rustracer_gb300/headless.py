"""Headless render with the positional arguments of rustracer's render_headless example
(rustracer-app/examples/render_headless.rs:5-11):

    python -m rustracer_gb300.headless <scene> [frames] [out.png] [denoise] [app_like] [photons] [spp]
        [accum] [w] [h] [debug_view] [zoom] [yaw] [pitch] [raw_save] [--checkpoint P] [--resume P]

<scene> is a glTF / GLB file (read by rustracer_gb300.gltf, with a sibling scene.toml applied as the
reference does) or a procedural scene: `cornell` (the 555-unit Cornell box) or
`icosphere[:level[:seed]]` (the displaced icosphere room).  Pass 1 for the boolean slots.  As in the
reference: app_like means spp 4 and a 32-frame accumulation; the camera frames the scene
(Camera::frame_scene) and is then zoomed / orbited; photon maps use 50,000 photons; the PNG is
the CPU Reinhard + gamma 2.2 of the accumulation (examples/common/mod.rs:37-47) and raw_save writes
the accumulation as raw f32 RGBA to <out>.bin instead.  --checkpoint writes the accumulation and
frame counters after the run, --resume continues a checkpointed run.
"""
from __future__ import annotations

import argparse
import struct
import sys
import zlib
from pathlib import Path

import numpy as np

from .renderer import RenderConfig, Renderer
from .scene import Scene


def make_scene(spec: str) -> Scene:
    if spec.lower().endswith((".gltf", ".glb")):
        from .gltf import load_gltf

        return load_gltf(spec)
    name, *rest = spec.split(":")
    if name == "cornell":
        return Scene.cornell555()
    if name == "icosphere":
        level = int(rest[0]) if rest else 8
        seed = int(rest[1]) if len(rest) > 1 else 0
        return Scene.icosphere_room(level, seed)
    raise SystemExit(f"unknown scene {spec!r}: use a .gltf / .glb file, cornell or icosphere[:level[:seed]]")


def reinhard_png_bytes(acc: np.ndarray) -> np.ndarray:
    """examples/common/mod.rs:37-47: (v / (1 + v)).clamp(0, 1)^(1/2.2) * 255, truncated to u8."""
    v = acc[..., :3].astype(np.float32)
    m = np.clip(v / (np.float32(1.0) + v), 0.0, 1.0) ** np.float32(1.0 / 2.2) * np.float32(255.0)
    out = np.empty(acc.shape[:2] + (4,), np.uint8)
    out[..., :3] = m.astype(np.uint8)
    out[..., 3] = 255
    return out


def write_png(path: Path, rgba: np.ndarray) -> None:
    h, w = rgba.shape[:2]
    raw = b"".join(b"\x00" + rgba[y].tobytes() for y in range(h))

    def chunk(tag: bytes, data: bytes) -> bytes:
        return struct.pack(">I", len(data)) + tag + data + struct.pack(">I", zlib.crc32(tag + data) & 0xFFFFFFFF)

    path.write_bytes(b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, 8, 6, 0, 0, 0)) +
                     chunk(b"IDAT", zlib.compress(raw, 6)) + chunk(b"IEND", b""))


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("scene")
    ap.add_argument("frames", nargs="?", type=int, default=128)
    ap.add_argument("out", nargs="?", default="render_headless.png")
    ap.add_argument("denoise", nargs="?", default="0")
    ap.add_argument("app_like", nargs="?", default="0")
    ap.add_argument("photons", nargs="?", default="0")
    ap.add_argument("spp", nargs="?", type=int, default=None)
    ap.add_argument("accum", nargs="?", type=int, default=None)
    ap.add_argument("w", nargs="?", type=int, default=800)
    ap.add_argument("h", nargs="?", type=int, default=600)
    ap.add_argument("debug_view", nargs="?", type=int, default=0)
    ap.add_argument("zoom", nargs="?", type=float, default=0.0)
    ap.add_argument("yaw", nargs="?", type=float, default=0.0)
    ap.add_argument("pitch", nargs="?", type=float, default=0.0)
    ap.add_argument("raw_save", nargs="?", default="0")
    ap.add_argument("--checkpoint", default=None, help="write the accumulation + frame counters here at the end")
    ap.add_argument("--resume", default=None, help="continue from a checkpoint written by --checkpoint")
    a = ap.parse_args(argv)
    app_like, denoise, photons = a.app_like == "1", a.denoise == "1", a.photons == "1"
    spp = a.spp if a.spp is not None else (4 if app_like else 1)
    accum = a.accum if a.accum is not None else (32 if app_like else a.frames)

    scene = make_scene(a.scene)
    cfg = RenderConfig(width=a.w, height=a.h, spp=spp, accumulate_frames=accum, enable_denoise=denoise or app_like,
                       enable_photon_map=photons, photon_count=50_000, debug_view=a.debug_view)
    r = Renderer(scene, cfg)
    if photons:
        r.rebuild_photons()
    cam = scene.frame_camera()
    if a.zoom != 0.0:
        cam.zoom(a.zoom)
    if a.yaw != 0.0 or a.pitch != 0.0:
        cam.orbit(a.yaw, a.pitch)
    r.update_camera(cam)
    if a.resume:
        r.resume(a.resume)
    r.render_frames(a.frames)
    acc = r.read_accumulation()
    if a.checkpoint:
        r.checkpoint(a.checkpoint)
    print(f"scene: {scene.triangle_count()} tris; {a.frames} frames of {a.w}x{a.h}, spp {spp}, "
          f"accumulate {accum}, sample count {r.sample_count()}")
    if a.raw_save == "1":
        path = Path(a.out + ".bin")
        path.write_bytes(acc.astype("<f4").tobytes())
        print(f"saved raw {path}")
        return 0
    write_png(Path(a.out), reinhard_png_bytes(acc))
    print(f"saved {a.out}")
    return 0


if __name__ == "__main__":
    sys.exit(main())
