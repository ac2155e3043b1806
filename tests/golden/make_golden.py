"""Generates the golden vectors in tests/golden/ from the oracle.

    python tests/golden/make_golden.py

The reference (Rust + WGSL on wgpu) cannot run on this machine, so these vectors pin the oracle's
restatement against regressions; the independent checks live in tests/test_oracle_pins.py.  Only the
oracle runs here: the scenes are the oracle's own (oracle/scene.cpp).
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))

import oracle  # noqa: E402

RNG_SEEDS = [0, 1, 12345, 0xFFFFFFFF, 2654435761, 1013904223]


def oracle_render(scene, cfg, frames):
    o = oracle.OracleRenderer(scene, cfg, camera_of(scene, cfg), threads=1)
    if cfg.enable_photon_map:
        o.rebuild_photons()
    for _ in range(frames):
        o.record_frame()
    return o


def camera_of(scene, cfg):
    """The camera uniform of an oracle scene's default camera at the config's size."""
    c = scene.camera()
    return oracle.camera_uniform(tuple(c.position), tuple(c.look_at), tuple(c.up), c.fov_degrees, cfg.width,
                                 cfg.height, c.near_plane, c.aperture, c.focus_dist)


def golden_inputs_denoise():
    rng = np.random.default_rng(11)
    h, w = 12, 16
    frame = rng.random((h, w, 4), np.float32) * np.float32(3)
    frame[..., 3] = 1
    n = rng.normal(size=(h, w, 3)).astype(np.float32)
    n /= np.linalg.norm(n, axis=-1, keepdims=True)
    gbuf = np.concatenate([n, rng.uniform(0.5, 4, (h, w, 1)).astype(np.float32)], -1)
    m = rng.random((h, w), np.float32)
    mom = np.stack([m, m * m + rng.random((h, w), np.float32) * np.float32(0.2), np.zeros_like(m), np.zeros_like(m)],
                   -1).astype(np.float32)
    return frame, gbuf, mom


def golden_photons(gp, n=3000, seed=5):
    rng = np.random.default_rng(seed)
    ph = np.zeros(n, oracle.PHOTON_DTYPE)
    lo = np.array([gp.room_min_x, gp.room_min_y, gp.room_min_z], np.float32)
    span = np.array([gp.grid_x, gp.grid_y, gp.grid_z], np.float32) * np.float32(gp.cell_size)
    ph["position"] = lo + rng.random((n, 3), np.float32) * span
    ph["power"] = rng.random((n, 3), np.float32)
    ph["power"][rng.random(n) < 0.25, 0] = 0.0
    ph["position"][50:400] = lo + span * np.float32(0.3)
    return ph


def main() -> None:
    oracle.build()
    out = {}
    # PCG sequences
    seqs = np.stack([oracle.rng_sequence(s, 32)[0] for s in RNG_SEEDS])
    np.savez_compressed(HERE / "rng.npz", seeds=np.array(RNG_SEEDS, np.uint32), u32=seqs)

    # Cornell (config-1 scene) at 32x32, spp 2, denoise on, 4 frames
    sc = oracle.OracleScene.cornell555()
    cfg = oracle.Config(width=32, height=32, spp=2, accumulate_frames=4, enable_denoise=True)
    o = oracle_render(sc, cfg, 4)
    np.savez_compressed(HERE / "cornell_32x32.npz", accum=o.accum, output=o.output, frame=o.frame,
                        moments=o.moments, gbuffer=o.gbuffer, counters=o.counters)
    out["cornell"] = o.counters.tolist()

    # textured icosphere room, all material kinds, depth 8
    ico = oracle.OracleScene.icosphere_room(2, 3, 0.02, 16)
    cfg2 = oracle.Config(width=24, height=16, spp=3, accumulate_frames=2, enable_denoise=False, max_bounces=8)
    o2 = oracle_render(ico, cfg2, 2)
    np.savez_compressed(HERE / "icosphere_24x16.npz", accum=o2.accum, counters=o2.counters)

    # photon trace of the Cornell box, 512 photons (the reference's GPU smoke-test size)
    cfg3 = oracle.Config(width=8, height=8, enable_photon_map=True, photon_count=512, spp=1)
    o3 = oracle_render(sc, cfg3, 0)
    np.savez_compressed(HERE / "photons_cornell_512.npz", photons=o3.photons.view(np.uint8),
                        counts=o3.grid_counts, meta=o3.grid_meta)

    # denoise on fixed inputs
    frame, gbuf, mom = golden_inputs_denoise()
    np.savez_compressed(HERE / "denoise.npz", frame=frame, gbuffer=gbuf, moments=mom,
                        out_a1=oracle.denoise(frame, gbuf, mom, 1.0, 2), out_a025=oracle.denoise(frame, gbuf, mom, 0.25, 2))

    # photon grid of a seeded buffer (config-mode 128^3 grid on the 555 box)
    gp, _ = oracle.derive_grid((np.zeros(3, np.float32), np.full(3, 555.0, np.float32)), 130, 1, 3000)
    ph = golden_photons(gp)
    counts, meta, srt, n = oracle.photon_grid(ph, gp)
    nz = np.nonzero(counts)[0]
    np.savez_compressed(HERE / "photon_grid.npz", photons=ph.view(np.uint8), keys=oracle.photon_keys(ph, gp),
                        nonzero_cells=nz.astype(np.uint32), counts_nz=counts[nz], meta_nz=meta[nz],
                        sorted=srt[:n].view(np.uint8))

    # tonemap with the light gizmo
    acc = (np.random.default_rng(2).random((10, 14, 4), np.float32) * np.float32(5)).astype(np.float32)
    g = np.full((10, 14, 4), 3.0, np.float32)
    np.savez_compressed(HERE / "tonemap.npz", accum=acc, gbuffer=g,
                        out=oracle.tonemap(acc, 1.5, 2.2, (6.0, 4.0, 2.5, 2.0), 1.2, g))
    print("golden vectors written:", sorted(p.name for p in HERE.glob("*.npz")), out)


if __name__ == "__main__":
    main()
